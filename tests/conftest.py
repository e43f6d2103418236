"""Test set-up: the `gpu` marker, and imports of the package (whose directory
name, ib3d-gpu_gb300, is not a Python identifier) and of the CPU oracle."""
from __future__ import annotations

import importlib.util
import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def load_package():
    if "ib3d_gpu_gb300" in sys.modules:
        return sys.modules["ib3d_gpu_gb300"]
    pkg = ROOT / "ib3d-gpu_gb300"
    spec = importlib.util.spec_from_file_location("ib3d_gpu_gb300", pkg / "__init__.py",
                                                  submodule_search_locations=[str(pkg)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["ib3d_gpu_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libib3d.so")


@pytest.fixture(scope="session")
def ib3d():
    return load_package()


@pytest.fixture(scope="session")
def grids(ib3d):
    return ib3d.grids


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    return oracle
