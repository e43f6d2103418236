"""CPU checks of the drop-in boundary: libib3d.so loads and exports every
function include/ib3d.h declares, and fails cleanly (an error code, no crash)
when no GPU is present."""
from __future__ import annotations

import ctypes
import pathlib

import numpy as np
import pytest


@pytest.fixture(scope="module")
def built_lib(ib3d):
    if not ib3d.LIB_PATH.exists():
        ib3d.build()
    return ib3d.LIB_PATH


def test_header_declares_the_step_routines(ib3d):
    names = ib3d.header_functions()
    for n in ("ib3d_create", "ib3d_ns_momentum", "ib3d_velocity_bc", "ib3d_solid_cell_bc", "ib3d_velocity_forcing",
              "ib3d_pressure_forcing", "ib3d_poisson_solver", "ib3d_stress", "ib3d_step", "ib3d_search",
              "ib3d_set_mesh", "ib3d_destroy", "ib3d_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(ib3d, built_lib):
    lib = ctypes.CDLL(str(built_lib))
    missing = [n for n in ib3d.header_functions() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_mirror_binds_every_symbol(ib3d, built_lib):
    L = ib3d.lib()
    for n in ib3d.header_functions():
        assert getattr(L, n).argtypes is not None or getattr(L, n).restype is not None, n


def test_params_struct_layout(ib3d, built_lib):
    p = ib3d.default_params()
    # 4 doubles, int64, 6 int32, double, 5 int32 + 4 bytes of tail padding
    assert ctypes.sizeof(ib3d.Params) == 8 * 4 + 8 + 4 * 6 + 8 + 5 * 4 + 4   # padded to 8 bytes
    assert ib3d.Params.omega_inner.offset == 64 and ib3d.Params.inner_schedule.offset == 72
    assert ib3d.Params.outlet.offset == 76 and ib3d.Params.momentum.offset == 80
    assert ib3d.Params.smooth_sweeps.offset == 84 and ib3d.Params.ramp_sweeps.offset == 88
    assert ctypes.sizeof(ib3d.SolveStats) == 7 * 8
    assert p.omega == 1.99 and p.eps == 1e-5 and p.criterion == ib3d.CRIT_UPDATE
    assert p.inner_schedule == ib3d.INNER_FIXED


def test_create_without_gpu_returns_error(ib3d, built_lib, grids):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    cs = grids.case("tiny")
    with pytest.raises(ib3d.IB3DError) as e:
        ib3d.Solver(cs.x, cs.y, cs.z, ib3d.default_params())
    assert e.value.code == ib3d.ERR_CUDA


def test_oracle_library_builds_and_loads(oracle_mod):
    L = oracle_mod.lib()
    for n in ("or_create", "or_step", "or_search", "or_poisson_solver", "or_stress"):
        assert hasattr(L, n)


@pytest.mark.parametrize("fmt", ["gmsh", "gambit"])
def test_surface_mesh_files_round_trip(ib3d, built_lib, grids, tmp_path, fmt):
    """ib3d_read_surface_mesh (host code, no GPU) reads back what grids writes in the
    record layout of readSurfaceMeshGmsh / readSurfaceMeshGambit, exactly."""
    nodes, tris = grids.icosphere(3, 0.5)
    path = tmp_path / f"body.{fmt}"
    if fmt == "gmsh":
        grids.write_gmsh(path, nodes, tris)
        got_n, got_t = ib3d.read_surface_mesh(path, ib3d.MESH_GMSH)
    else:
        grids.write_gambit(path, nodes, tris)
        got_n, got_t = ib3d.read_surface_mesh(path, ib3d.MESH_GAMBIT)
    assert np.array_equal(got_n, nodes) and np.array_equal(got_t, tris)
    # surGeoPoints: the first element lines are skipped
    if fmt == "gmsh":
        _, t2 = ib3d.read_surface_mesh(path, ib3d.MESH_GMSH, sur_geo_points=5)
        assert np.array_equal(t2, tris[5:])
    with pytest.raises(ib3d.IB3DError) as e:
        path.write_text(path.read_text()[:200])
        ib3d.read_surface_mesh(path, ib3d.MESH_GMSH if fmt == "gmsh" else ib3d.MESH_GAMBIT)
    assert e.value.code == ib3d.ERR_IO


def test_noalloc_rejects_extents_beyond_its_scratch_before_any_cuda_call(ib3d):
    """Absurd extents (whose product would overflow int64) are rejected up front,
    without touching a device, so this runs on a machine without a GPU."""
    import ctypes as C
    L = ib3d.lib()
    dummy = C.c_void_p(1)
    for n in ((2 ** 40, 2 ** 40, 2 ** 40), (2 ** 62, 8, 8), (200, 200, 200), (2 ** 21, 4, 4)):
        rc = L.ib3d_pressure_solve_noalloc(*n, dummy, dummy, dummy, dummy, dummy, 0.001, dummy, 1.9, 1e-6, 10, 4,
                                           None, None, None)
        assert rc == ib3d.ERR_TOO_LARGE, (n, rc)


def test_download_entry_points_reject_a_null_context(ib3d, built_lib):
    """The blocking and the asynchronous download and its wait check their context
    before touching the device: a null context is IB3D_ERR_ARG, with no CUDA call."""
    L = ib3d.lib()
    none = [None] * 7
    assert L.ib3d_download_fields(None, *none) == ib3d.ERR_ARG
    assert L.ib3d_download_fields_async(None, *none) == ib3d.ERR_ARG
    assert L.ib3d_download_wait(None) == ib3d.ERR_ARG


@pytest.mark.parametrize("field,value,accepted", [("sweep_kernel", 4, True), ("sweep_kernel", 5, False),
                                                  ("sweep_kernel", -1, False), ("precision", 2, True),
                                                  ("precision", 3, False), ("warm_start", 3, False)])
def test_create_validates_parameters_before_touching_the_device(ib3d, built_lib, grids, field, value, accepted):
    """ib3d_create checks its parameters before its first CUDA call: a value out of
    range is IB3D_ERR_ARG; an accepted one gets as far as the device query, which
    fails without a GPU (IB3D_ERR_CUDA)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    cs = grids.case("tiny")
    p = ib3d.default_params()
    setattr(p, field, value)
    with pytest.raises(ib3d.IB3DError) as e:
        ib3d.Solver(cs.x, cs.y, cs.z, p)
    assert e.value.code == (ib3d.ERR_CUDA if accepted else ib3d.ERR_ARG), (field, value)
