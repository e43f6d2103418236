"""Builds libib3d.so (the CUDA hot path behind include/ib3d.h) in-tree for sm_103a.

Translation units are compiled with -fmad=false (no contraction of FP64
multiply-adds, so the FP64 path keeps the reference's rounding), except the
fast momentum kernel of the mixed-precision path; host code always uses
-ffp-contract=off. The FP32 inner solve uses explicit fmaf().
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
LIB = HERE / "libib3d.so"
SOURCES = ["ib3d_api.cu", "k_pressure.cu", "k_momentum.cu", "k_ib.cu", "k_sor32.cu", "noalloc.cu", "k_momentum_fast.cu", "k_fast.cu", "k_unet.cu",
           "unet.cu", "restart.cu", "mesh_io.cu"]
# translation units whose multiply-adds may contract (results differ from the reference by rounding)
FMAD_TRUE = {"k_momentum_fast.cu", "k_fast.cu"}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libib3d.so")


def flags() -> list[str]:
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-I", str(HERE.parent / "include")]


def _compile(src: str, out_dir: pathlib.Path, extra: list[str]) -> pathlib.Path:
    obj = out_dir / (pathlib.Path(src).stem + ".o")
    fl = flags()
    if src in FMAD_TRUE:
        fl = [f for f in fl if f != "-fmad=false"] + ["-fmad=true"]
    cmd = [nvcc(), *fl, *extra, "-c", str(CSRC / src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> pathlib.Path:
    """Compiles the sources in parallel and links libib3d.so next to this file."""
    out_dir = HERE / "_build"
    out_dir.mkdir(exist_ok=True)
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, out_dir, extra), SOURCES))
    tmp = HERE / "libib3d.so.tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
