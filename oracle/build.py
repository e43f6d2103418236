"""Build recipe of the CPU oracle (test infrastructure): liboracle.so from
ib3d_oracle.c with gcc, -ffp-contract=off (no fused multiply-add, so every FP64
operation rounds as the reference's expressions do) and OpenMP for the timed
CPU baseline (the parallel loops are the ones the reference marks
`!$acc parallel`; their results do not depend on the thread count).

No reference sources are compiled: the reference is Fortran and no Fortran
compiler exists on either machine.
"""
from __future__ import annotations

import os
import pathlib
import shutil
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"


def build(verbose: bool = False) -> pathlib.Path:
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler found for the oracle")
    tmp = HERE / "liboracle.so.tmp"
    cmd = [cc, "-O3", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-o", str(tmp), str(HERE / "ib3d_oracle.c"), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
