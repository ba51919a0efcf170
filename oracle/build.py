"""Builds the CPU oracle (test infrastructure): oracle/_build/liblpm_oracle.so.

gcc -O3 -fopenmp -ffp-contract=off: no fused multiply-add anywhere, so each product and
sum rounds where the reference Fortran source rounds it (as an x86-64 gfortran build does).
The reference itself (Fortran + MPI) cannot be built here -- no Fortran compiler -- so
there is no oracle/_ref build.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
BUILD_DIR = ORACLE_DIR / "_build"
LIB_PATH = BUILD_DIR / "liblpm_oracle.so"
SOURCES = [ORACLE_DIR / "lpm_oracle.c"]
HEADERS = [ORACLE_DIR / "lpm_oracle.h"]
CFLAGS = ["-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-std=c11"]


def build(verbose: bool = False) -> Path:
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler found for the oracle")
    BUILD_DIR.mkdir(exist_ok=True)
    deps = SOURCES + HEADERS + [Path(__file__)]
    if LIB_PATH.exists() and all(d.stat().st_mtime <= LIB_PATH.stat().st_mtime for d in deps):
        return LIB_PATH
    cmd = [cc, *CFLAGS, "-o", str(LIB_PATH), *map(str, SOURCES), "-lm"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
