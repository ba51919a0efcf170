"""Builds liblpm_gpu.so in-tree with nvcc for sm_103a (GB300).

Each translation unit under csrc/ is compiled in parallel to _build/, then linked into
liblpm_gpu.so next to this file.  Host code is compiled with -ffp-contract=off so the mesh
generator and every host-side FP64 constant round identically on x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
BUILD_DIR = PKG_DIR / "_build"
LIB_PATH = PKG_DIR / "liblpm_gpu.so"
INCLUDE = REPO_DIR / "include"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON_FLAGS = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-Xcompiler",
    "-fPIC,-ffp-contract=off,-fno-fast-math",
    f"-I{INCLUDE}",
    f"-I{CSRC}",
]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblpm_gpu")
    return cand


def _sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h")))


def _needs_rebuild(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None, extra_flags: list[str] | None = None) -> Path:
    """Compiles (incrementally) and links liblpm_gpu.so; returns its path."""
    nvcc = _nvcc()
    BUILD_DIR.mkdir(exist_ok=True)
    headers = _headers()
    flags = ARCH_FLAGS + COMMON_FLAGS + list(extra_flags or [])
    cmds = []
    objs = []
    for src in _sources():
        obj = BUILD_DIR / (src.name + ".o")
        objs.append(obj)
        if _needs_rebuild(obj, [src] + headers + [Path(__file__)]):
            cmds.append([nvcc, *flags, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)

    workers = jobs or max(1, min(len(cmds), os.cpu_count() or 4))
    if cmds:
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            list(ex.map(run, cmds))
    if cmds or _needs_rebuild(LIB_PATH, objs):
        run([nvcc, *ARCH_FLAGS, "-shared", "-o", str(LIB_PATH), *map(str, objs)])
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
