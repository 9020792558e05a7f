"""Build recipe for libtecto.so (CUDA for sm_103a) - in-tree, no cmake.

Every translation unit is compiled in parallel with nvcc for sm_103a only, with multiply-add
contraction disabled on both the device (-fmad=false) and the host (-ffp-contract=off) side: the
engine's float arithmetic is defined operation by operation so that the CPU oracle can match it
bit for bit.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG.parent / "_build" / "tecto"
LIB = PKG / "libtecto.so"

SOURCES = [
    "tecto_api.cu",
    "tecto_batch.cu",
    "tecto_server.cu",
    "tecto_tune.cu",
    "k_uplift.cu",
    "k_sort.cu",
    "k_sort_noalloc.cu",
    "k_collide.cu",
    "k_dynamics.cu",
    "k_policy.cu",
    "k_resolve.cu",
    "k_erosion.cu",
    "k_ccl.cu",
    "tecto_export.cu",
    "tecto_init.cu",
    "tecto_packed.cu",
    "settings.cpp",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-fmad=false",
    "-prec-div=true",
    "-prec-sqrt=true",
    "-ftz=false",
    "-Xcompiler",
    "-fPIC,-ffp-contract=off,-fopenmp,-fno-fast-math",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compile the engine into master_thesis_gb300/libtecto.so; returns its path."""
    BUILD.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list((PKG.parent / "include").glob("*.h"))
    flags = COMMON + (extra_flags or [])

    def compile_one(src: str) -> Path:
        s = CSRC / src
        o = BUILD / (src + ".o")
        if _stale(o, [s, *headers]):
            cmd = [nvcc(), *ARCH, *flags, "-c", str(s), "-o", str(o)]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return o

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-Xcompiler", "-fopenmp", "-lgomp"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
