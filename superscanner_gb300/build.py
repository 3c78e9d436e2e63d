"""In-tree build of the native parts.

``build_native()`` compiles every ``csrc/*.cu`` for sm_103a in parallel and
links ``superscanner_gb300/libss.so`` (static CUDA runtime, C-ABI of
``include/ss_abi.h``).
Objects are rebuilt only when a source or header is newer than the library.
Host code is compiled with ``-ffp-contract=off`` so that the host-side pose
arithmetic (inverse, normalisation) rounds the same on x86 and Arm.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libss.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", *ARCH,
    "-Xcompiler", "-fPIC,-ffp-contract=off",
    "--expt-relaxed-constexpr", "-I", str(INCLUDE),
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libss.so")


def _newest(paths) -> float:
    return max((p.stat().st_mtime for p in paths), default=0.0)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_cuda(force: bool = False, verbose: bool = False) -> Path:
    sources = sorted(CSRC.glob("*.cu"))
    headers = list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    if not force and LIB.exists() and LIB.stat().st_mtime >= _newest(sources + headers + [Path(__file__)]):
        return LIB
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    objs = [BUILD / (s.stem + ".o") for s in sources]
    jobs = [[nvcc, *NVCC_FLAGS, "-c", str(s), "-o", str(o)] for s, o in zip(sources, objs)]
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        for cmd, fut in zip(jobs, [ex.submit(_run, c) for c in jobs]):
            fut.result()
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs), "-ldl"])
    os.replace(tmp, LIB)
    return LIB


SHIM_SRC = ROOT / "tests" / "cpp" / "shim_roundtrip.cpp"
SHIM_BIN = BUILD / "shim_roundtrip"


def build_shim_test(force: bool = False) -> Path:
    """C++ program that drives the reference-shaped shim header over libss.so."""
    deps = [SHIM_SRC, INCLUDE / "ss_gpu_voxel_grid.hpp", INCLUDE / "ss_abi.h", LIB]
    if not force and SHIM_BIN.exists() and SHIM_BIN.stat().st_mtime >= _newest(deps):
        return SHIM_BIN
    cuda = Path(_nvcc()).resolve().parent.parent
    BUILD.mkdir(exist_ok=True)
    _run(["g++", "-O2", "-std=c++17", "-I", str(INCLUDE), "-I", str(cuda / "include"), str(SHIM_SRC),
          "-o", str(SHIM_BIN), "-L", str(PKG), "-lss", "-L", str(cuda / "lib64"), "-lcudart",
          f"-Wl,-rpath,{PKG}", f"-Wl,-rpath,{cuda / 'lib64'}"])
    return SHIM_BIN


def build_native(force: bool = False, verbose: bool = False) -> None:
    build_cuda(force, verbose)
    build_shim_test(force)


if __name__ == "__main__":
    build_native(force="--force" in sys.argv, verbose=True)
    print(LIB)
