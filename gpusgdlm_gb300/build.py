"""Builds the in-tree CUDA shared library ``libsgdlm_gb300.so`` for sm_103a.

Each translation unit is compiled by its own nvcc process (in parallel), then
linked with ``nvcc -shared``.  Objects go to ``gpusgdlm_gb300/_build/``; the
library lands next to this file so that it is found without installation.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libsgdlm_gb300.so"
# the reference's C++ engine interface (SGDLM::HostWrapper<double> and its
# factory) on top of LIB: plain C++, no CUDA headers
HW_SRC = CSRC / "host_wrapper.cpp"
HW_LIB = HERE / "libsgdlm_hostwrapper.so"
SOURCES = [
    "state_kernels.cu",
    "sample_kernels.cu",
    "lu_kernels.cu",
    "vb_kernels.cu",
    "engine.cu",
    "elimination.cu",
    "noalloc.cu",
    "mlp_kernels.cu",
    "proposal_kernels.cu",
    "forecast_kernels.cu",
    "warp_lu.cu",
]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3"]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: the SGDLM CUDA library cannot be built")


def _stale(obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    if not LIB.exists():
        force = True  # objects from another machine must not be relinked
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.hpp")) + list((HERE.parent / "include").glob("*.h"))
    cc = nvcc()

    def compile_one(src: str) -> Path:
        s = CSRC / src
        obj = BUILD / (Path(src).stem + ".o")
        if force or _stale(obj, [s] + headers):
            cmd = [cc, *ARCH, *FLAGS, "-c", str(s), "-o", str(obj)]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or _stale(LIB, objs):
        cmd = [cc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    build_host_wrapper(verbose, force)
    return LIB


def build_host_wrapper(verbose: bool = False, force: bool = False) -> Path:
    """libsgdlm_hostwrapper.so: g++ on host_wrapper.cpp, linked against LIB and
    finding it next to itself at run time."""
    deps = [HW_SRC, LIB, HERE.parent / "include" / "sgdlm.h",
            HERE.parent / "include" / "sgdlm_hostwrapper.hpp"]
    if force or _stale(HW_LIB, deps):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", str(HW_SRC), "-o", str(HW_LIB),
               "-L", str(HERE), "-lsgdlm_gb300", "-Wl,-rpath,$ORIGIN"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed on host_wrapper.cpp:\n{r.stdout}\n{r.stderr}")
    return HW_LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
