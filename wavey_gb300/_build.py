"""Builds the package's native libraries in-tree.

libwavey_cuda.so  the sm_103a CUDA backend and its C-ABI (include/wavey_cuda.h)
libwavey_host.so  the host-side grid, material and signal library (include/wavey_host.h)

Both are compiled straight with nvcc / g++ (no cmake), in parallel, into
wavey_gb300/_lib/.  Host code is compiled with -ffp-contract=off so that
FP64 results do not depend on whether the compiler fuses multiply-adds
(GCC fuses by default on aarch64).
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB = PKG / "_lib"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libwavey_cuda.so")


def _cuda_cmd(out: Path) -> list[str]:
    return [
        nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-shared",
        "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off,-O2",
        "-I", str(INCLUDE),
        str(CSRC / "wavey_cuda.cu"), str(CSRC / "receiver_dft_noalloc.cu"), "-o", str(out), "-lgomp",
    ]


def _host_cmd(out: Path) -> list[str]:
    srcs = sorted(str(p) for p in (CSRC / "host").glob("*.cpp"))
    return ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
            "-I", str(INCLUDE), *srcs, "-o", str(out)]


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, cuda: bool = True) -> dict[str, Path]:
    """Compiles whatever is out of date and returns the library paths."""
    LIB.mkdir(exist_ok=True)
    jobs = {}
    host_out = LIB / "libwavey_host.so"
    host_deps = list((CSRC / "host").glob("*")) + list(INCLUDE.glob("*.h"))
    if force or _stale(host_out, host_deps):
        jobs[host_out] = _host_cmd(host_out)
    cuda_out = LIB / "libwavey_cuda.so"
    if cuda:
        cuda_deps = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
        if force or _stale(cuda_out, cuda_deps):
            jobs[cuda_out] = _cuda_cmd(cuda_out)
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(_run, jobs.values()))
    return {"host": host_out, "cuda": cuda_out}


if __name__ == "__main__":
    print(build(force=True))
