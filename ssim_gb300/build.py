"""Builds the CUDA library libssim_gb300.so in-tree with nvcc for sm_103a (GB300).

Few translation units compiled in parallel, one -gencode, static cudart: the
same recipe runs on x86_64 (cross-compile, no GPU needed) and on the aarch64
GPU hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libssim_gb300.so")
SOURCES = ["kernels_elem.cu", "kernels_sparse.cu", "kernels_adjoint.cu", "kernels_springs.cu", "kernels_lbfgs.cu", "kernels_tri.cu", "kernels_fused.cu",
           "timestep.cu",
           "topology.cpp", "noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3,-fvisibility=hidden", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build ssim_gb300")


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "ssim_gb.h"))
    cc = nvcc()
    jobs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        if _stale(obj, [path] + headers):
            cmd = [cc, *ARCH, *FLAGS, "-c", path, "-o", obj]
            if ptxas_info and src.endswith(".cu"):
                cmd.insert(1, "-Xptxas=-v")
            jobs.append((src, cmd))
    with cf.ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        futs = {ex.submit(subprocess.run, cmd, capture_output=True, text=True): src for src, cmd in jobs}
        for fut in cf.as_completed(futs):
            r = fut.result()
            if verbose or ptxas_info:
                sys.stdout.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {futs[fut]}:\n{r.stderr}")
    objs = [os.path.join(BUILD, s + ".o") for s in SOURCES]
    if jobs or _stale(LIB, objs):
        cmd = [cc, *ARCH, "-shared", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
