"""Builds libsanepic_gpu.so (and the drop-in `sanepic` executable) in-tree.

Every CUDA translation unit is compiled for sm_103a only, in parallel, with
plain nvcc (no cmake).  sg_pointing.cu is compiled with --fmad=false so the
HEALPix pixel arithmetic keeps the reference's IEEE operation order.
Outputs go to sanepic_gb300/lib/ (git-ignored).
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-I", os.path.join(ROOT, "include"), "-I", CSRC]
UNITS = {
    "sg_filter.cu": [],
    "sg_filter_spec.cu": [],
    "sg_filter_spec64.cu": [],
    "sg_setup.cu": [],
    "sg_pt.cu": [],
    "sg_group.cu": [],
    "sg_fft3.cu": [],
    "sg_recal.cu": [],
    "sg_cg.cu": [],
    "sg_api.cu": [],
    "sg_noalloc.cu": [],
    "sg_gemm.cu": [],
    "sg_mlp.cu": [],
    "sg_learn.cu": [],
    "sg_batch.cu": [],
    "sg_pointing.cu": ["--fmad=false"],
}
LIB = os.path.join(LIBDIR, "libsanepic_gpu.so")
CLI = os.path.join(LIBDIR, "sanepic")


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra: list[str], verbose: bool) -> str:
    obj = os.path.join(OBJDIR, src.replace(".cu", ".o").replace(".cpp", ".o"))
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    """Compile the library (and CLI); returns the path of the shared library."""
    os.makedirs(OBJDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "sanepic_gpu.h"))
    todo = {}
    for src, extra in UNITS.items():
        obj = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        if force or _stale(obj, [os.path.join(CSRC, src)] + headers):
            todo[src] = extra
    jobs = jobs or min(len(UNITS), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(_compile, s, e, verbose) for s, e in todo.items()]
        for f in futs:
            f.result()
    objs = [os.path.join(OBJDIR, s.replace(".cu", ".o")) for s in UNITS]
    if force or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    cli_src = os.path.join(CSRC, "sg_cli.cpp")
    if os.path.exists(cli_src) and (force or _stale(CLI, [cli_src, LIB])):
        cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), cli_src,
               "-o", CLI, "-L", LIBDIR, "-lsanepic_gpu", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
