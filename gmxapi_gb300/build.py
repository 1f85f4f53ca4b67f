"""Build recipe for the sm_103a engine library (no cmake, no torch).

Compiles gmxapi_gb300/csrc/*.cu with nvcc for sm_103a into
gmxapi_gb300/lib/libnbnxm_gb300.so.  The grid, search and prune translation
units are compiled with --fmad=false (their float arithmetic must round like
the reference's); host code everywhere with -ffp-contract=off.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libnbnxm_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I", os.path.join(os.path.dirname(HERE), "include")]
# translation unit -> extra flags
UNITS = {
    "nbx_grid.cu": ["--fmad=false"],
    "nbx_search.cu": ["--fmad=false"],
    "nbx_prune.cu": ["--fmad=false"],
    "nbx_force.cu": [],
    "nbx_force_x2.cu": [],
    "nbx_batch.cu": [],
    "nbx_batch_x2.cu": [],
    "nbx_adjoint.cu": [],
    "nbx_balance.cu": [],
    "nbx_api.cu": [],
    "nbx_pme.cu": [],
    "nbx_md.cu": [],
    "nbx_fep.cu": [],
    "nbx_fft.cu": [],
}


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(os.path.join(LIBDIR, "obj"), exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "nbnxm_gb300.h"))
    objs = []
    jobs = []
    for unit, extra in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(LIBDIR, "obj", unit.replace(".cu", ".o"))
        objs.append(obj)
        if force or not _newer(obj, [src] + headers + [__file__]):
            jobs.append([nvcc(), *ARCH, *COMMON, *extra, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            print(r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-cudart", "static"])
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=False))
