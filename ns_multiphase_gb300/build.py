"""Build of the sm_103a shared library ``_build/libslvof.so`` (in-tree, no cmake).

Each translation unit is compiled by nvcc in parallel.  The FP64 and shared kernels are
compiled with ``-fmad=false`` so that their arithmetic rounds exactly like the reference's
(and the CPU restatement's) expression order; the mixed-precision kernels keep FMA.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libslvof.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr", "-I", CSRC,
          "-I", INCLUDE]
UNITS = {
    "slvof_api.cu": ["-fmad=false"],
    "k_common.cu": ["-fmad=false"],
    "k_fp64.cu": ["-fmad=false"],
    "k_mixed.cu": ["-fmad=true"],
    "k_elvira_mixed.cu": ["-fmad=false"],
    "slvof_noalloc.cu": ["-fmad=false"],
    "k_adj64.cu": ["-fmad=false"],
    "k_adj32.cu": ["-fmad=true"],
}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the SL-VOF library needs the CUDA toolkit to build")


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "slvof.h"), __file__]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    extra = extra or []

    def compile_one(name):
        obj = os.path.join(OUT, name.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *COMMON, *UNITS[name], *extra, "-c", os.path.join(CSRC, name), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS))
    tmp = LIB + ".tmp"
    r = subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose=True, extra=sys.argv[1:]))
