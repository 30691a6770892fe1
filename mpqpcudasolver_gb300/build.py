"""In-tree build of libmpqp_gb300.so for sm_103a (nvcc, no cmake).

The two translation units compile in parallel; the shared library lands
next to this file so the Python front end and the tests load it from the
source tree.  Flags: -fmad=false keeps every multiply-add the explicit fma
written in the source (the FP64 kernels follow the CPU oracle's operation
order); host code is built with -ffp-contract=off for the same reason.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmpqp_gb300.so")
SOURCES = ["mpqp_kernels.cu", "mpqp_engine.cu", "mpqp_noalloc.cu", "mpqp_preprocess.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-I", os.path.join(HERE, "..", "include"), *extra]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    headers.append(os.path.join(HERE, "..", "include", "mpqp_gb300.h"))
    objs = []
    jobs = []
    for src in SOURCES:
        sp = os.path.join(CSRC, src)
        op = os.path.join(BUILD, src + ".o")
        objs.append(op)
        if force or _stale(op, [sp] + headers):
            extra = ["-Xptxas", "-v"] if ptxas_v else []
            jobs.append([nvcc(), *_flags(extra), "-c", sp, "-o", op])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0 or verbose:
            print(" ".join(cmd))
            print(r.stdout[-20000:], r.stderr[-20000:])
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        logs = list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            print(" ".join(cmd)); print(r.stdout, r.stderr)
            raise RuntimeError("link failed")
        os.replace(LIB + ".tmp", LIB)
    if ptxas_v:
        return "\n".join(logs)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True, ptxas_v="-v" in sys.argv))
