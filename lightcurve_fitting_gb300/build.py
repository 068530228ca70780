"""Build liblcf_gb300.so in-tree with nvcc for sm_103a.

Eight translation units are compiled in parallel (pso, polish, finalize,
plain, joint, likelihood, compat, host) and linked into lightcurve_fitting_gb300/liblcf_gb300.so with the CUDA runtime
linked statically.  No cmake; objects go to lightcurve_fitting_gb300/_build/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblcf_gb300.so")
SOURCES = ["pso.cu", "polish.cu", "finalize.cu", "plain.cu", "joint.cu", "likelihood.cu", "compat.cu", "host.cu"]
# Units whose FP32 arithmetic (the swarms, SVI and the joint swarm) uses nvcc's
# fast single-precision forms: SFU exp / log, approximate division and square
# root, denormals flushed.  FP64 arithmetic is unaffected by the flag.  The
# likelihood API (likelihood.cu), the refinement scans (finalize.cu) and the
# plain form keep the accurate library forms.
FAST_MATH = {"pso.cu", "polish.cu", "joint.cu"}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblcf_gb300.so")


def _needs_build(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    deps.append(os.path.join(ROOT, "include", "lcf.h"))
    deps.append(os.path.abspath(__file__))  # compiler flags
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]
    if verbose:
        flags += ["-Xptxas", "-v"]
    jobs = []
    objs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _needs_build(obj, src):
            extra = ["--use_fast_math"] if s in FAST_MATH else []
            jobs.append([cc, *flags, *extra, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for out in ex.map(run, jobs):
            if verbose and out:
                print(out)
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        run([cc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
