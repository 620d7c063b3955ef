"""Build recipe of libsoapbubble_gb300.so (sm_103a) and the soapBubble CLI.

Each translation unit is compiled by nvcc in parallel into _build/, then
linked into a shared library with a C ABI (include/soapbubble.h).  No cmake;
one -gencode, so a build takes well under a minute.
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
LIB = os.path.join(BUILD, "libsoapbubble_gb300.so")
CLI = os.path.join(BUILD, "soapBubble")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"), "-I", CSRC]

LIB_SOURCES = ["sb_step.cu", "sb_solver.cu", "sb_api.cu", "sb_exr.cpp", "sb_noalloc.cu"]
# The implicit solve is compiled without multiply-add contraction: the solver
# kernel is instantiated per row width of the largest system it serves, and
# contraction choices may differ between instantiations, while a bubble must
# get bit-identical results alone and inside any batch.
EXTRA_FLAGS = {"sb_solver.cu": ["-fmad=false"],
               # texture resampling: the same float rounding on x86 and Arm hosts
               "sb_exr.cpp": ["-Xcompiler", "-ffp-contract=off"]}
CLI_SOURCES = ["sb_bubble.cpp", "sb_main.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra=()) -> str:
    obj = os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0] + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *EXTRA_FLAGS.get(src, []), *extra, "-c",
           os.path.join(CSRC, src), "-o", obj]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{out.stdout}\n{out.stderr}")
    return obj


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _all_sources():
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(ROOT, "include", "soapbubble.h"))
    deps.append(os.path.abspath(__file__))
    return deps


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link; returns the library path.  Skips up-to-date builds."""
    os.makedirs(BUILD, exist_ok=True)
    deps = _all_sources()
    if not force and _newer(LIB, deps) and _newer(CLI, deps):
        return LIB
    srcs = LIB_SOURCES + CLI_SOURCES
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = dict(zip(srcs, ex.map(_compile, srcs)))
    lib_objs = [objs[s] for s in LIB_SOURCES]
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *lib_objs, "-lcudart"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{out.stdout}\n{out.stderr}")
    cmd = [nvcc(), *ARCH, "-o", CLI, objs["sb_bubble.cpp"], objs["sb_main.cpp"], *lib_objs,
           "-lcudart"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"CLI link failed: {' '.join(cmd)}\n{out.stdout}\n{out.stderr}")
    if verbose:
        print("built", LIB, "and", CLI)
    return LIB


def ptxas_report(src: str = "sb_step.cu") -> str:
    """Register / spill report of one translation unit (-Xptxas -v)."""
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *EXTRA_FLAGS.get(src, []), "-Xptxas", "-v", "-c",
           os.path.join(CSRC, src), "-o", os.devnull]
    out = subprocess.run(cmd, capture_output=True, text=True)
    return out.stdout + out.stderr


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "ptxas":
        print(ptxas_report(sys.argv[2] if len(sys.argv) > 2 else "sb_step.cu"))
    else:
        print(build(force="--force" in sys.argv, verbose=True))
