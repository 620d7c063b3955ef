"""Build recipe of oracle/_ref/libsbref.so: the reference's own step code
(kernel/bubble.cu, solver.cu, quantity.cu, initializer.cu, timer.cu of
RiverIntheSky/SoapBubble) compiled for host execution, as test
infrastructure that pins the FP64 oracle.

The sources are read where they lie (the reference checkout, default
/root/reference, or $SBREF_SOURCE) and written to oracle/_ref/src/ with two
mechanical changes a host compiler needs: every kernel launch
`k<<<grid, block>>>(args)` becomes `sbref::Launcher(grid, block).bind(&k)(args)`
(shim/cuda_runtime.h runs the grid on the host), and solver.cu's include of
the vendored OpenCV headers points at the shim's opencv2/opencv.hpp.  The
CUDA runtime, AmgX, Boost.Filesystem and OpenCV calls resolve to the shims
in oracle/ref/ (shim/, shim_runtime.cpp, ref_amgx.cpp); nothing of the
reference's build system is used.  Outputs go to oracle/_ref/ only.

    python oracle/ref/build_ref.py      # builds when the checkout is present
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
SRC_OUT = os.path.join(OUT, "src")
LIB = os.path.join(OUT, "libsbref.so")
# variants of the reference's compile-time switches (include/header.cuh:89-98)
# that a command-line definition can turn on: VISCOUS is off in the header
VARIANTS = {"default": [], "viscous": ["-DVISCOUS"]}


def lib_path(variant: str = "default") -> str:
    return LIB if variant == "default" else os.path.join(OUT, f"libsbref_{variant}.so")
SOURCES = ["bubble.cu", "solver.cu", "quantity.cu", "initializer.cu", "timer.cu"]
LAUNCH = re.compile(r"(\w+)\s*<<<(.*?)>>>", re.S)


def reference_dir() -> str:
    return os.environ.get("SBREF_SOURCE", "/root/reference")


def available() -> bool:
    ref = reference_dir()
    return all(os.path.exists(os.path.join(ref, "kernel", f)) for f in SOURCES)


def rewrite(text: str) -> str:
    text = LAUNCH.sub(lambda m: f"sbref::Launcher({m.group(2)}).bind(&{m.group(1)})", text)
    return text.replace('"../opencv_headers/opencv2/opencv.hpp"', "<opencv2/opencv.hpp>")


def _run(cmd):
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"failed: {' '.join(cmd)}\n{out.stdout[-4000:]}\n{out.stderr[-8000:]}")


def build(force: bool = False, variant: str = "default") -> str:
    lib = lib_path(variant)
    if not available():
        raise FileNotFoundError(f"reference sources not found under {reference_dir()}")
    ref = reference_dir()
    os.makedirs(SRC_OUT, exist_ok=True)
    own = [os.path.join(HERE, f) for f in ("ref_driver.cpp", "ref_amgx.cpp", "shim_runtime.cpp")]
    deps = own + [os.path.join(HERE, "shim", f) for f in os.listdir(os.path.join(HERE, "shim"))
                  if f.endswith(".h")] + [os.path.abspath(__file__)]
    deps += [os.path.join(ref, "kernel", f) for f in SOURCES]
    if not force and os.path.exists(lib) and all(os.path.getmtime(d) <= os.path.getmtime(lib)
                                                 for d in deps if os.path.exists(d)):
        return lib
    for f in SOURCES:
        with open(os.path.join(ref, "kernel", f)) as fh:
            text = rewrite(fh.read())
        with open(os.path.join(SRC_OUT, f + ".cpp"), "w") as fh:
            fh.write(text)
    flags = ["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-w", "-ffp-contract=off",
             *VARIANTS[variant],
             "-I", os.path.join(HERE, "shim"), "-I", HERE, "-I", os.path.join(ref, "kernel"),
             "-I", os.path.join(ref, "include"), "-I", os.path.join(ref, "cuda_util_headers")]
    units = [(os.path.join(HERE, "ref_driver.cpp"),
              [f'-DSBREF_BUBBLE_CU="{os.path.join(SRC_OUT, "bubble.cu.cpp")}"']),
             (os.path.join(HERE, "ref_amgx.cpp"), []),
             (os.path.join(HERE, "shim_runtime.cpp"), [])]
    units += [(os.path.join(SRC_OUT, f + ".cpp"), []) for f in SOURCES if f != "bubble.cu"]
    objs = []

    def compile_one(u):
        src, extra = u
        obj = os.path.join(OUT, f"{variant}.{os.path.basename(src)}.o")
        _run(flags + extra + ["-c", src, "-o", obj])
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(compile_one, units))
    _run(["g++", "-shared", "-fopenmp", "-Wl,-Bsymbolic", "-o", lib] + objs)
    return lib


if __name__ == "__main__":
    for v in VARIANTS:
        print(build(force="--force" in sys.argv, variant=v))
