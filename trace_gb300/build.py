"""Build the trace_gb300 CUDA library in-tree.

``python -m trace_gb300.build`` compiles ``csrc/*.cu`` for sm_103a with nvcc
(one -gencode, translation units in parallel) and links
``trace_gb300/_build/libtrace_gb300.so``. nvcc cross-compiles, so this works
on a host without a GPU.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libtrace_gb300.so")
SOURCES = ["tg_trace.cu", "tg_forward.cu", "tg_backward.cu", "tg_backward_k4.cu", "tg_backward_k8.cu", "tg_backward_k16.cu", "tg_backward_staged.cu", "tg_iter.cu", "tg_fp64.cu", "tg_tiles.cu", "tg_plan.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _flags(extra=()):
    return [*ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
            "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", *extra]


def _compile(src: str, extra=()) -> str:
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *_flags(extra), "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


DRIVER = os.path.join(OUT, "trace_recon")


def build_driver() -> str:
    """The C++ reconstruction driver over the drop-in classes."""
    src = os.path.join(HERE, "host", "trace_recon.cc")
    hdr = os.path.join(HERE, "host", "trace_gb300.hpp")
    if (os.path.exists(DRIVER) and os.path.getmtime(DRIVER) > max(
            os.path.getmtime(src), os.path.getmtime(hdr), os.path.getmtime(LIB))):
        return DRIVER
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", src, "-o", DRIVER, f"-L{OUT}",
           "-ltrace_gb300", f"-Wl,-rpath,{OUT}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")
    return DRIVER


def build(verbose: bool = False, extra=()) -> str:
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "trace_gb300.h"))
    if os.path.exists(LIB) and not extra:
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) < t for d in deps):
            build_driver()
            return LIB
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_driver()
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=tuple(sys.argv[1:]))
