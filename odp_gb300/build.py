"""Builds libodp_gb300 (shared and static) for sm_103a, in-tree.

    python -m odp_gb300.build            # or: python odp_gb300/build.py

Outputs odp_gb300/libodp_gb300.so and odp_gb300/libodp_gb300.a; objects go to
odp_gb300/_build/, with serve_load, a native client of the serving API that
bench.py drives (linked against the shared library, not part of it).  The CUDA translation unit is compiled with
`-gencode arch=compute_103a,code=sm_103a`; host C files with gcc.  The shared
library links the CUDA runtime statically, so loading it needs only the
driver (libcuda).
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc") if os.path.exists(os.path.join(CUDA_HOME, "bin", "nvcc")) else "nvcc"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["aspl_engine.cu", "anneal.cu"]
C_SOURCES = ["odp_graph.c", "odp_io.c", "odp_plan.c", "odp_aspl.c", "odp_batch.c", "odp_serve.c", "odp_anneal.c"]

SO_PATH = os.path.join(HERE, "libodp_gb300.so")
A_PATH = os.path.join(HERE, "libodp_gb300.a")
# a native client of the serving API that bench.py drives (not part of the library)
SERVE_LOAD = os.path.join(BUILD, "serve_load")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _obj(src):
    return os.path.join(BUILD, os.path.splitext(src)[0] + ".o")


def _compile(src, verbose_ptxas=False):
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [NVCC, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-I", INCLUDE, "-I", CSRC, "-c", path, "-o", _obj(src)]
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = ["gcc", "-O3", "-std=gnu11", "-fPIC", "-Wall", "-Wno-unused-function",
               "-I", INCLUDE, "-I", CSRC, "-c", path, "-o", _obj(src)]
    return _run(cmd)


def build(verbose_ptxas=False):
    """Compile and link; returns the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    sources = [s for s in CU_SOURCES + C_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with ThreadPoolExecutor(max_workers=8) as ex:
        logs = list(ex.map(lambda s: _compile(s, verbose_ptxas), sources))
    objs = [_obj(s) for s in sources]
    tmp_so = SO_PATH + ".tmp"
    _run([NVCC, ARCH, "-shared", "-cudart", "static", "-o", tmp_so] + objs + ["-lm", "-lpthread"])
    os.replace(tmp_so, SO_PATH)
    if os.path.exists(A_PATH):
        os.remove(A_PATH)
    _run(["ar", "rcs", A_PATH] + objs)
    _run(["gcc", "-O2", "-std=gnu11", "-Wall", "-I", INCLUDE, "-o", SERVE_LOAD, os.path.join(CSRC, "serve_load.c"),
          "-L", HERE, "-lodp_gb300", "-Wl,-rpath,$ORIGIN/..", "-lpthread", "-lm"])
    if verbose_ptxas:
        sys.stdout.write("".join(logs))
    return SO_PATH


def clean():
    shutil.rmtree(BUILD, ignore_errors=True)
    for p in (SO_PATH, A_PATH):
        if os.path.exists(p):
            os.remove(p)


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv))
