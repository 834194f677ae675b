"""TEST INFRASTRUCTURE ONLY -- the oracle for the ODP ASPL hot path.

Two checkers live here; the product (odp_gb300) never imports this package.

* ``aspl_oracle.c``: a CPU restatement of the reference's bitset-matrix ASPL
  (aspl.c:35-119, utils.c:1815-1996), built by :func:`build` into
  ``oracle/_build/liboracle.so`` and called through :func:`aspl`.  It runs
  anywhere gcc does, including the GPU host.
* ``oracle/_ref/``: the reference CPU library itself (libodp.a /
  libodp_threads.a) compiled by ``oracle/Makefile`` from the reference's own
  sources, as ``baseline/install_ref.sh`` installs them into
  ``baseline/_ref/src`` (git-ignored, so they travel with the working tree),
  driven through ``ref_driver``.  Used to pin the restatement and to generate
  the committed golden fixtures.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
ROOT = os.path.dirname(HERE)
REF_SOURCE = os.path.join(ROOT, "baseline", "_ref", "src")

KIND_DEFAULT, KIND_MATRIX, KIND_SAVING = 0, 1, 2


def build(force=False):
    """Compiles the restatement (and the reference, when its tree is here)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "aspl_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        tmp = LIB + ".tmp"
        subprocess.run(["gcc", "-O3", "-std=gnu11", "-fopenmp", "-fPIC", "-shared", "-o", tmp, src],
                       check=True)
        os.replace(tmp, LIB)
    import sys
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import baseline
    baseline.install()
    if baseline.sources_present():
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + REF_SOURCE], check=True,
                       stdout=subprocess.DEVNULL)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        lib = ctypes.CDLL(LIB)
        lib.oracle_new.restype = ctypes.c_void_p
        lib.oracle_new.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                   ctypes.c_int, ctypes.c_int]
        lib.oracle_set.restype = None
        lib.oracle_set.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                   ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_double)]
        lib.oracle_free.restype = None
        lib.oracle_free.argtypes = [ctypes.c_void_p]
        lib.oracle_kind.restype = ctypes.c_int
        lib.oracle_kind.argtypes = [ctypes.c_void_p]
        lib.oracle_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


class Oracle:
    """One Init / many Set / Finalize, like the reference API."""

    def __init__(self, nodes=0, degree=0, num_degrees=None, symmetries=1, grid=False, width=0, height=0,
                 kind=KIND_DEFAULT):
        self._nd = None if num_degrees is None else np.ascontiguousarray(num_degrees, dtype=np.int32)
        first = width if grid else nodes
        self._h = load().oracle_new(int(grid), first, height, degree,
                                    self._nd.ctypes.data if self._nd is not None else None, symmetries, kind)
        if not self._h:
            raise ValueError("invalid oracle shape")

    def set(self, adjacency):
        adj = np.ascontiguousarray(adjacency, dtype=np.int32)
        d, s, a = ctypes.c_int(), ctypes.c_long(), ctypes.c_double()
        load().oracle_set(self._h, adj.ctypes.data, ctypes.byref(d), ctypes.byref(s), ctypes.byref(a))
        return d.value, s.value, a.value

    @property
    def kind(self):
        return load().oracle_kind(self._h)

    def close(self):
        if self._h:
            load().oracle_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def aspl(adjacency, nodes=0, degree=None, num_degrees=None, symmetries=1, grid=False, width=0, height=0,
         kind=KIND_DEFAULT):
    """(diameter, sum, ASPL) of one graph, as ODP_Set_aspl returns them."""
    adjacency = np.ascontiguousarray(adjacency, dtype=np.int32)
    if degree is None:
        degree = adjacency.shape[1]
    o = Oracle(nodes, degree, num_degrees, symmetries, grid, width, height, kind)
    try:
        return o.set(adjacency)
    finally:
        o.close()


def threads():
    return load().oracle_threads()


# ---- the reference library itself (only where its tree was present) ----

def ref_driver(threads=False):
    path = os.path.join(REF_DIR, "ref_driver_threads" if threads else "ref_driver")
    return path if os.path.exists(path) else None


def ref_available():
    return ref_driver() is not None and os.path.isdir(REF_SOURCE)
