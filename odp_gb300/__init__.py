"""odp_gb300 -- Python host interface to libodp_gb300, the GB300 ODP library.

The C library is the product: the drop-in ``odp.h`` API (ODP_Init_aspl_*,
ODP_Set_aspl, ODP_Finalize_aspl and the graph utilities) plus the batch and
serving extensions of ``include/odp_gb300.h``.  This module binds those C
entry points with ctypes and mirrors them with the same names, argument
meaning and error behaviour, so tests and benchmarks read like the
reference's own sample programs (sample/general.c, sample/grid.c).

Loading fails loudly when the shared library has not been built (there is no
CPU fallback): run ``python -m odp_gb300.build`` or ``__graft_entry__.build()``.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libodp_gb300.so")

OK, ERR_INVALID, ERR_CUDA, ERR_ADJACENCY, ERR_TIMEOUT, ERR_MEMORY, ERR_STATE = range(7)
_ERR_NAMES = {1: "invalid shape", 2: "CUDA error", 3: "adjacency out of range",
              4: "device wait timed out", 5: "over memory budget", 6: "call out of order"}

INT_MAX = 2**31 - 1
LONG_MAX = 2**63 - 1


class ODPError(RuntimeError):
    def __init__(self, code, what=""):
        super().__init__("%s failed: %s (code %d)" % (what, _ERR_NAMES.get(code, "error"), code))
        self.code = code


class Restore(ctypes.Structure):
    """ODP_Restore (odp.h): the four adjacency slots a 2-opt swap rewrote."""
    _fields_ = [("u", ctypes.c_int * 2), ("v", ctypes.c_int * 2),
                ("u_d", ctypes.c_int * 2), ("v_d", ctypes.c_int * 2)]


class Graph(ctypes.Structure):
    """ODP_Graph (odp_gb300.h): one graph of a batch."""
    _fields_ = [("grid", ctypes.c_int), ("nodes", ctypes.c_int), ("width", ctypes.c_int),
                ("height", ctypes.c_int), ("degree", ctypes.c_int), ("symmetries", ctypes.c_int),
                ("num_degrees", ctypes.POINTER(ctypes.c_int)), ("adjacency", ctypes.POINTER(ctypes.c_int))]


_lib = None


def load():
    """Loads libodp_gb300.so (once); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libodp_gb300.so is not built (expected at %s); "
                          "run `python -m odp_gb300.build`" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    I = ctypes.c_int
    IP = ctypes.POINTER(ctypes.c_int)
    sig = {
        "ODP_Init_aspl_general": (None, [I, I, P]),
        "ODP_Init_aspl_general_s": (None, [I, I, P, I]),
        "ODP_Init_aspl_grid": (None, [I, I, I, P]),
        "ODP_Init_aspl_grid_s": (None, [I, I, I, P, I]),
        "ODP_Set_aspl": (None, [P, IP, ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_double)]),
        "ODP_Finalize_aspl": (None, []),
        "ODP_Srand": (None, [ctypes.c_uint]),
        "ODP_Generate_random_general": (None, [I, I, P]),
        "ODP_Generate_random_general_s": (None, [I, I, I, P]),
        "ODP_Generate_random_grid": (None, [I, I, I, I, P]),
        "ODP_Generate_random_grid_s": (None, [I, I, I, I, I, P]),
        "ODPX_Generate_random_general_seeded": (None, [ctypes.c_uint, I, I, I, P]),
        "ODPX_Generate_random_grid_seeded": (None, [ctypes.c_uint, I, I, I, I, I, P]),
        "ODP_Conv_edge2adjacency_general": (None, [I, I, I, P, P]),
        "ODP_Conv_edge2adjacency_general_s": (None, [I, I, I, P, I, P]),
        "ODP_Conv_edge2adjacency_grid": (None, [I, I, I, I, P, P]),
        "ODP_Conv_edge2adjacency_grid_s": (None, [I, I, I, I, P, I, P]),
        "ODP_Set_lbounds_general": (None, [I, I, IP, ctypes.POINTER(ctypes.c_double)]),
        "ODP_Set_lbounds_grid": (None, [I, I, I, I, IP, ctypes.POINTER(ctypes.c_double)]),
        "ODP_Conv_adjacency2edge_general": (None, [I, I, P, P, P]),
        "ODP_Conv_adjacency2edge_general_s": (None, [I, I, P, P, I, P]),
        "ODP_Conv_adjacency2edge_grid": (None, [I, I, I, P, P, P]),
        "ODP_Conv_adjacency2edge_grid_s": (None, [I, I, I, P, P, I, P]),
        "ODP_Mutate_adjacency_general": (None, [I, I, P, ctypes.POINTER(Restore), P]),
        "ODP_Mutate_adjacency_general_s": (None, [I, I, P, I, ctypes.POINTER(Restore), P]),
        "ODP_Mutate_adjacency_grid": (None, [I, I, I, P, I, ctypes.POINTER(Restore), P]),
        "ODP_Mutate_adjacency_grid_s": (None, [I, I, I, P, I, I, ctypes.POINTER(Restore), P]),
        "ODP_Restore_adjacency_general": (None, [Restore, P]),
        "ODP_Restore_adjacency_grid": (None, [Restore, P]),
        "ODP_Set_aspl_batch": (I, [I, ctypes.POINTER(Graph), IP, ctypes.POINTER(ctypes.c_long),
                                   ctypes.POINTER(ctypes.c_double)]),
        "ODPX_Batch_create": (I, [I, ctypes.POINTER(Graph), ctypes.POINTER(P)]),
        "ODPX_Batch_run": (I, [P, ctypes.POINTER(P), IP, ctypes.POINTER(ctypes.c_long),
                               ctypes.POINTER(ctypes.c_double)]),
        "ODPX_Batch_destroy": (None, [P]),
        "ODPX_Batch_time_mode": (I, [P, ctypes.POINTER(P), I, I, I, ctypes.POINTER(ctypes.c_float)]),
        "ODPX_Batch_tiles": (ctypes.c_ulonglong, [P]),
        "ODPX_Batch_info": (I, [P, I, IP, IP, IP, IP]),
        "ODPX_Batch_job_levels": (I, [P, IP, I]),
        "ODPX_Batch_job_profile": (I, [P, IP, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), I]),
        "ODPX_Batch_set_wait_limit": (None, [P, ctypes.c_ulonglong]),
        "ODPX_Batch_bytes_alg": (ctypes.c_double, [P]),
        "ODPX_Batch_kernel": (I, [P]),
        "ODPX_Batch_small_shape": (I, [P, IP, IP, IP]),
        "ODPX_Measure_l2_read_gbs": (ctypes.c_double, [I, I]),
        "ODPX_Set_tuning": (None, [I, I, I, I, I, I]),
        "ODPX_Current_plan": (P, []),
        "ODPX_Rng_size": (ctypes.c_size_t, []),
        "ODPX_Rng_seed": (None, [P, ctypes.c_uint]),
        "ODPX_Rng_next": (I, [P]),
        "ODPX_Mutate_adjacency_general_s_rng": (None, [P, I, I, P, I, ctypes.POINTER(Restore), P]),
        "ODPX_Restore_adjacency_general_s": (None, [I, I, I, Restore, P]),
        "ODPX_Mutate_adjacency_grid_s_rng": (None, [P, I, I, I, P, I, I, ctypes.POINTER(Restore), P]),
        "ODPX_Restore_adjacency_grid_s": (None, [I, I, I, I, Restore, P]),
        "ODPX_Version": (ctypes.c_char_p, []),
        "ODP_Get_lines": (I, [ctypes.c_char_p]),
        "ODP_Read_edge_general": (None, [ctypes.c_char_p, P]),
        "ODP_Read_edge_grid": (None, [ctypes.c_char_p, IP, IP, P]),
        "ODP_Write_edge_general": (None, [I, P, ctypes.c_char_p]),
        "ODP_Write_edge_grid": (None, [I, I, P, ctypes.c_char_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _iptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _ints(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.int32)
    if shape is not None:
        a = a.reshape(shape)
    return a


def _check(code, what):
    if code != OK:
        raise ODPError(code, what)


# --------------------------------------------------------------------------
# Drop-in ASPL API (odp.h).
# --------------------------------------------------------------------------

def init_aspl_general(nodes, degree, num_degrees=None):
    """ODP_Init_aspl_general."""
    global _nd_keep
    _nd_keep = None if num_degrees is None else _ints(num_degrees)
    load().ODP_Init_aspl_general(nodes, degree, _iptr(_nd_keep))


def init_aspl_general_s(nodes, degree, num_degrees, symmetries):
    """ODP_Init_aspl_general_s."""
    global _nd_keep
    _nd_keep = None if num_degrees is None else _ints(num_degrees)
    load().ODP_Init_aspl_general_s(nodes, degree, _iptr(_nd_keep), symmetries)


def init_aspl_grid(width, height, degree, num_degrees=None):
    """ODP_Init_aspl_grid."""
    global _nd_keep
    _nd_keep = None if num_degrees is None else _ints(num_degrees)
    load().ODP_Init_aspl_grid(width, height, degree, _iptr(_nd_keep))


def init_aspl_grid_s(width, height, degree, num_degrees, symmetries):
    """ODP_Init_aspl_grid_s."""
    global _nd_keep
    _nd_keep = None if num_degrees is None else _ints(num_degrees)
    load().ODP_Init_aspl_grid_s(width, height, degree, _iptr(_nd_keep), symmetries)


_nd_keep = None


def set_aspl(adjacency):
    """ODP_Set_aspl: returns (diameter, sum, ASPL)."""
    adj = _ints(adjacency)
    d = ctypes.c_int()
    s = ctypes.c_long()
    a = ctypes.c_double()
    load().ODP_Set_aspl(_iptr(adj), ctypes.byref(d), ctypes.byref(s), ctypes.byref(a))
    return d.value, s.value, a.value


def finalize_aspl():
    """ODP_Finalize_aspl."""
    load().ODP_Finalize_aspl()


# --------------------------------------------------------------------------
# Graph utilities.
# --------------------------------------------------------------------------

def srand(seed):
    load().ODP_Srand(seed)


def generate_random_general(nodes, degree, symmetries=1, seed=None):
    """Edge list int32[nodes*degree/2][2] from ODP_Generate_random_general(_s).

    With ``seed`` the private stream is used (same graph as ODP_Srand(seed)
    followed by the generator); without, the libc rand() stream."""
    lines = nodes * degree // 2
    edge = np.zeros((lines, 2), dtype=np.int32)
    lib = load()
    if seed is not None:
        lib.ODPX_Generate_random_general_seeded(seed, nodes, degree, symmetries, _iptr(edge))
    elif symmetries == 1:
        lib.ODP_Generate_random_general(nodes, degree, _iptr(edge))
    else:
        lib.ODP_Generate_random_general_s(nodes, degree, symmetries, _iptr(edge))
    return edge


def generate_random_grid(width, height, degree, length, symmetries=1, seed=None):
    """Edge list from ODP_Generate_random_grid(_s) (vertex id = x*height + y)."""
    lines = width * height * degree // 2
    edge = np.zeros((lines, 2), dtype=np.int32)
    lib = load()
    if seed is not None:
        lib.ODPX_Generate_random_grid_seeded(seed, width, height, degree, length, symmetries, _iptr(edge))
    elif symmetries == 1:
        lib.ODP_Generate_random_grid(width, height, degree, length, _iptr(edge))
    else:
        lib.ODP_Generate_random_grid_s(width, height, degree, length, symmetries, _iptr(edge))
    return edge


def conv_edge2adjacency_general(nodes, edge, degree, symmetries=1):
    """ODP_Conv_edge2adjacency_general(_s): int32[nodes/s][degree], -1 padded."""
    edge = _ints(edge)
    adj = np.zeros((nodes // symmetries, degree), dtype=np.int32)
    load().ODP_Conv_edge2adjacency_general_s(nodes, len(edge), degree, _iptr(edge), symmetries, _iptr(adj))
    return adj


def set_lbounds_general(nodes, degree):
    """ODP_Set_lbounds_general: (low_diameter, low_ASPL), the Moore bound."""
    d, a = ctypes.c_int(), ctypes.c_double()
    load().ODP_Set_lbounds_general(nodes, degree, ctypes.byref(d), ctypes.byref(a))
    return d.value, a.value


def set_lbounds_grid(width, height, degree, length):
    """ODP_Set_lbounds_grid: (low_diameter, low_ASPL), the lattice bound."""
    d, a = ctypes.c_int(), ctypes.c_double()
    load().ODP_Set_lbounds_grid(width, height, degree, length, ctypes.byref(d), ctypes.byref(a))
    return d.value, a.value


def get_lines(fname):
    """ODP_Get_lines: newline characters in the file."""
    return int(load().ODP_Get_lines(os.fsencode(fname)))


def read_edge_general(fname):
    """ODP_Read_edge_general: int32[lines][2] (lines = ODP_Get_lines)."""
    lines = get_lines(fname)
    edge = np.zeros((max(lines, 1), 2), dtype=np.int32)
    load().ODP_Read_edge_general(os.fsencode(fname), _iptr(edge))
    return edge[:lines]


def read_edge_grid(fname):
    """ODP_Read_edge_grid: (width, height, int32[lines][2])."""
    lines = get_lines(fname)
    edge = np.zeros((max(lines, 1), 2), dtype=np.int32)
    w, h = ctypes.c_int(), ctypes.c_int()
    load().ODP_Read_edge_grid(os.fsencode(fname), ctypes.byref(w), ctypes.byref(h), _iptr(edge))
    return w.value, h.value, edge[:lines]


def write_edge_general(edge, fname):
    edge = _ints(edge)
    load().ODP_Write_edge_general(len(edge), _iptr(edge), os.fsencode(fname))


def write_edge_grid(edge, height, fname):
    edge = _ints(edge)
    load().ODP_Write_edge_grid(len(edge), height, _iptr(edge), os.fsencode(fname))


def conv_edge2adjacency_grid(width, height, edge, degree, symmetries=1):
    """ODP_Conv_edge2adjacency_grid(_s): int32[w*h/s][degree], -1 padded."""
    edge = _ints(edge)
    adj = np.zeros((width * height // symmetries, degree), dtype=np.int32)
    load().ODP_Conv_edge2adjacency_grid_s(width, height, len(edge), degree, _iptr(edge), symmetries, _iptr(adj))
    return adj


def conv_adjacency2edge_general(nodes, degree, adjacency, symmetries=1, num_degrees=None):
    adj = _ints(adjacency)
    nd = None if num_degrees is None else _ints(num_degrees)
    total = nodes * degree if nd is None else int(np.sum(nd)) * symmetries
    edge = np.zeros((total // 2, 2), dtype=np.int32)
    load().ODP_Conv_adjacency2edge_general_s(nodes, degree, _iptr(nd), _iptr(adj), symmetries, _iptr(edge))
    return edge


def conv_adjacency2edge_grid(width, height, degree, adjacency, symmetries=1, num_degrees=None):
    adj = _ints(adjacency)
    nd = None if num_degrees is None else _ints(num_degrees)
    nodes = width * height
    total = nodes * degree if nd is None else int(np.sum(nd)) * symmetries
    edge = np.zeros((total // 2, 2), dtype=np.int32)
    load().ODP_Conv_adjacency2edge_grid_s(width, height, degree, _iptr(nd), _iptr(adj), symmetries, _iptr(edge))
    return edge


def mutate_adjacency_general(nodes, degree, adjacency, symmetries=1, num_degrees=None):
    """ODP_Mutate_adjacency_general(_s) in place; returns the Restore record."""
    r = Restore()
    nd = None if num_degrees is None else _ints(num_degrees)
    load().ODP_Mutate_adjacency_general_s(nodes, degree, _iptr(nd), symmetries, ctypes.byref(r), _iptr(adjacency))
    return r


def mutate_adjacency_grid(width, height, degree, length, adjacency, symmetries=1, num_degrees=None):
    r = Restore()
    nd = None if num_degrees is None else _ints(num_degrees)
    load().ODP_Mutate_adjacency_grid_s(width, height, degree, _iptr(nd), length, symmetries, ctypes.byref(r),
                                       _iptr(adjacency))
    return r


def restore_adjacency_general(r, adjacency):
    load().ODP_Restore_adjacency_general(r, _iptr(adjacency))


def restore_adjacency_grid(r, adjacency):
    load().ODP_Restore_adjacency_grid(r, _iptr(adjacency))


class Rng:
    """A private glibc-compatible random stream (ODPX_Rng_*)."""

    def __init__(self, seed):
        self._buf = ctypes.create_string_buffer(int(load().ODPX_Rng_size()))
        load().ODPX_Rng_seed(self._buf, seed)

    def next(self):
        return load().ODPX_Rng_next(self._buf)

    @property
    def state(self):
        return self._buf

    def mutate_general(self, nodes, degree, adjacency, symmetries=1, num_degrees=None):
        r = Restore()
        nd = None if num_degrees is None else _ints(num_degrees)
        load().ODPX_Mutate_adjacency_general_s_rng(self._buf, nodes, degree, _iptr(nd), symmetries,
                                                   ctypes.byref(r), _iptr(adjacency))
        return r

    @staticmethod
    def restore_general(nodes, degree, r, adjacency, symmetries=1):
        """Undoes a swap of mutate_general (the shape is given explicitly)."""
        load().ODPX_Restore_adjacency_general_s(nodes, degree, symmetries, r, _iptr(adjacency))

    def mutate_grid(self, width, height, degree, length, adjacency, symmetries=1, num_degrees=None):
        r = Restore()
        nd = None if num_degrees is None else _ints(num_degrees)
        load().ODPX_Mutate_adjacency_grid_s_rng(self._buf, width, height, degree, _iptr(nd), length, symmetries,
                                                ctypes.byref(r), _iptr(adjacency))
        return r

    @staticmethod
    def restore_grid(width, height, degree, r, adjacency, symmetries=1):
        """Undoes a swap of mutate_grid."""
        load().ODPX_Restore_adjacency_grid_s(width, height, degree, symmetries, r, _iptr(adjacency))


# --------------------------------------------------------------------------
# Batch API (odp_gb300.h).
# --------------------------------------------------------------------------

class GraphSpec:
    """One graph of a batch: the ODP_Init_aspl_* arguments and an adjacency."""

    def __init__(self, adjacency, nodes=0, degree=None, symmetries=1, num_degrees=None,
                 grid=False, width=0, height=0):
        self.grid = bool(grid)
        self.nodes = width * height if grid else nodes
        self.width, self.height = width, height
        self.symmetries = symmetries
        self.adjacency = _ints(adjacency)
        self.degree = self.adjacency.shape[1] if degree is None else degree
        self.num_degrees = None if num_degrees is None else _ints(num_degrees)

    def to_c(self):
        g = Graph()
        g.grid = int(self.grid)
        g.nodes = self.nodes
        g.width, g.height = self.width, self.height
        g.degree = self.degree
        g.symmetries = self.symmetries
        g.num_degrees = (self.num_degrees.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
                         if self.num_degrees is not None else None)
        g.adjacency = self.adjacency.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        return g


_batch_cache = [None]          # (specs, their adjacency and degree arrays, the ODP_Graph array)


def _results(d, s, a):
    return list(zip(d.tolist(), s.tolist(), a.tolist()))


def set_aspl_batch(specs):
    """ODP_Set_aspl_batch: list of (diameter, sum, ASPL), one per spec."""
    n = len(specs)
    # The ODP_Graph array is rebuilt only when a spec or one of its arrays is
    # replaced (identity checks; the cache holds references, so the arrays
    # the pointers name stay alive).
    c = _batch_cache[0]
    if (c is None or len(c[0]) != n or
            not all(x is y and x.adjacency is ay and x.num_degrees is dy
                    for x, y, ay, dy in zip(specs, c[0], c[1], c[2]))):
        specs = list(specs)
        c = (specs, [s.adjacency for s in specs], [s.num_degrees for s in specs],
             (Graph * n)(*[s.to_c() for s in specs]))
        _batch_cache[0] = c
    arr = c[3]
    d = np.zeros(n, dtype=np.int32)
    s = np.zeros(n, dtype=np.int64)
    a = np.zeros(n, dtype=np.float64)
    rc = load().ODP_Set_aspl_batch(n, arr, d.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                   s.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                                   a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    _check(rc, "ODP_Set_aspl_batch")
    return _results(d, s, a)


class Batch:
    """A reusable batch plan (ODPX_Batch_*): fixed shapes, new adjacency per run."""

    def __init__(self, specs):
        self.specs = list(specs)
        n = len(self.specs)
        arr = (Graph * n)(*[s.to_c() for s in self.specs])
        h = ctypes.c_void_p()
        _check(load().ODPX_Batch_create(n, arr, ctypes.byref(h)), "ODPX_Batch_create")
        self._h = h
        self.count = n

    def _adj_ptrs(self, adjacency=None):
        if adjacency is None:
            # the specs' own arrays: their pointers are taken once
            if getattr(self, "_own_ptrs", None) is None or any(
                    x.adjacency is not y for x, y in zip(self.specs, self._own_arrays)):
                self._own_arrays = [s.adjacency for s in self.specs]
                self._own_ptrs = (ctypes.c_void_p * self.count)(*[a.ctypes.data for a in self._own_arrays])
            return self._own_ptrs
        self._keep = [_ints(a) for a in adjacency]
        return (ctypes.c_void_p * self.count)(*[a.ctypes.data for a in self._keep])

    def run(self, adjacency=None):
        n = self.count
        d = np.zeros(n, dtype=np.int32)
        s = np.zeros(n, dtype=np.int64)
        a = np.zeros(n, dtype=np.float64)
        rc = load().ODPX_Batch_run(self._h, self._adj_ptrs(adjacency), d.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                   s.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                                   a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        _check(rc, "ODPX_Batch_run")
        return _results(d, s, a)

    def time(self, repeats, mode=1, flush_mb=0, adjacency=None):
        """Average device ms per run (CUDA events on the plan's stream)."""
        ms = ctypes.c_float()
        rc = load().ODPX_Batch_time_mode(self._h, self._adj_ptrs(adjacency), repeats, mode, flush_mb,
                                         ctypes.byref(ms))
        _check(rc, "ODPX_Batch_time_mode")
        return ms.value

    def tiles(self):
        return int(load().ODPX_Batch_tiles(self._h))

    def info(self, graph=0):
        v = [ctypes.c_int() for _ in range(4)]
        _check(load().ODPX_Batch_info(self._h, graph, *[ctypes.byref(x) for x in v]), "ODPX_Batch_info")
        return dict(njobs=v[0].value, nslots=v[1].value, wc_log2=v[2].value, tile_rows=v[3].value)

    def kernel(self):
        """'small' when every job runs in the small-graph kernel, else 'engine'."""
        return "small" if load().ODPX_Batch_kernel(self._h) == 1 else "engine"

    def small_shape(self):
        """(cluster CTAs per job, threads per CTA, partitioned 0/1) of a plan on the small-graph kernel."""
        c, t, q = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(load().ODPX_Batch_small_shape(self._h, ctypes.byref(c), ctypes.byref(t), ctypes.byref(q)),
               "ODPX_Batch_small_shape")
        return c.value, t.value, q.value

    def job_levels(self):
        """Per-job finishing level of the last run (plan order; negative: stalled)."""
        n = self.info(0)["njobs"]
        out = np.zeros(n, dtype=np.int32)
        load().ODPX_Batch_job_levels(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), n)
        return out

    def bytes_alg(self):
        """Algorithmic bytes of the last run (roofline numerator)."""
        return float(load().ODPX_Batch_bytes_alg(self._h))

    def job_profile(self):
        """(graph, loaded_us, done_us) arrays per job of the last run (plan order)."""
        n = self.info(0)["njobs"]
        g = np.zeros(n, dtype=np.int32)
        a = np.zeros(n, dtype=np.float64)
        b = np.zeros(n, dtype=np.float64)
        load().ODPX_Batch_job_profile(self._h, g.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                      a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                      b.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n)
        return g, a, b

    def set_wait_limit(self, ns):
        load().ODPX_Batch_set_wait_limit(self._h, int(ns))

    def close(self):
        if self._h:
            load().ODPX_Batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_tuning(wc_log2=0, slots=0, tile_rows=0, l2_budget_mb=0, local_kb=0, use_graph=-1):
    """ODPX_Set_tuning: knobs for plans created afterwards (0 = automatic)."""
    load().ODPX_Set_tuning(wc_log2, slots, tile_rows, l2_budget_mb, local_kb, use_graph)


def version():
    return load().ODPX_Version().decode()


def measure_l2_read_gbs(megabytes=48, reps=50):
    """Read bandwidth (GB/s) of an L2-resident stream: the L2 roofline ceiling."""
    return float(load().ODPX_Measure_l2_read_gbs(megabytes, reps))


# --------------------------------------------------------------------------
# Serving API (odp_gb300.h ODPX_Serve_*).
# --------------------------------------------------------------------------

PENDING = 7


class Delta(ctypes.Structure):
    """ODPX_Delta: adjacency[row][slot] = value (compact adjacency)."""
    _fields_ = [("row", ctypes.c_int), ("slot", ctypes.c_int), ("value", ctypes.c_int)]


class ServeConfig(ctypes.Structure):
    _fields_ = [("lanes", ctypes.c_int), ("max_batch", ctypes.c_int), ("max_nodes", ctypes.c_int),
                ("memory_mb", ctypes.c_int), ("wc_log2", ctypes.c_int)]


class ServeCounters(ctypes.Structure):
    _fields_ = [("requests_done", ctypes.c_longlong), ("batches", ctypes.c_longlong),
                ("batched_requests", ctypes.c_longlong), ("max_batch", ctypes.c_int),
                ("max_inflight_lanes", ctypes.c_int), ("slots_per_lane", ctypes.c_int),
                ("blocks_per_lane", ctypes.c_int)]


def _bind_serve(lib):
    if getattr(lib, "_serve_bound", False):
        return lib
    P, I = ctypes.c_void_p, ctypes.c_int
    out4 = [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_double),
            ctypes.POINTER(ctypes.c_double)]
    sig = {
        "ODPX_Serve_create": (I, [ctypes.POINTER(ServeConfig), ctypes.POINTER(P)]),
        "ODPX_Serve_register": (I, [P, ctypes.POINTER(Graph), ctypes.POINTER(I)]),
        "ODPX_Serve_submit": (I, [P, I, I, ctypes.POINTER(Delta), ctypes.POINTER(ctypes.c_longlong)]),
        "ODPX_Serve_wait": (I, [P, ctypes.c_longlong] + out4),
        "ODPX_Serve_poll": (I, [P, ctypes.c_longlong] + out4),
        "ODPX_Serve_stats": (I, [P, ctypes.POINTER(ServeCounters)]),
        "ODPX_Serve_adjacency": (I, [P, I, P]),
        "ODPX_Serve_destroy": (None, [P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    lib._serve_bound = True
    return lib


class Server:
    """A serving instance: resident graphs, in-place 2-opt deltas, continuous
    batching over `lanes` concurrent GPU streams."""

    def __init__(self, lanes=4, max_batch=16, max_nodes=32768, memory_mb=1024, wc_log2=4):
        lib = _bind_serve(load())
        cfg = ServeConfig(lanes, max_batch, max_nodes, memory_mb, wc_log2)
        h = ctypes.c_void_p()
        _check(lib.ODPX_Serve_create(ctypes.byref(cfg), ctypes.byref(h)), "ODPX_Serve_create")
        self._h = h
        self._specs = {}

    def register(self, spec):
        g = spec.to_c()
        handle = ctypes.c_int()
        _check(load().ODPX_Serve_register(self._h, ctypes.byref(g), ctypes.byref(handle)), "ODPX_Serve_register")
        self._specs[handle.value] = spec
        return handle.value

    def submit(self, handle, deltas=()):
        n = len(deltas)
        arr = (Delta * max(n, 1))(*[Delta(int(r), int(s), int(v)) for r, s, v in deltas])
        rid = ctypes.c_longlong()
        _check(load().ODPX_Serve_submit(self._h, handle, n, arr, ctypes.byref(rid)), "ODPX_Serve_submit")
        return rid.value

    def _out(self, fn, rid):
        d, s, a, lat = ctypes.c_int(), ctypes.c_long(), ctypes.c_double(), ctypes.c_double()
        rc = fn(self._h, rid, ctypes.byref(d), ctypes.byref(s), ctypes.byref(a), ctypes.byref(lat))
        return rc, (d.value, s.value, a.value, lat.value)

    def wait(self, rid):
        """(diameter, sum, ASPL, latency_s) of a request, blocking."""
        rc, out = self._out(load().ODPX_Serve_wait, rid)
        _check(rc, "ODPX_Serve_wait")
        return out

    def poll(self, rid):
        rc, out = self._out(load().ODPX_Serve_poll, rid)
        if rc == PENDING:
            return None
        _check(rc, "ODPX_Serve_poll")
        return out

    def stats(self):
        c = ServeCounters()
        _check(load().ODPX_Serve_stats(self._h, ctypes.byref(c)), "ODPX_Serve_stats")
        return {f: getattr(c, f) for f, _ in ServeCounters._fields_}

    def adjacency(self, handle):
        spec = self._specs[handle]
        out = np.zeros_like(spec.adjacency)
        _check(load().ODPX_Serve_adjacency(self._h, handle, out.ctypes.data), "ODPX_Serve_adjacency")
        return out

    def close(self):
        if self._h:
            load().ODPX_Serve_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def two_opt_deltas(adjacency, restore, nodes, symmetries=1):
    """The compact-adjacency slots a 2-opt swap (its ODP_Restore record)
    touched, with their current values: what a served graph must apply."""
    base = nodes // symmetries
    out = []
    for i in range(2):
        for vert, slot in ((restore.u[i], restore.u_d[i]), (restore.v[i], restore.v_d[i])):
            row = vert % base
            out.append((row, slot, int(adjacency[row, slot])))
    return out


# --------------------------------------------------------------------------
# Annealing chains on the GPU (odp_gb300.h ODPX_Anneal_*).
# --------------------------------------------------------------------------

class ChainC(ctypes.Structure):
    """ODPX_Chain."""
    _fields_ = [("nodes", ctypes.c_int), ("degree", ctypes.c_int), ("symmetries", ctypes.c_int),
                ("num_degrees", ctypes.c_void_p), ("adjacency", ctypes.c_void_p), ("seed", ctypes.c_uint),
                ("max_temp", ctypes.c_double), ("min_temp", ctypes.c_double), ("ncalcs", ctypes.c_longlong),
                ("hill_climbing", ctypes.c_int), ("aspl_priority", ctypes.c_int), ("grid", ctypes.c_int),
                ("width", ctypes.c_int), ("height", ctypes.c_int), ("length", ctypes.c_int)]


class ChainState(ctypes.Structure):
    """ODPX_Chain_state."""
    _fields_ = [("steps", ctypes.c_longlong), ("accepted", ctypes.c_longlong), ("status", ctypes.c_int),
                ("diameter", ctypes.c_int), ("sum", ctypes.c_long), ("aspl", ctypes.c_double),
                ("best_diameter", ctypes.c_int), ("best_sum", ctypes.c_long), ("best_aspl", ctypes.c_double),
                ("temp", ctypes.c_double)]


def _bind_anneal(lib):
    if getattr(lib, "_anneal_bound", False):
        return lib
    P = ctypes.c_void_p
    lib.ODPX_Anneal_create.restype = ctypes.c_int
    lib.ODPX_Anneal_create.argtypes = [ctypes.POINTER(ChainC), ctypes.c_int, ctypes.POINTER(P)]
    lib.ODPX_Anneal_run.restype = ctypes.c_int
    lib.ODPX_Anneal_run.argtypes = [P, ctypes.c_int]
    lib.ODPX_Anneal_state.restype = ctypes.c_int
    lib.ODPX_Anneal_state.argtypes = [P, ctypes.c_int, ctypes.POINTER(ChainState), P, P]
    lib.ODPX_Anneal_destroy.restype = None
    lib.ODPX_Anneal_destroy.argtypes = [P]
    lib._anneal_bound = True
    return lib


class Chain:
    """One annealing chain: the starting graph and the client's parameters
    (seed, max/min temperature over ncalcs steps, -Y hill climbing, -A ASPL
    priority), as the reference's sample/SA clients take them."""

    def __init__(self, adjacency, nodes=0, symmetries=1, num_degrees=None, seed=0, max_temp=100.0, min_temp=0.2,
                 ncalcs=10000, hill_climbing=False, aspl_priority=False, grid=False, width=0, height=0, length=0):
        self.adjacency = _ints(adjacency)
        self.grid, self.width, self.height, self.length = bool(grid), width, height, length
        self.nodes = width * height if grid else nodes
        self.symmetries = symmetries
        self.degree = self.adjacency.shape[1]
        self.num_degrees = None if num_degrees is None else _ints(num_degrees)
        self.seed, self.max_temp, self.min_temp, self.ncalcs = seed, max_temp, min_temp, ncalcs
        self.hill_climbing, self.aspl_priority = hill_climbing, aspl_priority

    def to_c(self):
        return ChainC(self.nodes, self.degree, self.symmetries, _iptr(self.num_degrees), _iptr(self.adjacency),
                      self.seed, self.max_temp, self.min_temp, self.ncalcs, int(self.hill_climbing),
                      int(self.aspl_priority), int(self.grid), self.width, self.height, self.length)


class Anneal:
    """Annealing chains whose proposals, evaluations and decisions all run on
    the GPU (ODPX_Anneal_*)."""

    def __init__(self, chains):
        lib = _bind_anneal(load())
        self._chains = list(chains)
        arr = (ChainC * len(self._chains))(*[c.to_c() for c in self._chains])
        h = ctypes.c_void_p()
        _check(lib.ODPX_Anneal_create(arr, len(self._chains), ctypes.byref(h)), "ODPX_Anneal_create")
        self._h = h

    def run(self, steps):
        _check(load().ODPX_Anneal_run(self._h, steps), "ODPX_Anneal_run")

    def state(self, k, graphs=False):
        """The chain's counters and results as a dict; with graphs=True also
        its current and best adjacency."""
        c = self._chains[k]
        st = ChainState()
        cur = best = None
        if graphs:
            cur = np.empty_like(c.adjacency)
            best = np.empty_like(c.adjacency)
        _check(load().ODPX_Anneal_state(self._h, k, ctypes.byref(st), _iptr(cur), _iptr(best)), "ODPX_Anneal_state")
        out = {f: getattr(st, f) for f, _ in ChainState._fields_}
        if graphs:
            out["adjacency"], out["best_adjacency"] = cur, best
        return out

    def close(self):
        if self._h:
            load().ODPX_Anneal_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
