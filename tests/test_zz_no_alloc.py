"""ODPX_Set_aspl_noalloc, the entry point for callers that cannot allocate
memory while they run (it takes its working memory from a fixed array in the
library's device image): through the C ABI, its results must equal the
drop-in ODP_Init_aspl_general(_s) + ODP_Set_aspl path bit for bit, on
consecutive calls that reuse the same array.  Collected last on purpose."""
import ctypes

import numpy as np
import pytest

import odp_gb300 as og
from conftest import same

pytestmark = pytest.mark.gpu


def _entry():
    f = og.load().ODPX_Set_aspl_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                  ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_double)]
    return f


def noalloc(n, s, adj):
    adj = np.ascontiguousarray(adj, dtype=np.int32)
    d, sm, a = ctypes.c_int(), ctypes.c_long(), ctypes.c_double()
    rc = _entry()(n, adj.shape[1], s, adj.ctypes.data, ctypes.byref(d), ctypes.byref(sm), ctypes.byref(a))
    return rc, (d.value, sm.value, a.value)


def drop_in(n, s, adj):
    if s == 1:
        og.init_aspl_general(n, adj.shape[1])
    else:
        og.init_aspl_general_s(n, adj.shape[1], None, s)
    try:
        return og.set_aspl(adj)
    finally:
        og.finalize_aspl()


def graph(n, d, s, seed):
    return og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, s, seed=seed), d, s)


def test_noalloc_matches_drop_in_on_consecutive_calls():
    big = (8192, 32, 1, graph(8192, 32, 1, 24))
    small = (1024, 8, 1, graph(1024, 8, 1, 1))
    sym = (4096, 12, 4, graph(4096, 12, 4, 5))
    expect = {id(g): drop_in(g[0], g[2], g[3]) for g in (big, small, sym)}
    # the larger graph first, then smaller ones that reuse the same array
    for g in (big, small, sym, small):
        rc, got = noalloc(g[0], g[2], g[3])
        assert rc == og.OK
        assert same(got, expect[id(g)]), (g[:3], got, expect[id(g)])
    assert expect[id(small)][:2] == (5, 1892906)


def test_noalloc_refuses_graphs_beyond_its_fixed_memory():
    n, d = 262144, 16
    adj = np.zeros((n, d), dtype=np.int32)
    rc, _ = noalloc(n, 1, adj)
    assert rc == og.ERR_MEMORY
    # and the entry point still works afterwards
    small = graph(512, 6, 1, 3)
    rc, got = noalloc(512, 1, small)
    assert rc == og.OK and same(got, drop_in(512, 1, small))


def device_free_bytes():
    """Free memory of the current device (driver API, on this thread's
    current context, which the library's calls have made current)."""
    cu = ctypes.CDLL("libcuda.so.1")
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert cu.cuMemGetInfo_v2(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def test_noalloc_allocates_nothing_after_its_first_call():
    graphs = [(8192, 1, graph(8192, 32, 1, 24)), (1024, 1, graph(1024, 8, 1, 1)), (4096, 4, graph(4096, 12, 4, 5)),
              (2048, 2, graph(2048, 6, 2, 9))]
    expect = [drop_in(n, s, a) for n, s, a in graphs]
    rc, _ = noalloc(*graphs[0])                      # the first call may set up (module load, symbol lookup)
    assert rc == og.OK
    before = device_free_bytes()
    for _ in range(3):
        for (n, s, a), want in zip(graphs, expect):
            rc, got = noalloc(n, s, a)
            assert rc == og.OK and same(got, want)
            assert device_free_bytes() == before


def test_noalloc_reports_disconnected_graphs_like_the_drop_in():
    # two disjoint copies of a 4-regular graph on 1024 vertices
    half = graph(1024, 4, 1, 7)
    adj = np.concatenate([half, half + 1024]).astype(np.int32)
    want = drop_in(2048, 1, adj)
    assert want[0] == 2 ** 31 - 1 and want[1] == 2 ** 63 - 1
    for _ in range(2):
        rc, got = noalloc(2048, 1, adj)
        assert rc == og.OK and same(got, want)


def test_noalloc_refuses_out_of_range_adjacency_and_recovers():
    n = 1024
    good = graph(n, 8, 1, 1)
    for bad_value in (n, -1, 10 ** 6):
        bad = good.copy()
        bad[17, 3] = bad_value
        rc, _ = noalloc(n, 1, bad)
        assert rc == og.ERR_ADJACENCY, bad_value
        rc, got = noalloc(n, 1, good)
        assert rc == og.OK and got[:2] == (5, 1892906)
