"""The library's host utilities (odp.h generators, conversions, 2-opt
mutate/restore) against the reference's outputs.  CPU only."""
import ctypes
import ctypes.util

import numpy as np
import pytest

import odp_gb300 as og
import oracle
from conftest import gen_record_adjacency, gen_record_edges, sha256


def test_private_stream_matches_libc_rand():
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    for seed in [0, 1, 2, 4, 12345, 2**31 - 1, 2**31 + 5, 2**32 - 1]:
        libc.srand(ctypes.c_uint(seed))
        expect = [libc.rand() for _ in range(5000)]
        r = og.Rng(seed)
        assert [r.next() for _ in range(5000)] == expect, seed


def test_generators_match_reference_hashes(golden):
    for g in golden["generators"]:
        if g.get("big"):
            continue
        assert sha256(gen_record_edges(og, g)) == g["sha256"], g


def test_libc_stream_generators_match_seeded():
    og.srand(5)
    a = og.generate_random_general(96, 6, 4)
    b = og.generate_random_general(96, 6, 4, seed=5)
    assert np.array_equal(a, b)
    og.srand(6)
    a = og.generate_random_grid(10, 10, 4, 4, 4)
    b = og.generate_random_grid(10, 10, 4, 4, 4, seed=6)
    assert np.array_equal(a, b)


def test_mutation_traces_match_reference(golden):
    for m in golden["mutations"]:
        if m["kind"] == "general":
            e = og.generate_random_general(m["nodes"], m["degree"], m["symmetries"], seed=m["graph_seed"])
            adj = og.conv_edge2adjacency_general(m["nodes"], e, m["degree"], m["symmetries"])
            og.srand(m["seed"])
            trace = []
            for _ in range(m["iters"]):
                r = og.mutate_adjacency_general(m["nodes"], m["degree"], adj, m["symmetries"])
                trace += list(r.u) + list(r.v) + list(r.u_d) + list(r.v_d)
        else:
            e = og.generate_random_grid(m["width"], m["height"], m["degree"], m["length"], m["symmetries"],
                                        seed=m["graph_seed"])
            adj = og.conv_edge2adjacency_grid(m["width"], m["height"], e, m["degree"], m["symmetries"])
            og.srand(m["seed"])
            trace = []
            for _ in range(m["iters"]):
                r = og.mutate_adjacency_grid(m["width"], m["height"], m["degree"], m["length"], adj, m["symmetries"])
                trace += list(r.u) + list(r.v) + list(r.u_d) + list(r.v_d)
        assert trace[:8] == m["first_restore"], m
        assert sha256(np.array(trace)) == m["trace_sha256"], m
        assert sha256(adj) == m["final_sha256"], m


@pytest.mark.parametrize("s", [1, 2, 4])
def test_restore_undoes_mutate_general(s):
    n, d = 240, 6
    adj = og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, s, seed=3), d, s)
    og.srand(9)
    for _ in range(200):
        before = adj.copy()
        r = og.mutate_adjacency_general(n, d, adj, s)
        assert not np.array_equal(before, adj) or True
        og.restore_adjacency_general(r, adj)
        assert np.array_equal(before, adj)
        og.mutate_adjacency_general(n, d, adj, s)


@pytest.mark.parametrize("s", [1, 2, 4])
def test_restore_undoes_mutate_grid(s):
    w = h = 12
    d, length = 4, 3
    adj = og.conv_edge2adjacency_grid(w, h, og.generate_random_grid(w, h, d, length, s, seed=4), d, s)
    og.srand(11)
    for _ in range(200):
        before = adj.copy()
        r = og.mutate_adjacency_grid(w, h, d, length, adj, s)
        og.restore_adjacency_grid(r, adj)
        assert np.array_equal(before, adj)
        og.mutate_adjacency_grid(w, h, d, length, adj, s)


@pytest.mark.parametrize("s", [1, 4, 8])
def test_edge_adjacency_round_trip(s):
    n, d = 128, 5
    e = og.generate_random_general(n, d, s, seed=21)
    adj = og.conv_edge2adjacency_general(n, e, d, s)
    e2 = og.conv_adjacency2edge_general(n, d, adj, s)
    assert np.array_equal(og.conv_edge2adjacency_general(n, e2, d, s), adj)


@pytest.mark.parametrize("s", [1, 2, 8])
def test_private_stream_mutate_and_explicit_restore(s):
    n, d = 240, 6
    adj = og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, s, seed=13), d, s)
    rng = og.Rng(17)
    for _ in range(100):
        before = adj.copy()
        r = rng.mutate_general(n, d, adj, symmetries=s)
        og.Rng.restore_general(n, d, r, adj, symmetries=s)
        assert np.array_equal(before, adj)
        rng.mutate_general(n, d, adj, symmetries=s)


def test_restore_before_any_mutate_is_refused():
    import subprocess, sys, textwrap
    from conftest import ROOT
    code = textwrap.dedent("""
        import sys; sys.path.insert(0, %r)
        import numpy as np, odp_gb300 as og
        og.restore_adjacency_general(og.Restore(), np.zeros((4, 2), dtype=np.int32))
    """ % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "before ODP_Mutate" in r.stderr


@pytest.mark.skipif(oracle.ref_driver() is None, reason="reference library not built")
def test_lower_bounds_match_reference():
    """ODP_Set_lbounds_general / _grid (the "gap" lines of the sample
    programs) give the reference's diameter and ASPL bits."""
    import subprocess
    drv = oracle.ref_driver()

    def ref(*args):
        out = subprocess.run([drv, "lbounds"] + [str(a) for a in args], capture_output=True, text=True,
                             timeout=60, check=True).stdout.split()
        return int(out[0]), float.fromhex(out[1])

    for n in (4, 5, 10, 12, 16, 17, 72, 100, 256, 1000, 65536, 10 ** 6):
        for d in (2, 3, 4, 6, 10, 16, 32):
            r, g = ref("general", n, d), og.set_lbounds_general(n, d)
            assert r[0] == g[0] and r[1].hex() == g[1].hex(), (n, d, r, g)
    for m, n, d, length in [(4, 4, 3, 2), (5, 5, 4, 2), (6, 6, 3, 2), (4, 6, 3, 2), (7, 9, 4, 3), (12, 12, 5, 3),
                            (20, 12, 6, 4), (30, 30, 8, 3), (40, 20, 8, 5), (64, 64, 4, 3), (90, 90, 32, 3)]:
        r, g = ref("grid", m, n, d, length), og.set_lbounds_grid(m, n, d, length)
        assert r[0] == g[0] and r[1].hex() == g[1].hex(), (m, n, d, length, r, g)
