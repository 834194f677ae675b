"""GPU parity: the library's ASPL path (through its C ABI) against the
reference's golden vectors and the oracle.  Every comparison is bit-exact:
diameter and sum as integers, ASPL by its IEEE-754 bits."""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import odp_gb300 as og
import oracle
from conftest import (ROOT, case_adjacency, case_degrees, edges_to_adjacency, gen_record_adjacency, gen_record_edges,
                      result_tuple, same, sha256)

pytestmark = pytest.mark.gpu


def gpu_aspl(adj, nodes=0, num_degrees=None, symmetries=1, grid=False, width=0, height=0):
    """Init / Set / Finalize through the drop-in API."""
    adj = np.ascontiguousarray(adj, dtype=np.int32)
    d = adj.shape[1]
    if grid:
        if symmetries == 1:
            og.init_aspl_grid(width, height, d, num_degrees)
        else:
            og.init_aspl_grid_s(width, height, d, num_degrees, symmetries)
    else:
        if symmetries == 1:
            og.init_aspl_general(nodes, d, num_degrees)
        else:
            og.init_aspl_general_s(nodes, d, num_degrees, symmetries)
    try:
        return og.set_aspl(adj)
    finally:
        og.finalize_aspl()


def test_sample_golden_tables(golden):
    for s in golden["samples"]:
        e = np.array(s["edges"], dtype=np.int32).reshape(-1, 2)
        if "expected" in s:
            if s["kind"] == "general":
                n = int(e.max()) + 1
                deg = int(np.bincount(e.reshape(-1), minlength=n).max())
                got = gpu_aspl(og.conv_edge2adjacency_general(n, e, deg), nodes=n)
            else:
                n = s["width"] * s["height"]
                deg = int(np.bincount(e.reshape(-1), minlength=n).max())
                got = gpu_aspl(og.conv_edge2adjacency_grid(s["width"], s["height"], e, deg), grid=True,
                               width=s["width"], height=s["height"])
            exp = s["expected"]
            assert (got[0], got[1], "%.10f" % got[2]) == (exp["diameter"], exp["sum"], exp["aspl"]), s["file"]
        else:
            if s["kind"] == "general":
                adj = og.conv_edge2adjacency_general(s["nodes"], e, s["degree"], s["symmetries"])
                got = gpu_aspl(adj, nodes=s["nodes"], symmetries=s["symmetries"])
            else:
                adj = og.conv_edge2adjacency_grid(s["width"], s["height"], e, s["degree"], s["symmetries"])
                got = gpu_aspl(adj, grid=True, width=s["width"], height=s["height"], symmetries=s["symmetries"])
            assert same(got, result_tuple(s["reference"])), s["file"]


def test_edge_cases(golden):
    for c in golden["cases"]:
        adj = case_adjacency(c)
        nd = case_degrees(c)
        if c["kind"] == "general":
            got = gpu_aspl(adj, nodes=c["nodes"], num_degrees=nd, symmetries=c["symmetries"])
        else:
            got = gpu_aspl(adj, grid=True, width=c["width"], height=c["height"], num_degrees=nd,
                           symmetries=c["symmetries"])
        assert same(got, result_tuple(c["reference"])), (c["name"], got, c["reference"])


def test_generated_fixtures(golden):
    for g in golden["generators"]:
        if g.get("big"):
            continue
        e = gen_record_edges(og, g)
        adj = gen_record_adjacency(og, g, e)
        if g["kind"] == "general":
            got = gpu_aspl(adj, nodes=g["nodes"], symmetries=g["symmetries"])
        else:
            got = gpu_aspl(adj, grid=True, width=g["width"], height=g["height"], symmetries=g["symmetries"])
        assert same(got, result_tuple(g["reference"])), (g, got)


def random_graph(rng):
    """A random generated graph of random kind/shape, with its batch spec."""
    if rng.random() < 0.7:
        s = int(rng.choice([1, 1, 2, 4, 8]))
        base = int(rng.integers(8, 400))
        n = base * s
        d = int(rng.integers(3, 12))
        if n % 2 and d % 2:
            d += 1
        e = og.generate_random_general(n, d, s, seed=int(rng.integers(1 << 30)))
        adj = og.conv_edge2adjacency_general(n, e, d, s)
        return og.GraphSpec(adj, nodes=n, symmetries=s), dict(nodes=n, symmetries=s)
    s = int(rng.choice([1, 2, 4]))
    w = 2 * int(rng.integers(2, 9))
    h = w if s == 4 else 2 * int(rng.integers(2, 9))
    d = int(rng.integers(3, 7))
    length = int(rng.integers(2, 5))
    e = og.generate_random_grid(w, h, d, length, s, seed=int(rng.integers(1 << 30)))
    adj = og.conv_edge2adjacency_grid(w, h, e, d, s)
    return (og.GraphSpec(adj, grid=True, width=w, height=h, symmetries=s),
            dict(grid=True, width=w, height=h, symmetries=s))


def test_random_graphs_against_oracle():
    rng = np.random.default_rng(123)
    for _ in range(40):
        spec, kw = random_graph(rng)
        assert same(gpu_aspl(spec.adjacency, **kw), oracle.aspl(spec.adjacency, **kw)), kw


def test_batch_matches_single_and_oracle(golden):
    rng = np.random.default_rng(5)
    specs, kws = [], []
    for _ in range(60):
        spec, kw = random_graph(rng)
        specs.append(spec)
        kws.append(kw)
    for c in golden["cases"]:        # non-regular, directed, disconnected, tiny graphs
        if c["kind"] == "general":
            specs.append(og.GraphSpec(case_adjacency(c), nodes=c["nodes"], symmetries=c["symmetries"],
                                      num_degrees=case_degrees(c)))
            kws.append(dict(nodes=c["nodes"], symmetries=c["symmetries"], num_degrees=case_degrees(c)))
    got = og.set_aspl_batch(specs)
    for spec, kw, g in zip(specs, kws, got):
        assert same(g, oracle.aspl(spec.adjacency, **kw)), kw
    # the cached plan is reused on a second call with new adjacency
    got2 = og.set_aspl_batch(specs)
    assert all(same(a, b) for a, b in zip(got, got2))


def test_engine_batch_with_new_arrays_and_a_bad_entry(golden, monkeypatch):
    """A batch on the engine (general, symmetric, grid, non-regular,
    directed and disconnected graphs): each call's pull kernel reads the
    descriptors of that call from pinned memory, copies the callers' arrays
    and resets the engine state, so a second call with other arrays of the
    same shapes gives their results, an out-of-range entry in any graph is
    reported, and the next call is right again."""
    monkeypatch.setenv("ODP_GB300_SMALL_N", "0")
    rng = np.random.default_rng(17)
    specs, kws = [], []
    for _ in range(44):
        spec, kw = random_graph(rng)
        specs.append(spec)
        kws.append(kw)
    for c in golden["cases"]:        # non-regular, directed, disconnected, tiny graphs
        if c["kind"] == "general":
            specs.append(og.GraphSpec(case_adjacency(c), nodes=c["nodes"], symmetries=c["symmetries"],
                                      num_degrees=case_degrees(c)))
            kws.append(dict(nodes=c["nodes"], symmetries=c["symmetries"], num_degrees=case_degrees(c)))
    assert len(specs) >= 32
    refs = [oracle.aspl(sp.adjacency, **kw) for sp, kw in zip(specs, kws)]
    got = og.set_aspl_batch(specs)
    for k, (g, r) in enumerate(zip(got, refs)):
        assert same(g, r), (k, kws[k])
    # same shapes, other arrays: the graphs of equal shape swapped
    swapped = list(specs)
    for i in range(len(specs)):
        for j in range(i + 1, len(specs)):
            a, b = specs[i], specs[j]
            if (a.grid, a.nodes, a.width, a.height, a.degree, a.symmetries) == \
               (b.grid, b.nodes, b.width, b.height, b.degree, b.symmetries) and a.num_degrees is None \
               and b.num_degrees is None and swapped[i] is a and swapped[j] is b:
                swapped[i] = og.GraphSpec(b.adjacency, grid=a.grid, nodes=a.nodes, width=a.width, height=a.height,
                                          symmetries=a.symmetries)
                swapped[j] = og.GraphSpec(a.adjacency, grid=b.grid, nodes=b.nodes, width=b.width, height=b.height,
                                          symmetries=b.symmetries)
    want = []
    for sp in swapped:
        k = next(i for i, x in enumerate(specs) if x.adjacency is sp.adjacency)
        want.append(refs[k])
    for k, (g, r) in enumerate(zip(og.set_aspl_batch(swapped), want)):
        assert same(g, r), k
    bad = [og.GraphSpec(sp.adjacency.copy(), grid=sp.grid, nodes=sp.nodes, width=sp.width, height=sp.height,
                        symmetries=sp.symmetries, num_degrees=sp.num_degrees) for sp in specs]
    bad[len(bad) // 2].adjacency[0, 0] = 1 << 20
    with pytest.raises(og.ODPError) as ei:
        og.set_aspl_batch(bad)
    assert ei.value.code == og.ERR_ADJACENCY
    for g, r in zip(og.set_aspl_batch(specs), refs):
        assert same(g, r)


def test_batch_plan_reuse_with_new_adjacency():
    n, d = 512, 6
    adjs = [og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, seed=s), d) for s in range(8)]
    b = og.Batch([og.GraphSpec(a, nodes=n) for a in adjs])
    first = b.run()
    rev = b.run(adjs[::-1])
    assert [same(x, y) for x, y in zip(first[::-1], rev)] == [True] * 8
    for a, r in zip(adjs, first):
        assert same(r, oracle.aspl(a, nodes=n))
    b.close()


@pytest.mark.parametrize("wc_log2,slots,tile_rows", [(1, 1, 0), (2, 3, 16), (4, 2, 64), (6, 0, 0), (3, 5, 8)])
def test_chunking_and_tiling_do_not_change_results(wc_log2, slots, tile_rows):
    """Column chunk width, concurrent slots and row tiles are free choices."""
    n, d = 3000, 7
    adj = og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, seed=77), d)
    ref = oracle.aspl(adj, nodes=n)
    og.set_tuning(wc_log2=wc_log2, slots=slots, tile_rows=tile_rows, local_kb=1)
    try:
        b = og.Batch([og.GraphSpec(adj, nodes=n)])
        assert same(b.run()[0], ref)
        b.close()
    finally:
        og.set_tuning()


def _saturation_cases():
    """Graphs whose rows saturate early, or never, or hold padding lanes."""
    cases = []
    g = lambda n, d, s=1, seed=1: og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, s, seed=seed), d, s)
    cases.append(og.GraphSpec(g(300, 40, seed=5), nodes=300))            # diameter 3: most lanes saturate at 2
    cases.append(og.GraphSpec(g(1000, 12, seed=6), nodes=1000))          # 1000 sources: padding lanes past 1000
    cases.append(og.GraphSpec(g(1000, 10, 4, seed=7), nodes=1000, symmetries=4))
    irr = g(500, 8, seed=8)
    u, v = 0, int(irr[0, 7])
    j = int(np.nonzero(irr[v] == u)[0][0])
    irr[v, j], irr[v, 7] = irr[v, 7], irr[v, j]
    irr[u, 7] = irr[v, 7] = -1
    deg = np.full(500, 8, dtype=np.int32)
    deg[u] = deg[v] = 7
    cases.append(og.GraphSpec(irr, nodes=500, num_degrees=deg))
    half = g(128, 4, seed=9)                                             # two components: never saturates
    cases.append(og.GraphSpec(np.concatenate([half, half + 128]).astype(np.int32), nodes=256))
    e = og.generate_random_grid(30, 30, 6, 3, 1, seed=10)
    cases.append(og.GraphSpec(og.conv_edge2adjacency_grid(30, 30, e, 6, 1), grid=True, width=30, height=30))
    return cases


@pytest.mark.parametrize("wc_log2", [1, 3, 5, 7])
def test_saturated_lanes_skip_only_what_cannot_change(wc_log2):
    """Lanes whose words hold every source bit of the chunk skip their
    gathers.  Chunk widths of 2 to 128 words (1 to 32 lanes per row, one to
    four vectors per lane), small multi-tile levels, and graphs that
    saturate at level 2, hold padding lanes, are symmetric or irregular,
    never saturate (disconnected) or are grids."""
    cases = _saturation_cases()
    refs = [oracle.aspl(c.adjacency, nodes=c.nodes, num_degrees=c.num_degrees, symmetries=c.symmetries,
                        grid=c.grid, width=c.width, height=c.height) for c in cases]
    assert refs[4][0] == 2147483647
    og.set_tuning(wc_log2=wc_log2, slots=3, tile_rows=16, local_kb=1)
    try:
        b = og.Batch(cases)
        got = b.run()
        b.close()
    finally:
        og.set_tuning()
    for k, (x, y) in enumerate(zip(got, refs)):
        assert same(x, y), (k, x, y)


@pytest.mark.parametrize("small_n", ["2048", "0"])
def test_small_graph_kernel_and_engine_agree(small_n, monkeypatch):
    """Plans whose graphs all have at most 2048 vertices run every job in
    the small-graph kernel (bitsets and neighbour table in shared memory);
    ODP_GB300_SMALL_N=0 sends them through the persistent engine.  Both give
    the oracle's results, singly and as one batch."""
    monkeypatch.setenv("ODP_GB300_SMALL_N", small_n)
    g = lambda n, d, s=1, seed=1: og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, s, seed=seed), d, s)
    cases = _saturation_cases()                                           # general, s = 4, irregular, disconnected, grid
    cases.append(og.GraphSpec(g(2048, 12, seed=11), nodes=2048))         # fits with 2-word chunks only
    cases.append(og.GraphSpec(g(16, 3, seed=12), nodes=16))
    for s_, w in ((2, 20), (4, 20)):
        e = og.generate_random_grid(w, w, 4, 3, s_, seed=13)
        cases.append(og.GraphSpec(og.conv_edge2adjacency_grid(w, w, e, 4, s_), grid=True, width=w, height=w,
                                  symmetries=s_))
    refs = [oracle.aspl(c.adjacency, nodes=c.nodes, num_degrees=c.num_degrees, symmetries=c.symmetries,
                        grid=c.grid, width=c.width, height=c.height) for c in cases]
    kernel = "engine" if small_n == "0" else "small"
    b = og.Batch(cases)
    assert b.kernel() == kernel
    got = b.run()
    b.close()
    for k, (x, y) in enumerate(zip(got, refs)):
        assert same(x, y), (k, x, y)
    for c, y in zip(cases, refs):
        b = og.Batch([c])
        assert b.kernel() == kernel
        assert same(b.run()[0], y)
        b.close()
    big = og.GraphSpec(g(16384, 8, seed=14), nodes=16384)               # one graph too large mixes in: engine
    b = og.Batch(cases[:2] + [big])
    assert b.kernel() == "engine"
    b.close()


@pytest.mark.parametrize("cluster,part", [(1, 0), (2, 0), (4, 0), (8, 0), (2, 1), (4, 1), (8, 1)])
def test_small_kernel_cluster_sizes(cluster, part, monkeypatch):
    """A small-kernel job runs on the CTAs of one thread-block cluster: each
    CTA computes its share of the rows and stores them into every CTA's copy
    of the level (distributed shared memory), and each builds the row-table
    entries of 1/cluster of the adjacency for the CTAs that own the rows.
    In the partitioned layout each CTA holds only its own rows and gathers
    the others' from their shared memory.  Forced cluster sizes of 1 to 8
    CTAs, in both layouts, give the oracle's results on row
    counts that do not divide evenly (n = 998, 1000) or are below the
    cluster size (n = 5, 6), symmetric general and grid graphs (rows placed
    through the rotation table), irregular and disconnected graphs, and the
    n = 1024 golden graph, one plan per graph and as one plan."""
    monkeypatch.setenv("ODP_GB300_SMALL_CLUSTER", str(cluster))
    monkeypatch.setenv("ODP_GB300_SMALL_PART", str(part))
    g = lambda n, d, s=1, seed=1: og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, s, seed=seed), d, s)
    cases = _saturation_cases()
    cases += [og.GraphSpec(g(n, d, seed=20 + n), nodes=n) for n, d in ((998, 3), (1000, 6), (6, 3), (5, 4), (1024, 8))]
    for s_, w in ((2, 20), (4, 20)):
        e = og.generate_random_grid(w, w, 4, 3, s_, seed=13)
        cases.append(og.GraphSpec(og.conv_edge2adjacency_grid(w, w, e, 4, s_), grid=True, width=w, height=w,
                                  symmetries=s_))
    refs = [oracle.aspl(c.adjacency, nodes=c.nodes, num_degrees=c.num_degrees, symmetries=c.symmetries,
                        grid=c.grid, width=c.width, height=c.height) for c in cases]
    for k, (c, y) in enumerate(zip(cases, refs)):
        b = og.Batch([c])
        assert b.kernel() == "small"
        assert b.small_shape()[0] == cluster and b.small_shape()[2] == part
        assert same(b.run()[0], y), (k, cluster, part)
        assert same(b.run()[0], y), (k, cluster, part)
        b.close()
    b = og.Batch(cases)
    assert b.kernel() == "small" and b.small_shape()[0] == cluster and b.small_shape()[2] == part
    for k, (x, y) in enumerate(zip(b.run(), refs)):
        assert same(x, y), (k, cluster, part)
    b.close()
    monkeypatch.delenv("ODP_GB300_SMALL_CLUSTER")
    monkeypatch.delenv("ODP_GB300_SMALL_PART")
    b = og.Batch([cases[-3]])                                  # n = 1024, d = 8: 8 jobs on clusters of 8
    assert b.small_shape()[:3:2] == (8, 0)
    b.close()


def test_small_kernel_mid_size_graphs():
    """With the row table split over a cluster, graphs up to n = 4096 whose
    bitset buffers fit run in the small kernel when their jobs fit on the SMs
    in one wave; larger grids (90 x 90) with the rows partitioned over the
    cluster; general graphs that would need two waves run in the engine.  All
    give the oracle's results."""
    g = lambda n, d, seed: og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, seed=seed), d)
    e = og.generate_random_grid(64, 64, 6, 3, 1, seed=3)
    e90 = og.generate_random_grid(90, 90, 4, 3, 1, seed=4)
    cases = [(og.GraphSpec(g(3000, 16, 31), nodes=3000), "small"),
             (og.GraphSpec(g(4096, 8, 32), nodes=4096), "small"),
             (og.GraphSpec(og.conv_edge2adjacency_grid(64, 64, e, 6, 1), grid=True, width=64, height=64), "small"),
             (og.GraphSpec(og.conv_edge2adjacency_grid(90, 90, e90, 4, 1), grid=True, width=90, height=90), "small"),
             (og.GraphSpec(g(4096, 24, 33), nodes=4096), "engine"),
             (og.GraphSpec(g(8192, 8, 34), nodes=8192), "engine")]
    for c, kernel in cases:
        want = oracle.aspl(c.adjacency, nodes=c.nodes, grid=c.grid, width=c.width, height=c.height)
        b = og.Batch([c])
        assert b.kernel() == kernel, (c.nodes, kernel)
        assert same(b.run()[0], want)
        b.close()


def test_config1_default_kind_and_saving():
    n, d = 1024, 8
    adj = og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, seed=1), d)
    assert gpu_aspl(adj, nodes=n) == (5, 1892906, pytest.approx(3.6139609299, abs=5e-11))
    assert same(gpu_aspl(adj, nodes=n), oracle.aspl(adj, nodes=n))


def _big(golden, name):
    for g in golden["generators"]:
        if g.get("name") == name:
            return g
    pytest.skip("fixture %s not recorded" % name)


def test_config2_single_large_graph(golden):
    g = _big(golden, "single_large_65536")
    e = gen_record_edges(og, g)
    assert sha256(e) == g["sha256"]
    adj = gen_record_adjacency(og, g, e)
    got = gpu_aspl(adj, nodes=g["nodes"])
    assert same(got, result_tuple(g["reference"]))


def test_config3_symmetric_graph(golden):
    g = _big(golden, "symmetric_262144")
    e = gen_record_edges(og, g)
    assert sha256(e) == g["sha256"]
    adj = gen_record_adjacency(og, g, e)
    assert same(gpu_aspl(adj, nodes=g["nodes"], symmetries=g["symmetries"]), result_tuple(g["reference"]))


def test_relabelling_invariance_full_size():
    """Size-independent property at the single-graph benchmark size: renaming
    vertices changes no result (checks every row/chunk of the big path)."""
    n, d = 65536, 16
    adj = og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, seed=9), d)
    base = gpu_aspl(adj, nodes=n)
    perm = np.random.default_rng(1).permutation(n).astype(np.int32)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(n, dtype=np.int32)
    adj2 = perm[adj[inv]]
    assert same(gpu_aspl(adj2, nodes=n), base)
    assert base[0] < 10 and base[1] > 0


def test_symmetric_equals_expanded_at_large_size():
    """Size-independent property: a graph with 32-fold circulant symmetry
    (n = 131072) gives the same results through the symmetric path (4096
    source rows, rotated neighbour tables) as its full adjacency through the
    plain path (131072 source rows), and so does a symmetric grid against
    its expanded form."""
    n, d, s = 131072, 12, 32
    e = og.generate_random_general(n, d, s, seed=6)
    sym = gpu_aspl(og.conv_edge2adjacency_general(n, e, d, s), nodes=n, symmetries=s)
    full = gpu_aspl(og.conv_edge2adjacency_general(n, e, d, 1), nodes=n)
    assert same(sym, full)
    assert sym[0] < 20 and sym[1] > 0
    w = 128
    e = og.generate_random_grid(w, w, 6, 5, 4, seed=7)
    sym = gpu_aspl(og.conv_edge2adjacency_grid(w, w, e, 6, 4), grid=True, width=w, height=w, symmetries=4)
    full = gpu_aspl(og.conv_edge2adjacency_grid(w, w, e, 6, 1), grid=True, width=w, height=w)
    assert same(sym, full)


def test_out_of_range_adjacency_is_reported():
    n, d = 64, 3
    adj = og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, seed=3), d)
    bad = adj.copy()
    bad[5, 1] = n + 7
    with pytest.raises(og.ODPError) as ei:
        og.set_aspl_batch([og.GraphSpec(bad, nodes=n)])
    assert ei.value.code == og.ERR_ADJACENCY
    # the context stays usable
    assert same(og.set_aspl_batch([og.GraphSpec(adj, nodes=n)])[0], oracle.aspl(adj, nodes=n))


def test_drop_in_errors_exit_like_the_reference(tmp_path):
    code = textwrap.dedent("""
        import sys; sys.path.insert(0, %r)
        import odp_gb300 as og
        og.init_aspl_general_s(10, 3, None, 3)
    """ % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    assert r.returncode == 1 and "must be divisible by symmetries" in r.stderr
    env = dict(os.environ, ODP_ASPL="BFS")
    code2 = code.replace("init_aspl_general_s(10, 3, None, 3)", "init_aspl_general(10, 3)")
    r = subprocess.run([sys.executable, "-c", code2], capture_output=True, text=True, env=env)
    assert r.returncode == 1 and "BFS for CUDA is not implemented" in r.stderr


def test_profile_report(tmp_path):
    code = textwrap.dedent("""
        import sys; sys.path.insert(0, %r)
        import odp_gb300 as og
        e = og.generate_random_general(256, 4, seed=1)
        adj = og.conv_edge2adjacency_general(256, e, 4)
        og.init_aspl_general(256, 4)
        og.set_aspl(adj); og.set_aspl(adj)
        og.finalize_aspl()
    """ % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                       env=dict(os.environ, ODP_PROFILE="1"))
    assert r.returncode == 0
    assert "Number of Times = 2" in r.stdout and "Algorithm       = MATRIX (CUDA)" in r.stdout


def test_reinit_cycles_of_every_variant():
    """Init/Finalize of different variants back to back (the reference
    double-frees after a grid_s session)."""
    w = h = 8
    e = og.generate_random_grid(w, h, 4, 3, 4, seed=2)
    adj4 = og.conv_edge2adjacency_grid(w, h, e, 4, 4)
    r1 = gpu_aspl(adj4, grid=True, width=w, height=h, symmetries=4)
    adj1 = og.conv_edge2adjacency_grid(w, h, e, 4, 1)
    r2 = gpu_aspl(adj1, grid=True, width=w, height=h)
    assert same(r1, r2)
    assert same(r1, oracle.aspl(adj1, grid=True, width=w, height=h))


def test_grid_256x256_fixture(golden):
    """The 256x256 grid (diameter 140): the reference's own graph, stored
    compactly because regenerating it takes minutes on a CPU."""
    import hashlib
    g = _big(golden, "grid_256x256")
    z = np.load(os.path.join(ROOT, "tests", "golden", "grid_256x256_d6_l4_seed4.npz"))
    codes = z["codes"].astype(np.int32)
    w = h = 256
    v = np.arange(w * h)[:, None]
    adj = ((v // h + codes // 9 - 4) * h + (v % h + codes % 9 - 4)).astype(np.int32)
    assert hashlib.sha256(adj.tobytes()).hexdigest() == bytes(z["adjacency_sha256"]).decode()
    edges = og.conv_adjacency2edge_grid(w, h, 6, adj)
    assert sha256(edges) == g["sha256"] == bytes(z["edges_sha256"]).decode()
    assert same(gpu_aspl(adj, grid=True, width=w, height=h), result_tuple(g["reference"]))


@pytest.mark.parametrize("s", [1, 2, 4])
@pytest.mark.parametrize("wc_log2", [1, 2, 4, 6])
def test_grid_source_tiles_and_chunk_widths(s, wc_log2):
    """Grid graphs use spatially compact source chunks; any chunk width and
    any source order give the reference's results."""
    w = h = 40
    d, length = 6, 3
    adj = og.conv_edge2adjacency_grid(w, h, og.generate_random_grid(w, h, d, length, s, seed=31 + s), d, s)
    ref = oracle.aspl(adj, grid=True, width=w, height=h, symmetries=s)
    og.set_tuning(wc_log2=wc_log2, slots=2, local_kb=1)
    try:
        b = og.Batch([og.GraphSpec(adj, grid=True, width=w, height=h, symmetries=s)])
        assert same(b.run()[0], ref)
        assert same(b.run()[0], ref)          # a second run on the same buffers
        b.close()
    finally:
        og.set_tuning()


def test_batch_workload_sample_against_oracle():
    """The first graphs of the benchmark's batched workload, evaluated
    together, against the oracle one by one."""
    from odp_gb300 import workloads
    shapes = workloads.batch_shapes(512)[:48]
    specs = workloads.build_graphs(shapes)
    got = og.set_aspl_batch(specs)
    for sp, g in zip(specs, got):
        o = oracle.aspl(sp.adjacency, nodes=sp.nodes, symmetries=sp.symmetries, grid=sp.grid, width=sp.width,
                        height=sp.height)
        assert same(g, o), (sp.nodes, sp.grid, sp.symmetries)


@pytest.mark.parametrize("activity", ["0", "1"])
def test_change_tracking_on_and_off(golden, activity, monkeypatch):
    """Both level passes (all neighbours / only neighbours whose words
    changed) on general graphs, grids and the golden edge cases."""
    monkeypatch.setenv("ODP_GB300_ACTIVITY", activity)
    rng = np.random.default_rng(99)
    specs, kws = [], []
    for _ in range(20):
        spec, kw = random_graph(rng)
        specs.append(spec)
        kws.append(kw)
    for c in golden["cases"]:
        if c["kind"] == "general":
            specs.append(og.GraphSpec(case_adjacency(c), nodes=c["nodes"], symmetries=c["symmetries"],
                                      num_degrees=case_degrees(c)))
            kws.append(dict(nodes=c["nodes"], symmetries=c["symmetries"], num_degrees=case_degrees(c)))
    b = og.Batch(specs)
    for g, spec, kw in zip(b.run(), specs, kws):
        assert same(g, oracle.aspl(spec.adjacency, **kw)), kw
    b.close()
    n, d = 4096, 10
    adj = og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, seed=4), d)
    og.set_tuning(wc_log2=3, slots=3, local_kb=1)
    try:
        b = og.Batch([og.GraphSpec(adj, nodes=n)])
        assert same(b.run()[0], oracle.aspl(adj, nodes=n))
        b.close()
    finally:
        og.set_tuning()


def test_learned_job_order():
    """After its first run a plan re-sorts its jobs by measured duration; the
    results, the per-job levels (matched to the new order) and the
    algorithmic byte count stay the same run after run."""
    from odp_gb300 import workloads
    specs = workloads.build_graphs(workloads.batch_shapes(40, first_seed=900, draw_seed=7))
    og.set_tuning(slots=2, local_kb=1)
    try:
        b = og.Batch(specs)
        first = b.run()
        lv1 = sorted(b.job_levels().tolist())
        by1 = b.bytes_alg()
        for _ in range(2):
            again = b.run()
            assert all(same(x, y) for x, y in zip(first, again))
            assert sorted(b.job_levels().tolist()) == lv1
            assert b.bytes_alg() == by1
        g, a, d = b.job_profile()
        assert np.all(d > 0) and np.all(d >= a)
        b.close()
    finally:
        og.set_tuning()
    for sp, r in zip(specs, first):
        o = oracle.aspl(sp.adjacency, nodes=sp.nodes, symmetries=sp.symmetries, grid=sp.grid, width=sp.width,
                        height=sp.height)
        assert same(r, o), (sp.nodes, sp.grid, sp.symmetries)


def test_staged_and_direct_adjacency_give_the_same_results(monkeypatch):
    """Plans read callers' arrays in place when the device can read pageable
    host memory, else through a pinned staging copy; both paths agree with
    each other and with the oracle, run after run with changing arrays."""
    from odp_gb300 import workloads
    specs = workloads.build_graphs(workloads.batch_shapes(24, first_seed=700, draw_seed=11))
    out = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("ODP_GB300_DIRECT", mode)
        b = og.Batch(specs)
        try:
            first = b.run()
            other = [s.adjacency.copy() for s in specs]
            rng = og.Rng(5)
            for k, s in enumerate(specs):           # a few 2-opt swaps on every general graph
                if not s.grid:
                    for _ in range(3):
                        rng.mutate_general(s.nodes, s.degree, other[k], symmetries=s.symmetries)
            second = b.run(other)
            third = b.run()
        finally:
            b.close()
        assert all(same(x, y) for x, y in zip(first, third))
        out[mode] = (first, second)
    assert all(same(x, y) for x, y in zip(out["1"][0], out["0"][0]))
    assert all(same(x, y) for x, y in zip(out["1"][1], out["0"][1]))
    for sp, r in zip(specs[:8], out["1"][0]):
        o = oracle.aspl(sp.adjacency, nodes=sp.nodes, symmetries=sp.symmetries, grid=sp.grid, width=sp.width,
                        height=sp.height)
        assert same(r, o)


def _ref_shape(c, seed=0):
    if c["kind"] == "grid":
        return dict(grid=True, width=c["width"], height=c["height"], degree=c["degree"], length=c.get("length", 0),
                    symmetries=c["symmetries"], seed=seed)
    return dict(grid=False, nodes=c["nodes"], degree=c["degree"], symmetries=c["symmetries"], seed=seed)


def test_reference_cuda_library_agrees(golden):
    """The reference's own libodp_cuda.a, rebuilt for sm_103a and run on this
    GPU in its own process, gives the same diameter, sum and ASPL bits as
    this library on the golden edge cases and the seeded generator graphs
    (cases with num_degrees excepted: the timing driver takes none)."""
    import baseline
    if not baseline.gpu_available():
        pytest.skip("the reference CUDA library is not built here")
    groups = {None: ([], []), "MATRIX_SAVING": ([], [])}
    for c in golden["cases"]:
        if c["num_degrees"] is not None:
            continue
        env = "MATRIX_SAVING" if c["name"].endswith("_matrix_saving") else None
        groups[env][0].append(_ref_shape(c))
        groups[env][1].append(case_adjacency(c))
    for g in golden["generators"]:
        if g.get("big"):
            continue
        groups[None][0].append(_ref_shape(g, g["seed"]))
        groups[None][1].append(gen_record_adjacency(og, g, gen_record_edges(og, g)))
    checked = 0
    for env, (shapes, adjs) in groups.items():
        if not shapes:
            continue
        ref = baseline.time_gpu(shapes, adjs, reps=1, env={"ODP_ASPL": env} if env else None)
        for sh, adj, r in zip(shapes, adjs, ref):
            mine = gpu_aspl(adj, nodes=sh.get("nodes", 0), symmetries=sh["symmetries"], grid=sh["grid"],
                            width=sh.get("width", 0), height=sh.get("height", 0))
            assert same(mine, r[:3]), (sh, mine, r[:3])
            checked += 1
    assert checked >= 40


def test_largest_degree_the_engine_takes():
    """Degree 508: rows of 508 neighbours (512 with padding), so a staged
    block holds only 8 rows; results equal the oracle's."""
    n, d = 1024, 508
    adj = og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, seed=77), d)
    want = oracle.aspl(adj, nodes=n)
    assert same(gpu_aspl(adj, nodes=n), want)
    b = og.Batch([og.GraphSpec(adj, nodes=n)])
    assert b.kernel() == "engine"
    assert same(b.run()[0], want)
    b.close()
