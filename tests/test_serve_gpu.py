"""Serving mode (ODPX_Serve_*): device-resident graphs updated in place by
2-opt deltas, evaluated in continuous batches.  Every result must equal the
same graph evaluated alone (a fresh plan) and the oracle, whatever else was
in flight with it."""
import threading

import numpy as np
import pytest

import odp_gb300 as og
import oracle
from conftest import same

pytestmark = pytest.mark.gpu


def alone(spec_adj, nodes, symmetries):
    b = og.Batch([og.GraphSpec(spec_adj, nodes=nodes, symmetries=symmetries)])
    try:
        return b.run()[0]
    finally:
        b.close()


def chain_graphs():
    out = []
    for i, (n, d, s) in enumerate([(256, 6, 1), (1024, 8, 1), (2048, 12, 4), (4096, 16, 1), (600, 5, 2),
                                   (3000, 10, 1)]):
        adj = og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, s, seed=300 + i), d, s)
        out.append((n, d, s, adj))
    return out


def test_results_alone_and_in_the_mix():
    srv = og.Server(lanes=3, max_batch=4, max_nodes=4096, memory_mb=256)
    chains = chain_graphs()
    handles = [srv.register(og.GraphSpec(adj.copy(), nodes=n, symmetries=s)) for n, d, s, adj in chains]
    results = {}
    errors = []

    def run_chain(k):
        try:
            n, d, s, adj = chains[k]
            host = adj.copy()
            rng = og.Rng(500 + k)
            for step in range(12):
                r = rng.mutate_general(n, d, host, symmetries=s)
                deltas = og.two_opt_deltas(host, r, n, s)
                rid = srv.submit(handles[k], deltas)
                got = srv.wait(rid)
                results[(k, step)] = (got[:3], host.copy())
        except Exception as e:       # surfaced below
            errors.append(e)

    threads = [threading.Thread(target=run_chain, args=(k,)) for k in range(len(chains))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    st = srv.stats()
    assert st["requests_done"] == len(chains) * 12
    for (k, step), (got, host) in results.items():
        n, d, s, _ = chains[k]
        assert same(got, alone(host, n, s)), (k, step)
        if step % 4 == 0:
            assert same(got, oracle.aspl(host, nodes=n, symmetries=s)), (k, step)
    # the resident adjacency followed every delta
    for k, h in enumerate(handles):
        assert np.array_equal(srv.adjacency(h), results[(k, 11)][1])
    srv.close()


def test_reject_restores_through_deltas():
    """An annealing step that is rejected sends the undo of its swap with the
    next request; the served graph must track the client's copy exactly."""
    n, d = 1024, 8
    adj = og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, seed=1), d)
    srv = og.Server(lanes=2, max_batch=2, max_nodes=2048, memory_mb=64)
    h = srv.register(og.GraphSpec(adj.copy(), nodes=n))
    host = adj.copy()
    rng = og.Rng(7)
    pending_undo = []
    current = srv.wait(srv.submit(h))[:3]
    for step in range(20):
        r = rng.mutate_general(n, d, host)
        deltas = pending_undo + og.two_opt_deltas(host, r, n)
        got = srv.wait(srv.submit(h, deltas))[:3]
        assert same(got, oracle.aspl(host, nodes=n))
        if got[2] <= current[2]:
            current, pending_undo = got, []
        else:
            og.Rng.restore_general(n, d, r, host)          # host undo; the server gets it with the next request
            pending_undo = og.two_opt_deltas(host, r, n)
    srv.wait(srv.submit(h, pending_undo))
    assert np.array_equal(srv.adjacency(h), host)
    srv.close()


def test_admission_and_bad_requests():
    srv = og.Server(lanes=1, max_batch=2, max_nodes=512, memory_mb=16)
    big = og.conv_edge2adjacency_general(1024, og.generate_random_general(1024, 4, seed=2), 4)
    with pytest.raises(og.ODPError) as ei:
        srv.register(og.GraphSpec(big, nodes=1024))
    assert ei.value.code == og.ERR_MEMORY
    small = og.conv_edge2adjacency_general(256, og.generate_random_general(256, 4, seed=3), 4)
    h = srv.register(og.GraphSpec(small, nodes=256))
    with pytest.raises(og.ODPError) as ei:
        srv.submit(h, [(0, 0, 999)])
    assert ei.value.code == og.ERR_ADJACENCY
    assert same(srv.wait(srv.submit(h))[:3], oracle.aspl(small, nodes=256))
    srv.close()


def test_delta_past_a_rows_degree_is_refused():
    """With num_degrees, slots past a row's degree hold no edge; a delta that
    targets one is refused, and an accepted delta still matches the graph
    evaluated alone."""
    n, d = 512, 6
    adj = og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, seed=5), d)
    deg = np.full(n, d, dtype=np.int32)
    deg[0] = d - 1
    adj[0, d - 1] = -1
    srv = og.Server(lanes=1, max_batch=2, max_nodes=1024, memory_mb=32)
    h = srv.register(og.GraphSpec(adj.copy(), nodes=n, num_degrees=deg))
    with pytest.raises(og.ODPError) as ei:
        srv.submit(h, [(0, d - 1, 7)])
    assert ei.value.code == og.ERR_ADJACENCY
    host = adj.copy()
    host[1, 0] = 9
    got = srv.wait(srv.submit(h, [(1, 0, 9)]))[:3]
    b = og.Batch([og.GraphSpec(host, nodes=n, num_degrees=deg)])
    try:
        assert same(got, b.run()[0])
    finally:
        b.close()
    assert same(got, oracle.aspl(host, nodes=n, num_degrees=deg))
    srv.close()


def test_served_results_at_the_served_sizes():
    """The served workload's large chains (n = 16384 and 32768, d = 24) share
    lanes, slots and L2 with small ones: every result must still equal the
    same graph evaluated alone, and the oracle at two of the steps."""
    sizes = [(16384, 24), (32768, 24), (1024, 8), (4096, 16), (2048, 8), (32768, 8)]
    chains = []
    for i, (n, d) in enumerate(sizes):
        chains.append((n, d, og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, seed=1000 + i), d)))
    srv = og.Server(lanes=4, max_batch=16, max_nodes=32768, memory_mb=4096)
    handles = [srv.register(og.GraphSpec(adj.copy(), nodes=n)) for n, d, adj in chains]
    steps = 8
    results, errors = {}, []

    def run_chain(k):
        try:
            n, d, adj = chains[k]
            host = adj.copy()
            rng = og.Rng(2000 + k)
            for step in range(steps):
                r = rng.mutate_general(n, d, host)
                got = srv.wait(srv.submit(handles[k], og.two_opt_deltas(host, r, n)))
                results[(k, step)] = (got[:3], host.copy())
        except Exception as e:       # surfaced below
            errors.append(e)

    threads = [threading.Thread(target=run_chain, args=(k,)) for k in range(len(chains))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    st = srv.stats()
    srv.close()
    assert st["requests_done"] == len(chains) * steps
    for k, (n, d, adj) in enumerate(chains):
        b = og.Batch([og.GraphSpec(adj, nodes=n)])
        for step in range(steps):
            got, host = results[(k, step)]
            assert same(got, b.run([host])[0]), (n, d, step)
            if n >= 16384 and step in (3, steps - 1):
                assert same(got, oracle.aspl(host, nodes=n)), (n, d, step)
        b.close()


def test_native_client_chains_match_their_graphs_alone():
    """serve_load (the native client bench.py drives): 12 chains of three
    sizes, one host thread each, first without think time and then with it;
    every chain's last served result must equal its graph evaluated alone
    (the program checks and exits non-zero otherwise)."""
    import json
    import subprocess
    from odp_gb300 import build as b
    chains = ["%d:%d:%d:%d" % (n, d, 3000 + i, 4000 + i)
              for i, (n, d) in enumerate([(1024, 8), (2048, 12), (4096, 16)] * 4)]
    for think_us in ("0", "200"):
        r = subprocess.run([b.SERVE_LOAD, "1.0", think_us, "4", "16", "1024", "50"] + chains, capture_output=True,
                           text=True, timeout=240)
        assert r.returncode == 0, r.stderr[-2000:]
        rep = json.loads(r.stdout.strip().splitlines()[-1])
        assert rep["checked"] == len(chains) and rep["mismatched"] == 0 and rep["errors"] == 0, rep
        assert rep["completed"] > 0
