"""Annealing chains on the GPU (ODPX_Anneal_*) against the reference's
annealing loop restated on the host: sample/SA/general.c:160-191,
general_s.c:170-191, grid.c:170-191 and grid_s.c:180-201 (Mutate, Set_aspl,
best tracking, accept_s, Restore when
rejected, temp *= cooling_rate) with accept_s and uniform_rand from
sample/SA/common.c:10-37.  On the host the 2-opt swaps come from the library's
host utilities on the same private stream (ODP_Srand(seed) equivalent) and the
oracle evaluates every proposal; the device chains must make the same moves
and report the same results bit for bit."""
import math

import numpy as np
import pytest

import odp_gb300 as og
import oracle
from conftest import same

pytestmark = pytest.mark.gpu


class HostChain:
    """The reference client's loop, one step at a time."""

    def __init__(self, c):
        self.c = c
        self.adj = c.adjacency.copy()
        self.rng = og.Rng(c.seed)
        r = self.evaluate()
        self.cur, self.best, self.best_adj = r, r, self.adj.copy()
        self.temp = 0.0 if c.hill_climbing else c.max_temp
        self.cooling = 0.0 if c.hill_climbing else math.pow(c.min_temp / c.max_temp, 1.0 / c.ncalcs)
        self.steps = self.accepted = 0

    def evaluate(self):
        c = self.c
        if c.grid:
            return tuple(oracle.aspl(self.adj, symmetries=c.symmetries, num_degrees=c.num_degrees, grid=True,
                                     width=c.width, height=c.height))
        return tuple(oracle.aspl(self.adj, nodes=c.nodes, symmetries=c.symmetries, num_degrees=c.num_degrees))

    def accept(self, d, a):                     # accept_s, common.c:15-37
        c = self.c
        if c.hill_climbing:
            return a <= self.cur[2]
        if d < self.cur[0] and not c.aspl_priority:
            return True
        if d > self.cur[0] and not c.aspl_priority:
            return False
        if a <= self.cur[2]:
            return True
        diff = ((self.cur[2] - a) * c.nodes * (c.nodes - 1)) / c.symmetries
        u = (self.rng.next() + 1.0) / (2147483647.0 + 2.0)
        return math.exp(diff / self.temp) > u

    def step(self):
        c = self.c
        if c.grid:
            r = self.rng.mutate_grid(c.width, c.height, c.degree, c.length, self.adj, symmetries=c.symmetries,
                                     num_degrees=c.num_degrees)
        else:
            r = self.rng.mutate_general(c.nodes, c.degree, self.adj, symmetries=c.symmetries,
                                        num_degrees=c.num_degrees)
        d, s, a = self.evaluate()
        self.steps += 1
        if d < self.best[0] or (d == self.best[0] and a < self.best[2]):
            self.best, self.best_adj = (d, s, a), self.adj.copy()
        if self.accept(d, a):
            self.cur = (d, s, a)
            self.accepted += 1
        elif c.grid:
            og.Rng.restore_grid(c.width, c.height, c.degree, r, self.adj, symmetries=c.symmetries)
        else:
            og.Rng.restore_general(c.nodes, c.degree, r, self.adj, symmetries=c.symmetries)
        self.temp *= self.cooling


def general(n, d, s=1, seed=1):
    return og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, s, seed=seed), d, s)


def irregular(n, d, seed):
    """A regular graph with one edge dropped: both end rows get degree d-1,
    the dropped edge moved to their last slots."""
    adj = general(n, d, seed=seed)
    u, v = 0, int(adj[0, d - 1])
    assert v != u
    j = int(np.nonzero(adj[v] == u)[0][0])
    adj[v, j], adj[v, d - 1] = adj[v, d - 1], adj[v, j]
    adj[u, d - 1] = adj[v, d - 1] = -1
    deg = np.full(n, d, dtype=np.int32)
    deg[u] = deg[v] = d - 1
    return adj, deg


def chains():
    irr, deg = irregular(96, 5 + 1, seed=9)
    return [
        og.Chain(general(128, 4, seed=11), 128, seed=3, max_temp=20.0, min_temp=0.2, ncalcs=60),
        og.Chain(general(120, 5, 4, seed=12), 120, symmetries=4, seed=4, max_temp=40.0, min_temp=0.5, ncalcs=60),
        og.Chain(general(100, 6, 2, seed=13), 100, symmetries=2, seed=5, max_temp=10.0, min_temp=0.1, ncalcs=60),
        og.Chain(general(64, 3, seed=14), 64, seed=6, hill_climbing=True),
        og.Chain(general(90, 4, seed=15), 90, seed=7, max_temp=30.0, min_temp=0.3, ncalcs=60, aspl_priority=True),
        og.Chain(irr, 96, num_degrees=deg, seed=8, max_temp=15.0, min_temp=0.2, ncalcs=60),
    ]


def test_device_chains_follow_the_reference_loop():
    cs = chains()
    host = [HostChain(c) for c in cs]
    dev = og.Anneal(cs)
    try:
        for k, h in enumerate(host):
            st = dev.state(k)
            assert same((st["diameter"], st["sum"], st["aspl"]), h.cur), k
        for run in (7, 13, 20):
            dev.run(run)
            for h in host:
                for _ in range(run):
                    h.step()
            for k, h in enumerate(host):
                st = dev.state(k, graphs=True)
                assert st["status"] == 0, (k, st["status"])
                assert st["steps"] == h.steps and st["accepted"] == h.accepted, (k, st, h.accepted)
                assert same((st["diameter"], st["sum"], st["aspl"]), h.cur), k
                assert same((st["best_diameter"], st["best_sum"], st["best_aspl"]), h.best), k
                assert float(st["temp"]).hex() == float(h.temp).hex(), k
                assert np.array_equal(st["adjacency"], h.adj), k
                assert np.array_equal(st["best_adjacency"], h.best_adj), k
        assert any(0 < h.accepted < h.steps for h in host)   # both outcomes were exercised
    finally:
        dev.close()


def grid(w, h, d, length, s=1, seed=1):
    e = og.generate_random_grid(w, h, d, length, s, seed=seed)
    return og.conv_edge2adjacency_grid(w, h, e, d, s)


def test_device_grid_chains_follow_the_reference_loop():
    """sample/SA/grid.c:170-191 and grid_s.c:180-201: the grid 2-opt with its
    length limit, for s = 1, 2 and 4."""
    cs = [og.Chain(grid(12, 12, 4, 3, seed=41), grid=True, width=12, height=12, length=3, seed=51, max_temp=20.0,
                   min_temp=0.2, ncalcs=60),
          og.Chain(grid(12, 10, 4, 4, 2, seed=42), grid=True, width=12, height=10, length=4, symmetries=2, seed=52,
                   max_temp=20.0, min_temp=0.2, ncalcs=60),
          og.Chain(grid(12, 12, 6, 3, 4, seed=43), grid=True, width=12, height=12, length=3, symmetries=4, seed=53,
                   max_temp=20.0, min_temp=0.2, ncalcs=60),
          og.Chain(grid(10, 10, 4, 5, seed=44), grid=True, width=10, height=10, length=5, seed=54, hill_climbing=True)]
    host = [HostChain(c) for c in cs]
    dev = og.Anneal(cs)
    try:
        for run in (9, 21):
            dev.run(run)
            for h in host:
                for _ in range(run):
                    h.step()
            for k, h in enumerate(host):
                st = dev.state(k, graphs=True)
                assert st["status"] == 0, (k, st["status"])
                assert st["steps"] == h.steps and st["accepted"] == h.accepted, (k, st, h.accepted)
                assert same((st["diameter"], st["sum"], st["aspl"]), h.cur), k
                assert same((st["best_diameter"], st["best_sum"], st["best_aspl"]), h.best), k
                assert np.array_equal(st["adjacency"], h.adj), k
                assert np.array_equal(st["best_adjacency"], h.best_adj), k
        assert any(0 < h.accepted < h.steps for h in host)
    finally:
        dev.close()


def test_device_chain_results_match_their_graphs():
    """Larger chains, no host replay: the reported current and best results
    are those of the graphs the device holds."""
    cs = [og.Chain(general(4096, 16, seed=21), 4096, seed=31, max_temp=50.0, min_temp=1.0, ncalcs=40),
          og.Chain(general(2048, 12, 2, seed=22), 2048, symmetries=2, seed=32, max_temp=50.0, min_temp=1.0,
                   ncalcs=40)]
    dev = og.Anneal(cs)
    try:
        dev.run(40)
        for k, c in enumerate(cs):
            st = dev.state(k, graphs=True)
            assert st["status"] == 0 and st["steps"] == 40
            b = og.Batch([og.GraphSpec(st["adjacency"], nodes=c.nodes, symmetries=c.symmetries),
                          og.GraphSpec(st["best_adjacency"], nodes=c.nodes, symmetries=c.symmetries)])
            try:
                cur, best = b.run()
            finally:
                b.close()
            assert same(cur, (st["diameter"], st["sum"], st["aspl"]))
            assert same(best, (st["best_diameter"], st["best_sum"], st["best_aspl"]))
            assert (best[0], best[2]) <= (cur[0], cur[2])
    finally:
        dev.close()


def test_bad_chains_are_refused():
    adj = general(64, 4, seed=1)
    with pytest.raises(og.ODPError) as ei:
        og.Anneal([og.Chain(adj, 63)])                       # 63 % 1 == 0 but the adjacency is 64 rows
    assert ei.value.code in (og.ERR_INVALID, og.ERR_ADJACENCY)
    with pytest.raises(og.ODPError) as ei:
        og.Anneal([og.Chain(adj, 64, symmetries=3)])
    assert ei.value.code == og.ERR_INVALID
    with pytest.raises(og.ODPError) as ei:
        og.Anneal([og.Chain(adj, 64, max_temp=0.0)])
    assert ei.value.code == og.ERR_INVALID
