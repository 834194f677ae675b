"""The autotuner only changes the schedule: results stay bit-exact."""
import pytest

import odp_gb300 as og
import oracle
from conftest import same
from odp_gb300 import autotune, workloads

pytestmark = pytest.mark.gpu


def test_tune_batch_keeps_results():
    specs = workloads.build_graphs(workloads.batch_shapes(512)[:24])
    ref = [oracle.aspl(s.adjacency, nodes=s.nodes, symmetries=s.symmetries, grid=s.grid, width=s.width,
                       height=s.height) for s in specs]
    try:
        rep = autotune.tune_batch(specs, slots=(16, 64), local_kb=(512,), widths=(3, 5), repeats=1, max_buckets=3)
        assert rep["tuned_ms"] <= rep["default_ms"] * 1.5
        b = og.Batch(specs)
        for g, r in zip(b.run(), ref):
            assert same(g, r)
        b.close()
    finally:
        autotune.clear()


def test_tune_batch_best_of_two_starts():
    specs = workloads.build_graphs(workloads.batch_shapes(512)[:24])
    ref = [oracle.aspl(s.adjacency, nodes=s.nodes, symmetries=s.symmetries, grid=s.grid, width=s.width,
                       height=s.height) for s in specs]
    try:
        rep = autotune.tune_batch_best(specs, starts=2, repeats=2, slots=(16, 64), local_kb=(512,), widths=(3, 5),
                                       max_buckets=2)
        assert len(rep["starts_ms"]) == 2 and rep["tuned_ms"] == min(rep["starts_ms"])
        b = og.Batch(specs)
        for g, r in zip(b.run(), ref):
            assert same(g, r)
        b.close()
    finally:
        autotune.clear()


def test_tune_single_keeps_results():
    n, d = 8192, 12
    adj = og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, seed=5), d)
    spec = og.GraphSpec(adj, nodes=n)
    try:
        autotune.tune_single(spec, widths=(3, 5), slots=(2, 8), tile_kb=(128,), repeats=1)
        b = og.Batch([spec])
        assert same(b.run()[0], oracle.aspl(adj, nodes=n))
        b.close()
    finally:
        autotune.clear()
