"""The batch autotuner's search (odp_gb300/autotune.py tune_batch) on a
synthetic cost model, without a GPU: the timer, the library's tuning state
and the size buckets are replaced by Python stand-ins, so these tests check
only the search itself."""
import pytest

import odp_gb300 as og
from odp_gb300 import autotune

A, B = (13, 0, 0), (11, 1, 0)          # two (ceil log2 n, degree class, grid) buckets


class Spec:
    def __init__(self, bk, nodes):
        self.bk, self.nodes, self.degree, self.symmetries = bk, nodes, 8, 1
        self.grid, self.width, self.height = False, 0, 0


class Model:
    """ms = a global term from (slots, local_kb) + one term per bucket from
    its table entry; the settings are the ones the tuner installed last."""

    def __init__(self, global_ms, bucket_ms):
        self.global_ms, self.bucket_ms = global_ms, bucket_ms
        self.tuning, self.table = dict(slots=0, local_kb=0), {}

    def set_tuning(self, wc_log2=0, slots=0, tile_rows=0, l2_budget_mb=0, local_kb=0, use_graph=-1):
        self.tuning = dict(slots=slots, local_kb=local_kb)

    def set_table(self, entries):
        self.table = {k: dict(v) for k, v in entries.items()}

    def measure(self, specs, repeats=3, flush_mb=256):
        ms = self.global_ms.get((self.tuning["slots"], self.tuning["local_kb"]), 5.0)
        for bk, f in self.bucket_ms.items():
            e = self.table.get(bk, {})
            ms += f(e.get("wc_log2", 0), e.get("tile_kb", 0))
        return ms


@pytest.fixture
def model(monkeypatch):
    def make(global_ms, bucket_ms):
        m = Model(global_ms, bucket_ms)
        monkeypatch.setattr(og, "set_tuning", m.set_tuning)
        monkeypatch.setattr(autotune, "set_table", m.set_table)
        monkeypatch.setattr(autotune, "measure", m.measure)
        monkeypatch.setattr(autotune, "bucket", lambda spec: spec.bk)
        return m
    return make


def test_finds_the_separable_optimum(model):
    m = model({(64, 256): 4.5, (128, 2048): 4.8},
              {A: lambda wl, tk: {7: 1.0}.get(wl, 2.0) - (0.2 if tk == 1280 else 0.0),
               B: lambda wl, tk: {4: 0.6}.get(wl, 1.0)})
    rep = autotune.tune_batch([Spec(A, 8000), Spec(B, 2000)], slots=(32, 64, 128), local_kb=(256, 2048))
    assert (rep["slots"], rep["local_kb"]) == (64, 256)
    assert m.tuning == dict(slots=64, local_kb=256)
    assert m.table == {A: {"wc_log2": 7, "tile_kb": 1280}, B: {"wc_log2": 4}}
    assert rep["buckets"] == {"13/0/0": {"wc_log2": 7, "tile_kb": 1280}, "11/1/0": {"wc_log2": 4}}
    assert rep["default_ms"] == pytest.approx(5.0 + 2.0 + 1.0)
    assert rep["tuned_ms"] == pytest.approx(4.5 + 0.8 + 0.6)


def test_ignores_gains_below_the_margin(model):
    """Candidates 0.1 % faster than the current choice are timing noise: the
    defaults stay."""
    m = model({(128, 2048): 5.0 * 0.999}, {A: lambda wl, tk: 2.0 * (0.999 if wl == 3 else 1.0)})
    rep = autotune.tune_batch([Spec(A, 8000)], slots=(128,), local_kb=(2048,), min_gain=0.003)
    assert (rep["slots"], rep["local_kb"]) == (0, 0)
    assert m.tuning == dict(slots=0, local_kb=0)
    assert m.table == {}
    assert rep["tuned_ms"] == rep["default_ms"]


def test_second_round_revisits_buckets(model):
    """Bucket B carries more work, so it is tuned first; its best width
    depends on bucket A's, which changes after B was tuned.  The second
    round finds B's new best."""
    m = model({}, {})

    def a(wl, tk):
        return 1.0 if wl == 5 else 2.0

    def b(wl, tk):
        if m.table.get(A, {}).get("wc_log2") == 5:
            return 0.5 if wl == 6 else 1.0
        return 0.9 if wl == 3 else 1.0

    m.bucket_ms = {A: a, B: b}
    rep = autotune.tune_batch([Spec(A, 100), Spec(B, 1000)], slots=(64,), local_kb=(256,), rounds=2)
    assert m.table == {A: {"wc_log2": 5}, B: {"wc_log2": 6}}
    assert rep["tuned_ms"] == pytest.approx(5.0 + 1.0 + 0.5)
    one = model({}, {})
    one.bucket_ms = {A: a, B: lambda wl, tk: (0.5 if wl == 6 else 1.0) if one.table.get(A, {}).get("wc_log2") == 5
                     else (0.9 if wl == 3 else 1.0)}
    autotune.tune_batch([Spec(A, 100), Spec(B, 1000)], slots=(64,), local_kb=(256,), rounds=1)
    assert one.table == {A: {"wc_log2": 5}, B: {"wc_log2": 3}}
