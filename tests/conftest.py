"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on a
CPU-only machine (the product library loads there for its host utilities;
its ASPL entry points need a GPU)."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _ensure_built():
    from odp_gb300 import build as b
    srcs = [os.path.join(b.CSRC, f) for f in os.listdir(b.CSRC)] + [os.path.join(ROOT, "include", f)
                                                                  for f in os.listdir(os.path.join(ROOT, "include"))]
    if not os.path.exists(b.SO_PATH) or os.path.getmtime(b.SO_PATH) < max(os.path.getmtime(s) for s in srcs):
        b.build()
    import oracle
    oracle.build()


@pytest.fixture(scope="session", autouse=True)
def built():
    _ensure_built()


@pytest.fixture(scope="session")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def result_tuple(r):
    """[diameter, sum, ASPL-hex] -> comparable tuple."""
    return (int(r[0]), int(r[1]), float.fromhex(r[2]))


def same(a, b):
    """Bit-exact comparison of (diameter, sum, ASPL) tuples (NaN == NaN)."""
    if a[0] != b[0] or a[1] != b[1]:
        return False
    x, y = float(a[2]), float(b[2])
    return (x != x and y != y) or x.hex() == y.hex()


def case_adjacency(c):
    n = c["width"] * c["height"] if c["kind"] == "grid" else c["nodes"]
    return np.array(c["adjacency"], dtype=np.int32).reshape(n // c["symmetries"], c["degree"])


def case_degrees(c):
    return None if c.get("num_degrees") is None else np.array(c["num_degrees"], dtype=np.int32)


def edges_to_adjacency(n, degree, edges, symmetries=1):
    """numpy restatement of ODP_Conv_edge2adjacency_general_s (rows in edge order)."""
    base = n // symmetries
    adj = -np.ones((base, degree), dtype=np.int32)
    cnt = np.zeros(base, dtype=np.int64)
    for a, b in np.asarray(edges).reshape(-1, 2):
        if a < base:
            adj[a, cnt[a]] = b
            cnt[a] += 1
        if b < base:
            adj[b, cnt[b]] = a
            cnt[b] += 1
    return adj


def gen_record_edges(og, g):
    """Edges of a generator record through the library's seeded generators."""
    if g["kind"] == "general":
        return og.generate_random_general(g["nodes"], g["degree"], g["symmetries"], seed=g["seed"])
    return og.generate_random_grid(g["width"], g["height"], g["degree"], g["length"], g["symmetries"], seed=g["seed"])


def gen_record_adjacency(og, g, edges):
    if g["kind"] == "general":
        return og.conv_edge2adjacency_general(g["nodes"], edges, g["degree"], g["symmetries"])
    return og.conv_edge2adjacency_grid(g["width"], g["height"], edges, g["degree"], g["symmetries"])


def sha256(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes()).hexdigest()
