"""Packs the reference's 256x256 grid graph (d=6, length 4, seed 4, produced
by ODP_Srand(4); ODP_Generate_random_grid(256, 256, 6, 4, edge)) into
tests/golden/grid_256x256_d6_l4_seed4.npz, because regenerating it takes
minutes on a CPU.  Each adjacency entry (rows from
ODP_Conv_edge2adjacency_grid) is stored as one byte, its lattice offset
(dx + 4) * 9 + (dy + 4) from the row's vertex, then zlib-compressed by
np.savez_compressed.

    python tests/golden/make_grid_fixture.py REFERENCE_EDGE_FILE

REFERENCE_EDGE_FILE holds the generator's raw int32 edge pairs (for example
from oracle/_ref/ref_driver gen grid 256 256 6 4 1 4 FILE).
"""
import hashlib
import os
import sys

import numpy as np

W = H = 256
D, L = 6, 4
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "grid_256x256_d6_l4_seed4.npz")


def edges_to_rows(edges, n, d):
    adj = -np.ones((n, d), dtype=np.int32)
    cnt = np.zeros(n, dtype=np.int64)
    for a, b in edges:
        adj[a, cnt[a]] = b
        cnt[a] += 1
        adj[b, cnt[b]] = a
        cnt[b] += 1
    return adj


def encode(adj):
    v = np.arange(W * H)[:, None]
    dx = adj // H - v // H
    dy = adj % H - v % H
    assert np.all(np.abs(dx) + np.abs(dy) <= L)
    return ((dx + L) * (2 * L + 1) + (dy + L)).astype(np.uint8)


def decode(codes):
    v = np.arange(W * H)[:, None]
    dx = codes.astype(np.int32) // (2 * L + 1) - L
    dy = codes.astype(np.int32) % (2 * L + 1) - L
    return ((v // H + dx) * H + (v % H + dy)).astype(np.int32)


def main(path):
    edges = np.fromfile(path, dtype=np.int32).reshape(-1, 2)
    adj = edges_to_rows(edges, W * H, D)
    codes = encode(adj)
    assert np.array_equal(decode(codes), adj)
    np.savez_compressed(OUT, codes=codes,
                        edges_sha256=np.frombuffer(hashlib.sha256(edges.tobytes()).hexdigest().encode(), np.uint8),
                        adjacency_sha256=np.frombuffer(hashlib.sha256(adj.tobytes()).hexdigest().encode(), np.uint8))
    print("wrote %s (%d bytes)" % (OUT, os.path.getsize(OUT)))


if __name__ == "__main__":
    main(sys.argv[1])
