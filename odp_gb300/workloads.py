"""Seeded synthetic workloads for benchmarks and tests.

The batched workload models many independent evaluations of uneven graphs:
512 graphs with seeds 100..611, n log-uniform in [256, 8192], d uniform in
{4, 6, ..., 32}, 80 % general / 20 % grid graphs (side = round(sqrt(n)),
length limit uniform in 3..6), symmetry s uniform over {1, 2, 4} where the
generator allows it (general: n % s == 0; grid: s = 2 or 4 needs an even
side).  The draw itself uses splitmix64 seeded with 100, so the list of
shapes is fixed; each graph is then built by the library's seeded generator
(the reference generator's graph for that seed).

The served workload models simulated-annealing chains: chain i has
n = (1024, 4096, 16384, 32768)[i % 4], d = (8, 16, 24)[(i // 4) % 3], graph seed
1000 + i, and proposes 2-opt swaps from its own random stream (seed 2000 + i).
"""
import math
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

MASK = (1 << 64) - 1


class SplitMix64:
    """splitmix64 (Steele, Lea, Flood 2014): x += 0x9E3779B97F4A7C15, then mix."""

    def __init__(self, seed):
        self.x = seed & MASK

    def next(self):
        self.x = (self.x + 0x9E3779B97F4A7C15) & MASK
        z = self.x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        return z ^ (z >> 31)

    def uniform(self):
        return (self.next() >> 11) * (1.0 / (1 << 53))


def batch_shapes(count=512, first_seed=100, draw_seed=100, n_lo=256, n_hi=8192):
    """The list of graph shapes of the batched workload (dicts)."""
    rng = SplitMix64(draw_seed)
    out = []
    for i in range(count):
        grid = rng.uniform() < 0.2
        n = int(round(math.exp(math.log(n_lo) + rng.uniform() * (math.log(n_hi) - math.log(n_lo)))))
        d = 4 + 2 * int(rng.uniform() * 15)
        if grid:
            side = max(4, int(round(math.sqrt(n))))
            length = 3 + int(rng.uniform() * 4)
            valid = [1, 2, 4] if side % 2 == 0 else [1]
            s = valid[int(rng.uniform() * len(valid))]
            out.append(dict(grid=True, width=side, height=side, nodes=side * side, degree=d, length=length,
                            symmetries=s, seed=first_seed + i))
        else:
            valid = [s for s in (1, 2, 4) if n % s == 0]
            s = valid[int(rng.uniform() * len(valid))]
            out.append(dict(grid=False, nodes=n, degree=d, symmetries=s, seed=first_seed + i))
    return out


def build_graph(shape):
    """GraphSpec for one shape (the reference generator's graph for its seed)."""
    import odp_gb300 as og
    if shape["grid"]:
        e = og.generate_random_grid(shape["width"], shape["height"], shape["degree"], shape["length"],
                                    shape["symmetries"], seed=shape["seed"])
        adj = og.conv_edge2adjacency_grid(shape["width"], shape["height"], e, shape["degree"], shape["symmetries"])
        return og.GraphSpec(adj, grid=True, width=shape["width"], height=shape["height"],
                            symmetries=shape["symmetries"])
    e = og.generate_random_general(shape["nodes"], shape["degree"], shape["symmetries"], seed=shape["seed"])
    adj = og.conv_edge2adjacency_general(shape["nodes"], e, shape["degree"], shape["symmetries"])
    return og.GraphSpec(adj, nodes=shape["nodes"], symmetries=shape["symmetries"])


def build_graphs(shapes, threads=None):
    """GraphSpecs for many shapes, generated concurrently (the seeded
    generators are thread-safe and release the GIL)."""
    threads = threads or max(1, min(32, os.cpu_count() or 1))
    # longest first: grid graphs cost ~ n^2 d / length^2
    cost = [(s["nodes"] ** 2 * s["degree"] / (s.get("length", 30) ** 2), i) for i, s in enumerate(shapes)]
    order = [i for _, i in sorted(cost, reverse=True)]
    out = [None] * len(shapes)
    with ThreadPoolExecutor(max_workers=threads) as ex:
        for i, g in zip(order, ex.map(lambda k: build_graph(shapes[k]), order)):
            out[i] = g
    return out


def chain_shapes(chains=64):
    """Shapes of the served annealing chains."""
    sizes = (1024, 4096, 16384, 32768)
    degrees = (8, 16, 24)
    return [dict(grid=False, nodes=sizes[i % 4], degree=degrees[(i // 4) % 3], symmetries=1, seed=1000 + i,
                 proposal_seed=2000 + i) for i in range(chains)]


def algorithmic_bytes(spec, levels, wc_log2):
    """Bytes of one evaluation by the roofline formula: per column chunk,
    levels x 8 x words x sum over vertices of (degree + 2)."""
    n = spec.width * spec.height if spec.grid else spec.nodes
    if spec.num_degrees is None:
        per_level = float(n) * (spec.degree + 2)
    else:
        per_level = float(np.sum(np.tile(spec.num_degrees, spec.symmetries)[:n] + 2))
    return 8.0 * (1 << wc_log2) * per_level * float(np.sum(np.abs(levels)))
