"""Generates tests/golden/golden.json from the REFERENCE library itself.

Run in a checkout where the reference tree is present (default
/root/reference, override with ODP_REFERENCE_DIR) after
``make -C oracle ref``.  Every expected value in the output comes from the
reference's own code: its sample golden tables (sample/graph/*/ASPL.txt), its
generators (sha256 of the edge lists), its ASPL driver (libodp.a via
oracle/_ref/ref_driver) and its 2-opt mutation.  The committed JSON is what
the tests check the oracle and the GPU library against on machines without
the reference.

    python tests/golden/make_golden.py [--big]

--big also records the large benchmark fixtures (n=65536 and n=262144
graphs, the 256x256 grid); their edge lists are not stored, only hashes and
results, so the tests regenerate them with the library's seeded generators.
"""
import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF = os.environ.get("ODP_REFERENCE_DIR", "/root/reference")
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
OUT = os.path.join(ROOT, "tests", "golden", "golden.json")
TMP = tempfile.mkdtemp(prefix="odp_golden_")


def run(*args, env=None):
    e = dict(os.environ)
    e.pop("ODP_ASPL", None)
    if env:
        e.update(env)
    r = subprocess.run([DRIVER] + [str(a) for a in args], capture_output=True, text=True, env=e)
    if r.returncode != 0:
        raise RuntimeError("ref_driver %s failed: %s" % (args, r.stderr))
    return r.stdout


def tmp(name):
    return os.path.join(TMP, name)


def ref_aspl_general(n, d, s, adj, num_degrees=None, kind=None):
    adj = np.ascontiguousarray(adj, dtype=np.int32)
    adj.tofile(tmp("adj"))
    nd = "-"
    if num_degrees is not None:
        np.ascontiguousarray(num_degrees, dtype=np.int32).tofile(tmp("nd"))
        nd = tmp("nd")
    out = run("aspl", "general", n, d, s, tmp("adj"), nd, env={"ODP_ASPL": kind} if kind else None)
    dia, sm, hx, _ = out.split()
    return [int(dia), int(sm), hx]


def ref_aspl_grid(w, h, d, s, adj, num_degrees=None, kind=None):
    adj = np.ascontiguousarray(adj, dtype=np.int32)
    adj.tofile(tmp("adj"))
    nd = "-"
    if num_degrees is not None:
        np.ascontiguousarray(num_degrees, dtype=np.int32).tofile(tmp("nd"))
        nd = tmp("nd")
    out = run("aspl", "grid", w, h, d, s, tmp("adj"), nd, env={"ODP_ASPL": kind} if kind else None)
    dia, sm, hx, _ = out.split()
    return [int(dia), int(sm), hx]


def ref_gen_general(n, d, s, seed):
    run("gen", "general", n, d, s, seed, tmp("e"))
    return np.fromfile(tmp("e"), dtype=np.int32).reshape(-1, 2)


def ref_gen_grid(w, h, d, length, s, seed):
    run("gen", "grid", w, h, d, length, s, seed, tmp("e"))
    return np.fromfile(tmp("e"), dtype=np.int32).reshape(-1, 2)


def ref_conv_general(n, d, s, edges):
    np.ascontiguousarray(edges, dtype=np.int32).tofile(tmp("e"))
    run("conv", "general", n, d, s, tmp("e"), tmp("a"))
    return np.fromfile(tmp("a"), dtype=np.int32).reshape(n // s, d)


def ref_conv_grid(w, h, d, s, edges):
    np.ascontiguousarray(edges, dtype=np.int32).tofile(tmp("e"))
    run("conv", "grid", w, h, d, s, tmp("e"), tmp("a"))
    return np.fromfile(tmp("a"), dtype=np.int32).reshape(w * h // s, d)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes()).hexdigest()


def flat(a):
    return [int(x) for x in np.asarray(a).reshape(-1)]


# ---------------------------------------------------------------- samples
def parse_aspl_txt(path):
    recs = []
    for block in re.findall(r"Diameter     = (\d+)\n.*?\nASPL         = ([0-9.]+) \((\d+)/", open(path).read(), re.S):
        recs.append({"diameter": int(block[0]), "aspl": block[1], "sum": int(block[2])})
    return recs


def samples():
    out = []
    gen_files = ["n12d3.edges", "n16d4.edges", "n72d4.edges", "n100d10.edges", "n256d5.edges", "n256d10.edges"]
    grid_files = ["w4h4d3r2.edges", "w5h5d4r2.edges", "w10h10d6r3.edges", "w10h10d8r4.edges"]
    for kind, files, table in (("general", gen_files, "sample/graph/general/ASPL.txt"),
                               ("grid", grid_files, "sample/graph/grid/ASPL.txt")):
        exp = parse_aspl_txt(os.path.join(REF, table))
        assert len(exp) == len(files)
        for f, e in zip(files, exp):
            path = os.path.join(REF, "sample/graph", kind, f)
            rec = {"file": f, "kind": kind, "expected": e, "source": "sample/graph/%s/ASPL.txt" % kind}
            if kind == "general":
                edges = np.loadtxt(path, dtype=np.int64).astype(np.int32).reshape(-1, 2)
            else:
                rows = [re.split(r"[ ,]+", ln.strip()) for ln in open(path) if ln.strip()]
                xy = np.array(rows, dtype=np.int64)
                w = int(max(xy[:, 0].max(), xy[:, 2].max())) + 1
                h = int(max(xy[:, 1].max(), xy[:, 3].max())) + 1
                edges = np.stack([xy[:, 0] * h + xy[:, 1], xy[:, 2] * h + xy[:, 3]], 1).astype(np.int32)
                rec["width"], rec["height"] = w, h
            rec["edges"] = flat(edges)
            out.append(rec)
    # symmetric fixtures in the same folders have no golden table: the
    # reference library supplies their values
    sym = [("general", "n24d4g4.edges", 4), ("grid", "w6h6d3r2g2.edges", 2), ("grid", "w6h6d3r2g4.edges", 4),
           ("grid", "w10h10d4r4g4.edges", 4), ("grid", "w4h6d3r2.edges", 1)]
    for kind, f, s in sym:
        path = os.path.join(REF, "sample/graph", kind, f)
        if kind == "general":
            edges = np.loadtxt(path, dtype=np.int64).astype(np.int32).reshape(-1, 2)
            n = int(edges.max()) + 1
            deg = int(np.bincount(edges.reshape(-1), minlength=n).max())
            adj = ref_conv_general(n, deg, s, edges)
            res = ref_aspl_general(n, deg, s, adj)
            out.append({"file": f, "kind": kind, "symmetries": s, "nodes": n, "degree": deg,
                        "edges": flat(edges), "reference": res})
        else:
            rows = [re.split(r"[ ,]+", ln.strip()) for ln in open(path) if ln.strip()]
            xy = np.array(rows, dtype=np.int64)
            w = int(max(xy[:, 0].max(), xy[:, 2].max())) + 1
            h = int(max(xy[:, 1].max(), xy[:, 3].max())) + 1
            edges = np.stack([xy[:, 0] * h + xy[:, 1], xy[:, 2] * h + xy[:, 3]], 1).astype(np.int32)
            deg = int(np.bincount(edges.reshape(-1), minlength=w * h).max())
            adj = ref_conv_grid(w, h, deg, s, edges)
            res = ref_aspl_grid(w, h, deg, s, adj)
            out.append({"file": f, "kind": kind, "symmetries": s, "width": w, "height": h, "degree": deg,
                        "edges": flat(edges), "reference": res})
    return out


# ---------------------------------------------------------- generators
GEN_SMALL = [("general", 1024, 8, 1, 1), ("general", 100, 10, 1, 7), ("general", 256, 5, 1, 3),
             ("general", 96, 6, 4, 5), ("general", 120, 7, 8, 9), ("general", 640, 4, 64, 2),
             ("general", 1000, 6, 10, 11), ("general", 512, 3, 2, 4), ("general", 4096, 8, 2, 21),
             ("general", 2048, 16, 4, 22), ("general", 6000, 12, 1, 23), ("general", 8192, 32, 1, 24)]
GRID_SMALL = [(4, 4, 3, 2, 1, 1), (5, 5, 4, 2, 1, 2), (10, 10, 6, 3, 1, 3), (6, 6, 3, 2, 2, 4), (6, 6, 3, 2, 4, 5),
              (10, 10, 4, 4, 4, 6), (4, 6, 3, 2, 2, 7), (12, 12, 5, 3, 4, 8), (14, 14, 5, 3, 4, 9),
              (10, 6, 6, 3, 2, 10), (20, 12, 6, 4, 2, 11), (16, 16, 4, 3, 4, 12), (7, 9, 4, 3, 1, 13),
              (30, 30, 8, 3, 1, 14), (32, 32, 6, 4, 4, 15), (40, 20, 8, 5, 2, 16)]


def generators(big):
    out = []
    for kind, n, d, s, seed in GEN_SMALL:
        e = ref_gen_general(n, d, s, seed)
        adj = ref_conv_general(n, d, s, e)
        out.append({"kind": kind, "nodes": n, "degree": d, "symmetries": s, "seed": seed, "sha256": sha(e),
                    "reference": ref_aspl_general(n, d, s, adj)})
    for w, h, d, length, s, seed in GRID_SMALL:
        e = ref_gen_grid(w, h, d, length, s, seed)
        adj = ref_conv_grid(w, h, d, s, e)
        out.append({"kind": "grid", "width": w, "height": h, "degree": d, "length": length, "symmetries": s,
                    "seed": seed, "sha256": sha(e), "reference": ref_aspl_grid(w, h, d, s, adj)})
    if big:
        # config 2: n=65536, d=16, seed 2, reference run with ODP_ASPL=MATRIX_SAVING
        e = ref_gen_general(65536, 16, 1, 2)
        adj = ref_conv_general(65536, 16, 1, e)
        out.append({"kind": "general", "nodes": 65536, "degree": 16, "symmetries": 1, "seed": 2, "sha256": sha(e),
                    "reference": ref_aspl_general(65536, 16, 1, adj, kind="MATRIX_SAVING"), "big": True,
                    "name": "single_large_65536"})
        for name, path, rec in (("symmetric_262144", os.environ.get("ODP_GOLDEN_C3"),
                                 {"kind": "general", "nodes": 262144, "degree": 24, "symmetries": 64, "seed": 3}),
                                ("grid_256x256", os.environ.get("ODP_GOLDEN_G"),
                                 {"kind": "grid", "width": 256, "height": 256, "degree": 6, "length": 4,
                                  "symmetries": 1, "seed": 4})):
            if not path or not os.path.exists(path):
                print("skipping %s (set ODP_GOLDEN_C3 / ODP_GOLDEN_G to the reference edge file)" % name)
                continue
            e = np.fromfile(path, dtype=np.int32).reshape(-1, 2)
            if rec["kind"] == "general":
                adj = ref_conv_general(rec["nodes"], rec["degree"], rec["symmetries"], e)
                res = ref_aspl_general(rec["nodes"], rec["degree"], rec["symmetries"], adj)
            else:
                adj = ref_conv_grid(rec["width"], rec["height"], rec["degree"], 1, e)
                res = ref_aspl_grid(rec["width"], rec["height"], rec["degree"], 1, adj)
            rec.update({"sha256": sha(e), "reference": res, "big": True, "name": name})
            out.append(rec)
    return out


# ------------------------------------------------------------ edge cases
def random_nonregular(rng, n, max_deg, directed=False, components=1):
    """Random multigraph adjacency with per-vertex degrees <= max_deg."""
    adj = -np.ones((n, max_deg), dtype=np.int32)
    deg = np.zeros(n, dtype=np.int32)
    comp = np.arange(n) % components
    if directed:            # a directed ring keeps every vertex reachable
        adj[:, 0] = (np.arange(n) + 1) % n
        deg[:] = 1
    for _ in range(n * max_deg):
        u = int(rng.integers(n))
        cand = np.flatnonzero(comp == comp[u])
        v = int(cand[rng.integers(len(cand))])
        if deg[u] >= max_deg:
            continue
        if directed:
            adj[u, deg[u]] = v
            deg[u] += 1
        else:
            if deg[v] >= max_deg or (u == v and deg[u] + 2 > max_deg):
                continue
            adj[u, deg[u]] = v
            deg[u] += 1
            adj[v, deg[v]] = u
            deg[v] += 1
    return adj, deg


def cases():
    rng = np.random.default_rng(20261203)
    out = []

    def add_general(name, n, d, s, adj, nd=None, kinds=(None,)):
        for k in kinds:
            res = ref_aspl_general(n, d, s, adj, nd, kind=k)
            out.append({"name": name + ("" if k is None else "_" + k.lower()), "kind": "general", "nodes": n,
                        "degree": d, "symmetries": s, "num_degrees": None if nd is None else flat(nd),
                        "adjacency": flat(adj), "reference": res, "aspl_kind": k})

    def add_grid(name, w, h, d, s, adj, nd=None):
        res = ref_aspl_grid(w, h, d, s, adj, nd)
        out.append({"name": name, "kind": "grid", "width": w, "height": h, "degree": d, "symmetries": s,
                    "num_degrees": None if nd is None else flat(nd), "adjacency": flat(adj), "reference": res})

    # regular generated graphs across symmetries, n/s below and off multiples of 64
    for n, d, s, seed in [(200, 6, 1, 31), (130, 5, 1, 32), (2000, 7, 1, 33), (96, 6, 4, 34), (120, 7, 8, 35),
                          (640, 4, 64, 36), (4096, 8, 2, 37), (300, 4, 3, 38), (64, 3, 1, 39), (66, 4, 2, 40)]:
        e = ref_gen_general(n, d, s, seed)
        add_general("gen_n%dd%ds%d" % (n, d, s), n, d, s, ref_conv_general(n, d, s, e),
                    kinds=(None, "MATRIX_SAVING") if n >= 2000 else (None,))
    for w, h, d, length, s, seed in [(10, 6, 6, 3, 2, 41), (12, 12, 5, 3, 4, 42), (16, 12, 5, 2, 1, 43),
                                     (20, 12, 6, 4, 2, 44), (16, 16, 4, 3, 4, 45), (9, 7, 4, 3, 1, 46)]:
        e = ref_gen_grid(w, h, d, length, s, seed)
        add_grid("grid_w%dh%dd%ds%d" % (w, h, d, s), w, h, d, s, ref_conv_grid(w, h, d, s, e))
    # non-regular graphs (num_degrees, -1 padding)
    for n, dmax in [(50, 5), (129, 7), (300, 9)]:
        adj, deg = random_nonregular(rng, n, dmax)
        add_general("nonreg_n%d" % n, n, dmax, 1, adj, deg)
    # non-regular with general symmetry: per-base-row degrees tiled over orbits
    for n, dmax, s in [(96, 5, 4), (200, 6, 8)]:
        base = n // s
        adj, deg = random_nonregular(rng, base, dmax, directed=True)
        shift = rng.integers(s, size=adj.shape) * base
        shift[:, 0] = 0
        adj = np.where(adj >= 0, (adj + shift) % n, -1).astype(np.int32)
        adj[:, 0] = np.arange(base) + 1           # ring through every orbit
        add_general("nonreg_sym_n%ds%d" % (n, s), n, dmax, s, adj, deg)
    adj, deg = random_nonregular(rng, 24, 3, directed=True)
    add_general("nonreg_sym_disconnected", 96, 3, 4, np.where(adj >= 0, adj % 24, -1).astype(np.int32), deg)
    # directed (asymmetric) adjacency: the level recurrence must still match
    for n, d in [(80, 3), (257, 4)]:
        adj, deg = random_nonregular(rng, n, d, directed=True)
        adj = np.where(adj >= 0, adj, rng.integers(n, size=adj.shape)).astype(np.int32)
        add_general("directed_n%d" % n, n, d, 1, adj)
    # disconnected inputs
    adj, deg = random_nonregular(rng, 100, 4, components=2)
    add_general("disconnected_nonreg", 100, 4, 1, adj, deg)
    a = ref_conv_general(128, 4, 1, ref_gen_general(64, 4, 1, 50))
    b = ref_conv_general(64, 4, 1, ref_gen_general(64, 4, 1, 51))
    two = np.concatenate([a[:64], b + 64]).astype(np.int32)
    add_general("disconnected_two_regular", 128, 4, 1, two)
    add_general("disconnected_two_regular_saving", 128, 4, 1, two, kinds=("MATRIX_SAVING",))
    add_general("isolated_vertices", 4, 1, 1, np.array([[1], [0], [-1], [-1]], dtype=np.int32),
                np.array([1, 1, 0, 0], dtype=np.int32))
    # tiny graphs
    add_general("single_edge", 2, 1, 1, np.array([[1], [0]], dtype=np.int32))
    add_general("triangle", 3, 2, 1, np.array([[1, 2], [0, 2], [0, 1]], dtype=np.int32))
    add_general("path4", 4, 2, 1, np.array([[1, -1], [0, 2], [1, 3], [2, -1]], dtype=np.int32),
                np.array([1, 2, 2, 1], dtype=np.int32))
    # self-loops and multi-edges (the generators emit them)
    add_general("loops_multi", 6, 3, 1, np.array([[0, 1, 1], [0, 0, 2], [1, 3, 3], [2, 2, 4], [3, 5, 5],
                                                  [4, 4, 5]], dtype=np.int32))
    # non-regular symmetric grid (s = 2)
    e = ref_gen_grid(8, 6, 4, 3, 2, 52)
    adj = ref_conv_grid(8, 6, 4, 2, e)
    nd = np.full(adj.shape[0], 4, dtype=np.int32)
    nd[::5] = 3
    adj2 = adj.copy()
    adj2[::5, 3] = -1
    add_grid("nonreg_grid_s2", 8, 6, 4, 2, adj2, nd)
    return out


# ------------------------------------------------------------ mutations
def mutations():
    out = []
    for n, d, s, seed_g, seed_m, iters in [(256, 6, 1, 60, 61, 500), (240, 6, 4, 62, 63, 500),
                                            (512, 5, 2, 64, 65, 300), (640, 8, 64, 66, 67, 300)]:
        e = ref_gen_general(n, d, s, seed_g)
        adj = ref_conv_general(n, d, s, e)
        adj.tofile(tmp("adj"))
        run("mutate", "general", n, d, s, seed_m, iters, tmp("adj"), tmp("m"))
        m = np.fromfile(tmp("m"), dtype=np.int32)
        trace, final = m[:8 * iters], m[8 * iters:]
        out.append({"kind": "general", "nodes": n, "degree": d, "symmetries": s, "graph_seed": seed_g,
                    "seed": seed_m, "iters": iters, "trace_sha256": sha(trace), "final_sha256": sha(final),
                    "first_restore": flat(trace[:8])})
    for w, h, d, length, s, seed_g, seed_m, iters in [(12, 12, 4, 3, 1, 70, 71, 300), (12, 8, 4, 3, 2, 72, 73, 300),
                                                       (12, 12, 5, 3, 4, 74, 75, 300)]:
        e = ref_gen_grid(w, h, d, length, s, seed_g)
        adj = ref_conv_grid(w, h, d, s, e)
        adj.tofile(tmp("adj"))
        run("mutate", "grid", w, h, d, length, s, seed_m, iters, tmp("adj"), tmp("m"))
        m = np.fromfile(tmp("m"), dtype=np.int32)
        trace, final = m[:8 * iters], m[8 * iters:]
        out.append({"kind": "grid", "width": w, "height": h, "degree": d, "length": length, "symmetries": s,
                    "graph_seed": seed_g, "seed": seed_m, "iters": iters, "trace_sha256": sha(trace),
                    "final_sha256": sha(final), "first_restore": flat(trace[:8])})
    return out


def main():
    if not os.path.exists(DRIVER):
        sys.exit("build the reference first: make -C oracle ref")
    big = "--big" in sys.argv
    doc = {
        "about": "Expected values produced by the reference ODP library (built from its sources by "
                 "oracle/Makefile) through tests/golden/make_golden.py; results are [diameter, sum, "
                 "ASPL as float.hex].",
        "samples": samples(),
        "sample_text": {k: open(os.path.join(REF, "sample/graph/%s/ASPL.txt" % k)).read() for k in ("general", "grid")},
        "generators": generators(big),
        "cases": cases(),
        "mutations": mutations(),
    }
    if not big and os.path.exists(OUT):
        old = json.load(open(OUT))
        doc["generators"] += [g for g in old.get("generators", []) if g.get("big")]
    with open(OUT, "w") as f:
        json.dump(doc, f, separators=(",", ":"))
    print("wrote %s (%d bytes)" % (OUT, os.path.getsize(OUT)))


if __name__ == "__main__":
    main()
