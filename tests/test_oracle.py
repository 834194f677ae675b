"""The oracle (CPU restatement of the reference ASPL) against the reference's
own golden vectors: the sample tables, the library-generated fixtures and
edge cases recorded from the reference library.  CPU only."""
import numpy as np
import pytest

import oracle
from conftest import (case_adjacency, case_degrees, edges_to_adjacency, gen_record_adjacency, gen_record_edges,
                      result_tuple, same)


def test_sample_golden_tables(golden):
    for s in golden["samples"]:
        if "expected" not in s:
            continue
        e = np.array(s["edges"], dtype=np.int32).reshape(-1, 2)
        if s["kind"] == "general":
            n = int(e.max()) + 1
        else:
            n = s["width"] * s["height"]
        deg = int(np.bincount(e.reshape(-1), minlength=n).max())
        adj = edges_to_adjacency(n, deg, e)
        if s["kind"] == "general":
            d, sm, a = oracle.aspl(adj, nodes=n)
        else:
            d, sm, a = oracle.aspl(adj, grid=True, width=s["width"], height=s["height"])
        exp = s["expected"]
        assert (d, sm, "%.10f" % a) == (exp["diameter"], exp["sum"], exp["aspl"]), s["file"]


def test_symmetric_sample_files(golden):
    for s in golden["samples"]:
        if "reference" not in s:
            continue
        e = np.array(s["edges"], dtype=np.int32).reshape(-1, 2)
        if s["kind"] == "general":
            adj = edges_to_adjacency(s["nodes"], s["degree"], e, s["symmetries"])
            got = oracle.aspl(adj, nodes=s["nodes"], symmetries=s["symmetries"])
        else:
            import odp_gb300 as og
            adj = og.conv_edge2adjacency_grid(s["width"], s["height"], e, s["degree"], s["symmetries"])
            got = oracle.aspl(adj, grid=True, width=s["width"], height=s["height"], symmetries=s["symmetries"])
        assert same(got, result_tuple(s["reference"])), s["file"]


@pytest.mark.parametrize("kind", [oracle.KIND_MATRIX, oracle.KIND_SAVING])
def test_edge_cases(golden, kind):
    for c in golden["cases"]:
        adj = case_adjacency(c)
        nd = case_degrees(c)
        if c["kind"] == "general":
            got = oracle.aspl(adj, nodes=c["nodes"], num_degrees=nd, symmetries=c["symmetries"], kind=kind)
        else:
            got = oracle.aspl(adj, grid=True, width=c["width"], height=c["height"], num_degrees=nd,
                              symmetries=c["symmetries"], kind=kind)
        assert same(got, result_tuple(c["reference"])), c["name"]


def test_generated_fixtures(golden):
    import odp_gb300 as og
    for g in golden["generators"]:
        if g.get("big"):
            continue
        e = gen_record_edges(og, g)
        adj = gen_record_adjacency(og, g, e)
        if g["kind"] == "general":
            got = oracle.aspl(adj, nodes=g["nodes"], symmetries=g["symmetries"])
        else:
            got = oracle.aspl(adj, grid=True, width=g["width"], height=g["height"], symmetries=g["symmetries"])
        assert same(got, result_tuple(g["reference"])), g


@pytest.mark.skipif(not oracle.ref_available(), reason="reference tree not present")
def test_against_reference_library_live(tmp_path):
    """Random graphs through the reference library itself (where it is built)."""
    import subprocess
    import odp_gb300 as og
    rng = np.random.default_rng(7)
    for trial in range(12):
        s = int(rng.choice([1, 2, 4, 8]))
        base = int(rng.integers(3, 90))
        n = base * s
        d = int(rng.integers(2, 7))
        if n % 2 and d % 2:
            d += 1
        e = og.generate_random_general(n, d, s, seed=1000 + trial)
        adj = og.conv_edge2adjacency_general(n, e, d, s)
        adj.tofile(tmp_path / "adj")
        out = subprocess.run([oracle.ref_driver(), "aspl", "general", str(n), str(d), str(s), str(tmp_path / "adj"),
                              "-"], capture_output=True, text=True, check=True).stdout.split()
        ref = (int(out[0]), int(out[1]), float.fromhex(out[2]))
        assert same(oracle.aspl(adj, nodes=n, symmetries=s), ref)
