"""Edge-file I/O (ODP_Get_lines, ODP_Read_edge_general/_grid,
ODP_Write_edge_general/_grid): the library parses and formats files by hand,
in parallel slices, and must give what the reference's fscanf/fprintf loops
give (utils.c:1153-1180, 1369-1429).  Checked against a restatement of those
loops here, and against the reference library itself where it is built in
this tree (oracle/_ref)."""
import os
import re
import subprocess

import numpy as np
import pytest

import odp_gb300 as og
import oracle

INT = re.compile(rb"[ \t\n\v\f\r]*([+-]?[0-9]+)")


def ref_ints(text):
    """The integers %d conversions read from text, up to the first that fails."""
    out, pos = [], 0
    while True:
        m = INT.match(text, pos)
        if not m:
            return out
        out.append(int(m.group(1)))
        pos = m.end()


def ref_read_general(text):
    """utils.c:1386-1401: pairs until fscanf returns EOF; an odd last integer
    still makes an edge whose second end is the previous edge's."""
    ints = ref_ints(text)
    edges = [ints[i:i + 2] for i in range(0, len(ints) - 1, 2)]
    if len(ints) % 2:
        edges.append([ints[-1], ints[-2]])
    return np.array(edges, dtype=np.int32).reshape(-1, 2)


def ref_driver_read(path, grid):
    drv = oracle.ref_driver()
    if drv is None:
        return None
    out = path + ".bin"
    res = subprocess.run([drv, "readedges", "grid" if grid else "general", path, out], capture_output=True,
                         text=True, check=True)
    fields = [int(x) for x in res.stdout.split()]
    edge = np.fromfile(out, dtype=np.int32).reshape(-1, 2)
    return fields, edge


def test_general_round_trip_and_text(tmp_path):
    n, d = 2000, 7
    edge = og.generate_random_general(n, d, seed=3)
    path = str(tmp_path / "g.edges")
    og.write_edge_general(edge, path)
    text = open(path, "rb").read()
    assert text == b"".join(b"%d %d\n" % (a, b) for a, b in edge)
    assert og.get_lines(path) == len(edge)
    assert np.array_equal(og.read_edge_general(path), edge)


def test_grid_round_trip_and_text(tmp_path):
    w = h = 24
    edge = og.generate_random_grid(w, h, 4, 3, seed=5)
    path = str(tmp_path / "g.edges")
    og.write_edge_grid(edge, h, path)
    text = open(path, "rb").read()
    assert text == b"".join(b"%d,%d %d,%d\n" % (a // h, a % h, b // h, b % h) for a, b in edge)
    rw, rh, got = og.read_edge_grid(path)
    mx = np.array([[a // h, a % h, b // h, b % h] for a, b in edge])
    assert (rw, rh) == (max(mx[:, 0].max(), mx[:, 2].max()) + 1, max(mx[:, 1].max(), mx[:, 3].max()) + 1)
    assert np.array_equal(got, np.array([[a // h * rh + a % h, b // h * rh + b % h] for a, b in edge]))


@pytest.mark.parametrize("name,text", [
    ("spaces", b"0 1\n  2\t3\n4   5  \n"),
    ("crlf", b"0 1\r\n2 3\r\n4 5\r\n"),
    ("signs", b"+0 1\n2 +3\n-4 5\n"),
    ("blank lines", b"0 1\n\n2 3\n\n\n"),
    ("two per line", b"0 1 2 3\n4 5\n"),
    ("odd count", b"0 1\n2 3\n4\n"),
    ("glued sign", b"10-3\n4 5\n"),
])
def test_general_parse_variants(tmp_path, name, text):
    path = str(tmp_path / "v.edges")
    open(path, "wb").write(text)
    want = ref_read_general(text)
    lines = text.count(b"\n")
    assert og.get_lines(path) == lines
    edge = np.zeros((max(lines, len(want)) + 1, 2), dtype=np.int32)
    og.load().ODP_Read_edge_general(os.fsencode(path), og._iptr(edge))
    assert np.array_equal(edge[:len(want)], want), name
    r = ref_driver_read(path, False) if len(want) <= lines else None
    if r is not None:
        assert r[0] == [lines]
        assert np.array_equal(r[1][:len(want)], want), name


def test_stops_at_a_token_that_is_not_an_integer(tmp_path):
    """The reference would loop for ever here; the library stops."""
    path = str(tmp_path / "bad.edges")
    open(path, "wb").write(b"0 1\n2 3\nx y\n4 5\n")
    edge = np.full((5, 2), -7, dtype=np.int32)
    og.load().ODP_Read_edge_general(os.fsencode(path), og._iptr(edge))
    assert np.array_equal(edge[:2], [[0, 1], [2, 3]]) and (edge[2:] == -7).all()


def test_large_file_parsed_in_parallel_slices(tmp_path):
    """Big enough for the multi-threaded path; slices are cut at newlines."""
    rng = np.random.default_rng(1)
    edge = rng.integers(0, 1 << 30, size=(600000, 2), dtype=np.int64).astype(np.int32)
    path = str(tmp_path / "big.edges")
    og.write_edge_general(edge, path)
    assert os.path.getsize(path) > (8 << 20)
    assert np.array_equal(og.read_edge_general(path), edge)
    r = ref_driver_read(path, False)
    if r is not None:
        assert np.array_equal(r[1], edge)


def test_reference_reads_our_files(tmp_path):
    """Files written here read back identically with the reference's readers."""
    if oracle.ref_driver() is None:
        pytest.skip("reference library not built in this tree")
    w = h = 16
    edge = og.generate_random_grid(w, h, 4, 2, seed=8)
    path = str(tmp_path / "grid.edges")
    og.write_edge_grid(edge, h, path)
    fields, got = ref_driver_read(path, True)
    rw, rh, mine = og.read_edge_grid(path)
    assert fields == [len(edge), rw, rh]
    assert np.array_equal(got, mine)
