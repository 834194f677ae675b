"""The C-ABI library loads without a GPU and exports every entry point that
include/*.h declares.  No compute calls (CPU only)."""
import ctypes
import os
import re

from conftest import ROOT


def declared_functions():
    names = set()
    for h in ("odp.h", "odp_gb300.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:extern\s+)?[A-Za-z_][\w\s\*]*?\b((?:ODP|ODPX)_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_drop_in_surface():
    names = declared_functions()
    for n in ["ODP_Init_aspl_general", "ODP_Init_aspl_general_s", "ODP_Init_aspl_grid", "ODP_Init_aspl_grid_s",
              "ODP_Set_aspl", "ODP_Finalize_aspl", "ODP_Set_aspl_batch"]:
        assert n in names


def test_library_exports_every_declared_symbol():
    import odp_gb300
    lib = ctypes.CDLL(odp_gb300.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_static_archive_built():
    import odp_gb300.build as b
    assert os.path.exists(b.A_PATH)


def test_invalid_batch_shapes_are_refused_before_the_device():
    """Shapes are validated before any device work, so they are refused with
    ODPX_ERR_INVALID on any machine: nodes not a multiple of the symmetries,
    a grid with s = 2 and an odd width, a grid with s = 4 that is not square."""
    import numpy as np
    import odp_gb300 as og
    cases = [dict(nodes=10, symmetries=3), dict(grid=True, width=5, height=6, symmetries=2),
             dict(grid=True, width=6, height=8, symmetries=4)]
    for kw in cases:
        n = kw.get("nodes") or kw["width"] * kw["height"]
        adj = np.zeros((max(1, n // kw["symmetries"]), 4), dtype=np.int32)
        try:
            og.Batch([og.GraphSpec(adj, **kw)])
        except og.ODPError as e:
            assert e.code == og.ERR_INVALID, (kw, e.code)
        else:
            raise AssertionError("accepted: %s" % kw)


def test_degrees_above_the_engine_limit_are_refused():
    """The engine stages neighbour lists of at most 512 entries per row: a
    degree above 508 is refused by the batch API (ODPX_ERR_INVALID) and by
    the drop-in, which exits with a message naming the limit."""
    import subprocess
    import sys
    import numpy as np
    import odp_gb300 as og
    for d in (509, 600):
        adj = np.zeros((16, d), dtype=np.int32)
        try:
            og.Batch([og.GraphSpec(adj, nodes=16)])
        except og.ODPError as e:
            assert e.code == og.ERR_INVALID
        else:
            raise AssertionError("degree %d accepted" % d)
    code = "import sys; sys.path.insert(0, %r); import odp_gb300 as og; og.init_aspl_general(1024, 600)" % ROOT
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 1 and "at most 508" in r.stderr, (r.returncode, r.stderr)
