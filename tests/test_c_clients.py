"""C clients of the drop-in API: a program linked against the static
archive prints the reference's sample report (stdout compared with the
reference's golden tables), and the reference's own sample programs link
against the archive unchanged."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from conftest import ROOT

CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
LINK = ["-L" + os.path.join(CUDA, "lib64"), "-lcudart_static", "-ldl", "-lrt", "-lpthread", "-lstdc++", "-lm"]
ARCHIVE = os.path.join(ROOT, "odp_gb300", "libodp_gb300.a")


def build_replay(tmp_path):
    exe = str(tmp_path / "replay")
    subprocess.run(["gcc", "-O2", "-I", os.path.join(ROOT, "include"), "-o", exe,
                    os.path.join(ROOT, "tests", "c", "replay.c"), ARCHIVE] + LINK, check=True)
    return exe


def test_replay_client_links_on_cpu(tmp_path):
    assert os.path.exists(build_replay(tmp_path))


@pytest.mark.skipif(not oracle.ref_available(), reason="reference tree not present")
def test_reference_samples_link_unchanged(tmp_path):
    for prog in ("general.c", "grid.c", "non_regular_general.c"):
        exe = str(tmp_path / prog.replace(".c", ""))
        subprocess.run(["gcc", "-O2", "-w", "-I", os.path.join(ROOT, "include"), "-o", exe,
                        os.path.join(oracle.REF_SOURCE, "sample", prog), ARCHIVE] + LINK, check=True)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference tree not present")
def test_reference_annealing_clients_link_unchanged(tmp_path):
    sa = os.path.join(oracle.REF_SOURCE, "sample", "SA")
    for prog in ("general", "general_s", "grid", "grid_s"):
        subprocess.run(["gcc", "-O2", "-w", "-I", os.path.join(ROOT, "include"), "-I", sa, "-o",
                        str(tmp_path / prog), os.path.join(sa, prog + ".c"), os.path.join(sa, "common.c"),
                        os.path.join(sa, "detect_temp.c"), ARCHIVE] + LINK, check=True)


@pytest.mark.gpu
def test_golden_tables_replayed_through_c(tmp_path, golden):
    exe = build_replay(tmp_path)
    for kind in ("general", "grid"):
        out = []
        for s in golden["samples"]:
            if s["kind"] != kind or "expected" not in s:
                continue
            e = np.array(s["edges"], dtype=np.int64).reshape(-1, 2)
            path = tmp_path / s["file"]
            with open(path, "w") as f:
                for a, b in e:
                    if kind == "general":
                        f.write("%d %d\n" % (a, b))
                    else:
                        h = s["height"]
                        f.write("%d,%d %d,%d\n" % (a // h, a % h, b // h, b % h))
            r = subprocess.run([exe, kind, str(path)], capture_output=True, text=True, check=True)
            out.append(r.stdout)
        assert "".join(out) == golden["sample_text"][kind], kind
