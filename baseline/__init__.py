"""The reference ODP library itself, built from its own sources, as the
baseline that the GB300 build is measured against.

``baseline/_ref/src`` (git-ignored) holds the reference's unmodified C/CUDA
sources, installed by ``install_ref.sh`` where the reference tree is present;
they travel with the working tree to machines where it is not.
``baseline/Makefile`` compiles them into ``libodp_threads.a`` (CPU, OpenMP)
and ``libodp_cuda.a`` (CUDA, sm_103a), each linked with the timing driver
``ref_bench.c``.  This module writes graph lists and adjacency files for that
driver, runs it, and parses what it prints.  It never loads libodp_gb300.
"""
import os
import shutil
import subprocess
import sys
import tempfile
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "_ref", "src")
BIN = os.path.join(HERE, "_ref", "bin")
CPU_BIN = os.path.join(BIN, "ref_bench_threads")
GPU_BIN = os.path.join(BIN, "ref_bench_cuda")


def reference_dir():
    """The reference tree to install from, when present."""
    d = os.environ.get("ODP_REFERENCE_DIR", "/root/reference")
    return d if os.path.isfile(os.path.join(d, "aspl.c")) else None


def sources_present():
    return os.path.isfile(os.path.join(SRC, "aspl.c")) and os.path.isfile(os.path.join(SRC, "include", "odp.h"))


_install_lock = threading.Lock()
_installed = False


def install():
    """Copies the reference sources into _ref/src when the reference tree is
    here (once per process)."""
    global _installed
    with _install_lock:
        ref = reference_dir()
        if ref is None or _installed:
            return sources_present()
        subprocess.run(["sh", os.path.join(HERE, "install_ref.sh"), ref], check=True, stdout=subprocess.DEVNULL)
        _installed = True
        return True


def build(cpu=True, gpu=True):
    """Builds the drivers that the sources allow; returns (cpu_ok, gpu_ok)."""
    install()
    if not sources_present():
        return False, False
    targets = (["cpu"] if cpu else []) + (["gpu"] if gpu else [])
    ok = {}
    for t in targets:
        r = subprocess.run(["make", "-s", "-C", HERE, t], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                           text=True)
        ok[t] = r.returncode == 0
        if r.returncode != 0:
            sys.stderr.write("baseline: make %s failed:\n%s\n" % (t, r.stdout[-3000:]))
    return ok.get("cpu", False), ok.get("gpu", False)


def cpu_available():
    return os.access(CPU_BIN, os.X_OK)


def gpu_available():
    return os.access(GPU_BIN, os.X_OK)


def host_description():
    """nproc and the CPU model of this host."""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                k = ln.split(":")[0].strip().lower()
                if k in ("model name", "cpu model") and model is None:
                    model = ln.split(":", 1)[1].strip()
    except OSError:
        pass
    if model is None:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
            for ln in out.splitlines():
                if ln.lower().startswith("model name"):
                    model = ln.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return {"nproc": os.cpu_count() or 1, "cpu_model": model or "unknown"}


def _shape_line(s):
    if s["grid"]:
        return "grid %d %d %d %d %d %d" % (s["width"], s["height"], s["degree"], s.get("length", 0),
                                          s["symmetries"], s.get("seed", 0))
    return "general %d %d %d %d" % (s["nodes"], s["degree"], s["symmetries"], s.get("seed", 0))


def _rows(s):
    n = s["width"] * s["height"] if s["grid"] else s["nodes"]
    return n // s["symmetries"]


def _write_shapes(path, shapes):
    with open(path, "w") as f:
        for s in shapes:
            f.write(_shape_line(s) + "\n")


def _write_adj(path, adjs):
    with open(path, "wb") as f:
        for a in adjs:
            f.write(np.ascontiguousarray(a, dtype="<i4").tobytes())


def generate(shapes, workers=None):
    """Each shape's graph by the reference generators (ODP_Srand(seed) then
    ODP_Generate_random_general_s / _grid_s and the matching conversion to
    adjacency): a list of int32[n/s][d] arrays."""
    workers = workers or (os.cpu_count() or 1)
    tmp = tempfile.mkdtemp(prefix="odp_ref_")
    try:
        sp, out = os.path.join(tmp, "shapes.txt"), os.path.join(tmp, "adj.bin")
        _write_shapes(sp, shapes)
        subprocess.run([CPU_BIN, "gen", sp, out, str(workers)], check=True)
        flat = np.fromfile(out, dtype="<i4")
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    res, off = [], 0
    for s in shapes:
        k = _rows(s) * s["degree"]
        res.append(flat[off:off + k].reshape(_rows(s), s["degree"]).astype(np.int32))
        off += k
    return res


def _parse(out):
    steps, graphs = [], {}
    for ln in out.splitlines():
        f = ln.split()
        if not f:
            continue
        if f[0] == "step":
            steps.append({"warm_ns": int(f[2]), "first_ns": int(f[3]), "wall_ns": int(f[4])})
        elif f[0] == "graph":
            graphs[int(f[1])] = (int(f[2]), int(f[3]), float.fromhex(f[4]), int(f[5]), int(f[6]))
    return steps, graphs


def time_cpu(shapes, adjs, steps=1, warmup=0, sets=2, threads=None, env=None):
    """libodp_threads.a on the host cores: every graph in a forked child
    (Init, `sets` x ODP_Set_aspl, Finalize), `warmup` + `steps` passes over
    the list.  Returns (steps, results): per timed step the summed time of the
    last Set of every graph (warm_ns), of the first (first_ns) and the wall
    time; per graph (diameter, sum, ASPL, last-Set ns, first-Set ns)."""
    e = dict(os.environ)
    e["OMP_NUM_THREADS"] = str(threads or (os.cpu_count() or 1))
    e.setdefault("OMP_PROC_BIND", "false")
    if env:
        e.update(env)
    tmp = tempfile.mkdtemp(prefix="odp_ref_")
    try:
        sp, ap = os.path.join(tmp, "shapes.txt"), os.path.join(tmp, "adj.bin")
        _write_shapes(sp, shapes)
        _write_adj(ap, adjs)
        r = subprocess.run([CPU_BIN, "cpu", sp, ap, str(steps), str(warmup), str(sets)], capture_output=True,
                           text=True, env=e)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    if r.returncode != 0:
        raise RuntimeError("reference CPU driver failed (%d): %s" % (r.returncode, r.stderr[-2000:]))
    st, g = _parse(r.stdout)
    return st, [g[i] for i in range(len(shapes))]


def gpu_order(shapes):
    """An order of the shapes that the reference's CUDA driver can run in one
    process: every grid graph with symmetries > 1 after all the others."""
    return sorted(range(len(shapes)), key=lambda i: 1 if (shapes[i]["grid"] and shapes[i]["symmetries"] > 1) else 0)


def time_gpu(shapes, adjs, reps=3, env=None):
    """libodp_cuda.a (sm_103a) on the GPU, one graph per call: per graph
    Init, one untimed and `reps` timed ODP_Set_aspl, Finalize.  Returns per
    graph (diameter, sum, ASPL, mean ns, min ns) in the input order."""
    order = gpu_order(shapes)
    e = dict(os.environ)
    if env:
        e.update(env)
    tmp = tempfile.mkdtemp(prefix="odp_ref_")
    try:
        sp, ap = os.path.join(tmp, "shapes.txt"), os.path.join(tmp, "adj.bin")
        _write_shapes(sp, [shapes[i] for i in order])
        _write_adj(ap, [adjs[i] for i in order])
        r = subprocess.run([GPU_BIN, "gpu", sp, ap, str(reps)], capture_output=True, text=True, env=e)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    if r.returncode != 0:
        raise RuntimeError("reference CUDA driver failed (%d): %s" % (r.returncode, r.stderr[-2000:]))
    _, g = _parse(r.stdout)
    out = [None] * len(shapes)
    for k, i in enumerate(order):
        out[i] = g[k]
    return out
