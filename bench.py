"""Benchmark of the ODP ASPL/diameter evaluation on GB300.

Workload (one "step" = one full ASPL evaluation of the graph): the single
large graph of the reference's MATRIX_SAVING configuration -- a random
16-regular graph on n = 65536 vertices, ODP_Srand(2) +
ODP_Generate_random_general (regenerated here with the library's seeded
generator, checked against the reference's sha256), no symmetry.

Reported (one JSON line on rank 0):
  value       evaluations/s of the engine on resident inputs (device time,
              CUDA events on the plan's stream, L2 flushed before every run)
  e2e         evaluations/s through the drop-in C API ODP_Set_aspl with the
              adjacency in host memory (upload + evaluation + read back)
  roofline    algorithmic bytes of the engine kernel per evaluation
              (sum over column chunks of levels x 8 x words x sum_v (d_v + 2))
              over its measured launch time, against the measured HBM peak
  cpu_baseline  the oracle port of the reference CPU library (OpenMP on all
              host cores) on a bounded sample of the same workload
  batched     (with --batch) evals/s of the batched engine vs one call per graph

--impl reference times the reference's CPU implementation (the oracle port,
all host threads) on the same workload and prints the same line shape.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

C2 = dict(nodes=65536, degree=16, seed=2, sha256="d855fb662f9e9557")
METRIC = "ASPL evals/s (single graph n=65536 d=16, MATRIX_SAVING config, bit-exact)"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="own", choices=["own", "reference"])
    p.add_argument("--flush-mb", type=int, default=512)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-evals", type=int, default=2)
    return p.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier and max-over-ranks for torchrun launches (gloo: host scalars only)."""

    def __init__(self, world):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x):
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0}, "fallback"


def workload_graph():
    import odp_gb300 as og
    import hashlib
    e = og.generate_random_general(C2["nodes"], C2["degree"], seed=C2["seed"])
    h = hashlib.sha256(np.ascontiguousarray(e, dtype=np.int32).tobytes()).hexdigest()
    if not h.startswith(C2["sha256"]):
        raise RuntimeError("generated workload graph differs from the reference's")
    return og.conv_edge2adjacency_general(C2["nodes"], e, C2["degree"])


def cpu_baseline(adj, evals):
    """The oracle port of libodp_threads.a (MATRIX_SAVING, all host threads)."""
    import oracle
    oracle.build()
    o = oracle.Oracle(C2["nodes"], C2["degree"], kind=oracle.KIND_SAVING)
    t0 = time.perf_counter()
    for _ in range(evals):
        res = o.set(adj)
    dt = (time.perf_counter() - t0) / evals
    o.close()
    return 1.0 / dt, res, oracle.threads()


def bytes_alg(batch, adj, degrees=None):
    """Algorithmic bytes of one evaluation (see module docstring)."""
    info = batch.info(0)
    levels = batch.job_levels()
    wc = 1 << info["wc_log2"]
    per_level = 8.0 * wc * float((adj.shape[1] + 2) * adj.shape[0] if degrees is None else np.sum(degrees + 2))
    return per_level * float(np.sum(levels))


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    adj = workload_graph()
    import oracle
    oracle.build()
    o = oracle.Oracle(C2["nodes"], C2["degree"], kind=oracle.KIND_SAVING)
    for _ in range(min(args.warmup, 1)):
        o.set(adj)
    steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(steps):
        o.set(adj)
    dt = (time.perf_counter() - t0) / steps
    o.close()
    v = 1.0 / dt
    line = {"metric": METRIC, "value": v, "unit": "evals/s", "n_gpus": world, "steps": steps, "warmup": args.warmup,
            "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64", "data": "synthetic (reference generator, seed 2)", "impl": "reference",
            "config": {"workload": "single graph n=65536 d=16 seed=2, MATRIX_SAVING", "nodes": 65536,
                       "degree": 16},
            "cpu_baseline": {"value": v, "unit": "evals/s", "cores": oracle.threads(), "kind": "port",
                             "sample": "%d full evaluations" % steps},
            "e2e": {"value": v, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_own(args):
    rank, world, local = dist_info()
    dist = Dist(world)
    import odp_gb300 as og
    og.load()
    adj = workload_graph()
    n, d = C2["nodes"], C2["degree"]

    # engine on resident inputs
    batch = og.Batch([og.GraphSpec(adj, nodes=n)])
    first = batch.run()[0]
    for _ in range(args.warmup):
        batch.time(1, mode=1, flush_mb=args.flush_mb)
    dist.barrier()
    with ClockSampler(local) as clk:
        ms = batch.time(args.steps, mode=1, flush_mb=args.flush_mb)
    ms = dist.max(ms)
    dist.barrier()
    value = world * 1000.0 / ms
    balg = bytes_alg(batch, adj)
    info = batch.info(0)
    tiles = batch.tiles()

    # end to end through the drop-in API with host buffers
    og.init_aspl_general(n, d)
    for _ in range(args.warmup):
        og.set_aspl(adj)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = og.set_aspl(adj)
    e2e_s = (time.perf_counter() - t0) / args.steps
    og.finalize_aspl()
    e2e_s = dist.max(e2e_s)
    assert r[0] == first[0] and r[1] == first[1]

    peaks, src = measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    achieved = balg / (ms * 1e-3) / 1e9
    line = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (reference generator, seed 2)",
            "config": {"workload": "single graph n=65536 d=16 seed=2, MATRIX_SAVING", "nodes": n, "degree": d,
                       "chunk_words": 1 << info["wc_log2"], "slots": info["nslots"], "jobs": info["njobs"],
                       "tile_rows": info["tile_rows"], "l2": "flushed (%d MB write) before every timed run"
                       % args.flush_mb, "parallelism": "replicas" if world > 1 else "single"},
            "result": {"diameter": first[0], "sum": first[1], "ASPL": first[2]},
            "e2e": {"value": world / e2e_s, "unit": "evals/s", "h2d_bytes_per_step": int(adj.nbytes),
                    "d2h_bytes_per_step": 64 + 64 + 16},
            "gpu_launches": args.steps,
            "tiles_per_eval": tiles,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": None, "peak_source": src,
                         "bytes_alg_per_launch": balg},
            "clocks": clk.summary()}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, res, cores = cpu_baseline(adj, args.cpu_evals)
        assert res[0] == first[0] and res[1] == first[1] and res[2].hex() == first[2].hex()
        line["cpu_baseline"] = {"value": v, "unit": "evals/s", "cores": cores, "kind": "port",
                                "sample": "%d full evaluations of the workload graph" % args.cpu_evals}
    if rank == 0:
        print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_own(args)


if __name__ == "__main__":
    main()
