"""Benchmark of the ODP ASPL/diameter evaluation on GB300.

Headline workload (one "step" = one evaluation of the whole batch): 512
graphs of uneven size, degree and symmetry (odp_gb300/workloads.py: seeds
100..611, n log-uniform in [256, 8192], d in {4..32}, 80 % general / 20 % grid,
s in {1, 2, 4}), each the reference generator's graph for its seed, evaluated
together by the batched engine (ODP_Set_aspl_batch).

Reported on rank 0 as one JSON line:
  value        batched evals/s of the engine on resident inputs (device time,
               CUDA events on the plan's stream, L2 flushed before each run)
  e2e          batched evals/s through ODP_Set_aspl_batch with the adjacency in
               host memory (upload, expand, engine, read back, decode)
  per_call     evals/s of the one-graph-per-call path on the same GPU: a plan
               per graph evaluated one after the other (the fastest per-call
               form), and the drop-in Init/Set/Finalize cycle
  single_graph the n=65536, d=16 graph of the reference's MATRIX_SAVING
               configuration: device and ODP_Set_aspl evals/s
  roofline     algorithmic bytes of the engine kernel per launch / its time,
               against the measured HBM peak; the measured L2 read ceiling
               is reported beside it (the working set is L2-resident)
  serving      64 simulated-annealing chains (n in {1024..32768}, d in {8,16,24})
               proposing 2-opt swaps to the serving mode (ODPX_Serve_*): closed
               loop, one request outstanding per chain, exponential think time
               for a 20k req/s offered cap; evals/s and p50/p99 latency, beside
               the same proposals evaluated one call at a time
  anneal       the same 64 chains with every step (2-opt proposal, evaluation,
               acceptance, undo) on the GPU (ODPX_Anneal), in 4 size groups
  cpu_baseline the oracle port of the reference CPU library (OpenMP, all host
               cores) on a bounded sample of the batch

--impl reference times the reference's CPU implementation (the oracle port,
all host threads) on the same batch and prints the same line shape.
"""
import argparse
import hashlib
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ASPL evals/s, batched vs per-call on 1 GB300 (bit-exact)"
C2 = dict(nodes=65536, degree=16, seed=2, sha256="d855fb662f9e9557", result=(6, 9346294313))
WORKLOAD = ("batched: 512 graphs, seeds 100..611, n log-uniform [256, 8192], d in {4..32}, "
            "80% general / 20% grid (length 3-6), s in {1,2,4}")
# One ncu capture of an engine_kernel launch on the first 128 graphs of the batch
# (profiles/engine_kernel_batch.md): DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum), bytes
# read from L2 by the SMs (l1tex__m_xbar2l1tex_read_bytes.sum), and that launch's algorithmic bytes.  A full
# batch launch's figures are taken as these scaled by algorithmic bytes.  The engine reads fewer bytes than
# the algorithmic count: level 1 is built from the neighbour lists, and lanes whose words are saturated
# gather nothing.
NCU_DRAM = {"bytes": 936275200.0 + 815841024.0, "l2_read_bytes": 14874844864.0, "bytes_alg": 24803482864.0,
            "graphs": 128}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="own", choices=["own", "reference"])
    p.add_argument("--flush-mb", type=int, default=512)
    p.add_argument("--graphs", type=int, default=512)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-single", action="store_true")
    p.add_argument("--no-per-call", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--no-serving", action="store_true")
    p.add_argument("--no-anneal", action="store_true")
    p.add_argument("--no-tune", action="store_true")
    p.add_argument("--serve-seconds", type=float, default=8.0)
    return p.parse_args()


def dist_info():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class Dist:
    """Barrier and max-over-ranks for torchrun launches (gloo, host scalars only)."""

    def __init__(self, world):
        self.world = world
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
        self.index, self.proc, self.lines, self.first = index, None, [], 0

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
            t0 = time.perf_counter()                 # sampling is running before the timed region starts
            while not self.lines and time.perf_counter() - t0 < 5.0:
                time.sleep(0.01)
            self.first = len(self.lines)
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
        for ln in self.lines[self.first:]:
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


def batch_workload(count):
    from odp_gb300 import workloads
    shapes = workloads.batch_shapes(count)
    return shapes, workloads.build_graphs(shapes)


def single_graph():
    import odp_gb300 as og
    e = og.generate_random_general(C2["nodes"], C2["degree"], seed=C2["seed"])
    if not hashlib.sha256(np.ascontiguousarray(e, dtype=np.int32).tobytes()).hexdigest().startswith(C2["sha256"]):
        raise RuntimeError("generated n=65536 graph differs from the reference's")
    return og.conv_edge2adjacency_general(C2["nodes"], e, C2["degree"])


def oracle_sample(specs, seconds):
    """Oracle port on graphs taken in order until `seconds` of CPU work."""
    import oracle
    oracle.build()
    done, t0, results = 0, time.perf_counter(), []
    for s in specs:
        results.append(oracle.aspl(s.adjacency, nodes=s.nodes, symmetries=s.symmetries, grid=s.grid,
                                   width=s.width, height=s.height, num_degrees=s.num_degrees))
        done += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    return done / dt, done, dt, results, oracle.threads()


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    shapes, specs = batch_workload(args.graphs)
    # every step is a bounded sample of the batch (its first graphs, in order,
    # for a fixed slice of CPU time), so the whole run stays near two minutes
    per_step = min(2.0, 120.0 / max(1, args.steps + args.warmup))
    for _ in range(args.warmup):
        oracle_sample(specs, per_step)
    total_done, total_s, cores = 0, 0.0, 1
    for _ in range(args.steps):
        _, done, dt, _, cores = oracle_sample(specs, per_step)
        total_done += done
        total_s += dt
    v = total_done / total_s
    line = {"metric": METRIC, "value": v, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * total_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (reference generators, seeded)",
            "impl": "reference", "config": {"workload": WORKLOAD, "graphs": len(specs)},
            "cpu_baseline": {"value": v, "unit": "evals/s", "cores": cores, "kind": "port",
                             "sample": "per step, the batch's first graphs for %.2f s of CPU time (%d graphs "
                                       "over %d steps)" % (per_step, total_done, args.steps)},
            "e2e": {"value": v, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def serving(seconds, rate=20000.0):
    """The served annealing workload; returns the report dict."""
    import threading
    import odp_gb300 as og
    from odp_gb300 import workloads
    shapes = workloads.chain_shapes(64)
    specs = workloads.build_graphs(shapes)
    srv = og.Server(lanes=4, max_batch=16, max_nodes=32768, memory_mb=4096)
    handles = [srv.register(og.GraphSpec(s.adjacency.copy(), nodes=s.nodes)) for s in specs]
    think_mean = len(shapes) / rate
    lat, done, lat_by_n = [], [0], {}
    lock = threading.Lock()
    stop_at = [0.0]
    checks = []

    def chain(k):
        sh, sp = shapes[k], specs[k]
        n, d = sh["nodes"], sh["degree"]
        host = sp.adjacency.copy()
        rng = og.Rng(sh["proposal_seed"])
        draw = np.random.default_rng(sh["proposal_seed"])
        current = srv.wait(srv.submit(handles[k]))[2]
        undo = []
        local = []
        while time.perf_counter() < stop_at[0]:
            time.sleep(draw.exponential(think_mean))
            r = rng.mutate_general(n, d, host)
            res = srv.wait(srv.submit(handles[k], undo + og.two_opt_deltas(host, r, n)))
            local.append(res[3])
            delta = (res[2] - current) * n * (n - 1) / 2.0
            if res[2] <= current or draw.random() < math.exp(-delta / 50.0):
                current, undo = res[2], []
            else:
                og.Rng.restore_general(n, d, r, host)
                undo = og.two_opt_deltas(host, r, n)
        srv.wait(srv.submit(handles[k], undo))
        with lock:
            lat.extend(local)
            lat_by_n.setdefault(n, []).extend(local)
            done[0] += len(local)
            if k < 4:
                checks.append((k, host, res))

    threads = [threading.Thread(target=chain, args=(k,)) for k in range(len(shapes))]
    t0 = time.perf_counter()
    stop_at[0] = t0 + seconds
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    wall = time.perf_counter() - t0
    st = srv.stats()
    for k, host, res in checks:                      # the resident graphs followed the clients exactly
        assert np.array_equal(srv.adjacency(handles[k]), host)
    srv.close()
    lat_ms = np.array(lat) * 1e3
    # the same proposals one call at a time: ODP_Set_aspl per proposal, as the reference's annealing samples do
    pc = []
    for sh, sp in zip(shapes[:12], specs[:12]):
        og.init_aspl_general(sh["nodes"], sh["degree"])
        og.set_aspl(sp.adjacency)
        t1 = time.perf_counter()
        for _ in range(3):
            og.set_aspl(sp.adjacency)
        pc.append((time.perf_counter() - t1) / 3)
        og.finalize_aspl()
    return {"workload": "64 annealing chains, n in {1024,4096,16384,32768}, d in {8,16,24}, 2-opt proposals, "
                        "closed loop (1 outstanding per chain), exponential think time for a %d req/s offered cap"
                        % int(rate),
            "seconds": wall, "completed": done[0], "evals_per_s": done[0] / wall,
            "offered_cap_req_per_s": rate,
            "latency_ms": {"p50": float(np.percentile(lat_ms, 50)), "p99": float(np.percentile(lat_ms, 99)),
                           "mean": float(lat_ms.mean())},
            "latency_ms_by_n": {str(k): {"p50": float(np.percentile(np.array(v) * 1e3, 50)),
                                         "p99": float(np.percentile(np.array(v) * 1e3, 99)), "requests": len(v)}
                                for k, v in sorted(lat_by_n.items())},
            "batches": st["batches"], "mean_batch": st["batched_requests"] / max(1, st["batches"]),
            "max_batch": st["max_batch"], "max_concurrent_lanes": st["max_inflight_lanes"],
            "per_call_evals_per_s_same_mix": 1.0 / float(np.mean(pc)),
            "note": "the offered cap exceeds what any GPU can serve for n=32768 chains; chains are closed loop"}


def anneal(seconds, temperature=50.0):
    """The served annealing chains with every step on the GPU (ODPX_Anneal):
    the same 64 chains, grouped by size into 4 sets of 16 that run
    concurrently, each on a quarter of the persistent grid, so that small
    chains do not step at the pace of large ones.  Constant temperature, as
    the serving leg."""
    import torch
    import odp_gb300 as og
    from odp_gb300 import workloads
    shapes = workloads.chain_shapes(64)
    specs = workloads.build_graphs(shapes)
    sizes = sorted({s["nodes"] for s in shapes})
    idx = [[i for i, s in enumerate(shapes) if s["nodes"] == n] for n in sizes]
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    os.environ["ODP_GB300_BLOCKS"] = str(max(1, sms * 4 // len(sizes)))
    try:
        groups = [og.Anneal([og.Chain(specs[i].adjacency, shapes[i]["nodes"], seed=shapes[i]["proposal_seed"],
                                      max_temp=temperature, min_temp=temperature, ncalcs=1) for i in g])
                  for g in idx]
    finally:
        del os.environ["ODP_GB300_BLOCKS"]
    for g in groups:
        g.run(1)
    counts = [0] * len(groups)
    stop = time.perf_counter() + seconds

    def work(k):
        while time.perf_counter() < stop:
            groups[k].run(8)
            counts[k] += 8 * len(idx[k])

    threads = [threading.Thread(target=work, args=(k,)) for k in range(len(groups))]
    t0 = time.perf_counter()
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    wall = time.perf_counter() - t0
    # the reported state is that of the graph each chain holds
    for g, members in zip(groups, idx):
        st = g.state(0, graphs=True)
        sp = specs[members[0]]
        b = og.Batch([og.GraphSpec(st["adjacency"], nodes=sp.nodes)])
        assert same(b.run()[0], (st["diameter"], st["sum"], st["aspl"])), "chain state differs from its graph"
        b.close()
    accepted = sum(g.state(k)["accepted"] for g, m in zip(groups, idx) for k in range(len(m)))
    for g in groups:
        g.close()
    return {"workload": "the 64 served chains, 2-opt proposal + evaluation + acceptance + undo per step on the GPU, "
                        "4 size groups of 16 on 4 streams, a quarter of the persistent grid each, temperature %g"
                        % temperature,
            "seconds": wall, "evals_per_s": sum(counts) / wall,
            "per_group_evals_per_s": {str(n): c / wall for n, c in zip(sizes, counts)},
            "accepted": accepted}


def same(a, b):
    return a[0] == b[0] and a[1] == b[1] and float(a[2]).hex() == float(b[2]).hex()


def run_own(args):
    rank, world, local = dist_info()
    dist = Dist(world)
    import odp_gb300 as og
    og.load()
    shapes, specs = batch_workload(args.graphs)
    count = len(specs)
    adj_bytes = int(sum(s.adjacency.nbytes for s in specs))

    # ---- autotune the schedule for this batch (outside every timed region) ----
    from odp_gb300 import autotune
    tune_report = autotune.tune_batch(specs) if not args.no_tune else None

    # ---- batched engine on resident inputs (headline) ----
    batch = og.Batch(specs)
    res = batch.run()
    for _ in range(args.warmup):
        batch.time(1, mode=1, flush_mb=args.flush_mb)
    dist.barrier()
    with ClockSampler(local) as clk:
        ms = batch.time(args.steps, mode=1, flush_mb=args.flush_mb)
    ms = dist.max(ms)
    dist.barrier()
    value = world * count * 1000.0 / ms
    balg = batch.bytes_alg()
    info = batch.info(0)
    ms_full = batch.time(max(3, args.steps // 4), mode=0, flush_mb=args.flush_mb)

    # ---- end to end through ODP_Set_aspl_batch (host adjacency) ----
    og.set_aspl_batch(specs)
    for _ in range(args.warmup):
        og.set_aspl_batch(specs)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        res_e2e = og.set_aspl_batch(specs)
    e2e_s = dist.max((time.perf_counter() - t0) / args.steps)
    assert all(same(a, b) for a, b in zip(res, res_e2e))

    line = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (reference generators, seeded)",
            "config": {"workload": WORKLOAD, "graphs": count, "jobs": info["njobs"], "slots": info["nslots"],
                       "l2": "flushed (%d MB write) before every timed run" % args.flush_mb,
                       "parallelism": "replicas" if world > 1 else "single"},
            "e2e": {"value": world * count / e2e_s, "unit": "evals/s", "h2d_bytes_per_step": adj_bytes,
                    "d2h_bytes_per_step": 16 * count + 128},
            "gpu_launches": args.steps,
            "batch_device_ms_with_transfers": ms_full,
            "autotune": tune_report}

    autotune.clear()

    # ---- one graph per call on the same GPU ----
    if not args.no_per_call:
        plans = [og.Batch([s]) for s in specs]
        for p in plans:
            p.run()
        t0 = time.perf_counter()
        reps = max(2, args.steps // 4)
        for _ in range(reps):
            pc = [p.run()[0] for p in plans]
        pc_s = (time.perf_counter() - t0) / reps
        assert all(same(a, b) for a, b in zip(res, pc)), "batched and per-call results differ"
        for p in plans:
            p.close()
        k = min(64, count)
        t0 = time.perf_counter()
        for s in specs[:k]:
            nd = s.num_degrees
            if s.grid:
                (og.init_aspl_grid(s.width, s.height, s.degree, nd) if s.symmetries == 1 else
                 og.init_aspl_grid_s(s.width, s.height, s.degree, nd, s.symmetries))
            else:
                (og.init_aspl_general(s.nodes, s.degree, nd) if s.symmetries == 1 else
                 og.init_aspl_general_s(s.nodes, s.degree, nd, s.symmetries))
            og.set_aspl(s.adjacency)
            og.finalize_aspl()
        dropin_s = (time.perf_counter() - t0) / k
        line["per_call"] = {"evals_per_s": count / pc_s, "form": "one plan per graph, ODPX_Batch_run each",
                            "drop_in_init_set_finalize_evals_per_s": 1.0 / dropin_s,
                            "batched_e2e_over_per_call": (count / e2e_s) / (count / pc_s),
                            "batched_device_over_per_call": (count * 1000.0 / ms) / (count / pc_s),
                            "reference_cuda_per_call": "unavailable: the reference CUDA library cannot be "
                                                       "built on the GPU host (its sources are not there)"}

    # ---- the single large graph (MATRIX_SAVING configuration) ----
    if not args.no_single:
        adj = single_graph()
        single_tune = autotune.tune_single(og.GraphSpec(adj, nodes=C2["nodes"])) if not args.no_tune else None
        sb = og.Batch([og.GraphSpec(adj, nodes=C2["nodes"])])
        r = sb.run()[0]
        assert r[:2] == C2["result"], r
        sb.time(2, mode=1, flush_mb=args.flush_mb)
        sms = sb.time(max(3, args.steps // 2), mode=1, flush_mb=args.flush_mb)
        sbytes = sb.bytes_alg()
        sinfo = sb.info(0)
        sb.close()
        og.init_aspl_general(C2["nodes"], C2["degree"])
        og.set_aspl(adj)
        t0 = time.perf_counter()
        for _ in range(max(3, args.steps // 2)):
            og.set_aspl(adj)
        s_e2e = (time.perf_counter() - t0) / max(3, args.steps // 2)
        og.finalize_aspl()
        line["single_graph"] = {"workload": "n=65536 d=16 seed=2 (MATRIX_SAVING config)", "evals_per_s": 1000.0 / sms,
                                "ms": sms, "e2e_evals_per_s": 1.0 / s_e2e, "bytes_alg": sbytes,
                                "achieved_gbs": sbytes / (sms * 1e-3) / 1e9, "chunk_words": 1 << sinfo["wc_log2"],
                                "slots": sinfo["nslots"], "tile_rows": sinfo["tile_rows"], "autotune": single_tune,
                                "result": {"diameter": r[0], "sum": r[1], "ASPL": r[2]}}
        autotune.clear()

    if not args.no_serving and world == 1:
        line["serving"] = serving(args.serve_seconds)
    if not args.no_anneal and world == 1:
        line["anneal"] = anneal(args.serve_seconds)

    peaks, src = measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    l2 = og.measure_l2_read_gbs(48, 40)
    achieved = balg / (ms * 1e-3) / 1e9
    traffic = NCU_DRAM["bytes"] * balg / NCU_DRAM["bytes_alg"]
    line["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                        "traffic": traffic, "peak_source": src + " (MEASURED_PEAKS.json hbm_gbs)",
                        "traffic_source": "ncu DRAM bytes of one launch on the first %d graphs, scaled by algorithmic "
                                          "bytes" % NCU_DRAM["graphs"],
                        "bytes_alg_per_launch": balg, "l2_read_peak_measured": l2,
                        "frac_of_l2_read_peak": achieved / l2 if l2 > 0 else None}
    moved = NCU_DRAM["l2_read_bytes"] * balg / NCU_DRAM["bytes_alg"]
    line["roofline"].update({"l2_read_bytes_per_launch": moved, "l2_read_gbs": moved / (ms * 1e-3) / 1e9,
                             "l2_read_frac_of_l2_read_peak": moved / (ms * 1e-3) / 1e9 / l2 if l2 > 0 else None,
                             "l2_read_source": "ncu L2-to-SM read bytes of one launch on the first %d graphs, scaled "
                                               "by algorithmic bytes" % NCU_DRAM["graphs"]})
    line["clocks"] = clk.summary()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, done, dt, cres, cores = oracle_sample(specs, args.cpu_seconds)
        assert all(same(a, b) for a, b in zip(res[:done], cres)), "GPU and oracle differ"
        line["cpu_baseline"] = {"value": v, "unit": "evals/s", "cores": cores, "kind": "port",
                                "sample": "first %d graphs of the batch, %.1f s" % (done, dt)}
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
