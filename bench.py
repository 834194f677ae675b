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
  per_call     evals/s of one graph per call on the same GPU over the same 512
               graphs: a plan per graph (ODPX_Batch_run), the drop-in
               Init/Set/Finalize cycle, and the reference's own libodp_cuda.a
               rebuilt for sm_103a (ODP_Set_aspl per graph, in its own process)
  configs      the reference's configurations one graph at a time: n=1024 d=8;
               n=65536 d=16 (MATRIX_SAVING); n=262144 d=24 s=64; the 256x256
               grid.  Device time, ODP_Set_aspl end to end, bytes, the
               roofline fraction, and the reference's CPU (libodp_threads.a)
               and GPU (libodp_cuda.a) times for the same graph
  single_graph the n=65536, d=16 graph, autotuned
  roofline     the batched engine kernel against the L2 read ceiling (its
               bitsets are L2-resident): bytes actually read from L2 per second
               over the ceiling measured live by a streaming probe; the
               algorithmic bytes, the DRAM traffic and the HBM peak beside it
  serving      64 simulated-annealing chains (n in {1024..32768}, d in {8,16,24})
               proposing 2-opt swaps to the serving mode (ODPX_Serve_*): closed
               loop, one request outstanding per chain, exponential think time
               for a 20k req/s offered cap; p50/p99 latency, results checked
               against each graph evaluated alone; a saturating run of the
               n <= 8192 chains; per-call evals/s of the same request mix
  anneal       the same 64 chains with every step (2-opt proposal, evaluation,
               acceptance, undo) on the GPU (ODPX_Anneal), in 4 size groups
  cpu_baseline the reference's libodp_threads.a (OpenMP, all host cores) on
               the batch

--impl reference times the reference's CPU library libodp_threads.a, built
from its own sources (baseline/), on the same 512 graphs, which it generates
with the reference's own generators; that process loads nothing of
libodp_gb300.
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
WORKLOAD = ("batched: 512 graphs, seeds 100..611, n log-uniform [256, 8192], d in {4..32}, "
            "80% general / 20% grid (length 3-6), s in {1,2,4}")
L2_NOTE = "GPU arm: L2 flushed (512 MB write) before every timed device run"
# sha256 over the 512 adjacency arrays of the batch, concatenated in order: the
# same for the reference generators (baseline/ref_bench.c gen) and the
# library's own; both arms check it, so they evaluate identical graphs.
BATCH_SHA256 = "cb594241cefc45d1"
# ncu counters of one engine_kernel launch per leg, per algorithmic byte of the
# same launch (ncu --metrics dram__bytes_read.sum, dram__bytes_write.sum,
# l1tex__m_xbar2l1tex_read_bytes.sum, one launch per leg selected by its NVTX
# range with --nvtx, bytes_alg from ODPX_Batch_bytes_alg):
# "batch" is the 512-graph batch with the saved autotuned schedule, C2, C3 and
# G the configuration graphs with the default schedule.  A launch's L2 read
# bytes and DRAM traffic are taken as its algorithmic bytes times these ratios.
NCU_RATIOS = {
    "batch": {"l2_read": 0.641194, "dram": 0.092754},
    "C2": {"l2_read": 0.654699, "dram": 0.106574},
    "C3": {"l2_read": 0.784801, "dram": 0.145122},
    "G": {"l2_read": 0.261177, "dram": 0.095565},
}


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
    p.add_argument("--no-configs", action="store_true")
    p.add_argument("--no-reference-gpu", action="store_true")
    p.add_argument("--no-serving", action="store_true")
    p.add_argument("--no-anneal", action="store_true")
    p.add_argument("--no-tune", action="store_true")
    p.add_argument("--serve-seconds", type=float, default=8.0)
    p.add_argument("--configs", default="C1,C2,C3,G", help="configurations to time (comma list)")
    p.add_argument("--save-tuning", default=None, help="write the batch autotuner's result to this file")
    p.add_argument("--tuning-file", default=None, help="install this saved batch tuning instead of tuning")
    p.add_argument("--nvtx", action="store_true",
                   help="after each leg, one more launch inside an NVTX range named after the leg (batch, C1, C2, "
                        "C3, G, single), for profilers")
    return p.parse_args()


class NvtxLeg:
    """An NVTX push/pop range around one profiling launch (no-op unless enabled)."""

    def __init__(self, enabled):
        self.nvtx = None
        if enabled:
            import torch
            self.nvtx = torch.cuda.nvtx

    def run(self, name, fn):
        if self.nvtx is None:
            return
        self.nvtx.range_push(name)
        try:
            fn()
        finally:
            self.nvtx.range_pop()


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


def same(a, b):
    return a[0] == b[0] and a[1] == b[1] and float(a[2]).hex() == float(b[2]).hex()


def adjacency_sha(adjs):
    h = hashlib.sha256()
    for a in adjs:
        h.update(np.ascontiguousarray(a, dtype="<i4").tobytes())
    return h.hexdigest()[:16]


def common_config(count):
    """The `config` of both arms (identical keys and values)."""
    return {"workload": WORKLOAD, "graphs": count, "l2": L2_NOTE}


# ---------------------------------------------------------------------------
# Reference arm: libodp_threads.a on the host cores.
# ---------------------------------------------------------------------------

def unavailable(why):
    print(json.dumps({"impl": "reference", "unavailable": why}))


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    import baseline
    from odp_gb300 import workloads       # the shape list only; nothing here loads libodp_gb300
    if not baseline.cpu_available():
        ok, _ = baseline.build(cpu=True, gpu=False)
        if not ok:
            return unavailable("the reference library could not be built from baseline/_ref/src "
                               "(reference sources %s)" % ("present" if baseline.sources_present() else "absent"))
    shapes = workloads.batch_shapes(args.graphs)
    t0 = time.perf_counter()
    adjs = baseline.generate(shapes)
    gen_s = time.perf_counter() - t0
    sha = adjacency_sha(adjs)
    if args.graphs == 512 and sha != BATCH_SHA256:
        raise RuntimeError("the reference generators gave other graphs than expected (%s)" % sha)
    steps, _ = baseline.time_cpu(shapes, adjs, steps=args.steps, warmup=args.warmup, sets=2)
    total_ns = sum(s["warm_ns"] for s in steps)
    v = len(shapes) * len(steps) / (total_ns * 1e-9)
    host = baseline.host_description()
    sample = ("every step the whole batch: per graph a forked child of libodp_threads.a (Init, an untimed "
              "ODP_Set_aspl, a timed ODP_Set_aspl, Finalize), OMP_NUM_THREADS=%d; %d graphs over %d steps, "
              "%.2f s of timed Set calls" % (host["nproc"], len(shapes) * len(steps), len(steps), total_ns * 1e-9))
    line = {"metric": METRIC, "value": v, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ns * 1e-6 / len(steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (reference generators, seeded)", "impl": "reference",
            "config": common_config(len(shapes)),
            "cpu_baseline": {"value": v, "unit": "evals/s", "cores": host["nproc"], "kind": "reference",
                             "cpu_model": host["cpu_model"], "nproc": host["nproc"], "sample": sample},
            "e2e": {"value": v, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reference": {"library": "libodp_threads.a built from the reference sources (-O3 -march=native "
                                     "-fopenmp)", "generation_s": gen_s, "adjacency_sha256": sha,
                          "first_set_evals_per_s": len(shapes) * len(steps) /
                          (sum(s["first_ns"] for s in steps) * 1e-9)}}
    line["reference"]["odp_gb300_mapped"] = odp_gb300_mapped()
    if line["reference"]["odp_gb300_mapped"]:
        raise RuntimeError("the reference arm mapped a libodp_gb300 library")
    print(json.dumps(line))


def odp_gb300_mapped():
    """True if this process has any libodp_gb300 library mapped."""
    try:
        with open("/proc/self/maps") as f:
            return any("libodp_gb300" in ln for ln in f)
    except OSError:
        return False


# ---------------------------------------------------------------------------
# Own arm.
# ---------------------------------------------------------------------------

def batch_workload(count):
    from odp_gb300 import workloads
    shapes = workloads.batch_shapes(count)
    return shapes, workloads.build_graphs(shapes)


def load_golden():
    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        return json.load(f)


def config_graphs():
    """The reference's four configurations: (name, workload, spec, shape,
    expected result, env for the reference library)."""
    import odp_gb300 as og
    gold = {g.get("name") or (g["kind"], g.get("nodes"), g.get("degree"), g.get("seed")): g
            for g in load_golden()["generators"]}

    def expect(r):
        return (r[0], r[1], float.fromhex(r[2]))

    out = []
    for name, key, n, d, s, seed, env in (
            ("C1", ("general", 1024, 8, 1), 1024, 8, 1, 1, None),
            ("C2", "single_large_65536", 65536, 16, 1, 2, {"ODP_ASPL": "MATRIX_SAVING"}),
            ("C3", "symmetric_262144", 262144, 24, 64, 3, None)):
        g = gold[key]
        e = og.generate_random_general(n, d, s, seed=seed)
        if hashlib.sha256(np.ascontiguousarray(e, dtype=np.int32).tobytes()).hexdigest() != g["sha256"]:
            raise RuntimeError("generated %s graph differs from the reference's" % name)
        adj = og.conv_edge2adjacency_general(n, e, d, s)
        out.append(dict(name=name, workload="general n=%d d=%d s=%d seed=%d" % (n, d, s, seed),
                        spec=og.GraphSpec(adj, nodes=n, symmetries=s),
                        shape=dict(grid=False, nodes=n, degree=d, symmetries=s, seed=seed),
                        expected=expect(g["reference"]), env=env))
    g = gold["grid_256x256"]
    z = np.load(os.path.join(ROOT, "tests", "golden", "grid_256x256_d6_l4_seed4.npz"))
    codes = z["codes"].astype(np.int32)
    w = h = 256
    v = np.arange(w * h)[:, None]
    adj = ((v // h + codes // 9 - 4) * h + (v % h + codes % 9 - 4)).astype(np.int32)
    if hashlib.sha256(adj.tobytes()).hexdigest() != bytes(z["adjacency_sha256"]).decode():
        raise RuntimeError("256x256 grid fixture damaged")
    out.append(dict(name="G", workload="grid 256x256 d=6 length 4 seed=4 (diameter 140)",
                    spec=og.GraphSpec(adj, grid=True, width=w, height=h),
                    shape=dict(grid=True, width=w, height=h, degree=6, length=4, symmetries=1, seed=4),
                    expected=expect(g["reference"]), env=None))
    return out


def live_bytes(spec, info):
    """Bytes of the bitset buffers a plan keeps live (both buffers of every slot)."""
    n = spec.width * spec.height if spec.grid else spec.nodes
    return 2.0 * info["nslots"] * n * 8.0 * (1 << info["wc_log2"])


def time_configs(args, l2_gbs, hbm_gbs, l2_bytes, nvtx):
    import odp_gb300 as og
    import baseline
    out = {}
    reps = {"C1": 200, "C2": 10, "C3": 20, "G": 4}
    wanted = set(args.configs.split(","))
    for c in config_graphs():
        spec, name = c["spec"], c["name"]
        if name not in wanted:
            continue
        b = og.Batch([spec])
        r = b.run()[0]
        assert same(r, c["expected"]), (name, r, c["expected"])
        b.time(2, mode=1, flush_mb=args.flush_mb)
        ms = b.time(reps[name], mode=1, flush_mb=args.flush_mb)
        balg = b.bytes_alg()
        info = b.info(0)
        kernel = b.kernel()
        shape = b.small_shape() if kernel == "small" else None
        nvtx.run(name, lambda: b.time(1, mode=1, flush_mb=args.flush_mb))
        b.close()
        # ODP_Set_aspl end to end: host adjacency, copies and decode included
        nd = None
        if spec.grid:
            og.init_aspl_grid(spec.width, spec.height, spec.degree, nd)
        elif spec.symmetries == 1:
            og.init_aspl_general(spec.nodes, spec.degree, nd)
        else:
            og.init_aspl_general_s(spec.nodes, spec.degree, nd, spec.symmetries)
        og.set_aspl(spec.adjacency)
        k = reps[name]
        t0 = time.perf_counter()
        for _ in range(k):
            r2 = og.set_aspl(spec.adjacency)
        e2e_ms = (time.perf_counter() - t0) * 1e3 / k
        og.finalize_aspl()
        assert same(r2, c["expected"])
        live = live_bytes(spec, info)
        rec = {"workload": c["workload"], "kernel": kernel, "device_ms": ms, "set_aspl_e2e_ms": e2e_ms,
               "bytes_alg": balg, "alg_gbs": balg / (ms * 1e-3) / 1e9, "live_bitset_bytes": live,
               "schedule": {"chunk_words": 1 << info["wc_log2"], "jobs": info["njobs"], "slots": info["nslots"],
                            "tile_rows": info["tile_rows"]},
               "result": {"diameter": r[0], "sum": r[1], "ASPL": r[2]}}
        if shape:
            rec["schedule"] = {"chunk_words": 1 << info["wc_log2"], "jobs": info["njobs"], "cluster_ctas": shape[0],
                               "threads_per_cta": shape[1], "rows_partitioned": bool(shape[2])}
        ratio = NCU_RATIOS.get(name)
        if ratio:
            # the bound is whichever of L2 reads and DRAM traffic is nearer its ceiling
            moved, dram = balg * ratio["l2_read"], balg * ratio["dram"]
            l2f = moved / (ms * 1e-3) / 1e9 / l2_gbs
            dramf = dram / (ms * 1e-3) / 1e9 / hbm_gbs
            rec.update({"l2_read_bytes": moved, "l2_read_gbs": moved / (ms * 1e-3) / 1e9, "l2_read_frac": l2f,
                        "dram_bytes": dram, "dram_gbs": dram / (ms * 1e-3) / 1e9, "dram_frac_of_hbm": dramf,
                        "bound": "l2" if l2f >= dramf else "hbm", "frac": max(l2f, dramf)})
        else:
            rec["bound"] = "l2" if live <= l2_bytes else "hbm"
        if baseline.cpu_available() and not args.no_cpu_baseline:
            sets = 1 if name == "G" else 2
            steps, res = baseline.time_cpu([c["shape"]], [spec.adjacency], steps=1 if name in ("G", "C2", "C3")
                                           else 20, warmup=0, sets=sets, env=c["env"])
            assert same(res[0][:3], c["expected"]), (name, res[0])
            rec["reference_cpu_ms"] = min(s["warm_ns"] for s in steps) * 1e-6
            rec["reference_cpu_env"] = c["env"] or {}
        if baseline.gpu_available() and not args.no_reference_gpu:
            res = baseline.time_gpu([c["shape"]], [spec.adjacency], reps=1 if name == "G" else 3, env=c["env"])
            assert same(res[0][:3], c["expected"]), (name, res[0])
            rec["reference_cuda_ms"] = res[0][3] * 1e-6
        out[name] = rec
    return out


def oracle_sample(specs, seconds):
    """The oracle port on graphs taken in order until `seconds` of CPU work
    (the CPU baseline where the reference library is not built)."""
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


def percentiles(v):
    a = np.array(v) * 1e3
    return {"p50": float(np.percentile(a, 50)), "p99": float(np.percentile(a, 99)), "mean": float(a.mean()),
            "requests": len(v)}


def serve_native(shapes, seconds, think_us, temperature=50.0, lanes=4, max_batch=16, memory_mb=4096):
    """The served annealing chains driven by the native client (serve_load):
    one host thread per chain, no Python in the loop.  Returns its report;
    it fails unless every chain's last served result equals its graph
    evaluated alone."""
    from odp_gb300 import build as b
    chains = ["%d:%d:%d:%d" % (s["nodes"], s["degree"], s["seed"], s["proposal_seed"]) for s in shapes]
    r = subprocess.run([b.SERVE_LOAD, "%g" % seconds, "%g" % think_us, str(lanes), str(max_batch), str(memory_mb),
                        "%g" % temperature] + chains, capture_output=True, text=True, timeout=seconds + 300)
    if r.returncode != 0:
        raise RuntimeError("serve_load failed (%d): %s" % (r.returncode, r.stderr[-2000:]))
    return json.loads(r.stdout.strip().splitlines()[-1])


def serving(seconds, rate=20000.0, saturate_seconds=4.0):
    """The served annealing workload; returns the report dict."""
    import odp_gb300 as og
    from odp_gb300 import workloads
    shapes = workloads.chain_shapes(64)
    specs = workloads.build_graphs(shapes)
    srv = og.Server(lanes=4, max_batch=16, max_nodes=32768, memory_mb=4096)
    handles = [srv.register(og.GraphSpec(s.adjacency.copy(), nodes=s.nodes)) for s in specs]
    hosts = [s.adjacency.copy() for s in specs]
    undos = [[] for _ in specs]
    lock = threading.Lock()

    def run(chains, secs, think_mean):
        lat, lat_by_n, stop_at = [], {}, time.perf_counter() + secs

        def chain(k):
            sh = shapes[k]
            n, d = sh["nodes"], sh["degree"]
            host = hosts[k]
            rng = og.Rng(sh["proposal_seed"] + (7919 if think_mean == 0 else 0))
            draw = np.random.default_rng(sh["proposal_seed"])
            current = srv.wait(srv.submit(handles[k], undos[k]))[2]
            undo, local = [], []
            while time.perf_counter() < stop_at:
                if think_mean > 0:
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
            undos[k] = undo
            with lock:
                lat.extend(local)
                lat_by_n.setdefault(n, []).extend(local)

        threads = [threading.Thread(target=chain, args=(k,)) for k in chains]
        t0 = time.perf_counter()
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        return time.perf_counter() - t0, lat, lat_by_n

    wall, lat, lat_by_n = run(range(len(shapes)), seconds, len(shapes) / rate)
    st = srv.stats()
    # every chain's resident graph followed its client, and its served result
    # equals the same graph evaluated alone, bit for bit
    finals = [srv.wait(srv.submit(handles[k], undos[k])) for k in range(len(shapes))]
    for k in range(len(shapes)):
        assert np.array_equal(srv.adjacency(handles[k]), hosts[k])
    srv.close()
    alone = og.Batch([og.GraphSpec(hosts[k], nodes=shapes[k]["nodes"]) for k in range(len(shapes))])
    ares = alone.run()
    alone.close()
    checked = {}
    for k, (f, a) in enumerate(zip(finals, ares)):
        assert same(f[:3], a), ("served and alone differ", k, f, a)
        checked[str(shapes[k]["nodes"])] = checked.get(str(shapes[k]["nodes"]), 0) + 1
    # one call at a time: ODP_Set_aspl per proposal, as the reference's annealing samples do
    per_call_ms = {}
    for n in sorted({s["nodes"] for s in shapes}):
        ts = []
        for k in [i for i, s in enumerate(shapes) if s["nodes"] == n][:3]:
            og.init_aspl_general(n, shapes[k]["degree"])
            og.set_aspl(hosts[k])
            t1 = time.perf_counter()
            for _ in range(5):
                og.set_aspl(hosts[k])
            ts.append((time.perf_counter() - t1) / 5)
            og.finalize_aspl()
        per_call_ms[n] = float(np.mean(ts)) * 1e3

    def same_mix(by_n):
        """Evals/s of one ODP_Set_aspl call per request, for the same requests."""
        cnt = sum(by_n.values())
        return cnt / sum(k * per_call_ms[n] * 1e-3 for n, k in by_n.items())

    # the same chains from the native client: at the offered cap, and saturating with the n <= 8192 chains
    native = serve_native(shapes, seconds, 1e6 * len(shapes) / rate)
    small = [s for s in shapes if s["nodes"] <= 8192]
    sat = serve_native(small, saturate_seconds, 0.0)
    for rep in (native, sat):
        rep["per_call_evals_per_s_same_mix"] = same_mix({int(k): v["requests"] for k, v in rep["by_n"].items()})
        rep["served_over_per_call"] = rep["evals_per_s"] / rep["per_call_evals_per_s_same_mix"]
    native["workload"] = "the 64 chains, native client (one host thread per chain), exponential think time for " \
                         "a %d req/s offered cap" % int(rate)
    sat["workload"] = "the %d chains with n <= 8192, native client, no think time" % len(small)

    done = len(lat)
    return {"workload": "64 annealing chains, n in {1024,4096,16384,32768}, d in {8,16,24}, 2-opt proposals, "
                        "closed loop (1 outstanding per chain), exponential think time for a %d req/s offered cap"
                        % int(rate),
            "seconds": wall, "completed": done, "evals_per_s": done / wall, "offered_cap_req_per_s": rate,
            "latency_ms": percentiles(lat),
            "latency_ms_by_n": {str(k): percentiles(v) for k, v in sorted(lat_by_n.items())},
            "evals_per_s_by_n": {str(k): len(v) / wall for k, v in sorted(lat_by_n.items())},
            "per_call_ms_by_n": {str(k): v for k, v in per_call_ms.items()},
            "per_call_evals_per_s_same_mix": same_mix({n: len(v) for n, v in lat_by_n.items()}),
            "client": "python threads (one per chain)",
            "batches": st["batches"], "mean_batch": st["batched_requests"] / max(1, st["batches"]),
            "max_batch": st["max_batch"], "max_concurrent_lanes": st["max_inflight_lanes"],
            "native_client": native,
            "saturating_small": sat,
            "results_checked_alone_by_n": checked,
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


def pin_local_gpu(local):
    """Under torchrun every rank evaluates on its own GPU: CUDA_VISIBLE_DEVICES
    is narrowed to the rank's local device before anything initialises CUDA
    in this process.  Returns the device's index for nvidia-smi."""
    visible = os.environ.get("CUDA_VISIBLE_DEVICES")
    devices = [d for d in visible.split(",") if d.strip()] if visible else None
    dev = devices[local % len(devices)].strip() if devices else str(local)
    os.environ["CUDA_VISIBLE_DEVICES"] = dev
    return int(dev) if dev.isdigit() else local


def run_own(args):
    rank, world, local = dist_info()
    smi_index = pin_local_gpu(local) if world > 1 else local
    dist = Dist(world)
    import odp_gb300 as og
    import baseline
    og.load()
    shapes, specs = batch_workload(args.graphs)
    count = len(specs)
    if count == 512 and adjacency_sha([s.adjacency for s in specs]) != BATCH_SHA256:
        raise RuntimeError("the batch's graphs differ from the reference generators'")
    adj_bytes = int(sum(s.adjacency.nbytes for s in specs))
    peaks, peak_src = measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    # the L2 read ceiling: the best of three probes of about a millisecond
    # each (probes of 0.1 ms, early in a short run, have read as low as
    # 12.8 TB/s on GPUs whose later probes read 18-19 TB/s)
    l2_gbs = max(og.measure_l2_read_gbs(48, 400) for _ in range(3))

    # ---- autotune the schedule for this batch (outside every timed region) ----
    from odp_gb300 import autotune
    nvtx = NvtxLeg(args.nvtx)
    if args.tuning_file:
        with open(args.tuning_file) as f:
            tune_report = json.load(f)
        autotune.apply(tune_report)
        tune_report = dict(tune_report, loaded_from=args.tuning_file)
    else:
        tune_report = autotune.tune_batch_best(specs) if not args.no_tune else None
    if args.save_tuning and tune_report is not None:
        with open(args.save_tuning, "w") as f:
            json.dump(tune_report, f)

    # ---- batched engine on resident inputs (headline) ----
    batch = og.Batch(specs)
    res = batch.run()
    for _ in range(args.warmup):
        batch.time(1, mode=1, flush_mb=args.flush_mb)
    dist.barrier()
    with ClockSampler(smi_index) as clk:
        ms = batch.time(args.steps, mode=1, flush_mb=args.flush_mb)
    ms = dist.max(ms)
    dist.barrier()
    value = world * count * 1000.0 / ms
    balg = batch.bytes_alg()
    info = batch.info(0)
    nvtx.run("batch", lambda: batch.time(1, mode=1, flush_mb=args.flush_mb))
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
            "config": common_config(count),
            "schedule": {"jobs": info["njobs"], "slots": info["nslots"],
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
        e2e_v = count / e2e_s
        pcd = {"evals_per_s": count / pc_s, "form": "one plan per graph, ODPX_Batch_run each",
               "drop_in_init_set_finalize_evals_per_s": 1.0 / dropin_s,
               "batched_e2e_over_per_call": e2e_v / (count / pc_s),
               "batched_device_over_per_call": (count * 1000.0 / ms) / (count / pc_s)}
        if baseline.gpu_available() and not args.no_reference_gpu:
            rg = baseline.time_gpu(shapes, [s.adjacency for s in specs], reps=2)
            assert all(same(a, b[:3]) for a, b in zip(res, rg)), "reference CUDA library and batch differ"
            ref_s = sum(r[3] for r in rg) * 1e-9
            pcd["reference_cuda_per_call"] = {
                "evals_per_s": count / ref_s,
                "form": "the reference's libodp_cuda.a built from its sources for sm_103a, in its own process: "
                        "per graph Init, an untimed and 2 timed ODP_Set_aspl (mean), Finalize",
                "results_equal_batch": True}
            pcd["batched_e2e_over_faster_per_call"] = e2e_v / max(count / pc_s, count / ref_s)
        else:
            pcd["reference_cuda_per_call"] = "unavailable: the reference CUDA library was not built here"
        line["per_call"] = pcd

    # ---- the reference's configurations, one graph each ----
    l2_bytes = 126.5e6
    if not args.no_configs:
        line["configs"] = time_configs(args, l2_gbs, hbm, l2_bytes, nvtx)

    # ---- the single large graph (MATRIX_SAVING configuration), autotuned ----
    if not args.no_single:
        c2 = [c for c in config_graphs() if c["name"] == "C2"][0]
        spec = c2["spec"]
        single_tune = autotune.tune_single(spec) if not args.no_tune else None
        sb = og.Batch([spec])
        r = sb.run()[0]
        assert same(r, c2["expected"]), r
        sb.time(2, mode=1, flush_mb=args.flush_mb)
        sms = sb.time(max(3, args.steps // 2), mode=1, flush_mb=args.flush_mb)
        sbytes = sb.bytes_alg()
        sinfo = sb.info(0)
        nvtx.run("single", lambda: sb.time(1, mode=1, flush_mb=args.flush_mb))
        sb.close()
        line["single_graph"] = {"workload": c2["workload"] + " (autotuned)", "evals_per_s": 1000.0 / sms,
                                "ms": sms, "bytes_alg": sbytes, "achieved_alg_gbs": sbytes / (sms * 1e-3) / 1e9,
                                "chunk_words": 1 << sinfo["wc_log2"], "slots": sinfo["nslots"],
                                "tile_rows": sinfo["tile_rows"], "autotune": single_tune,
                                "result": {"diameter": r[0], "sum": r[1], "ASPL": r[2]}}
        autotune.clear()

    if not args.no_serving and world == 1:
        line["serving"] = serving(args.serve_seconds)
    if not args.no_anneal and world == 1:
        line["anneal"] = anneal(args.serve_seconds)

    # ---- roofline of the headline kernel: the batched engine against L2 ----
    rat = NCU_RATIOS["batch"]
    moved = balg * rat["l2_read"]
    achieved = moved / (ms * 1e-3) / 1e9
    line["roofline"] = {"bound": "l2", "achieved": achieved, "peak": l2_gbs, "unit": "GB/s",
                        "frac": achieved / l2_gbs, "traffic": balg * rat["dram"],
                        "kernel": "engine_kernel",
                        "achieved_source": "bytes read from L2 by the SMs per launch (ncu "
                                           "l1tex__m_xbar2l1tex_read_bytes.sum per algorithmic byte, one launch of "
                                           "the tuned 512-graph batch, times this launch's algorithmic bytes) / the "
                                           "launch's CUDA-event time",
                        "peak_source": "L2 read ceiling measured live in this run by a streaming probe of 16-byte "
                                       "L2-only loads over a 48 MB L2-resident buffer (MEASURED_PEAKS.json has no "
                                       "L2 figure)",
                        "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per algorithmic byte, "
                                          "same capture, times this launch's algorithmic bytes",
                        "bytes_alg_per_launch": balg, "alg_gbs": balg / (ms * 1e-3) / 1e9,
                        "alg_frac_of_l2_peak": balg / (ms * 1e-3) / 1e9 / l2_gbs,
                        "dram_gbs": balg * rat["dram"] / (ms * 1e-3) / 1e9,
                        "dram_frac_of_hbm": balg * rat["dram"] / (ms * 1e-3) / 1e9 / hbm,
                        "hbm_peak": hbm, "hbm_peak_source": peak_src + " (MEASURED_PEAKS.json hbm_gbs)"}
    line["clocks"] = clk.summary()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        host = baseline.host_description()
        if baseline.cpu_available():
            steps, cres = baseline.time_cpu(shapes, [s.adjacency for s in specs], steps=1, warmup=0, sets=2)
            assert all(same(a, b[:3]) for a, b in zip(res, cres)), "GPU and reference CPU library differ"
            v = count / (steps[0]["warm_ns"] * 1e-9)
            line["cpu_baseline"] = {"value": v, "unit": "evals/s", "cores": host["nproc"], "kind": "reference",
                                    "cpu_model": host["cpu_model"], "nproc": host["nproc"],
                                    "sample": "the whole batch once: per graph a forked child of libodp_threads.a "
                                              "(Init, an untimed and a timed ODP_Set_aspl, Finalize), "
                                              "OMP_NUM_THREADS=%d; %.2f s of timed Set calls"
                                              % (host["nproc"], steps[0]["warm_ns"] * 1e-9)}
        else:
            v, done, dt, cres, cores = oracle_sample(specs, 10.0)
            assert all(same(a, b) for a, b in zip(res[:done], cres)), "GPU and oracle differ"
            line["cpu_baseline"] = {"value": v, "unit": "evals/s", "cores": cores, "kind": "port",
                                    "cpu_model": host["cpu_model"], "nproc": host["nproc"],
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
