"""Autotuner for the ASPL engine's schedule.

The engine's free choices do not change any result (they are checked bit for
bit in the tests): the column chunk width (64-bit words per row, which also
fixes the threads per row: words / 2 lanes, at most 32), the number of
concurrently active jobs (slots), the rows per tile (set through the traffic
per tile) and the per-level traffic below which one CTA runs a whole job.
This module measures candidates with the device timer (ODPX_Batch_time_mode,
CUDA events on the plan's stream, L2 flushed between runs) and installs the
winners:

* global knobs (slots, local-job threshold) through ODPX_Set_tuning;
* chunk width and tile traffic per (ceil log2 n, degree class, grid) bucket
  through ODPX_Set_tuning_table, which every plan created afterwards uses.

Typical use: ``report = tune_batch(specs)`` before timing a batch, or
``tune_single(spec)`` for one large graph.
"""
import ctypes
import math
import time

import odp_gb300 as og


class TuneEntry(ctypes.Structure):
    _fields_ = [("n_log2", ctypes.c_int), ("degree_class", ctypes.c_int), ("grid", ctypes.c_int),
                ("wc_log2", ctypes.c_int), ("tile_kb", ctypes.c_int), ("local_kb", ctypes.c_int)]


def _lib():
    lib = og.load()
    lib.ODPX_Set_tuning_table.restype = ctypes.c_int
    lib.ODPX_Set_tuning_table.argtypes = [ctypes.POINTER(TuneEntry), ctypes.c_int]
    lib.ODPX_Degree_class.restype = ctypes.c_int
    lib.ODPX_Degree_class.argtypes = [ctypes.c_int]
    return lib


def bucket(spec):
    n = spec.width * spec.height if spec.grid else spec.nodes
    return (int(math.ceil(math.log2(max(n, 2)))), int(_lib().ODPX_Degree_class(spec.degree)), int(spec.grid))


def set_table(entries):
    """Installs {bucket: dict(wc_log2=, tile_kb=, local_kb=)} in the library."""
    items = list(entries.items())
    arr = (TuneEntry * max(1, len(items)))(*[TuneEntry(b[0], b[1], b[2], v.get("wc_log2", 0), v.get("tile_kb", 0),
                                                       v.get("local_kb", 0)) for b, v in items])
    og._check(_lib().ODPX_Set_tuning_table(arr, len(items)), "ODPX_Set_tuning_table")


def clear():
    set_table({})
    og.set_tuning()


def measure(specs, repeats=3, flush_mb=256):
    """Device ms per evaluation of the whole list with the current settings."""
    b = og.Batch(specs)
    try:
        b.run()
        return b.time(repeats, mode=1, flush_mb=flush_mb)
    finally:
        b.close()


def tune_batch(specs, slots=(32, 64, 128), local_kb=(256, 2048), widths=(3, 4, 5, 6, 7), tile_kb=(128, 640, 1280),
               repeats=3, max_buckets=12, rounds=2, min_gain=0.003):
    """Tunes a batch: per-bucket passes over chunk widths and tile traffic
    (buckets in order of their share of the work, up to `rounds` times) from
    the built-in schedule, then a global pass over slots and the local-job
    threshold with the table installed.  A trial replaces the current choice
    only if it is faster by more than `min_gain` (a fraction): a greedy search
    that follows timing noise can settle on a worse schedule.  (A global pass
    before the buckets, as well, once took 128 slots on a noise-level gain
    and ended at 7.23 ms where other runs reached 6.86-6.90 ms on GB300.)
    Installs and returns the result."""
    t0 = time.perf_counter()
    clear()
    og.set_tuning()
    base = measure(specs, repeats)

    def better(ms, cur):
        return ms < cur * (1.0 - min_gain)

    def global_pass(cur, sl0, lk0):
        best = (cur, sl0, lk0)
        for sl in slots:
            for lk in local_kb:
                if (sl, lk) == (sl0, lk0):
                    continue
                og.set_tuning(slots=sl, local_kb=lk)
                ms = measure(specs, repeats)
                if better(ms, best[0]):
                    best = (ms, sl, lk)
        og.set_tuning(slots=best[1], local_kb=best[2])
        return best

    current, sl_best, lk_best = base, 0, 0
    weight = {}
    for s in specs:
        n = s.width * s.height if s.grid else s.nodes
        weight[bucket(s)] = weight.get(bucket(s), 0.0) + float(n) * n / s.symmetries * (s.degree + 2)
    order = sorted(weight, key=lambda k: -weight[k])[:max_buckets]
    table = {}
    for _ in range(rounds):
        changed = False
        for bk in order:
            for key, values in (("wc_log2", widths), ("tile_kb", tile_kb)):
                for v in values:
                    if table.get(bk, {}).get(key) == v:
                        continue
                    trial = dict(table)
                    trial[bk] = dict(table.get(bk, {}), **{key: v})
                    set_table(trial)
                    ms = measure(specs, repeats)
                    if better(ms, current):
                        current, table, changed = ms, trial, True
                set_table(table)
        if not changed:
            break
    current, sl_best, lk_best = global_pass(current, sl_best, lk_best)
    return {"default_ms": base, "tuned_ms": current, "slots": sl_best, "local_kb": lk_best,
            "buckets": {"%d/%d/%d" % k: v for k, v in table.items()},
            "seconds": time.perf_counter() - t0}


def tune_batch_best(specs, starts=2, repeats=10, **kw):
    """Runs tune_batch `starts` times and keeps the schedule that measures
    fastest over `repeats` further runs.  The greedy search ends at different
    schedules from one run to the next (on GB300, the 512-graph batch has
    ended anywhere from 6.86 to 7.17 ms), so the best of two is steadier than
    one.  Installs and returns the kept report, with every start's time."""
    best, times = None, []
    for _ in range(starts):
        r = tune_batch(specs, **kw)
        ms = measure(specs, repeats)
        times.append(ms)
        if best is None or ms < best[0]:
            best = (ms, r)
    apply(best[1])
    rep = dict(best[1])
    rep["tuned_ms"] = best[0]
    rep["starts_ms"] = times
    return rep


def tune_single(spec, widths=(3, 4, 5, 6), slots=(2, 4, 8, 16, 32), tile_kb=(128, 288, 640), repeats=3):
    """Tunes one graph's bucket (chunk width, tile traffic) and the slots."""
    clear()
    bk = bucket(spec)
    best = (measure([spec], repeats), None, 0, 0)
    for wl in widths:
        for tk in tile_kb:
            set_table({bk: {"wc_log2": wl, "tile_kb": tk}})
            for sl in slots:
                og.set_tuning(slots=sl)
                ms = measure([spec], repeats)
                if ms < best[0]:
                    best = (ms, wl, tk, sl)
                og.set_tuning()
    if best[1] is None:
        clear()
        return {"tuned_ms": best[0], "bucket": "%d/%d/%d" % bk, "default_kept": True}
    set_table({bk: {"wc_log2": best[1], "tile_kb": best[2]}})
    og.set_tuning(slots=best[3])
    return {"tuned_ms": best[0], "bucket": "%d/%d/%d" % bk, "wc_log2": best[1], "tile_kb": best[2],
            "slots": best[3]}


def apply(report):
    """Installs the result of an earlier tune_batch (its report dict): the
    per-bucket table, the slots and the local-job threshold."""
    clear()
    table = {tuple(int(x) for x in k.split("/")): v for k, v in report.get("buckets", {}).items()}
    set_table(table)
    og.set_tuning(slots=int(report.get("slots") or 0), local_kb=int(report.get("local_kb") or 0))
