#!/usr/bin/env python
"""Benchmark of the rule-based blocking hot path: pair-comparisons/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

Headline workload: C3, the configuration the batched-vs-plain target is
quoted on -- 1,000,000 x 1,000,000 seeded synthetic bibliographic rows (header
line included as data, as the reference reads it), 8 rules mixing 1-2
equalities with 1-3 Jaro-Winkler predicates (thresholds U[0.80, 0.95]), 64
hash partitions of Zipf(1.3) sizes.  A step is one pass of the hot path over
the whole workload: equality join, Jaro-Winkler pair evaluation and
compaction of the matching pairs.

* ``value``: pair-comparisons/s of the engine's default (batched: one
  persistent work-stealing launch replayed from a CUDA graph) with the inputs
  resident in HBM (about 200 MB a side, larger than L2; L2 is also flushed
  with a 256 MiB write before every timed step); every step is timed with
  CUDA events on the launching stream.
* ``plain``: the same with one launch per (partition, rule), like the
  reference's per-partition submission.
* ``e2e``: the same metric through the one-shot C-ABI call ``hbx_block``
  from host tables to host pair buffers (encode + H2D + run + D2H inside the
  timed region).
* ``parity``: the engine's pairs of a stratified sample of left rows (the
  same number from every partition) against the oracle's on the same rows;
  the oracle run is also the ``cpu_baseline`` (all host cores).
* ``roofline``: the pair-evaluation kernel against the measured rate of the
  bit-parallel scan step (libhbx_probe.so), with the fraction of the
  algorithmic count and of the scan operations actually executed.
* ``jw_fp64``: the reference's float/double Jaro-Winkler against a
  double-only restatement over the oracle runs (largest difference, decisions
  it would flip); the set is the reference's either way.

At N=1 more workloads are reported in the same line (``--sections``): ``c2``
(2,600 x 64,263 rows, 2 rules, 8 partitions, checked in full), ``c5`` (long
strings: one-shot vs partition windows streamed under a memory budget,
sampled parity), ``serve`` (10M resident right rows, a Poisson trace of
requests: p50/p99/p999 latency, small requests checked against the oracle)
and ``io`` (CSV tokenization and pair-file writing, device vs host).

``--impl reference`` times the CPU implementation of the path (the oracle:
the reference's brute-force algorithm restated in C++, all host cores) on
stratified samples of the same C3 workload and prints the same line with
``"impl": "reference"``.  With N > 1 GPUs (torchrun) every rank runs an
independent replica (weak scaling); the path needs no collective.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pair-comparisons/s, batched vs plain, same GPU, exact set; serving p50/p99 ms"
UNIT = "pair-comparisons/s"


def c3_desc(n: int) -> str:
    return (f"c3: {n:,} x {n:,} synthetic bibliographic rows (+1 header row each), 8 rules (1-2 "
            "equalities, 1-3 JW predicates, thresholds U[0.80,0.95]), 64 partitions keyed by a "
            "Zipf(1.3) column")


C2_DESC = ("c2: 2,600 x 64,263 synthetic bibliographic rows (+1 header row each), 5k true pairs, "
           "rules (year eq, JW(title)>=0.89, JW(authors)>=0.85) | (venue eq, JW(title)>=0.95), "
           "8 partitions")


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.proc:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                   "reasons": sorted(reasons), "samples": len(sm)}
        return out


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def _traffic_record():
    """DRAM bytes of one evaluation launch on C3 from the committed ncu summary
    (ncu cannot run inside the timed bench); labelled with its source."""
    p = os.path.join(ROOT, "profiles", "k_eval_c3_traffic.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return d.get("dram_bytes_per_launch"), f"profiles/k_eval_c3_traffic.json ({d.get('source', '')})"
    except Exception:
        return None, "not measured"


# ------------------------------------------------------------------ helpers
def oracle_plan(docs):
    from oracle import rules

    return rules.serialize(rules.sort_rules([rules.decode_rule(rules.parse_yaml(d)) for d in docs]))


def stratified_rows(ctable, plan_o, n_partitions, per_part, seed):
    """A left-row filter with up to per_part rows of every partition (rows
    drawn from PCG64(seed)); returns (uint8 filter, rows chosen)."""
    import numpy as np

    from oracle import api

    bucket = api.partition(ctable, plan_o, n_partitions)
    rng = np.random.Generator(np.random.PCG64(seed))
    filt = np.zeros(ctable.n_rows, dtype=np.uint8)
    for p in range(n_partitions):
        rows = np.nonzero(bucket == p)[0]
        if len(rows):
            filt[rng.choice(rows, size=min(per_part, len(rows)), replace=False)] = 1
    return filt, int(filt.sum())


def device_pairs_of_rows(out_l, out_r, n, filt, dev):
    """The engine's pairs (device arrays) whose left row is in filt, sorted."""
    import numpy as np
    import torch

    from tests._util import sorted_pairs

    mask = torch.from_numpy(filt).to(dev)
    keep = torch.index_select(mask, 0, out_l[:n]).bool()
    l = out_l[:n][keep].cpu().numpy().view(np.uint32)
    r = out_r[:n][keep].cpu().numpy().view(np.uint32)
    return sorted_pairs(np.stack([l, r], axis=1))


def fp64_block(res):
    return {"jw_evals": int(res.jw_evals), "fp64_flips": int(res.fp64_flips),
            "max_abs_diff": float(res.fp64_max_abs_diff), "fma_ambiguous": int(res.fma_ambiguous)}


def probe_scan_peak(device: int, words: int):
    """Measured rate of the bit-parallel scan step (libhbx_probe.so): best over
    CTA counts, in the roofline's unit (6 operations per 64-bit mask word per
    character)."""
    from hyperblocker_gb300 import build as hbuild

    lib = ctypes.CDLL(hbuild.PROBE_LIB)
    lib.hbx_probe_scan_rate.restype = ctypes.c_int
    lib.hbx_probe_scan_rate.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_uint32, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_double)]
    w = {1: 1, 2: 2, 3: 4, 4: 4}.get(words, 8)
    best, per = 0.0, {}
    for chains in (4, 8):
        iters = max(256, 16384 // w // (chains // 4))
        for bps in (1, 2, 3, 4, 6, 8):
            ops, ms = ctypes.c_double(), ctypes.c_double()
            rc = lib.hbx_probe_scan_rate(device, w, chains, bps, iters, ctypes.byref(ops),
                                         ctypes.byref(ms))
            if rc != 0:
                continue
            per[f"{chains}x{bps}"] = round(ops.value / 1e12, 3)
            best = max(best, ops.value)
    return {"tops": best / 1e12, "words": w, "per_chains_x_ctas_per_sm": per}


# ------------------------------------------------------------------ C3 (headline)
class C3:
    """The C3 workload, its engine session and device output buffers."""

    def __init__(self, args, ctx, dev):
        import torch

        import hyperblocker_gb300 as hb
        from hyperblocker_gb300 import synth_big

        self.n = args.c3_rows
        self.w = synth_big.c3(self.n, self.n, max(1, self.n // 50))
        self.plan = hb.Plan.from_yaml(self.w.rules, ctx)
        self.L = hb.Table.from_columns(self.w.left.cols, ctx)
        self.R = hb.Table.from_columns(self.w.right.cols, ctx)
        self.sess = hb.Session(ctx, self.plan, self.L, self.R, self.w.n_partitions)
        self.stream = torch.cuda.Stream(device=dev)
        self.dev = dev
        m = self.sess.count("batched", self.stream.cuda_stream)  # runs the autotuner too
        self.cap = max(1, m)
        self.out_l = torch.empty(self.cap, dtype=torch.int32, device=dev)
        self.out_r = torch.empty(self.cap, dtype=torch.int32, device=dev)
        self.flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step(self, mode):
        return self.sess.run_device(mode, self.out_l.data_ptr(), self.out_r.data_ptr(), self.cap,
                                    self.stream.cuda_stream)

    def timed(self, mode, k, warm):
        """warm untimed steps, then k timed ones, inside an NVTX range named
        c3_<mode> (an ncu capture can pick the form's launches by it)."""
        import torch

        torch.cuda.nvtx.range_push(f"c3_{mode}")
        for _ in range(warm):
            self.step(mode)
        rec = {"ms": [], "ms_eval": [], "ops": [], "scan_ops": [], "scanned": [], "cmp": [],
               "launches": 0, "matches": 0, "stats": None}
        with torch.cuda.stream(self.stream):
            for _ in range(k):
                self.flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(self.stream)
                n = self.step(mode)
                e1.record(self.stream)
                e1.synchronize()
                st = self.sess.stats()
                rec["ms"].append(e0.elapsed_time(e1))
                rec["ms_eval"].append(st.ms_eval)
                rec["ops"].append(st.jw_word_ops)
                rec["scan_ops"].append(st.scan_word_ops)
                rec["scanned"].append(st.pairs_scanned)
                rec.setdefault("rest", []).append(st.rest_scans)
                rec.setdefault("lane_util", []).append(
                    st.scan_steps / (128.0 * st.scan_warp_steps) if st.scan_warp_steps else None)
                rec["cmp"].append(st.pair_comparisons)
                rec["launches"] += st.n_launches
                rec["matches"] = n
                rec["stats"] = st  # of the form's last step
        torch.cuda.nvtx.range_pop()
        return rec

    def parity(self, args, n_matches):
        """Sampled check against the oracle; its run is the CPU baseline."""
        import numpy as np

        from oracle import api

        plan_o = oracle_plan(self.w.rules)
        Lo, Ro = api.CTable(self.w.left.cols), api.CTable(self.w.right.cols)
        filt, n_rows = stratified_rows(Lo, plan_o, self.w.n_partitions, args.c3_sample_per_part, 7)
        cores = os.cpu_count() or 1
        t = time.perf_counter()
        res = api.run_block(Lo, Ro, plan_o, self.w.n_partitions, n_threads=cores,
                            left_row_filter=filt)
        dt = time.perf_counter() - t
        got = device_pairs_of_rows(self.out_l, self.out_r, n_matches, filt, self.dev)
        equal = bool(np.array_equal(got, res.pairs))
        parity = {"sampled_left_rows": n_rows, "per_partition": args.c3_sample_per_part,
                  "rules": len(self.w.rules), "partitions": self.w.n_partitions,
                  "pairs": int(len(res.pairs)), "engine_pairs": int(len(got)),
                  "pairs_covered": int(res.pairs_covered), "equal": equal}
        cpu = {"value": res.pair_comparisons / dt, "unit": UNIT, "cores": cores, "kind": "port",
               "seconds": dt,
               "sample": f"{n_rows} left rows of C3 ({args.c3_sample_per_part} per partition, "
                         f"seed 7) against their partitions' right rows: {res.pairs_covered} "
                         f"pairs covered, {res.pair_comparisons} pair-comparisons in {dt:.2f} s"}
        return parity, cpu, fp64_block(res)

    def e2e(self, ctx, steps):
        """hbx_block from host tables to host pairs (caller-kept host buffers)."""
        import numpy as np

        import hyperblocker_gb300 as hb

        cap = self.cap + 1024
        out = (np.zeros(cap, dtype=np.uint32), np.zeros(cap, dtype=np.uint32))  # touched once
        hb.block(ctx, self.plan, self.L, self.R, self.w.n_partitions, hb.INT_MAX, "batched",
                 capacity=cap, out=out, stack=False)  # warm: page-locking, predicate order
        ts = []
        for _ in range(steps):
            t0 = time.perf_counter()
            # the C-ABI call into the caller's two row arrays (kept between calls)
            pairs, st = hb.block(ctx, self.plan, self.L, self.R, self.w.n_partitions, hb.INT_MAX,
                                 "batched", capacity=cap, out=out, stack=False)
            ts.append(time.perf_counter() - t0)
        s = statistics.mean(ts)
        return {"value": st.pair_comparisons / s, "unit": UNIT,
                "h2d_bytes_per_step": int(st.h2d_bytes),
                "d2h_bytes_per_step": int(8 * st.n_matches + 64),
                "ms_per_step": 1000.0 * s, "ms_create": float(st.ms_create),
                "ms_run_device": float(st.ms_last_run), "steps": steps,
                "ingest_on_device": int(st.ingest_on_device),
                "includes": "session creation (H2D of the plan's columns from page-locked host "
                            "tables, device encode: std::hash partition buckets, dictionaries, "
                            "symbol arenas, Peq tables) + join + evaluation + D2H of the pairs "
                            "into the caller's host arrays; the warm-up call page-locks the "
                            "tables and memoises the measured predicate order on the plan"}

    def close(self):
        self.sess.close()


# ------------------------------------------------------------------ C2
def bench_c2(args, ctx, dev):
    """C2 read from CSV files: batched vs plain, end to end, and the full
    pair set against the oracle (which is also its CPU baseline)."""
    import numpy as np
    import torch

    import hyperblocker_gb300 as hb
    from hyperblocker_gb300 import synth
    from oracle import api, csvref, rules
    from tests._util import sorted_pairs

    with tempfile.TemporaryDirectory() as d:
        w = synth.c2()
        paths = synth.materialize(w, d)
        plan = hb.Plan.from_rule_dir(paths["rules"], ctx)
        L = hb.Table.from_csv(paths["left"], ",", ctx)
        R = hb.Table.from_csv(paths["right"], ",", ctx)
        sess = hb.Session(ctx, plan, L, R, w.n_partitions)
        stream = torch.cuda.Stream(device=dev)
        cap = 1 << 20
        out_l = torch.empty(cap, dtype=torch.int32, device=dev)
        out_r = torch.empty(cap, dtype=torch.int32, device=dev)
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
        res = {}
        for mode in ("batched", "plain"):
            for _ in range(3):
                sess.run_device(mode, out_l.data_ptr(), out_r.data_ptr(), cap, stream.cuda_stream)
            ms, ms_eval, ms_join = [], [], []
            torch.cuda.nvtx.range_push(f"c2_{mode}")  # names the timed launches for profilers
            with torch.cuda.stream(stream):
                for _ in range(args.c2_steps):
                    flush.zero_()
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    n = sess.run_device(mode, out_l.data_ptr(), out_r.data_ptr(), cap,
                                        stream.cuda_stream)
                    e1.record(stream)
                    e1.synchronize()
                    ms.append(e0.elapsed_time(e1))
                    ms_eval.append(sess.stats().ms_eval)
                    ms_join.append(sess.stats().ms_join)
            torch.cuda.nvtx.range_pop()
            st = sess.stats()
            res[mode] = {"value": st.pair_comparisons / (statistics.mean(ms) / 1000.0),
                         "ms_per_step": statistics.mean(ms), "ms_eval": statistics.mean(ms_eval),
                         "ms_join": statistics.mean(ms_join), "launches_per_step": int(st.n_launches)}
        st = sess.stats()
        got = sorted_pairs(np.stack([out_l[:n].cpu().numpy().view(np.uint32),
                                     out_r[:n].cpu().numpy().view(np.uint32)], axis=1))
        hb.block(ctx, plan, L, R, w.n_partitions, hb.INT_MAX, "batched")  # warm
        t0 = time.perf_counter()
        e2e_steps = 5
        for _ in range(e2e_steps):
            pairs, st_e2e = hb.block(ctx, plan, L, R, w.n_partitions, hb.INT_MAX, "batched")
        e2e_s = (time.perf_counter() - t0) / e2e_steps
        # the oracle over every pair (all host cores): parity and CPU baseline
        cl = csvref.read_columns(paths["left"])
        cr = csvref.read_columns(paths["right"])
        cores = os.cpu_count() or 1
        t = time.perf_counter()
        o = api.run_block(api.CTable(cl), api.CTable(cr), rules.plan_from_dir(paths["rules"]),
                          w.n_partitions, n_threads=cores)
        dt = time.perf_counter() - t
        sess.close()
    return {"workload": C2_DESC, "unit": UNIT, "pair_comparisons_per_step": int(st.pair_comparisons),
            "pairs_covered_per_step": int(st.pairs_covered), "matches_per_step": int(n),
            "batched": res["batched"], "plain": res["plain"],
            "batched_vs_plain": res["batched"]["value"] / res["plain"]["value"],
            "e2e": {"value": st_e2e.pair_comparisons / e2e_s, "ms_per_step": 1000.0 * e2e_s,
                    "h2d_bytes_per_step": int(st_e2e.h2d_bytes),
                    "d2h_bytes_per_step": int(8 * st_e2e.n_matches + 64)},
            "parity": {"rows": "all", "pairs": int(len(o.pairs)), "engine_pairs": int(len(got)),
                       "equal": bool(np.array_equal(got, o.pairs) and
                                     sorted_pairs(pairs).shape == o.pairs.shape and
                                     np.array_equal(sorted_pairs(pairs), o.pairs)),
                       "pair_comparisons_equal": int(o.pair_comparisons) == int(st.pair_comparisons)},
            "cpu_baseline": {"value": o.pair_comparisons / dt, "unit": UNIT, "cores": cores,
                             "kind": "port", "sample": f"every pair of the workload ({dt:.2f} s)"},
            "jw_fp64": fp64_block(o)}


def c1_fp64():
    """The oracle over C1 in full: the FP64 report of its JW evaluations."""
    from hyperblocker_gb300 import synth
    from oracle import api

    w = synth.c1()
    cl, cr = synth.table_bytes(w.tables.left), synth.table_bytes(w.tables.right)
    res = api.run_block(api.CTable(cl), api.CTable(cr), oracle_plan(w.rules), w.n_partitions)
    return fp64_block(res)


# ------------------------------------------------------------------ C5
def bench_c5(args, ctx, dev):
    """C5 shape at args.c5_rows x args.c5_rows: titles and authors of 64-256
    characters, a Zipf(1.0) key over 2^20 values, 3 rules, 64 partitions.
    The same job runs once through hbx_block (both tables encoded on the
    device at once) and once through hbx_block_streamed with partition windows
    of at most args.c5_window_mb MiB (two windows in flight); both are timed
    end to end (host tables to host pairs), must give the same pairs, and a
    stratified sample of left rows is checked against the oracle."""
    import numpy as np

    import hyperblocker_gb300 as hb
    from hyperblocker_gb300 import synth_big
    from oracle import api
    from tests._util import sorted_pairs

    n = args.c5_rows
    w = synth_big.c5(n, n, max(1, n // 50))
    plan = hb.Plan.from_yaml(w.rules, ctx)
    L = hb.Table.from_columns(w.left.cols, ctx)
    R = hb.Table.from_columns(w.right.cols, ctx)
    budget = args.c5_window_mb << 20
    hb.block(ctx, plan, L, R, w.n_partitions, hb.INT_MAX, "batched")  # warm: tuning, page-locking
    t = time.perf_counter()
    one, s1 = hb.block(ctx, plan, L, R, w.n_partitions, hb.INT_MAX, "batched")
    t_one = time.perf_counter() - t
    hb.block_streamed(ctx, plan, L, R, w.n_partitions, budget)  # warm
    t = time.perf_counter()
    st_pairs, s2 = hb.block_streamed(ctx, plan, L, R, w.n_partitions, budget)
    t_st = time.perf_counter() - t
    one, st_pairs = sorted_pairs(one), sorted_pairs(st_pairs)
    same = len(one) == len(st_pairs) and np.array_equal(one, st_pairs)
    plan_o = oracle_plan(w.rules)
    Lo, Ro = api.CTable(w.left.cols), api.CTable(w.right.cols)
    filt, n_rows = stratified_rows(Lo, plan_o, w.n_partitions, args.c5_sample_per_part, 11)
    o = api.run_block(Lo, Ro, plan_o, w.n_partitions, left_row_filter=filt)
    mine = one[filt[one[:, 0]] == 1] if len(one) else one
    return {"workload": f"c5 shape: {n:,} x {n:,} rows, titles and authors 64-256 characters, "
                        "Zipf(1.0) key over 2^20 values, 3 rules, 64 partitions",
            "unit": UNIT, "pair_comparisons": int(s1.pair_comparisons),
            "matches": int(s1.n_matches), "same_pairs": bool(same),
            "long_string_pairs": int(s1.long_string_pairs),
            "one_shot": {"value": s1.pair_comparisons / t_one, "wall_ms": 1000 * t_one,
                         "ms_eval": s1.ms_eval, "ms_create": s1.ms_create,
                         "tile_right": int(s1.tile_right), "eval_variant": int(s1.eval_variant)},
            "streamed": {"value": s2.pair_comparisons / t_st, "wall_ms": 1000 * t_st,
                         "windows": int(s2.n_windows), "window_mib": args.c5_window_mb,
                         "tile_right": int(s2.tile_right), "eval_variant": int(s2.eval_variant),
                         "ms_eval_summed": s2.ms_eval, "ms_create_summed": s2.ms_create},
            "streamed_vs_one_shot": t_st / t_one,
            "parity": {"sampled_left_rows": n_rows, "per_partition": args.c5_sample_per_part,
                       "pairs": int(len(o.pairs)), "engine_pairs": int(len(mine)),
                       "equal": bool(np.array_equal(mine, o.pairs)),
                       "streamed_equal_one_shot": bool(same)},
            "jw_fp64": fp64_block(o),
            "timing": "end to end, host tables to host pairs, host clock"}


# ------------------------------------------------------------------ serving (C4)
def bench_serving(args, ctx):
    """C4: a resident right table of args.serve_rows rows; args.serve_requests
    requests of log-uniform 1-50k left records arriving Poisson at
    args.serve_rate per second, each naming one of 4 rules.  Requests are
    submitted at their arrival times from this thread and their results
    polled; latency = submit -> result ready (host clock).  Afterwards the
    smallest requests' results are checked against the oracle over the whole
    resident table."""
    import numpy as np

    import hyperblocker_gb300 as hb
    from hyperblocker_gb300 import synth_big
    from oracle import api

    right = synth_big.c4_right(args.serve_rows)
    reqs = synth_big.c4_requests(right, args.serve_requests, rate=args.serve_rate, seed=1)
    plans = [hb.Plan.from_yaml([d], ctx) for d in synth_big.SERVE_RULES]
    R = hb.Table.from_columns(right.cols, ctx)
    t = time.perf_counter()
    srv = hb.Server(ctx, plans, R)
    t_open = time.perf_counter() - t
    # warm: the trace's largest request once per plan, so that the server's
    # page-locked staging and device buffers have grown before the trace
    big = max(range(len(reqs)), key=lambda i: reqs[i].n_rows)
    for k in range(len(plans)):
        srv.submit(1 << 40 | k, k, reqs[big].cols)
        srv.poll(-1)
    s0 = srv.stats()
    n = len(reqs)
    got, sent = {}, 0
    t0 = time.perf_counter()
    while len(got) < n:
        now = time.perf_counter() - t0
        while sent < n and reqs[sent].t_arrival <= now:
            srv.submit(sent, reqs[sent].rule, reqs[sent].cols)
            sent += 1
        r = srv.poll(0 if sent < n else 50)
        while r is not None:
            got[r["id"]] = r
            r = srv.poll(0)
        if sent < n:
            dt = reqs[sent].t_arrival - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(min(dt, 0.0005))
    wall = time.perf_counter() - t0
    s1 = srv.stats()
    srv.close()
    lat = np.array([got[i]["ms_total"] for i in range(n)])
    size = np.array([reqs[i].n_rows for i in range(n)])
    mid = lat[(size >= 5000) & (size <= 20000)]
    cmp = sum(got[i]["comparisons"] for i in range(n))
    bad = sum(1 for i in range(n) if got[i]["status"] != hb.OK)
    pct = lambda a, q: float(np.percentile(a, q)) if len(a) else None
    # parity: the smallest requests, half of them among those that matched
    # something, against the oracle over the whole resident table (one
    # partition)
    by_size = sorted(range(n), key=lambda i: (size[i], i))
    with_pairs = [i for i in by_size if len(got[i]["pairs"])]
    chk = with_pairs[:args.serve_check // 2]
    chk += [i for i in by_size if i not in chk][:args.serve_check - len(chk)]
    Ro = api.CTable(right.cols)
    checked, equal, pairs_total, covered = [], True, 0, 0
    for i in chk:
        o = api.run_block(api.CTable(reqs[i].cols), Ro,
                          oracle_plan([synth_big.SERVE_RULES[reqs[i].rule]]), 1)
        mine = got[i]["pairs"]
        mine = mine[np.lexsort((mine[:, 1], mine[:, 0]))] if len(mine) else mine.reshape(0, 2)
        ok = len(mine) == len(o.pairs) and np.array_equal(mine, o.pairs)
        equal = equal and ok
        pairs_total += len(o.pairs)
        covered += o.pairs_covered
        checked.append({"request": i, "records": int(size[i]), "rule": int(reqs[i].rule),
                        "pairs": int(len(o.pairs)), "equal": bool(ok)})
    return {"workload": f"c4: {args.serve_rows:,} resident right rows; {n} requests of "
                        "log-uniform 1-50,000 left records, Poisson arrivals at "
                        f"{args.serve_rate:g}/s, one of 4 rules (year and venue equalities, "
                        "1-2 JW predicates) each", "requests": n, "failed": bad,
            "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "p999_ms": pct(lat, 99.9),
            "max_ms": float(lat.max()),
            "p50_ms_5k_20k_rows": pct(mid, 50), "p99_ms_5k_20k_rows": pct(mid, 99),
            "requests_5k_20k_rows": int(len(mid)),
            "pair_comparisons_per_s": cmp / wall, "unit": UNIT,
            "records_per_s": float(size.sum()) / wall, "trace_s": float(reqs[-1].t_arrival),
            "wall_s": wall, "device_busy_frac": (s1.ms_device - s0.ms_device) / 1000.0 / wall,
            "batches": int(s1.batches - s0.batches),
            "mean_batch_requests": float(np.mean([got[i]["batch_requests"] for i in range(n)])),
            "open_s": t_open, "resident_bytes": int(s1.resident_bytes),
            "parity": {"requests_checked": len(checked), "pairs": pairs_total,
                       "pairs_covered": int(covered), "equal": bool(equal),
                       "against": f"the oracle over all {args.serve_rows + 1:,} resident rows",
                       "requests": checked},
            "latency": "submit -> result ready, host clock; requests submitted at their "
                       "arrival times",
            "warm": f"the largest request ({reqs[big].n_rows:,} records) once per plan before "
                    "the trace"}


# ------------------------------------------------------------------ io
def bench_io(args, ctx, dev):
    """Ingest and output around the path, timed end to end (wall clock of
    the C-ABI calls, best of args.io_reps):

    * csv: a quoted CSV file of args.io_rows rows (the C3 schema, about 175
      bytes a row) read into a table with a context (tokenized on the device,
      csv_gpu.cu) and without one (the host tokenizer); columns compared.
    * write: args.io_pairs (left row, right row) pairs of two tables of
      args.io_rows rows written as id_l,id_r lines from device pairs
      (hbx_write_pairs_device, lines formatted on the device) and from host
      pairs by the host loop (hbx_write_pairs without a context); files
      compared byte for byte."""
    import numpy as np
    import torch

    import hyperblocker_gb300 as hb
    from hyperblocker_gb300 import synth_big

    reps = max(1, args.io_reps)

    def best(fn):
        ts, r = [], None
        for _ in range(reps):
            t = time.perf_counter()
            r = fn()
            ts.append(time.perf_counter() - t)
        return min(ts), r

    out = {}
    with tempfile.TemporaryDirectory() as d:
        w = synth_big.c3(args.io_rows, 1_000)
        cols = w.left.cols
        n = len(cols[0][1]) - 1
        path = os.path.join(d, "l.csv")
        with open(path, "wb") as f:
            f.write(b"\n".join(b",".join(b'"' + bytes(b_[o[i]:o[i + 1]]) + b'"' for b_, o in cols)
                               for i in range(n)) + b"\n")
        del w, cols
        size = os.path.getsize(path)
        hb.Table.from_csv(path, ",", ctx)  # warm: page-in, pools
        t_dev, D = best(lambda: hb.Table.from_csv(path, ",", ctx))
        t_host, H = best(lambda: hb.Table.from_csv(path, ","))
        same = D.n_rows == H.n_rows and all(
            np.array_equal(H.column(c)[0], D.column(c)[0]) and
            np.array_equal(H.column(c)[1], D.column(c)[1]) for c in range(H.n_cols))
        out["csv"] = {"bytes": size, "rows": int(H.n_rows), "device_s": t_dev, "host_s": t_host,
                      "device_gbs": size / t_dev / 1e9, "host_gbs": size / t_host / 1e9,
                      "same_columns": bool(same)}
        del D, H
        os.remove(path)

        m, nr = args.io_pairs, args.io_rows
        ids = [b"id"] + [str(100_000_000 + i).encode() for i in range(nr)]
        L = hb.Table.from_columns([ids, [b"x"] * (nr + 1)], ctx)
        R = hb.Table.from_columns([ids, [b"x"] * (nr + 1)], ctx)
        rng = np.random.Generator(np.random.PCG64(7))
        pairs = np.stack([rng.integers(0, nr + 1, size=m), rng.integers(0, nr + 1, size=m)],
                         axis=1).astype(np.uint32)
        dl = torch.from_numpy(pairs[:, 0].astype(np.int32)).to(dev)
        dr = torch.from_numpy(pairs[:, 1].astype(np.int32)).to(dev)
        torch.cuda.synchronize(dev)
        hp, dp = os.path.join(d, "host.txt"), os.path.join(d, "dev.txt")

        def host_write():
            if os.path.exists(hp):
                os.remove(hp)
            hb.write_pairs(L, R, pairs, hp)

        def dev_write():
            if os.path.exists(dp):
                os.remove(dp)
            hb.write_pairs_device(ctx, L, R, dl.data_ptr(), dr.data_ptr(), m, dp)

        dev_write()  # warm
        t_dev, _ = best(dev_write)
        t_host, _ = best(host_write)
        size = os.path.getsize(hp)
        with open(hp, "rb") as fh, open(dp, "rb") as fd:
            same = fh.read() == fd.read()
        out["write"] = {"pairs": m, "text_bytes": size, "device_s": t_dev, "host_s": t_host,
                        "device_gbs": size / t_dev / 1e9, "host_gbs": size / t_host / 1e9,
                        "same_bytes": bool(same)}
        del dl, dr
    out["timing"] = f"wall clock of the calls, best of {reps}; files in a temporary directory"
    return out


def max_over_ranks(dist, values, device):
    """Element-wise maximum over the ranks of per-rank timings: the slowest
    replica sets the job's time (values unchanged without a process group)."""
    if dist is None:
        return [float(v) for v in values]
    import torch

    t = torch.tensor([float(v) for v in values], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


# ------------------------------------------------------------------ reference arm
def run_reference(args, rank, world):
    """The CPU implementation of the path (the oracle, all host cores) on
    stratified samples of C3: step k takes args.ref_per_part left rows of
    every partition (seed 1000 + k) against their partitions' right rows."""
    if rank != 0:
        return 0
    from hyperblocker_gb300 import synth_big
    from oracle import api

    api.build()
    n = args.c3_rows
    w = synth_big.c3(n, n, max(1, n // 50))
    plan_o = oracle_plan(w.rules)
    Lo, Ro = api.CTable(w.left.cols), api.CTable(w.right.cols)
    cores = os.cpu_count() or 1
    secs, cmps, covered, rows = 0.0, 0, 0, 0
    for k in range(args.warmup + args.steps):
        filt, n_rows = stratified_rows(Lo, plan_o, w.n_partitions, args.ref_per_part, 1000 + k)
        t = time.perf_counter()
        res = api.run_block(Lo, Ro, plan_o, w.n_partitions, n_threads=cores, left_row_filter=filt)
        dt = time.perf_counter() - t
        if k >= args.warmup:
            secs += dt
            cmps += res.pair_comparisons
            covered += res.pairs_covered
            rows += n_rows
    value = cmps / secs
    sample = (f"per step {args.ref_per_part} left rows of each of the 64 partitions (seed 1000 + "
              f"step) against their partitions' right rows; {args.steps} steps: {rows} left rows, "
              f"{covered} pairs covered, {cmps} pair-comparisons in {secs:.2f} s")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * secs / max(args.steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded PCG64, C3 shape; no dataset download)",
        "config": {"workload": c3_desc(n), "n_partitions": w.n_partitions, "rules": len(w.rules)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ engine arm
def run_engine(args, rank, world, local_rank):
    import torch

    import hyperblocker_gb300 as hb

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local_rank)
    ctx = hb.Context(local_rank)
    c3 = C3(args, ctx, dev)

    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local_rank)
    sampler.start()
    bat = c3.timed("batched", args.steps, args.warmup)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    if dist:
        dist.barrier()
    pla = c3.timed("plain", args.c3_plain_steps, 1)
    total_ms, plain_ms = max_over_ranks(dist, [sum(bat["ms"]), sum(pla["ms"])], dev)
    cmp_step = bat["cmp"][0]
    value = world * cmp_step * args.steps / (total_ms / 1000.0)
    plain_value = world * cmp_step * args.c3_plain_steps / (plain_ms / 1000.0)

    line = None
    if rank == 0:
        st = bat["stats"]  # the batched form's last timed step
        e2e = c3.e2e(ctx, args.e2e_steps)
        e2e["value"] *= world
        peaks = _peaks()
        peak = probe_scan_peak(local_rank, int(st.scan_words))
        ms_eval = statistics.mean(bat["ms_eval"])
        ops = statistics.mean(bat["ops"])
        scan_ops = statistics.mean(bat["scan_ops"])
        achieved_exec = scan_ops / (ms_eval / 1000.0) / 1e12
        achieved_alg = ops / (ms_eval / 1000.0) / 1e12
        traffic, traffic_src = _traffic_record()
        roofline = {
            "bound": "alu", "kernel": "k_eval (Jaro-Winkler pair evaluation)",
            "achieved": achieved_exec, "peak": peak["tops"],
            "unit": "Tops/s (scan operations: 6 per 64-bit mask word per character)",
            "frac": achieved_exec / peak["tops"] if peak["tops"] else None,
            "traffic": traffic, "traffic_source": traffic_src,
            "frac_executed": achieved_exec / peak["tops"] if peak["tops"] else None,
            "frac_algorithmic": achieved_alg / peak["tops"] if peak["tops"] else None,
            "achieved_algorithmic": achieved_alg,
            "peak_source": ("measured: libhbx_probe.so hbx_probe_scan_rate, the scan step of the "
                            "evaluation kernel with Peq rows in shared memory, "
                            f"{peak['words']} mask words, best of (independent chains per "
                            "thread x CTAs per SM) = "
                            f"{json.dumps(peak['per_chains_x_ctas_per_sm'])} Tops/s, this GPU, "
                            "this run"),
            "scan_word_ops_per_launch": scan_ops, "jw_word_ops_per_launch": ops,
            "ms_per_launch": ms_eval, "scan_words": int(st.scan_words),
            "pairs_scanned_per_launch": int(statistics.mean(bat["scanned"])),
            "pairs_scanned_per_launch_plain": int(statistics.mean(pla["scanned"])),
            "rest_scans_per_launch": int(statistics.mean(bat["rest"])),
            "rest_scans_per_launch_plain": int(statistics.mean(pla["rest"])),
            "scan_lane_utilisation": bat["lane_util"][-1],
            "scan_lane_utilisation_plain": pla["lane_util"][-1],
            "scan_word_ops_per_step_plain": statistics.mean(pla["scan_ops"]),
            "tile_right": int(st.tile_right), "eval_variant": int(st.eval_variant),
            "join_ms_per_step": statistics.mean([m - e for m, e in zip(bat["ms"], bat["ms_eval"])]),
            "hbm_gbs_measured": peaks.get("hbm_gbs"),
        }
        extra, cb, par, fp = {}, None, None, {}
        if world == 1:
            par, cb, fp["c3_sample"] = c3.parity(args, bat["matches"])
        c3.close()
        if world == 1:
            fp["c1"] = c1_fp64()
            if "c2" in args.sections:
                extra["c2"] = bench_c2(args, ctx, dev)
                fp["c2"] = extra["c2"].pop("jw_fp64")
            if "c5" in args.sections:
                extra["c5"] = bench_c5(args, ctx, dev)
                fp["c5_sample"] = extra["c5"].pop("jw_fp64")
            if "serve" in args.sections:
                extra["serving"] = bench_serving(args, ctx)
            if "io" in args.sections:
                extra["io"] = bench_io(args, ctx, dev)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded PCG64, C3 shape; no dataset download)",
            "config": {"workload": c3_desc(c3.n), "n_left_rows": c3.L.n_rows,
                       "n_right_rows": c3.R.n_rows, "rules": len(c3.w.rules),
                       "n_partitions": c3.w.n_partitions, "mode": "batched",
                       "pair_comparisons_per_step": cmp_step,
                       "pairs_covered_per_step": int(st.pairs_covered),
                       "matches_per_step": int(bat["matches"]),
                       "l2": "inputs larger than L2 (about 200 MB a side); L2 also flushed "
                             "before every timed step (256 MiB write, outside the events)",
                       "parallelism": f"replicas x{world}"},
            "plain": {"value": plain_value, "ms_per_step": plain_ms / args.c3_plain_steps,
                      "steps": args.c3_plain_steps,
                      "ms_eval": statistics.mean(pla["ms_eval"]),
                      "launches_per_step": pla["launches"] // max(args.c3_plain_steps, 1)},
            "batched_vs_plain": value / plain_value,
            "ms_eval_batched": ms_eval,
            "gpu_launches": bat["launches"],
            "clocks": {k: clocks[k] for k in ("sm_mhz", "sm_max_mhz", "reasons")},
            "e2e": e2e,
            "roofline": roofline,
        }
        if cb:
            line["cpu_baseline"] = cb
        if par:
            line["parity"] = par
        if fp:
            line["jw_fp64"] = {"workloads": fp,
                               "fp64_flips": sum(v["fp64_flips"] for v in fp.values()),
                               "max_abs_diff": max(v["max_abs_diff"] for v in fp.values()),
                               "set_unchanged": "the engine decides with the reference's "
                                                "float/double arithmetic; parity blocks compare "
                                                "its set with the oracle's"}
        line.update(extra)
        print(json.dumps(line), flush=True)
    else:
        c3.close()
    ctx.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--sections", default="c2,c5,serve",
                    help="extra measurements at N=1, comma separated: c2 (2,600 x 64,263 rows, "
                         "checked in full), c5 (long strings, one-shot vs streamed partition "
                         "windows), serve (resident-table serving trace), io (CSV tokenization "
                         "and pair-file writing, device vs host); '' for none")
    ap.add_argument("--c3-rows", type=int, default=1_000_000)
    ap.add_argument("--c3-plain-steps", type=int, default=2)
    ap.add_argument("--c3-sample-per-part", type=int, default=64)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--ref-per-part", type=int, default=16)
    ap.add_argument("--c2-steps", type=int, default=20)
    ap.add_argument("--c5-rows", type=int, default=500_000)
    ap.add_argument("--c5-window-mb", type=int, default=512)
    ap.add_argument("--c5-sample-per-part", type=int, default=16)
    ap.add_argument("--serve-rows", type=int, default=10_000_000)
    ap.add_argument("--serve-requests", type=int, default=800)
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-check", type=int, default=6)
    ap.add_argument("--io-rows", type=int, default=1_000_000)
    ap.add_argument("--io-pairs", type=int, default=20_000_000)
    ap.add_argument("--io-reps", type=int, default=3)
    args = ap.parse_args()
    args.sections = [x for x in args.sections.split(",") if x]
    if args.warmup < 3:
        args.warmup = 3
    rank = _env_int("RANK", 0)
    world = _env_int("WORLD_SIZE", args.gpus)
    local_rank = _env_int("LOCAL_RANK", 0)
    if "WORLD_SIZE" not in os.environ:
        world = 1 if args.gpus <= 1 else args.gpus
        if world > 1:
            print("bench.py: launch N>1 with torch.distributed.run", file=sys.stderr)
            return 2
    if args.impl == "reference":
        return run_reference(args, rank, world)
    import __graft_entry__

    __graft_entry__.build()
    return run_engine(args, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
