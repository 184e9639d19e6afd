#!/usr/bin/env python
"""Benchmark of the rule-based blocking hot path: pair-comparisons/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

Workload (default): the C2 configuration -- 2,600 x 64,263 seeded synthetic
bibliographic rows (header line included as data, as the reference reads it),
5k perturbed true pairs, two rules ((year eq, JW(title) >= 0.89,
JW(authors) >= 0.85) or (venue eq, JW(title) >= 0.95)), 8 hash partitions.
A step is one pass of the hot path over the whole workload: equality join,
Jaro-Winkler pair evaluation and compaction of the matching pairs.

* ``value``: pair-comparisons/s of the engine's default (batched: one
  persistent work-stealing launch replayed from a CUDA graph) with the inputs
  resident in HBM; L2 is flushed (256 MiB write) before every timed step and
  every step is timed with CUDA events on the launching stream.
* ``plain``: the same with one launch per (partition, rule), like the
  reference's per-partition submission.
* ``e2e``: the same metric through the one-shot C-ABI call ``hbx_block`` from
  host tables to host pair buffers (encode + H2D + run + D2H inside the timed
  region).
* ``roofline``: the pair-evaluation kernel against the INT32 issue peak (see
  the ``roofline`` block for the conventions), ``cpu_baseline``: the oracle
  (the reference's brute-force algorithm restated in C++) on all host cores.

At N=1 more workloads are measured and reported in the same line: ``c3``
(1M x 1M rows, 8 rules, 64 Zipf-sized partitions: batched vs plain), ``c5``
(long strings, one-shot vs partition windows streamed under a memory budget)
``serving`` (10M resident right rows, a Poisson trace of left-record
requests: p50/p99/p999 latency and pair-comparisons/s) and ``io`` (CSV
tokenization and pair-file writing, device vs host); ``--sections`` picks.

``--impl reference`` times that CPU implementation alone and prints the same
line with ``"impl": "reference"``.  With N > 1 GPUs (torchrun) every rank runs
an independent replica (weak scaling); the path needs no collective.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pair-comparisons/s, batched vs plain, same GPU, exact set; serving p50/p99 ms"
UNIT = "pair-comparisons/s"
WORKLOAD_DESC = ("c2: 2,600 x 64,263 synthetic bibliographic rows (+1 header row each), 5k true "
                 "pairs, rules (year eq, JW(title)>=0.89, JW(authors)>=0.85) | (venue eq, "
                 "JW(title)>=0.95), 8 partitions")


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
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def _traffic_per_launch():
    """dram bytes of one k_eval launch on this workload from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "k_eval_c2_traffic.json")
    try:
        with open(p) as f:
            return json.load(f).get("dram_bytes_per_launch")
    except Exception:
        return None


def load_workload(tmpdir: str):
    import hyperblocker_gb300 as hb
    from hyperblocker_gb300 import synth

    w = synth.c2()
    paths = synth.materialize(w, tmpdir)
    return w, paths


def cpu_baseline(paths, n_partitions, target_s=15.0, steps=1, warmup=0, step_fraction=None):
    """The oracle on all host cores over a bounded sample of left rows.

    Returns dict(value, cores, sample, seconds)."""
    import numpy as np

    from oracle import api, csvref, rules

    api.build()
    cl = csvref.read_columns(paths["left"])
    cr = csvref.read_columns(paths["right"])
    plan = rules.plan_from_dir(paths["rules"])
    L, R = api.CTable(cl), api.CTable(cr)
    n_l = len(cl[0])
    cores = os.cpu_count() or 1
    # size the sample: time a small probe, then scale to ~target_s of CPU work
    if step_fraction is None:
        probe = np.zeros(n_l, dtype=np.uint8)
        probe[::64] = 1
        t = time.perf_counter()
        api.run_block(L, R, plan, n_partitions, n_threads=cores, left_row_filter=probe)
        dt = max(time.perf_counter() - t, 1e-3)
        frac = min(1.0, (target_s / dt) / 64.0)
    else:
        frac = step_fraction
    stride = max(1, int(round(1.0 / frac)))
    vals, secs, cmps = [], [], []
    for k in range(warmup + steps):
        filt = np.zeros(n_l, dtype=np.uint8)
        filt[(k % stride)::stride] = 1
        t = time.perf_counter()
        res = api.run_block(L, R, plan, n_partitions, n_threads=cores, left_row_filter=filt)
        dt = time.perf_counter() - t
        if k >= warmup:
            vals.append(res.pair_comparisons / dt)
            secs.append(dt)
            cmps.append(res.pair_comparisons)
    return {"value": sum(cmps) / sum(secs), "cores": cores, "seconds": sum(secs),
            "sample": f"every {stride}th left row of the workload per step ({steps} step(s), "
                      f"{sum(cmps)} pair-comparisons in {sum(secs):.2f} s)"}


def bench_c3(args, ctx, dev):
    """C3: 1M x 1M rows, 8 rules, 64 Zipf-sized partitions; batched vs plain.

    One untimed batched step (it also runs the tile autotuner and sizes the
    output), then args.c3_steps timed steps of each form, CUDA events around
    each step on the launching stream; the inputs (about 200 MB a side) are
    larger than L2."""
    import torch

    import hyperblocker_gb300 as hb
    from hyperblocker_gb300 import synth_big

    n = args.c3_rows
    w = synth_big.c3(n, n, max(1, n // 50))
    plan = hb.Plan.from_yaml(w.rules, ctx)
    L = hb.Table.from_columns(w.left.cols, ctx)
    R = hb.Table.from_columns(w.right.cols, ctx)
    sess = hb.Session(ctx, plan, L, R, w.n_partitions)
    stream = torch.cuda.Stream(device=dev)
    m = sess.count("batched", stream.cuda_stream)
    cap = max(1, m)
    out_l = torch.empty(cap, dtype=torch.int32, device=dev)
    out_r = torch.empty(cap, dtype=torch.int32, device=dev)
    res = {}
    for mode in ("batched", "plain"):
        sess.run_device(mode, out_l.data_ptr(), out_r.data_ptr(), cap, stream.cuda_stream)  # warm
        ms, ms_eval, ops = [], [], []
        for _ in range(args.c3_steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                e0.record(stream)
                sess.run_device(mode, out_l.data_ptr(), out_r.data_ptr(), cap, stream.cuda_stream)
                e1.record(stream)
            e1.synchronize()
            st = sess.stats()
            ms.append(e0.elapsed_time(e1))
            ms_eval.append(st.ms_eval)
            ops.append(st.jw_word_ops)
        res[mode] = {"value": st.pair_comparisons / (statistics.mean(ms) / 1000.0),
                     "ms_per_step": statistics.mean(ms), "ms_eval": statistics.mean(ms_eval),
                     "launches_per_step": int(st.n_launches)}
    st = sess.stats()
    out = {"workload": f"c3: {n:,} x {n:,} synthetic rows (+1 header row each), 8 rules (1-2 "
                       "equalities, 1-3 JW predicates, thresholds U[0.80,0.95]), 64 partitions "
                       "keyed by a Zipf(1.3) column", "steps": args.c3_steps,
           "pair_comparisons_per_step": int(st.pair_comparisons),
           "pairs_covered_per_step": int(st.pairs_covered),
           "matches_per_step": int(m), "unit": UNIT,
           "batched": res["batched"], "plain": res["plain"],
           "batched_vs_plain": res["batched"]["value"] / res["plain"]["value"],
           "jw_word_ops_per_step": int(statistics.mean(ops)),
           "alu_tops_eval": statistics.mean(ops) / (res["batched"]["ms_eval"] / 1000.0) / 1e12}
    sess.close()
    return out


def bench_c5(args, ctx):
    """C5 shape at args.c5_rows x args.c5_rows: titles and authors of 64-256
    characters, a Zipf(1.0) key over 2^20 values, 3 rules, 64 partitions.
    The same job runs once through hbx_block (both tables encoded on the
    device at once) and once through hbx_block_streamed with partition windows
    of at most args.c5_window_mb MiB (two windows in flight, each window's
    copies and encoding overlapping the other's evaluation); both are timed
    end to end (host tables to host pairs) and must give the same pairs."""
    import numpy as np

    import hyperblocker_gb300 as hb
    from hyperblocker_gb300 import synth_big

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
    same = len(one) == len(st_pairs) and np.array_equal(
        one[np.lexsort((one[:, 1], one[:, 0]))], st_pairs[np.lexsort((st_pairs[:, 1], st_pairs[:, 0]))])
    return {"workload": f"c5 shape: {n:,} x {n:,} rows, titles and authors 64-256 characters, "
                        "Zipf(1.0) key over 2^20 values, 3 rules, 64 partitions",
            "unit": UNIT, "pair_comparisons": int(s1.pair_comparisons),
            "matches": int(s1.n_matches), "same_pairs": bool(same),
            "long_string_pairs": int(s1.long_string_pairs),
            "one_shot": {"value": s1.pair_comparisons / t_one, "wall_ms": 1000 * t_one,
                         "ms_eval": s1.ms_eval},
            "streamed": {"value": s2.pair_comparisons / t_st, "wall_ms": 1000 * t_st,
                         "windows": int(s2.n_windows), "window_mib": args.c5_window_mb,
                         "ms_eval_summed": s2.ms_eval, "ms_create_summed": s2.ms_create},
            "timing": "end to end, host tables to host pairs, host clock"}


def bench_serving(args, ctx):
    """C4: a resident right table of args.serve_rows rows; args.serve_requests
    requests of log-uniform 1-50k left records arriving Poisson at
    args.serve_rate per second, each naming one of 4 rules.  Requests are
    submitted at their arrival times from this thread and their results
    polled; latency = submit -> result ready (host clock)."""
    import numpy as np

    import hyperblocker_gb300 as hb
    from hyperblocker_gb300 import synth_big

    right = synth_big.c4_right(args.serve_rows)
    reqs = synth_big.c4_requests(right, args.serve_requests, rate=args.serve_rate, seed=1)
    plans = [hb.Plan.from_yaml([d], ctx) for d in synth_big.SERVE_RULES]
    R = hb.Table.from_columns(right.cols, ctx)
    del right
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
            "latency": "submit -> result ready, host clock; requests submitted at their "
                       "arrival times",
            "warm": f"the largest request ({reqs[big].n_rows:,} records) once per plan before "
                    "the trace"}


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


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    with tempfile.TemporaryDirectory() as d:
        w, paths = load_workload(d)
        # each step: 1/8 of the left rows, brute force over their partitions
        cb = cpu_baseline(paths, w.n_partitions, steps=args.steps, warmup=args.warmup,
                          step_fraction=1.0 / 8.0)
    line = {
        "impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * cb["seconds"] / max(args.steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic (seeded, C2 shape)",
        "config": {"workload": WORKLOAD_DESC, "n_partitions": w.n_partitions, "rules": 2},
        "cpu_baseline": {"value": cb["value"], "unit": UNIT, "cores": cb["cores"], "kind": "port",
                         "sample": cb["sample"]},
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_engine(args, rank, world, local_rank):
    import numpy as np
    import torch

    import hyperblocker_gb300 as hb

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local_rank)
    tmp = tempfile.TemporaryDirectory()
    w, paths = load_workload(tmp.name)
    ctx = hb.Context(local_rank)
    plan = hb.Plan.from_rule_dir(paths["rules"], ctx)
    L = hb.Table.from_csv(paths["left"], ",", ctx)
    R = hb.Table.from_csv(paths["right"], ",", ctx)
    sess = hb.Session(ctx, plan, L, R, w.n_partitions)
    stream = torch.cuda.Stream(device=dev)
    cap = 1 << 20
    out_l = torch.empty(cap, dtype=torch.int32, device=dev)
    out_r = torch.empty(cap, dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step(mode):
        return sess.run_device(mode, out_l.data_ptr(), out_r.data_ptr(), cap, stream.cuda_stream)

    def timed(mode, k, w_):
        for _ in range(w_):
            step(mode)
        ms, ms_eval, ops, cmp, launches = [], [], [], [], 0
        with torch.cuda.stream(stream):
            for _ in range(k):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                n = step(mode)
                e1.record(stream)
                e1.synchronize()
                ms.append(e0.elapsed_time(e1))
                st = sess.stats()
                ms_eval.append(st.ms_eval)
                ops.append(st.jw_word_ops)
                cmp.append(st.pair_comparisons)
                launches += st.n_launches
        return {"ms": ms, "ms_eval": ms_eval, "ops": ops, "cmp": cmp, "launches": launches,
                "matches": n}

    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local_rank)
    sampler.start()
    t_wall = time.perf_counter()
    bat = timed("batched", args.steps, args.warmup)
    torch.cuda.synchronize()
    wall_batched = time.perf_counter() - t_wall
    clocks = sampler.stop()
    pla = timed("plain", args.steps, args.warmup)
    total_ms, plain_ms = max_over_ranks(dist, [sum(bat["ms"]), sum(pla["ms"])], dev)
    cmp_step = bat["cmp"][0]
    value = world * cmp_step * args.steps / (total_ms / 1000.0)
    plain_value = world * cmp_step * args.steps / (plain_ms / 1000.0)

    # end to end through the one-shot C-ABI call (host tables -> host pairs)
    e2e_steps = max(1, min(args.steps, 5))
    hb.block(ctx, plan, L, R, w.n_partitions, hb.INT_MAX, "batched")  # warm
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        pairs, st_e2e = hb.block(ctx, plan, L, R, w.n_partitions, hb.INT_MAX, "batched")
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e = {"value": world * st_e2e.pair_comparisons / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(st_e2e.h2d_bytes),
           "d2h_bytes_per_step": int(8 * st_e2e.n_matches + 64),
           "ms_per_step": 1000.0 * e2e_s,
           "ms_create": float(st_e2e.ms_create),
           "ingest_on_device": int(st_e2e.ingest_on_device),
           "includes": "session creation (H2D of the plan's columns from the page-locked "
                       "host tables, device encode: std::hash partition buckets, "
                       "dictionaries, symbol arenas) + join + evaluation + D2H of the pairs "
                       "into host memory; the warm-up call page-locks the tables and "
                       "memoises the measured predicate order on the plan"}

    line = None
    if rank == 0:
        peaks = _peaks()
        props = torch.cuda.get_device_properties(dev)
        n_sm = props.multi_processor_count
        sm_max = float(peaks.get("sm_max_mhz") or clocks.get("sm_max_mhz") or 2070.0)
        # 1 algorithmic op = one 64-bit word operation = 2 INT32 issue slots;
        # an SM issues 128 INT32 lane-ops per cycle.
        peak_tops = n_sm * 64 * sm_max * 1e6 / 1e12
        ms_eval = statistics.mean(bat["ms_eval"])
        ops = statistics.mean(bat["ops"])
        achieved = ops / (ms_eval / 1000.0) / 1e12
        roofline = {
            "bound": "alu", "kernel": "k_eval (Jaro-Winkler pair evaluation)",
            "achieved": achieved, "peak": peak_tops, "unit": "Tops/s (64-bit word ops)",
            "frac": achieved / peak_tops,
            "traffic": _traffic_per_launch(),
            "ops_per_launch": ops, "ms_per_launch": ms_eval,
            "pairs_scanned_per_launch": int(sess.stats().pairs_scanned),
            "scan_steps_per_launch": int(sess.stats().scan_steps),
            "tile_right": int(sess.stats().tile_right),
            "eval_variant": int(sess.stats().eval_variant),
            "peak_source": f"nominal: {n_sm} SMs x 128 INT32 lanes / 2 per 64-bit op x "
                           f"{sm_max:.0f} MHz (sm_max_mhz of MEASURED_PEAKS.json); "
                           "MEASURED_PEAKS.json has no integer-pipe figure",
            "join_ms_per_step": statistics.mean([m - e for m, e in zip(bat["ms"], bat["ms_eval"])]),
        }
        cb = None
        if world == 1 and not args.no_cpu_baseline:
            cb = cpu_baseline(paths, w.n_partitions)
        extra = {}
        if world == 1 and "c3" in args.sections:
            extra["c3"] = bench_c3(args, ctx, dev)
        if world == 1 and "c5" in args.sections:
            extra["c5"] = bench_c5(args, ctx)
        if world == 1 and "serve" in args.sections:
            extra["serving"] = bench_serving(args, ctx)
        if world == 1 and "io" in args.sections:
            extra["io"] = bench_io(args, ctx, dev)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded PCG64, C2 shape; no dataset download)",
            "config": {"workload": WORKLOAD_DESC, "n_left_rows": L.n_rows, "n_right_rows": R.n_rows,
                       "rules": 2, "n_partitions": w.n_partitions, "mode": "batched",
                       "pair_comparisons_per_step": cmp_step,
                       "pairs_covered_per_step": int(sess.stats().pairs_covered),
                       "matches_per_step": int(bat["matches"]),
                       "l2": "flushed before every timed step (256 MiB write, outside the events)",
                       "parallelism": f"replicas x{world}"},
            "plain": {"value": plain_value, "ms_per_step": plain_ms / args.steps,
                      "launches_per_step": pla["launches"] // max(args.steps, 1)},
            "batched_vs_plain": value / plain_value,
            "gpu_launches": bat["launches"],
            "clocks": {k: clocks[k] for k in ("sm_mhz", "sm_max_mhz", "reasons")},
            "wall_s_batched": wall_batched,
            "e2e": e2e,
            "roofline": roofline,
        }
        if cb:
            line["cpu_baseline"] = {"value": cb["value"], "unit": UNIT, "cores": cb["cores"],
                                    "kind": "port", "sample": cb["sample"]}
        line.update(extra)
        print(json.dumps(line), flush=True)
    sess.close()
    ctx.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sections", default="c3,serve",
                    help="extra measurements at N=1, comma separated: c3 (1M x 1M batching "
                         "workload), serve (resident-table serving trace), c5 (long strings, "
                         "one-shot vs streamed partition windows; minutes), io (CSV "
                         "tokenization and pair-file writing, device vs host); '' for none")
    ap.add_argument("--c3-rows", type=int, default=1_000_000)
    ap.add_argument("--c3-steps", type=int, default=2)
    ap.add_argument("--c5-rows", type=int, default=500_000)
    ap.add_argument("--c5-window-mb", type=int, default=512)
    ap.add_argument("--serve-rows", type=int, default=10_000_000)
    ap.add_argument("--serve-requests", type=int, default=800)
    ap.add_argument("--serve-rate", type=float, default=200.0)
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
