"""Benchmark of the GB300 alignment stage (one JSON line on rank 0).

Workload (default, config 3): 100,000 uneven pairs in one batch -- query lengths log-normal
(median 1,200, sigma 0.8) clipped to 200..20,000, 5-12% ONT-like errors -- each pair a Myers
Infix distance against the target with 50-base flanks and a banded affine Global pass with
traceback (band clamp(32 * ceil(0.1 * L / 32), 64, 512), Affine{2,4,4,2}, score + CIGAR).
`--config c1` (10,000 Myers pairs of 1 kb), `--config c2` (20,000 banded affine pairs of
2 kb with CIGARs) and `--config c5` (the served stream) run the other workloads.

  value   GCUPS of the batched, persistent, graph-captured plan on inputs resident in HBM
          (CUDA events on the plan's stream; L2 flushed between steps).  `split` gives the
          Myers and the affine kernels' cells, GCUPS and share of the step apart.
  e2e     the same GCUPS through the C ABI call a user makes (sf_batch_run): job
          descriptors and byte-code pool from pinned host memory to the device, execute,
          results and CIGARs back to the host, every step.
  plain   GCUPS of the one-launch-per-pair form (one C-ABI call per pair) on a sample; for
          config 3 both on its own pairs and on config 2's (the form config 3 is compared with).
  parity  outside the timed region: the timed plan's distances and scores against the
          oracle on the pairs the CPU baseline computed, and every CIGAR re-scored; the run
          exits non-zero on a mismatch.
  cpu_baseline  the CPU restatement of the reference's path (scalar rows, NEON rows on
          aarch64) on all host cores, on a bounded sample.
  sub     with config 3: config 2 measured the same way, and a short served stream
          (config 5) with its latency percentiles.

`--impl reference` times that CPU path alone as the reference arm.
GCUPS counts band cells as the reference's DP_WORK does (align.rs:2573-2578) and m*n for
Myers (every block of every column, k = u32::MAX).
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GOLD = {"c1": "myers-infix-10k", "c2": "affine-global-band128-cigar-20k",
        "c5": "serving-poisson-2000rps-bursts5x",
        "c2-score": "affine-global-band128-score-20k",
        "c3": "uneven-myers+affine-100k"}
# Variants of a workload (--variant): the windowed read-end extension the mapper runs on the
# config-2 pairs (align.rs:957-982; window x + 20 + x / 10, X-drop 50, end bonus 5,
# map/src/lib.rs:2101, 235-239), and config 1 with each pair capped at its distance + 16.
VARIANTS = {("c2", "window"): "affine-extend-window-band128-xdrop50",
            ("c1", "kslack"): "myers-infix-10k-cap-d+16",
            ("c1", "kdecoy"): "myers-global-10k-decoys-cap160"}
DECOY_K = 160  # 16% of the 1 kb queries: the unrelated texts' distances are ~3x that
WINDOW = (20, 10, 50, 5)  # pad, pad_div, xdrop, end bonus
K_SLACK = 16
NONE32 = 0xFFFFFFFF
# What the kernels compute in: affine passes in packed 16-bit fields rebased every 64 rows
# where `fits16` admits them (results equal the 32-bit rows'), 32-bit rows otherwise; Myers
# in 64-bit bit vectors.
DTYPE = {"c1": "u64 bit vectors (Myers)",
         "c2": "int16x2 rebased (exact); int32 fallback",
         "c3": "int16x2 rebased (exact); int32 fallback (affine); u64 bit vectors (Myers)",
         "c5": "int16x2 rebased (exact); int32 fallback (affine); u64 bit vectors (Myers)"}


def workload_name(cfg, variant="base", cigar=True) -> str:
    if variant != "base":
        name = VARIANTS[(cfg, variant)]
        return name + ("-cigar" if cfg == "c2" and cigar else "")
    return GOLD[cfg if cigar or cfg != "c2" else "c2-score"]


OPS_PER_CELL = {"affine_tb": 12, "affine": 10, "myers": 0.625}
# sf_int_peak counts 3 int32 ops per chain step; ncu counts 2.094 instructions per step (an
# IMAD on the FMA pipe and a fused add-max on the ALU pipe, the loop included; one capture of
# the probe kernel alone), so its rate in instructions is Tops x 2.094 / 3.
INT_PEAK_INSTR_PER_STEP = 2.094


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist


def max_over_ranks(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for k, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(k)
            except (ValueError, IndexError):
                continue
        busy = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(busy) if busy else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_jobs(B, pairs, kind, mode, want_cigar, band=None):
    jobs = B.new_jobs(len(pairs))
    jobs["p_off"] = pairs.p_off
    jobs["t_off"] = pairs.t_off
    jobs["m"] = pairs.m
    jobs["n"] = pairs.n
    jobs["kind"] = kind
    jobs["mode"] = mode
    jobs["want_cigar"] = 1 if want_cigar else 0
    if kind != B.JOB_MYERS:
        jobs["band"] = pairs.band if band is None else band
    return jobs


def workload(cfg: str, scale: float, cigar: bool = True, variant: str = "base"):
    """(pool, jobs, pairs, kind) of a workload; for config 3 `pairs` is (Myers pairs, affine
    pairs) and the jobs are the Myers jobs followed by the affine jobs of the same queries."""
    from spearfish_gb300 import batch as B
    from spearfish_gb300 import workloads as W
    if cfg == "c1":
        w = W.config1(int(10_000 * scale))
        if variant == "kdecoy":
            # The tie-break's rejected candidates: Global distances capped at DECOY_K against
            # unrelated texts (a capped pair stops once a column is wholly past its cap).
            w = W.decoys(w)
            jobs = make_jobs(B, w, B.JOB_MYERS, 2, False)
            jobs["k"] = DECOY_K
            return w.pool, jobs, [w], "myers"
        return w.pool, make_jobs(B, w, B.JOB_MYERS, 0, False), [w], "myers"
    if cfg == "c2":
        w = W.config2(int(20_000 * scale))
        if variant == "window":
            pad, div, xdrop, bonus = WINDOW
            jobs = make_jobs(B, w, B.JOB_EXTEND_WINDOW, 1, cigar)
            jobs["window"] = jobs["m"].astype(np.uint64) + pad + jobs["m"] // div
            jobs["xdrop"] = xdrop
            jobs["end_bonus"] = bonus
            return w.pool, jobs, [w], "affine_tb" if cigar else "affine"
        return w.pool, make_jobs(B, w, B.JOB_AFFINE, 2, cigar), [w], "affine_tb" if cigar else "affine"
    my, af = W.config3(int(100_000 * scale))
    # One pool: the affine pairs' offsets shift past the Myers pool.
    shift = np.uint64(my.pool.size)
    pool = np.concatenate([my.pool, af.pool])
    jm = make_jobs(B, my, B.JOB_MYERS, 0, False)
    ja = make_jobs(B, af, B.JOB_AFFINE, 2, cigar)
    ja["p_off"] += shift
    ja["t_off"] += shift
    return pool, np.concatenate([jm, ja]), [my, af], "mixed"


def cpu_baseline(cfg, pairs_list, seconds: float, threads: int, variant: str = "base",
                 caps=None):
    """The reference's path restated in C (oracle), all host cores, bounded sample.  caps:
    per-pair Myers caps (the kslack variant).  Besides the rate, returns what it computed
    (`checked`: the sampled pair indices and each one's distance and/or score), which the
    GPU arm compares with its own results."""
    import oracle as O
    level = O.set_level(1)  # NEON rows where the host has them (the reference's level there)
    w = pairs_list[-1]
    kind = 0 if cfg == "c1" else (2 if variant == "window" else 1)
    mode = (2 if variant == "kdecoy" else 0) if cfg == "c1" else (1 if variant == "window" else 2)
    if variant == "kdecoy":
        caps = np.full(len(pairs_list[-1]), DECOY_K, np.uint32)
    total_cells, total_t, done = 0, 0.0, 0
    idx = np.arange(len(w))
    rng = np.random.default_rng(7)
    rng.shuffle(idx)
    chunk = max(threads * 8, 64)
    got_my, got_af = [], []
    while total_t < seconds and done < len(w):
        sel = idx[done:done + chunk]
        sub = w.subset(sel)
        t0 = time.perf_counter()
        if cfg == "c3":
            # per pair: Myers on the flanked target and affine with its own band
            my = pairs_list[0].subset(sel)
            d, c1 = O.run_pairs(0, threads, my.pool, my.p_off, my.m, my.pool, my.t_off, my.n, 0)
            s, c2 = O.run_pairs(1, threads, sub.pool, sub.p_off, sub.m, sub.pool, sub.t_off,
                                sub.n, 2, sc=O.ONT, bands=sub.band)
            cells = c1 + c2
            got_my.append(d)
            got_af.append(s)
        else:
            r, cells = O.run_pairs(kind, threads, sub.pool, sub.p_off, sub.m, sub.pool, sub.t_off,
                                   sub.n, mode, sc=O.ONT,
                                   bands=None if cfg == "c1" else sub.band,
                                   kv=None if caps is None else caps[sel],
                                   extend=WINDOW if variant == "window" else None)
            (got_my if cfg == "c1" else got_af).append(r)
        total_t += time.perf_counter() - t0
        total_cells += cells
        done += len(sel)
        chunk *= 2
    checked = {"idx": idx[:done],
               "myers": np.concatenate(got_my) if got_my else None,
               "affine": np.concatenate(got_af) if got_af else None}
    return {"value": total_cells / total_t / 1e9, "unit": "GCUPS", "cores": threads,
            "kind": "port", "level": "neon" if level == 1 else "scalar",
            "sample": f"{done} of {len(w)} pairs ({total_cells / 1e9:.2f} Gcells, "
                      f"{total_t:.1f} s wall on {threads} threads, score only: the reference "
                      f"computes no traceback)",
            "wall_s": total_t, "arch": platform.machine()}, checked


def kslack_caps(w, threads: int) -> np.ndarray:
    """Per-pair caps of the kslack variant: each pair's distance + 16 (the oracle's
    uncapped distances; the GPU's are the same, as the parity tests check)."""
    import oracle as O
    d, _ = O.run_pairs(0, threads, w.pool, w.p_off, w.m, w.pool, w.t_off, w.n, 0)
    return (d.astype(np.int64) + K_SLACK).astype(np.uint32)


def run_reference(args, ws, rank):
    """Reference arm: the CPU restatement on all host threads, rank 0 only."""
    if rank != 0:
        return
    import oracle as O
    _, jobs, pairs_list, _ = workload(args.config, args.scale, True, args.variant)
    threads = O.host_threads()
    caps = kslack_caps(pairs_list[-1], threads) if args.variant == "kslack" else None
    per_step = []
    for s in range(args.warmup + args.steps):
        r, _ = cpu_baseline(args.config, pairs_list, args.ref_seconds, threads, args.variant, caps)
        if s >= args.warmup:
            per_step.append(r)
    v = statistics.mean(r["value"] for r in per_step)
    # A step is one bounded sample of the workload (about ref_seconds of work).
    ms = 1e3 * statistics.mean(r["wall_s"] for r in per_step)
    line = {"metric": "alignment GCUPS", "value": v, "unit": "GCUPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32 (score only)",
            "data": "synthetic",
            "impl": "reference",
            "config": {"workload": workload_name(args.config, args.variant, bool(args.cigar)),
                       "parallelism": "host threads",
                       "step": "a bounded sample of the workload's pairs"},
            "cpu_baseline": {"value": v, "unit": "GCUPS", "cores": threads, "kind": "port",
                             "sample": per_step[-1]["sample"], "level": per_step[-1]["level"]},
            "e2e": {"value": v, "unit": "GCUPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def pct(xs, q):
    return float(np.percentile(np.asarray(xs), q)) if xs else None


def serve_measure(seconds: float, slots: int, use_store: bool, rank: int, local: int):
    """Config 5: a bursty Poisson stream of read batches (mean 2,000 reads/s, bursts 5x,
    1..4,096 reads a batch) fed in real time through the serving loop, then the same batches
    all at once (saturation).  Returns (live, saturation, server counters, batches)."""
    import threading

    from spearfish_gb300 import batch as B
    from spearfish_gb300 import serve as S
    from spearfish_gb300 import workloads as W

    stream = W.serving_stream(seconds, seed=5 + rank)
    rng = np.random.default_rng(505 + rank)
    batches = []
    store = ctx = tx = None
    if use_store:
        # The transcripts live in HBM for the whole stream; requests carry reads only.
        tx = W.Transcriptome()
        ctx = B.Context(local)
        store = B.Store(ctx, tx.txs)
    for _, size in stream:
        if store is not None:
            reads = [W.serving_store_read(tx, rng, hifi=rng.random() < 0.1) for _ in range(size)]
            batches.append(W.serving_store_jobs(tx, reads, B))
        else:
            reads = [W.serving_read(rng, hifi=rng.random() < 0.1) for _ in range(size)]
            batches.append(W.serving_jobs(reads, B))
    srv = S.Server(local, slots=slots, store=store)
    try:
        for pool, jobs in batches[:3]:  # warm-up: buffers grow to a working size
            srv.wait(srv.submit(pool, jobs))
        # Real time: each batch is submitted at its arrival time.
        tickets = [None] * len(batches)
        late = [0.0] * len(batches)
        t0 = time.perf_counter()

        def feeder():
            for q, ((at, _), (pool, jobs)) in enumerate(zip(stream, batches)):
                d = at - (time.perf_counter() - t0)
                if d > 0:
                    time.sleep(d)
                late[q] = max(0.0, (time.perf_counter() - t0) - at)
                tickets[q] = srv.submit(pool, jobs)

        th = threading.Thread(target=feeder)
        th.start()
        lat, qlat, rlat, cells, t_last = [], [], [], 0, t0
        for q in range(len(batches)):
            while tickets[q] is None:
                time.sleep(0.0002)
            out, st = srv.wait(tickets[q])
            lat.append(st.total_ms)
            qlat.append(st.queue_ms)
            rlat.append(st.run_ms)
            cells += st.cells
            t_last = time.perf_counter()
        th.join()
        reads = sum(n for _, n in stream)
        span = stream[-1][0] if stream else seconds  # first arrival at ~0, last at span
        wall = t_last - t0
        live = {"p50_ms": pct(lat, 50), "p95_ms": pct(lat, 95), "p99_ms": pct(lat, 99),
                "max_ms": max(lat), "batches": len(batches), "reads": reads,
                "stream_s": seconds, "arrival_span_s": span,
                "offered_reads_per_s": reads / span if span > 0 else None,
                "served_reads_per_s": reads / wall,
                "submit_late_ms_max": 1e3 * max(late),
                "queue_p99_ms": pct(qlat, 99), "run_p50_ms": pct(rlat, 50),
                "run_p99_ms": pct(rlat, 99),
                "sustained_gcups": cells / wall / 1e9, "wall_s": wall,
                "latency": "submit to results on the host (sf_server_submit .. sf_server_wait)"}
        # Saturation: every batch submitted at once.
        t1 = time.perf_counter()
        tks = [srv.submit(p, j) for p, j in batches]
        lat2, cells2 = [], 0
        for t in tks:
            _, st = srv.wait(t)
            lat2.append(st.total_ms)
            cells2 += st.cells
        wall2 = time.perf_counter() - t1
        sat = {"p50_ms": pct(lat2, 50), "p99_ms": pct(lat2, 99), "gcups": cells2 / wall2 / 1e9,
               "wall_s": wall2, "reads_per_s": reads / wall2}
        q = srv.query()
    finally:
        srv.close()
        if store is not None:
            store.close()
            ctx.close()
    return live, sat, {k: int(v) for k, v in q.items()}, batches


def run_serving(args, ws, rank, local):
    """Config 5 as the headline line."""
    from spearfish_gb300 import build
    build.build()
    live, sat, server, batches = serve_measure(args.serve_seconds, args.slots, bool(args.store),
                                               rank, local)
    if rank == 0:
        line = {"metric": "alignment GCUPS", "value": sat["gcups"], "unit": "GCUPS",
                "n_gpus": ws, "steps": 1, "warmup": 3, "ms_per_step": sat["wall_s"] * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": DTYPE["c5"], "data": "synthetic (seeded read model; sim.rs error model)",
                "config": {"workload": GOLD["c5"], "serve_seconds": args.serve_seconds,
                           "slots": args.slots, "jobs_per_read": 4,
                           "texts": "transcript store (HBM), windows sliced on the device"
                           if args.store else "in each request's pool",
                           "parallelism": f"replicas x{ws}"},
                "latency": live, "saturation": sat, "server": server,
                "e2e": {"value": sat["gcups"], "unit": "GCUPS",
                        "h2d_bytes_per_step": int(sum(p.size + j.nbytes for p, j in batches)),
                        "d2h_bytes_per_step": int(sum(len(j) * 64 for _, j in batches)),
                        "call": "sf_server_submit / sf_server_wait (C ABI)"}}
        print(json.dumps(line))


def bucket_name(b: dict, lanes: bool = False) -> str:
    s = f"{b['kind']}-c{b['c']}{'-wide' if b['wide'] else ''}{'-tb' if b['traceback'] else ''}"
    return s + (f"-x{b['lanes']}" if lanes and b["lanes"] != 32 else "")


def plain_rate(cfg, pairs_list, n, variant="base", cigar=True):
    """The one-launch-per-pair form: one C-ABI call per pair (two for a config-3 pair: its
    Myers distance and its affine pass) on the first n pairs."""
    from spearfish_gb300 import align as A
    w = pairs_list[-1]
    n = min(n, len(w))
    c0, _ = A.dp_work()
    my_cells = 0
    t0 = time.perf_counter()
    for q in range(n):
        if cfg in ("c1", "c3"):
            my = pairs_list[0]
            if variant == "kdecoy":
                A.distance(my.pattern(q), my.text(q), A.Mode.Global, DECOY_K)
            else:
                A.distance(my.pattern(q), my.text(q), A.Mode.Infix)
            my_cells += int(my.m[q]) * int(my.n[q])
            if cfg == "c1":
                continue
        if variant == "window":
            win = int(w.m[q]) + WINDOW[0] + int(w.m[q]) // WINDOW[1]
            f = A.affine_extend_window_cigar if cigar else A.affine_extend_window
            f(w.pattern(q), w.text(q), win, A.Affine.ONT, int(w.band[q]), WINDOW[3], WINDOW[2])
        elif not cigar:
            A.affine(w.pattern(q), w.text(q), A.Mode.Global, A.Affine.ONT, int(w.band[q]))
        else:
            A.affine_cigar(w.pattern(q), w.text(q), A.Mode.Global, A.Affine.ONT, int(w.band[q]))
    dt = time.perf_counter() - t0
    c1, _ = A.dp_work()
    cells = (c1 - c0) + my_cells
    call = {"c1": "sf_distance", "c3": "sf_distance + sf_affine_cigar"}.get(
        cfg, ("sf_affine_extend_window" if variant == "window" else "sf_affine") +
        ("_cigar" if cigar else ""))
    return {"value": cells / dt / 1e9, "unit": "GCUPS", "pairs": n, "workload": workload_name(
        cfg, variant, cigar), "call": call, "ms_per_pair": dt / n * 1e3}


def parity_check(cfg, pairs_list, res, ops, checked, threads) -> dict:
    """The timed plan's results against the oracle (outside the timed region): distances
    and scores of the pairs the CPU baseline computed, and every CIGAR re-scored (it must
    consume the pattern, end at the reported cell and score the reported score)."""
    import oracle as O
    idx = checked["idx"]
    n_my = len(pairs_list[0]) if cfg == "c3" else 0
    bad = 0
    if checked["myers"] is not None:
        got = res["distance"][idx].astype(np.int64)
        got[got == NONE32] = -1  # None on both sides
        bad += int((got != checked["myers"]).sum())
    if checked["affine"] is not None:
        bad += int((res["score"][n_my + idx].astype(np.int64) != checked["affine"]).sum())
    out = {"against": "oracle (C restatement of align.rs)", "pairs_checked": int(len(idx)),
           "mismatches": bad}
    if cfg in ("c2", "c3"):  # Global passes: the path's own score is the pair's score
        w = pairs_list[-1]
        r = res[n_my:]
        want = r["n_ops"] > 0
        if want.any():
            code = O.check_cigars(threads, w.pool, w.p_off, w.m, w.pool, w.t_off, w.n, ops,
                                  r["cigar_off"], r["n_ops"], r["text_start"], r["text_end"],
                                  r["score"], O.ONT)
            out["cigars_rescored"] = int(want.sum())
            out["cigar_failures"] = int((code[want] != 0).sum())
    return out


def measure_batch(args, cfg, variant, cigar, steps, warmup, dist, ws, rank, local, lib,
                  with_cpu, plain_pairs, e2e_steps):
    """One workload as a batched plan: device-timed steps, per-kernel split, roofline of the
    top kernel, e2e through sf_batch_run, parity against the oracle, CPU baseline, plain."""
    import ctypes as C

    import torch
    from spearfish_gb300 import _abi
    from spearfish_gb300 import batch as B

    pool, jobs, pairs_list, kind = workload(cfg, args.scale, cigar, variant)
    ctx = B.Context(local)
    caps = None
    if variant == "kslack":
        # Untimed: each pair's distance from an uncapped run, then the cap d + 16.
        pre = B.Plan(ctx, jobs, pool.size)
        pre.upload(pool)
        pre.execute()
        pre.sync()
        d = pre.download().results["distance"].astype(np.int64)
        pre.close()
        caps = (d + K_SLACK).astype(np.uint32)
        jobs["k"] = caps
    plan = B.Plan(ctx, jobs, pool.size)
    plan.upload(pool)
    tune_report = None
    if args.tune is None or args.tune:
        # Untimed: the autotuner picks each length bucket's kernel class (sf_plan_tune).
        tune_report = plan.tune(pool, reps=2)
    stream = torch.cuda.ExternalStream(plan.stream(), device=local)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")  # 256 MB
    for _ in range(warmup):
        plan.execute()
    plan.sync()
    out = plan.download()
    res = out.results
    cells = int(res["cells"].astype(np.uint64).sum())
    bad_status = int((res["status"] != 0).sum())
    # Timed region: K executes, L2 flushed before each, events on the plan's stream.
    clocks = Clocks(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    with torch.cuda.stream(stream):
        for s in range(steps):
            flush.zero_()
            ev[s][0].record(stream)
            plan.execute()
            ev[s][1].record(stream)
    plan.sync()
    torch.cuda.synchronize()
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = max_over_ranks(dist, statistics.mean(step_ms))
    value = cells * ws / (ms * 1e-3) / 1e9
    launches = plan.launches() * steps

    # Per-kernel attribution: each job's bucket from the library, each bucket's time from
    # per-stage events (one execute in order on the plan's stream; averaged over 3).
    prof = [plan.profile() for _ in range(3)]
    desc = json.loads(plan.describe())
    buckets = desc["buckets"]
    stages = ["pack"] + [bucket_name(b, lanes=True) for b in buckets]
    if len(prof[0]) == len(stages) + 2:
        stages += ["walk", "cigar-compact"]
    elif len(prof[0]) > len(stages):
        stages.append("cigar-compact")
    avg = [statistics.mean(p[i] for p in prof) for i in range(len(prof[0]))]
    jb = plan.job_buckets()
    on = jb != NONE32
    cells_b = np.bincount(jb[on].astype(np.int64), weights=res["cells"][on].astype(np.float64),
                          minlength=len(buckets))
    serial_ms = sum(avg[1:1 + len(buckets)])
    split = {}
    for fam in ("myers", "affine"):
        ids = [u for u, b in enumerate(buckets) if (b["kind"] == "myers") == (fam == "myers")]
        if not ids:
            continue
        c = float(sum(cells_b[u] for u in ids))
        t = float(sum(avg[1 + u] for u in ids))
        share = t / serial_ms if serial_ms else None
        split[fam] = {"cells": int(c), "pairs": int(sum(b["jobs"] for u, b in enumerate(buckets)
                                                         if u in ids)),
                      "kernel_ms_serial": t, "share_of_kernel_time": share,
                      "gcups_serial": c / (t * 1e-3) / 1e9 if t else None,
                      "gcups_in_step": c / (ms * 1e-3 * share) / 1e9 if share else None}
    if split:
        split["note"] = ("per-stage events, buckets run one after another on one stream; "
                         "gcups_in_step charges each family its share of the timed step")
    top = max(range(len(buckets)), key=lambda u: avg[1 + u])
    tb = buckets[top]
    top_cells = int(cells_b[top])
    top_ms = avg[1 + top]
    ops_cell = OPS_PER_CELL["myers"] if tb["kind"] == "myers" else (
        OPS_PER_CELL["affine_tb"] if tb["traceback"] else OPS_PER_CELL["affine"])
    achieved = top_cells * ops_cell / (top_ms * 1e-3) / 1e12
    peak = C.c_double()
    lib.sf_int_peak(local, C.byref(peak), None)
    peak_instr = peak.value * INT_PEAK_INSTR_PER_STEP / 3
    props = torch.cuda.get_device_properties(local)
    # HBM side of the same kernel: algorithmic bytes = its pairs' packed inputs (2 bits a base)
    # + 8 B of result each + half a byte of traceback bits per DP cell when it keeps them;
    # measured bytes = the ncu DRAM bytes per cell of this kernel, scaled to this launch.
    sel_jobs = jobs[jb == top]
    alg_bytes = int((sel_jobs["m"].astype(np.uint64) + sel_jobs["n"]).sum()) // 4 + 8 * len(sel_jobs)
    if tb.get("traceback"):
        alg_bytes += top_cells // 2
    hbm_gbs = alg_bytes / (top_ms * 1e-3) / 1e9
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            tr = json.load(f).get(bucket_name(tb))
        if tr:
            traffic = int(tr["bytes_per_cell"] * top_cells)
    except (OSError, ValueError):
        pass
    issue = props.multi_processor_count * 4 * 32 * (clk.get("sm_mhz") or 0) * 1e6 / 1e12
    roofline = {"bound": "int32", "kernel": stages[1 + top], "achieved": achieved,
                "peak": peak_instr, "unit": "T int32-instr/s",
                "frac": achieved / peak_instr if peak_instr else None,
                "achieved_note": "12 int32 ops per cell (10 without traceback), each one 32-bit "
                                 "instruction in a scalar row; the kernel does two cells per "
                                 "packed instruction where it can",
                "peak_source": "sf_int_peak measured live on this GPU (add-then-max chains); "
                               "restated in instructions: Tops x 2.094 / 3, the instructions "
                               "ncu counts per 3-op step (profiles/int_peak.md)",
                "peak_ops_tops": peak.value,
                "frac_of_ops_peak": achieved / peak.value if peak.value else None,
                "issue_ceiling": issue or None,
                "issue_ceiling_note": "SMs x 4 schedulers x 32 lanes x median SM clock: one "
                                      "instruction per scheduler per cycle",
                "ops_per_cell": ops_cell, "cells_per_launch": top_cells,
                "cells_source": "sf_plan_job_buckets (the library's bucketing) x DP_WORK cells",
                "kernel_ms": top_ms, "share_of_kernel_time": top_ms / serial_ms if serial_ms else None,
                "traffic": traffic,
                "traffic_source": "profiles/traffic.json (ncu small case, scaled by cells)",
                "hbm": {"algorithmic_bytes": alg_bytes, "achieved_gbs": hbm_gbs,
                        "measured_gbs": (traffic / (top_ms * 1e-3) / 1e9) if traffic else None,
                        "peak_gbs": hbm_peak, "frac": hbm_gbs / hbm_peak,
                        "measured_frac": (traffic / (top_ms * 1e-3) / 1e9 / hbm_peak)
                        if traffic else None,
                        "note": "top kernel only: packed inputs + results + 0.5 B/cell of "
                                "traceback bits (algorithmic); measured = ncu DRAM bytes"},
                "stages_ms": dict(zip(stages, [round(a, 4) for a in avg]))}

    # e2e through the C ABI from pinned host buffers.
    pin = torch.empty(pool.size, dtype=torch.uint8, pin_memory=True)
    pin.numpy()[:] = pool
    pin_np = pin.numpy()
    res2 = np.zeros(len(jobs), dtype=B.RESULT_DTYPE)
    want = jobs["want_cigar"] != 0
    cap = int((jobs["m"][want].astype(np.uint64) + jobs["n"][want] + 2).sum()) if want.any() else 1
    ops2 = torch.empty(max(1, cap), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    used = C.c_uint64()
    sc = (_abi.Affine * 1)(_abi.Affine(2, 4, 4, 2))

    def e2e_once():
        _abi.check(lib.sf_batch_run(ctx.handle, pin_np.ctypes.data_as(C.POINTER(C.c_uint8)),
                                    pool.size, jobs.ctypes.data_as(C.POINTER(_abi.JobT)),
                                    len(jobs), sc, 1, res2.ctypes.data_as(C.POINTER(_abi.ResultT)),
                                    ops2.ctypes.data_as(C.POINTER(C.c_uint32)), cap,
                                    C.byref(used)))

    e2e_once()
    if dist:
        dist.barrier()
    calls = []
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        c0 = time.perf_counter()
        e2e_once()
        calls.append(time.perf_counter() - c0)
    e2e_s = max_over_ranks(dist, (time.perf_counter() - t0) / e2e_steps)
    e2e_cells = int(res2["cells"].astype(np.uint64).sum())
    same = all(np.array_equal(res[f], res2[f]) for f in
               ("score", "distance", "pattern_end", "text_start", "text_end", "cells", "n_ops",
                "status")) and e2e_cells == cells
    h2d = int(pool.size + jobs.nbytes)
    d2h = int(res2.nbytes + used.value * 4)
    e2e = {"value": e2e_cells * ws / e2e_s / 1e9, "unit": "GCUPS", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3,
           "call_ms_median": statistics.median(calls) * 1e3, "call_ms_min": min(calls) * 1e3,
           "timing": "value and ms_per_step: the mean over the timed calls; the median and "
                     "minimum call show host interference on a shared machine",
           "pairs_per_s": len(pairs_list[-1]) * ws / e2e_s,
           "call": "sf_batch_run (C ABI), pinned host pool"}
    plan.close()
    ctx.close()

    plain = plain_rate(cfg, pairs_list, plain_pairs, variant, cigar) \
        if plain_pairs and rank == 0 else None

    cpu = checked = None
    parity = {"e2e_results_equal_plan": bool(same)}
    if rank == 0:
        import oracle as O
        threads = O.host_threads()
        if with_cpu:
            cpu, checked = cpu_baseline(cfg, pairs_list, args.cpu_seconds, threads, variant, caps)
        else:  # the parity check alone, on a small sample
            _, checked = cpu_baseline(cfg, pairs_list, 0.5, threads, variant, caps)
        parity.update(parity_check(cfg if variant == "base" else cfg + "-" + variant, pairs_list,
                                   res, out.ops, checked, threads))
        parity["status_nonzero"] = bad_status
    return {"value": value, "ms": ms, "cells": cells, "pairs": len(pairs_list[-1]),
            "jobs": int(len(jobs)), "e2e": e2e, "plain": plain, "roofline": roofline,
            "split": split, "clocks": clk, "launches": launches, "buckets": len(buckets),
            "tune": tune_report, "cpu": cpu, "parity": parity, "kind": kind}


def tune_summary(rep):
    if rep is None:
        return None
    ch = [g for g in rep["groups"] if (g["chosen"]["c"], g["chosen"]["lanes"]) != (g["c"], g["lanes"])]
    return {"groups": len(rep["groups"]), "changed": len(ch), "seconds": rep["seconds"],
            "choices": [f'{g["kind"]}-c{g["c"]}x{g["lanes"]}->c{g["chosen"]["c"]}x'
                        f'{g["chosen"]["lanes"]}' for g in ch]}


def parity_ok(p: dict) -> bool:
    return p.get("mismatches", 0) == 0 and p.get("cigar_failures", 0) == 0 and \
        p.get("status_nonzero", 0) == 0 and p.get("e2e_results_equal_plan", True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c3", choices=["c1", "c2", "c3", "c5"])
    ap.add_argument("--serve-seconds", type=float, default=20.0, help="c5: stream length")
    ap.add_argument("--sub-serve-seconds", type=float, default=30.0,
                    help="c3: length of the served stream in the `sub` object (0: none)")
    ap.add_argument("--sub", type=int, default=1,
                    help="c3: also measure config 2 and a served stream (1) or not (0)")
    ap.add_argument("--slots", type=int, default=8, help="c5: requests on the device at once")
    ap.add_argument("--store", type=int, default=1,
                    help="c5: texts as windows of a device-resident transcript store (1) or in "
                         "each request's pool (0)")
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of the workload's pairs")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-seconds", type=float, default=8.0)
    ap.add_argument("--ref-seconds", type=float, default=8.0)
    ap.add_argument("--plain-pairs", type=int, default=200)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cigar", type=int, default=1, help="c2/c3: traceback + CIGAR (1) or score only (0)")
    ap.add_argument("--variant", default="base", choices=["base", "window", "kslack", "kdecoy"],
                    help="c2: window = the mapper's windowed read-end extension; "
                         "c1: kslack = each pair capped at its distance + 16; "
                         "c1: kdecoy = Global distances capped at 160 against unrelated texts")
    ap.add_argument("--tune", type=int, default=None,
                    help="autotune the length buckets' kernel classes first (default: on)")
    args = ap.parse_args()
    if args.variant != "base" and (args.config, args.variant) not in VARIANTS:
        ap.error(f"--variant {args.variant} does not apply to {args.config}")
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.config == "c5":
        run_serving(args, ws, rank, local)
        return
    dist = dist_init(ws)

    import torch
    from spearfish_gb300 import _abi, build

    build.build()
    lib = _abi.load()
    torch.cuda.set_device(local)
    cigar = bool(args.cigar)
    h = measure_batch(args, args.config, args.variant, cigar, args.steps, args.warmup, dist, ws,
                      rank, local, lib, not args.no_cpu, args.plain_pairs, args.e2e_steps)
    sub = None
    if args.config == "c3" and args.sub and args.scale == 1.0:
        c2 = measure_batch(args, "c2", "base", cigar, args.steps, args.warmup, dist, ws, rank,
                           local, lib, not args.no_cpu, args.plain_pairs, args.e2e_steps)
        sub = {"c2": {"workload": workload_name("c2", "base", cigar), "value": c2["value"],
                      "ms_per_step": c2["ms"], "cells_per_step": c2["cells"],
                      "e2e": c2["e2e"], "plain": c2["plain"],
                      "batched_vs_plain": c2["value"] / c2["plain"]["value"] if c2["plain"] else None,
                      "roofline": {k: c2["roofline"][k] for k in
                                   ("kernel", "achieved", "peak", "frac", "kernel_ms", "traffic")},
                      "cpu_baseline": c2["cpu"], "parity": c2["parity"], "clocks": c2["clocks"]}}
        if not parity_ok(c2["parity"]):
            h["parity"]["sub_c2_failed"] = True
        if args.sub_serve_seconds > 0:
            live, sat, server, _ = serve_measure(args.sub_serve_seconds, args.slots, True, rank,
                                                 local)
            sub["c5"] = {"workload": GOLD["c5"], "latency": live, "saturation": sat,
                         "slots": args.slots,
                         "texts": "transcript store (HBM), windows sliced on the device"}
    if rank == 0:
        plain = h["plain"]
        ref_plain = sub["c2"]["plain"] if sub else None
        line = {"metric": "alignment GCUPS", "value": h["value"], "unit": "GCUPS", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": h["ms"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": DTYPE[args.config], "data": "synthetic (seeded; error model of sim.rs)",
                "config": {"workload": workload_name(args.config, args.variant, cigar),
                           "pairs": h["pairs"], "jobs": h["jobs"],
                           "cells_per_step": h["cells"], "l2": "flushed (256 MB write) before each step",
                           "parallelism": f"replicas x{ws}", "form": "batched persistent plan, CUDA graph",
                           "buckets": h["buckets"], "autotune": tune_summary(h["tune"])},
                "pairs_per_s": h["pairs"] * ws / (h["ms"] * 1e-3),
                "split": h["split"],
                "e2e": h["e2e"], "plain": plain,
                "batched_vs_plain": (h["value"] / plain["value"]) if plain else None,
                "plain_c2": ref_plain,
                "batched_vs_plain_c2": (h["value"] / ref_plain["value"]) if ref_plain else None,
                "parity": h["parity"],
                "roofline": h["roofline"], "cpu_baseline": h["cpu"], "clocks": h["clocks"],
                "gpu_launches": h["launches"], "gpu": torch.cuda.get_device_name(local),
                "sub": sub}
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0 and not parity_ok(h["parity"]):
        print("bench: GPU results differ from the oracle: " + json.dumps(h["parity"]),
              file=sys.stderr)
        sys.exit(3)


if __name__ == "__main__":
    main()
