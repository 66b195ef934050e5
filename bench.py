"""Benchmark of the GB300 alignment stage (one JSON line on rank 0).

Workload (default): banded affine alignment with traceback, 20,000 seeded pairs, query 2,000
bases, target = query with 10% ONT-like errors, band 128, Affine{2,4,4,2}, Global mode,
score + CIGAR per pair.  `--config c1` (Myers, 10,000 pairs) and `--config c3` (100,000
uneven Myers + affine pairs) run the other workloads.

  value   GCUPS of the batched, persistent, graph-captured plan on inputs resident in HBM
          (CUDA events on the plan's stream; L2 flushed between steps).
  e2e     the same GCUPS through the C ABI call a user makes (sf_batch_run): job
          descriptors and byte-code pool from pinned host memory to the device, execute,
          results and CIGARs back to the host, every step.
  plain   GCUPS of the one-launch-per-pair form (sf_affine_cigar per pair) on a sample.
  cpu_baseline  the CPU restatement of the reference's path (scalar rows, NEON rows on
          aarch64) on all host cores, on a bounded sample.

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
            ("c1", "kslack"): "myers-infix-10k-cap-d+16"}
WINDOW = (20, 10, 50, 5)  # pad, pad_div, xdrop, end bonus
K_SLACK = 16


def workload_name(args) -> str:
    if args.variant != "base":
        name = VARIANTS[(args.config, args.variant)]
        return name + ("-cigar" if args.config == "c2" and args.cigar else "")
    return GOLD[args.config if args.cigar or args.config != "c2" else "c2-score"]
OPS_PER_CELL = {"affine_tb": 12, "affine": 10, "myers": 0.625}


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
    from spearfish_gb300 import batch as B
    from spearfish_gb300 import workloads as W
    if cfg == "c1":
        w = W.config1(int(10_000 * scale))
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


AFFINE_C = (4, 6, 8, 9, 10, 11, 12, 14, 16, 20, 24, 28, 32, 40, 48)  # 32-bit register classes
AFFINE16_C = (4, 6, 8, 10, 12, 14, 16, 20, 24, 28, 32, 40, 48, 56, 64)  # packed 16-bit classes
AFFINE16H_C = (8, 10, 12, 14, 16, 18, 20, 24)  # the same with 16 lanes a pass


def fits16(j, w, sc, B) -> bool:
    """sf_plan.cu fits16: Global/Prefix banded passes whose values fit 16-bit fields."""
    if j["kind"] == B.JOB_LOCAL or j["mode"] == 0 or int(j["band"]) == 2 ** 64 - 1:
        return False
    mat, mis, opn, ext = sc
    if min(sc) < 0 or max(sc) > 1000 or w > 32 * AFFINE16_C[-1]:
        return False
    go = opn + ext
    step = max(mat, mis, go)
    return (mat + ext) * w + go + 2 * 64 * step + 2 * (go + mis + ext) + mat + 256 <= 16384 \
        and os.environ.get("SF_AFFINE16", "1")[:1] != "0"
MYERS_B = (1, 2, 3, 4, 6, 8, 12, 16)


def job_classes(jobs, B, scores=((2, 4, 4, 2),)):
    """The kernel class each job runs in, by the library's bucketing rule (sf_plan.cu)."""
    out = []
    for j in jobs:
        m, n = int(j["m"]), int(j["n"])
        if j["kind"] == B.JOB_MYERS:
            blocks = (m + 63) // 64
            if blocks <= 32:
                lanes = 1
                while lanes < blocks:
                    lanes <<= 1
                out.append(("myers", 1, lanes))
            else:
                out.append(("myers", next(b for b in MYERS_B if 32 * b >= blocks), 32))
            continue
        band = int(j["band"])
        if j["kind"] == B.JOB_LOCAL:
            w = int(j["dhi"]) - int(j["dlo"]) + 1
        elif j["mode"] == 0 or band == 2 ** 64 - 1:
            w = n + 1
        else:
            geom = max(int(j["window"]), n) if j["kind"] == B.JOB_EXTEND_WINDOW else n
            w = 2 * band + 1 + abs(m - geom)
        w = max(0, min(w, n + 1))
        tbf = bool(j["want_cigar"]) and j["kind"] != B.JOB_LOCAL
        if fits16(j, w, scores[int(j["sc_index"])], B):
            if os.environ.get("SF_AFFINE16_LANES") == "16" and w <= 16 * AFFINE16H_C[-1]:
                out.append(("affine16", next(c for c in AFFINE16H_C if 16 * c >= w), False, tbf,
                            16))
            else:
                out.append(("affine16", next(c for c in AFFINE16_C if 32 * c >= w), False, tbf,
                            32))
            continue
        c = next((c for c in AFFINE_C if 32 * c >= w), None)
        out.append(("affine", c, False, tbf, 32) if c else ("affine", 16, True, tbf, 32))
    return out


def cells_of(jobs, results, B) -> int:
    """Myers: m*n; affine: the band cells the passes computed (DP_WORK)."""
    return int(results["cells"].astype(np.uint64).sum())


def cpu_baseline(cfg, pairs_list, seconds: float, threads: int, variant: str = "base",
                 caps=None):
    """The reference's path restated in C (oracle), all host cores, bounded sample.  caps:
    per-pair Myers caps (the kslack variant)."""
    import oracle as O
    level = O.set_level(1)  # NEON rows where the host has them (the reference's level there)
    w = pairs_list[-1]
    kind = 0 if cfg == "c1" else (2 if variant == "window" else 1)
    mode = 0 if cfg == "c1" else (1 if variant == "window" else 2)
    band = None if cfg == "c1" else int(w.band[0]) if cfg == "c2" else None
    total_cells, total_t, done = 0, 0.0, 0
    idx = np.arange(len(w))
    rng = np.random.default_rng(7)
    rng.shuffle(idx)
    chunk = max(threads * 8, 64)
    while total_t < seconds and done < len(w):
        sel = idx[done:done + chunk]
        sub = w.subset(sel)
        t0 = time.perf_counter()
        if cfg == "c3":
            # per pair: Myers on the flanked target and affine with its own band
            my = pairs_list[0].subset(sel)
            _, c1 = O.run_pairs(0, threads, my.pool, my.p_off, my.m, my.pool, my.t_off, my.n, 0)
            c2 = 0
            for b in np.unique(sub.band):
                s2 = sub.subset(np.flatnonzero(sub.band == b))
                _, cc = O.run_pairs(1, threads, s2.pool, s2.p_off, s2.m, s2.pool, s2.t_off,
                                    s2.n, 2, sc=O.ONT, band=int(b))
                c2 += cc
            cells = c1 + c2
        else:
            _, cells = O.run_pairs(kind, threads, sub.pool, sub.p_off, sub.m, sub.pool, sub.t_off,
                                   sub.n, mode, sc=O.ONT, band=band,
                                   kv=None if caps is None else caps[sel],
                                   extend=WINDOW if variant == "window" else None)
        total_t += time.perf_counter() - t0
        total_cells += cells
        done += len(sel)
        chunk *= 2
    return {"value": total_cells / total_t / 1e9, "unit": "GCUPS", "cores": threads,
            "kind": "port", "level": "neon" if level == 1 else "scalar",
            "sample": f"{done} of {len(w)} pairs ({total_cells / 1e9:.2f} Gcells, "
                      f"{total_t:.1f} s wall on {threads} threads, score only: the reference "
                      f"computes no traceback)",
            "wall_s": total_t, "arch": platform.machine()}


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
        r = cpu_baseline(args.config, pairs_list, args.ref_seconds, threads, args.variant, caps)
        if s >= args.warmup:
            per_step.append(r)
    v = statistics.mean(r["value"] for r in per_step)
    # A step is one bounded sample of the workload (about ref_seconds of work).
    ms = 1e3 * statistics.mean(r["wall_s"] for r in per_step)
    line = {"metric": "alignment GCUPS", "value": v, "unit": "GCUPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": workload_name(args), "parallelism": "host threads",
                       "step": "a bounded sample of the workload's pairs"},
            "cpu_baseline": {"value": v, "unit": "GCUPS", "cores": threads, "kind": "port",
                             "sample": per_step[-1]["sample"], "level": per_step[-1]["level"]},
            "e2e": {"value": v, "unit": "GCUPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def pct(xs, q):
    return float(np.percentile(np.asarray(xs), q)) if xs else None


def run_serving(args, ws, rank, local):
    """Config 5: a bursty Poisson stream of read batches through the serving loop."""
    import threading

    from spearfish_gb300 import batch as B, build
    from spearfish_gb300 import serve as S
    from spearfish_gb300 import workloads as W

    build.build()
    stream = W.serving_stream(args.serve_seconds, seed=5 + rank)
    rng = np.random.default_rng(505 + rank)
    batches = []
    store = ctx = tx = None
    if args.store:
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
    srv = S.Server(local, slots=args.slots, store=store)
    try:
        for pool, jobs in batches[:3]:  # warm-up: buffers grow to a working size
            srv.wait(srv.submit(pool, jobs))
        # Real time: each batch is submitted at its arrival time.
        tickets = [None] * len(batches)
        t0 = time.perf_counter()

        def feeder():
            for q, ((at, _), (pool, jobs)) in enumerate(zip(stream, batches)):
                d = at - (time.perf_counter() - t0)
                if d > 0:
                    time.sleep(d)
                tickets[q] = srv.submit(pool, jobs)

        th = threading.Thread(target=feeder)
        th.start()
        lat, cells, t_last = [], 0, t0
        for q in range(len(batches)):
            while tickets[q] is None:
                time.sleep(0.0002)
            out, st = srv.wait(tickets[q])
            lat.append(st.total_ms)
            cells += st.cells
            t_last = time.perf_counter()
        th.join()
        wall = t_last - t0
        reads = sum(n for _, n in stream)
        live = {"p50_ms": pct(lat, 50), "p95_ms": pct(lat, 95), "p99_ms": pct(lat, 99),
                "max_ms": max(lat), "batches": len(batches), "reads": reads,
                "offered_reads_per_s": reads / args.serve_seconds,
                "sustained_gcups": cells / wall / 1e9, "wall_s": wall}
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
    if rank == 0:
        line = {"metric": "alignment GCUPS", "value": sat["gcups"], "unit": "GCUPS",
                "n_gpus": ws, "steps": 1, "warmup": 3, "ms_per_step": wall2 * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "int32", "data": "synthetic (seeded read model; sim.rs error model)",
                "config": {"workload": GOLD["c5"], "serve_seconds": args.serve_seconds,
                           "slots": args.slots, "jobs_per_read": 4,
                           "texts": "transcript store (HBM), windows sliced on the device"
                           if store is not None else "in each request's pool",
                           "parallelism": f"replicas x{ws}"},
                "latency": live, "saturation": sat,
                "server": {k: int(v) for k, v in q.items()},
                "e2e": {"value": sat["gcups"], "unit": "GCUPS",
                        "h2d_bytes_per_step": int(sum(p.size + j.nbytes for p, j in batches)),
                        "d2h_bytes_per_step": int(sum(len(j) * 64 for _, j in batches)),
                        "call": "sf_server_submit / sf_server_wait (C ABI)"}}
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c5"])
    ap.add_argument("--serve-seconds", type=float, default=20.0, help="c5: stream length")
    ap.add_argument("--slots", type=int, default=8, help="c5: requests on the device at once")
    ap.add_argument("--store", type=int, default=1,
                    help="c5: texts as windows of a device-resident transcript store (1) or in "
                         "each request's pool (0)")
    ap.add_argument("--scale", type=float, default=1.0, help="fraction of the workload's pairs")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-seconds", type=float, default=8.0)
    ap.add_argument("--ref-seconds", type=float, default=8.0)
    ap.add_argument("--plain-pairs", type=int, default=200)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cigar", type=int, default=1, help="c2/c3: traceback + CIGAR (1) or score only (0)")
    ap.add_argument("--variant", default="base", choices=["base", "window", "kslack"],
                    help="c2: window = the mapper's windowed read-end extension; "
                         "c1: kslack = each pair capped at its distance + 16")
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
    from spearfish_gb300 import align as A
    from spearfish_gb300 import batch as B
    import ctypes as C

    build.build()
    lib = _abi.load()
    torch.cuda.set_device(local)
    pool, jobs, pairs_list, kind = workload(args.config, args.scale, bool(args.cigar), args.variant)
    ctx = B.Context(local)
    caps = None
    if args.variant == "kslack":
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
    tune_map = {}
    for g in (tune_report or {}).get("groups", []):
        key = ("myers", g["c"], g["lanes"]) if g["kind"] == "myers" else \
            (g["kind"], g["c"], bool(g["wide"]), bool(g["traceback"]), g["lanes"])
        ch = g["chosen"]
        tune_map[key] = ("myers", ch["c"], ch["lanes"]) if g["kind"] == "myers" else \
            (g["kind"], ch["c"], bool(g["wide"]), bool(g["traceback"]), ch["lanes"])
    stream = torch.cuda.ExternalStream(plan.stream(), device=local)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")  # 256 MB
    for _ in range(args.warmup):
        plan.execute()
    plan.sync()
    out = plan.download()
    cells = cells_of(jobs, out.results, B)
    bad = int((out.results["status"] != 0).sum())
    # Timed region: K executes, L2 flushed before each, events on the plan's stream.
    clocks = Clocks(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for s in range(args.steps):
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
    launches = plan.launches() * args.steps

    # Roofline of the dominant kernel: per-stage events (same stream), averaged.
    prof = [plan.profile() for _ in range(3)]
    desc = json.loads(plan.describe())
    stages = ["pack"] + [f"{b['kind']}-c{b['c']}{'-wide' if b['wide'] else ''}"
                         f"{'-tb' if b['traceback'] else ''}" for b in desc["buckets"]]
    if len(prof[0]) == len(stages) + 2:
        stages += ["walk", "cigar-compact"]
    elif len(prof[0]) > len(stages):
        stages.append("cigar-compact")
    avg = [statistics.mean(p[i] for p in prof) for i in range(len(prof[0]))]
    top = max(range(1, 1 + len(desc["buckets"])), key=lambda i: avg[i])
    tb = desc["buckets"][top - 1]
    cls = [tune_map.get(c, c) for c in job_classes(jobs, B)]
    key = ("myers", tb["c"], tb["lanes"]) if tb["kind"] == "myers" else \
        (tb["kind"], tb["c"], bool(tb["wide"]), bool(tb["traceback"]), tb["lanes"])
    sel = np.array([c == key for c in cls])
    top_cells = int(out.results["cells"][sel].astype(np.uint64).sum())
    ops_cell = OPS_PER_CELL["myers"] if tb["kind"] == "myers" else (
        OPS_PER_CELL["affine_tb"] if tb["traceback"] else OPS_PER_CELL["affine"])
    achieved = top_cells * ops_cell / (avg[top] * 1e-3) / 1e12
    peak = C.c_double()
    lib.sf_int_peak(local, C.byref(peak), None)
    # HBM side of the same kernel: algorithmic bytes = its pairs' packed inputs (2 bits a base)
    # + 8 B of result each + half a byte of traceback bits per DP cell when it keeps them;
    # measured bytes = the ncu DRAM bytes per cell of this kernel, scaled to this launch.
    sel_jobs = jobs[sel]
    alg_bytes = int((sel_jobs["m"].astype(np.uint64) + sel_jobs["n"]).sum()) // 4 + 8 * len(sel_jobs)
    if tb.get("traceback"):
        alg_bytes += top_cells // 2
    hbm_gbs = alg_bytes / (avg[top] * 1e-3) / 1e9
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
            tr = json.load(f).get(stages[top])
        if tr:
            traffic = int(tr["bytes_per_cell"] * top_cells)
    except (OSError, ValueError):
        pass
    roofline = {"bound": "int32", "kernel": stages[top], "achieved": achieved,
                "peak": peak.value, "unit": "Tops/s", "frac": achieved / peak.value if peak.value else None,
                "peak_source": "measured on this GPU by sf_int_peak (int32 add-then-max mix)",
                "ops_per_cell": ops_cell, "cells_per_launch": top_cells,
                "kernel_ms": avg[top], "traffic": traffic,
                "traffic_source": "profiles/traffic.json (ncu small case, scaled by cells)",
                "hbm": {"algorithmic_bytes": alg_bytes, "achieved_gbs": hbm_gbs,
                        "measured_gbs": (traffic / (avg[top] * 1e-3) / 1e9) if traffic else None,
                        "peak_gbs": hbm_peak, "frac": hbm_gbs / hbm_peak,
                        "measured_frac": (traffic / (avg[top] * 1e-3) / 1e9 / hbm_peak)
                        if traffic else None,
                        "note": "top kernel only: packed inputs + results + 0.5 B/cell of "
                                "traceback bits (algorithmic); measured = ncu DRAM bytes"},
                "stages_ms": dict(zip(stages, [round(a, 4) for a in avg]))}

    # e2e through the C ABI from pinned host buffers.
    pin = torch.empty(pool.size, dtype=torch.uint8, pin_memory=True)
    pin.numpy()[:] = pool
    pin_np = pin.numpy()
    res = np.zeros(len(jobs), dtype=B.RESULT_DTYPE)
    want = jobs["want_cigar"] != 0
    cap = int((jobs["m"][want].astype(np.uint64) + jobs["n"][want] + 2).sum()) if want.any() else 1
    ops = torch.empty(max(1, cap), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    used = C.c_uint64()
    sc = (_abi.Affine * 1)(_abi.Affine(2, 4, 4, 2))

    def e2e_once():
        _abi.check(lib.sf_batch_run(ctx.handle, pin_np.ctypes.data_as(C.POINTER(C.c_uint8)),
                                    pool.size, jobs.ctypes.data_as(C.POINTER(_abi.JobT)),
                                    len(jobs), sc, 1, res.ctypes.data_as(C.POINTER(_abi.ResultT)),
                                    ops.ctypes.data_as(C.POINTER(C.c_uint32)), cap,
                                    C.byref(used)))

    e2e_once()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        e2e_once()
    e2e_s = max_over_ranks(dist, (time.perf_counter() - t0) / args.e2e_steps)
    e2e_cells = int(res["cells"].astype(np.uint64).sum())
    assert e2e_cells == cells
    h2d = int(pool.size + jobs.nbytes)
    d2h = int(res.nbytes + used.value * 4)
    e2e = {"value": e2e_cells * ws / e2e_s / 1e9, "unit": "GCUPS", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3,
           "pairs_per_s": len(pairs_list[-1]) * ws / e2e_s,
           "call": "sf_batch_run (C ABI), pinned host pool"}

    # Plain form: one launch (one C-ABI call) per pair on a sample.
    plain = None
    if args.plain_pairs and rank == 0:
        w = pairs_list[-1]
        n = min(args.plain_pairs, len(w))
        c0, _ = A.dp_work()
        t0 = time.perf_counter()
        for q in range(n):
            if kind == "myers":
                A.distance(w.pattern(q), w.text(q), A.Mode.Infix)
            elif args.variant == "window":
                win = int(jobs["window"][q])
                if args.cigar:
                    A.affine_extend_window_cigar(w.pattern(q), w.text(q), win, A.Affine.ONT,
                                                 int(w.band[q]), WINDOW[3], WINDOW[2])
                else:
                    A.affine_extend_window(w.pattern(q), w.text(q), win, A.Affine.ONT,
                                           int(w.band[q]), WINDOW[3], WINDOW[2])
            elif not args.cigar:
                A.affine(w.pattern(q), w.text(q), A.Mode.Global, A.Affine.ONT, int(w.band[q]))
            else:
                A.affine_cigar(w.pattern(q), w.text(q), A.Mode.Global, A.Affine.ONT,
                               int(w.band[q]))
        dt = time.perf_counter() - t0
        c1, _ = A.dp_work()
        pc = (c1 - c0) if kind != "myers" else int(
            sum(int(w.m[q]) * int(w.n[q]) for q in range(n)))
        plain = {"value": pc / dt / 1e9, "unit": "GCUPS", "pairs": n,
                 "call": ("sf_distance" if kind == "myers" else
                          ("sf_affine_extend_window" if args.variant == "window" else "sf_affine") +
                          ("_cigar" if args.cigar else "")),
                 "ms_per_pair": dt / n * 1e3}

    cpu = None
    if rank == 0 and not args.no_cpu:
        import oracle as O
        cpu = cpu_baseline(args.config, pairs_list, args.cpu_seconds, O.host_threads(),
                           args.variant, caps)

    if rank == 0:
        line = {"metric": "alignment GCUPS", "value": value, "unit": "GCUPS", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "int32", "data": "synthetic (seeded; error model of sim.rs)",
                "config": {"workload": workload_name(args),
                           "pairs": int(len(jobs)),
                           "cells_per_step": cells, "l2": "flushed (256 MB write) before each step",
                           "parallelism": f"replicas x{ws}", "form": "batched persistent plan, CUDA graph",
                           "buckets": len(desc["buckets"]), "status_nonzero": bad,
                           "autotune": None if tune_report is None else {
                               "groups": len(tune_report["groups"]),
                               "changed": sum(1 for g in tune_report["groups"]
                                              if (g["chosen"]["c"], g["chosen"]["lanes"]) !=
                                              (g["c"], g["lanes"])),
                               "seconds": tune_report["seconds"],
                               "choices": [f'{g["kind"]}-c{g["c"]}x{g["lanes"]}->'
                                           f'c{g["chosen"]["c"]}x{g["chosen"]["lanes"]}'
                                           for g in tune_report["groups"]
                                           if (g["chosen"]["c"], g["chosen"]["lanes"]) !=
                                           (g["c"], g["lanes"])]}},
                "pairs_per_s": len(pairs_list[-1]) * ws / (ms * 1e-3),
                "e2e": e2e, "plain": plain,
                "batched_vs_plain": (value / plain["value"]) if plain else None,
                "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
                "gpu_launches": launches, "gpu": torch.cuda.get_device_name(local)}
        print(json.dumps(line))
    plan.close()
    ctx.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
