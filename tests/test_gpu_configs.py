"""Parity at the benchmarked workloads: every seeded pair that bench.py times, at full size,
through the same two paths the bench times, against the oracle.

  config 1  10,000 Myers Infix pairs (1 kb query, 8% errors, 50-base flanks);
  config 2  20,000 banded affine Global pairs with CIGARs (2 kb query, 10% ONT-like errors,
            band 128, Affine{2,4,4,2});
  config 3  100,000 uneven pairs (200 b - 20 kb), each a Myers Infix job and a banded
            affine Global job with a CIGAR (band 64-512 by length).

Each workload runs (1) as an autotuned batched plan (`sf_plan_tune`, then `sf_plan_execute`,
as the bench's device-timed steps) and (2) through `sf_batch_run` in the same context (the
bench's end-to-end call; configs 1 and 2 run in segments there).  Checks, bit-exact:
  - every Myers distance and every affine score equals the oracle's (align.rs:87-168
    `distance_with`, 2446-2666 `run_core`), every end cell is (m, n) and every status 0;
  - every pass's DP cells (the GCUPS numerator) equal the oracle's DP_WORK count
    (align.rs:2573-2578), and m * n for Myers;
  - every CIGAR consumes the whole pattern, ends at the text's end and re-scores exactly to
    the pair's score;
  - a seeded sample of 1,000 CIGARs per workload equals the oracle's full-matrix traceback
    (its tie order: CIGARs are not pinned by the reference, which computes none);
  - both paths give the same results and the same CIGAR ops.
"""
import os
import sys

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

SAMPLE = 1000


@pytest.fixture(scope="module")
def lib():
    from spearfish_gb300 import build
    build.build()


def _ops_in_job_order(out) -> np.ndarray:
    r = out.results
    lens = r["n_ops"].astype(np.int64)
    starts = r["cigar_off"].astype(np.int64)
    total = int(lens.sum())
    if total == 0:
        return np.zeros(0, np.uint32)
    first = np.cumsum(lens) - lens
    idx = np.repeat(starts - first, lens) + np.arange(total)
    return out.ops[idx]


def _run_both(jobs, pool, tune=True):
    """(plan output, sf_batch_run output) in one context, the plan autotuned first."""
    from spearfish_gb300 import batch as B
    ctx = B.Context(0)
    try:
        plan = B.Plan(ctx, jobs, pool.size)
        plan.upload(pool)
        if tune:
            plan.tune(pool, reps=1)
        plan.execute()
        plan.execute()  # a replay of the captured graph, as the timed steps are
        plan.sync()
        a = plan.download()
        plan.close()
        b = B.run(ctx, pool, jobs)
    finally:
        ctx.close()
    return a, b


def _same(a, b):
    for f in ("score", "distance", "pattern_end", "text_start", "text_end", "text_read",
              "cells", "n_ops", "status"):
        assert np.array_equal(a.results[f], b.results[f]), f
    assert np.array_equal(_ops_in_job_order(a), _ops_in_job_order(b))


def _check_myers(res, w, threads):
    d, cells = O.run_pairs(0, threads, w.pool, w.p_off, w.m, w.pool, w.t_off, w.n, O.INFIX)
    assert (res["status"] == 0).all()
    bad = np.flatnonzero(res["distance"].astype(np.int64) != d)
    assert bad.size == 0, f"{bad.size} distances differ, first pair {bad[:5]}"
    assert np.array_equal(res["cells"].astype(np.uint64),
                          w.m.astype(np.uint64) * w.n.astype(np.uint64))
    assert int(res["cells"].astype(np.uint64).sum()) == cells


def _check_affine(out, res, q0, w, threads, seed):
    """Affine jobs q0 .. q0 + len(w) of `out` (results `res` of those jobs) against the
    oracle: scores, ends, cells, every CIGAR re-scored, a sample traced back."""
    s, cells = O.run_pairs(1, threads, w.pool, w.p_off, w.m, w.pool, w.t_off, w.n, O.GLOBAL,
                           sc=O.ONT, bands=w.band, per_pair_cells=True)
    assert (res["status"] == 0).all()
    bad = np.flatnonzero(res["score"].astype(np.int64) != s)
    assert bad.size == 0, f"{bad.size} scores differ, first pairs {bad[:5]}"
    assert np.array_equal(res["pattern_end"], w.m.astype(np.uint64))
    assert np.array_equal(res["text_end"], w.n.astype(np.uint64))
    bad = np.flatnonzero(res["cells"].astype(np.uint64) != cells)
    assert bad.size == 0, f"{bad.size} cell counts differ, first pairs {bad[:5]}"
    code = O.check_cigars(threads, w.pool, w.p_off, w.m, w.pool, w.t_off, w.n, out.ops,
                          res["cigar_off"], res["n_ops"], res["text_start"], res["text_end"],
                          res["score"], O.ONT)
    bad = np.flatnonzero(code)
    assert bad.size == 0, f"{bad.size} CIGARs fail (codes {np.unique(code[bad])}), first {bad[:5]}"
    rng = np.random.default_rng(seed)
    for q in rng.choice(len(w), size=min(SAMPLE, len(w)), replace=False):
        q = int(q)
        o = O.traceback(w.pattern(q), w.text(q), O.TB_AFFINE, O.GLOBAL, O.ONT, int(w.band[q]))
        assert o["status"] == 0
        assert out.cigar(q0 + q) == o["cigar"], q
        assert int(res["text_start"][q]) == o["text_start"], q


def test_config1_myers_10k(lib):
    import bench
    pool, jobs, (w,), _ = bench.workload("c1", 1.0)
    assert len(w) == 10_000
    a, b = _run_both(jobs, pool)
    _same(a, b)
    _check_myers(a.results, w, O.host_threads())


def test_config2_affine_cigar_20k(lib):
    import bench
    pool, jobs, (w,), _ = bench.workload("c2", 1.0)
    assert len(w) == 20_000 and (w.band == 128).all()
    a, b = _run_both(jobs, pool)
    _same(a, b)
    _check_affine(a, a.results, 0, w, O.host_threads(), seed=22)


def test_config3_uneven_100k(lib):
    import bench
    pool, jobs, (my, af), _ = bench.workload("c3", 1.0)
    assert len(my) == len(af) == 100_000
    a, b = _run_both(jobs, pool)
    _same(a, b)
    n = len(my)
    threads = O.host_threads()
    _check_myers(a.results[:n], my, threads)
    _check_affine(a, a.results[n:], n, af, threads, seed=33)
