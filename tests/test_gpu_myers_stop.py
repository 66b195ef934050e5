"""Capped Global and Prefix Myers pairs stop at the first column wholly past their cap
(sf_myers.cu, KC): the results equal the oracle's `distance_with` (align.rs:93-168, whose
Ukkonen cutoff answers None past k) for pairs that stop early (unrelated texts), late
(related texts with k just below their distance) or never (k at or above it); for every
Myers class (1..16 blocks a lane, 1..32 lanes a pair); with Infix and uncapped pairs in the
same plan (they run on the same kernel and never stop); and equal to the same plan with the
stop turned off (SF_MYERS_STOP=0)."""
import os

import numpy as np
import pytest

import oracle as O
import refcases as R

pytestmark = pytest.mark.gpu
NONE = 0xFFFFFFFF


@pytest.fixture(scope="module")
def ctx():
    from spearfish_gb300 import build
    build.build()
    from spearfish_gb300 import batch as B
    c = B.Context(0)
    yield c
    c.close()


def _run(ctx, pool, jobs, stop=True):
    from spearfish_gb300 import batch as B
    old = os.environ.get("SF_MYERS_STOP")
    os.environ["SF_MYERS_STOP"] = "1" if stop else "0"
    try:
        return B.run(ctx, pool, jobs).results["distance"].astype(np.int64)
    finally:
        if old is None:
            del os.environ["SF_MYERS_STOP"]
        else:
            os.environ["SF_MYERS_STOP"] = old


def test_capped_global_prefix_stop(ctx):
    from spearfish_gb300 import batch as B
    rng = np.random.default_rng(2601)
    pb = B.PoolBuilder()
    rows = []
    for m in (1, 40, 64, 65, 300, 1000, 2100, 4200, 9000, 20000):
        for kind in ("unrelated", "related", "related", "flank"):
            p = rng.integers(0, 4, m).astype(np.uint8)
            if kind == "unrelated":
                t = rng.integers(0, 4, m + int(rng.integers(0, 60))).astype(np.uint8)
            else:
                t = np.asarray(R.mutate(p.tolist(), R.rand_edits(rng, max(1, m // 12), m)),
                               np.uint8)
                if kind == "flank":
                    t = np.concatenate([t, rng.integers(0, 4, 80).astype(np.uint8)])
            for mode in (R.GLOBAL, R.PREFIX, R.INFIX):
                d = O.myers_distance(p, t, mode)
                for k in {0, max(0, d - 40), max(0, d - 1), d, d + 5, NONE}:
                    rows.append((pb.add(p), m, pb.add(t), len(t), mode, k, p, t))
    order = rng.permutation(len(rows))  # mixed classes and modes in every bucket
    rows = [rows[i] for i in order]
    jobs = B.new_jobs(len(rows))
    for q, (po, m, to, n, mode, k, _, _) in enumerate(rows):
        jobs[q]["p_off"], jobs[q]["m"], jobs[q]["t_off"], jobs[q]["n"] = po, m, to, n
        jobs[q]["kind"], jobs[q]["mode"], jobs[q]["k"] = B.JOB_MYERS, mode, k
    pool = pb.build()
    got = _run(ctx, pool, jobs)
    for q, (_, _, _, _, mode, k, p, t) in enumerate(rows):
        want = O.myers_distance(p, t, mode, k)
        assert got[q] == (NONE if want is None else want), (q, len(p), mode, k)
    assert np.array_equal(got, _run(ctx, pool, jobs, stop=False))


def test_every_class_with_caps(ctx):
    """Patterns of every Myers class, the tuner's alternatives included: each class's lanes
    and blocks pass the column verdict down the pipeline."""
    from spearfish_gb300 import batch as B
    rng = np.random.default_rng(2602)
    pb = B.PoolBuilder()
    rows = []
    for m in (60, 120, 250, 500, 1000, 2000, 4000, 8000, 12000, 16000, 24000):
        for _ in range(3):
            p = rng.integers(0, 4, m).astype(np.uint8)
            t = rng.integers(0, 4, m).astype(np.uint8) if rng.random() < 0.5 else \
                np.asarray(R.mutate(p.tolist(), R.rand_edits(rng, m // 15, m)), np.uint8)
            mode = [R.GLOBAL, R.PREFIX][int(rng.integers(0, 2))]
            k = int(rng.integers(0, m // 3 + 2))
            rows.append((pb.add(p), m, pb.add(t), len(t), mode, k, p, t))
    jobs = B.new_jobs(len(rows))
    for q, (po, m, to, n, mode, k, _, _) in enumerate(rows):
        jobs[q]["p_off"], jobs[q]["m"], jobs[q]["t_off"], jobs[q]["n"] = po, m, to, n
        jobs[q]["kind"], jobs[q]["mode"], jobs[q]["k"] = B.JOB_MYERS, mode, k
    pool = pb.build()
    ctx2 = B.Context(0)
    try:
        plan = B.Plan(ctx2, jobs, pool.size)
        plan.upload(pool)
        plan.tune(pool, reps=1)  # alternative classes per group, all checked below
        plan.close()
        got = B.run(ctx2, pool, jobs).results["distance"].astype(np.int64)
    finally:
        ctx2.close()
    for q, (_, _, _, _, mode, k, p, t) in enumerate(rows):
        want = O.myers_distance(p, t, mode, k)
        assert got[q] == (NONE if want is None else want), (q, len(p), mode, k)
