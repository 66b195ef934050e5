"""The autotuner (sf_plan_tune): it may move each length bucket to another kernel class --
Myers blocks per lane x lanes per pair, affine row widths -- and results must not change
(bit-exact), in the tuned plan and in later plans of the same context."""
import json

import numpy as np
import pytest

import oracle as O
import refcases as R

pytestmark = pytest.mark.gpu


def _jobs(B, rng):
    pb = B.PoolBuilder()
    rows, want = [], []
    for q in range(160):
        m = int(rng.choice([60, 130, 300, 700, 1500, 2600, 5000]))
        p, t = R.rand_pair(m, int(rng.integers(3, 12)), int(rng.integers(1, 2 ** 62)))
        f = {"p_off": pb.add(p), "m": len(p), "t_off": pb.add(t), "n": len(t)}
        if q % 2 == 0:
            f.update(kind=B.JOB_MYERS, mode=R.INFIX)
            want.append(("m", O.myers_distance(p, t, R.INFIX)))
        else:
            band = int(rng.integers(8, 200))
            f.update(kind=B.JOB_AFFINE, mode=R.GLOBAL, band=band, want_cigar=1)
            want.append(("a", p, t, band))
        rows.append(f)
    jobs = B.new_jobs(len(rows))
    for q, f in enumerate(rows):
        for k, v in f.items():
            jobs[q][k] = v
    return pb.build(), jobs, want


def _same(a, b):
    for f in ("score", "distance", "pattern_end", "text_end", "cells", "n_ops", "status"):
        assert np.array_equal(a.results[f], b.results[f]), f
    for q in range(len(a.results)):
        assert a.cigar(q) == b.cigar(q), q


def test_tuned_plans_give_the_same_results():
    from spearfish_gb300 import build
    build.build()
    from spearfish_gb300 import batch as B
    rng = np.random.default_rng(1701)
    pool, jobs, want = _jobs(B, rng)
    ctx = B.Context(0)
    try:
        plan = B.Plan(ctx, jobs, pool.size)
        plan.upload(pool)
        plan.execute()
        before = plan.download()
        rep = plan.tune(pool, reps=1)
        assert rep["groups"] and all(g["tried"] for g in rep["groups"])
        myers = [g for g in rep["groups"] if g["kind"] == "myers"]
        assert any(len(g["tried"]) > 1 for g in myers)  # lanes per pair were swept
        plan.execute()
        after = plan.download()
        _same(before, after)
        # A later plan in the same context runs in the chosen classes.
        p2 = B.Plan(ctx, jobs, pool.size)
        p2.upload(pool)
        p2.execute()
        _same(before, p2.download())
        chosen = {(g["kind"], g["chosen"]["c"]) for g in rep["groups"]}
        kinds = {(b["kind"], b["c"]) for b in json.loads(p2.describe())["buckets"]}
        assert kinds <= chosen | {(b, c) for b, c in kinds if b == "local"}
        p2.close()
        ctx.untune()
        p3 = B.Plan(ctx, jobs, pool.size)
        p3.upload(pool)
        p3.execute()
        _same(before, p3.download())
        p3.close()
        plan.close()
    finally:
        ctx.close()
    # And the oracle agrees.
    for q, w in enumerate(want):
        r = before.results[q]
        if w[0] == "m":
            assert int(r["distance"]) == w[1]
        else:
            _, p, t, band = w
            o = O.traceback(p, t, O.TB_AFFINE, R.GLOBAL, R.ONT, band)
            assert (int(r["score"]), before.cigar(q)) == (o["score"], o["cigar"])
