"""The packed 16-bit banded affine kernel (sf_affine16_impl.cuh) against the oracle.

Passes whose values fit 16-bit fields run two cells per register with a per-pass offset that
is rebased every 64 rows.  These tests drive it where that matters -- long passes (many
rebases), sequences whose row maximum climbs (identical) or falls (unrelated) for thousands
of rows, every 16-bit class from 4 to 64 cells per lane, scores near the admission bound,
Prefix passes with X-drop and cut bookkeeping -- and check scores, end cells and CIGARs
bit-exactly against the oracle, and against the 32-bit kernel on the same jobs
(SF_AFFINE16=0 routes every pass to it)."""
import json
import os

import numpy as np
import pytest

import oracle as O
import refcases as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from spearfish_gb300 import build
    build.build()
    from spearfish_gb300 import batch as B
    c = B.Context(0)
    yield c
    c.close()


class Jobs:
    def __init__(self):
        from spearfish_gb300 import batch as B
        self.B = B
        self.pool = B.PoolBuilder()
        self.rows = []
        self.want = []

    def add(self, want, **f):
        p, t = f.pop("p"), f.pop("t")
        f["p_off"] = self.pool.add(p)
        f["m"] = len(p)
        f["t_off"] = self.pool.add(t)
        f["n"] = len(t)
        self.rows.append(f)
        self.want.append((want, p, t))

    def jobs(self):
        jobs = self.B.new_jobs(len(self.rows))
        for q, f in enumerate(self.rows):
            for k, v in f.items():
                jobs[q][k] = v
        return jobs

    def run(self, ctx, scores, int16=True, lanes=32, w64=True):
        """Runs the jobs in one plan (16-bit passes on `lanes` lanes each where they fit; with
        w64, rows wider than 32 x 40 cells on two warps); returns the output and the bucket
        kinds it used (affine16h: 16 lanes a pass, affine16w: 64)."""
        env = {"SF_AFFINE16": "1" if int16 else "0", "SF_AFFINE16_LANES": str(lanes),
               "SF_AFFINE16_W64": "1" if w64 else "0"}
        old = {k: os.environ.get(k) for k in env}
        os.environ.update(env)
        try:
            pool = self.pool.build()
            jobs = self.jobs()
            plan = self.B.Plan(ctx, jobs, pool.size, scores)
            try:
                plan.upload(pool)
                plan.execute()
                out = plan.download()
                name = {16: "affine16h", 32: "affine16", 64: "affine16w"}
                kinds = {(b["kind"], b["c"]) if b["kind"] != "affine16"
                         else (name[b["lanes"]], b["c"])
                         for b in json.loads(plan.describe())["buckets"]}
            finally:
                plan.close()
        finally:
            for k, v in old.items():
                if v is None:
                    del os.environ[k]
                else:
                    os.environ[k] = v
        return out, kinds


def _check(J, out, scores):
    for q, (w, p, t) in enumerate(J.want):
        f = J.rows[q]
        r = out.results[q]
        sc = scores[int(f.get("sc_index", 0))]
        band = None if f.get("band", 2 ** 64 - 1) == 2 ** 64 - 1 else int(f["band"])
        if f["kind"] == 1:
            if f.get("want_cigar"):
                o = O.traceback(p, t, O.TB_AFFINE, int(f["mode"]), sc, band)
                assert (int(r["status"]), int(r["score"]), int(r["text_end"])) == \
                    (o["status"], o["score"], o["end_j"]), (q, f["m"], band)
                if o["status"] == 0:
                    assert out.cigar(q) == o["cigar"], (q, f["m"], band)
            else:
                assert int(r["score"]) == O.affine(p, t, int(f["mode"]), sc, band), (q, band)
        else:
            win, bonus, xd = int(f["window"]), int(f["end_bonus"]), int(f["xdrop"])
            if f.get("want_cigar"):
                o = O.traceback(p, t, O.TB_EXTEND, O.PREFIX, sc, band, win, bonus, xd)
                assert (int(r["status"]), int(r["score"]), int(r["pattern_end"]),
                        int(r["text_end"])) == (o["status"], o["score"], o["end_i"],
                                                o["end_j"]), (q, band)
                if o["status"] == 0:
                    assert out.cigar(q) == o["cigar"], (q, band)
            else:
                got = (int(r["score"]), int(r["pattern_end"]), int(r["text_end"]),
                       int(r["text_read"]))
                assert got == O.affine_extend_window(p, t, win, sc, band, bonus, xd), (q, band)


def _same(a, b):
    for f in ("score", "pattern_end", "text_start", "text_end", "text_read", "cells", "n_ops",
              "status"):
        assert np.array_equal(a.results[f], b.results[f]), f
    for q in range(len(a.results)):
        assert a.cigar(q) == b.cigar(q), q


def test_long_passes_rebase(ctx):
    """Passes of 4k-20k rows: the row maximum climbs (identical sequences), falls (unrelated
    sequences) or wanders (10% errors); the offset is rebased every 64 rows."""
    rng = np.random.default_rng(1601)
    J = Jobs()
    for m, band, kind in ((20000, 40, "same"), (12000, 64, "unrelated"), (16000, 100, "noisy"),
                          (4000, 300, "noisy"), (9000, 16, "unrelated")):
        q = rng.integers(0, 4, m).tolist()
        if kind == "same":
            t = list(q)
        elif kind == "unrelated":
            t = rng.integers(0, 4, m + int(rng.integers(-20, 20))).tolist()
        else:
            t = R.mutate(q, R.rand_edits(rng, m // 10, m))
        for cig in (0, 1):
            J.add(None, p=q, t=t, kind=1, mode=R.GLOBAL, band=band, want_cigar=cig)
        J.add(None, p=q, t=t, kind=2, band=band, window=len(t) + 50, xdrop=R.I32_MAX,
              end_bonus=5, want_cigar=1)
    out, kinds = J.run(ctx, (R.ONT,))
    assert any(k == "affine16" for k, _ in kinds), kinds
    _check(J, out, (R.ONT,))


def test_every_class(ctx):
    """Row widths reaching each 16-bit class (4..64 cells per lane), Global and Prefix, with
    and without CIGARs; the same jobs on the 32-bit kernel give identical results."""
    rng = np.random.default_rng(1602)
    J = Jobs()
    for band in (1, 40, 70, 100, 130, 170, 200, 260, 330, 400, 470, 520, 680, 800, 940):
        for rep in range(2):
            m = int(rng.integers(max(300, 2 * band + 100), 2 * band + 1200))
            p, t = R.rand_pair(m, int(rng.integers(3, 15)), int(rng.integers(1, 2 ** 62)))
            mode = R.GLOBAL if rep == 0 else R.PREFIX
            sci = int(rng.integers(0, 2))
            J.add(None, p=p, t=t, kind=1, mode=mode, band=band, want_cigar=rep, sc_index=sci)
            w = len(t) + int(rng.integers(0, 100))
            xd = int(rng.integers(10, 200)) if rng.random() < 0.7 else R.I32_MAX
            J.add(None, p=p, t=t, kind=2, band=band, window=w, xdrop=xd,
                  end_bonus=int(rng.integers(0, 9)), want_cigar=1 - rep, sc_index=sci)
    scores = (R.ONT, R.HIFI)
    out, kinds = J.run(ctx, scores, w64=False)
    classes = {c for k, c in kinds if k == "affine16"}
    assert classes >= {4, 8, 16, 32, 48, 64}, sorted(classes)
    _check(J, out, scores)
    out32, kinds32 = J.run(ctx, scores, int16=False)
    assert not any(k.startswith("affine16") for k, _ in kinds32)
    _same(out, out32)
    # By default the rows wider than 32 x 40 cells run on two warps: the same results.
    outw, kindsw = J.run(ctx, scores)
    assert {c for k, c in kindsw if k == "affine16w"} >= {24, 32}, sorted(kindsw)
    _same(out, outw)


def test_scores_near_the_bound(ctx):
    """Score sets whose admission bound is tight (large match bonus and extension, wide rows),
    and ones just past it (32-bit kernel): all equal the oracle."""
    rng = np.random.default_rng(1603)
    scores = ((20, 30, 10, 20), (9, 1, 0, 1), (1, 9, 40, 3), (0, 0, 0, 0), (3, 5, 7, 11),
              (50, 60, 70, 80))
    J = Jobs()
    for sci, sc in enumerate(scores):
        for band in (10, 60, 150, 190, 230):
            m = int(rng.integers(200, 3000))
            p, t = R.rand_pair(m, int(rng.integers(2, 20)), int(rng.integers(1, 2 ** 62)))
            J.add(None, p=p, t=t, kind=1, mode=R.GLOBAL, band=band, want_cigar=1, sc_index=sci)
            J.add(None, p=p, t=t, kind=2, band=band, window=len(t) + 30,
                  xdrop=int(rng.integers(5, 400)), end_bonus=3, want_cigar=1, sc_index=sci)
    out, kinds = J.run(ctx, scores)
    assert any(k == "affine16" for k, _ in kinds) and any(k == "affine" for k, _ in kinds)
    _check(J, out, scores)


def test_sorted_cut_bookkeeping(ctx):
    """Cut maxima, bonus placement and X-drop stops (row bookkeeping in field arithmetic)
    through the sorted-texts entry points, on texts long enough to rebase."""
    gpu = R.GpuImpl()
    rng = np.random.default_rng(1604)
    for _ in range(6):
        base = rng.integers(0, 4, int(rng.integers(200, 1500))).tolist()
        p = R.mutate(base, R.rand_edits(rng, int(rng.integers(0, 60)), len(base)))
        variants = [(int(rng.integers(0, len(base))),
                     rng.integers(0, 4, int(rng.integers(0, 80))).tolist(),
                     int(rng.integers(0, 200))) for _ in range(int(rng.integers(1, 6)))]
        texts = R.sorted_texts(base, variants)
        band, xd, bonus = int(rng.integers(8, 120)), int(rng.integers(20, 300)), int(rng.integers(0, 8))
        w = max(len(t) for t in texts) + 40
        c = min(len(t) for t in texts) - int(rng.integers(0, 100))
        for sc in (R.ONT, R.HIFI):
            for args in ((bonus, xd, False, w, None, True, False),
                         (bonus, R.I32_MAX, False, w, max(c, 0), True, False),
                         (bonus, xd, False, w, max(c, 0), True, True),
                         (bonus, xd, True, w, max(c, 0), False, True)):
                got = gpu.affine_extend_sorted_cut_bonus(p, texts, sc, band, *args)
                want = O.affine_extend_sorted_cut_bonus(p, texts, sc, band, *args)
                assert got == want, args


def test_half_warp_passes(ctx):
    """Two passes per warp (16 lanes each): every half-warp class, passes of uneven lengths
    paired in one warp, Global and Prefix with CIGARs, X-drop and bonuses -- identical to the
    one-pass-per-warp kernel and to the oracle."""
    rng = np.random.default_rng(1605)
    J = Jobs()
    for band in (2, 30, 55, 70, 90, 110, 120, 130, 150, 170):
        for rep in range(4):
            m = int(rng.integers(max(20, 2 * band), 2 * band + 1500))
            p, t = R.rand_pair(m, int(rng.integers(3, 15)), int(rng.integers(1, 2 ** 62)))
            mode = R.GLOBAL if rep % 2 == 0 else R.PREFIX
            sci = int(rng.integers(0, 2))
            J.add(None, p=p, t=t, kind=1, mode=mode, band=band, want_cigar=rep % 3 != 2,
                  sc_index=sci)
            w = len(t) + int(rng.integers(0, 100))
            xd = int(rng.integers(10, 200)) if rng.random() < 0.7 else R.I32_MAX
            J.add(None, p=p, t=t, kind=2, band=band, window=w, xdrop=xd,
                  end_bonus=int(rng.integers(0, 9)), want_cigar=rep % 2, sc_index=sci)
    for m in (0, 1, 5):  # short and empty patterns among long ones
        p, t = R.rand_pair(m, 5, int(rng.integers(1, 2 ** 62)))
        J.add(None, p=p, t=t, kind=1, mode=R.GLOBAL, band=40, want_cigar=1)
    scores = (R.ONT, R.HIFI)
    out, kinds = J.run(ctx, scores, lanes=16)
    half = {c for k, c in kinds if k == "affine16h"}
    assert half >= {8, 10, 12, 16, 20, 24}, sorted(half)
    _check(J, out, scores)
    out32, _ = J.run(ctx, scores, lanes=32)
    _same(out, out32)


def test_two_warp_passes(ctx):
    """Two warps per pass (64 lanes): every two-warp class, with every 16-bit pass routed to
    them (SF_AFFINE16_LANES=64) -- short and empty passes, passes whose band starts at column
    0 for many rows, Global and Prefix with CIGARs, X-drop stops, clip cells and end bonuses --
    identical to one warp per pass and to the oracle."""
    rng = np.random.default_rng(1606)
    J = Jobs()
    for band in (3, 40, 150, 300, 380, 420, 500, 620, 700, 820, 900, 1000):
        for rep in range(3):
            m = int(rng.integers(max(20, band // 2), 2 * band + 1500))
            p, t = R.rand_pair(m, int(rng.integers(3, 15)), int(rng.integers(1, 2 ** 62)))
            mode = R.GLOBAL if rep != 1 else R.PREFIX
            sci = int(rng.integers(0, 2))
            J.add(None, p=p, t=t, kind=1, mode=mode, band=band, want_cigar=rep != 2,
                  sc_index=sci)
            w = len(t) + int(rng.integers(0, 100))
            xd = int(rng.integers(10, 200)) if rng.random() < 0.7 else R.I32_MAX
            J.add(None, p=p, t=t, kind=2, band=band, window=w, xdrop=xd,
                  end_bonus=int(rng.integers(0, 9)), want_cigar=rep % 2, sc_index=sci)
    for m in (0, 1, 5, 70):  # short and empty patterns among long ones
        p, t = R.rand_pair(m, 5, int(rng.integers(1, 2 ** 62)))
        J.add(None, p=p, t=t, kind=1, mode=R.GLOBAL, band=600, want_cigar=1)
    # Substitutions only (m = n): rows of exactly 2 * band + 1 cells, one band per class
    # (64 lanes x 12, 16, 20, 24, 28, 32 cells).
    for band in (300, 450, 600, 700, 830, 950):
        p = rng.integers(0, 4, 2 * band + 900)
        t = p.copy()
        hit = rng.random(t.size) < 0.08
        t[hit] = (t[hit] + 1) & 3
        J.add(None, p=p.tolist(), t=t.tolist(), kind=1, mode=R.GLOBAL, band=band,
              want_cigar=1)
    # A long pass of 12 kb whose maximum wanders (rebases on both warps).
    q = rng.integers(0, 4, 12000).tolist()
    t = R.mutate(q, R.rand_edits(rng, 1200, 12000))
    J.add(None, p=q, t=t, kind=1, mode=R.GLOBAL, band=560, want_cigar=1)
    J.add(None, p=q, t=t, kind=2, band=560, window=len(t) + 40, xdrop=150, end_bonus=5,
          want_cigar=1)
    scores = (R.ONT, R.HIFI)
    out, kinds = J.run(ctx, scores, lanes=64)
    two = {c for k, c in kinds if k == "affine16w"}
    assert two >= {12, 16, 20, 24, 28, 32}, sorted(kinds)
    assert not any(k == "affine16" for k, _ in kinds), sorted(kinds)
    _check(J, out, scores)
    out32, kinds32 = J.run(ctx, scores, lanes=32, w64=False)
    assert not any(k == "affine16w" for k, _ in kinds32)
    _same(out, out32)


def test_two_warp_sorted_cut(ctx):
    """Cut maxima (both warps' row maxima up to the cut), bonuses and X-drop through the
    sorted-texts entry points on two-warp passes."""
    gpu = R.GpuImpl()
    rng = np.random.default_rng(1607)
    old = os.environ.get("SF_AFFINE16_LANES")
    os.environ["SF_AFFINE16_LANES"] = "64"
    try:
        for _ in range(4):
            base = rng.integers(0, 4, int(rng.integers(800, 2500))).tolist()
            p = R.mutate(base, R.rand_edits(rng, int(rng.integers(0, 80)), len(base)))
            variants = [(int(rng.integers(0, len(base))),
                         rng.integers(0, 4, int(rng.integers(0, 80))).tolist(),
                         int(rng.integers(0, 200))) for _ in range(int(rng.integers(1, 5)))]
            texts = R.sorted_texts(base, variants)
            band, xd, bonus = int(rng.integers(200, 700)), int(rng.integers(20, 300)), \
                int(rng.integers(0, 8))
            w = max(len(t) for t in texts) + 40
            c = min(len(t) for t in texts) - int(rng.integers(0, 100))
            for args in ((bonus, xd, False, w, None, True, False),
                         (bonus, xd, False, w, max(c, 0), True, True),
                         (bonus, xd, True, w, max(c, 0), False, True)):
                got = gpu.affine_extend_sorted_cut_bonus(p, texts, R.ONT, band, *args)
                want = O.affine_extend_sorted_cut_bonus(p, texts, R.ONT, band, *args)
                assert got == want, args
    finally:
        if old is None:
            del os.environ["SF_AFFINE16_LANES"]
        else:
            os.environ["SF_AFFINE16_LANES"] = old
