"""Sorted-text row sharing (align.rs:2210-2315 `affine_dp_sorted`) on the GPU.  With
SF_SORTED_CHAINS=1 the passes of a sorted call run as chains, one warp each, every pass
resuming from a row snapshot of an earlier one where the texts share the bases those rows
read, or taking the previous result outright; by default every pass runs separately.  Either
way the results equal the oracle's separate passes text by text, and the DP work counted
(align.rs:2571-2576) equals the reference driver's on the same inputs -- rows a pass resumes
past and passes it copies are not counted -- with the driver restated below over the
oracle's per-pass results.  Texts are isoform-like: variants of one transcript that differ
after long shared prefixes (other 3' ends, skipped exons, point changes), sorted and
distinct."""
import numpy as np
import pytest

import oracle as O
import refcases as R
from spearfish_gb300 import align as A
from spearfish_gb300 import tiebreak as T

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["1", "0"], ids=["chains", "separate"])
def chains(request, monkeypatch):
    """SF_SORTED_CHAINS=1 runs the passes that can share rows as chains; otherwise (the
    default) every pass runs separately."""
    monkeypatch.setenv("SF_SORTED_CHAINS", request.param)
    return request.param


@pytest.fixture(scope="module")
def ctx():
    from spearfish_gb300 import build
    build.build()
    from spearfish_gb300 import batch as B
    c = B.Context(0)
    yield c
    c.close()


def band_cells(rows, below, above, n):
    """DP_WORK cells of rows 1 .. rows (align.rs:2571-2576)."""
    tot = 0
    for i in range(1, rows + 1):
        lo, hi = max(0, i - below), min(i + above, n)
        if lo <= hi:
            tot += hi - lo + 1
    return tot


def lcp(a, b):
    n = 0
    for x, y in zip(a, b):
        if x != y:
            break
        n += 1
    return n


def driver(p, texts, mode, sc, band, clip, geom, cut):
    """align.rs:2215-2315 over the oracle's passes: per text its Dp, and the (cells, rows)
    the reference's DP_WORK counts for the whole call."""
    m = len(p)

    def shape(n):
        g = geom(n)
        return band + max(m - g, 0), band + max(g - m, 0)

    full = mode == R.INFIX or band is None
    resume = []
    for k, t in enumerate(texts):
        if k == 0 or full or shape(len(t)) != shape(len(texts[k - 1])):
            resume.append(0)
            continue
        resume.append(min(max(lcp(t, texts[k - 1]) - shape(len(t))[1], 0), max(m - 1, 0)))
    out, cells, rows = [], 0, 0
    for k, t in enumerate(texts):
        r = resume[k]
        if k > 0 and clip is not None and not full:
            pv, tr = texts[k - 1], out[k - 1]["text_read"]
            if (shape(len(t)) == shape(len(pv)) and tr < len(pv) and tr < len(t)
                    and list(t[:tr]) == list(pv[:tr])):
                out.append(out[k - 1])
                continue
        if r > 0 and out[k - 1]["last_row"] <= r:
            out.append(out[k - 1])
            continue
        d = O.affine_dp(p, t, mode, sc, band, geom=geom(len(t)), clip=clip, cut=cut)
        below, above = shape(len(t))
        last = min(d["last_row"], len(t) + below)  # a row past the text's end is not counted
        cells += band_cells(last, below, above, len(t)) - band_cells(r, below, above, len(t))
        rows += last - r
        out.append(d)
    return out, cells, rows


def isoforms(rng, length, count):
    """Sorted distinct variants of one random transcript."""
    base = rng.integers(0, 4, length).tolist()
    texts = [base]
    for _ in range(count):
        kind = int(rng.integers(0, 4))
        v = list(base)
        a = int(rng.integers(length // 8, length))
        if kind == 0:  # another 3' end
            v = v[:a] + rng.integers(0, 4, int(rng.integers(0, 400))).tolist()
        elif kind == 1:  # a skipped exon
            v = v[:a] + v[min(length, a + int(rng.integers(20, 300))):]
        elif kind == 2:  # a point change
            v[a] = (v[a] + 1) % 4
        else:  # shorter at the 3' end
            v = v[:a]
        texts.append(v)
    return [list(x) for x in sorted({tuple(x) for x in texts})]


def read_of(rng, texts, m, errors):
    t = texts[int(rng.integers(0, len(texts)))]
    return R.mutate(t[:m], R.rand_edits(rng, errors, m))


def _work():
    return A.dp_work()


def _extend_case(rng, texts, p):
    band = int(rng.integers(4, 90))
    xd = int(rng.integers(15, 250)) if rng.random() < 0.8 else R.I32_MAX
    bonus = int(rng.integers(0, 8))
    diag = bool(rng.random() < 0.3)
    w = max(len(t) for t in texts) + int(rng.integers(0, 60))
    cut = None if rng.random() < 0.4 else int(rng.integers(0, min(len(t) for t in texts) + 1))
    track = bool(rng.random() < 0.7)
    within = bool(rng.random() < 0.5)
    return band, bonus, xd, diag, w, cut, track, within


def test_sorted_chains_equal_separate_passes(ctx, chains):
    rng = np.random.default_rng(2210)
    shared_rows = 0
    for trial in range(24):
        texts = isoforms(rng, int(rng.integers(300, 2500)), int(rng.integers(1, 9)))
        m = int(rng.integers(50, 1500))
        p = read_of(rng, texts, m, int(rng.integers(0, m // 10 + 1)))
        for sc in (R.ONT, R.HIFI):
            band, bonus, xd, diag, w, cut, track, within = _extend_case(rng, texts, p)
            c0, r0 = _work()
            got = A.affine_extend_sorted_cut_bonus(p, texts, sc, band, bonus, xd, diag, w, cut,
                                                   track, within)
            c1, r1 = _work()
            want = O.affine_extend_sorted_cut_bonus(p, texts, sc, band, bonus, xd, diag, w, cut,
                                                    track, within)
            assert got == want, (trial, sc)
            mm = len(p)
            geom = (lambda n: min(mm, n)) if diag else (lambda n: max(n, w))
            _, cells, rows = driver(p, texts, R.PREFIX, sc, band, (xd, track and cut is not None),
                                    geom, cut)
            assert (c1 - c0, r1 - r0) == (cells, rows), (trial, sc)
            alone = sum(O.affine_dp(p, t, R.PREFIX, sc, band, geom=geom(len(t)),
                                    clip=(xd, track and cut is not None), cut=cut)["last_row"]
                        for t in texts)
            shared_rows += max(0, alone - rows)
            for mode in (R.GLOBAL, R.PREFIX):
                c0, r0 = _work()
                got = A.affine_sorted(p, texts, mode, sc, band)
                c1, r1 = _work()
                assert got == O.affine_sorted(p, texts, mode, sc, band), (trial, mode)
                _, cells, rows = driver(p, texts, mode, sc, band, None, lambda n: n, None)
                assert (c1 - c0, r1 - r0) == (cells, rows), (trial, mode)
    assert shared_rows > 0  # the chains did resume


def test_chains_off_same_results_and_work(ctx, monkeypatch):
    """SF_SORTED_CHAINS=0 runs the same calls as separate passes: the same results, and the
    same DP work counted (the reference's, replayed from the results)."""
    rng = np.random.default_rng(2211)
    for trial in range(4):
        texts = isoforms(rng, 1200, 6)
        p = read_of(rng, texts, 600, 20)
        got = {}
        for flag in ("0", "1"):
            monkeypatch.setenv("SF_SORTED_CHAINS", flag)
            c0, r0 = _work()
            a = A.affine_sorted(p, texts, R.GLOBAL, R.ONT, 40)
            b = A.affine_extend_sorted_cut_bonus(p, texts, R.ONT, 40, 5, 50, False,
                                                 len(p) + 80, None, True, False)
            c1, r1 = _work()
            got[flag] = (a, b, c1 - c0, r1 - r0)
        assert got["0"] == got["1"]
        assert got["0"][0] == O.affine_sorted(p, texts, R.GLOBAL, R.ONT, 40)
        _, c_a, r_a = driver(p, texts, R.GLOBAL, R.ONT, 40, None, lambda n: n, None)
        w = len(p) + 80
        _, c_b, r_b = driver(p, texts, R.PREFIX, R.ONT, 40, (50, False), lambda n: max(n, w), None)
        assert got["0"][2:] == (c_a + c_b, r_a + r_b)


def test_deep_shared_prefixes(ctx, chains):
    """Calls whose texts share most of their length with each other: passes resume deep
    into the rows of earlier ones, with resume rows rising and falling along the sorted
    order (snapshots saved by passes several texts back)."""
    rng = np.random.default_rng(2213)
    for trial in range(6):
        base = rng.integers(0, 4, 3000).tolist()
        texts = [base]
        for _ in range(10):
            a = int(rng.integers(1500, 2990))
            v = list(base)
            v[a] = (v[a] + 1 + int(rng.integers(0, 3))) % 4
            texts.append(v)
        texts = [list(x) for x in sorted({tuple(x) for x in texts})]
        p = R.mutate(base[:2800], R.rand_edits(rng, 60, 2800))
        for band in (16, 60):
            c0, r0 = _work()
            got = A.affine_sorted(p, texts, R.GLOBAL, R.ONT, band)
            c1, r1 = _work()
            assert got == O.affine_sorted(p, texts, R.GLOBAL, R.ONT, band), (trial, band)
            _, cells, rows = driver(p, texts, R.GLOBAL, R.ONT, band, None, lambda n: n, None)
            assert (c1 - c0, r1 - r0) == (cells, rows)


def test_sorted_batch_many_chains(ctx, chains):
    """Many segments' sorted calls in one batch (one chain kernel launch, a snapshot arena
    slice per chain), chains of both entry points and both scorings side by side."""
    rng = np.random.default_rng(2212)
    calls, want = [], []
    for q in range(160):
        texts = isoforms(rng, int(rng.integers(200, 1800)), int(rng.integers(0, 10)))
        m = int(rng.integers(30, 900))
        p = read_of(rng, texts, m, int(rng.integers(0, m // 12 + 1)))
        sci = int(rng.integers(0, 2))
        sc = (R.ONT, R.HIFI)[sci]
        if q % 3 == 0:
            mode = (R.GLOBAL, R.PREFIX)[q % 2]
            band = int(rng.integers(2, 120))
            calls.append(dict(kind=T.SORTED_AFFINE, read=p, texts=texts, mode=mode, band=band,
                              sc_index=sci))
            want.append([(x, x, 0) for x in O.affine_sorted(p, texts, mode, sc, band)])
        else:
            band, bonus, xd, diag, w, cut, track, within = _extend_case(rng, texts, p)
            calls.append(dict(kind=T.SORTED_EXTEND_CUT, read=p, texts=texts, band=band,
                              end_bonus=bonus, xdrop=xd, diagonal=diag, window=w, cut=cut,
                              track_cut=track, bonus_within_cut=within, sc_index=sci))
            want.append(O.affine_extend_sorted_cut_bonus(p, texts, sc, band, bonus, xd, diag, w,
                                                         cut, track, within))
    got = T.sorted_batch(ctx, calls, scores=(R.ONT, R.HIFI))
    assert got == want
