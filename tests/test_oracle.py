"""Pins the CPU oracle to the reference: its known-answer tests, its saved proptest
regressions and its property tests (the naive definitions of align.rs:2801-3014), on
seeded random inputs."""
import numpy as np
import pytest

import oracle as O
import refcases as R

IMPL = R.OracleImpl()


def test_kats():
    R.check_kats(IMPL)


def test_extend_kat_equals_naive():
    # align.rs:3118-3129
    for c in R.golden()["kats"]:
        if c["fn"] == "affine_extend_vs_naive":
            a = c["args"]
            assert O.affine_extend(a["p"], a["t"], a["sc"], a["band"], a["end_bonus"],
                                   a["xdrop"]) == O.naive_extend(a["p"], a["t"], a["sc"])


def test_window_relations():
    R.check_window_relations(IMPL)


def _check_myers(p, t, k):
    # align.rs:2899-2906 `check`
    for mode in (R.INFIX, R.PREFIX, R.GLOBAL):
        want = O.myers_naive(p, t, mode)
        got = O.myers_distance(p, t, mode, k)
        assert got == (want if want <= k else None), (mode, k, len(p), len(t))


def test_regressions():
    for c in R.golden()["regressions"]:
        a = c["args"]
        if c["test"] == "random_vs_naive":
            _check_myers(a["p"], a["t"], a["k"])
        elif c["test"] == "related_vs_naive":
            t = a["t"]
            end = min(a["a"] + a["len"], len(t))
            p = R.mutate(t[min(a["a"], end):end], a["edits"])
            d = O.myers_naive(p, t, R.INFIX)
            for k in (max(d - 1, 0), d, d + a["slack"], R.U32_MAX):
                _check_myers(p, t, k)
        elif c["test"] == "local_band_matches_definition":
            b = a["bonus"] if isinstance(a["bonus"], list) else [a["bonus"], a["bonus"]]
            for sc in (R.ONT, R.HIFI):
                m, n = len(a["p"]), len(a["t"])
                assert O.local_band_ends(a["p"], a["t"], sc, -m, n, b) == \
                    O.naive_local(a["p"], a["t"], sc, b)


def test_myers_random_vs_naive():
    rng = np.random.default_rng(11)
    for _ in range(150):
        p = rng.integers(0, 4, int(rng.integers(0, 300))).tolist()
        t = rng.integers(0, 4, int(rng.integers(0, 300))).tolist()
        k = R.U32_MAX if rng.random() < 0.3 else int(rng.integers(0, 400))
        _check_myers(p, t, k)


def test_myers_related_vs_naive():
    rng = np.random.default_rng(12)
    for _ in range(60):
        p, t = R.related(rng)
        d = O.myers_naive(p, t, R.INFIX)
        for k in (max(d - 1, 0), d, d + int(rng.integers(0, 20)), R.U32_MAX):
            _check_myers(p, t, k)


def test_batch_lanes_match_single():
    # align.rs:3376-3432: lockstep lanes of any width equal one call per text.
    rng = np.random.default_rng(13)
    for _ in range(25):
        base = rng.integers(0, 4, int(rng.integers(0, 700))).tolist()
        pa, pl = int(rng.integers(0, 300)), int(rng.integers(0, 500))
        end = min(pa + pl, len(base))
        p = R.mutate(base[min(pa, end):end], R.rand_edits(rng, int(rng.integers(0, 40)), 700))
        rnd = rng.integers(0, 4, int(rng.integers(0, 300))).tolist()
        texts = []
        for _ in range(int(rng.integers(1, 20))):
            a, ln = int(rng.integers(0, 700)), int(rng.integers(0, 700))
            if rng.random() < 0.5:
                texts.append(rnd[:min(ln, len(rnd))])
            else:
                e = min(a + ln, len(base))
                texts.append(R.mutate(base[min(a, e):e],
                                      R.rand_edits(rng, int(rng.integers(0, 25)), 700)))
        for mode in (R.INFIX, R.PREFIX, R.GLOBAL):
            exact = [O.myers_distance(p, t, mode) for t in texts]
            k = R.U32_MAX if rng.random() < 0.4 else min(exact) + int(rng.integers(0, 60))
            want = [O.myers_distance(p, t, mode, k) for t in texts]
            if p:
                for L in (1, 2, 4, 8):
                    assert O.myers_batch_lanes(p, texts, mode, k, L) == want, (mode, L)


def test_affine_vs_naive():
    # align.rs:3311-3340
    rng = np.random.default_rng(14)
    sc = R.ONT
    for _ in range(80):
        p, t = R.affine_case(rng)
        for mode in (R.GLOBAL, R.PREFIX, R.INFIX):
            want = O.naive_affine(p, t, mode, sc)
            assert O.affine(p, t, mode, sc, None) == want
            assert O.affine(p, t, mode, sc, 8) <= want
            assert O.affine(p, t, mode, sc, 400) == want
        if len(p) <= 40 and len(t) <= 60:
            assert O.affine_extend(p, t, sc, None, 0, R.I32_MAX) == O.naive_extend(p, t, sc)


def test_local_band_definition_and_matrix():
    # align.rs:3047-3116
    rng = np.random.default_rng(15)
    for _ in range(120):
        p = rng.integers(0, 4, int(rng.integers(0, 8))).tolist()
        t = rng.integers(0, 4, int(rng.integers(0, 8))).tolist()
        b = (int(rng.integers(0, 8)), int(rng.integers(0, 8)))
        for sc in (R.ONT, R.HIFI):
            m, n = len(p), len(t)
            assert O.local_band_ends(p, t, sc, -m, n, b) == O.naive_local(p, t, sc, b)
            assert O.local_band(p, t, sc, -m, n, b[0]) == O.local_band_ends(p, t, sc, -m, n,
                                                                            (b[0], b[0]))
    for _ in range(150):
        base = rng.integers(0, 4, int(rng.integers(1, 60))).tolist()
        c0, c1 = int(rng.integers(0, 60)), int(rng.integers(0, 60))
        p = base[c0 % len(base):]
        p = p[:max(0, len(p) - c1 % 20)]
        p = R.mutate(p, R.rand_edits(rng, int(rng.integers(0, 10)), 60))
        dlo, width = int(rng.integers(-70, 70)), int(rng.integers(0, 40))
        b = (int(rng.integers(0, 8)), int(rng.integers(0, 8)))
        for sc in (R.ONT, R.HIFI):
            got = O.local_band_ends(p, base, sc, dlo, dlo + width, b)
            assert got == O.naive_local_band(p, base, sc, dlo, dlo + width, b)
            assert got <= O.local_band_ends(p, base, sc, dlo - 3, dlo + width + 5, b)


def test_local_band_wide_with_ambiguous_bases():
    # align.rs:3080-3115 `local_band_matches_matrix_wide`
    rng = np.random.default_rng(16)
    for _ in range(25):
        base = rng.integers(0, 4, int(rng.integers(1, 300))).tolist()
        c0, c1 = int(rng.integers(0, 300)), int(rng.integers(0, 100))
        p = base[c0 % len(base):]
        p = p[:max(0, len(p) - c1)]
        p = R.mutate(p, R.rand_edits(rng, int(rng.integers(0, 30)), 300, base_max=5))
        j0 = rng.integers(0, 4, int(rng.integers(0, 30))).tolist()
        j1 = rng.integers(0, 4, int(rng.integers(0, 30))).tolist()
        p = j0 + p + j1
        dlo, width = int(rng.integers(-320, 320)), int(rng.integers(0, 200))
        b = (int(rng.integers(0, 8)), int(rng.integers(0, 8)))
        for sc in (R.ONT, R.HIFI):
            assert O.local_band_ends(p, base, sc, dlo, dlo + width, b) == \
                O.naive_local_band(p, base, sc, dlo, dlo + width, b)


@pytest.mark.parametrize("kind", ["affine", "extend"])
def test_traceback_rescores(kind):
    """The traceback oracle's CIGAR re-scores to the pass's score, ends at its end cell
    and spans the pattern (no reference counterpart: CIGARs are new)."""
    rng = np.random.default_rng(17 if kind == "affine" else 18)
    for it in range(120):
        p, t = R.rand_pair(int(rng.integers(1, 400)), int(rng.integers(3, 20)),
                           int(rng.integers(1, 2 ** 63)))
        if rng.random() < 0.2:
            p = p + rng.integers(0, 4, int(rng.integers(0, 40))).tolist()
        sc = R.ONT if it % 2 == 0 else R.HIFI
        band = [None, 8, 16, 64][it % 4]
        if kind == "affine":
            for mode in (R.GLOBAL, R.PREFIX, R.INFIX):
                tb = O.traceback(p, t, O.TB_AFFINE, mode, sc, band)
                assert tb["score"] == O.affine(p, t, mode, sc, band)
                if tb["status"] == 1:
                    continue
                assert tb["status"] == 0
                s, pu, te = O.cigar_score(p, t, tb["cigar"], tb["text_start"], sc)
                assert (s, pu, te) == (tb["score"], len(p), tb["end_j"]), (mode, band)
        else:
            w = len(t) + int(rng.integers(0, 40))
            xd = int(rng.integers(5, 80))
            bonus = int(rng.integers(0, 8))
            tb = O.traceback(p, t, O.TB_EXTEND, O.PREFIX, sc, band, w, bonus, xd)
            want = O.affine_extend_window(p, t, w, sc, band, bonus, xd)
            assert (tb["score"], tb["end_i"], tb["end_j"]) == want[:3]
            assert tb["status"] == 0
            s, pu, te = O.cigar_score(p, t, tb["cigar"], tb["text_start"], sc)
            whole = tb["end_i"] == len(p) and not any((c & 15) == O.OP_S for c in tb["cigar"])
            assert s + (bonus if whole and tb["score"] != s else 0) == tb["score"]
            assert (pu, te) == (len(p), tb["end_j"])


def test_run_pairs_matches_single():
    rng = np.random.default_rng(19)
    ps = [rng.integers(0, 4, int(rng.integers(0, 300))).astype(np.uint8) for _ in range(40)]
    ts = [rng.integers(0, 4, int(rng.integers(0, 300))).astype(np.uint8) for _ in range(40)]

    def cat(xs):
        lens = np.array([len(x) for x in xs], dtype=np.uint64)
        offs = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.uint64)
        return np.concatenate(xs), offs, lens

    pc, po, pl = cat(ps)
    tc, to, tl = cat(ts)
    out, cells = O.run_pairs(0, 4, pc, po, pl, tc, to, tl, R.INFIX)
    assert [int(x) for x in out] == [O.myers_distance(p, t, R.INFIX) for p, t in zip(ps, ts)]
    out, cells = O.run_pairs(1, 3, pc, po, pl, tc, to, tl, R.GLOBAL, sc=R.ONT, band=16)
    assert [int(x) for x in out] == [O.affine(p, t, R.GLOBAL, R.ONT, 16) for p, t in zip(ps, ts)]
    assert cells == sum(O.affine_dp(p, t, R.GLOBAL, R.ONT, 16)["cells"] for p, t in zip(ps, ts))
    # Per-pair caps (Myers) and windowed extensions (the window rule x + 20 + x / 10).
    kv = rng.integers(0, 200, len(ps)).astype(np.uint32)
    out, _ = O.run_pairs(0, 2, pc, po, pl, tc, to, tl, R.PREFIX, kv=kv)
    want = [O.myers_distance(p, t, R.PREFIX, int(k)) for p, t, k in zip(ps, ts, kv)]
    assert [None if int(x) < 0 else int(x) for x in out] == want
    out, cells = O.run_pairs(2, 3, pc, po, pl, tc, to, tl, R.PREFIX, sc=R.ONT, band=16,
                             extend=(20, 10, 50, 5))
    win = [len(p) + 20 + len(p) // 10 for p in ps]
    assert [int(x) for x in out] == [O.affine_extend_window(p, t, w, R.ONT, 16, 5, 50)[0]
                                     for p, t, w in zip(ps, ts, win)]
    assert cells == sum(O.affine_dp(p, t, R.PREFIX, R.ONT, 16, geom=max(w, len(t)),
                                    clip=(50, True))["cells"] for p, t, w in zip(ps, ts, win))
    # A band per pair, and each pair's cells.
    bands = rng.integers(0, 40, len(ps)).astype(np.uint64)
    out, cpp = O.run_pairs(1, 3, pc, po, pl, tc, to, tl, R.GLOBAL, sc=R.ONT, bands=bands,
                           per_pair_cells=True)
    assert [int(x) for x in out] == [O.affine(p, t, R.GLOBAL, R.ONT, int(b))
                                     for p, t, b in zip(ps, ts, bands)]
    assert [int(c) for c in cpp] == [O.affine_dp(p, t, R.GLOBAL, R.ONT, int(b))["cells"]
                                     for p, t, b in zip(ps, ts, bands)]


def test_check_cigars_batch():
    """The batch CIGAR checker passes the oracle's own tracebacks and flags planted faults
    (a changed op, a wrong score, a wrong text end, a truncated path)."""
    rng = np.random.default_rng(23)
    ps, ts, cig, offs, nops, starts, ends, scores = [], [], [], [], [], [], [], []
    at = 0
    for _ in range(30):
        p, t = R.rand_pair(int(rng.integers(20, 400)), int(rng.integers(3, 15)),
                           int(rng.integers(1, 2 ** 62)))
        tb = O.traceback(p, t, O.TB_AFFINE, R.GLOBAL, R.ONT, 32)
        assert tb["status"] == 0
        ps.append(np.asarray(p, np.uint8))
        ts.append(np.asarray(t, np.uint8))
        cig.append(np.asarray(tb["cigar"], np.uint32))
        offs.append(at)
        at += len(tb["cigar"])
        nops.append(len(tb["cigar"]))
        starts.append(tb["text_start"])
        ends.append(tb["end_j"])
        scores.append(tb["score"])

    def cat(xs):
        lens = np.array([len(x) for x in xs], dtype=np.uint64)
        o = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.uint64)
        return np.concatenate(xs), o, lens

    pc, po, pl = cat(ps)
    tc, to, tl = cat(ts)
    ops = np.concatenate(cig)
    args = [np.array(offs, np.uint64), np.array(nops, np.uint32), np.array(starts, np.uint64),
            np.array(ends, np.uint64), np.array(scores, np.int32)]
    code = O.check_cigars(3, pc, po, pl, tc, to, tl, ops, *args, sc=R.ONT)
    assert (code == 0).all()
    bad_score = args[4].copy()
    bad_score[3] += 1
    assert list(np.flatnonzero(O.check_cigars(2, pc, po, pl, tc, to, tl, ops, *args[:4],
                                              bad_score, sc=R.ONT))) == [3]
    bad_end = args[3].copy()
    bad_end[5] += 1
    code = O.check_cigars(2, pc, po, pl, tc, to, tl, ops, *args[:3], bad_end, args[4],
                          sc=R.ONT)
    assert list(np.flatnonzero(code)) == [5] and code[5] == 3
    short = args[1].copy()
    short[7] -= 1
    code = O.check_cigars(2, pc, po, pl, tc, to, tl, ops, args[0], short, *args[2:], sc=R.ONT)
    assert code[7] != 0 and (np.delete(code, 7) == 0).all()
    bad_op = ops.copy()
    bad_op[offs[9]] = (bad_op[offs[9]] & ~np.uint32(15)) | 7  # an unknown op
    code = O.check_cigars(2, pc, po, pl, tc, to, tl, bad_op, *args, sc=R.ONT)
    assert code[9] == 4 and (np.delete(code, 9) == 0).all()
