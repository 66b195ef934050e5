"""Tie-break batching (sf_banded, sf_banded_batch) against the sequential definition of
`Mapper::banded` (map/src/lib.rs:3008-3034 `sequential`), replaying the reference's property
test `banded_matches_sequential` (lib.rs:3058-3118) on seeded inputs: texts are mutated
excerpts of the read's source, some empty or unrelated, with repeats; caps range from 0 to
near u32::MAX (where k saturates); every mode; with and without `distinct`."""
import numpy as np
import pytest

import oracle as O
import refcases as R

pytestmark = pytest.mark.gpu

U32 = 0xFFFFFFFF


def sat(a, b):
    return min(a + b, U32)


def sequential(read, texts, mode, cap):
    """lib.rs:3016-3034, with the oracle's distance_with."""
    seen, best, out = {}, U32, []
    for t in texts:
        key = tuple(t)
        k = sat(best, cap)
        if key in seen:
            d = seen[key]
            out.append(d if d <= k else sat(k, 1))
            continue
        d = O.myers_distance(read, t, mode, k)
        d = sat(k, 1) if d is None else d
        best = min(best, d)
        seen[key] = d
        out.append(d)
    return out


def mutate(s, edits):
    """lib.rs:3036-3056: substitutions (0), insertions (1), deletions (2) at positions
    taken modulo the length."""
    v = list(s)
    for pos, b, kind in edits:
        if not v:
            if kind == 1:
                v.append(b)
            continue
        i = pos % len(v)
        if kind == 0:
            v[i] = b
        elif kind == 1:
            v.insert(i, b)
        else:
            del v[i]
    return v


def case(rng):
    base = rng.integers(0, 4, int(rng.integers(0, 300))).tolist()
    edits = lambda n: [(int(rng.integers(0, 300)), int(rng.integers(0, 4)), int(rng.integers(0, 3)))
                       for _ in range(n)]
    read = mutate(base, edits(int(rng.integers(0, 30))))
    texts = []
    for _ in range(int(rng.integers(1, 24))):
        ed = edits(int(rng.integers(0, 40)))
        a, b = int(rng.integers(0, 40)), int(rng.integers(0, 40))
        if rng.random() < 0.5:
            texts.append([e[1] for e in ed])  # unrelated
        else:
            t = mutate(base, ed)
            lo = min(a, len(t))
            hi = max(len(t) - b, lo)
            texts.append(t[lo:hi])
    for _ in range(int(rng.integers(0, 8))):
        f, to = int(rng.integers(0, 64)), int(rng.integers(0, 64))
        texts.insert(to % (len(texts) + 1), list(texts[f % len(texts)]))
    once, uniq = set(), []
    for t in texts:
        if tuple(t) not in once:
            once.add(tuple(t))
            uniq.append(t)
    r = rng.random()
    cap = int(rng.integers(0, 6)) if r < 0.34 else (int(rng.integers(6, 40)) if r < 0.67
                                                    else int(rng.integers(U32 - 3, U32 + 1)))
    return read, texts, uniq, cap


def test_banded_matches_sequential():
    from spearfish_gb300 import build
    build.build()
    from spearfish_gb300 import batch as B, tiebreak as T
    rng = np.random.default_rng(1801)
    batch, want = [], []
    for _ in range(64):
        read, texts, uniq, cap = case(rng)
        for mode in (R.GLOBAL, R.PREFIX, R.INFIX):
            w = sequential(read, texts, mode, cap)
            wu = sequential(read, uniq, mode, cap)
            assert T.banded(read, texts, mode, cap, False) == w, (mode, cap)
            assert T.banded(read, uniq, mode, cap, True) == wu, (mode, cap)
            batch += [(read, texts, mode, cap, False), (read, uniq, mode, cap, True)]
            want += [w, wu]
    ctx = B.Context(0)
    try:
        got = T.banded_batch(ctx, batch)
    finally:
        ctx.close()
    assert got == want


def test_banded_batch_long_reads():
    """Reads of 1-5 kb against 1-40 candidate windows each, through one batch."""
    from spearfish_gb300 import build
    build.build()
    from spearfish_gb300 import batch as B, tiebreak as T
    rng = np.random.default_rng(1802)
    batch, want = [], []
    for _ in range(40):
        src = rng.integers(0, 4, int(rng.integers(1000, 5000))).tolist()
        read = R.mutate(src, R.rand_edits(rng, len(src) // 12, len(src)))
        texts = []
        for _ in range(int(rng.integers(1, 40))):
            t = R.mutate(src, R.rand_edits(rng, int(rng.integers(0, len(src) // 5)), len(src)))
            texts.append(t if rng.random() < 0.8 else rng.integers(0, 4, len(src)).tolist())
        if rng.random() < 0.5:
            texts.append(list(texts[0]))
        mode = int(rng.integers(0, 3))
        cap = int(rng.choice([0, 5, 50, 1000, U32]))
        batch.append((read, texts, mode, cap, False))
        want.append(sequential(read, texts, mode, cap))
    ctx = B.Context(0)
    try:
        assert T.banded_batch(ctx, batch) == want
    finally:
        ctx.close()


def test_sorted_batch_equals_sorted_calls():
    """sf_sorted_batch (many segments' sorted calls in one batch) equals the oracle's
    affine_sorted / affine_extend_sorted_cut_bonus call by call (align.rs:3245-3309
    `sorted_batch_matches_single` inputs: sorted variants of a base sequence)."""
    from spearfish_gb300 import build
    build.build()
    from spearfish_gb300 import batch as B, tiebreak as T
    rng = np.random.default_rng(1803)
    calls, want = [], []
    for _ in range(60):
        base = rng.integers(0, 4, int(rng.integers(1, 300))).tolist()
        p = R.mutate(base, R.rand_edits(rng, int(rng.integers(0, 20)), max(1, len(base))))
        variants = [(int(rng.integers(0, max(1, len(base)))),
                     rng.integers(0, 4, int(rng.integers(0, 40))).tolist(),
                     int(rng.integers(0, 60))) for _ in range(int(rng.integers(1, 8)))]
        texts = R.sorted_texts(base, variants)
        band = int(rng.integers(2, 40))
        sci = int(rng.integers(0, 2))
        sc = (R.ONT, R.HIFI)[sci]
        if rng.random() < 0.4:
            mode = int(rng.choice([R.GLOBAL, R.PREFIX]))
            calls.append({"read": p, "texts": texts, "kind": T.SORTED_AFFINE, "mode": mode,
                          "band": band, "sc_index": sci})
            want.append([(x, x, 0) for x in (O.affine(p, t, mode, sc, band) for t in texts)])
        else:
            bonus, xd = int(rng.integers(0, 8)), int(rng.integers(5, 80))
            diag = bool(rng.random() < 0.3)
            w = max(len(t) for t in texts) + int(rng.integers(0, 40))
            cut = None if rng.random() < 0.3 else int(rng.integers(0, w + 1))
            track, within = bool(rng.random() < 0.8), bool(rng.random() < 0.5)
            calls.append({"read": p, "texts": texts, "kind": T.SORTED_EXTEND_CUT, "band": band,
                          "end_bonus": bonus, "xdrop": xd, "diagonal": diag, "window": w,
                          "cut": cut, "track_cut": track, "bonus_within_cut": within,
                          "sc_index": sci})
            want.append([tuple(x) for x in O.affine_extend_sorted_cut_bonus(
                p, texts, sc, band, bonus, xd, diag, w, cut, track, within)])
    ctx = B.Context(0)
    try:
        got = T.sorted_batch(ctx, calls, scores=(R.ONT, R.HIFI))
    finally:
        ctx.close()
    assert got == want
