"""Span-end extensions in one batch (sf_extend_ends_batch) against `extend_ends`
(map/src/lib.rs:2020-2114) restated with the oracle's `affine_extend_window`: the left flank
(read prefix and transcript flank before the span, both backwards), the right flank (cut at
the transcript's end), spans touching either end, and the default `Ends` parameters
(lib.rs:235-239: band 16, X-drop 50, end bonus 5; transcript flank x + 20 + x / 10)."""
import numpy as np
import pytest

import oracle as O
import refcases as R

pytestmark = pytest.mark.gpu

ENDS = {"sc": R.ONT, "band": 16, "end_bonus": 5, "xdrop": 50, "pad": 20, "pad_div": 10}


def extend_ends(read, tx, span, e):
    window = lambda x: x + e["pad"] + x // e["pad_div"]
    qs, qe, ts, te = span
    if qs > 0 and ts > 0:
        lo = max(0, ts - window(qs))
        text = tx[lo:ts][::-1]
        rd = read[:qs][::-1]
        _, qi, tj, _ = O.affine_extend_window(rd, text, window(len(rd)), e["sc"], e["band"],
                                              e["end_bonus"], e["xdrop"])
        qs, ts = qs - qi, ts - tj
    rest = len(read) - qe
    if rest > 0 and te < len(tx):
        hi = min(te + rest + e["pad"] + rest // e["pad_div"], len(tx))
        _, qi, tj, _ = O.affine_extend_window(read[qe:], tx[te:hi], window(rest), e["sc"],
                                              e["band"], e["end_bonus"], e["xdrop"])
        qe, te = qe + qi, te + tj
    return qs, qe, ts, te


def test_extend_ends_batch_matches_restatement():
    from spearfish_gb300 import build
    build.build()
    from spearfish_gb300 import batch as B, tiebreak as T
    rng = np.random.default_rng(2001)
    txs = [rng.integers(0, 4, int(rng.integers(200, 4000)), dtype=np.uint8) for _ in range(80)]
    starts = np.concatenate([[0], np.cumsum([t.size for t in txs])[:-1]]).astype(np.uint64)
    pb = B.PoolBuilder()
    hits, want = [], []
    for q in range(400):
        x = int(rng.integers(0, len(txs)))
        tx = txs[x]
        a = int(rng.integers(0, tx.size // 2))
        b = int(rng.integers(a + 1, tx.size + 1))
        if q % 7 == 0:
            a = 0  # the read starts at the transcript's start
        if q % 11 == 0:
            b = tx.size
        read = np.array(R.mutate(tx[a:b].tolist(), R.rand_edits(rng, (b - a) // 14, b - a)),
                        dtype=np.uint8)
        if read.size < 2:
            continue
        # An anchored span inside the read's true placement.
        qs = int(rng.integers(0, read.size // 2))
        qe = int(rng.integers(qs + 1, read.size + 1))
        ts = min(tx.size, a + qs)
        te = max(ts, min(tx.size, a + qe))
        if q % 13 == 0:
            qs, ts = 0, ts  # nothing to extend on the left
        off = pb.add(read)
        hits.append((off, int(starts[x]), read.size, tx.size, qs, qe, ts, te))
        want.append(extend_ends(read.tolist(), tx.tolist(), (qs, qe, ts, te), ENDS))
    h = np.zeros(len(hits), dtype=T.HIT_DTYPE)
    for i, v in enumerate(hits):
        h[i] = v
    ctx = B.Context(0)
    store = B.Store(ctx, txs)
    try:
        ctx.use_store(store)
        got = T.extend_ends_batch(ctx, pb.build(), ENDS, h)
    finally:
        ctx.use_store(None)
        store.close()
        ctx.close()
    for i, w in enumerate(want):
        assert tuple(int(got[i][k]) for k in ("qstart", "qend", "tstart", "tend")) == w, (i, hits[i])
