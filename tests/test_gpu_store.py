"""The device-resident transcript store (sf_store_*): texts named as windows of the index's
packed transcripts (crates/index/src/lib.rs `tx_seq` / `tx_range`) are sliced on the device;
results equal the same jobs with the window's codes in the byte pool, bit-exactly, and the
oracle's on a sample.  A store made from the index's packed words gives the same."""
import numpy as np
import pytest

import oracle as O
import refcases as R

pytestmark = pytest.mark.gpu


def pack_u64(codes):
    """The index's packed layout: 32 bases per u64, base p at bits 2 * (p % 32)."""
    c = np.asarray(codes, dtype=np.uint64)
    n = (c.size + 31) // 32
    out = np.zeros(n, dtype=np.uint64)
    pad = np.zeros(n * 32, dtype=np.uint64)
    pad[:c.size] = c
    pad = pad.reshape(n, 32)
    for b in range(32):
        out |= pad[:, b] << np.uint64(2 * b)
    return out


def _setup(B, rng):
    txs = [rng.integers(0, 4, int(rng.integers(300, 5000)), dtype=np.uint8) for _ in range(60)]
    starts = np.concatenate([[0], np.cumsum([t.size for t in txs])[:-1]]).astype(np.uint64)
    pb = B.PoolBuilder()
    rows, copies, wins = [], [], []
    for q in range(240):
        x = int(rng.integers(0, len(txs)))
        t = txs[x]
        a = int(rng.integers(0, t.size // 2))
        b = int(rng.integers(a, t.size + 1))
        win = t[a:b]
        read = R.mutate(win.tolist(), R.rand_edits(rng, max(1, len(win) // 12), max(1, len(win))))
        p_off = pb.add(read)
        t_copy = pb.add(win)
        kind = q % 3
        f = {"p_off": p_off, "m": len(read), "n": int(win.size), "kind": kind}
        if kind == B.JOB_MYERS:
            f["mode"] = R.INFIX
        elif kind == B.JOB_AFFINE:
            f.update(mode=R.GLOBAL, band=int(rng.integers(10, 150)), want_cigar=1)
        else:
            f.update(band=16, window=int(win.size) + 20, xdrop=50, end_bonus=5, want_cigar=1)
        rows.append(dict(f, t_off=int(starts[x]) + a, text_src=B.TEXT_STORE))
        copies.append(dict(f, t_off=t_copy, text_src=B.TEXT_POOL))
        wins.append((read, win))
    return txs, pb.build(), rows, copies, wins


def _jobs(B, rows):
    jobs = B.new_jobs(len(rows))
    for q, f in enumerate(rows):
        for k, v in f.items():
            jobs[q][k] = v
    return jobs


def _same(a, b):
    for f in ("score", "distance", "pattern_end", "text_start", "text_end", "text_read", "cells",
              "n_ops", "status"):
        assert np.array_equal(a.results[f], b.results[f]), f
    for q in range(len(a.results)):
        assert a.cigar(q) == b.cigar(q), q


def test_store_windows_equal_pool_texts():
    from spearfish_gb300 import build
    build.build()
    from spearfish_gb300 import batch as B, _abi
    rng = np.random.default_rng(1901)
    txs, pool, rows, copies, wins = _setup(B, rng)
    ctx = B.Context(0)
    try:
        ref = B.run(ctx, pool, _jobs(B, copies))
        store = B.Store(ctx, txs)
        assert store.bases == sum(t.size for t in txs)
        with pytest.raises(_abi.SfError):  # no store in use yet
            B.run(ctx, pool, _jobs(B, rows))
        ctx.use_store(store)
        got = B.run(ctx, pool, _jobs(B, rows))
        _same(ref, got)
        # The index's own packed words give the same store.
        cat = np.concatenate(txs)
        packed = B.Store(ctx, packed=pack_u64(cat), bases=cat.size)
        ctx.use_store(packed)
        _same(ref, B.run(ctx, pool, _jobs(B, rows)))
        # A window past the store's end is refused.
        bad = _jobs(B, rows[:1])
        bad["t_off"][0] = cat.size - 3
        bad["n"][0] = 10
        with pytest.raises(_abi.SfError):
            B.run(ctx, pool, bad)
        ctx.use_store(None)
        packed.close()
        store.close()
    finally:
        ctx.close()
    for q in range(0, len(rows), 7):
        read, win = wins[q]
        r = got.results[q]
        if rows[q]["kind"] == 0:
            assert int(r["distance"]) == O.myers_distance(read, win, R.INFIX)
        elif rows[q]["kind"] == 1:
            o = O.traceback(read, win, O.TB_AFFINE, R.GLOBAL, R.ONT, rows[q]["band"])
            assert (int(r["score"]), got.cigar(q)) == (o["score"], o["cigar"])
        else:
            o = O.traceback(read, win, O.TB_EXTEND, O.PREFIX, R.ONT, 16, rows[q]["window"], 5, 50)
            assert (int(r["score"]), got.cigar(q)) == (o["score"], o["cigar"])


def test_store_windows_read_backwards():
    """SF_TEXT_STORE_REV: a window read backwards equals its reversed codes in the pool."""
    from spearfish_gb300 import build
    build.build()
    from spearfish_gb300 import batch as B
    rng = np.random.default_rng(1902)
    txs = [rng.integers(0, 4, int(rng.integers(100, 3000)), dtype=np.uint8) for _ in range(30)]
    starts = np.concatenate([[0], np.cumsum([t.size for t in txs])[:-1]]).astype(np.uint64)
    pb = B.PoolBuilder()
    rows, copies = [], []
    for q in range(150):
        x = int(rng.integers(0, len(txs)))
        t = txs[x]
        a = int(rng.integers(0, t.size))
        b = int(rng.integers(a, t.size + 1))
        win = t[a:b][::-1]
        read = R.mutate(win.tolist(), R.rand_edits(rng, max(1, len(win) // 10), max(1, len(win))))
        f = {"p_off": pb.add(read), "m": len(read), "n": int(win.size),
             "kind": 2 if q % 2 else 0, "band": 16, "window": int(win.size) + 20, "xdrop": 50,
             "end_bonus": 5, "mode": R.INFIX if q % 2 == 0 else 1}
        copies.append(dict(f, t_off=pb.add(win), text_src=B.TEXT_POOL))
        rows.append(dict(f, t_off=int(starts[x]) + a, text_src=2))
    pool = pb.build()
    ctx = B.Context(0)
    store = B.Store(ctx, txs)
    try:
        ref = B.run(ctx, pool, _jobs(B, copies))
        ctx.use_store(store)
        _same(ref, B.run(ctx, pool, _jobs(B, rows)))
    finally:
        ctx.use_store(None)
        store.close()
        ctx.close()
