"""Shared helpers of the segmented tie-break tests: the oracle as a DP runner, the golden
cases, and a seeded generator of read batches with near-tied candidate transcripts."""
import json
import os

import numpy as np

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
U32 = 0xFFFFFFFF


def golden(fn):
    with open(os.path.join(HERE, "golden", "reference_kats.json")) as f:
        return [k for k in json.load(f)["kats"] if k["fn"] == fn]


def _banded_sequential(read, texts, mode, cap, distinct):
    """map/src/lib.rs:3016-3034 `sequential` (the definition `banded` equals)."""
    seen, best, out = {}, U32, []
    for t in texts:
        key = tuple(int(c) for c in t)
        k = min(best + cap, U32)
        if key in seen and not distinct:
            d = seen[key]
            out.append(d if d <= k else min(k + 1, U32))
            continue
        d = O.myers_distance(read, t, mode, k)
        d = min(k + 1, U32) if d is None else d
        best = min(best, d)
        seen[key] = d
        out.append(d)
    return out


def oracle_runner(sorted_calls, banded_calls):
    """The batch's DP calls on the CPU oracle, one call at a time."""
    s = []
    for c in sorted_calls:
        if c["kind"] == 1:
            s.append(O.affine_extend_sorted_cut_bonus(
                c["read"], c["texts"], c["sc"], c["band"], c["end_bonus"], c["xdrop"],
                c["diagonal"], c["window"], c["cut"], c["track_cut"], c["bonus_within_cut"]))
        else:
            s.append([(x, x, 0) for x in O.affine_sorted(c["read"], c["texts"], c["mode"],
                                                          c["sc"], c["band"])])
    b = [_banded_sequential(*c) for c in banded_calls]
    return s, b


def _edit(seq, rng, rate):
    """seq with substitutions, insertions and deletions at `rate`; returns (new, map) where
    map[i] is the new position of seq[i] when it is kept unchanged, else -1."""
    out, mp = [], np.full(len(seq), -1, np.int64)
    for i, c in enumerate(seq):
        r = rng.random()
        if r < rate / 3:
            continue  # deleted
        if r < 2 * rate / 3:
            out.append((int(c) + int(rng.integers(1, 4))) & 3)  # substituted
        else:
            mp[i] = len(out)
            out.append(int(c))
        if rng.random() < rate / 3:
            out.append(int(rng.integers(0, 4)))  # inserted
    return np.array(out, np.uint8), mp


def read_batch(seed, n_reads=40, anchor=15, step=35):
    """Reads with 2-6 candidate transcripts each: isoforms of one base sequence that differ
    by skipped or inserted segments, substitutions and their 3' ends; the read is a stretch
    of the base with 5% errors, sometimes a poly(A) tail and leading junk.  Anchors are
    error-free stretches of `anchor` bases every `step` read bases, placed in every candidate
    that keeps them (some dropped at random).  Returns (reads, txs)."""
    rng = np.random.default_rng(seed)
    txs, reads = [], []
    for _ in range(n_reads):
        base = rng.integers(0, 4, int(rng.integers(300, 2500)), dtype=np.uint8)
        cands = []
        for c in range(int(rng.integers(2, 7))):
            seq, mp = base.copy(), np.arange(len(base))
            for _ in range(int(rng.integers(0, 4)) if c else 0):
                kind = int(rng.integers(0, 3))
                at = int(rng.integers(0, len(seq)))
                ln = int(rng.integers(1, 60))
                if kind == 0:  # skipped segment
                    seq = np.delete(seq, np.arange(at, min(len(seq), at + ln)))
                    mp = np.where(mp >= at + ln, mp - min(ln, len(base)), np.where(mp >= at, -1, mp))
                elif kind == 1:  # inserted segment
                    seq = np.insert(seq, at, rng.integers(0, 4, ln, dtype=np.uint8))
                    mp = np.where(mp >= at, mp + ln, mp)
                else:  # substitutions
                    pos = rng.integers(0, len(seq), 3)
                    seq[pos] = (seq[pos] + 1) & 3
                    bad = np.isin(mp, pos)
                    mp = np.where(bad, -1, mp)
            if c and rng.random() < 0.5:  # another 3' end
                cutb = int(rng.integers(0, min(200, len(seq) - 1)))
                if cutb:
                    seq = seq[:-cutb]
                    mp = np.where(mp >= len(seq), -1, mp)
            cands.append((seq, mp))
        s = int(rng.integers(0, 200))
        e = max(len(base) - int(rng.integers(0, 150)), s + 50)
        read, rmap = _edit(base[s:e], rng, 0.05)
        junk = 0
        if rng.random() < 0.3:  # leading junk (adapter) before the read's first base
            junk = int(rng.integers(1, 30))
            read = np.concatenate([rng.integers(0, 4, junk, dtype=np.uint8), read])
        if rng.random() < 0.4:  # a poly(A) tail, sometimes with adapter bases after it
            read = np.concatenate([read, np.zeros(int(rng.integers(18, 40)), np.uint8),
                                   rng.integers(0, 4, int(rng.integers(0, 20)), dtype=np.uint8)])
        # Read position of base position b (unchanged bases only).
        rpos = np.full(len(base), -1, np.int64)
        ok = rmap >= 0
        rpos[np.arange(s, e)[ok]] = rmap[ok] + junk
        hits = [(len(txs) + c, []) for c in range(len(cands))]
        for b in range(s, len(base) - anchor, step):
            q = rpos[b]
            if q < 0 or not np.all(rpos[b:b + anchor] == q + np.arange(anchor)):
                continue
            for c, (seq, mp) in enumerate(cands):
                t = mp[b]
                if t < 0 or not np.all(mp[b:b + anchor] == t + np.arange(anchor)):
                    continue
                if c and rng.random() < 0.1:
                    continue
                hits[c][1].append((int(q), int(t), anchor))
        txs.extend(seq for seq, _ in cands)
        reads.append((read, hits))
    return reads, txs
