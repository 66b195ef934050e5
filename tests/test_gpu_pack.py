"""The pack kernel (byte codes -> 2-bit words on the device) at every alignment.

Patterns start at each of the 16 byte offsets of a 16-byte line (texts at another), at
lengths around the edges of the kernel's two-line load path (a word takes two aligned 16-byte
loads only when both lines lie inside its sequence; the first word and the last ones take
byte loads).  Every byte carries random upper bits: a code is byte & 3 (align.rs:78, 120).
Each pair runs as a Myers Global job and a banded affine Global job through sf_batch_run,
against the oracle (align.rs:87-168 `distance_with`, 2446-2666 `run_core`).
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

LENGTHS = [1, 2, 15, 16, 17, 31, 32, 33, 34, 47, 48, 49, 63, 64, 65, 95, 96, 97, 130, 257,
           1000, 2049]
BAND = 64


def _pool():
    rng = np.random.default_rng(61)
    parts, at = [], 0
    po, to, lens = [], [], []

    def put(seq, align):
        nonlocal at
        pad = (align - at) % 16
        parts.append(rng.integers(0, 256, pad, dtype=np.uint8))
        at += pad
        off = at
        parts.append(seq)
        at += seq.size
        return off

    for o in range(16):
        for n in LENGTHS:
            p = rng.integers(0, 256, n, dtype=np.uint8)
            flip = (rng.random(n) < 0.1).astype(np.uint8)
            t = ((p & 3) ^ flip) | (rng.integers(0, 64, n, dtype=np.uint8) << 2)
            po.append(put(p, o))
            to.append(put(t.astype(np.uint8), (o + 7) % 16))
            lens.append(n)
    pool = np.concatenate(parts)
    return (pool, np.array(po, np.uint64), np.array(to, np.uint64),
            np.array(lens, np.uint64))


@pytest.fixture(scope="module")
def lib():
    from spearfish_gb300 import build
    build.build()


def test_every_alignment(lib):
    from spearfish_gb300 import batch as B
    pool, po, to, lens = _pool()
    count = len(lens)
    jobs = B.new_jobs(2 * count)
    for h, kind in enumerate((B.JOB_MYERS, B.JOB_AFFINE)):
        j = jobs[h * count:(h + 1) * count]
        j["p_off"], j["t_off"], j["m"], j["n"] = po, to, lens, lens
        j["kind"] = kind
        j["mode"] = 2  # Global
        if kind == B.JOB_AFFINE:
            j["band"] = BAND
    ctx = B.Context(0)
    try:
        out = B.run(ctx, pool, jobs)
    finally:
        ctx.close()
    res = out.results
    assert (res["status"] == 0).all()
    threads = os.cpu_count() or 4
    d, _ = O.run_pairs(0, threads, pool, po, lens, pool, to, lens, O.GLOBAL)
    got = res["distance"][:count].astype(np.int64)
    bad = np.flatnonzero(got != d)
    assert bad.size == 0, [(int(q % len(LENGTHS)), int(q // len(LENGTHS))) for q in bad[:5]]
    s, _ = O.run_pairs(1, threads, pool, po, lens, pool, to, lens, O.GLOBAL, sc=O.ONT,
                       band=BAND)
    got = res["score"][count:].astype(np.int64)
    bad = np.flatnonzero(got != s)
    assert bad.size == 0, [(int(q % len(LENGTHS)), int(q // len(LENGTHS))) for q in bad[:5]]
