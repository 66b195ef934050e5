"""The host plan build on large batches, split into chunks on host threads: sequences shared
by consecutive jobs (a pass aligning a sequence to itself) are stored once, also where a
chunk starts on such a repeat, and pools out of job order take the sorting path; every
result is checked against its definition."""
import numpy as np
import pytest

import oracle as O
import refcases as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    from spearfish_gb300 import build
    build.build()
    from spearfish_gb300 import batch as B
    c = B.Context(0)
    yield B, c
    c.close()


@pytest.mark.parametrize("count", [10001, 12347])
def test_self_alignments_across_chunks(env, count):
    B, ctx = env
    rng = np.random.default_rng(count)
    pool = B.PoolBuilder()
    seqs = []
    jobs = B.new_jobs(count)
    for q in range(count):
        s = rng.integers(0, 4, int(rng.integers(1, 90))).astype(np.uint8)
        off = pool.add(s)
        seqs.append(s)
        j = jobs[q]
        j["p_off"] = j["t_off"] = off  # pattern and text: the same sequence
        j["m"] = j["n"] = s.size
        j["kind"] = B.JOB_MYERS if q % 3 else B.JOB_AFFINE
        j["mode"] = R.GLOBAL
        j["band"] = 8
    out = B.run(ctx, pool.build(), jobs)
    for q in range(count):
        r = out.results[q]
        if q % 3:
            assert int(r["distance"]) == 0, q
        else:
            assert int(r["score"]) == 2 * seqs[q].size, q  # ONT match score 2


def test_pool_out_of_job_order(env):
    """Jobs whose sequences lie in the pool in reverse order (the sorting path), with one
    pattern shared by every job."""
    B, ctx = env
    rng = np.random.default_rng(7)
    count = 9000
    p = rng.integers(0, 4, 120).astype(np.uint8)
    texts = [R.mutate(list(p), R.rand_edits(rng, int(rng.integers(0, 12)), 120))
             for _ in range(count)]
    pool = B.PoolBuilder()
    toffs = [pool.add(np.array(t, np.uint8)) for t in reversed(texts)][::-1]
    poff = pool.add(p)
    jobs = B.new_jobs(count)
    for q in range(count):
        j = jobs[q]
        j["p_off"], j["t_off"], j["m"], j["n"] = poff, toffs[q], p.size, len(texts[q])
        j["kind"] = B.JOB_MYERS
        j["mode"] = R.INFIX
    out = B.run(ctx, pool.build(), jobs)
    for q in range(0, count, 37):
        assert int(out.results[q]["distance"]) == O.myers_distance(p, texts[q], R.INFIX), q


@pytest.mark.parametrize("count", [10001, 16411])
def test_neighbours_share_sequences_across_chunks(env, count):
    """Job q aligns sequence q to sequence q + 1, so each job's text is the next job's
    pattern: one stored copy per sequence, also where a chunk of jobs starts."""
    B, ctx = env
    rng = np.random.default_rng(count + 1)
    pool = B.PoolBuilder()
    seqs, offs = [], []
    for _ in range(count + 1):
        s = rng.integers(0, 4, int(rng.integers(1, 70))).astype(np.uint8)
        offs.append(pool.add(s))
        seqs.append(s)
    jobs = B.new_jobs(count)
    for q in range(count):
        j = jobs[q]
        j["p_off"], j["t_off"] = offs[q], offs[q + 1]
        j["m"], j["n"] = seqs[q].size, seqs[q + 1].size
        j["kind"] = B.JOB_MYERS if q % 2 else B.JOB_AFFINE
        j["mode"] = R.GLOBAL
        j["band"] = 80
    out = B.run(ctx, pool.build(), jobs)
    for q in range(0, count, 7):
        r = out.results[q]
        if q % 2:
            assert int(r["distance"]) == O.myers_distance(seqs[q], seqs[q + 1], R.GLOBAL), q
        else:
            assert int(r["score"]) == O.affine(seqs[q], seqs[q + 1], R.GLOBAL, R.ONT, 80), q


@pytest.mark.parametrize("count", [8192, 13001, 40000])
def test_segmented_batch_equals_one_plan(env, count, monkeypatch):
    """A large batch runs in segments (each its own plan, the next built while the last
    runs): every result field and every CIGAR op equals the one-plan run's, CIGAR offsets
    follow job order across segments, and the CIGARs score what the results say."""
    B, ctx = env
    rng = np.random.default_rng(count + 2)
    pool = B.PoolBuilder()
    jobs = B.new_jobs(count)
    pairs = []
    for q in range(count):
        t = rng.integers(0, 4, int(rng.integers(100, 260))).astype(np.uint8)
        p = t[rng.random(t.size) > 0.04]  # deletions, then substitutions
        sub = rng.random(p.size) < 0.05
        p[sub] = (p[sub] + 1) & 3
        j = jobs[q]
        j["p_off"], j["t_off"] = pool.add(p), pool.add(t)
        j["m"], j["n"] = p.size, t.size
        kind = q % 4
        j["kind"] = B.JOB_MYERS if kind == 0 else B.JOB_AFFINE
        j["mode"] = (R.GLOBAL, R.PREFIX, R.INFIX)[q % 3] if kind == 0 else (R.GLOBAL, R.PREFIX)[q % 2]
        j["want_cigar"] = kind in (1, 2)
        j["band"] = int(rng.integers(20, 100))  # even work: the batch runs in segments
        pairs.append((p, t))
    built = pool.build()
    monkeypatch.setenv("SF_BATCH_SEGMENTS", "0")
    one = B.run(ctx, built, jobs)
    monkeypatch.setenv("SF_BATCH_SEGMENTS", "1")
    seg = B.run(ctx, built, jobs)
    for name in one.results.dtype.names:
        assert np.array_equal(one.results[name], seg.results[name]), name
    assert np.array_equal(one.ops, seg.ops)
    cig = np.nonzero(jobs["want_cigar"])[0]
    offs = seg.results["cigar_off"][cig]
    assert np.all(np.diff(offs.astype(np.int64)) >= 0)
    for q in cig[:: max(1, len(cig) // 60)]:
        r = seg.results[q]
        assert r["status"] == 0, q
        p, t = pairs[q]
        score, used, _ = O.cigar_score(p, t, seg.cigar(q), int(r["text_start"]), R.ONT)
        assert (score, used) == (int(r["score"]), int(r["pattern_end"])), q


@pytest.mark.parametrize("count", [300, 9000])
def test_ops_buffer_too_small(env, count):
    """An ops buffer smaller than the CIGARs: SF_ERR_CAPACITY with ops_used set to what the
    CIGARs need (one plan, and a batch in segments), and the context stays usable."""
    import ctypes as C
    from spearfish_gb300 import _abi
    B, ctx = env
    rng = np.random.default_rng(count + 3)
    pool = B.PoolBuilder()
    jobs = B.new_jobs(count)
    for q in range(count):
        t = rng.integers(0, 4, int(rng.integers(150, 200))).astype(np.uint8)
        p = t[rng.random(t.size) > 0.03]
        j = jobs[q]
        j["p_off"], j["t_off"], j["m"], j["n"] = pool.add(p), pool.add(t), p.size, t.size
        j["kind"], j["mode"], j["want_cigar"], j["band"] = B.JOB_AFFINE, R.GLOBAL, 1, 40
    built = pool.build()
    good = B.run(ctx, built, jobs)
    need = good.ops.size
    assert need > 0
    lib = _abi.load()
    sc = (_abi.Affine * 1)(_abi.Affine(2, 4, 4, 2))
    res = np.zeros(count, dtype=B.RESULT_DTYPE)
    ops = np.zeros(need, dtype=np.uint32)
    used = C.c_uint64()
    rc = lib.sf_batch_run(ctx.handle, built.ctypes.data_as(C.POINTER(C.c_uint8)), built.size,
                          jobs.ctypes.data_as(C.POINTER(_abi.JobT)), count, sc, 1,
                          res.ctypes.data_as(C.POINTER(_abi.ResultT)),
                          ops.ctypes.data_as(C.POINTER(C.c_uint32)), need // 2, C.byref(used))
    assert rc == -6  # SF_ERR_CAPACITY (include/sf_align.h)
    assert used.value == need
    again = B.run(ctx, built, jobs)
    assert np.array_equal(again.results, good.results) and np.array_equal(again.ops, good.ops)
