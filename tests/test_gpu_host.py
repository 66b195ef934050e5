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
