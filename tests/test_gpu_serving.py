"""The serving loop (sf_server_*): continuous batching on one GPU.

Each request's results must be the same alone and in a mix of concurrent requests (bit-exact:
integer work), a small HBM budget must serialise admission without changing results, and the
bounded waits and error paths must report cleanly.  Results are also checked against the
oracle on a sample."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    from spearfish_gb300 import build
    build.build()
    from spearfish_gb300 import batch as B, serve as S, workloads as W
    return B, S, W


def _requests(W, B, count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for q in range(count):
        n = int(rng.integers(1, 40))
        reads = [W.serving_read(rng, hifi=(q * 7 + i) % 11 == 0) for i in range(n)]
        out.append(W.serving_jobs(reads, B))
    return out


def _same(a, b):
    ra, rb = a.results, b.results
    for f in ("score", "distance", "pattern_end", "text_start", "text_end", "text_read",
              "cells", "n_ops", "status"):
        assert np.array_equal(ra[f], rb[f]), f
    for q in range(len(ra)):
        assert a.cigar(q) == b.cigar(q)


def test_same_alone_and_in_mix(mods):
    B, S, W = mods
    reqs = _requests(W, B, 12, 51)
    srv = S.Server(0, slots=4)
    try:
        alone = []
        for pool, jobs in reqs:
            out, st = srv.wait(srv.submit(pool, jobs))
            alone.append(out)
            assert st.total_ms >= st.run_ms >= 0
        tickets = [srv.submit(pool, jobs) for pool, jobs in reqs]
        mixed = [srv.wait(t) for t in tickets]
        used = {st.slot for _, st in mixed}
        for a, (m, _) in zip(alone, mixed):
            _same(a, m)
        assert len(used) > 1  # the mix ran on several slots
        q = srv.query()
        assert q["completed"] == 2 * len(reqs) and q["failed"] == 0
    finally:
        srv.close()
    # A sample against the oracle: affine scores and CIGARs, Myers distances.
    pool, jobs = reqs[3]
    out = alone[3]
    for q in range(min(len(jobs), 24)):
        j = jobs[q]
        p = pool[j["p_off"]:j["p_off"] + j["m"]]
        t = pool[j["t_off"]:j["t_off"] + j["n"]]
        r = out.results[q]
        if j["kind"] == B.JOB_MYERS:
            assert int(r["distance"]) == O.myers_distance(p, t, O.INFIX)
        elif j["kind"] == B.JOB_AFFINE:
            tb = O.traceback(p, t, O.TB_AFFINE, O.GLOBAL, O.ONT, int(j["band"]))
            assert (int(r["score"]), out.cigar(q)) == (tb["score"], tb["cigar"])
        else:
            tb = O.traceback(p, t, O.TB_EXTEND, O.PREFIX, O.ONT, int(j["band"]),
                             int(j["window"]), int(j["end_bonus"]), int(j["xdrop"]))
            assert (int(r["score"]), int(r["pattern_end"]), int(r["text_end"]),
                    out.cigar(q)) == (tb["score"], tb["end_i"], tb["end_j"], tb["cigar"])


def test_budget_serialises_admission(mods):
    B, S, W = mods
    reqs = _requests(W, B, 6, 52)
    ref = S.Server(0, slots=2)
    try:
        want = [ref.wait(ref.submit(p, j))[0] for p, j in reqs]
    finally:
        ref.close()
    # A budget that holds about one request at a time.
    srv = S.Server(0, slots=4, hbm_budget=256 << 20)
    try:
        tickets = []
        for p, j in reqs:
            try:
                tickets.append(srv.submit(p, j))
            except Exception as e:  # larger than the whole budget: refused at submit
                assert "budget" in str(e)
                tickets.append(None)
        for t, w in zip(tickets, want):
            if t is not None:
                _same(srv.wait(t)[0], w)
    finally:
        srv.close()


def test_errors_and_bounded_waits(mods):
    B, S, W = mods
    from spearfish_gb300 import _abi
    srv = S.Server(0, slots=2, hbm_budget=64 << 20)
    try:
        with pytest.raises(_abi.SfError):
            srv.wait(999_999, 0)  # unknown ticket
        # A request larger than the whole budget is refused at submission.
        rng = np.random.default_rng(53)
        big = [W.serving_read(rng, hifi=True) for _ in range(40)]
        pool, jobs = W.serving_jobs(big, B)
        with pytest.raises(_abi.SfError) as e:
            srv.submit(pool, jobs)
        assert e.value.code == -3
        # A bad job (text outside the pool) is refused at submission.
        pool, jobs = _requests(W, B, 1, 54)[0]
        bad = jobs.copy()
        bad["t_off"][0] = pool.size + 10
        with pytest.raises(_abi.SfError):
            srv.submit(pool, bad)
        # A zero timeout returns at once: finished or not yet.
        t = srv.submit(pool, jobs)
        r = srv.try_wait(t)
        if r is None:
            r = srv.wait(t, 60_000)
        assert len(r[0].results) == len(jobs)
    finally:
        srv.close()


def test_store_requests_equal_pool_requests(mods):
    """Requests whose texts are windows of the server's transcript store give the same
    results as the same requests with the windows' codes in their pools."""
    B, S, W = mods
    tx = W.Transcriptome(n_ont=300, n_long=20, seed=56)
    rng = np.random.default_rng(57)
    reqs = []
    for _ in range(6):
        reads = [W.serving_store_read(tx, rng, hifi=rng.random() < 0.1)
                 for _ in range(int(rng.integers(1, 30)))]
        reqs.append(W.serving_store_jobs(tx, reads, B))
    cat = np.concatenate(tx.txs)

    def copied(pool, jobs):
        parts, at = [pool], pool.size
        j2 = jobs.copy()
        for q in range(len(jobs)):
            if jobs["text_src"][q] == B.TEXT_STORE:
                o, n = int(jobs["t_off"][q]), int(jobs["n"][q])
                parts.append(cat[o:o + n])
                j2["t_off"][q], j2["text_src"][q] = at, B.TEXT_POOL
                at += n
        return np.concatenate(parts), j2

    ctx = B.Context(0)
    store = B.Store(ctx, tx.txs)
    srv = S.Server(0, slots=3, store=store)
    try:
        tickets = [srv.submit(p, j) for p, j in reqs]
        got = [srv.wait(t)[0] for t in tickets]
        want = [srv.wait(srv.submit(*copied(p, j)))[0] for p, j in reqs]
        for a, b in zip(got, want):
            _same(a, b)
    finally:
        srv.close()
        store.close()
        ctx.close()
