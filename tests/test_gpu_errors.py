"""Bad jobs in a batch: sf_batch_run reports the first bad job's error -- also when the batch
is large enough to be converted on several host threads -- and the context stays usable:
the next good batch gives the oracle's results."""
import numpy as np
import pytest

import oracle as O
import refcases as R

pytestmark = pytest.mark.gpu

INVALID, TOO_LONG = -1, -4  # SF_ERR_INVALID, SF_ERR_TOO_LONG (include/sf_align.h)


@pytest.fixture(scope="module")
def env():
    from spearfish_gb300 import build
    build.build()
    from spearfish_gb300 import _abi
    from spearfish_gb300 import batch as B
    c = B.Context(0)
    yield B, _abi, c
    c.close()


def batch(B, count, rng):
    pool = B.PoolBuilder()
    rows = []
    for q in range(count):
        p, t = R.rand_pair(int(rng.integers(20, 120)), 10, int(rng.integers(1, 2 ** 62)))
        rows.append((pool.add(np.array(p, np.uint8)), pool.add(np.array(t, np.uint8)), p, t))
    jobs = B.new_jobs(count)
    for q, (po, to, p, t) in enumerate(rows):
        jobs[q]["p_off"], jobs[q]["t_off"] = po, to
        jobs[q]["m"], jobs[q]["n"] = len(p), len(t)
        jobs[q]["kind"] = B.JOB_MYERS if q % 2 else B.JOB_AFFINE
        jobs[q]["mode"] = R.GLOBAL
        jobs[q]["band"] = 16
    return pool.build(), jobs, rows


@pytest.mark.parametrize("count", [40, 20000])
def test_first_bad_job_reported(env, count):
    B, _abi, ctx = env
    rng = np.random.default_rng(31 + count)
    pool, jobs, rows = batch(B, count, rng)
    cases = [
        ("kind", 9, INVALID, "bad job kind"),
        ("p_off", pool.size + 5, INVALID, "outside the pool"),
        ("m", 0x7fffffff, TOO_LONG, "too long"),
    ]
    for field, value, code, text in cases:
        bad = jobs.copy()
        # Two bad jobs: the earlier one's error is the one reported.
        first, second = count // 3, (2 * count) // 3
        bad[first][field] = value
        bad[second]["kind"] = 9
        with pytest.raises(_abi.SfError) as e:
            B.run(ctx, pool, bad)
        assert e.value.code == code, (field, str(e.value))
        assert text in str(e.value), (field, str(e.value))
    # The context is still usable.
    out = B.run(ctx, pool, jobs)
    for q in range(0, count, max(1, count // 50)):
        _, _, p, t = rows[q]
        if q % 2:
            assert int(out.results[q]["distance"]) == O.myers_distance(p, t, R.GLOBAL), q
        else:
            assert int(out.results[q]["score"]) == O.affine(p, t, R.GLOBAL, R.ONT, 16), q


def test_myers_pattern_too_long(env):
    B, _abi, ctx = env
    rng = np.random.default_rng(32)
    big = B.PoolBuilder()
    po = big.add(rng.integers(0, 4, 40000).astype(np.uint8))
    to = big.add(rng.integers(0, 4, 100).astype(np.uint8))
    j = B.new_jobs(1)
    j[0]["p_off"], j[0]["t_off"], j[0]["m"], j[0]["n"] = po, to, 40000, 100
    j[0]["kind"] = B.JOB_MYERS
    with pytest.raises(_abi.SfError) as e:
        B.run(ctx, big.build(), j)
    assert e.value.code == TOO_LONG
