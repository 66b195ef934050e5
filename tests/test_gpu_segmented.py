"""`Mapper::segmented` for read batches with its DP on the device (one sf_sorted_batch, or
sf_banded_batch for unit costs, per batch): the reference's paper example
(map/src/lib.rs:3236-3300, costs [-28, -21, -13, -13]) and seeded batches of near-tied
isoforms -- skipped and inserted segments, other 3' ends, poly(A) tails, leading junk --
under the default TieBreak and variants of it (flank rule, end bonus cut, diagonal ends,
unit costs, `affine_within`'s unit-cost prefilter, no tail handling, a wider band), equal
read by read to the same host logic with its DP on the oracle."""
import dataclasses

import numpy as np
import pytest

import segcases as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from spearfish_gb300 import build
    build.build()
    from spearfish_gb300 import batch as B
    c = B.Context(0)
    yield c
    c.close()


def test_paper_example_on_the_device(ctx):
    from spearfish_gb300 import segmented as G
    (k,) = S.golden("segmented")
    a = k["args"]
    tb = dataclasses.replace(G.TieBreak(), **a["tb"])
    hits = [(tx, [tuple(x) for x in chain]) for tx, chain in a["hits"]]
    reads = [(np.array(a["read"], np.uint8), hits)] * 3  # one batch of three copies
    out = G.segmented_batch(ctx, reads, [np.array(t, np.uint8) for t in a["texts"]], tb)
    assert [o[0] for o in out] == [k["want"]] * 3


@pytest.mark.parametrize("variant", [
    {}, {"flank_min": 20}, {"end_bonus_cut": False}, {"end_diagonal": True},
    {"affine": None}, {"tail_trim": False, "tail_bonus": 0}, {"band": 40, "xdrop": 80},
    {"affine": (1, 4, 6, 2), "end_bonus": 3}, {"affine_within": 4}, {"affine_within": 0},
    {"affine_within": 30, "flank_min": 20}])
def test_batches_equal_the_oracle(ctx, variant):
    from spearfish_gb300 import segmented as G
    tb = dataclasses.replace(G.TieBreak(), **variant)
    reads, txs = S.read_batch(100 + len(str(variant)), 60)
    got = G.segmented_batch(ctx, reads, txs, tb)
    want = G.segmented_batch(None, reads, txs, tb, runner=S.oracle_runner)
    assert sum(o is not None for o in got) >= 40
    for q, (g, w) in enumerate(zip(got, want)):
        assert g == w, (q, variant)
