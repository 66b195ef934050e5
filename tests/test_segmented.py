"""`Mapper::segmented`'s host logic (spearfish_gb300/segmented.py) on the CPU, its DP calls
run on the oracle: the reference's paper example (map/src/lib.rs:3236-3300: the costs
[-28, -21, -13, -13]), its `shared_blocks` cases (lib.rs:3162-3233) and its `tail_start`
cases (lib.rs:3307-3313), all from tests/golden/reference_kats.json.  The device batch is
checked against the same host logic on the oracle in test_gpu_segmented.py."""
import dataclasses

import numpy as np

import segcases as S
from spearfish_gb300 import segmented as G


def test_paper_example_costs():
    (k,) = S.golden("segmented")
    a = k["args"]
    tb = dataclasses.replace(G.TieBreak(), **a["tb"])
    hits = [(tx, [tuple(x) for x in chain]) for tx, chain in a["hits"]]
    out = G.segmented_batch(None, [(np.array(a["read"], np.uint8), hits)],
                            [np.array(t, np.uint8) for t in a["texts"]], tb,
                            runner=S.oracle_runner)
    assert out[0][0] == k["want"] and out[0][1] == 1.0
    # The per-segment totals the example states (lib.rs:3293) are the costs negated.
    (tot,) = S.golden("segment_totals")
    assert [-c for c in out[0][0]] == tot["want"]


def test_shared_blocks_cases():
    cases = S.golden("shared_blocks")
    assert len(cases) == 7
    for k in cases:
        got = G.shared_blocks([[tuple(x) for x in ch] for ch in k["args"]["chains"]])
        want = k["want"]
        if want is None:
            assert got is None, k["cite"]
        else:
            assert [[list(b.query), [list(t) for t in b.targets]] for b in got] == want, k["cite"]


def test_tail_start_cases():
    for k in S.golden("tail_start"):
        got = G.tail_start(k["args"]["rest"], G.A_CODE, k["args"]["run"])
        assert (None if got is None else list(got)) == k["want"], k["cite"]


def test_batch_on_the_oracle_runs():
    """A seeded read batch through the host logic: every read with a shared block gets one
    cost per hit; reads whose candidates share nothing get None."""
    reads, txs = S.read_batch(11, 12)
    out = G.segmented_batch(None, reads, txs, runner=S.oracle_runner)
    for (r, hits), o in zip(reads, out):
        if G.shared_blocks([h[1] for h in hits]) is None:
            assert o is None
        else:
            assert len(o[0]) == len(hits)
