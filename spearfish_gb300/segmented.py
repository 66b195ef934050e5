"""Tie-break by segments for a read batch: map/src/lib.rs:1294-1884 `Mapper::segmented`.

The mapper compares near-tied candidate transcripts of a read by aligning only where they can
differ: the read between consecutive anchor blocks that every candidate shares (globally,
and only where the candidates' texts differ), and the read's two ends against windows that
start at the outermost shared blocks (prefix alignment with an end bonus and X-drop, the left
end reversed).  Each candidate's cost is the sum of its negated segment scores, less a bonus
where its window ends at the read's poly(A) tail.

Here a whole read batch is planned first -- every segment of every read becomes one sorted
DP call (`affine_sorted` / `affine_extend_sorted_cut_bonus` over the segment's distinct
texts in sorted order, lib.rs:1363-1445) -- then all calls run in one device batch
(`sf_sorted_batch`; with unit costs, `sf_banded_batch`), and the costs are assembled from the
results.  The results equal the reference's read by read.

Scope: parsed reads without raw read ends (the reference's `raw = None` path: no raw
midpoints, no templated tails).  With `affine_within` the batch runs in two device
launches: the unit-cost (Myers) calls, then the affine calls they select.
Sequences are byte codes (A0 C1 G2 T3)."""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Optional, Sequence

import numpy as np

A_CODE = 0       # lcp_core::encode::CODE[b'A'] & 3
TAIL_TOL = 15    # lib.rs:2882
TAIL_AFTER = 80  # lib.rs:2884
MODE_PREFIX, MODE_GLOBAL = 1, 2


@dataclass(frozen=True)
class TieBreak:
    """The TieBreak fields `segmented` reads, with the reference's defaults (lib.rs:222-266).
    affine: (mat, mis, open, ext) or None (unit costs, Myers with `cap`); affine_within: with
    affine scores, only texts within that many edits of the segment's best get one."""
    cap: int = 16
    affine: Optional[tuple] = (2, 4, 4, 2)
    affine_within: Optional[int] = None
    lambda_: float = 1.0
    kappa: float = 6.0
    band: int = 16
    clip_ends: bool = True
    end_bonus: int = 5
    xdrop: int = 50
    end_diagonal: bool = False
    pad: int = 20
    pad_div: int = 10
    tail_bonus: int = 10
    tail_trim: bool = True
    tail_run: int = 15
    flank_min: int = 0
    end_bonus_cut: bool = True

    def window(self, x: int) -> int:
        """lib.rs:217-219: transcript bases searched for an unanchored read end of x bases."""
        return x + self.pad + x // self.pad_div


@dataclass
class Block:
    """lib.rs:551-554 `SharedBlock`: a query range and each candidate's target range."""
    query: tuple
    targets: list


def shared_blocks(chains: Sequence[Sequence[tuple]]) -> Optional[list]:
    """lib.rs:562-630: anchors (query start, length) shared by every candidate, in query order;
    an overlapping anchor extends the block before it when every candidate places it on the
    same diagonal, else it is dropped, as is one whose targets run backwards.  chains: per
    candidate, (q, t, len) anchors ordered by q.  None if nothing is shared."""
    if not chains:
        return None
    first = chains[0]
    cursors = [0] * len(chains)
    blocks: list[Block] = []
    group = 0
    while group < len(first):
        q = first[group][0]
        nxt = group + 1
        while nxt < len(first) and first[nxt][0] == q:
            nxt += 1
        lengths = sorted({a[2] for a in first[group:nxt]})
        group = nxt
        for h, ch in enumerate(chains):
            while cursors[h] < len(ch) and ch[cursors[h]][0] < q:
                cursors[h] += 1
        for ln in lengths:
            targets = []
            for h, ch in enumerate(chains):
                t = None
                for a in ch[cursors[h]:]:
                    if a[0] != q:
                        break
                    if a[2] == ln:
                        t = a[1]
                        break
                if t is None:
                    break
                targets.append((t, t + ln))
            if len(targets) != len(chains):
                continue
            end = q + ln
            if blocks:
                b = blocks[-1]
                if q < b.query[1]:
                    d = q - b.query[0]
                    if any(old[0] + d != new[0] for old, new in zip(b.targets, targets)):
                        continue
                    b.targets = [(old[0], max(old[1], new[1]))
                                 for old, new in zip(b.targets, targets)]
                    b.query = (b.query[0], max(b.query[1], end))
                    continue
                if any(a[1] > bb[0] for a, bb in zip(b.targets, targets)):
                    continue
            blocks.append(Block((q, end), list(targets)))
    return blocks or None


def tail_start(rest, a: int, run: int, after: int = TAIL_AFTER) -> Optional[tuple]:
    """lib.rs:2935-2969: the read's poly(A) tail past its last block -- the first window of
    `run` bases with at most one other base that leaves at most `after` read bases after
    the run -- as (start, run end), or None."""
    rest = [int(c) for c in rest]
    if len(rest) < run:
        return None
    others = lambda w: sum(1 for c in w if c != a)  # noqa: E731
    i, other = 0, others(rest[:run])
    while True:
        if other <= 1:
            s = i + next((k for k, c in enumerate(rest[i:]) if c == a), 0)
            end, non = s, 0
            for k in range(s, len(rest)):
                non += rest[k] != a
                if rest[k] == a and non * 10 <= k + 1 - s:
                    end = k + 1
            if len(rest) - end <= after:
                return (s, end)
            i = max(end, i + 1)
            if i + run > len(rest):
                return None
            other = others(rest[i:i + run])
        else:
            if i + run >= len(rest):
                return None
            other = other + (rest[i + run] != a) - (rest[i] != a)
            i += 1


def _count_other(t: np.ndarray, frm: int, code: int) -> int:
    return int(np.count_nonzero(t[frm:] != code))


class _Plan:
    """DP calls of a batch, filled in when the batch has run: the unit-cost (Myers) calls run
    first, then `stage2` turns their results into the affine calls that depend on them
    (`affine_within`), then the sorted affine calls run."""

    def __init__(self):
        self.sorted: list = []
        self.banded: list = []
        self.stage2: list = []
        self.sorted_out: list = []
        self.banded_out: list = []


def _seg(P: _Plan, tb: TieBreak, texts: list, read: np.ndarray, mode: int, rev: bool,
         cut: Optional[int]):
    """lib.rs:1307-1456 `seg`: each candidate's cost for one segment, and with a cut its cost
    against its text cut there and the text bases its alignment covers.  Returns None (every
    text the same: equal costs) or a function giving (delta, delta_cut, cols) once the
    batch has run."""
    n = len(texts)
    if all(np.array_equal(texts[0], t) for t in texts[1:]):
        return None
    if mode == MODE_GLOBAL and len(read) == 0 and tb.affine is not None and \
            tb.affine_within is None:
        # An insertion-only global gap costs by its length alone (lib.rs:1320-1332).
        _, _, opn, ext = tb.affine
        d = [opn + ext * len(t) if len(t) else 0 for t in texts]
        return lambda: (list(d), list(d), [0] * n)
    # Each distinct text once (rep0: each candidate's distinct text).
    distinct: list = []
    rep0 = []
    for t in texts:
        for u, dd in enumerate(distinct):
            if np.array_equal(dd, t):
                rep0.append(u)
                break
        else:
            distinct.append(t)
            rep0.append(len(distinct) - 1)
    decoded = [np.ascontiguousarray(t[::-1]) if rev else np.ascontiguousarray(t)
               for t in distinct]
    rd = np.ascontiguousarray(read[::-1]) if rev else np.ascontiguousarray(read)
    if tb.affine is None:
        # Unit costs: `banded` over the candidates' texts in order (lib.rs:1447-1455).
        at = len(P.banded)
        P.banded.append((rd, [decoded[d] for d in rep0], mode, tb.cap, False))

        def fin_unit():
            xs = P.banded_out[at]
            return list(xs), list(xs), [0] * n
        return fin_unit
    # Distinct texts in sorted order (rep: each candidate's place), scored once each.
    uniq = sorted(range(len(decoded)), key=lambda u: bytes(decoded[u]))
    place = [0] * len(decoded)
    for k, u in enumerate(uniq):
        place[u] = k
    rep = [place[d] for d in rep0]
    tx_all = [decoded[u] for u in uniq]
    diag = mode == MODE_PREFIX and tb.clip_ends and tb.end_diagonal

    def sorted_call(tx):
        call = {"read": rd, "texts": tx, "band": tb.band}
        if mode == MODE_PREFIX and tb.clip_ends:
            window = max(tb.window(len(rd)), max(len(t) for t in tx))
            call.update(kind=1, end_bonus=tb.end_bonus, xdrop=tb.xdrop, diagonal=diag,
                        window=window, cut=cut, track_cut=tb.flank_min > 0,
                        bonus_within_cut=tb.end_bonus_cut)
        else:
            call.update(kind=0, mode=mode)
        P.sorted.append(call)
        return len(P.sorted) - 1

    st = {}  # the sorted call's index, the texts it scores (todo), the unit distances
    if tb.affine_within is not None and len(uniq) > 1:
        # `affine_within` (lib.rs:1377-1405): a capped unit-cost pass over the distinct texts
        # first; only the texts within that many edits of the best get an affine score.
        w = int(tb.affine_within)
        at_u = len(P.banded)
        P.banded.append((rd, tx_all, mode, w, True))

        def stage2():
            d = P.banded_out[at_u]
            dmin = min(d)
            st["unit"] = d
            st["todo"] = [k for k in range(len(uniq)) if d[k] <= dmin + w]
            st["at"] = sorted_call([tx_all[k] for k in st["todo"]])
        P.stage2.append(stage2)
    else:
        st["unit"] = None
        st["todo"] = list(range(len(uniq)))
        st["at"] = sorted_call(tx_all)

    def fin():
        xs = P.sorted_out[st["at"]]
        unit, todo = st["unit"], st["todo"]
        score, score_cut, cols_k = {}, {}, {}
        best = None  # (unit distance, affine score), the least distance then the best score
        for k, (x, xc, cc) in zip(todo, xs):
            score[k], score_cut[k], cols_k[k] = x, xc, cc
            du = unit[k] if unit is not None else 0
            if best is None or (du, -x) < (best[0], -best[1]):
                best = (du, x)
        per_edit = tb.affine[0] + tb.affine[1]  # one mismatch per extra edit (lib.rs:1448)
        delta, delta_cut, cols = [0] * n, [0] * n, [0] * n
        for i in range(n):
            k = rep[i]
            x = score[k] if k in score else best[1] - per_edit * (unit[k] - best[0])
            delta[i] = -x
            delta_cut[i] = -score_cut.get(k, x)
            cols[i] = cols_k.get(k, 0)
        return delta, delta_cut, cols
    return fin


def _end(P: _Plan, tb: TieBreak, texts: list, read: np.ndarray, rev: bool, short: list):
    """lib.rs:1461-1533 `end`: a read end against each candidate's window; past the shortest
    window that stops at its transcript's end, gains count only as `flank_min` and
    `end_bonus_cut` say.  Returns None or a function giving the costs."""
    lens = [len(t) for t, s in zip(texts, short) if s]
    cut = min(lens) if lens else None
    if cut is None or not ((tb.flank_min > 0 or tb.end_bonus_cut) and
                           any(len(t) > cut for t in texts)):
        f = _seg(P, tb, texts, read, MODE_PREFIX, rev, None)
        return None if f is None else (lambda: f()[0])
    f = _seg(P, tb, texts, read, MODE_PREFIX, rev, cut)
    if f is None:
        return None
    if tb.flank_min <= 0:
        return lambda: f()[0]
    long = [len(t) > cut for t in texts]
    mat = tb.affine[0] if tb.affine is not None else 1

    def fin():
        out, near, cols = f()
        out = list(out)
        for i in range(len(out)):
            gain = near[i] - out[i]
            past = max(0, cols[i] - cut)
            if long[i] and gain < tb.flank_min and not (past > 0 and 4 * gain >= 3 * mat * past):
                out[i] = near[i]
        return out
    return fin


def _plan_read(P: _Plan, tb: TieBreak, codes: np.ndarray, hits: Sequence, txs: Sequence,
               hpc: bool):
    """One read's segments (lib.rs:1294-1884 with raw = None); returns None (no shared
    block) or a function giving (cost, unit) once the batch has run."""
    blocks = shared_blocks([h[1] for h in hits])
    if blocks is None:
        return None
    plen = len(codes)
    tx_of = [h[0] for h in hits]
    parts = []
    # Interior segments between consecutive blocks, where the candidates' texts differ.
    for left, right in zip(blocks, blocks[1:]):
        gaps = [txs[tx][left.targets[i][1]:right.targets[i][0]] for i, tx in enumerate(tx_of)]
        if all(len(g) == len(gaps[0]) and np.array_equal(g, gaps[0]) for g in gaps[1:]):
            continue
        f = _seg(P, tb, gaps, codes[left.query[1]:right.query[0]], MODE_GLOBAL, False, None)
        if f is not None:
            parts.append(lambda f=f: f()[0])
    # Left end: read[0, q0) against windows ending at each candidate's first block.
    first = blocks[0]
    q0 = first.query[0]
    if q0 > 0:
        spans = [(tx, max(0, first.targets[i][0] - tb.window(q0)), first.targets[i][0])
                 for i, tx in enumerate(tx_of)]
        short = [lo == 0 for _, lo, _ in spans]
        f = _end(P, tb, [txs[tx][lo:hi] for tx, lo, hi in spans], codes[:q0], True, short)
        if f is not None:
            parts.append(f)
    # Right end: read[last block's end, plen) against windows from each candidate's block end.
    last = blocks[-1]
    ql = last.query[1]
    rest = plen - ql
    spans = [(tx, last.targets[i][1], min(last.targets[i][1] + tb.window(rest), len(txs[tx])))
             for i, tx in enumerate(tx_of)]
    tail = None
    if (tb.tail_trim or tb.tail_bonus > 0) and not hpc:
        tail = tail_start(codes[ql:], A_CODE, tb.tail_run)
    short = [hi == len(txs[tx]) for tx, _, hi in spans]
    texts = [txs[tx][lo:hi] for tx, lo, hi in spans]
    cut = tail[0] if tail else plen - ql
    run_end = tail[1] if tail else cut
    at_end = None
    if tail:
        tol = TAIL_TOL + cut // 10
        at_end = [abs(len(t) - cut) <= tol or
                  (len(t) > cut and len(t) <= run_end + tol and
                   _count_other(t, cut, A_CODE) * 10 <= len(t) - cut) for t in texts]
    read = codes[ql:]
    if tb.tail_trim:
        read = read[:cut]
    f = _end(P, tb, texts, read, False, short)
    if f is not None:
        parts.append(f)
    unit = tb.lambda_ if tb.affine is not None else tb.kappa

    def fin():
        cost = [0] * len(hits)
        for part in parts:
            for i, x in enumerate(part()):
                cost[i] += x
        # Candidates whose 3' end is where the read's tail starts gain the bonus.
        if at_end is not None and tb.tail_bonus > 0:
            for i, ((tx, _, hi), ok) in enumerate(zip(spans, at_end)):
                if ok and hi == len(txs[tx]):
                    cost[i] -= tb.tail_bonus
        return cost, unit
    return fin


Runner = Callable[[list, list], tuple]


def gpu_runner(ctx) -> Runner:
    """Runs a batch's DP calls on the device: the sorted affine calls in one sf_sorted_batch,
    the unit-cost ones in one sf_banded_batch."""
    from . import tiebreak as T

    def run(sorted_calls: list, banded_calls: list):
        s = T.sorted_batch(ctx, sorted_calls, (sorted_calls[0]["sc"],)) if sorted_calls else []
        b = T.banded_batch(ctx, banded_calls) if banded_calls else []
        return s, b
    return run


def segmented_batch(ctx, reads: Sequence, txs: Sequence, tb: TieBreak = TieBreak(),
                    hpc: bool = False, runner: Optional[Runner] = None) -> list:
    """`Mapper::segmented` for a batch of reads (lib.rs:1294-1884, raw = None): reads =
    [(codes, hits)], hits = [(transcript, [(query start, transcript start, length), ...])]
    with each chain ordered by query start; txs: each transcript's codes.  Returns per read
    (costs per hit, unit) or None when no anchor is shared by every hit.  The DP calls of the
    whole batch run in one device batch -- two with `affine_within` -- (or through
    `runner`)."""
    P = _Plan()
    tx_arr = [np.ascontiguousarray(np.asarray(t, dtype=np.uint8)) for t in txs]
    fins = [_plan_read(P, tb, np.ascontiguousarray(np.asarray(r, dtype=np.uint8)), hits,
                       tx_arr, hpc) for r, hits in reads]
    run = runner if runner is not None else gpu_runner(ctx)
    if P.banded:
        _, P.banded_out = run([], P.banded)
    for f in P.stage2:
        f()
    for c in P.sorted:
        c["sc"] = tb.affine
    if P.sorted:
        P.sorted_out, _ = run(P.sorted, [])
    return [None if f is None else f() for f in fins]


__all__ = ["TieBreak", "Block", "shared_blocks", "tail_start", "segmented_batch", "gpu_runner"]
