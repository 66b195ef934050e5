"""Tie-break batching: the mapper's per-read distance calls (map/src/lib.rs:851-911
`Mapper::banded`) for one read, or for a whole read batch in one device launch
(include/sf_align.h, "tie-break batching").

``banded(read, texts, mode, cap, distinct)`` returns, per text in order, the edit distance
or k + 1 when it exceeds k = (best so far + cap), as the reference does.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _abi
from .align import _codes, _ptr, _Texts
from .batch import Context, PoolBuilder

NONE = 0xFFFFFFFF


def banded(read, texts: Sequence, mode: int, cap: int, distinct: bool = False) -> list[int]:
    """lib.rs:851-911 `Mapper::banded` (one read; the one-call context)."""
    if not texts:
        return []
    r = _codes(read)
    tx = _Texts(texts)
    out = np.zeros(len(texts), dtype=np.uint32)
    _abi.check(_abi.load().sf_banded(_ptr(r), r.size, *tx.args(), int(mode), int(cap),
                                     int(bool(distinct)),
                                     out.ctypes.data_as(C.POINTER(C.c_uint32))))
    return [int(v) for v in out]


def banded_batch(ctx: Context, reads: Sequence) -> list[list[int]]:
    """`banded` for many reads in one device batch: reads = [(read, texts, mode, cap,
    distinct), ...]; returns each read's list."""
    pb = PoolBuilder()
    rs = (_abi.BandedReadT * max(1, len(reads)))()
    spans = []
    for i, (read, texts, mode, cap, distinct) in enumerate(reads):
        r = rs[i]
        r.p_off = pb.add(read)
        r.m = len(read)
        r.first = len(spans)
        r.count = len(texts)
        r.mode = int(mode)
        r.cap = int(cap)
        r.distinct = int(bool(distinct))
        for t in texts:
            spans.append((pb.add(t), len(t)))
    pool = pb.build()
    sp = (_abi.SpanT * max(1, len(spans)))(*[_abi.SpanT(o, n) for o, n in spans])
    out = np.zeros(max(1, len(spans)), dtype=np.uint32)
    _abi.check(_abi.load().sf_banded_batch(
        ctx.handle, pool.ctypes.data_as(C.POINTER(C.c_uint8)), pool.size, rs, len(reads), sp,
        len(spans), out.ctypes.data_as(C.POINTER(C.c_uint32))))
    res, at = [], 0
    for _, texts, *_ in reads:
        res.append([int(v) for v in out[at:at + len(texts)]])
        at += len(texts)
    return res


def extend_ends_batch(ctx: Context, pool: np.ndarray, ends: dict, hits: np.ndarray) -> np.ndarray:
    """lib.rs:2020-2114 `extend_ends` for many hits in one device batch (texts from the
    context's transcript store).  `ends`: sc (mat, mis, open, ext), band, end_bonus, xdrop,
    pad, pad_div.  `hits`: a HIT_DTYPE array (read_off, tx_start, read_len, tx_len, qstart,
    qend, tstart, tend); returns a copy with the spans extended."""
    from .align import _aff
    out = np.ascontiguousarray(hits, dtype=HIT_DTYPE).copy()
    pool = np.ascontiguousarray(pool, dtype=np.uint8)
    e = _abi.EndsT(_aff(ends["sc"]), int(ends["band"]), int(ends["end_bonus"]), int(ends["xdrop"]),
                   int(ends["pad"]), int(ends["pad_div"]))
    _abi.check(_abi.load().sf_extend_ends_batch(
        ctx.handle, pool.ctypes.data_as(C.POINTER(C.c_uint8)), pool.size, C.byref(e),
        out.ctypes.data_as(C.POINTER(_abi.HitT)), len(out)))
    return out


HIT_DTYPE = np.dtype([("read_off", "<u8"), ("tx_start", "<u8"), ("read_len", "<u4"),
                      ("tx_len", "<u4"), ("qstart", "<u4"), ("qend", "<u4"), ("tstart", "<u4"),
                      ("tend", "<u4")], align=True)
assert HIT_DTYPE.itemsize == C.sizeof(_abi.HitT)


SORTED_AFFINE, SORTED_EXTEND_CUT = 0, 1


def sorted_batch(ctx: Context, calls: Sequence, scores: Sequence = ((2, 4, 4, 2),)) -> list:
    """The tie-break's sorted DP calls for many read segments in one batch (sf_sorted_batch).
    Each call: dict(read, texts, kind, band, and for SORTED_AFFINE mode; for
    SORTED_EXTEND_CUT end_bonus, xdrop, diagonal, window, cut (None: none), track_cut,
    bonus_within_cut; sc_index).  Returns per call the list of (whole, cut, cols)."""
    from .align import _aff
    pb = PoolBuilder()
    cs = (_abi.SortedCallT * max(1, len(calls)))()
    spans = []
    for i, k in enumerate(calls):
        c = cs[i]
        c.p_off = pb.add(k["read"])
        c.m = len(k["read"])
        c.first = len(spans)
        c.count = len(k["texts"])
        c.kind = int(k["kind"])
        c.mode = int(k.get("mode", 2))
        c.band = _abi.SF_NOLIMIT if k["band"] is None else int(k["band"])
        c.window = int(k.get("window", 0))
        cut = k.get("cut")
        c.cut = _abi.SF_NOLIMIT if cut is None else int(cut)
        c.end_bonus = int(k.get("end_bonus", 0))
        c.xdrop = int(k.get("xdrop", 2 ** 31 - 1))
        c.diagonal = int(bool(k.get("diagonal", False)))
        c.track_cut = int(bool(k.get("track_cut", True)))
        c.bonus_within_cut = int(bool(k.get("bonus_within_cut", False)))
        c.sc_index = int(k.get("sc_index", 0))
        for t in k["texts"]:
            spans.append((pb.add(t), len(t)))
    pool = pb.build()
    sp = (_abi.SpanT * max(1, len(spans)))(*[_abi.SpanT(o, n) for o, n in spans])
    sc = (_abi.Affine * max(1, len(scores)))(*[_aff(s) for s in scores])
    out = (_abi.CutT * max(1, len(spans)))()
    _abi.check(_abi.load().sf_sorted_batch(
        ctx.handle, pool.ctypes.data_as(C.POINTER(C.c_uint8)), pool.size, sc, len(scores), cs,
        len(calls), sp, len(spans), out))
    res, at = [], 0
    for k in calls:
        res.append([(int(out[at + q].whole), int(out[at + q].cut), int(out[at + q].cols))
                    for q in range(len(k["texts"]))])
        at += len(k["texts"])
    return res
