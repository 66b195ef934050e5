"""CPU oracle for the spearfish alignment stage -- TEST INFRASTRUCTURE ONLY.

A plain-C restatement of ``crates/map/src/align.rs`` (spearfish v0.3.2), loaded
through ctypes.  Tests use it as the checker for the CUDA path; the bench uses it
as the timed CPU baseline / reference arm.  The product package never imports it.

Sequences are byte codes (0..3 for A, C, G, T; local-band reads may hold 4+ for an
ambiguous base), as the reference's ``&[u8]`` inputs.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

from . import build as _build

INFIX, PREFIX, GLOBAL = 0, 1, 2
NEG = -(2 ** 31) // 4
NOLIMIT = (1 << 64) - 1
OP_M, OP_I, OP_D, OP_S = 0, 1, 2, 4
TB_AFFINE, TB_EXTEND = 0, 1

ONT = (2, 4, 4, 2)   # align.rs:678-683
HIFI = (1, 4, 6, 2)  # align.rs:685-690


class Affine(C.Structure):
    _fields_ = [("mat", C.c_int32), ("mis", C.c_int32), ("open", C.c_int32), ("ext", C.c_int32)]


class ExtendOpts(C.Structure):
    _fields_ = [("pad", C.c_uint64), ("pad_div", C.c_uint64), ("xdrop", C.c_int32),
                ("end_bonus", C.c_int32)]


class Dp(C.Structure):
    _fields_ = [("score", C.c_int32), ("clip_best", C.c_int32), ("cut_best", C.c_int32),
                ("cut_score", C.c_int32), ("score_col", C.c_uint64), ("clip_i", C.c_uint64),
                ("clip_j", C.c_uint64), ("text_read", C.c_uint64), ("last_row", C.c_uint64),
                ("cells", C.c_uint64), ("rows", C.c_uint64)]


class Tb(C.Structure):
    _fields_ = [("score", C.c_int32), ("status", C.c_int32), ("end_i", C.c_uint64),
                ("end_j", C.c_uint64), ("text_start", C.c_uint64), ("n_ops", C.c_uint64)]


_lib = None

_u8p = C.POINTER(C.c_uint8)
_u64p = C.POINTER(C.c_uint64)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)
_u32p = C.POINTER(C.c_uint32)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.or_myers_distance.restype = C.c_int64
        L.or_myers_distance.argtypes = [_u8p, C.c_uint64, _u8p, C.c_uint64, C.c_int, C.c_uint32]
        L.or_myers_naive.restype = C.c_uint32
        L.or_myers_naive.argtypes = [_u8p, C.c_uint64, _u8p, C.c_uint64, C.c_int]
        L.or_myers_batch_lanes.restype = None
        L.or_myers_batch_lanes.argtypes = [_u8p, C.c_uint64, _u8p, _u64p, _u64p, C.c_uint64,
                                           C.c_int, C.c_int, C.c_uint32, _i64p]
        L.or_affine_dp.restype = None
        L.or_affine_dp.argtypes = [_u8p, C.c_uint64, _u8p, C.c_uint64, C.c_int,
                                   C.POINTER(Affine), C.c_uint64, C.c_uint64, C.c_int,
                                   C.c_int32, C.c_int, C.c_uint64, C.POINTER(Dp)]
        L.or_affine.restype = C.c_int32
        L.or_affine.argtypes = [_u8p, C.c_uint64, _u8p, C.c_uint64, C.c_int, C.POINTER(Affine),
                                C.c_uint64]
        L.or_affine_extend.restype = C.c_int32
        L.or_affine_extend.argtypes = [_u8p, C.c_uint64, _u8p, C.c_uint64, C.POINTER(Affine),
                                       C.c_uint64, C.c_int32, C.c_int32]
        L.or_affine_extend_window.restype = None
        L.or_affine_extend_window.argtypes = [_u8p, C.c_uint64, _u8p, C.c_uint64, C.c_uint64,
                                              C.POINTER(Affine), C.c_uint64, C.c_int32,
                                              C.c_int32, _i64p]
        L.or_affine_extend_sorted_cut_bonus.restype = None
        L.or_affine_extend_sorted_cut_bonus.argtypes = [
            _u8p, C.c_uint64, _u8p, _u64p, _u64p, C.c_uint64, C.POINTER(Affine), C.c_uint64,
            C.c_int32, C.c_int32, C.c_int, C.c_uint64, C.c_uint64, C.c_int, C.c_int, _i64p]
        L.or_affine_sorted.restype = None
        L.or_affine_sorted.argtypes = [_u8p, C.c_uint64, _u8p, _u64p, _u64p, C.c_uint64, C.c_int,
                                       C.POINTER(Affine), C.c_uint64, _i32p]
        L.or_local_band_ends.restype = C.c_int32
        L.or_local_band_ends.argtypes = [_u8p, C.c_uint64, _u8p, C.c_uint64, C.POINTER(Affine),
                                         C.c_int64, C.c_int64, C.c_int32, C.c_int32]
        L.or_naive_affine.restype = C.c_int32
        L.or_naive_affine.argtypes = [_u8p, C.c_uint64, _u8p, C.c_uint64, C.c_int,
                                      C.POINTER(Affine)]
        L.or_naive_extend.restype = C.c_int32
        L.or_naive_extend.argtypes = [_u8p, C.c_uint64, _u8p, C.c_uint64, C.POINTER(Affine)]
        L.or_naive_local.restype = C.c_int32
        L.or_naive_local.argtypes = [_u8p, C.c_uint64, _u8p, C.c_uint64, C.POINTER(Affine),
                                     C.c_int32, C.c_int32]
        L.or_naive_local_band.restype = C.c_int32
        L.or_naive_local_band.argtypes = [_u8p, C.c_uint64, _u8p, C.c_uint64, C.POINTER(Affine),
                                          C.c_int64, C.c_int64, C.c_int32, C.c_int32]
        L.or_affine_traceback.restype = None
        L.or_affine_traceback.argtypes = [_u8p, C.c_uint64, _u8p, C.c_uint64, C.c_int, C.c_int,
                                          C.POINTER(Affine), C.c_uint64, C.c_uint64, C.c_int32,
                                          C.c_int32, _u32p, C.c_uint64, C.POINTER(Tb)]
        L.or_cigar_score.restype = C.c_int64
        L.or_cigar_score.argtypes = [_u8p, C.c_uint64, _u8p, C.c_uint64, _u32p, C.c_uint64,
                                     C.c_uint64, C.POINTER(Affine), _u64p, _u64p]
        L.or_set_level.restype = C.c_int
        L.or_set_level.argtypes = [C.c_int]
        L.or_get_level.restype = C.c_int
        L.or_get_level.argtypes = []
        L.or_run_pairs.restype = C.c_uint64
        L.or_run_pairs.argtypes = [C.c_int, C.c_int, _u8p, _u64p, _u64p, _u8p, _u64p, _u64p,
                                   C.c_uint64, C.c_int, C.c_uint32, C.POINTER(C.c_uint32),
                                   C.POINTER(Affine), C.c_uint64, _u64p, C.POINTER(ExtendOpts),
                                   _i64p, _u64p]
        L.or_check_cigars.restype = C.c_uint64
        L.or_check_cigars.argtypes = [C.c_int, _u8p, _u64p, _u64p, _u8p, _u64p, _u64p,
                                      C.c_uint64, _u32p, _u64p, _u32p, _u64p, _u64p, _i32p,
                                      C.POINTER(Affine), _i32p]
        _lib = L
    return _lib


def _seq(x) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(x, dtype=np.uint8))
    if a.size == 0:
        a = np.zeros(1, dtype=np.uint8)[:0]
    return a


def _p(a: np.ndarray, t=_u8p):
    # A valid pointer even for empty arrays (never dereferenced then).
    if a.size == 0:
        return C.cast(C.c_void_p(0), t)
    return a.ctypes.data_as(t)


def _sc(sc) -> Affine:
    if isinstance(sc, Affine):
        return sc
    return Affine(*[int(v) for v in sc])


def _band(b) -> int:
    return NOLIMIT if b is None else int(b)


def _pack(texts: Sequence) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    arrs = [_seq(t) for t in texts]
    lens = np.array([a.size for a in arrs], dtype=np.uint64)
    offs = np.zeros(len(arrs), dtype=np.uint64)
    if len(arrs) > 1:
        offs[1:] = np.cumsum(lens[:-1])
    cat = np.concatenate(arrs) if arrs and lens.sum() > 0 else np.zeros(1, dtype=np.uint8)
    return np.ascontiguousarray(cat, dtype=np.uint8), offs, lens


# ---- Myers -----------------------------------------------------------------

def myers_distance(p, t, mode: int, k: int = 0xFFFFFFFF) -> Optional[int]:
    p, t = _seq(p), _seq(t)
    d = lib().or_myers_distance(_p(p), p.size, _p(t), t.size, mode, k)
    return None if d < 0 else int(d)


def myers_naive(p, t, mode: int) -> int:
    p, t = _seq(p), _seq(t)
    return int(lib().or_myers_naive(_p(p), p.size, _p(t), t.size, mode))


def myers_batch_lanes(p, texts, mode: int, k: int, lanes: int) -> list[Optional[int]]:
    p = _seq(p)
    cat, offs, lens = _pack(texts)
    out = np.zeros(len(texts), dtype=np.int64)
    lib().or_myers_batch_lanes(_p(p), p.size, _p(cat), _p(offs, _u64p), _p(lens, _u64p),
                               len(texts), lanes, mode, k, _p(out, _i64p))
    return [None if d < 0 else int(d) for d in out]


# ---- Affine ----------------------------------------------------------------

def affine_dp(p, t, mode: int, sc, band, geom: Optional[int] = None, clip=None,
              cut: Optional[int] = None) -> dict:
    """One `run_core` pass; clip = (xdrop, cell) or None."""
    p, t = _seq(p), _seq(t)
    d = Dp()
    g = t.size if geom is None else int(geom)
    c = clip is not None
    xd, cell = (clip if c else (0, False))
    lib().or_affine_dp(_p(p), p.size, _p(t), t.size, mode, C.byref(_sc(sc)), _band(band), g,
                       int(c), int(xd), int(bool(cell)), NOLIMIT if cut is None else int(cut),
                       C.byref(d))
    return {f: getattr(d, f) for f, _ in Dp._fields_}


def affine(p, t, mode: int, sc, band) -> int:
    p, t = _seq(p), _seq(t)
    return int(lib().or_affine(_p(p), p.size, _p(t), t.size, mode, C.byref(_sc(sc)),
                               _band(band)))


def affine_extend(p, t, sc, band, end_bonus: int, xdrop: int) -> int:
    p, t = _seq(p), _seq(t)
    return int(lib().or_affine_extend(_p(p), p.size, _p(t), t.size, C.byref(_sc(sc)),
                                      _band(band), end_bonus, xdrop))


def affine_extend_window(p, t, window: int, sc, band, end_bonus: int, xdrop: int):
    p, t = _seq(p), _seq(t)
    out = np.zeros(4, dtype=np.int64)
    lib().or_affine_extend_window(_p(p), p.size, _p(t), t.size, window, C.byref(_sc(sc)),
                                  _band(band), end_bonus, xdrop, _p(out, _i64p))
    return tuple(int(v) for v in out)


def affine_extend_sorted_cut_bonus(p, texts, sc, band, end_bonus, xdrop, diagonal, window,
                                   cut, track_cut, bonus_within_cut):
    p = _seq(p)
    cat, offs, lens = _pack(texts)
    out = np.zeros(3 * len(texts), dtype=np.int64)
    lib().or_affine_extend_sorted_cut_bonus(
        _p(p), p.size, _p(cat), _p(offs, _u64p), _p(lens, _u64p), len(texts),
        C.byref(_sc(sc)), _band(band), end_bonus, xdrop, int(diagonal), int(window),
        NOLIMIT if cut is None else int(cut), int(track_cut), int(bonus_within_cut),
        _p(out, _i64p))
    return [tuple(int(v) for v in out[3 * q:3 * q + 3]) for q in range(len(texts))]


def affine_sorted(p, texts, mode, sc, band) -> list[int]:
    p = _seq(p)
    cat, offs, lens = _pack(texts)
    out = np.zeros(len(texts), dtype=np.int32)
    lib().or_affine_sorted(_p(p), p.size, _p(cat), _p(offs, _u64p), _p(lens, _u64p),
                           len(texts), mode, C.byref(_sc(sc)), _band(band), _p(out, _i32p))
    return [int(v) for v in out]


def local_band_ends(read, t, sc, dlo: int, dhi: int, bonus: tuple[int, int]) -> int:
    r, t = _seq(read), _seq(t)
    return int(lib().or_local_band_ends(_p(r), r.size, _p(t), t.size, C.byref(_sc(sc)),
                                        dlo, dhi, bonus[0], bonus[1]))


def local_band(read, t, sc, dlo: int, dhi: int, end_bonus: int) -> int:
    return local_band_ends(read, t, sc, dlo, dhi, (end_bonus, end_bonus))


def naive_affine(p, t, mode, sc) -> int:
    p, t = _seq(p), _seq(t)
    return int(lib().or_naive_affine(_p(p), p.size, _p(t), t.size, mode, C.byref(_sc(sc))))


def naive_extend(p, t, sc) -> int:
    p, t = _seq(p), _seq(t)
    return int(lib().or_naive_extend(_p(p), p.size, _p(t), t.size, C.byref(_sc(sc))))


def naive_local(p, t, sc, bonus) -> int:
    p, t = _seq(p), _seq(t)
    return int(lib().or_naive_local(_p(p), p.size, _p(t), t.size, C.byref(_sc(sc)),
                                    bonus[0], bonus[1]))


def naive_local_band(p, t, sc, dlo, dhi, bonus) -> int:
    p, t = _seq(p), _seq(t)
    return int(lib().or_naive_local_band(_p(p), p.size, _p(t), t.size, C.byref(_sc(sc)),
                                         dlo, dhi, bonus[0], bonus[1]))


# ---- Traceback ----------------------------------------------------------------

def traceback(p, t, kind: int, mode: int, sc, band, window: int = 0, end_bonus: int = 0,
              xdrop: int = 2 ** 31 - 1) -> dict:
    p, t = _seq(p), _seq(t)
    cap = p.size + t.size + 4
    cig = np.zeros(cap, dtype=np.uint32)
    tb = Tb()
    lib().or_affine_traceback(_p(p), p.size, _p(t), t.size, kind, mode, C.byref(_sc(sc)),
                              _band(band), window, end_bonus, xdrop, _p(cig, _u32p), cap,
                              C.byref(tb))
    r = {f: getattr(tb, f) for f, _ in Tb._fields_}
    r["cigar"] = [int(v) for v in cig[:tb.n_ops]] if tb.status == 0 else []
    return r


def cigar_score(p, t, cigar, text_start: int, sc):
    p, t = _seq(p), _seq(t)
    cg = np.ascontiguousarray(np.asarray(cigar, dtype=np.uint32))
    pu, te = C.c_uint64(), C.c_uint64()
    s = lib().or_cigar_score(_p(p), p.size, _p(t), t.size, _p(cg, _u32p), cg.size, text_start,
                             C.byref(_sc(sc)), C.byref(pu), C.byref(te))
    return int(s), int(pu.value), int(te.value)


def cigar_string(cigar) -> str:
    return "".join(f"{c >> 4}{'MIDNSHP=X'[c & 15]}" for c in cigar)


# ---- CPU baseline -------------------------------------------------------------

def set_level(level: int) -> int:
    return int(lib().or_set_level(level))


def run_pairs(kind: int, threads: int, pseq, poff, plen, tseq, toff, tlen, mode: int,
              k: int = 0xFFFFFFFF, sc=ONT, band=None, kv=None,
              extend: Optional[tuple] = None, bands=None,
              per_pair_cells: bool = False):
    """All pairs on `threads` host threads; returns (per-pair result, cells), or (per-pair
    result, per-pair cells) with per_pair_cells.  kind 0: Myers (cap k, or per pair kv);
    1: affine; 2: extend window, extend = (pad, pad_div, xdrop, end_bonus).  bands: a band
    per pair (instead of `band`)."""
    count = len(plen)
    out = np.zeros(count, dtype=np.int64)
    arrs = [np.ascontiguousarray(a, dtype=dt) for a, dt in
            ((pseq, np.uint8), (poff, np.uint64), (plen, np.uint64), (tseq, np.uint8),
             (toff, np.uint64), (tlen, np.uint64))]
    kva = None if kv is None else np.ascontiguousarray(kv, dtype=np.uint32)
    bva = None if bands is None else np.ascontiguousarray(bands, dtype=np.uint64)
    cpp = np.zeros(count, dtype=np.uint64) if per_pair_cells else None
    ext = ExtendOpts(*extend) if extend is not None else None
    cells = lib().or_run_pairs(kind, threads, _p(arrs[0]), _p(arrs[1], _u64p),
                               _p(arrs[2], _u64p), _p(arrs[3]), _p(arrs[4], _u64p),
                               _p(arrs[5], _u64p), count, mode, k,
                               None if kva is None else _p(kva, C.POINTER(C.c_uint32)),
                               C.byref(_sc(sc)), _band(band),
                               None if bva is None else _p(bva, _u64p),
                               None if ext is None else C.byref(ext), _p(out, _i64p),
                               None if cpp is None else _p(cpp, _u64p))
    if per_pair_cells:
        return out, cpp
    return out, int(cells)


def check_cigars(threads: int, pseq, poff, plen, tseq, toff, tlen, ops, cig_off, n_ops,
                 text_start, text_end, score, sc=ONT) -> np.ndarray:
    """Re-scores every pair's CIGAR (or_check_cigars); returns a code per pair: 0 the path
    consumes the pattern, ends at text_end and scores `score`; 1 another score; 2 the
    pattern not consumed exactly; 3 another text end; 4 an op outside the sequences."""
    count = len(plen)
    code = np.zeros(count, dtype=np.int32)
    a = [np.ascontiguousarray(x, dtype=dt) for x, dt in
         ((pseq, np.uint8), (poff, np.uint64), (plen, np.uint64), (tseq, np.uint8),
          (toff, np.uint64), (tlen, np.uint64), (ops, np.uint32), (cig_off, np.uint64),
          (n_ops, np.uint32), (text_start, np.uint64), (text_end, np.uint64),
          (score, np.int32))]
    lib().or_check_cigars(threads, _p(a[0]), _p(a[1], _u64p), _p(a[2], _u64p), _p(a[3]),
                          _p(a[4], _u64p), _p(a[5], _u64p), count, _p(a[6], _u32p),
                          _p(a[7], _u64p), _p(a[8], _u32p), _p(a[9], _u64p), _p(a[10], _u64p),
                          _p(a[11], _i32p), C.byref(_sc(sc)), _p(code, _i32p))
    return code


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1
