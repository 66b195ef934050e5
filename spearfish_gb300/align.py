"""The entry points of spearfish's ``map::align`` (crates/map/src/align.rs), computed on the
GPU through libsf_align.so.  Same names, argument meanings and results as the reference:

* sequences are byte codes (``&[u8]``: 0..3 = A, C, G, T; any buffer-protocol object or
  list of ints),
* ``band=None`` / ``cut=None`` stand for ``usize::MAX``,
* Myers' ``Option<u32>`` is ``int | None``,
* unreachable affine scores are ``NEG`` (``i32::MIN / 4``, align.rs:693).
"""
from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _abi

NEG = _abi.SF_NEG
U32_MAX = 0xFFFFFFFF
I32_MAX = 2 ** 31 - 1


class Mode(enum.IntEnum):
    """align.rs:40-45."""
    Infix = 0
    Prefix = 1
    Global = 2


@dataclass(frozen=True)
class Affine:
    """align.rs:660-691: +mat per match, -mis per mismatch, -(open + ext*l) per gap."""
    mat: int = 2
    mis: int = 4
    open: int = 4
    ext: int = 2

    def c(self) -> _abi.Affine:
        return _abi.Affine(self.mat, self.mis, self.open, self.ext)


Affine.ONT = Affine(2, 4, 4, 2)   # align.rs:678-683
Affine.HIFI = Affine(1, 4, 6, 2)  # align.rs:685-690


def _aff(sc) -> _abi.Affine:
    if isinstance(sc, Affine):
        return sc.c()
    if isinstance(sc, _abi.Affine):
        return sc
    return _abi.Affine(*[int(v) for v in sc])


def _codes(x) -> np.ndarray:
    if isinstance(x, np.ndarray) and x.dtype == np.uint8 and x.flags.c_contiguous:
        return x
    return np.ascontiguousarray(np.asarray(bytearray(x) if isinstance(x, (bytes, bytearray))
                                           else x, dtype=np.uint8))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint8)) if a.size else C.POINTER(C.c_uint8)()


def _band(b) -> int:
    return _abi.SF_NOLIMIT if b is None else int(b)


class _Texts:
    """An array of text pointers and lengths kept alive for one call."""

    def __init__(self, texts: Sequence):
        self.arrs = [_codes(t) for t in texts]
        self.ptrs = (C.POINTER(C.c_uint8) * max(1, len(self.arrs)))(*[_ptr(a) for a in self.arrs])
        self.lens = np.array([a.size for a in self.arrs] or [0], dtype=np.uint64)

    def args(self):
        return (self.ptrs, self.lens.ctypes.data_as(C.POINTER(C.c_uint64)), len(self.arrs))


class Pattern:
    """align.rs:68-85 `Pattern`: a pattern prepared once for several texts.  The match masks
    are built on the device per call; this keeps the codes."""

    def __init__(self, pattern):
        self.codes = _codes(pattern)
        self.m = int(self.codes.size)


def _lib():
    return _abi.load()


def distance(pattern, text, mode: Mode, k: int = U32_MAX) -> Optional[int]:
    """align.rs:88-91: edit distance in `mode`, or None if it exceeds `k`."""
    p, t = _codes(pattern), _codes(text)
    out = C.c_uint32()
    _abi.check(_lib().sf_distance(_ptr(p), p.size, _ptr(t), t.size, int(mode), int(k),
                                  C.byref(out)))
    return None if out.value == U32_MAX else int(out.value)


def distance_with(pat: Pattern, text, mode: Mode, k: int = U32_MAX) -> Optional[int]:
    """align.rs:93-168."""
    return distance(pat.codes, text, mode, k)


def batch_distances(pat: Pattern, texts: Sequence, mode: Mode, k: int = U32_MAX) -> list:
    """align.rs:174-200: `distance_with` for each text with one threshold."""
    if not texts:
        return []
    tx = _Texts(texts)
    out = np.zeros(len(texts), dtype=np.uint32)
    _abi.check(_lib().sf_batch_distances(_ptr(pat.codes), pat.m, *tx.args(), int(mode), int(k),
                                         out.ctypes.data_as(C.POINTER(C.c_uint32))))
    return [None if v == U32_MAX else int(v) for v in out]


def infix_distance(pattern, text) -> int:
    """align.rs:655-658."""
    return distance(pattern, text, Mode.Infix, U32_MAX)


def affine(pattern, text, mode: Mode, sc, band) -> int:
    """align.rs:699-701: best Gotoh score in `mode` within `band` (None: exact)."""
    p, t = _codes(pattern), _codes(text)
    out = C.c_int32()
    _abi.check(_lib().sf_affine(_ptr(p), p.size, _ptr(t), t.size, int(mode), C.byref(_aff(sc)),
                                _band(band), C.byref(out)))
    return int(out.value)


def affine_extend(pattern, text, sc, band, end_bonus: int, xdrop: int) -> int:
    """align.rs:710-729."""
    p, t = _codes(pattern), _codes(text)
    out = C.c_int32()
    _abi.check(_lib().sf_affine_extend(_ptr(p), p.size, _ptr(t), t.size, C.byref(_aff(sc)),
                                       _band(band), int(end_bonus), int(xdrop), C.byref(out)))
    return int(out.value)


def affine_extend_window(pattern, text, window: int, sc, band, end_bonus: int, xdrop: int):
    """align.rs:957-982: (score, pattern bases, text bases, text bases read)."""
    p, t = _codes(pattern), _codes(text)
    out = _abi.ExtendT()
    _abi.check(_lib().sf_affine_extend_window(_ptr(p), p.size, _ptr(t), t.size, int(window),
                                              C.byref(_aff(sc)), _band(band), int(end_bonus),
                                              int(xdrop), C.byref(out)))
    return (int(out.score), int(out.pattern_bases), int(out.text_bases), int(out.text_read))


def affine_sorted(pattern, texts: Sequence, mode: Mode, sc, band) -> list:
    """align.rs:854-861."""
    if not texts:
        return []
    p = _codes(pattern)
    tx = _Texts(texts)
    out = np.zeros(len(texts), dtype=np.int32)
    _abi.check(_lib().sf_affine_sorted(_ptr(p), p.size, *tx.args(), int(mode), C.byref(_aff(sc)),
                                       _band(band), out.ctypes.data_as(C.POINTER(C.c_int32))))
    return [int(v) for v in out]


def affine_extend_sorted_cut_bonus(pattern, texts: Sequence, sc, band, end_bonus: int,
                                   xdrop: int, diagonal: bool, window: int, cut,
                                   track_cut: bool, bonus_within_cut: bool) -> list:
    """align.rs:903-949: per text (whole, cut, cols)."""
    if not texts:
        return []
    p = _codes(pattern)
    tx = _Texts(texts)
    out = (_abi.CutT * len(texts))()
    _abi.check(_lib().sf_affine_extend_sorted_cut_bonus(
        _ptr(p), p.size, *tx.args(), C.byref(_aff(sc)), _band(band), int(end_bonus), int(xdrop),
        int(bool(diagonal)), int(window), _band(cut), int(bool(track_cut)),
        int(bool(bonus_within_cut)), out))
    return [(int(o.whole), int(o.cut), int(o.cols)) for o in out]


def affine_extend_sorted_cut(pattern, texts: Sequence, sc, band, end_bonus: int, xdrop: int,
                             diagonal: bool, window: int, cut) -> list:
    """align.rs:880-901."""
    return affine_extend_sorted_cut_bonus(pattern, texts, sc, band, end_bonus, xdrop, diagonal,
                                          window, cut, True, False)


def local_band_ends(read, text, sc, dlo: int, dhi: int, end_bonus) -> int:
    """align.rs:741-760 (`end_bonus` = (start, end))."""
    r, t = _codes(read), _codes(text)
    out = C.c_int32()
    _abi.check(_lib().sf_local_band_ends(_ptr(r), r.size, _ptr(t), t.size, C.byref(_aff(sc)),
                                         int(dlo), int(dhi), int(end_bonus[0]),
                                         int(end_bonus[1]), C.byref(out)))
    return int(out.value)


def local_band(read, text, sc, dlo: int, dhi: int, end_bonus: int) -> int:
    """align.rs:731-737."""
    return local_band_ends(read, text, sc, dlo, dhi, (end_bonus, end_bonus))


def dp_work() -> tuple[int, int]:
    """align.rs:2172-2176: (cells, rows) of this thread's affine passes."""
    c, r = C.c_uint64(), C.c_uint64()
    _lib().sf_dp_work(C.byref(c), C.byref(r))
    return int(c.value), int(r.value)


# ---- CIGARs (new: the reference computes no traceback) -------------------------------

OPS = "MIDNSHP=X"


def cigar_string(ops: Sequence[int]) -> str:
    return "".join(f"{o >> 4}{OPS[o & 15]}" for o in ops)


def _cigar_result(out: _abi.CigarT, ops: np.ndarray) -> dict:
    return {"score": int(out.score), "status": int(out.status),
            "pattern_end": int(out.pattern_end), "text_start": int(out.text_start),
            "text_end": int(out.text_end), "cigar": [int(v) for v in ops[:out.n_ops]]}


def affine_cigar(pattern, text, mode: Mode, sc, band) -> dict:
    """`affine` with the path of its best cell: score, end cell, CIGAR ops."""
    p, t = _codes(pattern), _codes(text)
    cap = p.size + t.size + 4
    ops = np.zeros(cap, dtype=np.uint32)
    out = _abi.CigarT()
    _abi.check(_lib().sf_affine_cigar(_ptr(p), p.size, _ptr(t), t.size, int(mode),
                                      C.byref(_aff(sc)), _band(band),
                                      ops.ctypes.data_as(C.POINTER(C.c_uint32)), cap,
                                      C.byref(out)))
    return _cigar_result(out, ops)


def affine_extend_window_cigar(pattern, text, window: int, sc, band, end_bonus: int,
                               xdrop: int) -> dict:
    """`affine_extend_window` with the path of the extension."""
    p, t = _codes(pattern), _codes(text)
    cap = p.size + t.size + 4
    ops = np.zeros(cap, dtype=np.uint32)
    out = _abi.CigarT()
    _abi.check(_lib().sf_affine_extend_window_cigar(
        _ptr(p), p.size, _ptr(t), t.size, int(window), C.byref(_aff(sc)), _band(band),
        int(end_bonus), int(xdrop), ops.ctypes.data_as(C.POINTER(C.c_uint32)), cap,
        C.byref(out)))
    return _cigar_result(out, ops)


def version() -> str:
    return _lib().sf_version().decode()
