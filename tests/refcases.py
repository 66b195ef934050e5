"""Shared cases for the parity tests: the reference's known answers, its proptest
generators restated with seeded numpy randomness, and checks that run against any
implementation of the ``map::align`` entry points (the oracle here, the CUDA library on
a GPU).

Implementations are objects with these methods (the reference's names, align.rs):
``distance``, ``batch_distances``, ``affine``, ``affine_extend``, ``affine_extend_window``,
``affine_sorted``, ``affine_extend_sorted_cut_bonus``, ``local_band_ends``.
"""
from __future__ import annotations

import json
import os

import numpy as np

MODES = {"Infix": 0, "Prefix": 1, "Global": 2}
INFIX, PREFIX, GLOBAL = 0, 1, 2
ONT = (2, 4, 4, 2)
HIFI = (1, 4, 6, 2)
I32_MAX = 2 ** 31 - 1
U32_MAX = 0xFFFFFFFF

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_kats.json")


def golden() -> dict:
    with open(GOLDEN) as f:
        return json.load(f)


class OracleImpl:
    """The oracle under the reference's entry-point names."""

    def __init__(self):
        import oracle
        self.o = oracle

    def distance(self, p, t, mode, k=U32_MAX):
        return self.o.myers_distance(p, t, mode, k)

    def batch_distances(self, p, texts, mode, k=U32_MAX):
        return [self.o.myers_distance(p, t, mode, k) for t in texts]

    def affine(self, p, t, mode, sc, band):
        return self.o.affine(p, t, mode, sc, band)

    def affine_extend(self, p, t, sc, band, end_bonus, xdrop):
        return self.o.affine_extend(p, t, sc, band, end_bonus, xdrop)

    def affine_extend_window(self, p, t, window, sc, band, end_bonus, xdrop):
        return self.o.affine_extend_window(p, t, window, sc, band, end_bonus, xdrop)

    def affine_sorted(self, p, texts, mode, sc, band):
        return self.o.affine_sorted(p, texts, mode, sc, band)

    def affine_extend_sorted_cut_bonus(self, p, texts, sc, band, end_bonus, xdrop, diagonal,
                                       window, cut, track_cut, bonus_within_cut):
        return self.o.affine_extend_sorted_cut_bonus(p, texts, sc, band, end_bonus, xdrop,
                                                     diagonal, window, cut, track_cut,
                                                     bonus_within_cut)

    def local_band_ends(self, read, t, sc, dlo, dhi, bonus):
        return self.o.local_band_ends(read, t, sc, dlo, dhi, tuple(bonus))


# ---- generators (restated from the reference's proptests) -------------------------

def rand_pair(n: int, div: int, seed: int):
    """align.rs:3503-3522 `rand_pair`: xorshift64 codes and a copy with ~1 edit in `div`."""
    mask = (1 << 64) - 1
    x = seed & mask

    def nxt():
        nonlocal x
        x ^= (x << 13) & mask
        x ^= x >> 7
        x ^= (x << 17) & mask
        return x

    t = [nxt() & 3 for _ in range(n)]
    p = []
    for b in t:
        r = nxt() % (3 * div)
        if r == 0:
            p.append((b + 1) & 3)
        elif r == 1:
            pass
        elif r == 2:
            p.extend([b, nxt() & 3])
        else:
            p.append(b)
    return p, t


def mutate(v, edits):
    """The proptests' edit loop (e.g. align.rs:3099-3104): (pos, base, kind)."""
    v = list(v)
    for pos, b, kind in edits:
        if not v:
            break
        i = pos % len(v)
        if kind == 0:
            v[i] = b
        elif kind == 1:
            v.insert(i, b)
        else:
            v.pop(i)
    return v


def rand_edits(rng, count, pos_max, base_max=4):
    return [(int(rng.integers(0, pos_max)), int(rng.integers(0, base_max)),
             int(rng.integers(0, 3))) for _ in range(count)]


def related(rng, tlen=(100, 500), plen=(60, 450), nedit=30):
    """`related_vs_naive`'s inputs (align.rs:3354-3365): a mutated substring of t."""
    t = rng.integers(0, 4, int(rng.integers(*tlen))).tolist()
    a, ln = int(rng.integers(0, 50)), int(rng.integers(*plen))
    end = min(a + ln, len(t))
    p = mutate(t[min(a, end):end], rand_edits(rng, int(rng.integers(0, nedit)), 500))
    return p, t


def affine_case(rng):
    """`affine_vs_naive`'s inputs (align.rs:3313-3323)."""
    t = rng.integers(0, 4, int(rng.integers(0, 200))).tolist()
    a, ln = int(rng.integers(0, 30)), int(rng.integers(0, 180))
    end = min(a + ln, len(t))
    p = mutate(t[min(a, end):end], rand_edits(rng, int(rng.integers(0, 20)), 200))
    return p, t


def sorted_texts(base, variants):
    """`sorted_batch_matches_single`'s texts (align.rs:3259-3268)."""
    texts = [list(base)]
    for keep, tail, cut in variants:
        k = min(keep, len(base))
        v = list(base[:k]) + list(tail) + list(base[k:])
        v = v[:max(0, len(v) - cut % 20)]
        texts.append(v)
    uniq = sorted({tuple(x) for x in texts})
    return [list(x) for x in uniq]


def narrow_texts(t, variants):
    """`narrow_cells_match_wide`'s texts (align.rs:3455-3465)."""
    texts = [list(t)]
    for keep, tail, drop in variants:
        k = min(keep, len(t))
        v = list(t[:k]) + list(tail) + list(t[k:])
        v = v[:max(0, len(v) - drop)]
        texts.append(v)
    uniq = sorted({tuple(x) for x in texts})
    return [list(x) for x in uniq]


# ---- checks ------------------------------------------------------------------

def check_kats(impl, kats=None):
    """Every KAT whose answer is a number, against `impl`."""
    kats = golden()["kats"] if kats is None else kats
    seg = []
    for c in kats:
        a, fn, want = c["args"], c["fn"], c["want"]
        if fn == "distance":
            got = impl.distance(a["p"], a["t"], MODES[a["mode"]], a["k"])
        elif fn == "affine":
            got = impl.affine(a["p"], a["t"], MODES[a["mode"]], a["sc"], a["band"])
        elif fn == "affine_extend":
            got = impl.affine_extend(a["p"], a["t"], a["sc"], a["band"], a["end_bonus"],
                                     a["xdrop"])
        elif fn == "affine_extend_end":
            r = impl.affine_extend_window(a["p"], a["t"], len(a["t"]), a["sc"], a["band"],
                                          a["end_bonus"], a["xdrop"])
            got = list(r[:3])
        elif fn == "local_band_ends":
            got = impl.local_band_ends(a["p"], a["t"], a["sc"], a["dlo"], a["dhi"], a["bonus"])
        elif fn == "segment_scores":
            left = impl.affine_extend(a["left_p"], a["left_t"], a["sc"], a["band"],
                                      a["end_bonus"], a["xdrop"])
            interior = impl.affine([], a["gap_t"], GLOBAL, a["sc"], a["band"])
            right = impl.affine_extend(a["right_p"], a["right_t"], a["sc"], a["band"],
                                       a["end_bonus"], a["xdrop"])
            got = [left, interior, right]
            seg.append(sum(got))
        elif fn == "segment_totals":
            got = seg
        else:
            continue
        assert got == want, (c["cite"], fn, got, want)


def check_window_relations(impl):
    """align.rs:3147-3181: a text cut anywhere after the bases read gives the same result,
    a text read to its end is matched only at that length, and bases past those read do not
    matter."""
    g = {c["fn"]: c for c in golden()["kats"]}
    a = g["affine_extend_window_cuts"]["args"]
    p, t = a["p"], a["t"]
    r = impl.affine_extend_window(p, t, len(t), a["sc"], a["band"], a["end_bonus"], a["xdrop"])
    assert r[3] < len(t)
    for cut in (r[3], r[3] + 1, len(t) - 1):
        x = impl.affine_extend_window(p, t[:cut], len(t), a["sc"], a["band"], a["end_bonus"],
                                      a["xdrop"])
        assert x[0] == r[0]
    short = impl.affine_extend_window(p, t[:40], len(t), a["sc"], a["band"], a["end_bonus"],
                                      a["xdrop"])
    assert (short[2], short[3]) == (40, 40)
    a = g["affine_extend_end_reads_a_prefix"]["args"]
    p, t = a["p"], a["t"]
    r = impl.affine_extend_window(p, t, len(t), a["sc"], a["band"], a["end_bonus"], a["xdrop"])
    assert r[3] < len(t)
    u = list(t)
    for i in range(r[3], len(u)):
        u[i] = 3 - u[i]
    assert impl.affine_extend_window(p, u, len(u), a["sc"], a["band"], a["end_bonus"],
                                     a["xdrop"]) == r


class GpuImpl:
    """The CUDA library's one-call entry points (spearfish_gb300.align)."""

    def __init__(self):
        from spearfish_gb300 import align as A
        self.A = A

    def distance(self, p, t, mode, k=U32_MAX):
        return self.A.distance(p, t, mode, k)

    def batch_distances(self, p, texts, mode, k=U32_MAX):
        return self.A.batch_distances(self.A.Pattern(p), texts, mode, k)

    def affine(self, p, t, mode, sc, band):
        return self.A.affine(p, t, mode, sc, band)

    def affine_extend(self, p, t, sc, band, end_bonus, xdrop):
        return self.A.affine_extend(p, t, sc, band, end_bonus, xdrop)

    def affine_extend_window(self, p, t, window, sc, band, end_bonus, xdrop):
        return self.A.affine_extend_window(p, t, window, sc, band, end_bonus, xdrop)

    def affine_sorted(self, p, texts, mode, sc, band):
        return self.A.affine_sorted(p, texts, mode, sc, band)

    def affine_extend_sorted_cut_bonus(self, p, texts, sc, band, end_bonus, xdrop, diagonal,
                                       window, cut, track_cut, bonus_within_cut):
        return self.A.affine_extend_sorted_cut_bonus(p, texts, sc, band, end_bonus, xdrop,
                                                     diagonal, window, cut, track_cut,
                                                     bonus_within_cut)

    def local_band_ends(self, read, t, sc, dlo, dhi, bonus):
        return self.A.local_band_ends(read, t, sc, dlo, dhi, tuple(bonus))
