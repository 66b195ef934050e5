// Traceback walk (no reference counterpart: spearfish computes no alignment path).  The warp
// that computed a pass walks it right after, from the end cell back to row 0 / column 0
// through the decision bits the pass stored, with the tie order they encode (H from H'
// before E, diagonal before vertical, opening before extending), writing the CIGAR
// run-length encoded, BAM-style (len << 4 | op), end first (the compaction reverses it).
//
// The warp caches the word pairs of 32 rows at one column slot, one row per lane, so a step
// costs two shuffles, not a memory round trip; a refill (a path that leaves the slot or the
// 32 rows) is one coalesced-free load per lane whose latency other warps' rows hide.  Paths
// run mostly diagonally, and along a diagonal of the banded rows (lo moving right by one per
// row) a cell keeps its band offset: every lane decodes its own row's cell at that offset,
// and one ballot gives the whole run of diagonal steps, taken in one iteration.  Reads stay
// inside the pass's rows; a path that leaves the band reports "no path".
#pragma once
#include "sf_internal.cuh"

namespace {

using namespace sf;

// Where band offset K of a row sits in the traceback layout: chunk qc (wide rows), lane L,
// cell c of the lane -- kept incrementally as the walk moves (offsets change by -1, 0 or +1
// per step), so no step divides.
struct Pos {
  int32_t qc, L, c;
};

struct TbLayout {
  int32_t C, C2, TG;
  bool wide, p16;
  int32_t lanes;  // lanes of a pass: 32; 16 for the half-warp, 64 for the two-warp 16-bit rows
  uint32_t row;   // word pairs per row

  __device__ __forceinline__ Pos at(int32_t K) const {
    Pos p;
    p.qc = wide ? K / (32 * C) : 0;
    const int32_t r = K - p.qc * 32 * C;
    p.L = r / C;
    p.c = r - p.L * C;
    return p;
  }
  // Lanes wrap into the next chunk only in wide rows; a register row's lanes (16, 32 or 64
  // of them) hold its whole band.
  __device__ __forceinline__ void move(Pos& p, int32_t delta) const {
    p.c += delta;
    if (p.c < 0) {
      p.c += C;
      if (--p.L < 0 && wide) {
        p.L += 32;
        --p.qc;
      }
    } else if (p.c >= C) {
      p.c -= C;
      if (++p.L >= 32 && wide) {
        p.L -= 32;
        ++p.qc;
      }
    }
  }
  // Word pair of the cell within its row, and the cell's bit position in it.
  __device__ __forceinline__ int32_t slot(const Pos& p, int& sh) const {
    if (p16) {
      const int hi = p.c >= C2, k = hi ? p.c - C2 : p.c;
      const int g = k >> 3, t = k & 7;
      sh = 8 * hi + t;
      return g * lanes + p.L;
    }
    const int g = p.c >> 4, q = p.c & 15;
    const int gs = (C - 16 * g) < 16 ? (C - 16 * g) : 16;
    sh = 2 * (gs - 1 - q);
    return p.qc * TG * 32 + g * 32 + p.L;
  }
  // The cell's decisions as a nibble: bit 0 "H' came from F", bit 1 "H came from E",
  // bit 2 "E opened", bit 3 "F opened".
  __device__ __forceinline__ uint32_t decode(uint2 w, int sh) const {
    if (p16) {
      // A: bytes (F extended lo, hi, diagonal lost lo, hi); B: (E extended .., H from E ..).
      const uint32_t f_ext = (w.x >> sh) & 1u, dg_lost = (w.x >> (sh + 16)) & 1u;
      const uint32_t e_ext = (w.y >> sh) & 1u, from_e = (w.y >> (sh + 16)) & 1u;
      return dg_lost | (from_e << 1) | ((e_ext ^ 1u) << 2) | ((f_ext ^ 1u) << 3);
    }
    // Two bits per cell and plane word: A (F extended, diagonal lost), B (E extended, H
    // from E).
    const uint32_t a = (w.x >> sh) & 3u, b = (w.y >> sh) & 3u;
    return (a & 1u) | ((b & 1u) << 1) | (((b >> 1) ^ 1u) << 2) | (((a >> 1) ^ 1u) << 3);
  }
};


template <int C>
__device__ __forceinline__ TbLayout tb_layout(bool wide, bool p16, const DJob& J, uint32_t flags,
                                              int lanes = 32) {
  TbLayout Y;
  Y.C = C;
  Y.C2 = C / 2;
  Y.TG = (C + 15) / 16;
  Y.wide = wide;
  Y.p16 = p16;
  Y.lanes = lanes;
  const int64_t chunks = wide ? wide_chunks(C, band_wmax(J, flags)) : 1;
  Y.row = (uint32_t)(tb_row_words(C, chunks) / 2 * lanes / 32);
  return Y;
}

// Walks pass jid (the whole warp, after its rows): geometry `full`, `below`, `above`, n.
__device__ void walk_lean(const sfk::AffLaunch& a, uint32_t jid, const TbLayout& Y, const DJob& J,
                          uint32_t flags, const DRes& R, int lane) {
  const TJob T = a.tjobs[jid];
  const uint2* tb = reinterpret_cast<const uint2*>(a.tb + J.tb_word);
  const bool full = (flags & F_FULL) != 0;
  const int64_t kcap = int64_t(1) << 30;
  const int32_t below = (int32_t)(J.below > kcap ? kcap : J.below);
  const int32_t above = (int32_t)(J.above > kcap ? kcap : J.above);
  const int32_t m = (int32_t)J.m, n = (int32_t)J.n;
  auto lo_of = [&](int32_t i) { return full ? 0 : (i > below ? i - below : 0); };
  auto hi_of = [&](int32_t i) { return full ? n : (i + above < n ? i + above : n); };
  // End cell (align.rs:2643-2650 score_col; 975-981 the window's choice).
  int32_t score, ei, ej, tail = 0;
  bool ok = true;
  if (T.kind == 0) {
    score = R.score;
    ei = m;
    ej = (int32_t)R.score_col;
    ok = R.score > NEG / 2;
  } else {
    const int32_t whole = sat_add(R.score, T.end_bonus);
    if (R.clip_best >= whole) {
      score = R.clip_best;
      ei = (int32_t)R.clip_i;
      ej = (int32_t)R.clip_j;
      tail = m - ei;
    } else {
      score = whole;
      ei = m;
      ej = (int32_t)R.score_col;
      ok = R.score > NEG / 2;
    }
  }
  uint32_t* out = a.ops + T.ops_off;
  const uint32_t cap = T.ops_cap;
  uint32_t n_ops = 0, cur_op = 15, cur_len = 0;
  int status = ok ? 0 : 1;
  auto flush = [&]() {
    if (cur_len == 0) return;
    if (n_ops == cap) {
      status = -1;
      return;
    }
    if (lane == 0) out[n_ops] = (cur_len << 4) | cur_op;
    ++n_ops;
  };
  auto push = [&](uint32_t op, uint32_t len) {
    if (len == 0 || status) return;
    if (op == cur_op) {
      cur_len += len;
      return;
    }
    flush();
    cur_op = op;
    cur_len = len;
  };
  int32_t text_start = 0;
  if (ok) {
    push(4, (uint32_t)tail);
    int32_t i = ei, j = ej;
    int state = 0;  // 0 H, 1 E, 2 F
    int32_t K = j - lo_of(i);
    Pos pos = Y.at(K > 0 ? K : 0);
    int32_t rbase = -64, S = -1;  // lane q caches row rbase - q at word pair S
    uint2 cw = make_uint2(0, 0);
    const int64_t guard = 2 * ((int64_t)m + n) + 8;
    for (int64_t it = 0; !status; ++it) {
      if (it > guard) {
        status = 1;
        break;
      }
      if (state == 0 && i == 0) {
        if ((flags & F_MODE) == 0)
          text_start = j;
        else
          push(2, (uint32_t)j);
        break;
      }
      if (state == 0 && j == 0) {
        push(1, (uint32_t)i);
        break;
      }
      if (i <= 0 || j <= 0 || K < 0 || j > hi_of(i)) {
        status = 1;
        break;
      }
      int sh;
      const int32_t s = Y.slot(pos, sh);
      if (s != S || i > rbase || i <= rbase - 32) {
        rbase = i;
        S = s;
        const int32_t r = i - lane;
        cw = r >= 1 ? tb[(uint64_t)(r - 1) * Y.row + (uint32_t)S] : make_uint2(0, 0);
      }
      const int p = rbase - i;
      const uint2 w = make_uint2(__shfl_sync(FULL, cw.x, p), __shfl_sync(FULL, cw.y, p));
      const uint32_t nib = Y.decode(w, sh);
      const int32_t d = lo_of(i) - lo_of(i - 1);  // 0 or 1: how lo moves up to row i - 1
      int32_t delta = 0;
      if (state == 0) {
        if (nib & 2u) {
          state = 1;
        } else if (!(nib & 1u)) {
          // A diagonal run: rows i, i - 1, ... keep band offset K while lo moves by one per
          // row (rows above `below`), so each lane's cached row decodes the same cell.
          int32_t run = 1;
          if (!full && i - 1 > below) {
            const uint32_t mine = Y.decode(cw, sh);
            const uint32_t diag = __ballot_sync(FULL, (mine & 3u) == 0u) >> p;
            run = __ffs(~diag) - 1;  // consecutive diagonal rows from row i (>= 1)
            if (run < 0) run = 32 - p;
            const int32_t lim = i - below;  // rows i .. below + 1 keep the offset
            run = run < lim ? run : lim;
            run = run < j ? run : j;
            run = run < i ? run : i;
          }
          push(0, (uint32_t)run);
          if (run == 1) delta = d - 1;
          i -= run;
          j -= run;
        } else {
          state = 2;
        }
      } else if (state == 1) {
        push(2, 1);
        state = (nib & 4u) ? 0 : 1;
        --j;
        delta = -1;
      } else {
        push(1, 1);
        state = (nib & 8u) ? 0 : 2;
        --i;
        delta = d;
      }
      K += delta;
      if (K >= 0 && delta != 0) Y.move(pos, delta);
    }
    if (!status) flush();
  }
  if (lane == 0) {
    TRes tr;
    tr.score = score;
    tr.status = status;
    tr.end_i = (uint32_t)ei;
    tr.end_j = (uint32_t)ej;
    tr.text_start = (uint32_t)text_start;
    tr.n_ops = status == 0 ? n_ops : 0;
    a.tres[jid] = tr;
  }
}

}  // namespace
