// Banded affine (Gotoh) passes -- align.rs:2446-2666 `run_core` and align.rs:783-852
// `local_band_core` -- one warp per pass.  Included by the per-C translation units
// (sf_aff_c*.cu), which nvcc compiles in parallel.
//
// Row i covers text columns [lo_i, hi_i]; from one row to the next lo moves right by 0 or
// 1 (d), so band offset K = j - lo_i reads the previous row at offsets K + d - 1 (diagonal)
// and K + d (vertical).  Lane l keeps offsets [l*C, l*C + C) of the previous row's H and F
// in registers (wide rows: in a global scratch row, 32*C offsets per chunk) and per row
//   pass 1  (in lane)  F = max(Hup - go, Fup - ext, NEG); H' = max(Hdiag + s, F, floor)
//                      and the lane's own horizontal-gap chain,
//   scan    (warp)     the gap value entering each lane: a prefix max in which a value
//                      decays by ext per column (one shuffle + one DPX max per step),
//   pass 2  (in lane)  E = max(entering - ext*c, own chain); H = max(H', E).
// This is the reference row (align.rs:1027-1072): E[k] = max(e - ext*k,
// max_{k'<k} H'[k'] - go - ext*(k-k'-1)), written as a recurrence in the same i32
// arithmetic, so every cell -- NEG-adjacent ones included -- equals the reference's.
// The per-row bookkeeping (row maximum, leftmost best cell, X-drop stop, cut maxima) runs
// after each row, in row order, as the reference does.
//
// Traceback: four decisions per cell -- "F extended" (vs opened from H above), "diagonal
// lost" (H' came from F), "E extended" (vs opened from H' on the left), "H came from E" --
// kept as sign bits in bit-plane words (tb_push), stored per row as one (A, B) word pair per
// lane and 16 cells, lane-fastest; the same warp then walks them into a CIGAR (sf_walk.cuh).
#pragma once
#include <type_traits>

#include "sf_internal.cuh"
#include "sf_walk.cuh"

namespace {

using namespace sf;

struct Geo {
  bool full, local;
  int64_t below, above;  // local: dlo, dhi
  int64_t n;
  // Row i's columns [lo, hi] (hi < lo: an empty row, local band only).
  __device__ __forceinline__ void range(int64_t i, int64_t& lo, int64_t& hi) const {
    if (local) {
      // align.rs:800-805 `rng` (half-open there).
      int64_t l = i + below, h = i + above + 1;
      l = l < 0 ? 0 : (l > n + 1 ? n + 1 : l);
      h = h < 0 ? 0 : (h > n + 1 ? n + 1 : h);
      if (h < l) h = l;
      lo = l;
      hi = h - 1;
    } else if (full) {
      lo = 0;
      hi = n;
    } else {
      // align.rs:2462-2468 `range`.
      lo = i > below ? i - below : 0;
      hi = i + above < n ? i + above : n;
    }
  }
};

template <int C>
struct Win {
  static constexpr int NW = (C + 15) / 16;
  uint32_t w[NW];
  // Text bases of columns s .. s + C - 1 (packed position = column; the pad sits at 0).
  __device__ __forceinline__ void load(const uint32_t* __restrict__ pool, uint64_t t_word,
                                       int64_t s) {
    const uint64_t wi = t_word + ((uint64_t)s >> 4);
    const uint32_t sh = 2u * ((uint32_t)s & 15u);
    uint32_t prev = __ldg(pool + wi);
#pragma unroll
    for (int g = 0; g < NW; ++g) {
      const uint32_t nx = __ldg(pool + wi + g + 1);
      w[g] = __funnelshift_r(prev, nx, sh);
      prev = nx;
    }
  }
  __device__ __forceinline__ uint32_t at(int c) const {
    return (w[c >> 4] >> (2 * (c & 15))) & 3u;
  }
};

// Traceback words of one lane and row: cells in groups of 16, each group two 32-bit words of
// two bit-planes pushed MSB-first (see row_chunk).
template <int C>
using TbWords = uint32_t[2 * ((C + 15) / 16)];

// The pass's scoring, with `one` an opaque 1: `a * one + b` issues on the FMA pipe (IMAD)
// instead of the integer ALU pipe, which the maxima keep busy.
struct Sc {
  int32_t mat, nmis, go, ext, one;
};

__device__ __forceinline__ int32_t opaque_one() {
  int32_t v;
  asm volatile("mov.b32 %0, 1;" : "=r"(v));
  return v;
}

// Traceback bits are the signs of differences, shifted into bit-plane words: for each group
// of 16 cells of a lane, word A receives per cell (pass 1) "F extended" (ho < fo) then
// "diagonal lost" (dg < fj), word B (pass 2) "E extended" (xo < ee) then "H from E" (x < e).
// A push is one funnel shift: acc = (acc << 1) | (diff >> 31).  After a row, cell p of a
// group of g cells holds its first bit at position 2*(g-1-p)+1 and its second at 2*(g-1-p).
__device__ __forceinline__ uint32_t tb_push(uint32_t acc, int32_t diff) {
  return __funnelshift_l((uint32_t)diff, acc, 1);
}

// Pass 1 + scan + pass 2 for one chunk of cells (offsets Q + lane*C + c).
//   d        lo_i - lo_{i-1}
//   nH, nF   previous row at offset Q + lane*C + C (the next lane's first, or beyond)
//   pHl      previous row at offset Q + lane*C - 1 (the previous lane's last)
//   e0       horizontal gap entering offset Q (NEG at the band's left end)
//   xprev0   H' of offset Q - 1 (traceback only)
// h, f hold the previous row on entry and this row on exit.  ecarry / xlast: what enters
// the next chunk.  Cells past the band are computed too (garbage); the caller masks what
// later rows read.
template <int C, bool TB, bool LOCAL>
__device__ __forceinline__ void row_chunk(int32_t (&h)[C], int32_t (&f)[C], int d, int32_t nH,
                                          int32_t nF, int32_t pHl, const Win<C>& win,
                                          uint32_t cpat, const Sc& sc, int32_t floor_,
                                          bool col0, int32_t e0, int32_t xprev0, int lane,
                                          TbWords<C>& tbw, int32_t& ecarry, int32_t& xlast) {
  constexpr int NW = Win<C>::NW;
  const int32_t go = sc.go, ext = sc.ext, one = sc.one;
  // Match bits: bit 2k of eqm[g] is set when text base k of group g equals the row's base.
  uint32_t eqm[NW];
  {
    const uint32_t rep = (cpat & 3u) * 0x55555555u;
    const bool amb = cpat > 3u;  // local band: a read code of 4+ matches nothing
#pragma unroll
    for (int g = 0; g < NW; ++g) {
      const uint32_t x = win.w[g] ^ rep;
      eqm[g] = amb ? 0u : (~(x | (x >> 1)) & 0x55555555u);
    }
  }
  constexpr int TG = (C + 15) / 16;
  if constexpr (TB) {
#pragma unroll
    for (int q = 0; q < 2 * TG; ++q) tbw[q] = 0;
  }
  int32_t chain = NEG_INF;
  auto cell = [&](int c, int32_t hd, int32_t hu, int32_t fu, bool first_col) {
    const int32_t ho = hu * one - go;
    const int32_t fo = addmax(fu, -ext, NEG);  // max(fu - ext, NEG)
    const int32_t fj = max(ho, fo);
    if constexpr (TB) tbw[c >> 4] = tb_push(tbw[c >> 4], ho * one - fo);  // F extended
    int32_t x;
    if (first_col) {
      // Column 0: only a vertical gap reaches it (align.rs:2558-2566; local: 818-825).
      x = LOCAL ? max(fj, floor_) : fj;
      if constexpr (TB) tbw[c >> 4] = tb_push(tbw[c >> 4], 0);
    } else {
      const int32_t dg = hd * one + (((eqm[c >> 4] >> (2 * (c & 15))) & 1u) ? sc.mat : sc.nmis);
      x = max(dg, fj);
      if constexpr (TB) tbw[c >> 4] = tb_push(tbw[c >> 4], dg * one - fj);  // diagonal lost
      if constexpr (LOCAL) x = max(x, floor_);
    }
    chain = addmax(chain, -ext, x * one - go);
    f[c] = fj;
    return x;
  };
  if (d) {
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int32_t hu = c + 1 < C ? h[c + 1] : nH;
      const int32_t fu = c + 1 < C ? f[c + 1] : nF;
      h[c] = cell(c, h[c], hu, fu, false);
    }
  } else {
    int32_t hd = pHl;
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int32_t hu = h[c];
      h[c] = cell(c, hd, hu, f[c], c == 0 && col0);
      hd = hu;
    }
  }
  // Gap entering each lane: S_l = max_{l' <= l} chain_l' - ext*C*(l - l').  A low lane's
  // shuffle returns its own S, which max(S - k, S) leaves unchanged.
  const int32_t dC = ext * C;
  int32_t S = chain;
#pragma unroll
  for (int sft = 1; sft < 32; sft <<= 1)
    S = addmax(__shfl_up_sync(FULL, S, sft), -dC * sft, S);
  const int32_t Sp = __shfl_up_sync(FULL, S, 1);
  const int32_t ein = lane == 0 ? e0 : addmax(e0, -dC * lane, Sp);
  ecarry = __shfl_sync(FULL, addmax(e0, -dC * 32, S), 31);
  int32_t xp = 0;
  if constexpr (TB) {
    const int32_t xl = __shfl_up_sync(FULL, h[C - 1], 1);
    xp = lane == 0 ? xprev0 : xl;
  }
  xlast = __shfl_sync(FULL, h[C - 1], 31);
  // Pass 2: E_c = max(H'_{c-1} - go, E_{c-1} - ext), H = max(H', E).
  int32_t e = ein;
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const int32_t x = h[c];
    const int32_t xo = xp * one - go;  // H'_{c-1} - go (c = 0: the previous lane's last)
    if (c > 0) {
      if constexpr (TB) {
        const int32_t ee = e * one - ext;
        e = max(xo, ee);
        tbw[TG + (c >> 4)] = tb_push(tbw[TG + (c >> 4)], xo * one - ee);  // E extended
      } else {
        e = addmax(e, -ext, xo);
      }
    } else if constexpr (TB) {
      // ein was formed by the scan: it opened here iff it equals the left cell's H' - go.
      tbw[TG] = tb_push(tbw[TG], e == xo ? 0 : -1);
    }
    if constexpr (TB) tbw[TG + (c >> 4)] = tb_push(tbw[TG + (c >> 4)], x * one - e);  // H from E
    xp = x;
    h[c] = max(x, e);
  }
}

// Leftmost offset (within the lane layout) holding v; some lane must hold it.
template <int C>
__device__ __forceinline__ uint32_t leftmost(const int32_t (&h)[C], int32_t v, int lane) {
  int cf = C;
#pragma unroll
  for (int c = C - 1; c >= 0; --c)
    if (h[c] == v) cf = c;
  const uint32_t bal = __ballot_sync(FULL, cf < C);
  const int src = __ffs(bal) - 1;
  const int cs = __shfl_sync(FULL, cf, src < 0 ? 0 : src);
  return (uint32_t)(src < 0 ? 0 : src) * C + (uint32_t)cs;
}

template <int C>
__device__ __forceinline__ int32_t lane_max(const int32_t (&h)[C]) {
  int32_t v = h[0];
#pragma unroll
  for (int c = 1; c < C; ++c) v = max(v, h[c]);
  return v;
}

// Max over cells with offset < lim (offset = base + c).
template <int C>
__device__ __forceinline__ int32_t lane_max_below(const int32_t (&h)[C], int64_t base,
                                                  int64_t lim) {
  // max over cells with offset base + c < lim
  int32_t v = NEG;
#pragma unroll
  for (int c = 0; c < C; ++c)
    if (base + c < lim) v = max(v, h[c]);
  return v;
}

template <int C>
__device__ __forceinline__ int32_t select_c(const int32_t (&h)[C], int cs) {
  int32_t v = NEG;
#pragma unroll
  for (int c = 0; c < C; ++c)
    if (c == cs) v = h[c];
  return v;
}

struct PassCtx {
  DJob J;
  DParams P;
  Geo g;
  int mode;
  bool local, clip, cell, cuton, rowmax_on;
  int32_t mat, mis, ext, go;
  int64_t m, n;
};

__device__ __forceinline__ PassCtx make_ctx(const sfk::AffLaunch& a, uint32_t jid) {
  PassCtx x;
  x.J = a.jobs[jid];
  x.P = a.params[jid];
  const uint32_t fl = x.P.flags;
  x.mode = (int)(fl & F_MODE);
  x.local = fl & F_LOCAL;
  x.clip = fl & F_CLIP;
  x.cell = fl & F_CELL;
  x.cuton = fl & F_CUT;
  x.rowmax_on = fl & F_ROWMAX;
  x.mat = x.P.mat;
  x.mis = x.P.mis;
  x.ext = x.P.ext;
  x.go = x.P.open + x.P.ext;
  x.m = x.J.m;
  x.n = x.J.n;
  x.g = Geo{(fl & F_FULL) != 0, x.local, x.J.below, x.J.above, x.n};
  return x;
}

__device__ __forceinline__ int32_t row0_value(const PassCtx& x, int64_t j) {
  if (x.local) return x.P.bonus0;
  return (j == 0 || x.mode == 0) ? 0 : -(x.P.open + x.P.ext * (int32_t)j);
}

__device__ __forceinline__ uint32_t pattern_code(const sfk::AffLaunch& a, const PassCtx& x,
                                                 int64_t i, uint32_t& pw) {
  if (x.local) return a.bytes[x.J.p_byte + i - 1];
  if (i == 1 || (i & 15) == 0) pw = __ldg(a.pool + x.J.p_word + (i >> 4));
  return (pw >> (2 * (i & 15))) & 3u;
}

// Row bookkeeping shared by both drivers.  Returns true when the pass stops here.
struct Book {
  int32_t clip_best = 0, cut_best = 0, best_local = 0;
  uint32_t ci = 0, cj = 0;
  uint64_t cells = 0;
  uint32_t rows = 0;
};

// ---------------------------------------------------------------------------------------
// Register rows: the band fits 32 * C offsets.

// Row geometry in 32-bit arithmetic (sequences are shorter than 2^30 bases; the host clamps
// the band reaches to +-2^30).
struct Geo32 {
  bool full, local;
  int32_t below, above, n;
  __device__ __forceinline__ void range(int32_t i, int32_t& lo, int32_t& hi) const {
    if (local) {
      int32_t l = i + below, h = i + above + 1;
      l = l < 0 ? 0 : (l > n + 1 ? n + 1 : l);
      h = h < 0 ? 0 : (h > n + 1 ? n + 1 : h);
      lo = l;
      hi = (h < l ? l : h) - 1;
    } else if (full) {
      lo = 0;
      hi = n;
    } else {
      lo = i > below ? i - below : 0;
      hi = i + above < n ? i + above : n;
    }
  }
};

__device__ __forceinline__ int32_t clamp30(int64_t v) {
  const int64_t k = int64_t(1) << 30;
  return (int32_t)(v < -k ? -k : (v > k ? k : v));
}

// Sets cell c of the lane to NEG (a jump to the one cell, not a scan over all of them).
template <int C>
__device__ __forceinline__ void set_neg(int32_t (&h)[C], int32_t (&f)[C], int c) {
  switch (c) {
#define SF_NEG_CASE(k)            \
  case k:                         \
    if constexpr (k < C) {        \
      h[k] = NEG;                 \
      f[k] = NEG;                 \
    }                             \
    break;
    SF_NEG_CASE(0) SF_NEG_CASE(1) SF_NEG_CASE(2) SF_NEG_CASE(3) SF_NEG_CASE(4) SF_NEG_CASE(5)
    SF_NEG_CASE(6) SF_NEG_CASE(7) SF_NEG_CASE(8) SF_NEG_CASE(9) SF_NEG_CASE(10) SF_NEG_CASE(11)
    SF_NEG_CASE(12) SF_NEG_CASE(13) SF_NEG_CASE(14) SF_NEG_CASE(15) SF_NEG_CASE(16)
    SF_NEG_CASE(17) SF_NEG_CASE(18) SF_NEG_CASE(19) SF_NEG_CASE(20) SF_NEG_CASE(21)
    SF_NEG_CASE(22) SF_NEG_CASE(23) SF_NEG_CASE(24) SF_NEG_CASE(25) SF_NEG_CASE(26)
    SF_NEG_CASE(27) SF_NEG_CASE(28) SF_NEG_CASE(29) SF_NEG_CASE(30) SF_NEG_CASE(31)
    SF_NEG_CASE(32) SF_NEG_CASE(33) SF_NEG_CASE(34) SF_NEG_CASE(35) SF_NEG_CASE(36)
    SF_NEG_CASE(37) SF_NEG_CASE(38) SF_NEG_CASE(39) SF_NEG_CASE(40) SF_NEG_CASE(41)
    SF_NEG_CASE(42) SF_NEG_CASE(43) SF_NEG_CASE(44) SF_NEG_CASE(45) SF_NEG_CASE(46)
    SF_NEG_CASE(47)
#undef SF_NEG_CASE
    default:
      break;
  }
  static_assert(C <= 48, "set_neg covers 48 cells per lane");
}

// The band of a row occupies offsets [0, W); a lane's cells past W hold garbage.  A later row
// reads the previous row at offsets up to W only (each end of the band moves right by 0 or 1
// per row), so offset W -- the reference's sentinel right of the band (align.rs:2490-2494)
// -- is set to NEG and nothing past it is ever read.  Row maxima mask the garbage.
template <int C, bool TB, bool LOCAL>
__device__ void pair_regs(const sfk::AffLaunch& a, uint32_t jid, int lane) {
  const PassCtx x = make_ctx(a, jid);
  const Sc sc{x.mat, -x.mis, x.go, x.ext, opaque_one()};
  constexpr int CW = 2 * ((C + 15) / 16);
  DRes r{};
  if (LOCAL && (x.m == 0 || x.J.below > x.J.above)) {
    if (lane == 0) {
      r.score = 0;
      a.out[jid] = r;
    }
    return;
  }
  const int32_t m = (int32_t)x.m, n = (int32_t)x.n;
  const Geo32 g{(x.P.flags & F_FULL) != 0, LOCAL, clamp30(x.J.below), clamp30(x.J.above), n};
  const int32_t cut = x.cuton ? (int32_t)(x.J.cut < (uint64_t)n + 1 ? x.J.cut : (uint64_t)n + 1) : INT32_MAX;
  const int32_t kb = lane * C;  // this lane's first offset
  int32_t h[C], f[C];
  int32_t plo, phi;
  g.range(0, plo, phi);
  {
    const int32_t w0 = phi - plo + 1;
#pragma unroll
    for (int c = 0; c < C; ++c) {
      h[c] = kb + c < w0 ? row0_value(x, plo + kb + c) : NEG;
      f[c] = NEG;
    }
  }
  Book b;
  bool stopped = false;
  uint32_t pw = 0;
  uint2* tbp = TB ? reinterpret_cast<uint2*>(a.tb + x.J.tb_word) + lane : nullptr;
  for (int32_t i = 1; i <= m; ++i) {
    int32_t lo, hi;
    g.range(i, lo, hi);
    if (!LOCAL && lo > hi) {
      r = DRes{NEG, b.clip_best, b.cut_best, NEG, 0, b.ci, b.cj, (uint32_t)n, (uint32_t)i,
               b.rows, b.cells};
      stopped = true;
      break;
    }
    const int d = lo - plo;
    const int32_t W = hi - lo + 1;
    const uint32_t cpat = pattern_code(a, x, i, pw);
    const int32_t floor_ = LOCAL ? (i < m ? 0 : NEG) : NEG;
    int32_t nH = __shfl_down_sync(FULL, h[0], 1), nF = __shfl_down_sync(FULL, f[0], 1);
    if (lane == 31) nH = nF = NEG;
    const int32_t pHl = __shfl_up_sync(FULL, h[C - 1], 1);
    Win<C> win;
    win.load(a.pool, x.J.t_word, lo + kb);
    const bool col0 = lo == 0 && lane == 0 && W > 0;
    int32_t ecarry, xlast;
    TbWords<C> tbw;
    row_chunk<C, TB, LOCAL>(h, f, d, nH, nF, pHl, win, cpat, sc, floor_, col0, NEG, NEG_INF,
                            lane, tbw, ecarry, xlast);
    if (W < 32 * C && lane == W / C) set_neg(h, f, W - kb);
    if constexpr (TB) {
      constexpr int TG = CW / 2;
#pragma unroll
      for (int q = 0; q < TG; ++q) tbp[q * 32] = make_uint2(tbw[q], tbw[TG + q]);
      tbp += TG * 32;
    }
    b.cells += (uint64_t)(W > 0 ? W : 0);
    b.rows += 1;
    if (x.rowmax_on) {
      const int32_t rmax = __reduce_max_sync(FULL, lane_max_below(h, kb, W));
      if (x.cuton && lo <= cut) {
        int32_t row = rmax;
        if (hi > cut) row = __reduce_max_sync(FULL, lane_max_below(h, kb, cut - lo + 1));
        b.cut_best = max(b.cut_best, row);
      }
      if (x.clip) {
        if (rmax > b.clip_best) {
          b.clip_best = rmax;
          if (x.cell) {
            b.ci = (uint32_t)i;
            b.cj = (uint32_t)(lo + leftmost(h, rmax, lane));
          }
        }
        if (rmax < sat_sub(b.clip_best, x.P.xdrop)) {
          r = DRes{NEG, b.clip_best, b.cut_best, NEG, 0, b.ci, b.cj, (uint32_t)hi, (uint32_t)i,
                   b.rows, b.cells};
          stopped = true;
          break;
        }
      }
      if (LOCAL) {
        b.best_local = max(b.best_local, rmax);
        if (i == m) b.best_local = max(b.best_local, sat_add(rmax, x.P.bonus1));
      }
    }
    plo = lo;
    phi = hi;
  }
  if (!stopped) {
    const int32_t W = phi - plo + 1;
    r.clip_best = b.clip_best;
    r.cut_best = b.cut_best;
    r.clip_i = b.ci;
    r.clip_j = b.cj;
    r.text_read = (uint32_t)phi;
    r.last_row = (uint32_t)m;
    r.rows = b.rows;
    r.cells = b.cells;
    if (LOCAL) {
      r.score = b.best_local;
    } else if (x.mode == 2) {
      const int32_t K = n - plo;
      r.score = __shfl_sync(FULL, select_c(h, K % C), (K / C) & 31);
      r.score_col = (uint32_t)n;
    } else {
      const int32_t rmax = __reduce_max_sync(FULL, lane_max_below(h, kb, W));
      r.score = rmax;
      r.score_col = (uint32_t)(plo + leftmost(h, rmax, lane));
    }
    r.cut_score = NEG;
    if (x.cuton && plo <= cut) {
      const int32_t lim = min(phi, cut) - plo + 1;
      r.cut_score = __reduce_max_sync(FULL, lane_max_below(h, kb, lim));
    }
  }
  if (lane == 0) a.out[jid] = r;
  if constexpr (TB) {
    // __syncwarp orders the lanes' traceback stores before the walk reads them.
    __syncwarp();
    walk_lean(a, jid, tb_layout<C>(false, false, x.J, x.P.flags), x.J, x.P.flags, r, lane);
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------------------
// Wide rows: two row buffers per warp in global scratch, processed 32*C offsets at a time
// (offset K of a row at chunk K / 32C, cell (K % 32C) % C of lane (K % 32C) / C, stored
// lane-fastest so each chunk loads and stores coalesced).
template <int C>
__device__ __forceinline__ uint64_t widx(int64_t K) {
  const int64_t q = K / (32 * C), r = K % (32 * C);
  return (uint64_t)(q * 32 * C + (r % C) * 32 + r / C);
}

template <int C, bool TB, bool LOCAL>
__device__ void pair_wide(const sfk::AffLaunch& a, uint32_t jid, int lane, int32_t* scr) {
  const PassCtx x = make_ctx(a, jid);
  const Sc sc{x.mat, -x.mis, x.go, x.ext, opaque_one()};
  constexpr int CW = 2 * ((C + 15) / 16);
  constexpr int64_t CH = 32 * C;
  DRes r{};
  if (x.local && (x.m == 0 || x.J.below > x.J.above)) {
    if (lane == 0) {
      r.score = 0;
      a.out[jid] = r;
    }
    return;
  }
  const uint64_t cap = a.scratch_cells;
  int32_t* hb[2] = {scr, scr + 2 * cap};
  int32_t* fb[2] = {scr + cap, scr + 3 * cap};
  const uint64_t tb_stride = tb_row_words(C, wide_chunks(C, band_wmax(x.J, x.P.flags)));
  int cur = 0;
  int64_t plo, phi;
  x.g.range(0, plo, phi);
  int64_t pnch;  // chunks the previous row wrote
  {
    const int64_t w0 = phi - plo + 1;
    pnch = wide_chunks(C, w0 > 0 ? w0 : 0);
    for (int64_t q = 0; q < pnch; ++q)
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const int64_t K = q * CH + (int64_t)lane * C + c;
        const uint64_t at = (uint64_t)(q * CH + c * 32 + lane);
        hb[cur][at] = K < w0 ? row0_value(x, plo + K) : NEG;
        fb[cur][at] = NEG;
      }
  }
  Book b;
  bool stopped = false;
  uint32_t pw = 0;
  for (int64_t i = 1; i <= x.m; ++i) {
    int64_t lo, hi;
    x.g.range(i, lo, hi);
    if (!x.local && lo > hi) {
      r = DRes{NEG, b.clip_best, b.cut_best, NEG, 0, b.ci, b.cj, (uint32_t)x.n, (uint32_t)i,
               b.rows, b.cells};
      stopped = true;
      break;
    }
    const int d = (int)(lo - plo);
    const int64_t W = hi - lo + 1;
    const int64_t nch = wide_chunks(C, W > 0 ? W : 0);
    const uint32_t cpat = pattern_code(a, x, i, pw);
    const int32_t floor_ = x.local ? (i < x.m ? 0 : NEG) : NEG;
    const int32_t* ph = hb[cur];
    const int32_t* pf = fb[cur];
    int32_t* nh = hb[cur ^ 1];
    int32_t* nf = fb[cur ^ 1];
    int32_t e0 = NEG, xprev0 = NEG_INF;
    int32_t rbest = NEG, rcut = NEG;  // row max and its leftmost offset; max up to the cut
    int64_t rpos = 0;
    for (int64_t q = 0; q < nch; ++q) {
      const int64_t Q = q * CH;
      int32_t h[C], f[C];
      const bool have = q < pnch;
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const uint64_t at = (uint64_t)(Q + c * 32 + lane);
        h[c] = have ? ph[at] : NEG;
        f[c] = have ? pf[at] : NEG;
      }
      int32_t nH = __shfl_down_sync(FULL, h[0], 1), nF = __shfl_down_sync(FULL, f[0], 1);
      if (lane == 31) {
        const bool nx = q + 1 < pnch;
        nH = nx ? ph[Q + CH] : NEG;
        nF = nx ? pf[Q + CH] : NEG;
      }
      int32_t pHl = __shfl_up_sync(FULL, h[C - 1], 1);
      if (lane == 0) pHl = q > 0 ? ph[widx<C>(Q - 1)] : NEG;
      Win<C> win;
      win.load(a.pool, x.J.t_word, lo + Q + (int64_t)lane * C);
      const bool col0 = lo == 0 && q == 0 && lane == 0 && W > 0;
      int32_t ecarry, xlast;
      TbWords<C> tbw;
      row_chunk<C, TB, LOCAL>(h, f, d, nH, nF, pHl, win, cpat, sc, floor_, col0, e0, xprev0,
                              lane, tbw, ecarry, xlast);
      e0 = ecarry;
      xprev0 = xlast;
      const int64_t kb = Q + (int64_t)lane * C;
      if (kb + C > W) {
#pragma unroll
        for (int c = 0; c < C; ++c)
          if (kb + c >= W) h[c] = f[c] = NEG;
      }
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const uint64_t at = (uint64_t)(Q + c * 32 + lane);
        nh[at] = h[c];
        nf[at] = f[c];
      }
      if constexpr (TB) {
        constexpr int TG = CW / 2;
        uint2* dst = reinterpret_cast<uint2*>(a.tb + x.J.tb_word + (uint64_t)(i - 1) * tb_stride) +
                     (uint64_t)q * TG * 32;
#pragma unroll
        for (int w = 0; w < TG; ++w) dst[w * 32 + lane] = make_uint2(tbw[w], tbw[TG + w]);
      }
      if (x.rowmax_on) {
        const int32_t cm = __reduce_max_sync(FULL, lane_max(h));
        if (cm > rbest) {
          rbest = cm;
          rpos = Q + leftmost(h, cm, lane);
        }
        if (x.cuton)
          rcut = max(rcut, __reduce_max_sync(
                               FULL, lane_max_below(h, kb, (int64_t)x.J.cut - lo + 1)));
      }
    }
    b.cells += (uint64_t)(W > 0 ? W : 0);
    b.rows += 1;
    cur ^= 1;
    pnch = nch;
    if (x.rowmax_on) {
      const int32_t rmax = rbest;
      if (x.cuton && lo <= (int64_t)x.J.cut) b.cut_best = max(b.cut_best, rcut);
      if (x.clip) {
        if (rmax > b.clip_best) {
          b.clip_best = rmax;
          if (x.cell) {
            b.ci = (uint32_t)i;
            b.cj = (uint32_t)(lo + rpos);
          }
        }
        if (rmax < sat_sub(b.clip_best, x.P.xdrop)) {
          r = DRes{NEG, b.clip_best, b.cut_best, NEG, 0, b.ci, b.cj, (uint32_t)hi, (uint32_t)i,
                   b.rows, b.cells};
          stopped = true;
          break;
        }
      }
      if (x.local) {
        b.best_local = max(b.best_local, rmax);
        if (i == x.m) b.best_local = max(b.best_local, sat_add(rmax, x.P.bonus1));
      }
    }
    plo = lo;
    phi = hi;
  }
  if (!stopped) {
    // The last row is in buffer `cur`.
    const int32_t* lh = hb[cur];
    int32_t best = NEG, cutm = NEG;
    int64_t pos = 0;
    const int64_t W = phi - plo + 1;
    const int64_t lim = x.cuton ? min(phi, (int64_t)x.J.cut) - plo + 1 : 0;
    for (int64_t q = 0; q < pnch; ++q) {
      const int64_t Q = q * CH;
      int32_t h[C];
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const int64_t K = Q + (int64_t)lane * C + c;
        h[c] = K < W ? lh[Q + c * 32 + lane] : NEG;
      }
      const int32_t cm = __reduce_max_sync(FULL, lane_max(h));
      if (cm > best) {
        best = cm;
        pos = Q + leftmost(h, cm, lane);
      }
      cutm = max(cutm, __reduce_max_sync(FULL, lane_max_below(h, Q + (int64_t)lane * C, lim)));
    }
    r.clip_best = b.clip_best;
    r.cut_best = b.cut_best;
    r.clip_i = b.ci;
    r.clip_j = b.cj;
    r.text_read = (uint32_t)phi;
    r.last_row = (uint32_t)x.m;
    r.rows = b.rows;
    r.cells = b.cells;
    if (x.local) {
      r.score = b.best_local;
    } else if (x.mode == 2) {
      r.score = lh[widx<C>(x.n - plo)];
      r.score_col = (uint32_t)x.n;
    } else {
      r.score = best;
      r.score_col = (uint32_t)(plo + pos);
    }
    r.cut_score = (x.cuton && plo <= (int64_t)x.J.cut) ? cutm : NEG;
  }
  __syncwarp();
  if (lane == 0) a.out[jid] = r;
  if constexpr (TB) {
    __syncwarp();
    walk_lean(a, jid, tb_layout<C>(true, false, x.J, x.P.flags), x.J, x.P.flags, r, lane);
  }
  __syncwarp();
}

// One warp per pass; warps take passes from the bucket's queue, longest first.
// Blocks per SM the register budget aims at: rows of up to 12 cells per lane fit in ~80
// registers (6 blocks of 4 warps), 16 in ~100; wider rows and the wide-row kernel take what
// they need.
template <int C, bool WIDE>
struct MinBlocks {
  static constexpr int value =
      WIDE ? 3 : (C <= 12 ? 6 : (C <= 16 ? 5 : (C <= 20 ? 4 : 3)));
};

template <int C, bool WIDE, bool TB, bool LOCAL>
__global__ void __launch_bounds__(128, MinBlocks<C, WIDE>::value) affine_kernel(sfk::AffLaunch a) {
  const int lane = threadIdx.x & 31;
  const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int32_t* scr = WIDE ? a.scratch + gw * 4 * a.scratch_cells : nullptr;
  for (;;) {
    uint32_t q = 0;
    if (lane == 0) q = atomicAdd(a.counter, 1u);
    q = __shfl_sync(FULL, q, 0);
    if (q >= a.njobs) break;
    const uint32_t jid = a.order[q];
    if constexpr (WIDE)
      pair_wide<C, TB, LOCAL>(a, jid, lane, scr);
    else
      pair_regs<C, TB, LOCAL>(a, jid, lane);
  }
}

}  // namespace

namespace sfk {

template <int C, bool WIDE>
cudaError_t launch_affine_c(bool tb, bool local, const AffLaunch& a, int grid, int block,
                            cudaStream_t s) {
  if (local)
    affine_kernel<C, WIDE, false, true><<<grid, block, 0, s>>>(a);
  else if (tb)
    affine_kernel<C, WIDE, true, false><<<grid, block, 0, s>>>(a);
  else
    affine_kernel<C, WIDE, false, false><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace sfk
