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
// Traceback: one nibble per cell -- bits 0-1 the source of H (0 diagonal, 1 vertical F,
// 2 horizontal E), bit 2 "E opened from H' of the cell to the left", bit 3 "F opened from H
// of the cell above" -- stored per row as 32 lanes x ceil(C/8) words, lane-fastest.
#pragma once
#include <type_traits>

#include "sf_internal.cuh"

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

template <int C>
using TbWords = uint32_t[(C + 7) / 8];

// Pass 1 + scan + pass 2 for one chunk of cells (offsets Q + lane*C + c).
//   d        lo_i - lo_{i-1}
//   nH, nF   previous row at offset Q + lane*C + C (the next lane's first, or beyond)
//   pHl      previous row at offset Q + lane*C - 1 (the previous lane's last)
//   e0       horizontal gap entering offset Q (NEG at the band's left end)
//   xprev0   H' of offset Q - 1 (traceback only)
// h, f hold the previous row on entry and this row on exit.  ecarry / xlast: what enters
// the next chunk.
template <int C, bool TB>
__device__ __forceinline__ void row_chunk(int32_t (&h)[C], int32_t (&f)[C], int d, int32_t nH,
                                          int32_t nF, int32_t pHl, const Win<C>& win,
                                          uint32_t cpat, int32_t mat, int32_t mis, int32_t go,
                                          int32_t ext, int32_t floor_, bool col0, bool local,
                                          int32_t e0, int32_t xprev0, int lane, TbWords<C>& tbw,
                                          int32_t& ecarry, int32_t& xlast) {
  constexpr bool KEEP = C <= 16;
  int32_t el[KEEP ? C : 1];
  // Traceback: per cell "diagonal >= vertical" and "F opened" (one bit per cell of the lane).
  using Mask = typename std::conditional<(C > 32), uint64_t, uint32_t>::type;
  Mask dgb = 0, fob = 0;
  int32_t chain = NEG_INF;
  const int32_t nmis = -mis;
  if (d) {
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int32_t hd = h[c];
      const int32_t hu = c + 1 < C ? h[c + 1] : nH;
      const int32_t fu = c + 1 < C ? f[c + 1] : nF;
      const int32_t fo = fu - ext, ho = hu - go;
      const int32_t fj = max3(ho, fo, NEG);
      const int32_t dg = hd + (win.at(c) == cpat ? mat : nmis);
      const int32_t x = max3(dg, fj, floor_);
      if constexpr (TB) {
        dgb |= (Mask)(dg >= fj) << c;
        fob |= (Mask)(ho >= fo) << c;
      }
      if constexpr (KEEP) el[c] = chain;
      chain = addmax(chain, -ext, x - go);
      h[c] = x;
      f[c] = fj;
    }
  } else {
    int32_t hd = pHl;
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int32_t hu = h[c], fu = f[c];
      const int32_t fo = fu - ext, ho = hu - go;
      int32_t fj, x;
      if (c == 0 && col0) {
        // Column 0: only a vertical gap reaches it (align.rs:2558-2566; local: 818-825).
        fj = local ? max3(ho, fo, NEG) : max(ho, fo);
        x = local ? max(fj, floor_) : fj;
        if constexpr (TB) fob |= (Mask)(ho >= fo);
      } else {
        fj = max3(ho, fo, NEG);
        const int32_t dg = hd + (win.at(c) == cpat ? mat : nmis);
        x = max3(dg, fj, floor_);
        if constexpr (TB) {
          dgb |= (Mask)(dg >= fj) << c;
          fob |= (Mask)(ho >= fo) << c;
        }
      }
      if constexpr (KEEP) el[c] = chain;
      chain = addmax(chain, -ext, x - go);
      hd = hu;
      h[c] = x;
      f[c] = fj;
    }
  }
  // Gap entering each lane: S_l = max_{l' <= l} chain_l' - ext*C*(l - l').
  const int32_t dC = ext * C;
  int32_t S = chain;
#pragma unroll
  for (int sft = 1; sft < 32; sft <<= 1) {
    const int32_t tv = __shfl_up_sync(FULL, S, sft);
    if (lane >= sft) S = addmax(tv, -dC * sft, S);
  }
  const int32_t Sp = __shfl_up_sync(FULL, S, 1);
  const int32_t ein = lane == 0 ? e0 : addmax(e0, -dC * lane, Sp);
  ecarry = __shfl_sync(FULL, addmax(e0, -dC * 32, S), 31);
  int32_t xprev = 0;
  if constexpr (TB) {
    const int32_t xl = __shfl_up_sync(FULL, h[C - 1], 1);
    xprev = lane == 0 ? xprev0 : xl;
#pragma unroll
    for (int q = 0; q < (C + 7) / 8; ++q) tbw[q] = 0;
  }
  xlast = __shfl_sync(FULL, h[C - 1], 31);
  // Pass 2.
  int32_t e = ein, xp = 0;
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const int32_t x = h[c];
    if constexpr (KEEP) {
      if (c > 0) e = addmax(ein, -ext * c, el[c]);
    } else {
      if (c > 0) e = addmax(e, -ext, xp - go);
      xp = x;
    }
    if constexpr (TB) {
      const uint32_t hs = e > x ? 2u : (((dgb >> c) & 1u) ? 0u : 1u);
      const uint32_t eo = (uint32_t)(e == xprev - go);
      tbw[c >> 3] |= (hs | (eo << 2) | ((uint32_t)((fob >> c) & 1u) << 3)) << (4 * (c & 7));
      xprev = x;
    }
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
template <int C, bool TB>
__device__ void pair_regs(const sfk::AffLaunch& a, uint32_t jid, int lane) {
  const PassCtx x = make_ctx(a, jid);
  constexpr int CW = (C + 7) / 8;
  DRes r{};
  if (x.local && (x.m == 0 || x.J.below > x.J.above)) {
    if (lane == 0) {
      r.score = 0;
      a.out[jid] = r;
    }
    return;
  }
  int32_t h[C], f[C];
  int64_t plo, phi;
  x.g.range(0, plo, phi);
  {
    const int64_t w0 = phi - plo + 1;
#pragma unroll
    for (int c = 0; c < C; ++c) {
      const int64_t K = (int64_t)lane * C + c;
      h[c] = K < w0 ? row0_value(x, plo + K) : NEG;
      f[c] = NEG;
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
    const uint32_t cpat = pattern_code(a, x, i, pw);
    const int32_t floor_ = x.local ? (i < x.m ? 0 : NEG) : NEG;
    int32_t nH = __shfl_down_sync(FULL, h[0], 1), nF = __shfl_down_sync(FULL, f[0], 1);
    if (lane == 31) nH = nF = NEG;
    const int32_t pHl = __shfl_up_sync(FULL, h[C - 1], 1);
    Win<C> win;
    win.load(a.pool, x.J.t_word, lo + (int64_t)lane * C);
    const bool col0 = lo == 0 && lane == 0 && W > 0;
    int32_t ecarry, xlast;
    TbWords<C> tbw;
    row_chunk<C, TB>(h, f, d, nH, nF, pHl, win, cpat, x.mat, x.mis, x.go, x.ext, floor_, col0,
                     x.local, NEG, NEG_INF, lane, tbw, ecarry, xlast);
    if ((int64_t)lane * C + C > W) {
#pragma unroll
      for (int c = 0; c < C; ++c)
        if ((int64_t)lane * C + c >= W) h[c] = f[c] = NEG;
    }
    if constexpr (TB) {
      uint32_t* dst = a.tb + x.J.tb_word + (uint64_t)(i - 1) * (CW * 32);
#pragma unroll
      for (int q = 0; q < CW; ++q) dst[q * 32 + lane] = tbw[q];
    }
    b.cells += (uint64_t)(W > 0 ? W : 0);
    b.rows += 1;
    if (x.rowmax_on) {
      const int32_t rmax = __reduce_max_sync(FULL, lane_max(h));
      if (x.cuton && lo <= (int64_t)x.J.cut) {
        int32_t row = rmax;
        if (hi > (int64_t)x.J.cut)
          row = __reduce_max_sync(
              FULL, lane_max_below(h, (int64_t)lane * C, (int64_t)x.J.cut - lo + 1));
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
      if (x.local) {
        b.best_local = max(b.best_local, rmax);
        if (i == x.m) b.best_local = max(b.best_local, sat_add(rmax, x.P.bonus1));
      }
    }
    plo = lo;
    phi = hi;
  }
  if (!stopped) {
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
      const int64_t K = x.n - plo;
      const int owner = (int)(K / C), cs = (int)(K % C);
      r.score = __shfl_sync(FULL, select_c(h, cs), owner & 31);
      r.score_col = (uint32_t)x.n;
    } else {
      const int32_t rmax = __reduce_max_sync(FULL, lane_max(h));
      r.score = rmax;
      r.score_col = (uint32_t)(plo + leftmost(h, rmax, lane));
    }
    r.cut_score = NEG;
    if (x.cuton && plo <= (int64_t)x.J.cut) {
      const int64_t lim = min(phi, (int64_t)x.J.cut) - plo + 1;
      r.cut_score = __reduce_max_sync(FULL, lane_max_below(h, (int64_t)lane * C, lim));
    }
  }
  if (lane == 0) a.out[jid] = r;
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

template <int C, bool TB>
__device__ void pair_wide(const sfk::AffLaunch& a, uint32_t jid, int lane, int32_t* scr) {
  const PassCtx x = make_ctx(a, jid);
  constexpr int CW = (C + 7) / 8;
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
      row_chunk<C, TB>(h, f, d, nH, nF, pHl, win, cpat, x.mat, x.mis, x.go, x.ext, floor_, col0,
                       x.local, e0, xprev0, lane, tbw, ecarry, xlast);
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
        uint32_t* dst = a.tb + x.J.tb_word + (uint64_t)(i - 1) * tb_stride + (uint64_t)q * CW * 32;
#pragma unroll
        for (int w = 0; w < CW; ++w) dst[w * 32 + lane] = tbw[w];
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
  if (lane == 0) a.out[jid] = r;
}

// One warp per pass; warps take passes from the bucket's queue, longest first.
template <int C, bool WIDE, bool TB>
__global__ void __launch_bounds__(128) affine_kernel(sfk::AffLaunch a) {
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
      pair_wide<C, TB>(a, jid, lane, scr);
    else
      pair_regs<C, TB>(a, jid, lane);
  }
}

}  // namespace

namespace sfk {

template <int C, bool WIDE>
cudaError_t launch_affine_c(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  if (tb)
    affine_kernel<C, WIDE, true><<<grid, block, 0, s>>>(a);
  else
    affine_kernel<C, WIDE, false><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace sfk
