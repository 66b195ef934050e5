// Banded affine (Gotoh) passes with two cells per 32-bit register: the same rows as
// sf_affine_impl.cuh (align.rs:2446-2666 `run_core`), with every H/F/E value held as a
// 16-bit field relative to a per-pass offset, as the reference's `run16_avx512`
// (align.rs:1380-1877) holds its rows in 16-bit lanes when `narrow` (align.rs:2388-2426)
// allows.  Results, row bookkeeping and traceback decisions equal the 32-bit kernel's.
//
// Why 16 bits suffice.  In a Global or Prefix pass every cell of row i's band is reached
// from the origin, and every band cell is at least the row maximum M_i minus
// (mat + ext) * width + go (follow the best path to the column, then a vertical gap down;
// right of the maximum, a horizontal gap).  From one row to the next M moves by at most
// max(mat, mis, go).  The kernel subtracts the row maximum from every cell each 64 rows
// (`rebase`), so all reachable values stay within a window of 16384 below and a few hundred
// above field 0x8000; NEG is field 0x4000, below every reachable value by more than any
// single step can add.  The host admits a pass only when its widest row, its scores and this
// bound fit (sf_host.cu `fits16`); everything else runs on the 32-bit kernel.
//
// Layout.  A field holds value - offset (offset = -0x8000 at row 0), unsigned, so the DPX
// u16x2 maxima order fields as values, and a - b + 0x7fff7fff has bit 15 (31) set exactly
// when the low (high) field of a exceeds b's: one IADD3 per pair of traceback decisions.
// Lane l holds band offsets [l*C, l*C + C) as C/2 words: word k = (offset l*C + k,
// offset l*C + C/2 + k).  Both halves of a word advance together through pass 1, the
// lane's horizontal-gap chain and pass 2; the warp scan works on per-lane 32-bit values.
// Match scores come from one byte permute per word: a per-row table of the score of each
// text code against the row's pattern base, indexed by per-word selectors of the two text
// columns, which shift one column per row with the band.  Traceback decisions go out as one
// (A, B) word pair per lane and group of 8 words; sf_walk.cuh decodes that layout.
#pragma once
#include "sf_affine_impl.cuh"

namespace {

constexpr uint32_t kBias16 = 0x8000u;
constexpr uint32_t kNeg16 = 0x4000u;
constexpr uint32_t kOne2 = 0x00010001u;
constexpr uint32_t kNeg2 = kNeg16 * kOne2;
constexpr uint32_t kGt2 = 0x7fff7fffu;
constexpr int kRebaseRows = 64;

__device__ __forceinline__ uint32_t pk2(uint32_t lo, uint32_t hi) { return lo | (hi << 16); }

// Bit 15 / 31: the low / high field of a exceeds b's (fields within 0x7fff of each other).
__device__ __forceinline__ uint32_t gt2(uint32_t a, uint32_t b) { return a - b + kGt2; }

// Two decisions of one word into a traceback word: bytes (d1 lo, d1 hi, d2 lo, d2 hi), each
// byte receiving the decision at bit 7 after shifting the earlier ones down.
__device__ __forceinline__ uint32_t push2(uint32_t acc, uint32_t d1, uint32_t d2) {
  const uint32_t w = __byte_perm(d1, d2, 0x7531);
  return ((acc >> 1) & 0x7f7f7f7fu) | (w & 0x80808080u);
}

// Score of each text code against the row's pattern base p, as a 16-bit field: low bytes in
// ta, high bytes in tb, byte t for code t.
__device__ __forceinline__ void score_tables(uint32_t p, int32_t mat, int32_t mis, uint32_t& ta,
                                             uint32_t& tb) {
  const uint32_t nm = (uint32_t)(-mis) & 0xffffu, mt = (uint32_t)mat & 0xffffu;
  const uint32_t sh = 8u * (p & 3u), keep = ~(0xffu << sh);
  ta = (((nm & 0xffu) * 0x01010101u) & keep) | ((mt & 0xffu) << sh);
  tb = (((nm >> 8) * 0x01010101u) & keep) | ((mt >> 8) << sh);
}

// Selector byte of a text code for __byte_perm(ta, tb, .): nibbles (t, t + 4).
__device__ __forceinline__ uint32_t sel_byte(uint32_t t) { return 0x40u + t * 0x11u; }

template <int C2>
__device__ __forceinline__ uint32_t lane_max16(const uint32_t (&h)[C2], int32_t kb, int32_t lim) {
  const int32_t cnt = lim - kb;  // this lane's cells below offset lim
  uint32_t v = 0;
#pragma unroll
  for (int k = 0; k < C2; ++k) {
    const uint32_t mk = (k < cnt ? 0xffffu : 0u) | (C2 + k < cnt ? 0xffff0000u : 0u);
    v = __vmaxu2(v, h[k] & mk);
  }
  return max(v & 0xffffu, v >> 16);
}

// Leftmost offset holding field v (some lane holds it).
template <int C2>
__device__ __forceinline__ uint32_t leftmost16(const uint32_t (&h)[C2], uint32_t v, int lane) {
  constexpr int C = 2 * C2;
  int cf = C;
#pragma unroll
  for (int c = C - 1; c >= 0; --c) {
    const uint32_t u = c < C2 ? (h[c] & 0xffffu) : (h[c - C2] >> 16);
    if (u == v) cf = c;
  }
  const uint32_t bal = __ballot_sync(FULL, cf < C);
  const int src = __ffs(bal) - 1;
  const int cs = __shfl_sync(FULL, cf, src < 0 ? 0 : src);
  return (uint32_t)(src < 0 ? 0 : src) * C + (uint32_t)cs;
}

template <int C2>
__device__ __forceinline__ uint32_t field_at(const uint32_t (&h)[C2], int c) {
  uint32_t v = 0;
#pragma unroll
  for (int k = 0; k < C2; ++k) {
    if (k == c) v = h[k] & 0xffffu;
    if (C2 + k == c) v = h[k] >> 16;
  }
  return v;
}

// Sets the field of lane cell c (H and F) to NEG.
template <int C2>
__device__ __forceinline__ void set_neg16(uint32_t (&h)[C2], uint32_t (&f)[C2], int c) {
  const bool hi = c >= C2;
  const int k = hi ? c - C2 : c;
  const uint32_t mk = hi ? 0xffff0000u : 0xffffu;
  switch (k) {
#define SF_NEG16_CASE(q)                        \
  case q:                                       \
    if constexpr (q < C2) {                     \
      h[q] = (h[q] & ~mk) | (kNeg2 & mk);       \
      f[q] = (f[q] & ~mk) | (kNeg2 & mk);       \
    }                                           \
    break;
    SF_NEG16_CASE(0) SF_NEG16_CASE(1) SF_NEG16_CASE(2) SF_NEG16_CASE(3) SF_NEG16_CASE(4)
    SF_NEG16_CASE(5) SF_NEG16_CASE(6) SF_NEG16_CASE(7) SF_NEG16_CASE(8) SF_NEG16_CASE(9)
    SF_NEG16_CASE(10) SF_NEG16_CASE(11) SF_NEG16_CASE(12) SF_NEG16_CASE(13) SF_NEG16_CASE(14)
    SF_NEG16_CASE(15) SF_NEG16_CASE(16) SF_NEG16_CASE(17) SF_NEG16_CASE(18) SF_NEG16_CASE(19)
    SF_NEG16_CASE(20) SF_NEG16_CASE(21) SF_NEG16_CASE(22) SF_NEG16_CASE(23) SF_NEG16_CASE(24)
    SF_NEG16_CASE(25) SF_NEG16_CASE(26) SF_NEG16_CASE(27) SF_NEG16_CASE(28) SF_NEG16_CASE(29)
    SF_NEG16_CASE(30) SF_NEG16_CASE(31)
#undef SF_NEG16_CASE
    default:
      break;
  }
  static_assert(C2 <= 32, "set_neg16 covers 32 words per lane");
}

template <int C2, bool TB>
__device__ void pair16(const sfk::AffLaunch& a, uint32_t jid, int lane) {
  constexpr int C = 2 * C2;
  constexpr int G = (C2 + 7) / 8;
  constexpr int CW = 2 * G;
  static_assert(CW == 2 * ((C + 15) / 16), "same traceback row size as the 32-bit kernel");
  const PassCtx x = make_ctx(a, jid);
  DRes r{};
  const int32_t m = (int32_t)x.m, n = (int32_t)x.n;
  const Geo32 g{(x.P.flags & F_FULL) != 0, false, clamp30(x.J.below), clamp30(x.J.above), n};
  const int32_t cut =
      x.cuton ? (int32_t)(x.J.cut < (uint64_t)n + 1 ? x.J.cut : (uint64_t)n + 1) : INT32_MAX;
  const int32_t kb = lane * C;
  // `one` is an opaque 1: `v * one - go2` issues on the FMA pipe (IMAD), off the ALU pipe the
  // maxima keep busy.  go2 subtracts go from both fields (no borrow: reachable fields and
  // NEG exceed go; a low field past the band has a high field past it too).
  const uint32_t one = (uint32_t)opaque_one();
  const uint32_t go2 = (uint32_t)x.go * kOne2;
  const uint32_t next2 = ((uint32_t)(-x.ext) & 0xffffu) * kOne2;  // + (-ext) mod 2^16
  int32_t off = -(int32_t)kBias16;  // value = field + off
  uint32_t h[C2], f[C2], sel[C2];
  int32_t plo, phi;
  g.range(0, plo, phi);
  {
    const int32_t w0 = phi - plo + 1;
#pragma unroll
    for (int k = 0; k < C2; ++k) {
      const int32_t K = kb + k, K2 = kb + C2 + k;
      const uint32_t lo = K < w0 ? (uint32_t)(row0_value(x, plo + K) - off) : kNeg16;
      const uint32_t hi = K2 < w0 ? (uint32_t)(row0_value(x, plo + K2) - off) : kNeg16;
      h[k] = pk2(lo, hi);
      f[k] = kNeg2;
      sel[k] = 0;
    }
  }
  Book b;
  bool stopped = false;
  uint32_t pw = 0;
  uint2* tbp = TB ? reinterpret_cast<uint2*>(a.tb + x.J.tb_word) + lane : nullptr;
  for (int32_t i = 1; i <= m; ++i) {
    int32_t lo, hi;
    g.range(i, lo, hi);
    if (lo > hi) {
      r = DRes{NEG, b.clip_best, b.cut_best, NEG, 0, b.ci, b.cj, (uint32_t)n, (uint32_t)i,
               b.rows, b.cells};
      stopped = true;
      break;
    }
    const int d = lo - plo;
    const int32_t W = hi - lo + 1;
    const uint32_t cpat = pattern_code(a, x, i, pw);
    uint32_t ta, tbl;
    score_tables(cpat, x.mat, x.mis, ta, tbl);
    // Selectors of this row's text columns: loaded at row 1, then shifted with the band.
    if (i == 1) {
      Win<C> win;
      win.load(a.pool, x.J.t_word, lo + kb);
#pragma unroll
      for (int k = 0; k < C2; ++k) sel[k] = sel_byte(win.at(k)) | (sel_byte(win.at(C2 + k)) << 8);
    } else if (d) {
      const uint32_t s0 = sel[0];
      uint32_t nx = __shfl_down_sync(FULL, s0, 1);
      const uint32_t far = sel_byte(base_at(a.pool, x.J.t_word, (uint64_t)(lo + 32 * C - 1)));
      if (lane == 31) nx = far;
#pragma unroll
      for (int k = 0; k + 1 < C2; ++k) sel[k] = sel[k + 1];
      sel[C2 - 1] = __byte_perm(s0, nx, 0x2241);  // (old word 0 high column, next lane's low)
    }

    // Pass 1: F, H' and the lane's horizontal-gap chain.
    uint32_t chain = kNeg2;
    uint32_t acc1[G];
#pragma unroll
    for (int q = 0; q < G; ++q) acc1[q] = 0;
    auto cell = [&](int k, uint32_t hd, uint32_t hu, uint32_t fu) {
      const uint32_t ho = hu * one - go2;
      const uint32_t fo = __viaddmax_u16x2(fu, next2, kNeg2);
      const uint32_t fj = __vmaxu2(ho, fo);
      const uint32_t s2 = __byte_perm(ta, tbl, sel[k]);
      const uint32_t dg = __viaddmax_u16x2(hd, s2, 0u);
      const uint32_t xx = __vmaxu2(dg, fj);
      if constexpr (TB) acc1[k >> 3] = push2(acc1[k >> 3], gt2(fj, ho), gt2(xx, dg));
      chain = __viaddmax_u16x2(chain, next2, xx * one - go2);
      f[k] = fj;
      h[k] = xx;
    };
    if (d) {
      uint32_t nH = __shfl_down_sync(FULL, h[0], 1), nF = __shfl_down_sync(FULL, f[0], 1);
      if (lane == 31) nH = nF = kNeg2;
      const uint32_t upH = __byte_perm(h[0], nH, 0x5432), upF = __byte_perm(f[0], nF, 0x5432);
#pragma unroll
      for (int k = 0; k < C2; ++k)
        cell(k, h[k], k + 1 < C2 ? h[k + 1] : upH, k + 1 < C2 ? f[k + 1] : upF);
    } else {
      // d = 0 only while lo = 0: lane 0's first cell is column 0, reached by a vertical gap
      // alone (align.rs:2558-2566); its diagonal gets a field no F can lose to.
      const uint32_t pl = __shfl_up_sync(FULL, h[C2 - 1], 1);
      uint32_t hd = __byte_perm(pl, h[C2 - 1], 0x5432);
      if (lane == 0) hd = (hd & 0xffff0000u) | (kNeg16 - (uint32_t)x.mat - 1u);
#pragma unroll
      for (int k = 0; k < C2; ++k) {
        const uint32_t hu = h[k];
        cell(k, hd, hu, f[k]);
        hd = hu;
      }
    }

    // Gap entering each lane (32-bit fields): the lane's chain leaves its low half decayed
    // by ext * C/2 and meets its high half's.
    const int32_t clo = (int32_t)(chain & 0xffffu), chi = (int32_t)(chain >> 16);
    const int32_t dC = x.ext * C;
    int32_t S = addmax(clo, -x.ext * C2, chi);
#pragma unroll
    for (int sft = 1; sft < 32; sft <<= 1)
      S = addmax(__shfl_up_sync(FULL, S, sft), -dC * sft, S);
    const int32_t Sp = __shfl_up_sync(FULL, S, 1);
    const int32_t ein = lane == 0 ? (int32_t)kNeg16 : addmax((int32_t)kNeg16, -dC * lane, Sp);
    const int32_t ehi = addmax(ein, -x.ext * C2, clo);
    uint32_t e = pk2((uint32_t)ein, (uint32_t)ehi);
    // H' left of each half's first cell (lane 0: none -- a field below NEG, so that lane 0's
    // entering E, NEG, counts as extended whatever go is, as in the 32-bit kernel).
    const uint32_t pl2 = __shfl_up_sync(FULL, h[C2 - 1], 1);
    uint32_t xp = __byte_perm(pl2, h[C2 - 1], 0x5432);
    if (lane == 0) xp = (xp & 0xffff0000u) | (kNeg16 - 1u);

    // Pass 2: E and H.
    uint32_t acc2[G];
#pragma unroll
    for (int q = 0; q < G; ++q) acc2[q] = 0;
#pragma unroll
    for (int k = 0; k < C2; ++k) {
      const uint32_t xx = h[k];
      const uint32_t xo = xp * one - go2;
      if (k > 0) e = __viaddmax_u16x2(e, next2, xo);
      if constexpr (TB) acc2[k >> 3] = push2(acc2[k >> 3], gt2(e, xo), gt2(e, xx));
      h[k] = __vmaxu2(xx, e);
      xp = xx;
    }
    if constexpr (TB) {
#pragma unroll
      for (int q = 0; q < G; ++q) tbp[q * 32] = make_uint2(acc1[q], acc2[q]);
      tbp += G * 32;
    }
    b.cells += (uint64_t)W;
    b.rows += 1;
    const bool rebase = (i & (kRebaseRows - 1)) == 0;
    if (x.rowmax_on || rebase) {
      const uint32_t rmu = __reduce_max_sync(FULL, lane_max16(h, kb, W));
      if (x.rowmax_on) {
        const int32_t rmax = (int32_t)rmu + off;
        if (x.cuton && lo <= cut) {
          int32_t row = rmax;
          if (hi > cut) row = (int32_t)__reduce_max_sync(FULL, lane_max16(h, kb, cut - lo + 1)) + off;
          b.cut_best = max(b.cut_best, row);
        }
        if (x.clip) {
          if (rmax > b.clip_best) {
            b.clip_best = rmax;
            if (x.cell) {
              b.ci = (uint32_t)i;
              b.cj = (uint32_t)(lo + leftmost16(h, rmu, lane));
            }
          }
          if (rmax < sat_sub(b.clip_best, x.P.xdrop)) {
            r = DRes{NEG, b.clip_best, b.cut_best, NEG, 0, b.ci, b.cj, (uint32_t)hi, (uint32_t)i,
                     b.rows, b.cells};
            stopped = true;
            break;
          }
        }
      }
      if (rebase) {
        const int32_t delta = (int32_t)rmu - (int32_t)kBias16;
        const uint32_t dd = ((uint32_t)(-delta) & 0xffffu) * kOne2;
#pragma unroll
        for (int k = 0; k < C2; ++k) {
          h[k] = __viaddmax_u16x2(h[k], dd, kNeg2);
          f[k] = __viaddmax_u16x2(f[k], dd, kNeg2);
        }
        off += delta;
      }
    }
    // The sentinel right of the band (align.rs:2490-2494), after any rebase.
    if (W < 32 * C && lane == W / C) set_neg16(h, f, W - kb);
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
    if (x.mode == 2) {
      const int32_t K = n - plo;
      const uint32_t u = __shfl_sync(FULL, field_at(h, K % C), (K / C) & 31);
      r.score = (int32_t)u + off;
      r.score_col = (uint32_t)n;
    } else {
      const uint32_t rmu = __reduce_max_sync(FULL, lane_max16(h, kb, W));
      r.score = (int32_t)rmu + off;
      r.score_col = (uint32_t)(plo + leftmost16(h, rmu, lane));
    }
    r.cut_score = NEG;
    if (x.cuton && plo <= cut) {
      const int32_t lim = min(phi, cut) - plo + 1;
      r.cut_score = (int32_t)__reduce_max_sync(FULL, lane_max16(h, kb, lim)) + off;
    }
  }
  if (lane == 0) a.out[jid] = r;
  if constexpr (TB) {
    __syncwarp();
    walk_lean(a, jid, tb_layout<C>(false, true, x.J, x.P.flags), x.J, x.P.flags, r, lane);
  }
  __syncwarp();
}

template <int C2>
struct MinBlocks16 {
  static constexpr int value = C2 <= 8 ? 6 : (C2 <= 14 ? 5 : (C2 <= 16 ? 4 : (C2 <= 24 ? 3 : 2)));
};

template <int C2, bool TB>
__global__ void __launch_bounds__(128, MinBlocks16<C2>::value) affine16_kernel(sfk::AffLaunch a) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    uint32_t q = 0;
    if (lane == 0) q = atomicAdd(a.counter, 1u);
    q = __shfl_sync(FULL, q, 0);
    if (q >= a.njobs) break;
    pair16<C2, TB>(a, a.order[q], lane);
  }
}

}  // namespace

namespace sfk {

template <int C2>
cudaError_t launch_affine16_c(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  if (tb)
    affine16_kernel<C2, true><<<grid, block, 0, s>>>(a);
  else
    affine16_kernel<C2, false><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace sfk
