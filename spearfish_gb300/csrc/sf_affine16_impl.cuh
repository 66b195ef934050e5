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
// bound fit (sf_plan.cu `fits16`); everything else runs on the 32-bit kernel.
//
// Layout.  A field holds value - offset (offset = -0x8000 at row 0, falling by ext a row, so
// that F's recurrence is one add-max), unsigned, so the DPX u16x2 maxima order fields as
// values, and a - b + 0x7fff7fff has bit 15 (31) set exactly when the low (high) field of a
// exceeds b's: one IADD3 per pair of traceback decisions.
// Lane l holds band offsets [l*C, l*C + C) as C/2 words: word k = (offset l*C + k,
// offset l*C + C/2 + k).  Both halves of a word advance together through pass 1, the
// lane's horizontal-gap chain and pass 2; the warp scan works on per-lane 32-bit values.
// Match scores come from one byte permute per word: a per-row table of the score of each
// text code against the row's pattern base, indexed by per-word selectors of the two text
// columns, which shift one column per row with the band.  Traceback decisions go out as one
// (A, B) word pair per lane and group of 8 words; sf_walk.cuh decodes that layout.
#pragma once
#include <utility>

#include "sf_affine_impl.cuh"

namespace {

constexpr uint32_t kBias16 = 0x8000u;
constexpr uint32_t kNeg16 = 0x4000u;
constexpr uint32_t kOne2 = 0x00010001u;
constexpr uint32_t kNeg2 = kNeg16 * kOne2;
constexpr uint32_t kGt2 = 0x7fff7fffu;
constexpr int kRebaseRows = 64;
// Score-only classes of up to this many words a lane run their steady rows in groups of C/2
// with the text selectors rotated by renaming (one copy of the row per group position).
// Measured on GB300: score-only 20,000 x 2 kb, band 128, 1,750 -> 1,880 GCUPS; with
// traceback the longer rows lost 4-14% (classes 8-16) and stay on register moves.
constexpr int kRenameC2 = 8;

__device__ __forceinline__ uint32_t pk2(uint32_t lo, uint32_t hi) { return lo | (hi << 16); }

// Calls f(std::integral_constant<int, k>) for k = 0 .. N - 1 (compile-time word indices).
template <int N, class F, int... K>
__device__ __forceinline__ void sf_unroll_impl(F&& f, std::integer_sequence<int, K...>) {
  (f(std::integral_constant<int, K>{}), ...);
}
template <int N, class F>
__device__ __forceinline__ void sf_unroll(F&& f) {
  sf_unroll_impl<N>(f, std::make_integer_sequence<int, N>{});
}

// Bit 15 / 31: the low / high field of a exceeds b's (fields within 0x7fff of each other).
__device__ __forceinline__ uint32_t gt2(uint32_t a, uint32_t b) { return a - b + kGt2; }

// Two decisions of word t (of its group of 8) into a traceback word: byte 0 / 1 receive the
// low / high field's decision of d1 at bit t, bytes 2 / 3 those of d2.  The byte permute
// (PTX prmt, whose selector nibbles with bit 3 set replicate the selected byte's msb; the
// __byte_perm intrinsic uses only 3 selector bits) spreads each compare bit (bit 15 / 31)
// over its byte, the mask keeps bit t.
template <int T>
__device__ __forceinline__ uint32_t push2(uint32_t acc, uint32_t d1, uint32_t d2) {
  uint32_t w;
  asm("prmt.b32 %0, %1, %2, 0xFDB9;" : "=r"(w) : "r"(d1), "r"(d2));
  return acc | (w & (0x01010101u << T));
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


// Sets word k's fields selected by ms (H and F) to NEG; k is the same in every lane (a
// uniform jump), ms is zero in the lanes that hold no field to set.
template <int C2>
__device__ __forceinline__ void set_word16(uint32_t (&h)[C2], uint32_t (&f)[C2], int k,
                                           uint32_t ms) {
  switch (k) {
#define SF_WORD16_CASE(q)                     \
  case q:                                     \
    if constexpr (q < C2) {                   \
      h[q] = (h[q] & ~ms) | (kNeg2 & ms);     \
      f[q] = (f[q] & ~ms) | (kNeg2 & ms);     \
    }                                         \
    break;
    SF_WORD16_CASE(0) SF_WORD16_CASE(1) SF_WORD16_CASE(2) SF_WORD16_CASE(3) SF_WORD16_CASE(4)
    SF_WORD16_CASE(5) SF_WORD16_CASE(6) SF_WORD16_CASE(7) SF_WORD16_CASE(8) SF_WORD16_CASE(9)
    SF_WORD16_CASE(10) SF_WORD16_CASE(11) SF_WORD16_CASE(12) SF_WORD16_CASE(13) SF_WORD16_CASE(14)
    SF_WORD16_CASE(15) SF_WORD16_CASE(16) SF_WORD16_CASE(17) SF_WORD16_CASE(18) SF_WORD16_CASE(19)
    SF_WORD16_CASE(20) SF_WORD16_CASE(21) SF_WORD16_CASE(22) SF_WORD16_CASE(23) SF_WORD16_CASE(24)
    SF_WORD16_CASE(25) SF_WORD16_CASE(26) SF_WORD16_CASE(27) SF_WORD16_CASE(28) SF_WORD16_CASE(29)
    SF_WORD16_CASE(30) SF_WORD16_CASE(31)
#undef SF_WORD16_CASE
    default:
      break;
  }
}

// A chained pass (align.rs:2210-2315): the row it resumes after (0: from row 0) and that
// row's slot; the chain's snapshot rows [base, want_end) of the want list, from `want` on the
// ones this pass may save, and the chain's first slot (word offset in the arena).
struct ChainRun {
  int32_t resume = 0;
  uint32_t base = 0, want = 0, want_end = 0;
  uint64_t slot0 = 0;
  uint32_t slot = 0;
};

template <int C2, bool TB, bool CH = false>
__device__ __forceinline__ DRes pair16(const sfk::AffLaunch& a, uint32_t jid, int lane, const ChainRun cr) {
  constexpr int C = 2 * C2;
  constexpr uint64_t kSlot = snap_slot_words(C2);
  constexpr int G = (C2 + 7) / 8;
  static_assert(2 * G == 2 * ((C + 15) / 16), "same traceback row size as the 32-bit kernel");
  // Rows of at most 8 words keep the sentinel's position as per-word masks; wider rows jump
  // to it (a switch), short of registers for the masks.
  constexpr bool kMasks = C2 <= 8;
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
  const uint32_t ext2 = (uint32_t)x.ext * kOne2;
  // Match scores enter as s + mis (mat + mis or 0, so that a plain add of both fields cannot
  // borrow); the maximum that takes the diagonal adds ext - mis (the row's drift, below, less
  // mis).  A row's table holds mat + mis in byte p (its pattern base) of ta (low bytes) and tb
  // (high bytes), 0 elsewhere.
  const uint32_t dgx2 = ((uint32_t)(x.ext - x.mis) & 0xffffu) * kOne2;  // mod 2^16 a field
  const uint32_t mpm = (uint32_t)(x.mat + x.mis) & 0xffffu;
  const uint32_t kGtDg = kGt2 + (uint32_t)(x.mis - x.ext) * kOne2;  // gt2 against that diagonal
  // Products with the opaque -1 issue on the FMA pipe too: a decision a - b + K becomes
  // a * one + (b * mone + K), two IMADs instead of one IADD3 on the ALU pipe, which the
  // maxima, table lookups and pushes keep busier.
  const uint32_t mone = 0u - one;
  const uint32_t fgx2 = ((uint32_t)(x.ext - x.go) & 0xffffu) * kOne2;  // + (ext - go) mod 2^16
  const uint32_t kGtFo = kGt2 + (uint32_t)(x.go - x.ext) * kOne2;    // gt2 against Hup + ext - go
  const uint32_t kGtGo = kGt2 + go2;                                  // gt2 against a value less go
  // Warp-scan decays: a lane's gap value falls by ext * C per lane it crosses.  The lane's
  // own chain is the maximum over its cells of H' + ext * k, less go + ext * (C/2 - 1).
  const int32_t dC = x.ext * C, dH = -x.ext * C2;
  const int32_t goX = x.go + x.ext * (C2 - 1);
  const int32_t e_lane = (int32_t)kNeg16 - dC * lane;  // NEG at the band's left end, decayed
  // value = field + off, and off falls by ext every row: a row's fields hold its values plus
  // ext for every row since row 0 (less the rebases), so that F = max(Hup - go, Fup - ext)
  // is one add-max on fields, F' = max(Hup' + ext - go, Fup'), and the diagonal gains ext.
  int32_t off = -(int32_t)kBias16;
  uint32_t h[C2], f[C2], sel[C2], smask[kMasks ? C2 : 1];
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
    }
  }
  {
    // Text selectors of row 1's columns; later rows shift them with the band.
    int32_t lo1, hi1;
    g.range(1, lo1, hi1);
    Win<C> win;
    win.load(a.pool, x.J.t_word, lo1 + kb);
#pragma unroll
    for (int k = 0; k < C2; ++k) sel[k] = sel_byte(win.at(k)) | (sel_byte(win.at(C2 + k)) << 8);
  }
  int32_t Wm = -1;  // the row width the sentinel masks are for
  auto set_masks = [&](int32_t W) {
    const int32_t c = W - kb;
#pragma unroll
    for (int k = 0; k < (kMasks ? C2 : 1); ++k)
      smask[k] = (c == k ? 0xffffu : 0u) | (c == C2 + k ? 0xffff0000u : 0u);
    Wm = W;
  };
  Book b;
  uint32_t pw = m > 0 ? __ldg(a.pool + x.J.p_word) >> 2 : 0;  // pattern bases from row 1
  uint2* tbp = TB ? reinterpret_cast<uint2*>(a.tb + x.J.tb_word) + lane : nullptr;
  // Chained passes: rows first .. m, with row first - 1 restored from its snapshot
  // (align.rs:2513-2524), and snapshots saved at the chain's rows from `wnext` on
  // (align.rs:2631-2641).
  int32_t first = 1;
  uint32_t wnext = cr.want;
  int32_t wrow = INT32_MAX;
  if constexpr (CH) {
    if (cr.resume > 0) {
      const int32_t rr = cr.resume;
      const uint32_t* s = a.snap + cr.slot0 + (uint64_t)cr.slot * kSlot;
#pragma unroll
      for (int k = 0; k < C2; ++k) {
        h[k] = __ldcg(s + k * 32 + lane);
        f[k] = __ldcg(s + (C2 + k) * 32 + lane);
      }
      off = (int32_t)__ldcg(s + 64 * C2);
      b.clip_best = (int32_t)__ldcg(s + 64 * C2 + 1);
      b.cut_best = (int32_t)__ldcg(s + 64 * C2 + 2);
      b.ci = __ldcg(s + 64 * C2 + 3);
      b.cj = __ldcg(s + 64 * C2 + 4);
      g.range(rr, plo, phi);
      // Row rr's text selectors (the band's columns from plo), and the pattern bases from
      // row rr + 1.
      Win<C> win;
      win.load(a.pool, x.J.t_word, plo + kb);
#pragma unroll
      for (int k = 0; k < C2; ++k)
        sel[k] = sel_byte(win.at(k)) | (sel_byte(win.at(C2 + k)) << 8);
      pw = __ldg(a.pool + x.J.p_word + ((uint32_t)(rr + 1) >> 4)) >> (2u * ((uint32_t)(rr + 1) & 15u));
      first = rr + 1;
    }
    wrow = wnext < cr.want_end ? (int32_t)__ldg(a.want + wnext) : INT32_MAX;
  }

  // One row.  D1: lo moved right by one (offset K reads the previous row at K + 1 above and
  // K diagonally); else lo stayed (K above, K - 1 diagonally; lo = 0, column 0 in lane 0).
  // Returns true when the pass stops at this row.
  // Rows whose band lies inside the text (lo > 0, i + above <= n) all have the width
  // below + above + 1: their sentinel sits in one word of one lane (ks, ms).
  int32_t Wc = 0, ks = 0;
  uint32_t ms = 0;
  bool sent = false;
  // ROT < 0: the row shifts the text selectors down one register (sel[k] = column k).
  // ROT = r >= 0 (steady rows in groups of C2, the group's row r): the selectors rotate by
  // renaming instead, register (k + r) mod C2 holding column k before the row's shift, and
  // the shift overwrites the register of the column that leaves.
  auto row = [&](int32_t i, auto modetag, auto rottag) -> bool {
    // MODE 0: lo = 0; 1: lo moves right by one; 2: as 1, with i + above <= n.
    constexpr int MODE = decltype(modetag)::value;
    constexpr int ROT = decltype(rottag)::value;
    constexpr bool D1 = MODE >= 1, ST = MODE == 2;
    // align.rs:2462-2468; rows past n + below (empty) never get here.
    const int32_t lo = D1 ? i - g.below : 0, hi = ST ? i + g.above : min(i + g.above, n);
    const int32_t W = ST ? Wc : hi - lo + 1;
    off -= x.ext;
    if ((i & 15) == 0) pw = __ldg(a.pool + x.J.p_word + (i >> 4));
    const uint32_t pb = 8u * (pw & 3u);
    pw >>= 2;
    const uint32_t ta = (mpm & 0xffu) << pb, tbl = (mpm >> 8) << pb;
    if (D1 && i > 1) {
      constexpr int R0 = ROT < 0 ? 0 : ROT;
      const uint32_t s0 = sel[R0];
      uint32_t nx = __shfl_down_sync(FULL, s0, 1);
      // The column entering lane 31 (32-bit positions: texts are shorter than 2^31).
      const uint32_t fcol = (uint32_t)(lo + 32 * C - 1);
      const uint32_t fw = __ldg(a.pool + x.J.t_word + (fcol >> 4));
      const uint32_t far = sel_byte((fw >> (2u * (fcol & 15u))) & 3u);
      if (lane == 31) nx = far;
      if constexpr (ROT < 0) {
#pragma unroll
        for (int k = 0; k + 1 < C2; ++k) sel[k] = sel[k + 1];
      }
      // (old word 0 high column, next lane's low)
      sel[ROT < 0 ? C2 - 1 : R0] = __byte_perm(s0, nx, 0x2241);
    }

    // Pass 1: F, H' and the lane's horizontal-gap chain.  F = max(Hup - go, Fup - ext): the
    // 32-bit kernel's floor at NEG only ever lifts values that lose to a reachable one, so
    // it is left out (F from the band's sentinel stays at NEG).
    uint32_t red = 0, pend = 0;  // maximum of H' + ext * k over the lane's words
    uint32_t acc1[G];
#pragma unroll
    for (int q = 0; q < G; ++q) acc1[q] = 0;
    auto cell = [&](auto kt, uint32_t hd, uint32_t hu, uint32_t fu) {
      constexpr int k = decltype(kt)::value;
      // F = max(Hup - go, Fup - ext), on fields that drift by ext a row.
      const uint32_t fj = __viaddmax_u16x2(hu, fgx2, fu);
      // This row's column k, after its shift.
      constexpr int sk = (D1 && ROT >= 0) ? (k + ROT + 1) % C2 : k;
      const uint32_t dgp = hd * one + __byte_perm(ta, tbl, sel[sk]);  // diagonal + s + mis
      const uint32_t xx = __viaddmax_u16x2(dgp, dgx2, fj);
      // "F extended": fj > Hup + ext - go; "diagonal lost": xx > dgp + ext - mis.
      if constexpr (TB)
        acc1[k >> 3] = push2<k & 7>(acc1[k >> 3], fj * one + (hu * mone + kGtFo),
                                    xx * one + (dgp * mone + kGtDg));
      const uint32_t t = xx * one + ext2 * (uint32_t)k;
      if constexpr (k == 0)
        red = t;
      else if constexpr (k & 1)
        pend = t;
      else
        red = __vimax3_u16x2(red, pend, t);
      f[k] = fj;
      h[k] = xx;
    };
    if constexpr (D1) {
      uint32_t nH = __shfl_down_sync(FULL, h[0], 1), nF = __shfl_down_sync(FULL, f[0], 1);
      if (lane == 31) nH = nF = kNeg2;
      const uint32_t upH = __byte_perm(h[0], nH, 0x5432), upF = __byte_perm(f[0], nF, 0x5432);
      sf_unroll<C2>([&](auto kt) {
        constexpr int k = decltype(kt)::value;
        cell(kt, h[k], k + 1 < C2 ? h[k + 1 < C2 ? k + 1 : 0] : upH,
             k + 1 < C2 ? f[k + 1 < C2 ? k + 1 : 0] : upF);
      });
    } else {
      // Lane 0's first cell is column 0, reached by a vertical gap alone
      // (align.rs:2558-2566); its diagonal gets a field no F can lose to.
      const uint32_t pl = __shfl_up_sync(FULL, h[C2 - 1], 1);
      uint32_t hd = __byte_perm(pl, h[C2 - 1], 0x5432);
      if (lane == 0) hd = (hd & 0xffff0000u) | (kNeg16 - (uint32_t)x.mat - 1u);
      sf_unroll<C2>([&](auto kt) {
        constexpr int k = decltype(kt)::value;
        const uint32_t hu = h[k];
        cell(kt, hd, hu, f[k]);
        hd = hu;
      });
    }

    if constexpr (C2 % 2 == 0) red = __vmaxu2(red, pend);
    // Gap entering each lane (32-bit fields): the lane's chain leaves its low half decayed
    // by ext * C/2 and meets its high half's.
    const int32_t clo = (int32_t)(red & 0xffffu) - goX, chi = (int32_t)(red >> 16) - goX;
    int32_t S = addmax(clo, dH, chi);
    S = addmax(__shfl_up_sync(FULL, S, 1), -dC, S);
    S = addmax(__shfl_up_sync(FULL, S, 2), -2 * dC, S);
    S = addmax(__shfl_up_sync(FULL, S, 4), -4 * dC, S);
    S = addmax(__shfl_up_sync(FULL, S, 8), -8 * dC, S);
    S = addmax(__shfl_up_sync(FULL, S, 16), -16 * dC, S);
    const int32_t Sp = __shfl_up_sync(FULL, S, 1);
    const int32_t ein = lane == 0 ? (int32_t)kNeg16 : max(e_lane, Sp);
    const int32_t ehi = addmax(ein, dH, clo);
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
    sf_unroll<C2>([&](auto kt) {
      constexpr int k = decltype(kt)::value;
      const uint32_t xx = h[k];
      const uint32_t xo = xp * one - go2;
      if (k > 0) e = __viaddmax_u16x2(e, next2, xo);
      // "E extended": e > H'left - go (FMA pipe); "H from E": e > H' (ALU pipe).
      if constexpr (TB)
        acc2[k >> 3] = push2<k & 7>(acc2[k >> 3], e * one + (xp * mone + kGtGo), gt2(e, xx));
      h[k] = __vmaxu2(xx, e);
      xp = xx;
    });
    if constexpr (TB) {
#pragma unroll
      for (int q = 0; q < G; ++q) tbp[q * 32] = make_uint2(acc1[q], acc2[q]);
      tbp += G * 32;
    }
    const bool rebase = (i & (kRebaseRows - 1)) == 0;
    if (x.rowmax_on || rebase) {
      const uint32_t rmu = __reduce_max_sync(FULL, lane_max16(h, kb, W));
      if (x.rowmax_on) {
        const int32_t rmax = (int32_t)rmu + off;
        if (x.cuton && lo <= cut) {
          int32_t rowv = rmax;
          if (hi > cut)
            rowv = (int32_t)__reduce_max_sync(FULL, lane_max16(h, kb, cut - lo + 1)) + off;
          b.cut_best = max(b.cut_best, rowv);
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
            r = DRes{NEG, b.clip_best, b.cut_best, NEG, 0, b.ci, b.cj, (uint32_t)hi,
                     (uint32_t)i, (uint32_t)i, band_cells(i, g.below, g.above, n)};
            return true;
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
    if constexpr (ST) {
      if (sent) set_word16(h, f, ks, ms);
    } else if (W < 32 * C) {
      if constexpr (kMasks) {
        if (W != Wm) set_masks(W);
#pragma unroll
        for (int k = 0; k < C2; ++k) {
          h[k] = (h[k] & ~smask[k]) | (kNeg2 & smask[k]);
          f[k] = (f[k] & ~smask[k]) | (kNeg2 & smask[k]);
        }
      } else if (lane == W / C) {
        set_neg16(h, f, W - kb);
      }
    }
    plo = lo;
    phi = hi;
    if constexpr (CH) {
      if (i == wrow) {
        uint32_t* s = a.snap + cr.slot0 + (uint64_t)(wnext - cr.base) * kSlot;
#pragma unroll
        for (int k = 0; k < C2; ++k) {
          __stcg(s + k * 32 + lane, h[k]);
          __stcg(s + (C2 + k) * 32 + lane, f[k]);
        }
        if (lane == 0) {
          __stcg(s + 64 * C2, (uint32_t)off);
          __stcg(s + 64 * C2 + 1, (uint32_t)b.clip_best);
          __stcg(s + 64 * C2 + 2, (uint32_t)b.cut_best);
          __stcg(s + 64 * C2 + 3, b.ci);
          __stcg(s + 64 * C2 + 4, b.cj);
        }
        ++wnext;
        wrow = wnext < cr.want_end ? (int32_t)__ldg(a.want + wnext) : INT32_MAX;
      }
    }
    return false;
  };

  // Rows 1 .. below keep lo = 0 (align.rs:2462-2468); later rows move it right by one.
  bool stopped = false;
  const int32_t endA = m < g.below ? m : g.below;
  const int64_t lastB = (int64_t)n + g.below;  // the last row whose band is not empty
  const int32_t endB = (int64_t)m < lastB ? m : (int32_t)lastB;
  const int32_t endS = min(endB, n - g.above);  // the last row with i + above <= n
  using Shift = std::integral_constant<int, -1>;
  using Steady = std::integral_constant<int, 2>;
  for (int32_t i = first; i <= endA && !stopped; ++i)
    stopped = row(i, std::integral_constant<int, 0>{}, Shift{});
  int32_t i1 = max(endA + 1, first);
  if (i1 <= endS) {
    Wc = g.below + g.above + 1;
    sent = Wc < 32 * C;
    const int32_t Ls = Wc / C, c = Wc - Ls * C;
    ks = c < C2 ? c : c - C2;
    ms = lane == Ls ? (c < C2 ? 0xffffu : 0xffff0000u) : 0u;
    Wm = -1;
    if constexpr (C2 <= kRenameC2 && !TB) {
      // Whole groups of C2 rows rotate the selectors by renaming (back in place after each
      // group); the rows left over shift them.  Row 1 shifts nothing: it runs first.
      if (i1 == 1 && !stopped) stopped = row(i1++, Steady{}, Shift{});
      while (i1 + C2 - 1 <= endS && !stopped) {
        sf_unroll<C2>([&](auto rt) {
          if (stopped) return;
          stopped = row(i1, Steady{}, std::integral_constant<int, decltype(rt)::value>{});
          ++i1;
        });
      }
    }
    for (; i1 <= endS && !stopped; ++i1) stopped = row(i1, Steady{}, Shift{});
  }
  for (int32_t i = i1; i <= endB && !stopped; ++i)
    stopped = row(i, std::integral_constant<int, 1>{}, Shift{});
  if (!stopped && endB < m) {
    // Row endB + 1 lies past the text: the pass ends there with no score (align.rs:2543-2553).
    r = DRes{NEG, b.clip_best, b.cut_best, NEG, 0, b.ci, b.cj, (uint32_t)n, (uint32_t)(endB + 1),
             (uint32_t)endB, band_cells(endB, g.below, g.above, n)};
    stopped = true;
  }
  if (!stopped) {
    const int32_t W = phi - plo + 1;
    r.clip_best = b.clip_best;
    r.cut_best = b.cut_best;
    r.clip_i = b.ci;
    r.clip_j = b.cj;
    r.text_read = (uint32_t)phi;
    r.last_row = (uint32_t)m;
    r.rows = (uint32_t)m;
    r.cells = band_cells(m, g.below, g.above, n);
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
  return r;
}

// ---------------------------------------------------------------------------------------
// Two-warp passes: the same rows on 64 lanes, the two warps of a 64-thread block each holding
// 32 lanes of C cells, for bands too wide for one warp to run at speed: a long pass is bound
// by its own row latency (one warp's dependent chain per row), and splitting its row shortens
// that chain.  Lane l (0..63, warp l / 32) holds offsets [l*C, l*C + C).  Per row the warps
// exchange values through shared memory, each exchange behind a block barrier:
//  - after pass 1 and each warp's gap scan: warp 0's scan total (the gap entering warp 1) and
//    its last H' (left of warp 1's first cell);
//  - after the row: warp 1's first H and F (above warp 0's last cell in the next row) and
//    warp 0's last H (left of warp 1's first cell in the next row while lo = 0);
//  - in rows that need a row maximum (the rebase every 64 rows, clip and X-drop, cut): each
//    warp's maximum, so that both warps take the same decisions.
// Every barrier sits on a path both warps take (every branch around one tests values both
// warps hold alike), and the block is the pass's two warps alone, so a barrier is the plain
// block barrier.  Warp 0 walks the traceback; its layout is the one-warp layout with 64 lanes
// to a group.
struct Team16 {
  uint32_t nh, nf;   // warp 1's first H and F after the last row
  uint32_t ph;       // warp 0's last H after the last row
  uint32_t hx;       // warp 0's last H' of this row
  int32_t s0;        // warp 0's gap total of this row
  uint32_t v[4][2];  // per-warp values of a row's maxima and leftmost cells; the score
  uint32_t job;
};

template <int C2, bool TB>
__device__ __forceinline__ void pair16w(const sfk::AffLaunch& a, uint32_t jid, int lane, int w,
                                        Team16& X) {
  constexpr int C = 2 * C2;
  constexpr int G = (C2 + 7) / 8;
  constexpr int LP = 64;
  constexpr bool kMasks = C2 <= 8;
  const int l = 32 * w + lane;
  const PassCtx x = make_ctx(a, jid);
  DRes r{};
  const int32_t m = (int32_t)x.m, n = (int32_t)x.n;
  const Geo32 g{(x.P.flags & F_FULL) != 0, false, clamp30(x.J.below), clamp30(x.J.above), n};
  const int32_t cut =
      x.cuton ? (int32_t)(x.J.cut < (uint64_t)n + 1 ? x.J.cut : (uint64_t)n + 1) : INT32_MAX;
  const int32_t kb = l * C;
  const uint32_t one = (uint32_t)opaque_one();
  const uint32_t go2 = (uint32_t)x.go * kOne2;
  const uint32_t next2 = ((uint32_t)(-x.ext) & 0xffffu) * kOne2;
  const uint32_t ext2 = (uint32_t)x.ext * kOne2;
  const uint32_t dgx2 = ((uint32_t)(x.ext - x.mis) & 0xffffu) * kOne2;
  const uint32_t mpm = (uint32_t)(x.mat + x.mis) & 0xffffu;
  const uint32_t kGtDg = kGt2 + (uint32_t)(x.mis - x.ext) * kOne2;
  const uint32_t mone = 0u - one;
  const uint32_t fgx2 = ((uint32_t)(x.ext - x.go) & 0xffffu) * kOne2;
  const uint32_t kGtFo = kGt2 + (uint32_t)(x.go - x.ext) * kOne2;
  const uint32_t kGtGo = kGt2 + go2;
  const int32_t dC = x.ext * C, dH = -x.ext * C2;
  const int32_t goX = x.go + x.ext * (C2 - 1);
  const int32_t e_lane = (int32_t)kNeg16 - dC * l;
  int32_t off = -(int32_t)kBias16;
  uint32_t h[C2], f[C2], sel[C2], smask[kMasks ? C2 : 1];
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
    }
  }
  {
    int32_t lo1, hi1;
    g.range(1, lo1, hi1);
    Win<C> win;
    win.load(a.pool, x.J.t_word, lo1 + kb);
#pragma unroll
    for (int k = 0; k < C2; ++k) sel[k] = sel_byte(win.at(k)) | (sel_byte(win.at(C2 + k)) << 8);
  }
  int32_t Wm = -1;
  auto set_masks = [&](int32_t W) {
    const int32_t c = W - kb;
#pragma unroll
    for (int k = 0; k < (kMasks ? C2 : 1); ++k)
      smask[k] = (c == k ? 0xffffu : 0u) | (c == C2 + k ? 0xffff0000u : 0u);
    Wm = W;
  };
  // The pass's maximum of a per-lane value (slot s of this row's exchanges).
  auto team_max = [&](uint32_t v, int s) -> uint32_t {
    v = __reduce_max_sync(FULL, v);
    if (lane == 0) X.v[s][w] = v;
    __syncthreads();
    return max(X.v[s][0], X.v[s][1]);
  };
  // Leftmost offset of the pass holding field v (some lane holds it).
  auto team_leftmost = [&](uint32_t v, int s) -> uint32_t {
    int cf = C;
#pragma unroll
    for (int c = C - 1; c >= 0; --c) {
      const uint32_t u = c < C2 ? (h[c] & 0xffffu) : (h[c - C2] >> 16);
      if (u == v) cf = c;
    }
    const uint32_t bal = __ballot_sync(FULL, cf < C);
    const int src = __ffs(bal) - 1;
    const int cs = __shfl_sync(FULL, cf, src < 0 ? 0 : src);
    const uint32_t mine = src < 0 ? 0xffffffffu : (uint32_t)(32 * w + src) * C + (uint32_t)cs;
    if (lane == 0) X.v[s][w] = mine;
    __syncthreads();
    return min(X.v[s][0], X.v[s][1]);
  };
  Book b;
  uint32_t pw = m > 0 ? __ldg(a.pool + x.J.p_word) >> 2 : 0;
  uint2* tbp = TB ? reinterpret_cast<uint2*>(a.tb + x.J.tb_word) + l : nullptr;
  // Row 0's values at the seam, for row 1.
  if (w == 1 && lane == 0) {
    X.nh = h[0];
    X.nf = f[0];
  }
  if (w == 0 && lane == 31) X.ph = h[C2 - 1];
  __syncthreads();

  int32_t Wc = 0, ks = 0;
  uint32_t ms = 0;
  bool sent = false;
  auto row = [&](int32_t i, auto modetag) -> bool {
    constexpr int MODE = decltype(modetag)::value;
    constexpr bool D1 = MODE >= 1, ST = MODE == 2;
    const int32_t lo = D1 ? i - g.below : 0, hi = ST ? i + g.above : min(i + g.above, n);
    const int32_t W = ST ? Wc : hi - lo + 1;
    off -= x.ext;  // fields drift by ext a row (pair16)
    if ((i & 15) == 0) pw = __ldg(a.pool + x.J.p_word + (i >> 4));
    const uint32_t pb = 8u * (pw & 3u);
    pw >>= 2;
    const uint32_t ta = (mpm & 0xffu) << pb, tbl = (mpm >> 8) << pb;
    if (D1 && i > 1) {
      const uint32_t s0 = sel[0];
      uint32_t nx = __shfl_down_sync(FULL, s0, 1);
      // The column entering this warp's lane 31: the next warp's first, or past the band.
      const uint32_t fcol = (uint32_t)(lo + 32 * (w + 1) * C - 1);
      const uint32_t fw = __ldg(a.pool + x.J.t_word + (fcol >> 4));
      const uint32_t far = sel_byte((fw >> (2u * (fcol & 15u))) & 3u);
      if (lane == 31) nx = far;
#pragma unroll
      for (int k = 0; k + 1 < C2; ++k) sel[k] = sel[k + 1];
      sel[C2 - 1] = __byte_perm(s0, nx, 0x2241);
    }

    uint32_t red = 0, pend = 0;
    uint32_t acc1[G];
#pragma unroll
    for (int q = 0; q < G; ++q) acc1[q] = 0;
    auto cell = [&](auto kt, uint32_t hd, uint32_t hu, uint32_t fu) {
      constexpr int k = decltype(kt)::value;
      const uint32_t fj = __viaddmax_u16x2(hu, fgx2, fu);
      const uint32_t dgp = hd * one + __byte_perm(ta, tbl, sel[k]);
      const uint32_t xx = __viaddmax_u16x2(dgp, dgx2, fj);
      if constexpr (TB)
        acc1[k >> 3] = push2<k & 7>(acc1[k >> 3], fj * one + (hu * mone + kGtFo),
                                    xx * one + (dgp * mone + kGtDg));
      const uint32_t t = xx * one + ext2 * (uint32_t)k;
      if constexpr (k == 0)
        red = t;
      else if constexpr (k & 1)
        pend = t;
      else
        red = __vimax3_u16x2(red, pend, t);
      f[k] = fj;
      h[k] = xx;
    };
    if constexpr (D1) {
      uint32_t nH = __shfl_down_sync(FULL, h[0], 1), nF = __shfl_down_sync(FULL, f[0], 1);
      if (lane == 31) {
        nH = w == 0 ? X.nh : kNeg2;
        nF = w == 0 ? X.nf : kNeg2;
      }
      const uint32_t upH = __byte_perm(h[0], nH, 0x5432), upF = __byte_perm(f[0], nF, 0x5432);
      sf_unroll<C2>([&](auto kt) {
        constexpr int k = decltype(kt)::value;
        cell(kt, h[k], k + 1 < C2 ? h[k + 1 < C2 ? k + 1 : 0] : upH,
             k + 1 < C2 ? f[k + 1 < C2 ? k + 1 : 0] : upF);
      });
    } else {
      uint32_t pl = __shfl_up_sync(FULL, h[C2 - 1], 1);
      if (lane == 0 && w == 1) pl = X.ph;
      uint32_t hd = __byte_perm(pl, h[C2 - 1], 0x5432);
      if (l == 0) hd = (hd & 0xffff0000u) | (kNeg16 - (uint32_t)x.mat - 1u);
      sf_unroll<C2>([&](auto kt) {
        constexpr int k = decltype(kt)::value;
        const uint32_t hu = h[k];
        cell(kt, hd, hu, f[k]);
        hd = hu;
      });
    }

    if constexpr (C2 % 2 == 0) red = __vmaxu2(red, pend);
    const int32_t clo = (int32_t)(red & 0xffffu) - goX, chi = (int32_t)(red >> 16) - goX;
    int32_t S = addmax(clo, dH, chi);
    S = addmax(__shfl_up_sync(FULL, S, 1), -dC, S);
    S = addmax(__shfl_up_sync(FULL, S, 2), -2 * dC, S);
    S = addmax(__shfl_up_sync(FULL, S, 4), -4 * dC, S);
    S = addmax(__shfl_up_sync(FULL, S, 8), -8 * dC, S);
    S = addmax(__shfl_up_sync(FULL, S, 16), -16 * dC, S);
    // Warp 0's total and last H' to warp 1: the gap entering lane 32 + j is the larger of its
    // warp's own scan and warp 0's total decayed over j + 1 lanes.
    if (w == 0 && lane == 31) {
      X.s0 = S;
      X.hx = h[C2 - 1];
    }
    __syncthreads();
    int32_t Sp;
    uint32_t pl2 = __shfl_up_sync(FULL, h[C2 - 1], 1);
    if (w == 1) {
      const int32_t T = X.s0;
      S = addmax(T, -dC * (lane + 1), S);
      Sp = __shfl_up_sync(FULL, S, 1);
      if (lane == 0) {
        Sp = T;
        pl2 = X.hx;
      }
    } else {
      Sp = __shfl_up_sync(FULL, S, 1);
    }
    const int32_t ein = l == 0 ? (int32_t)kNeg16 : max(e_lane, Sp);
    const int32_t ehi = addmax(ein, dH, clo);
    uint32_t e = pk2((uint32_t)ein, (uint32_t)ehi);
    uint32_t xp = __byte_perm(pl2, h[C2 - 1], 0x5432);
    if (l == 0) xp = (xp & 0xffff0000u) | (kNeg16 - 1u);

    uint32_t acc2[G];
#pragma unroll
    for (int q = 0; q < G; ++q) acc2[q] = 0;
    sf_unroll<C2>([&](auto kt) {
      constexpr int k = decltype(kt)::value;
      const uint32_t xx = h[k];
      const uint32_t xo = xp * one - go2;
      if (k > 0) e = __viaddmax_u16x2(e, next2, xo);
      if constexpr (TB)
        acc2[k >> 3] = push2<k & 7>(acc2[k >> 3], e * one + (xp * mone + kGtGo), gt2(e, xx));
      h[k] = __vmaxu2(xx, e);
      xp = xx;
    });
    if constexpr (TB) {
#pragma unroll
      for (int q = 0; q < G; ++q) tbp[q * LP] = make_uint2(acc1[q], acc2[q]);
      tbp += G * LP;
    }
    const bool rebase = (i & (kRebaseRows - 1)) == 0;
    if (x.rowmax_on || rebase) {
      const uint32_t rmu = team_max(lane_max16(h, kb, W), 0);
      if (x.rowmax_on) {
        const int32_t rmax = (int32_t)rmu + off;
        if (x.cuton && lo <= cut) {
          int32_t rowv = rmax;
          if (hi > cut) rowv = (int32_t)team_max(lane_max16(h, kb, cut - lo + 1), 1) + off;
          b.cut_best = max(b.cut_best, rowv);
        }
        if (x.clip) {
          if (rmax > b.clip_best) {
            b.clip_best = rmax;
            if (x.cell) {
              b.ci = (uint32_t)i;
              b.cj = (uint32_t)lo + team_leftmost(rmu, 2);
            }
          }
          if (rmax < sat_sub(b.clip_best, x.P.xdrop)) {
            r = DRes{NEG, b.clip_best, b.cut_best, NEG, 0, b.ci, b.cj, (uint32_t)hi,
                     (uint32_t)i, (uint32_t)i, band_cells(i, g.below, g.above, n)};
            return true;
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
    if constexpr (ST) {
      if (sent) set_word16(h, f, ks, ms);
    } else if (W < LP * C) {
      if constexpr (kMasks) {
        if (W != Wm) set_masks(W);
#pragma unroll
        for (int k = 0; k < C2; ++k) {
          h[k] = (h[k] & ~smask[k]) | (kNeg2 & smask[k]);
          f[k] = (f[k] & ~smask[k]) | (kNeg2 & smask[k]);
        }
      } else if (l == W / C) {
        set_neg16(h, f, W - kb);
      }
    }
    plo = lo;
    phi = hi;
    // The seam values for the next row.
    if (w == 1 && lane == 0) {
      X.nh = h[0];
      X.nf = f[0];
    }
    if (w == 0 && lane == 31) X.ph = h[C2 - 1];
    __syncthreads();
    return false;
  };

  bool stopped = false;
  const int32_t endA = m < g.below ? m : g.below;
  const int64_t lastB = (int64_t)n + g.below;
  const int32_t endB = (int64_t)m < lastB ? m : (int32_t)lastB;
  const int32_t endS = min(endB, n - g.above);
  for (int32_t i = 1; i <= endA && !stopped; ++i)
    stopped = row(i, std::integral_constant<int, 0>{});
  int32_t i1 = endA + 1;
  if (i1 <= endS) {
    Wc = g.below + g.above + 1;
    sent = Wc < LP * C;
    const int32_t Ls = Wc / C, c = Wc - Ls * C;
    ks = c < C2 ? c : c - C2;
    ms = l == Ls ? (c < C2 ? 0xffffu : 0xffff0000u) : 0u;
    Wm = -1;
    for (; i1 <= endS && !stopped; ++i1) stopped = row(i1, std::integral_constant<int, 2>{});
  }
  for (int32_t i = i1; i <= endB && !stopped; ++i)
    stopped = row(i, std::integral_constant<int, 1>{});
  if (!stopped && endB < m) {
    r = DRes{NEG, b.clip_best, b.cut_best, NEG, 0, b.ci, b.cj, (uint32_t)n, (uint32_t)(endB + 1),
             (uint32_t)endB, band_cells(endB, g.below, g.above, n)};
    stopped = true;
  }
  if (!stopped) {
    const int32_t W = phi - plo + 1;
    r.clip_best = b.clip_best;
    r.cut_best = b.cut_best;
    r.clip_i = b.ci;
    r.clip_j = b.cj;
    r.text_read = (uint32_t)phi;
    r.last_row = (uint32_t)m;
    r.rows = (uint32_t)m;
    r.cells = band_cells(m, g.below, g.above, n);
    if (x.mode == 2) {
      const int32_t K = n - plo;
      const uint32_t u = __shfl_sync(FULL, field_at(h, K % C), (K / C) & 31);
      if (lane == 0 && w == ((K / C) >> 5)) X.v[3][0] = u;
      __syncthreads();
      r.score = (int32_t)X.v[3][0] + off;
      r.score_col = (uint32_t)n;
    } else {
      const uint32_t rmu = team_max(lane_max16(h, kb, W), 0);
      r.score = (int32_t)rmu + off;
      r.score_col = (uint32_t)plo + team_leftmost(rmu, 2);
    }
    r.cut_score = NEG;
    if (x.cuton && plo <= cut) {
      const int32_t lim = min(phi, cut) - plo + 1;
      r.cut_score = (int32_t)team_max(lane_max16(h, kb, lim), 1) + off;
    }
  }
  if (w == 0) {
    if (lane == 0) a.out[jid] = r;
    if constexpr (TB) {
      __syncwarp();
      walk_lean(a, jid, tb_layout<C>(false, true, x.J, x.P.flags, LP), x.J, x.P.flags, r, lane);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------------------
// Half-warp passes: the same rows with 16 lanes to a pass and two passes to a warp, so that a
// row's fixed costs (the gap scan, the neighbour shuffles, table and bookkeeping work) are
// shared between the warp's two passes and a lane holds twice the cells.  Lane l of segment
// s = lane / 16 holds offsets [(l % 16) * C, (l % 16) * C + C) of its own pass.  The two
// passes run their rows in lockstep; each keeps its own geometry, band shift, offset and
// bookkeeping, and a pass that has ended (or stopped) computes on without storing until its
// partner ends.

// Maximum over the 16 lanes of a segment.
__device__ __forceinline__ uint32_t seg_max(uint32_t v) {
#pragma unroll
  for (int s = 8; s >= 1; s >>= 1) v = max(v, __shfl_xor_sync(FULL, v, s, 16));
  return v;
}

// Leftmost offset holding field v in the lane's segment (some lane of it holds it).
template <int C2>
__device__ __forceinline__ uint32_t seg_leftmost(const uint32_t (&h)[C2], uint32_t v, int lane) {
  constexpr int C = 2 * C2;
  int cf = C;
#pragma unroll
  for (int c = C - 1; c >= 0; --c) {
    const uint32_t u = c < C2 ? (h[c] & 0xffffu) : (h[c - C2] >> 16);
    if (u == v) cf = c;
  }
  const uint32_t bal = (__ballot_sync(FULL, cf < C) >> (lane & 16)) & 0xffffu;
  const int src = __ffs(bal) - 1;
  const int cs = __shfl_sync(FULL, cf, src < 0 ? 0 : src, 16);
  return (uint32_t)(src < 0 ? 0 : src) * C + (uint32_t)cs;
}

template <int C2, bool TB>
__device__ void pair16h(const sfk::AffLaunch& a, uint32_t jid, bool has, int lane) {
  constexpr int P = 16;
  constexpr int C = 2 * C2;
  constexpr int G = (C2 + 7) / 8;
  constexpr bool kMasks = C2 <= 8;
  const int l = lane & 15;
  const PassCtx x = make_ctx(a, jid);
  const int32_t m = (int32_t)x.m, n = (int32_t)x.n;
  const Geo32 g{(x.P.flags & F_FULL) != 0, false, clamp30(x.J.below), clamp30(x.J.above), n};
  const int32_t cut =
      x.cuton ? (int32_t)(x.J.cut < (uint64_t)n + 1 ? x.J.cut : (uint64_t)n + 1) : INT32_MAX;
  const int32_t kb = l * C;
  const uint32_t one = (uint32_t)opaque_one();
  const uint32_t go2 = (uint32_t)x.go * kOne2;
  const uint32_t next2 = ((uint32_t)(-x.ext) & 0xffffu) * kOne2;
  const uint32_t ext2 = (uint32_t)x.ext * kOne2;
  const uint32_t dgx2 = ((uint32_t)(x.ext - x.mis) & 0xffffu) * kOne2;
  const uint32_t mpm = (uint32_t)(x.mat + x.mis) & 0xffffu;
  const uint32_t kGtDg = kGt2 + (uint32_t)(x.mis - x.ext) * kOne2;
  const uint32_t mone = 0u - one;
  const uint32_t fgx2 = ((uint32_t)(x.ext - x.go) & 0xffffu) * kOne2;
  const uint32_t kGtFo = kGt2 + (uint32_t)(x.go - x.ext) * kOne2;
  const uint32_t kGtGo = kGt2 + go2;
  const int32_t dC = x.ext * C, dH = -x.ext * C2;
  const int32_t goX = x.go + x.ext * (C2 - 1);
  const int32_t e_lane = (int32_t)kNeg16 - dC * l;
  int32_t off = -(int32_t)kBias16;
  uint32_t h[C2], f[C2], sel[C2], smask[kMasks ? C2 : 1];
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
    }
  }
  {
    int32_t lo1, hi1;
    g.range(1, lo1, hi1);
    Win<C> win;
    win.load(a.pool, x.J.t_word, lo1 + kb);
#pragma unroll
    for (int k = 0; k < C2; ++k) sel[k] = sel_byte(win.at(k)) | (sel_byte(win.at(C2 + k)) << 8);
  }
  int32_t Wm = -1;
  auto set_masks = [&](int32_t W) {
    const int32_t c = W - kb;
#pragma unroll
    for (int k = 0; k < (kMasks ? C2 : 1); ++k)
      smask[k] = (c == k ? 0xffffu : 0u) | (c == C2 + k ? 0xffff0000u : 0u);
    Wm = W;
  };
  Book b;
  uint32_t pw = m > 0 ? __ldg(a.pool + x.J.p_word) >> 2 : 0;
  uint2* tb0 = TB ? reinterpret_cast<uint2*>(a.tb + x.J.tb_word) + l : nullptr;
  // This pass's rows: 1 .. endA keep lo = 0; endA + 1 .. endB move it; rows past n + below
  // are empty (the pass ends there with no score).  The warp runs to its longer pass's end.
  const int32_t endA = m < g.below ? m : g.below;
  const int64_t lastB = (int64_t)n + g.below;
  const int32_t endB = (int64_t)m < lastB ? m : (int32_t)lastB;
  const int32_t endA2 = max(endA, __shfl_xor_sync(FULL, endA, 16));
  const int32_t endW = max(endB, __shfl_xor_sync(FULL, endB, 16));
  int32_t fin = has ? 0 : -1;  // 0: running; > 0 ended at that row; -1: nothing to store
  DRes r{};

  // The pass's result from its last row i (band [lo, hi], values in h).  Every lane of the
  // warp runs it (segment shuffles); a lane keeps it only for its own ending pass.
  auto result = [&](int32_t i, int32_t lo, int32_t hi) {
    const int32_t W = hi - lo + 1;
    DRes q{};
    q.clip_best = b.clip_best;
    q.cut_best = b.cut_best;
    q.clip_i = b.ci;
    q.clip_j = b.cj;
    q.text_read = (uint32_t)hi;
    q.last_row = (uint32_t)m;
    q.rows = (uint32_t)m;
    q.cells = band_cells(m, g.below, g.above, n);
    const int32_t K = n - lo;
    const uint32_t u = __shfl_sync(FULL, field_at(h, K % C), (K / C) & 15, 16);
    const uint32_t rmu = seg_max(lane_max16(h, kb, W));
    const uint32_t lm = seg_leftmost(h, rmu, lane);
    const int32_t lim = min(hi, cut) - lo + 1;
    const uint32_t cm = seg_max(lane_max16(h, kb, lim));
    if (x.mode == 2) {
      q.score = (int32_t)u + off;
      q.score_col = (uint32_t)n;
    } else {
      q.score = (int32_t)rmu + off;
      q.score_col = (uint32_t)(lo + lm);
    }
    q.cut_score = (x.cuton && lo <= cut) ? (int32_t)cm + off : NEG;
    (void)i;
    return q;
  };

  // One row of both passes.  MODE 1: both passes' lo moves right by one (compile time);
  // MODE 0: per pass (d1), the rows before the band leaves column 0.
  auto row = [&](int32_t i, auto modetag, bool d1) {
    constexpr bool ALL1 = decltype(modetag)::value;
    const bool D1 = ALL1 ? true : d1;
    const bool act = fin == 0 && i <= endB;
    const int32_t lo = D1 ? i - g.below : 0, hi = min(i + g.above, n);
    const int32_t W = hi - lo + 1;
    off -= x.ext;  // fields drift by ext a row (pair16)
    if ((i & 15) == 0) pw = __ldg(a.pool + x.J.p_word + ((i <= m ? i : m) >> 4));
    const uint32_t pb = 8u * (pw & 3u);
    pw >>= 2;
    const uint32_t ta = (mpm & 0xffu) << pb, tbl = (mpm >> 8) << pb;
    {
      const uint32_t s0 = sel[0];
      uint32_t nx = __shfl_down_sync(FULL, s0, 1, 16);
      int32_t fc = lo + P * C - 1;
      fc = fc < n ? fc : n;
      const uint32_t far = sel_byte(base_at(a.pool, x.J.t_word, (uint64_t)(fc > 0 ? fc : 0)));
      if (l == 15) nx = far;
      const bool shift = D1 && i > 1;
      const uint32_t last = __byte_perm(s0, nx, 0x2241);
      if (ALL1) {
        if (i > 1) {
#pragma unroll
          for (int k = 0; k + 1 < C2; ++k) sel[k] = sel[k + 1];
          sel[C2 - 1] = last;
        }
      } else {
#pragma unroll
        for (int k = 0; k + 1 < C2; ++k) sel[k] = shift ? sel[k + 1] : sel[k];
        sel[C2 - 1] = shift ? last : sel[C2 - 1];
      }
    }
    uint32_t nH = __shfl_down_sync(FULL, h[0], 1, 16), nF = __shfl_down_sync(FULL, f[0], 1, 16);
    if (l == 15) nH = nF = kNeg2;
    const uint32_t upH = __byte_perm(h[0], nH, 0x5432), upF = __byte_perm(f[0], nF, 0x5432);
    uint32_t hdp = 0;
    if (!ALL1) {
      const uint32_t pl = __shfl_up_sync(FULL, h[C2 - 1], 1, 16);
      hdp = __byte_perm(pl, h[C2 - 1], 0x5432);
      if (l == 0) hdp = (hdp & 0xffff0000u) | (kNeg16 - (uint32_t)x.mat - 1u);
    }
    uint32_t red = 0, pend = 0;
    uint32_t acc1[G];
#pragma unroll
    for (int q = 0; q < G; ++q) acc1[q] = 0;
    sf_unroll<C2>([&](auto kt) {
      constexpr int k = decltype(kt)::value;
      const uint32_t hk = h[k], fk = f[k];
      const uint32_t hu1 = k + 1 < C2 ? h[k + 1 < C2 ? k + 1 : 0] : upH;
      const uint32_t fu1 = k + 1 < C2 ? f[k + 1 < C2 ? k + 1 : 0] : upF;
      uint32_t hu, fu, hd;
      if (ALL1) {
        hu = hu1;
        fu = fu1;
        hd = hk;
      } else {
        hu = D1 ? hu1 : hk;
        fu = D1 ? fu1 : fk;
        hd = D1 ? hk : hdp;
        hdp = hk;
      }
      const uint32_t fj = __viaddmax_u16x2(hu, fgx2, fu);
      const uint32_t dgp = hd * one + __byte_perm(ta, tbl, sel[k]);
      const uint32_t xx = __viaddmax_u16x2(dgp, dgx2, fj);
      if constexpr (TB)
        acc1[k >> 3] = push2<k & 7>(acc1[k >> 3], fj * one + (hu * mone + kGtFo),
                                    xx * one + (dgp * mone + kGtDg));
      const uint32_t t = xx * one + ext2 * (uint32_t)k;
      if constexpr (k == 0)
        red = t;
      else if constexpr (k & 1)
        pend = t;
      else
        red = __vimax3_u16x2(red, pend, t);
      f[k] = fj;
      h[k] = xx;
    });
    if constexpr (C2 % 2 == 0) red = __vmaxu2(red, pend);
    const int32_t clo = (int32_t)(red & 0xffffu) - goX, chi = (int32_t)(red >> 16) - goX;
    int32_t S = addmax(clo, dH, chi);
    S = addmax(__shfl_up_sync(FULL, S, 1, 16), -dC, S);
    S = addmax(__shfl_up_sync(FULL, S, 2, 16), -2 * dC, S);
    S = addmax(__shfl_up_sync(FULL, S, 4, 16), -4 * dC, S);
    S = addmax(__shfl_up_sync(FULL, S, 8, 16), -8 * dC, S);
    const int32_t Sp = __shfl_up_sync(FULL, S, 1, 16);
    const int32_t ein = l == 0 ? (int32_t)kNeg16 : max(e_lane, Sp);
    const int32_t ehi = addmax(ein, dH, clo);
    uint32_t e = pk2((uint32_t)ein, (uint32_t)ehi);
    const uint32_t pl2 = __shfl_up_sync(FULL, h[C2 - 1], 1, 16);
    uint32_t xp = __byte_perm(pl2, h[C2 - 1], 0x5432);
    if (l == 0) xp = (xp & 0xffff0000u) | (kNeg16 - 1u);
    uint32_t acc2[G];
#pragma unroll
    for (int q = 0; q < G; ++q) acc2[q] = 0;
    sf_unroll<C2>([&](auto kt) {
      constexpr int k = decltype(kt)::value;
      const uint32_t xx = h[k];
      const uint32_t xo = xp * one - go2;
      if (k > 0) e = __viaddmax_u16x2(e, next2, xo);
      // "E extended": e > H'left - go (FMA pipe); "H from E": e > H' (ALU pipe).
      if constexpr (TB)
        acc2[k >> 3] = push2<k & 7>(acc2[k >> 3], e * one + (xp * mone + kGtGo), gt2(e, xx));
      h[k] = __vmaxu2(xx, e);
      xp = xx;
    });
    if constexpr (TB) {
      if (act) {
        uint2* tp = tb0 + (uint64_t)(i - 1) * (G * P);
#pragma unroll
        for (int q = 0; q < G; ++q) tp[q * P] = make_uint2(acc1[q], acc2[q]);
      }
    }
    // Row bookkeeping (align.rs:2580-2640), each pass for itself; the segment shuffles run
    // on every lane.
    const bool want = act && x.rowmax_on;
    const bool rebase = (i & (kRebaseRows - 1)) == 0;
    if (__any_sync(FULL, want) || rebase) {
      const uint32_t rmu = seg_max(lane_max16(h, kb, W));
      const int32_t limc = (x.cuton && lo <= cut && hi > cut) ? cut - lo + 1 : W;
      const uint32_t rcut = seg_max(lane_max16(h, kb, limc));
      bool raise = false;
      if (want) {
        const int32_t rmax = (int32_t)rmu + off;
        if (x.cuton && lo <= cut) b.cut_best = max(b.cut_best, (int32_t)rcut + off);
        if (x.clip && rmax > b.clip_best) {
          b.clip_best = rmax;
          if (x.cell) {
            b.ci = (uint32_t)i;
            raise = true;
          }
        }
      }
      if (__any_sync(FULL, raise)) {
        const uint32_t lm = seg_leftmost(h, rmu, lane);
        if (raise) b.cj = (uint32_t)(lo + lm);
      }
      if (want && x.clip && (int32_t)rmu + off < sat_sub(b.clip_best, x.P.xdrop)) {
        r = DRes{NEG, b.clip_best, b.cut_best, NEG, 0, b.ci, b.cj, (uint32_t)hi, (uint32_t)i,
                 (uint32_t)i, band_cells(i, g.below, g.above, n)};
        fin = i;
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
    if (W < P * C) {
      if constexpr (kMasks) {
        if (W != Wm) set_masks(W);
#pragma unroll
        for (int k = 0; k < C2; ++k) {
          h[k] = (h[k] & ~smask[k]) | (kNeg2 & smask[k]);
          f[k] = (f[k] & ~smask[k]) | (kNeg2 & smask[k]);
        }
      } else if (l == W / C) {
        set_neg16(h, f, W - kb);
      }
    }
    const bool last = fin == 0 && i == endB;
    if (__any_sync(FULL, last)) {
      const DRes q = result(i, lo, hi);
      if (last) {
        r = endB < m ? DRes{NEG, b.clip_best, b.cut_best, NEG, 0, b.ci, b.cj, (uint32_t)n,
                            (uint32_t)(endB + 1), (uint32_t)endB,
                            band_cells(endB, g.below, g.above, n)}
                     : q;
        fin = i;
      }
    }
    plo = lo;
    phi = hi;
  };

  // Passes with no rows end at row 0 (m = 0: its row-0 values), or with an empty band
  // before row 1 when n + below < 1 (no score).
  const bool zero = fin == 0 && endB < 1;
  if (__any_sync(FULL, zero)) {
    const DRes q = result(0, plo, phi);
    if (zero) {
      r = m == 0 ? q
                 : DRes{NEG, b.clip_best, b.cut_best, NEG, 0, b.ci, b.cj, (uint32_t)n, 1u, 0u, 0ull};
      if (m == 0) r.text_read = (uint32_t)phi;
      fin = 0x7fffffff;
    }
  }
  for (int32_t i = 1; i <= endA2; ++i) row(i, std::false_type{}, i > endA);
  for (int32_t i = endA2 + 1; i <= endW; ++i) row(i, std::true_type{}, true);
  if (has && l == 0) a.out[jid] = r;
  if constexpr (TB) {
    __syncwarp();
    // Walk each segment's pass with the whole warp.
    for (int s = 0; s < 2; ++s) {
      const uint32_t js = __shfl_sync(FULL, jid, 16 * s);
      const bool hs = __shfl_sync(FULL, (int)has, 16 * s) != 0;
      if (!hs) continue;
      const DJob Js = a.jobs[js];
      const DParams Ps = a.params[js];
      const DRes Rs = a.out[js];
      walk_lean(a, js, tb_layout<C>(false, true, Js, Ps.flags, P), Js, Ps.flags, Rs, lane);
      __syncwarp();
    }
  }
  __syncwarp();
}

template <int C2, bool TB>
__global__ void __launch_bounds__(128, (C2 == 8 || C2 >= 10) ? 3 : 4)
    affine16h_kernel(sfk::AffLaunch a) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    uint32_t q = 0;
    if (lane == 0) q = atomicAdd(a.counter, 2u);
    q = __shfl_sync(FULL, q, 0);
    if (q >= a.njobs) break;
    const uint32_t mine = q + (uint32_t)(lane >> 4);
    const bool has = mine < a.njobs;
    pair16h<C2, TB>(a, a.order[has ? mine : q], has, lane);
  }
}

template <int C2>
struct MinBlocks16 {
  static constexpr int value = min_blocks16(C2);
};

// Two-warp passes: a 64-thread block per pass, the pass's two warps taking jobs together.
template <int C2, bool TB>
__global__ void __launch_bounds__(64, 2 * MinBlocks16<C2>::value) affine16w_kernel(sfk::AffLaunch a) {
  __shared__ Team16 X;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (;;) {
    if (threadIdx.x == 0) X.job = atomicAdd(a.counter, 1u);
    __syncthreads();
    const uint32_t q = X.job;
    if (q >= a.njobs) break;
    pair16w<C2, TB>(a, a.order[q], lane, w, X);
    __syncthreads();
  }
}

template <int C2, bool TB>
__global__ void __launch_bounds__(128, MinBlocks16<C2>::value) affine16_kernel(sfk::AffLaunch a) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    uint32_t q = 0;
    if (lane == 0) q = atomicAdd(a.counter, 1u);
    q = __shfl_sync(FULL, q, 0);
    if (q >= a.njobs) break;
    pair16<C2, TB>(a, a.order[q], lane, ChainRun{});
  }
}

// One chain of sorted texts (align.rs:2210-2315 `affine_dp_sorted`), its passes in order.
// A pass whose text agrees with the previous one over every base that pass read, with a
// band of the same shape, takes its result (align.rs:2262-2266); so does one that would
// resume within rows the previous pass never got past (2283-2285); the others resume from
// the snapshot of their shared rows.  Every pass reports the rows and cells of its whole
// pass; the host counts the rows the reference computes.
template <int C2>
__device__ __forceinline__ void chain16(const sfk::AffLaunch& a, const DChain& ch, int lane) {
  DRes prev{};
  uint32_t n_prev = 0;
  for (uint32_t u = 0; u < ch.count; ++u) {
    const uint32_t jid = ch.first + u;
    const DLink L = a.links[jid];
    const uint32_t n = a.jobs[jid].n;
    const bool clip = (a.params[jid].flags & F_CLIP) != 0;
    const uint32_t tr = prev.text_read;
    const bool same = u > 0 && clip && L.same_shape && tr < n_prev && tr < n && tr <= L.lcp;
    if (same || (u > 0 && L.resume > 0 && prev.last_row <= L.resume)) {
      if (lane == 0) a.out[jid] = prev;
    } else {
      ChainRun cr;
      cr.resume = u > 0 ? (int32_t)L.resume : 0;
      cr.slot = L.slot;
      cr.base = ch.want;
      cr.want = ch.want + (cr.resume > 0 ? L.slot + 1 : 0);
      cr.want_end = ch.want + ch.n_want;
      cr.slot0 = ch.snap_word;
      prev = pair16<C2, false, true>(a, jid, lane, cr);
    }
    n_prev = n;
  }
}

template <int C2>
__global__ void __launch_bounds__(128, MinBlocks16<C2>::value)
    affine16_chain_kernel(sfk::AffLaunch a) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    uint32_t q = 0;
    if (lane == 0) q = atomicAdd(a.counter, 1u);
    q = __shfl_sync(FULL, q, 0);
    if (q >= a.njobs) break;
    chain16<C2>(a, a.chains[a.order[q]], lane);
  }
}

}  // namespace

namespace sfk {

template <int C2>
cudaError_t launch_affine16h_c(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  if (tb)
    affine16h_kernel<C2, true><<<grid, block, 0, s>>>(a);
  else
    affine16h_kernel<C2, false><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

template <int C2>
cudaError_t launch_affine16w_c(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  if (tb)
    affine16w_kernel<C2, true><<<grid, block, 0, s>>>(a);
  else
    affine16w_kernel<C2, false><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

template <int C2>
cudaError_t launch_affine16_chain_c(const AffLaunch& a, int grid, int block, cudaStream_t s) {
  affine16_chain_kernel<C2><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

template <int C2>
cudaError_t launch_affine16_c(bool tb, const AffLaunch& a, int grid, int block, cudaStream_t s) {
  if (tb)
    affine16_kernel<C2, true><<<grid, block, 0, s>>>(a);
  else
    affine16_kernel<C2, false><<<grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace sfk
