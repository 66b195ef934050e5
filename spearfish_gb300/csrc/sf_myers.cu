// Myers' bit-parallel edit distance (align.rs:47-168), one pair per P-lane segment of a warp.
//
// The pattern's 64-row blocks are spread over the segment's lanes, B consecutive blocks per
// lane.  Within one text column the blocks form a chain (block b needs the horizontal delta
// leaving block b - 1), across columns each block depends only on itself, so the segment runs
// a diagonal pipeline: at step t lane l processes column t - l, taking the delta (and the
// column's text base) that lane l - 1 produced at step t - 1 through one __shfl_up per step.
//
// Every block of every column is computed (no Ukkonen band): the reference's cutoff is
// exact whenever the distance is <= k and reports None otherwise (align.rs:87-168, pinned by
// its tests `random_vs_naive` / `related_vs_naive`), so comparing the full-column distance
// with k gives the same Option<u32>.  The band's skipped blocks would save no time here: the
// lanes holding them still step every column their upper neighbours step.
//
// What does save time is the end of a capped Global or Prefix pair (KC): once every cell of
// a column exceeds k -- row 0 holds the column index there, and each block's bottom row is
// at least k + 64, so its 64 rows exceed k -- every later cell does too (every path to a
// later column crosses this one), and the pair's answer is fixed: None (Global) or the best
// so far (Prefix).  Each lane tracks its blocks' bottom-row scores; the verdict for a column
// travels down the segment with the column's pipeline payload, and the warp stops when every
// segment has its verdict or has run out of text.  Infix pairs never stop (row 0 is 0).
#include <type_traits>
#include <utility>

#include "sf_internal.cuh"

namespace {

using sf::FULL;

__device__ __forceinline__ uint32_t match16(uint32_t w, uint32_t c) {
  // Bit k of the result: base k of the 16-base word w equals c.
  uint32_t x = w ^ (c * 0x55555555u);
  uint32_t y = ~(x | (x >> 1)) & 0x55555555u;
  y = (y | (y >> 1)) & 0x33333333u;
  y = (y | (y >> 2)) & 0x0F0F0F0Fu;
  y = (y | (y >> 4)) & 0x00FF00FFu;
  y = (y | (y >> 8)) & 0x0000FFFFu;
  return y;
}

// Calls f(std::integral_constant<int, k>{}) for k = 0 .. 15.
template <class F, int... K>
__device__ __forceinline__ void sf_unroll16_impl(F&& f, std::integer_sequence<int, K...>) {
  (f(std::integral_constant<int, K>{}), ...);
}
template <class F>
__device__ __forceinline__ void sf_unroll16(F&& f) {
  sf_unroll16_impl(f, std::make_integer_sequence<int, 16>{});
}

// align.rs:50-66 `block`.  The horizontal delta entering and leaving the block travels as
// two bits (pos: +1, neg: -1); the delta leaving is read at the block's last row `ob`
// (63, or the pattern's last row in its last block), as bit 0 of
// funnelshift_rc(lo, hi, ob) >> sub with sub = max(ob - 32, 0).
__device__ __forceinline__ void myers_step(uint64_t& pv, uint64_t& mv, uint64_t eq,
                                           uint32_t& pos, uint32_t& neg, uint32_t ob,
                                           uint32_t sub) {
  const uint64_t p = pv, m = mv;
  const uint64_t xv = eq | m;
  eq |= neg;
  const uint64_t xh = (((eq & p) + p) ^ p) | eq;
  uint64_t ph = m | ~(xh | p);
  uint64_t mh = p & xh;
  const uint32_t po =
      (__funnelshift_rc((uint32_t)ph, (uint32_t)(ph >> 32), ob) >> sub) & 1u;
  const uint32_t no =
      (__funnelshift_rc((uint32_t)mh, (uint32_t)(mh >> 32), ob) >> sub) & 1u;
  ph = (ph << 1) | pos;
  mh = (mh << 1) | neg;
  pv = mh | ~(xv | ph);
  mv = ph & xv;
  pos = po;
  neg = no;
}

template <int B, bool KC>
__global__ void __launch_bounds__(B <= 4 ? 128 : (B <= 8 ? 64 : 32))
    myers_kernel(sfk::MyersLaunch a) {
  constexpr bool SMEM = B > 4;
  extern __shared__ uint64_t smem[];
  const int lane = threadIdx.x & 31;
  const int P = a.lanes;
  const int seg = lane / P, l = lane % P, nseg = 32 / P;
  uint64_t* speq = smem + (size_t)(threadIdx.x >> 5) * 32 * B * 4;

  for (;;) {
    uint32_t q0 = 0;
    if (lane == 0) q0 = atomicAdd(a.counter, (uint32_t)nseg);
    q0 = __shfl_sync(FULL, q0, 0);
    if (q0 >= a.njobs) break;
    const uint32_t qi = q0 + seg;
    const bool has = qi < a.njobs;
    sf::MJob J{};
    uint32_t jid = 0;
    if (has) {
      jid = a.order[qi];
      J = a.jobs[jid];
    }
    const uint32_t m = J.m, n = J.n;
    const uint32_t blocks = (m + 63) / 64;
    const uint32_t last_block = blocks ? blocks - 1 : 0;
    const uint32_t last_bit = m ? (m - 1) % 64 : 0;

    // Match masks of this lane's blocks (align.rs:75-84): in shared memory per code for wide
    // lanes; in registers as the pattern's two bit planes otherwise, eq(c) = bits whose code
    // equals c.  Bits past the pattern's last row (and blocks past it) hold codes too: the
    // row recurrences only move information to higher rows, so they never reach the rows the
    // distance is read at.
    uint64_t pl0[SMEM ? 1 : B], pl1[SMEM ? 1 : B];
    uint64_t pv[B], mv[B];
    uint32_t ob[B], osub[B];
    // KC: each block's bottom-row score in this lane's current column (D[i][0] = i), and
    // the threshold a block must reach for all its 64 rows to exceed k.
    int32_t sb[KC ? B : 1];
    const int64_t kk = (int64_t)min((uint64_t)J.k, (uint64_t)m + (uint64_t)n);
    const int64_t thr = kk + 64;
#pragma unroll
    for (int bb = 0; bb < B; ++bb) {
      const uint32_t b = (uint32_t)l * B + bb;
      uint64_t q[4] = {0, 0, 0, 0}, b0 = 0, b1 = 0;
      if (has && b < blocks) {
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const uint64_t wi = J.p_word + (uint64_t)b * 4 + h;
          const uint32_t w = __funnelshift_r(__ldg(a.pool + wi), __ldg(a.pool + wi + 1), 2);
          if constexpr (SMEM) {
#pragma unroll
            for (int c = 0; c < 4; ++c) q[c] |= (uint64_t)match16(w, (uint32_t)c) << (16 * h);
          } else {
            // Gather the 16 codes' low and high bits.
            uint32_t lo = w & 0x55555555u, hi = (w >> 1) & 0x55555555u;
            lo = (lo | (lo >> 1)) & 0x33333333u;
            lo = (lo | (lo >> 2)) & 0x0F0F0F0Fu;
            lo = (lo | (lo >> 4)) & 0x00FF00FFu;
            lo = (lo | (lo >> 8)) & 0x0000FFFFu;
            hi = (hi | (hi >> 1)) & 0x33333333u;
            hi = (hi | (hi >> 2)) & 0x0F0F0F0Fu;
            hi = (hi | (hi >> 4)) & 0x00FF00FFu;
            hi = (hi | (hi >> 8)) & 0x0000FFFFu;
            b0 |= (uint64_t)lo << (16 * h);
            b1 |= (uint64_t)hi << (16 * h);
          }
        }
      }
      if constexpr (SMEM) {
#pragma unroll
        for (int c = 0; c < 4; ++c) speq[((size_t)bb * 4 + c) * 32 + lane] = q[c];
      } else {
        pl0[bb] = b0;
        pl1[bb] = b1;
      }
      pv[bb] = ~0ull;
      mv[bb] = 0;
      if constexpr (KC) sb[bb] = has && b < blocks ? (int32_t)min((b + 1) * 64u, m) : INT32_MAX / 2;
      ob[bb] = b == last_block ? last_bit : 63u;
      osub[bb] = ob[bb] >= 32 ? ob[bb] - 32 : 0u;
    }
    if constexpr (SMEM) __syncwarp();

    const int top = J.mode == 0 ? 0 : 1;  // Infix: free text start
    const bool owner = has && m > 0 && (uint32_t)l == last_block / B;
    const int own_bb = (int)(last_block % B);
    int score = (int)m, best = (int)m;
    const int seg_steps = has && m > 0 ? (int)n + P - 1 : 0;
    const int steps = __reduce_max_sync(FULL, seg_steps);
    uint32_t payload = 0;  // (column past k << 4) | (text code << 2) | (pos << 1) | neg
    bool dead = false;     // KC, the segment's last lane: a column wholly past k went by
    uint32_t tw = 0;       // the text word holding base t + 1 (used by lane 0)
    const bool glob = J.mode == 2;
    // One step of the pipeline.  Lanes keep their state only while they are past the fill
    // (FILL: some lanes have not reached column 0 yet); past its text's end a lane computes
    // on state nothing reads any more, so the steady loop needs no masking and no branches.
    // K < 0: the step reads its text base itself; K = 0..15: the step is the K-th of a run of
    // 16 whose bases all sit in `tw`, loaded before the run.  Every lane keeps a running
    // score (only the owner's is used): the column's distance while the lane's column lies in
    // the text, and the least of them (Infix, Prefix; Global takes the last).
    const int jend = (int)n + l;  // steps t < jend have this lane's column j = t - l < n
    auto step = [&](int t, auto fill, auto kk) {
      constexpr bool FILL = decltype(fill)::value;
      constexpr int K = decltype(kk)::value;
      const int j = t - l;
      const bool live = FILL ? (j >= 0 && t < jend) : t < jend;
      const uint32_t in = __shfl_up_sync(FULL, payload, 1, P);
      uint32_t c0;
      if constexpr (K < 0) {
        // A new text word every 16 steps, read only while it lies inside this text (base
        // t + 1 of a text of n bases sits in word (t + 1) / 16 after the leading pad base).
        if ((((t + 1) & 15) == 0 || t == 0) && (uint32_t)(t + 1) <= n)
          tw = __ldg(a.pool + J.t_word + ((uint32_t)(t + 1) >> 4));
        c0 = (tw >> (2 * ((t + 1) & 15))) & 3u;
      } else {
        c0 = (tw >> (2 * K)) & 3u;
      }
      const uint32_t c = l == 0 ? c0 : ((in >> 2) & 3u);
      uint32_t pos = l == 0 ? (uint32_t)top : (in >> 1) & 1u;
      uint32_t neg = l == 0 ? 0u : in & 1u;
      // eq(c) from the bit planes: both code bits equal c's.
      [[maybe_unused]] const uint64_t m0 = (c & 1u) ? ~0ull : 0ull, m1 = (c & 2u) ? ~0ull : 0ull;
      int hlast = 0;
#pragma unroll
      for (int bb = 0; bb < B; ++bb) {
        uint64_t eq;
        if constexpr (SMEM)
          eq = speq[((size_t)bb * 4 + c) * 32 + lane];
        else
          eq = ~(pl0[bb] ^ m0) & ~(pl1[bb] ^ m1);
        if constexpr (FILL) {
          uint64_t p2 = pv[bb], m2 = mv[bb];
          myers_step(p2, m2, eq, pos, neg, ob[bb], osub[bb]);
          if (j >= 0) {
            pv[bb] = p2;
            mv[bb] = m2;
            if constexpr (KC) sb[bb] += (int32_t)pos - (int32_t)neg;
          }
        } else {
          myers_step(pv[bb], mv[bb], eq, pos, neg, ob[bb], osub[bb]);
          if constexpr (KC) sb[bb] += (int32_t)pos - (int32_t)neg;
        }
        hlast = bb == own_bb ? (int)pos - (int)neg : hlast;
      }
      score += live ? hlast : 0;
      best = min(best, score);
      uint32_t past = 0;
      if constexpr (KC) {
        // Column j wholly past k down to this lane's blocks: row 0 (lane 0: D[0][j + 1] =
        // j + 1) and every block above, as the lane before found; then this lane's blocks.
        bool ex = l == 0 ? (int64_t)t + 1 > kk : ((in >> 4) & 1u) != 0;
#pragma unroll
        for (int bb = 0; bb < B; ++bb) ex = ex && sb[bb] >= thr;
        ex = ex && live;
        if (ex && l == P - 1) dead = true;
        past = ex ? 16u : 0u;
      }
      payload = past | (c << 2) | (pos << 1) | neg;
    };
    // KC: every segment has its column past k, or has stepped through its text.
    auto all_done = [&](int t) -> bool {
      const uint32_t bal = __ballot_sync(FULL, dead);
      const bool sd = ((bal >> (seg * P + P - 1)) & 1u) != 0;
      return __all_sync(FULL, sd || t >= seg_steps);
    };
    bool stop = false;
    using kAny = std::integral_constant<int, -1>;
    const int fill = steps < P - 1 ? steps : P - 1;
    int t = 0;
    for (; t < fill; ++t) step(t, std::true_type{}, kAny{});
    // Steady steps: with register blocks, single ones up to a text-word boundary, then runs of
    // 16 with one load each (wider lanes keep the loop short: their step is long already).
    if constexpr (!SMEM) {
      for (; t < steps && ((t + 1) & 15) != 0; ++t) step(t, std::false_type{}, kAny{});
      for (; t + 16 <= steps; t += 16) {
        if constexpr (KC) {
          if (all_done(t)) {
            stop = true;
            break;
          }
        }
        if ((uint32_t)(t + 1) <= n) tw = __ldg(a.pool + J.t_word + ((uint32_t)(t + 1) >> 4));
        sf_unroll16([&](auto kt) { step(t + decltype(kt)::value, std::false_type{}, kt); });
      }
    }
    for (; t < steps && !stop; ++t) {
      if constexpr (KC) {
        if ((t & 15) == 0 && all_done(t)) break;
      }
      step(t, std::false_type{}, kAny{});
    }
    if (glob) best = score;
    if constexpr (KC) {
      // A segment whose column went past k: Global ends past k; Prefix keeps its best.
      const uint32_t bal = __ballot_sync(FULL, dead);
      if (((bal >> (seg * P + P - 1)) & 1u) && glob) best = INT32_MAX;
    }
    if (has) {
      if (m == 0) {
        if (l == 0) {
          const uint32_t d = J.mode == 2 ? n : 0;
          a.out[jid] = d <= J.k ? d : 0xffffffffu;
        }
      } else if (owner) {
        a.out[jid] = (uint32_t)best <= J.k ? (uint32_t)best : 0xffffffffu;
      }
    }
    __syncwarp();
  }
}

template <int B>
cudaError_t launch_b(const sfk::MyersLaunch& a, int grid, int block, cudaStream_t s) {
  const size_t sm = B > 4 ? (size_t)(block / 32) * 32 * B * 4 * sizeof(uint64_t) : 0;
  if (a.kcut)
    myers_kernel<B, true><<<grid, block, sm, s>>>(a);
  else
    myers_kernel<B, false><<<grid, block, sm, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

namespace sfk {

const int kMyersB[] = {1, 2, 3, 4, 6, 8, 12, 16};
const int kMyersNB = 8;

cudaError_t launch_myers(int b, const MyersLaunch& a, int grid, int block, cudaStream_t s) {
  switch (b) {
    case 1: return launch_b<1>(a, grid, block, s);
    case 2: return launch_b<2>(a, grid, block, s);
    case 3: return launch_b<3>(a, grid, block, s);
    case 4: return launch_b<4>(a, grid, block, s);
    case 6: return launch_b<6>(a, grid, block, s);
    case 8: return launch_b<8>(a, grid, block, s);
    case 12: return launch_b<12>(a, grid, block, s);
    case 16: return launch_b<16>(a, grid, block, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace sfk
