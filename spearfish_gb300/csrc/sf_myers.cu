// Myers' bit-parallel edit distance (align.rs:47-168), one pair per P-lane segment of a warp.
//
// The pattern's 64-row blocks are spread over the segment's lanes, B consecutive blocks per
// lane.  Within one text column the blocks form a chain (block b needs the horizontal delta
// leaving block b - 1), across columns each block depends only on itself, so the segment runs
// a diagonal pipeline: at step t lane l processes column t - l, taking the delta (and the
// column's text base) that lane l - 1 produced at step t - 1 through one __shfl_up per step.
//
// Every block of every column is computed (no Ukkonen cutoff): the reference's cutoff is
// exact whenever the distance is <= k and reports None otherwise (align.rs:87-168, pinned by
// its tests `random_vs_naive` / `related_vs_naive`), so comparing the full-column distance
// with k gives the same Option<u32>.
#include <type_traits>

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

// align.rs:50-66 `block`, with the output row given as a one-bit mask.
__device__ __forceinline__ int myers_step(uint64_t& pv, uint64_t& mv, uint64_t eq, int hin,
                                          uint64_t outbit) {
  const uint64_t neg = (uint64_t)(hin < 0), pos = (uint64_t)(hin > 0);
  const uint64_t p = pv, m = mv;
  const uint64_t xv = eq | m;
  eq |= neg;
  const uint64_t xh = (((eq & p) + p) ^ p) | eq;
  uint64_t ph = m | ~(xh | p);
  uint64_t mh = p & xh;
  const int hout = (int)((ph & outbit) != 0) - (int)((mh & outbit) != 0);
  ph = (ph << 1) | pos;
  mh = (mh << 1) | neg;
  pv = mh | ~(xv | ph);
  mv = ph & xv;
  return hout;
}

template <int B>
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

    // Match masks of this lane's blocks (align.rs:75-84).
    uint64_t peq[SMEM ? 1 : B][4];
    uint64_t pv[B], mv[B], outbit[B];
#pragma unroll
    for (int bb = 0; bb < B; ++bb) {
      const uint32_t b = (uint32_t)l * B + bb;
      uint64_t q[4] = {0, 0, 0, 0};
      if (has && b < blocks) {
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const uint64_t wi = J.p_word + (uint64_t)b * 4 + h;
          const uint32_t w = __funnelshift_r(__ldg(a.pool + wi), __ldg(a.pool + wi + 1), 2);
#pragma unroll
          for (int c = 0; c < 4; ++c) q[c] |= (uint64_t)match16(w, (uint32_t)c) << (16 * h);
        }
        if (b == last_block && last_bit < 63) {
          const uint64_t keep = (1ull << (last_bit + 1)) - 1;
#pragma unroll
          for (int c = 0; c < 4; ++c) q[c] &= keep;
        }
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        if constexpr (SMEM)
          speq[((size_t)bb * 4 + c) * 32 + lane] = q[c];
        else
          peq[bb][c] = q[c];
      }
      pv[bb] = ~0ull;
      mv[bb] = 0;
      outbit[bb] = 1ull << (b == last_block ? last_bit : 63);
    }
    if constexpr (SMEM) __syncwarp();

    const int top = J.mode == 0 ? 0 : 1;  // Infix: free text start
    const bool owner = has && m > 0 && (uint32_t)l == last_block / B;
    const int own_bb = (int)(last_block % B);
    int score = (int)m, best = (int)m;
    int steps = has && m > 0 ? (int)n + P - 1 : 0;
    steps = __reduce_max_sync(FULL, steps);
    uint32_t payload = 0;  // (text code << 2) | (h + 1)
    uint32_t tw = 0;       // the text word holding base t + 1 (used by lane 0)
    const bool glob = J.mode == 2;
    // One step of the pipeline.  Lanes keep their state only while they are past the fill
    // (FILL: some lanes have not reached column 0 yet); past its text's end a lane computes
    // on state nothing reads any more, so the steady loop needs no masking and no branches.
    auto step = [&](int t, auto fill) {
      constexpr bool FILL = decltype(fill)::value;
      const int j = t - l;
      const bool live = has && m > 0 && j >= 0 && j < (int)n;
      const uint32_t in = __shfl_up_sync(FULL, payload, 1, P);
      // A new text word every 16 steps, read only while it lies inside this text (base t + 1
      // of a text of n bases sits in word (t + 1) / 16 after the leading pad base).
      if ((((t + 1) & 15) == 0 || t == 0) && (uint32_t)(t + 1) <= n)
        tw = __ldg(a.pool + J.t_word + ((uint32_t)(t + 1) >> 4));
      const uint32_t c0 = (tw >> (2 * ((t + 1) & 15))) & 3u;
      const uint32_t c = l == 0 ? c0 : (in >> 2);
      int h = l == 0 ? top : (int)(in & 3) - 1;
      int hlast = 0;
#pragma unroll
      for (int bb = 0; bb < B; ++bb) {
        uint64_t eq;
        if constexpr (SMEM)
          eq = speq[((size_t)bb * 4 + c) * 32 + lane];
        else
          eq = c == 0 ? peq[bb][0] : c == 1 ? peq[bb][1] : c == 2 ? peq[bb][2] : peq[bb][3];
        if constexpr (FILL) {
          uint64_t p2 = pv[bb], m2 = mv[bb];
          h = myers_step(p2, m2, eq, h, outbit[bb]);
          if (j >= 0) {
            pv[bb] = p2;
            mv[bb] = m2;
          }
        } else {
          h = myers_step(pv[bb], mv[bb], eq, h, outbit[bb]);
        }
        hlast = bb == own_bb ? h : hlast;
      }
      const bool upd = owner && live;
      score = upd ? score + hlast : score;
      best = upd ? (glob ? (j + 1 == (int)n ? score : best) : min(best, score)) : best;
      payload = (c << 2) | (uint32_t)(h + 1);
    };
    const int fill = steps < P - 1 ? steps : P - 1;
    int t = 0;
    for (; t < fill; ++t) step(t, std::true_type{});
    for (; t < steps; ++t) step(t, std::false_type{});
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
  myers_kernel<B><<<grid, block, sm, s>>>(a);
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
