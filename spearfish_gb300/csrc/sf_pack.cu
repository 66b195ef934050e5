// Byte codes -> 2-bit packed sequences in HBM, and the compaction of CIGAR ops.
//
// Packing is HBM-bound byte work: one warp per sequence, each lane building whole 16-base
// words from 16 consecutive bytes (two aligned 16-byte loads inside the sequence, coalesced
// 512-byte spans per warp), written once.
#include "sf_internal.cuh"

namespace {

// Four byte codes (their low two bits) -> one byte, code b at bits 2b: the multiply moves byte
// b's bits 8b..8b+1 to 24 + 2b, and the other products land below bit 24 in fields that do not
// overlap, so nothing carries into the top byte.
__device__ __forceinline__ uint32_t pack4(uint32_t u) {
  return ((u & 0x03030303u) * 0x01041040u) >> 24;
}

// Word w of a sequence read forwards: bases 16w .. 16w + 15, base x at byte x - 1 (base 0, the
// pad, reads as 0).  Every word's first byte sits at the same offset in its 16-byte line, sh =
// 4Q + r8 / 8 (uniform for the sequence, so Q is a template argument).  Words whose two lines
// lie inside the sequence's bytes take two 16-byte loads and four funnel shifts; the first
// word and the words at the sequence's end take byte loads.  No load leaves the sequence.
template <int Q>
__device__ __forceinline__ void pack_forward(uint32_t* dst, const uint8_t* src, uint64_t len,
                                             uint64_t words, int lane, uint32_t r8) {
  const uint64_t s0 = (uint64_t)(uintptr_t)src;
  for (uint64_t w = lane; w < words; w += 32) {
    const uint64_t a0 = s0 + 16 * w - 1;
    const uint64_t al = a0 & ~uint64_t(15);
    uint32_t v = 0;
    if (w > 0 && al >= s0 && al + 32 <= s0 + len) {
      const uint4 c0 = __ldg(reinterpret_cast<const uint4*>(al));
      const uint4 c1 = __ldg(reinterpret_cast<const uint4*>(al + 16));
      const uint32_t x[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
      v = pack4(__funnelshift_r(x[Q], x[Q + 1], r8)) |
          pack4(__funnelshift_r(x[Q + 1], x[Q + 2], r8)) << 8 |
          pack4(__funnelshift_r(x[Q + 2], x[Q + 3], r8)) << 16 |
          pack4(__funnelshift_r(x[Q + 3], x[Q + 4], r8)) << 24;
    } else {
#pragma unroll
      for (int b = 0; b < 16; ++b) {
        const uint64_t pos = 16 * w + b;
        if (pos >= 1 && pos - 1 < len) v |= (uint32_t)(src[pos - 1] & 3) << (2 * b);
      }
    }
    dst[w] = v;
  }
}

__global__ void __launch_bounds__(256) pack_kernel(sfk::PackLaunch a) {
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t s = warp; s < a.nseq; s += nwarps) {
    const uint64_t off = a.byte_off[s];
    const uint64_t len = a.len[s];
    const uint64_t words = (len + 1 + 15) / 16;  // one leading pad base
    uint32_t* dst = a.pool + a.word_off[s];
    const bool rev = (off >> 62) & 1;  // read backwards (the mapper's leftward extensions)
    if (off >> 63) {
      const uint64_t pos = (off & ~(uint64_t(3) << 62)) - 1;
      if (!rev) {
        // A window of the transcript store: packed base x (x >= 1) is store position
        // pos + x - 1; the pad base takes the store base before the window (never matched).
        for (uint64_t w = lane; w < words; w += 32) {
          const uint64_t b0 = pos + 16 * w, wi = b0 >> 4;
          uint32_t v = __funnelshift_r(__ldg(a.store + wi), __ldg(a.store + wi + 1),
                                       2u * (uint32_t)(b0 & 15));
          const uint64_t valid = len + 1 - 16 * w;  // bases of this word inside the window
          if (valid < 16) v &= (1u << (2 * valid)) - 1u;
          dst[w] = v;
        }
      } else {
        // The window read backwards: packed base x (1 <= x <= len) is store position
        // pos + len - x + 1.
        for (uint64_t w = lane; w < words; w += 32) {
          uint32_t v = 0;
#pragma unroll
          for (int b = 0; b < 16; ++b) {
            const uint64_t x = 16 * w + b;
            if (x >= 1 && x <= len) {
              const uint64_t sp = pos + len - x + 1;
              v |= ((__ldg(a.store + (sp >> 4)) >> (2 * (sp & 15))) & 3u) << (2 * b);
            }
          }
          dst[w] = v;
        }
      }
      continue;
    }
    const uint8_t* src = a.bytes + (off & ~(uint64_t(3) << 62));
    if (!rev) {
      const uint32_t sh = (uint32_t)(((uint64_t)(uintptr_t)src + 15) & 15);  // (src - 1) mod 16
      const uint32_t r8 = 8 * (sh & 3);
      switch (sh >> 2) {
        case 0: pack_forward<0>(dst, src, len, words, lane, r8); break;
        case 1: pack_forward<1>(dst, src, len, words, lane, r8); break;
        case 2: pack_forward<2>(dst, src, len, words, lane, r8); break;
        default: pack_forward<3>(dst, src, len, words, lane, r8); break;
      }
      continue;
    }
    for (uint64_t w = lane; w < words; w += 32) {
      uint32_t v = 0;
#pragma unroll
      for (int b = 0; b < 16; ++b) {
        const uint64_t pos = 16 * w + b;
        if (pos >= 1 && pos - 1 < len) v |= (uint32_t)(src[len - pos] & 3) << (2 * b);
      }
      dst[w] = v;
    }
  }
}

// Exclusive scan of the walk's op counts over `nlist` jobs, in one block.
__global__ void __launch_bounds__(1024) scan_kernel(const sf::TRes* tres, const uint32_t* list,
                                                    uint32_t nlist, uint64_t* offs,
                                                    uint64_t* total) {
  __shared__ uint64_t warp_sums[32];
  __shared__ uint64_t carry;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (tid == 0) carry = 0;
  __syncthreads();
  for (uint32_t base = 0; base < nlist; base += 1024) {
    const uint32_t q = base + tid;
    uint64_t v = 0;
    if (q < nlist) {
      const sf::TRes r = tres[list[q]];
      v = r.status == 0 ? r.n_ops : 0;
    }
    uint64_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      uint64_t y = __shfl_up_sync(sf::FULL, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
      uint64_t s = warp_sums[lane];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        uint64_t y = __shfl_up_sync(sf::FULL, s, d);
        if (lane >= d) s += y;
      }
      warp_sums[lane] = s;
    }
    __syncthreads();
    const uint64_t before = carry + (wid > 0 ? warp_sums[wid - 1] : 0) + x - v;
    if (q < nlist) offs[q] = before;
    __syncthreads();
    if (tid == 1023) carry = before + v;
    __syncthreads();
  }
  if (tid == 0) *total = carry;
}

__global__ void __launch_bounds__(256) gather_kernel(const sf::TRes* tres, const sf::TJob* tjobs,
                                                     const uint32_t* list, uint32_t nlist,
                                                     const uint64_t* offs, const uint32_t* in,
                                                     uint32_t* out) {
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t q = warp; q < nlist; q += nwarps) {
    const uint32_t j = list[q];
    const sf::TRes r = tres[j];
    if (r.status != 0) continue;
    const uint32_t* src = in + tjobs[j].ops_off;
    uint32_t* dst = out + offs[q];
    // The walk wrote the ops end first.
    for (uint32_t x = lane; x < r.n_ops; x += 32) dst[x] = src[r.n_ops - 1 - x];
  }
}

// Store words from byte codes: word w holds positions 16w .. 16w + 15, base p at p + 16.
__global__ void __launch_bounds__(256) store_pack_kernel(const uint8_t* codes, uint64_t bases,
                                                         uint64_t nwords, uint32_t* words) {
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwords;
       w += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t v = 0;
    if (w > 0) {
#pragma unroll
      for (int b = 0; b < 16; ++b) {
        const uint64_t p = 16 * (w - 1) + b;
        if (p < bases) v |= (uint32_t)(codes[p] & 3) << (2 * b);
      }
    }
    words[w] = v;
  }
}

}  // namespace

namespace sfk {

cudaError_t launch_store_pack(const uint8_t* codes, uint64_t bases, uint32_t* words,
                              cudaStream_t s) {
  const uint64_t nwords = (bases + 15) / 16 + 1;
  const uint64_t blocks = (nwords + 255) / 256;
  store_pack_kernel<<<(unsigned)(blocks < 152u * 32u ? blocks : 152u * 32u), 256, 0, s>>>(
      codes, bases, nwords, words);
  return cudaGetLastError();
}

cudaError_t launch_pack(const PackLaunch& a, cudaStream_t s) {
  if (a.nseq == 0) return cudaSuccess;
  const uint32_t warps = a.nseq < 152u * 64u ? a.nseq : 152u * 64u;
  pack_kernel<<<(warps + 7) / 8, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_compact(const sf::TRes* tres, const sf::TJob* tjobs, const uint32_t* list,
                           uint32_t nlist, uint64_t* offs, const uint32_t* ops_in,
                           uint32_t* ops_out, uint64_t* total, cudaStream_t s) {
  scan_kernel<<<1, 1024, 0, s>>>(tres, list, nlist, offs, total);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || nlist == 0) return e;
  const uint32_t warps = nlist < 152u * 64u ? nlist : 152u * 64u;
  gather_kernel<<<(warps + 7) / 8, 256, 0, s>>>(tres, tjobs, list, nlist, offs, ops_in, ops_out);
  return cudaGetLastError();
}

}  // namespace sfk
