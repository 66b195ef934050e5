// Traceback walk (no reference counterpart: spearfish computes no alignment path) and the
// dispatcher over the banded affine kernels.
//
// One thread per pass walks from the pass's end cell back to row 0 / column 0 through the
// nibbles the affine kernel wrote, with the tie order the nibbles encode (H from H' before
// E, diagonal before vertical, opening before extending), and writes the CIGAR run-length
// encoded, BAM-style (len << 4 | op).  Every nibble address is range-checked against the
// row's band before it is read; a path that leaves the band reports "no path".
#include "sf_internal.cuh"

namespace {

using namespace sf;

__device__ __forceinline__ void band_range(const DJob& J, uint32_t flags, int64_t i,
                                           int64_t& lo, int64_t& hi) {
  const int64_t n = J.n;
  if (flags & F_LOCAL) {
    int64_t l = i + J.below, h = i + J.above + 1;
    l = l < 0 ? 0 : (l > n + 1 ? n + 1 : l);
    h = h < 0 ? 0 : (h > n + 1 ? n + 1 : h);
    if (h < l) h = l;
    lo = l;
    hi = h - 1;
  } else if (flags & F_FULL) {
    lo = 0;
    hi = n;
  } else {
    lo = i > J.below ? i - J.below : 0;
    hi = i + J.above < n ? i + J.above : n;
  }
}

struct OpWriter {
  uint32_t* out;
  uint32_t cap, n = 0;
  int status = 0;
  __device__ void push(uint32_t op, uint64_t len) {
    if (len == 0 || status) return;
    if (n > 0 && (out[n - 1] & 15u) == op) {
      out[n - 1] += (uint32_t)(len << 4);
      return;
    }
    if (n == cap) {
      status = -1;
      return;
    }
    out[n++] = (uint32_t)(len << 4) | op;
  }
};

__global__ void __launch_bounds__(128) walk_kernel(sfk::WalkLaunch a) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < a.nlist; q += stride) {
    const uint32_t jid = a.list[q];
    const DJob J = a.jobs[jid];
    const DParams P = a.params[jid];
    const DRes R = a.res[jid];
    const TJob T = a.tjobs[jid];
    const uint32_t cls = a.cls[jid];
    const bool wide = cls & 0x80u;
    const int C = (int)(cls & 0x7fu);
    const int CW = (C + 7) / 8;
    const uint64_t stride_w =
        wide ? tb_row_words(C, wide_chunks(C, band_wmax(J, P.flags))) : tb_row_words(C, 1);
    const int mode = (int)(P.flags & F_MODE);
    const int64_t m = J.m;
    // End cell (align.rs:2643-2650 score_col; 975-981 the window's choice).
    int32_t score;
    int64_t ei, ej, tail = 0;
    bool ok = true;
    if (T.kind == 0) {
      score = R.score;
      ei = m;
      ej = R.score_col;
      ok = R.score > NEG / 2;
    } else {
      const int32_t whole = sat_add(R.score, T.end_bonus);
      if (R.clip_best >= whole) {
        score = R.clip_best;
        ei = R.clip_i;
        ej = R.clip_j;
        tail = m - ei;
      } else {
        score = whole;
        ei = m;
        ej = R.score_col;
        ok = R.score > NEG / 2;
      }
    }
    OpWriter w{a.ops + T.ops_off, T.ops_cap};
    int64_t text_start = 0;
    if (!ok) {
      w.status = 1;
    } else {
      w.push(4, (uint64_t)tail);
      int64_t i = ei, j = ej;
      int state = 0;  // 0 H, 1 E, 2 F
      const int64_t guard = 2 * (m + (int64_t)J.n) + 8;
      for (int64_t it = 0;; ++it) {
        if (it > guard) {
          w.status = 1;
          break;
        }
        if (state == 0 && i == 0) {
          if (mode == 0) {
            text_start = j;
          } else {
            w.push(2, (uint64_t)j);
          }
          break;
        }
        if (state == 0 && j == 0) {
          w.push(1, (uint64_t)i);
          break;
        }
        if (i <= 0 || j <= 0) {
          w.status = 1;
          break;
        }
        int64_t lo, hi;
        band_range(J, P.flags, i, lo, hi);
        const int64_t K = j - lo;
        if (K < 0 || j > hi) {
          w.status = 1;
          break;
        }
        uint64_t word;
        int c;
        if (wide) {
          const int64_t qc = K / (32 * C), r = K % (32 * C);
          c = (int)(r % C);
          word = J.tb_word + (uint64_t)(i - 1) * stride_w + (uint64_t)qc * CW * 32 +
                 (uint64_t)(c >> 3) * 32 + (uint64_t)(r / C);
        } else {
          c = (int)(K % C);
          word = J.tb_word + (uint64_t)(i - 1) * stride_w + (uint64_t)(c >> 3) * 32 +
                 (uint64_t)(K / C);
        }
        const uint32_t nib = (__ldg(a.tb + word) >> (4 * (c & 7))) & 15u;
        if (state == 0) {
          const uint32_t hs = nib & 3u;
          if (hs == 2) {
            state = 1;
          } else if (hs == 0) {
            w.push(0, 1);
            --i;
            --j;
          } else {
            state = 2;
          }
        } else if (state == 1) {
          w.push(2, 1);
          state = (nib & 4u) ? 0 : 1;
          --j;
        } else {
          w.push(1, 1);
          state = (nib & 8u) ? 0 : 2;
          --i;
        }
        if (w.status) break;
      }
    }
    if (w.status == 0) {
      for (uint32_t x = 0, y = w.n ? w.n - 1 : 0; x < y; ++x, --y) {
        const uint32_t t = w.out[x];
        w.out[x] = w.out[y];
        w.out[y] = t;
      }
    }
    TRes tr;
    tr.score = score;
    tr.status = w.status;
    tr.end_i = (uint32_t)ei;
    tr.end_j = (uint32_t)ej;
    tr.text_start = (uint32_t)text_start;
    tr.n_ops = w.status == 0 ? w.n : 0;
    a.tres[jid] = tr;
  }
}

}  // namespace

namespace sfk {

cudaError_t launch_affine_regs_4(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_8(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_12(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_16(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_24(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_32(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_regs_48(bool, const AffLaunch&, int, int, cudaStream_t);
cudaError_t launch_affine_wide(bool, const AffLaunch&, int, int, cudaStream_t);

const int kAffineC[] = {4, 8, 12, 16, 24, 32, 48};
const int kAffineNC = 7;

cudaError_t launch_affine(int c, bool wide, bool tb, const AffLaunch& a, int grid, int block,
                          cudaStream_t s) {
  if (wide) return launch_affine_wide(tb, a, grid, block, s);
  switch (c) {
    case 4: return launch_affine_regs_4(tb, a, grid, block, s);
    case 8: return launch_affine_regs_8(tb, a, grid, block, s);
    case 12: return launch_affine_regs_12(tb, a, grid, block, s);
    case 16: return launch_affine_regs_16(tb, a, grid, block, s);
    case 24: return launch_affine_regs_24(tb, a, grid, block, s);
    case 32: return launch_affine_regs_32(tb, a, grid, block, s);
    case 48: return launch_affine_regs_48(tb, a, grid, block, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_walk(const WalkLaunch& a, cudaStream_t s) {
  if (a.nlist == 0) return cudaSuccess;
  const uint32_t threads = a.nlist;
  const uint32_t blocks = (threads + 127) / 128;
  walk_kernel<<<blocks, 128, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace sfk
