// Internal device-side definitions shared by the kernels and the host engine.
//
// Sequence layout in HBM: 2-bit codes, 16 bases per 32-bit word, base x at bits
// 2*(x % 16) of word x / 16 -- the same bit order as spearfish's packed transcript store
// (crates/index/src/lib.rs:253-280, 32 bases per u64, read as little-endian words).  Each
// sequence starts on a word boundary and carries ONE leading pad base, so that DP row i
// (pattern base i - 1) and DP column j (text base j - 1) read packed position i / j
// directly, as the reference's rows and columns are numbered (align.rs:2557, 1027-1072).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sf {

constexpr int32_t NEG = INT32_MIN / 4;      // align.rs:693
constexpr int32_t NEG_INF = INT32_MIN / 2;  // "no predecessor" inside a lane's gap chain
constexpr uint32_t FULL = 0xffffffffu;

// Job flag bits (DJob::flags).
enum : uint32_t {
  F_MODE = 3u,        // sf_mode
  F_CLIP = 1u << 2,   // clip = Some((xdrop, cell))
  F_CELL = 1u << 3,   //   ... with the best cell tracked
  F_FULL = 1u << 4,   // unbanded rows (Infix or band = usize::MAX)
  F_TB = 1u << 5,     // write traceback nibbles
  F_CUT = 1u << 6,    // track the cut column
  F_LOCAL = 1u << 7,  // local band (floor 0, diagonal range, end bonuses)
  F_ROWMAX = 1u << 8  // per-row maximum needed (clip, cut or local)
};

// One affine / local pass.  64 bytes.
struct DJob {
  uint64_t p_word;   // packed pattern (word offset in the pool)
  uint64_t t_word;   // packed text
  uint64_t p_byte;   // local band: the read's byte codes (unmasked) in the byte pool
  int64_t below;     // banded rows: below / above (align.rs:2458-2461); local: dlo / dhi
  int64_t above;
  uint64_t cut;      // cut column (UINT64_MAX: none)
  uint64_t tb_word;  // traceback nibbles: word offset in the traceback arena
  uint32_t m, n;
};

struct DParams {
  uint32_t flags;
  int32_t xdrop;
  int32_t bonus0, bonus1;  // local: start / end bonus
  int32_t mat, mis, open, ext;
};

// What one pass found: align.rs:2111-2129 `Dp`, plus its DP_WORK cells.  48 bytes.
struct DRes {
  int32_t score, clip_best, cut_best, cut_score;
  uint32_t score_col, clip_i, clip_j, text_read, last_row, rows;
  uint64_t cells;
};

// One Myers job: align.rs:88-168 `distance`.
struct MJob {
  uint64_t p_word, t_word;
  uint32_t m, n;
  uint32_t mode, k;
};

// Traceback walk: which end cell, and where the CIGAR goes.
struct TJob {
  uint64_t ops_off;   // first op slot
  uint32_t ops_cap;
  uint32_t kind;      // 0: affine end (m, score_col); 1: extend window end
  int32_t end_bonus;
  uint32_t pad;
};

struct TRes {
  int32_t score, status;
  uint32_t end_i, end_j, text_start, n_ops;
};

// Sorted texts against one pattern (align.rs:2210-2315 `affine_dp_sorted`): a chain of
// consecutive jobs that one warp runs in order, each resuming from a row snapshot of an
// earlier one where the texts share the bases those rows read.  A chain starts at a pass
// that resumes nothing.
struct DChain {
  uint32_t first, count;   // jobs [first, first + count)
  uint32_t want, n_want;   // snapshot rows: want list [want, want + n_want), ascending
  uint64_t snap_word;      // the chain's n_want snapshot slots in the snapshot arena
};

// Per chained job: the row it resumes after (0: none) and that row's slot, the common
// prefix with the previous text and whether both bands have the same shape
// (align.rs:2229-2243).
struct DLink {
  uint32_t resume, slot, lcp, same_shape;
};

// 4-warp blocks of the 16-bit register kernel resident per SM (its launch bounds), by words
// per lane: the most that compile without spills (C = 24, 28: 4 blocks in at most 128
// registers; C = 40: 3 in 160).  Measured on config 3 with the autotuner on: 91.0 -> 87.9 ms
// a step together with the rebalanced decision compares; one more block each spilled and
// ran slower.
__host__ __device__ constexpr int min_blocks16(int c2) {
  return c2 <= 8 ? 6 : (c2 <= 14 ? 4 : (c2 <= 20 ? 3 : 2));
}

// A snapshot slot of the 16-bit kernel with C2 words per lane: H words, F words (word k of
// lane l at k * 32 + l), then the offset and the clip state (align.rs:2130-2148 `Snap`).
__host__ __device__ constexpr uint64_t snap_slot_words(int c2) { return (uint64_t)64 * c2 + 32; }

// Traceback words per lane and row: two bit-plane words per group of 16 cells, stored as one
// 8-byte pair (A, B) per lane and group, lane-fastest: pair g*32 + lane of the row.
__host__ __device__ inline uint32_t tb_words_per_lane(int c) { return (uint32_t)(2 * ((c + 15) / 16)); }

// The widest row of a pass: banded rows are at most below + above + 1 cells
// (align.rs:2458-2468), local rows at most dhi - dlo + 1 (align.rs:800-805), and no row has
// more than the n + 1 columns of the text.
__host__ __device__ inline int64_t band_wmax(const DJob& J, uint32_t flags) {
  const int64_t n = J.n;
  int64_t w;
  if (flags & F_LOCAL)
    w = J.above - J.below + 1;
  else if (flags & F_FULL)
    w = n + 1;
  else
    w = J.below + J.above + 1;
  return w < 0 ? 0 : (w > n + 1 ? n + 1 : w);
}

// Traceback words of one row: `chunks` chunks of 32 lanes x tb_words_per_lane(C) words.
__host__ __device__ inline uint64_t tb_row_words(int c, int64_t chunks) {
  return (uint64_t)chunks * 32u * tb_words_per_lane(c);
}

// Chunks of 32*C offsets a wide row needs: its cells plus the NEG sentinel after them.
__host__ __device__ inline int64_t wide_chunks(int c, int64_t w) {
  return (w + 1 + 32 * c - 1) / (32 * c);
}

// DP_WORK cells of rows 1 .. R of a banded pass (align.rs:2573-2578): the sum of
// hi_i - lo_i + 1 with lo_i = max(0, i - below), hi_i = min(i + above, n), rows whose band is
// not empty.
__host__ __device__ inline uint64_t band_cells(int64_t R, int64_t below, int64_t above,
                                               int64_t n) {
  if (R <= 0) return 0;
  const int64_t t = n - above;  // rows with i + above <= n
  int64_t s1;                   // sum of hi_i
  if (t >= R)
    s1 = R * (R + 1) / 2 + R * above;
  else if (t < 1)
    s1 = R * n;
  else
    s1 = t * (t + 1) / 2 + t * above + (R - t) * n;
  const int64_t u = R - below;  // rows with lo_i > 0
  const int64_t s2 = u > 0 ? u * (u + 1) / 2 : 0;
  return (uint64_t)(s1 - s2 + R);
}

__device__ __forceinline__ uint32_t base_at(const uint32_t* __restrict__ pool, uint64_t word,
                                            uint64_t pos) {
  return (__ldg(pool + word + (pos >> 4)) >> (2 * (pos & 15))) & 3u;
}

// max(a + b, c) and 3-way max via the sm_90+ DPX integer instructions.
__device__ __forceinline__ int32_t addmax(int32_t a, int32_t b, int32_t c) {
  return __viaddmax_s32(a, b, c);
}
__device__ __forceinline__ int32_t max3(int32_t a, int32_t b, int32_t c) {
  return __vimax3_s32(a, b, c);
}
__device__ __forceinline__ int32_t sat_add(int32_t a, int32_t b) {
  long long s = (long long)a + b;
  return s > INT32_MAX ? INT32_MAX : s < INT32_MIN ? INT32_MIN : (int32_t)s;
}
__device__ __forceinline__ int32_t sat_sub(int32_t a, int32_t b) {
  long long s = (long long)a - b;
  return s > INT32_MAX ? INT32_MAX : s < INT32_MIN ? INT32_MIN : (int32_t)s;
}

}  // namespace sf

// Launch entry points implemented by the kernel translation units.
namespace sfk {

struct AffLaunch {
  const sf::DJob* jobs;
  const sf::DParams* params;  // per job
  const uint32_t* order;      // job indices of this bucket, longest first
  uint32_t njobs;
  uint32_t* counter;          // work-queue head
  const uint32_t* pool;
  const uint8_t* bytes;       // byte pool (local band reads)
  sf::DRes* out;
  uint32_t* tb;               // traceback arena
  int32_t* scratch;           // WIDE rows: per warp 4 * scratch_cells int32
  uint64_t scratch_cells;
  const sf::TJob* tjobs;      // traceback: end cell kind and CIGAR slot per job
  uint32_t* ops;              // CIGAR slots
  sf::TRes* tres;             // walk results
  // Chain buckets (sorted texts): `order` holds chain indices.
  const sf::DChain* chains;
  const sf::DLink* links;     // per job
  const uint32_t* want;       // snapshot rows of every chain
  uint32_t* snap;             // snapshot arena
};

// C: cells per lane (register rows); wide: rows in global scratch, chunked.
cudaError_t launch_affine(int c, bool wide, bool tb, bool local, const AffLaunch& a, int grid,
                          int block, cudaStream_t s);
// The C values the register kernel is built for (ascending), and the wide chunk C.
extern const int kAffineC[];
extern const int kAffineNC;
constexpr int kWideC = 16;
// Packed 16-bit register kernel (two cells per register): C cells per lane, even.
cudaError_t launch_affine16(int c, bool tb, const AffLaunch& a, int grid, int block,
                            cudaStream_t s);
extern const int kAffine16C[];
extern const int kAffine16NC;
// The same rows with 16 lanes to a pass, two passes per warp.
cudaError_t launch_affine16h(int c, bool tb, const AffLaunch& a, int grid, int block,
                             cudaStream_t s);
extern const int kAffine16HC[];
extern const int kAffine16HNC;
// The same rows with 64 lanes to a pass: two warps of a 64-thread block (wide bands).
cudaError_t launch_affine16w(int c, bool tb, const AffLaunch& a, int grid, int block,
                             cudaStream_t s);
extern const int kAffine16WC[];
extern const int kAffine16WNC;
// Chains of sorted texts on the 16-bit register kernel (C from kAffine16C, no traceback).
cudaError_t launch_affine16_chain(int c, const AffLaunch& a, int grid, int block,
                                  cudaStream_t s);


struct MyersLaunch {
  const sf::MJob* jobs;
  const uint32_t* order;
  uint32_t njobs;
  uint32_t* counter;
  const uint32_t* pool;
  uint32_t* out;
  int lanes;  // lanes per pair (power of two <= 32)
  int kcut;   // some pair is Global or Prefix with k < m + n: stop pairs early (see kernel)
};
cudaError_t launch_myers(int blocks_per_lane, const MyersLaunch& a, int grid, int block,
                         cudaStream_t s);
extern const int kMyersB[];
extern const int kMyersNB;

// Sequences of a batch into its packed pool: from the byte pool, or (byte_off with bit 63
// set) sliced from the transcript store's packed words at that base position; bit 62 reads
// the sequence backwards.
struct PackLaunch {
  const uint8_t* bytes;
  const uint64_t* byte_off;  // per sequence
  const uint32_t* len;
  const uint64_t* word_off;
  uint32_t nseq;
  uint32_t* pool;
  const uint32_t* store;     // transcript store words (may be null)
};
// Byte codes -> store words: base p at position p + 16 (one leading word of padding).
cudaError_t launch_store_pack(const uint8_t* codes, uint64_t bases, uint32_t* words,
                              cudaStream_t s);
cudaError_t launch_pack(const PackLaunch& a, cudaStream_t s);

// Exclusive scan of per-job op counts (single block) and the gather that compacts ops.
cudaError_t launch_compact(const sf::TRes* tres, const sf::TJob* tjobs, const uint32_t* list,
                           uint32_t nlist, uint64_t* offs, const uint32_t* ops_in,
                           uint32_t* ops_out, uint64_t* total, cudaStream_t s);

}  // namespace sfk

namespace sfk {
// INT32 throughput probe: the DP's instruction mix (add-then-max on independent chains).
// Runs grid = sms * 8 blocks of 256 threads; returns the elapsed ms and the ops counted.
cudaError_t run_int_peak(int sms, int32_t* out, float* ms, uint64_t* ops);
}  // namespace sfk

// Records `msg` as the calling thread's sf_last_error() and returns `code`.
int sf_internal_set_error(int code, const char* msg);
