// Internal engine of libsf_align: buffers, passes, plans and contexts shared by the plans
// (sf_plan.cu), the C ABI (sf_host.cu) and the serving loop (sf_server.cu).  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <tuple>
#include <memory>
#include <string>
#include <vector>

#include "../../include/sf_align.h"
#include "sf_internal.cuh"

namespace sfe {

using namespace sf;

// Records the calling thread's sf_last_error() message and returns `code`.
int fail(int code, const std::string& msg);
// The calling thread's last message.
const std::string& last_error();

#define CK(call)                                                                    \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return fail(e_ == cudaErrorMemoryAllocation ? SF_ERR_NOMEM : SF_ERR_CUDA,     \
                  std::string(#call) + ": " + cudaGetErrorString(e_));              \
  } while (0)

inline uint64_t usat_add(uint64_t a, uint64_t b) { return a > UINT64_MAX - b ? UINT64_MAX : a + b; }
inline uint64_t usat_sub(uint64_t a, uint64_t b) { return a > b ? a - b : 0; }
inline int32_t sat_add32(int32_t a, int32_t b) {
  int64_t s = (int64_t)a + b;
  return s > INT32_MAX ? INT32_MAX : s < INT32_MIN ? INT32_MIN : (int32_t)s;
}
constexpr int64_t kGeoCap = int64_t(1) << 40;  // band geometry beyond any text length

// ---- device and pinned buffers ---------------------------------------------------------

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  int ensure(size_t n) {
    if (n <= cap) return SF_OK;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = n + n / 4 + 256;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      p = nullptr;
      (void)cudaGetLastError();
      return fail(SF_ERR_NOMEM, "cudaMalloc(" + std::to_string(want) + "): " + cudaGetErrorString(e));
    }
    cap = want;
    return SF_OK;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

struct PinBuf {
  void* p = nullptr;
  size_t cap = 0;
  ~PinBuf() {
    if (p) cudaFreeHost(p);
  }
  int ensure(size_t n) {
    if (n <= cap) return SF_OK;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    size_t want = n + n / 4 + 256;
    cudaError_t e = cudaMallocHost(&p, want);
    if (e != cudaSuccess) {
      p = nullptr;
      (void)cudaGetLastError();
      return fail(SF_ERR_NOMEM, "cudaMallocHost: " + std::string(cudaGetErrorString(e)));
    }
    cap = want;
    return SF_OK;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

// ---- passes ----------------------------------------------------------------------------

// PK_AFFINE16 and PK_CHAIN16 only classify buckets: an affine pass the packed 16-bit kernel
// runs, and a chain of sorted-text passes it runs in order.
enum PassKind : uint8_t {
  PK_MYERS = 0,
  PK_AFFINE = 1,
  PK_LOCAL = 2,
  PK_AFFINE16 = 3,
  PK_CHAIN16 = 4
};

// One DP pass as the reference's `affine_dp` / `distance` / `local_band_core` receive it.
struct Pass {
  PassKind kind;
  uint8_t mode = 0;
  bool clip = false, cell = false, want_cigar = false;
  uint8_t tb_kind = 0;  // 0: affine end, 1: extend-window end
  uint64_t p_off = 0, t_off = 0;  // byte offsets in the pool
  uint32_t m = 0, n = 0;
  uint64_t band = SF_NOLIMIT, geom = 0, cut = SF_NOLIMIT;
  int32_t xdrop = 0, end_bonus = 0, bonus0 = 0, bonus1 = 0;
  int64_t dlo = 0, dhi = 0;
  uint32_t k = SF_NONE;
  sf_affine_t sc{2, 4, 4, 2};
  // Sorted texts (align.rs:2210-2315 `affine_dp_sorted`): on a chain's first pass, how many
  // consecutive passes the chain holds; on each chained pass, the row its pass resumes after
  // (0: none), the common prefix of its text with the previous one and whether both bands
  // have the same shape.
  uint32_t chain = 0, resume = 0, lcp = 0;
  bool same_shape = false;
};

// A kernel class: what a pass runs on (kind, cells or blocks per lane, wide rows,
// traceback, Myers lanes per pair).
struct ClassKey {
  int kind = 0, c = 0, wide = 0, tb = 0, lanes = 0;
  bool operator<(const ClassKey& o) const {
    return std::tie(kind, c, wide, tb, lanes) < std::tie(o.kind, o.c, o.wide, o.tb, o.lanes);
  }
  bool operator==(const ClassKey& o) const {
    return kind == o.kind && c == o.c && wide == o.wide && tb == o.tb && lanes == o.lanes;
  }
};
// The autotuner's choices (sf_plan_tune): default class of a pass -> the class it runs in
// (affine: another C of the same kernel; Myers: blocks per lane and lanes per pair).
struct ClassChoice {
  int c = 0, lanes = 0;
};
using TuneTable = std::map<ClassKey, ClassChoice>;

struct Bucket {
  PassKind kind;
  int c = 0;       // affine: cells per lane; Myers: blocks per lane
  bool wide = false, tb = false;
  int lanes = 32;  // Myers: lanes per pair
  uint32_t first = 0, count = 0;  // range in the order array
  int grid = 0, block = 128;
  uint64_t scratch_off = 0;       // wide rows: this bucket's slice of the scratch (int32s)
  uint64_t work = 0;              // estimated work (cells of its passes' widest rows)
  uint64_t lat = 0;               // its longest pass's time, roughly (launch order)
  int stream = 0;                 // auxiliary stream it runs on
};

}  // namespace sfe

struct sf_store;
namespace sfe {
struct BuildScratch;
}

struct sf_plan {
  using Pass = sfe::Pass;
  using Bucket = sfe::Bucket;
  using DevBuf = sfe::DevBuf;
  using PinBuf = sfe::PinBuf;
  sf_context* ctx = nullptr;
  bool owns_ctx = false;
  std::vector<Pass> passes;
  // Sequences: unique (byte offset, length), packed word offsets.
  std::vector<uint64_t> seq_boff, seq_woff;
  std::vector<uint32_t> seq_len;
  uint64_t pool_bytes = 0, pool_words = 0;
  // Per pass: index in its kind's device arrays.
  std::vector<uint32_t> slot;
  uint32_t n_aff = 0, n_my = 0, n_walk = 0;
  bool myers_kcut = false;  // a Myers pass is Global or Prefix with k < m + n
  std::vector<Bucket> buckets;
  uint64_t tb_words = 0, ops_words = 0, scratch_cells = 0;
  int wide_warps = 0;
  std::string desc;
  // Device buffers.
  DevBuf d_bytes, d_pool, d_seq, d_djobs, d_params, d_res, d_mjobs, d_mout, d_tjobs, d_tres,
      d_tb, d_ops, d_opsc, d_offs, d_order, d_counters, d_wlist, d_cls, d_scratch, d_total,
      d_chains, d_links, d_want, d_snap;
  // Chains of sorted-call passes the plan runs on the chain kernel, their passes, and per
  // pass whether it is one of them.
  uint32_t n_chains = 0, n_chained = 0;
  std::vector<uint8_t> chained;
  // Pinned staging.
  PinBuf h_stage, h_res, h_mout, h_tres, h_ops, h_total;
  // Recorded after the last copies out of h_stage (its next writer waits for it).
  cudaEvent_t staged = nullptr;
  // The device byte pool of another plan this one reads instead of its own d_bytes (the
  // later segments of a segmented batch), or null.
  const uint8_t* bytes_from = nullptr;
  cudaGraphExec_t graph = nullptr;
  bool graph_tried = false;
  uint64_t launches = 0;
  // The transcript store SF_TEXT_STORE texts were resolved in (the context's at build time).
  const sf_store* store = nullptr;
  // Class overrides for this plan only (the autotuner's trial plans); else the context's.
  const sfe::TuneTable* tune_override = nullptr;
  // Host-side build arrays kept between builds (sf_plan.cu).
  std::unique_ptr<sfe::BuildScratch> scratch;
  // Out of line (sf_plan.cu): deleting an owned context needs sf_context complete, and the
  // build arrays their type.
  sf_plan();
  ~sf_plan();
};

// ---- context ---------------------------------------------------------------------------

// The transcript store: packed words, base p of the index's concatenation at position
// p + kStorePad (one leading word of padding, so that every window has a base before it).
struct sf_store {
  int dev = 0;
  uint64_t bases = 0;
  sfe::DevBuf words;
};
constexpr uint64_t kStorePad = 16;
// Pass::t_off of a store window: the flag plus the window's first position in the store.
constexpr uint64_t kStoreFlag = uint64_t(1) << 63;
// Pass::p_off / t_off read backwards (byte pool or store), as the mapper's leftward
// extensions read their read prefix and transcript flank.
constexpr uint64_t kRevFlag = uint64_t(1) << 62;
constexpr uint64_t kOffMask = ~(kStoreFlag | kRevFlag);

struct sf_context {
  int dev = 0;
  int sms = 0;
  cudaStream_t s = nullptr;
  // Auxiliary streams: kMain that buckets share round robin, then kSide for buckets of a
  // few long passes, so that no other bucket waits behind them.
  static constexpr int kMain = 8, kSide = 4, kAux = kMain + kSide;
  cudaStream_t aux[kAux] = {};
  cudaEvent_t fork = nullptr, join[kAux] = {};
  std::unique_ptr<sf_plan> cache;  // reused by sf_batch_run
  // sf_batch_run's later segments of a large batch (the first is `cache`), and the stream
  // each segment's tail (CIGAR compaction, copies back) runs on while later segments run,
  // with an event per segment at its tail's end.
  static constexpr int kSegs = 4;
  std::unique_ptr<sf_plan> segs[kSegs - 1];
  cudaStream_t tail = nullptr;
  cudaEvent_t seg_done[kSegs] = {};
  sfe::TuneTable tune;             // autotuner choices, applied to every later plan
  sf_store* store = nullptr;       // transcript store for SF_TEXT_STORE texts
  ~sf_context() {
    for (auto& p : segs) p.reset();
    cache.reset();
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(dev);
    for (int i = 0; i < kAux; ++i) {
      if (aux[i]) cudaStreamDestroy(aux[i]);
      if (join[i]) cudaEventDestroy(join[i]);
    }
    for (auto& e : seg_done)
      if (e) cudaEventDestroy(e);
    if (tail) cudaStreamDestroy(tail);
    if (fork) cudaEventDestroy(fork);
    if (s) cudaStreamDestroy(s);
    cudaSetDevice(prev);
  }
};


namespace sfe {

int make_context(int device, sf_context** out);
int jobs_to_passes(const sf_job_t* jobs, uint64_t count, const sf_affine_t* scores,
                   uint32_t n_scores, uint64_t pool_bytes, std::vector<Pass>& ps,
                   const sf_store* store = nullptr);
// Descriptors, buckets and device buffers for P->passes (pool not yet uploaded).
int plan_build(sf_plan* P);
int plan_job_buckets(const sf_plan* P, uint32_t* out, uint64_t count);
int plan_upload_from(sf_plan* P, const uint8_t* pool);
int plan_execute(sf_plan* P, bool use_graph);
int plan_fetch(sf_plan* P);
// The copies of plan_fetch, queued on `s` without waiting.
int plan_fetch_async(sf_plan* P, cudaStream_t s);
int plan_fetch_ops(sf_plan* P, uint64_t& total);
// Converts a fetched plan's results to sf_result_t (and copies compacted ops).
// `ops_base` is added to every cigar_off (the ops of earlier segments before `ops`).
int plan_results(sf_plan* P, sf_result_t* results, uint32_t* ops, uint64_t ops_cap,
                 uint64_t total, bool copy_ops = true, uint64_t ops_base = 0);
// Argument checks shared by the entry points: a mode of SF_INFIX/PREFIX/GLOBAL, and scores
// with non-negative gap costs.
bool ok_mode(int mode);
bool ok_sc(const sf_affine_t* sc);
// Kernel classes (sf_plan.cu).
bool allow16();
int default_lanes16();
void classify_affine(const Pass& p, uint32_t flags, int64_t wmax, bool use16, PassKind& kind,
                     int& c, bool& wide, int& lanes, int lanes16 = 32);
int choose_myers_class(uint32_t m, int& b, int& lanes);
DJob make_djob(const Pass& p, uint32_t& flags);
// Whether large sf_batch_run batches may run in segments (SF_BATCH_SEGMENTS).
bool batch_segments_on();
// The plan's pinned staging: stage_done marks the end of the copies issued out of it so
// far; stage_wait waits for that before it is written again.
int stage_wait(sf_plan* P);
int stage_done(sf_plan* P);
// One execute in parts: the pack and the buckets (each on its auxiliary stream, the main
// ones rotated by soff; also a single bucket with fan_one; `used` collects the streams),
// the auxiliary streams joined back into `s`, then the CIGAR compaction.  plan_launch runs
// all three; with `evs`, everything runs in order on `s` with an event after each stage.
int plan_launch_buckets(sf_plan* P, cudaStream_t s, std::vector<cudaEvent_t>* evs, int soff,
                        bool fan_one, bool* used);
int join_aux(sf_context* ctx, cudaStream_t s, const bool* used);
int plan_launch_compact(sf_plan* P, cudaStream_t s, std::vector<cudaEvent_t>* evs);
int plan_launch(sf_plan* P, cudaStream_t s, std::vector<cudaEvent_t>* evs = nullptr);
// Device bytes a plan of these passes needs (upper bound, before building it).
uint64_t plan_bytes_estimate(const std::vector<Pass>& passes, uint64_t pool_bytes);
// Device bytes the plan's buffers hold now.
uint64_t plan_bytes_held(const sf_plan* P);

}  // namespace sfe
