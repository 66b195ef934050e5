// Host side of the C ABI (include/sf_align.h): device contexts, batch plans (length
// bucketing, HBM layout, persistent launches captured in a CUDA graph) and the one-call
// entry points that mirror crates/map/src/align.rs.
#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <functional>
#include <deque>
#include <condition_variable>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include <unistd.h>

#include "sf_engine.h"

namespace sfe {

thread_local std::string g_err;
thread_local uint64_t g_dp_cells = 0, g_dp_rows = 0;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

const std::string& last_error() { return g_err; }

}  // namespace sfe

using namespace sfe;

namespace sfe {

int make_context(int device, sf_context** out) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    (void)cudaGetLastError();
    return fail(SF_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
  }
  if (device < 0 || device >= n) return fail(SF_ERR_INVALID, "device index out of range");
  std::unique_ptr<sf_context> c(new sf_context);
  c->dev = device;
  CK(cudaSetDevice(device));
  CK(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device));
  CK(cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking));
  for (int i = 0; i < sf_context::kAux; ++i) {
    CK(cudaStreamCreateWithFlags(&c->aux[i], cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&c->join[i], cudaEventDisableTiming));
  }
  CK(cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming));
  *out = c.release();
  return SF_OK;
}

int choose_affine_class(int64_t wmax, int& c, bool& wide) {
  for (int q = 0; q < sfk::kAffineNC; ++q)
    if (32 * (int64_t)sfk::kAffineC[q] >= wmax) {
      c = sfk::kAffineC[q];
      wide = false;
      return SF_OK;
    }
  c = sfk::kWideC;
  wide = true;
  return SF_OK;
}

// Whether a banded pass runs on the packed 16-bit kernel (sf_affine16_impl.cuh): Global or
// Prefix rows of a finite band with non-negative scores, whose reachable values all stay within
// 16384 below the row maximum the kernel rebases to every 64 rows -- the band's spread
// (mat + ext) * width + go, 64 rows of drift of the maximum either way, and a step of slack --
// and whose rows fit the widest 16-bit class.
bool fits16(const Pass& p, uint32_t flags, int64_t wmax) {
  if (p.kind != PK_AFFINE || (flags & F_FULL) || p.mode == SF_INFIX) return false;
  const sf_affine_t& s = p.sc;
  if (s.mat < 0 || s.mis < 0 || s.open < 0 || s.ext < 0) return false;
  if (s.mat > 1000 || s.mis > 1000 || s.open > 1000 || s.ext > 1000) return false;
  if (wmax > 32 * (int64_t)sfk::kAffine16C[sfk::kAffine16NC - 1]) return false;
  const int64_t go = (int64_t)s.open + s.ext;
  const int64_t step = std::max<int64_t>({(int64_t)s.mat, (int64_t)s.mis, go});
  const int64_t spread = ((int64_t)s.mat + s.ext) * wmax + go;
  return spread + 2 * 64 * step + 2 * (go + s.mis + s.ext) + s.mat + 256 <= 16384;
}

// SF_AFFINE16=0 in the environment turns the 16-bit kernel off (every pass then runs on the
// 32-bit kernel); read once per plan.
bool allow16() {
  const char* env = std::getenv("SF_AFFINE16");
  return !(env && env[0] == '0');
}

// Lanes per 16-bit pass by default: 32, or 16 (two passes per warp) with SF_AFFINE16_LANES=16
// in the environment; the autotuner chooses per length bucket either way.
int default_lanes16() {
  const char* env = std::getenv("SF_AFFINE16_LANES");
  return env && env[0] == '1' && env[1] == '6' ? 16 : 32;
}

// Row sharing between sorted texts on the GPU: SF_SORTED_CHAINS=1 in the environment runs
// the passes of a sorted call that can share rows as chains; by default every pass runs
// separately (the results are the same either way, and separate passes finish sooner on the
// batches measured: a chain runs its passes one after another); read once per plan.
// Large sf_batch_run batches run in segments (SF_BATCH_SEGMENTS=0 turns it off).
bool batch_segments_on() {
  const char* e = std::getenv("SF_BATCH_SEGMENTS");
  return !(e && e[0] == '0');
}

bool allow_chains() {
  const char* env = std::getenv("SF_SORTED_CHAINS");
  return env && env[0] == '1';
}

// Kernel class of an affine or local pass: the packed 16-bit kernel when the pass fits it,
// else the 32-bit register kernel, else (rows wider than 32 * 48 cells) the wide-row kernel.
void classify_affine(const Pass& p, uint32_t flags, int64_t wmax, bool use16, PassKind& kind,
                     int& c, bool& wide, int& lanes, int lanes16 = 32) {
  wide = false;
  lanes = 32;
  if (use16 && fits16(p, flags, wmax)) {
    if (lanes16 == 16)
      for (int q = 0; q < sfk::kAffine16HNC; ++q)
        if (16 * (int64_t)sfk::kAffine16HC[q] >= wmax) {
          kind = PK_AFFINE16;
          c = sfk::kAffine16HC[q];
          lanes = 16;
          return;
        }
    for (int q = 0; q < sfk::kAffine16NC; ++q)
      if (32 * (int64_t)sfk::kAffine16C[q] >= wmax) {
        kind = PK_AFFINE16;
        c = sfk::kAffine16C[q];
        return;
      }
  }
  kind = p.kind == PK_LOCAL ? PK_LOCAL : PK_AFFINE;
  choose_affine_class(wmax, c, wide);
}

// The autotuner's override for a pass's default class, if it chose one.
void apply_tune(const TuneTable* tune, int kind, int& c, bool wide, bool tb, int& lanes) {
  if (!tune || tune->empty()) return;
  auto it = tune->find(ClassKey{kind, c, wide ? 1 : 0, tb ? 1 : 0, lanes});
  if (it == tune->end()) return;
  c = it->second.c;
  lanes = it->second.lanes;
}

// Whether choose_myers_class takes a pattern of m bases (a check that sets no error).
bool myers_class_ok(uint32_t m) {
  if (m > SF_MYERS_MAX_PATTERN) return false;
  const uint32_t blocks = (m + 63) / 64;
  if (blocks <= 32) return true;
  for (int q = 0; q < sfk::kMyersNB; ++q)
    if (32u * (uint32_t)sfk::kMyersB[q] >= blocks) return true;
  return false;
}

int choose_myers_class(uint32_t m, int& b, int& lanes) {
  const uint32_t blocks = (m + 63) / 64;
  if (m > SF_MYERS_MAX_PATTERN) return fail(SF_ERR_TOO_LONG, "Myers pattern longer than SF_MYERS_MAX_PATTERN");
  if (blocks <= 32) {
    b = 1;
    lanes = 1;
    while ((uint32_t)lanes < blocks) lanes <<= 1;
    return SF_OK;
  }
  lanes = 32;
  for (int q = 0; q < sfk::kMyersNB; ++q)
    if (32u * (uint32_t)sfk::kMyersB[q] >= blocks) {
      b = sfk::kMyersB[q];
      return SF_OK;
    }
  return fail(SF_ERR_TOO_LONG, "pattern too long for the Myers kernels");
}

DJob make_djob(const Pass& p, uint32_t& flags) {
  DJob j{};
  j.m = p.m;
  j.n = p.n;
  flags = 0;
  if (p.kind == PK_LOCAL) {
    flags = F_LOCAL | F_ROWMAX;
    j.below = std::max<int64_t>(std::min<int64_t>(p.dlo, kGeoCap), -kGeoCap);
    j.above = std::max<int64_t>(std::min<int64_t>(p.dhi, kGeoCap), -kGeoCap);
  } else {
    flags = p.mode & 3u;
    const bool full = p.mode == SF_INFIX || p.band == SF_NOLIMIT;
    if (full) flags |= F_FULL;
    const uint64_t below = usat_add(p.band, usat_sub(p.m, p.geom));
    const uint64_t above = usat_add(p.band, usat_sub(p.geom, p.m));
    j.below = (int64_t)std::min<uint64_t>(below, (uint64_t)kGeoCap);
    j.above = (int64_t)std::min<uint64_t>(above, (uint64_t)kGeoCap);
    if (p.clip) flags |= F_CLIP | F_ROWMAX;
    if (p.clip && p.cell) flags |= F_CELL;
    if (p.cut != SF_NOLIMIT) flags |= F_CUT | F_ROWMAX;
    j.cut = p.cut;
  }
  return j;
}

}  // namespace sfe

namespace sfe {

// A bucket's key (kernel class) and one work item of it.
struct BucketKey {
  int kind, c, wide, tb, lanes;
  bool operator<(const BucketKey& o) const {
    return std::tie(kind, c, wide, tb, lanes) < std::tie(o.kind, o.c, o.wide, o.tb, o.lanes);
  }
  bool operator==(const BucketKey& o) const {
    return kind == o.kind && c == o.c && wide == o.wide && tb == o.tb && lanes == o.lanes;
  }
};
struct BucketItem {
  uint32_t slot;
  uint64_t work;
  uint64_t lat = 0;  // its warp's time, roughly: rows (steps) x the class's work per row
};

// Consecutive passes [first, first + count) of one sorted call that the chain kernel runs
// as one chain, on class C.
struct ChainSub {
  size_t first;
  uint32_t count;
  int c;
};

// A plan's host-side build arrays, kept between builds: a rebuild of a similar batch reuses
// their memory instead of faulting in fresh pages.  The build's phases pass their results
// to the next ones here.
struct BuildScratch {
  std::vector<uint64_t> word_of, pass_work, pass_lat, tb_need, ops_need;
  std::vector<DJob> dj;
  std::vector<DParams> dp;
  std::vector<TJob> tj;
  std::vector<uint16_t> cls;
  std::vector<MJob> mj;
  std::vector<uint32_t> wlist, kid, order;
  std::vector<std::pair<BucketKey, BucketItem>> items, per;
  std::vector<uint8_t> has_item;
  std::vector<std::pair<uint64_t, uint32_t>> byb, byb_tmp;
  std::vector<uint64_t> code_bits;
  std::vector<ChainSub> subs;
  std::vector<DChain> chains;
  std::vector<DLink> links;
  std::vector<uint32_t> want;
  uint64_t snap_words = 0;     // snapshot arena of the chains
  uint64_t scratch_total = 0;  // wide buckets' scratch, all slices
};

}  // namespace sfe

sf_plan::sf_plan() = default;

sf_plan::~sf_plan() {
  if (graph) cudaGraphExecDestroy(graph);
  if (staged) {
    cudaEventSynchronize(staged);  // copies out of h_stage end before it is freed
    cudaEventDestroy(staged);
  }
  if (owns_ctx) delete ctx;
}

namespace sfe {

uint64_t seq_words(uint64_t len) { return (len + 1 + 15) / 16; }

// Host worker threads for the plan build, started on first use and kept for the process:
// starting threads per call would cost more than small batches save.  A process that forks
// gets a fresh pool in the child (the parent's threads do not exist there).
class HostPool {
 public:
  static HostPool& get() {
    static std::mutex mu;
    static HostPool* pool = nullptr;
    std::lock_guard<std::mutex> g(mu);
    if (!pool || pool->pid_ != getpid()) pool = new HostPool();  // a child's old pool is abandoned
    return *pool;
  }
  size_t workers() const { return threads_.size(); }
  // Queues fn; returns false if it could not be queued.
  bool post(std::function<void()> fn) {
    try {
      std::lock_guard<std::mutex> g(m_);
      q_.push_back(std::move(fn));
      queued_.fetch_add(1, std::memory_order_release);
    } catch (...) {
      return false;
    }
    cv_.notify_one();
    return true;
  }
  // How long a worker (or a caller waiting for its chunks) polls before it sleeps: a plan
  // build posts its phases back to back, and a sleeping thread takes tens of microseconds
  // to wake.
  static constexpr std::chrono::microseconds kSpin{200};

 private:
  HostPool() : pid_(getpid()) {
    const unsigned hw = std::thread::hardware_concurrency();
    const unsigned n = std::min(7u, hw > 1 ? hw - 1 : 0u);
    try {
      for (unsigned k = 0; k < n; ++k) threads_.emplace_back([this] { loop(); });
    } catch (...) {
    }
    for (auto& t : threads_) t.detach();
  }
  void loop() {
    for (;;) {
      const auto t0 = std::chrono::steady_clock::now();
      while (queued_.load(std::memory_order_acquire) == 0 &&
             std::chrono::steady_clock::now() - t0 < kSpin) {
      }
      std::function<void()> fn;
      {
        std::unique_lock<std::mutex> g(m_);
        cv_.wait(g, [this] { return !q_.empty(); });
        fn = std::move(q_.front());
        q_.pop_front();
        queued_.fetch_sub(1, std::memory_order_relaxed);
      }
      fn();
    }
  }
  pid_t pid_;
  std::vector<std::thread> threads_;
  std::mutex m_;
  std::condition_variable cv_;
  std::deque<std::function<void()>> q_;
  std::atomic<size_t> queued_{0};  // q_.size(), readable without the lock
};

// f(begin, end, k) for the k-th of up to max_threads contiguous chunks of [0, n), chunks 1..
// on the host pool's threads, when every chunk gets at least min_per_thread items (else one
// chunk on the calling thread).  The same (n, min_per_thread, max_threads) always gives the
// same chunks; a chunk the pool cannot take runs on the calling thread.
// How many chunks parallel_chunks(n, min_per_thread, max_threads, ...) makes.
size_t chunks_for(size_t n, size_t min_per_thread, int max_threads) {
  const size_t t = std::min<size_t>({HostPool::get().workers() + 1, (size_t)max_threads,
                                     min_per_thread ? n / min_per_thread : 1});
  return std::max<size_t>(t, 1);
}

template <class F>
void parallel_chunks(size_t n, size_t min_per_thread, int max_threads, F&& f) {
  HostPool& pool = HostPool::get();
  const size_t t = chunks_for(n, min_per_thread, max_threads);
  if (t <= 1) {
    f(size_t(0), n, 0);
    return;
  }
  const size_t chunk = (n + t - 1) / t;
  // `left` changes only under `m`, so that a worker is out of `done` once the caller has
  // taken `m` after seeing it reach zero.
  struct Done {
    std::mutex m;
    std::condition_variable cv;
    std::atomic<size_t> left{0};
  } done;
  for (size_t k = 1; k < t; ++k) {
    const size_t b = k * chunk, e = std::min(n, (k + 1) * chunk);
    {
      std::lock_guard<std::mutex> g(done.m);
      done.left.fetch_add(1, std::memory_order_relaxed);
    }
    const bool queued = pool.post([&f, &done, b, e, k] {
      f(b, e, (int)k);
      std::lock_guard<std::mutex> g(done.m);
      if (done.left.fetch_sub(1, std::memory_order_acq_rel) == 1) done.cv.notify_all();
    });
    if (!queued) {
      {
        std::lock_guard<std::mutex> g(done.m);
        done.left.fetch_sub(1, std::memory_order_relaxed);
      }
      f(b, e, (int)k);
    }
  }
  f(size_t(0), std::min(n, chunk), 0);
  const auto t0 = std::chrono::steady_clock::now();
  while (done.left.load(std::memory_order_acquire) != 0 &&
         std::chrono::steady_clock::now() - t0 < HostPool::kSpin) {
  }
  std::unique_lock<std::mutex> g(done.m);
  done.cv.wait(g, [&] { return done.left.load(std::memory_order_acquire) == 0; });
}

// Builds descriptors, buckets and device buffers for `passes` (pool not yet uploaded).
// h_stage holds data for asynchronous copies on the context's stream: stage_done marks the
// end of the copies issued so far, and stage_wait waits for it before the staging is written
// or reallocated again.
int stage_wait(sf_plan* P) {
  if (P->staged) CK(cudaEventSynchronize(P->staged));
  return SF_OK;
}

int stage_done(sf_plan* P) {
  if (!P->staged) CK(cudaEventCreateWithFlags(&P->staged, cudaEventDisableTiming));
  CK(cudaEventRecord(P->staged, P->ctx->s));
  return SF_OK;
}

// The plan build, in phases: sequences, chains, pass descriptors, output offsets, chain
// descriptors, buckets, upload, description.

// Checks every pass's sequences against the pool (and the store), and lists the distinct
// sequences with their packed word offsets: P->seq_* per distinct sequence, S.word_of[u]
// per sequence u.
int build_sequences(sf_plan* P, BuildScratch& S) {
  const sf_context* ctx = P->ctx;
  const size_t np = P->passes.size();
  // Unique sequences.
  struct Key {
    uint64_t off;
    uint32_t len;
    uint32_t idx;
  };
  // Sequence u is pass u / 2's pattern (u even) or text (u odd).  Pass order is already in
  // (offset, length) order for a pool built in job order, the usual case: then no sort.
  auto seq_of = [&](size_t u, uint64_t& off, uint32_t& len) {
    const Pass& p = P->passes[u >> 1];
    off = (u & 1) ? p.t_off : p.p_off;
    len = (u & 1) ? p.n : p.m;
  };
  constexpr int kChunks = 8;
  bool in_order = true;
  // Per chunk of passes (the same chunks below): its new sequences and their words, counted
  // as if the pool were in order (a sequence equal to the one before it shares its words).
  size_t cnt[kChunks] = {};
  uint64_t wsum[kChunks] = {};
  {
    auto bad_pass = [&](const Pass& p) {
      return (p.p_off & kOffMask) + p.m > P->pool_bytes ||
             (!(p.t_off & kStoreFlag) && (p.t_off & kOffMask) + p.n > P->pool_bytes) ||
             ((p.t_off & kStoreFlag) && !ctx->store);
    };
    uint64_t first_bad[kChunks];
    bool ordered[kChunks];
    for (int k = 0; k < kChunks; ++k) {
      first_bad[k] = UINT64_MAX;
      ordered[k] = true;
    }
    parallel_chunks(np, 2048, kChunks, [&](size_t q0, size_t q1, int k) {
      uint64_t po = 0;
      uint32_t pl = 0;
      if (q0 > 0) seq_of(2 * q0 - 1, po, pl);
      for (size_t q = q0; q < q1; ++q) {
        if (bad_pass(P->passes[q])) {
          first_bad[k] = q;
          return;
        }
        for (size_t h = 0; h < 2; ++h) {
          uint64_t o;
          uint32_t l;
          seq_of(2 * q + h, o, l);
          if (q + h > 0 && (o < po || (o == po && l < pl))) ordered[k] = false;
          if (q + h == 0 || o != po || l != pl) {
            cnt[k]++;
            wsum[k] += seq_words(l);
          }
          po = o;
          pl = l;
        }
      }
    });
    uint64_t bad = UINT64_MAX;
    for (int k = 0; k < kChunks; ++k) {
      bad = std::min(bad, first_bad[k]);
      in_order = in_order && ordered[k];
    }
    if (bad != UINT64_MAX) {
      const Pass& p = P->passes[bad];
      if ((p.p_off & kOffMask) + p.m > P->pool_bytes ||
          (!(p.t_off & kStoreFlag) && (p.t_off & kOffMask) + p.n > P->pool_bytes))
        return fail(SF_ERR_INVALID, "job sequence outside the pool");
      return fail(SF_ERR_INVALID, "store text but the context uses no store");
    }
  }
  std::vector<Key> keys;
  if (!in_order) {
    keys.reserve(2 * np);
    for (size_t u = 0; u < 2 * np; ++u) {
      Key k;
      seq_of(u, k.off, k.len);
      k.idx = (uint32_t)u;
      keys.push_back(k);
    }
    std::sort(keys.begin(), keys.end(), [](const Key& a, const Key& b) {
      return a.off != b.off ? a.off < b.off : a.len < b.len;
    });
  }
  auto& word_of = S.word_of;
  word_of.resize(2 * np);
  uint64_t words = 0;
  if (in_order) {
    // Each chunk's new sequences at their places, from the counts above.
    size_t at0[kChunks] = {};
    uint64_t w0[kChunks] = {};
    size_t total = 0;
    for (int k = 0; k < kChunks; ++k) {
      at0[k] = total;
      w0[k] = words;
      total += cnt[k];
      words += wsum[k];
    }
    P->seq_boff.resize(total);
    P->seq_len.resize(total);
    P->seq_woff.resize(total);
    parallel_chunks(np, 2048, kChunks, [&](size_t q0, size_t q1, int k) {
      const size_t u0 = 2 * q0, u1 = 2 * q1;
      size_t at = at0[k];
      uint64_t w = w0[k], cur = 0, po = 0;
      uint32_t pl = 0;
      if (u0 > 0) {
        seq_of(u0 - 1, po, pl);
        cur = w - seq_words(pl);  // the last sequence before the chunk ends where it starts
      }
      for (size_t u = u0; u < u1; ++u) {
        uint64_t o;
        uint32_t l;
        seq_of(u, o, l);
        if (u == 0 || o != po || l != pl) {
          P->seq_boff[at] = o;
          P->seq_len[at] = l;
          P->seq_woff[at] = w;
          cur = w;
          w += seq_words(l);
          ++at;
        }
        word_of[u] = cur;
        po = o;
        pl = l;
      }
    });
  } else {
    P->seq_boff.clear();
    P->seq_len.clear();
    P->seq_woff.clear();
    uint64_t last_off = 0;
    uint32_t last_len = 0;
    for (size_t q = 0; q < 2 * np; ++q) {
      const uint64_t off = keys[q].off;
      const uint32_t len = keys[q].len;
      if (q == 0 || off != last_off || len != last_len) {
        P->seq_boff.push_back(off);
        P->seq_len.push_back(len);
        P->seq_woff.push_back(words);
        words += seq_words(len);
        last_off = off;
        last_len = len;
      }
      word_of[keys[q].idx] = P->seq_woff.back();
    }
  }
  P->pool_words = words + 512;  // slack: kernels read whole windows past a sequence's end
  return SF_OK;
}

// Sorted calls the chain kernel takes (Pass::chain on a call's first pass), when chains are
// on: every pass a 16-bit Global / Prefix pass without traceback, on the class of the call's
// widest row.  A call's passes form chains, each starting at a pass that resumes nothing (it
// depends on no earlier pass), which one warp runs in order.  Chains of one pass, and chains
// whose snapshots would pass the arena's cap, run as separate passes.  Fills S.subs and
// P->chained.
void choose_chains(sf_plan* P, BuildScratch& S, bool use16) {
  const size_t np = P->passes.size();
  auto& subs = S.subs;
  subs.clear();
  P->chained.assign(np, 0);
  {
    constexpr uint64_t kSnapCapWords = (uint64_t(1) << 30) / 4;
    uint64_t snap_total = 0;
    const bool on = use16 && allow_chains();
    for (size_t q = 0; on && q < np;) {
      const uint32_t cnt = P->passes[q].chain;
      if (cnt < 2 || cnt > np - q) {
        ++q;
        continue;
      }
      int64_t wm = 0;
      bool ok = true;
      for (size_t u = q; u < q + cnt && ok; ++u) {
        const Pass& p = P->passes[u];
        uint32_t fl = 0;
        const DJob j = make_djob(p, fl);
        const int64_t w = band_wmax(j, fl);
        ok = p.kind == PK_AFFINE && !p.want_cigar && fits16(p, fl, w) &&
             (!p.resume || (u > q && p.resume < p.m));
        wm = std::max(wm, w);
      }
      int c = 0;
      for (int k = 0; ok && k < sfk::kAffine16NC; ++k)
        if (32 * (int64_t)sfk::kAffine16C[k] >= wm) {
          c = sfk::kAffine16C[k];
          break;
        }
      for (size_t h = q; c && h < q + cnt;) {
        size_t e = h + 1;
        while (e < q + cnt && P->passes[e].resume) ++e;
        const uint64_t words = (e - h - 1) * snap_slot_words(c / 2);  // at most one per pass
        if (e - h >= 2 && snap_total + words <= kSnapCapWords) {
          snap_total += words;
          subs.push_back(ChainSub{h, (uint32_t)(e - h), c});
          for (size_t u = h; u < e; ++u) P->chained[u] = 1;
        }
        h = e;
      }
      q += cnt;
    }
  }
}

// Gives each pass its slot in its kind's arrays and writes its descriptor there, with its
// bucket key and work item (S.per, S.has_item) unless a chain takes it.
int describe_passes(sf_plan* P, BuildScratch& S, bool use16) {
  using Key2 = BucketKey;
  using Item = BucketItem;
  const sf_context* ctx = P->ctx;
  const size_t np = P->passes.size();
  const int lanes16 = default_lanes16();
  const TuneTable* tune = P->tune_override ? P->tune_override : &ctx->tune;
  const auto& word_of = S.word_of;
  auto& dj = S.dj;
  auto& dp = S.dp;
  auto& tj = S.tj;
  auto& cls = S.cls;
  auto& mj = S.mj;
  // Slots in each kind's arrays, in pass order: each chunk's Myers passes counted, then the
  // slots written.  Myers classes are checked here, so that the parallel part below cannot
  // fail.
  constexpr int kT = 8;
  uint64_t nmy[kT + 1] = {}, bad[kT];
  for (int k = 0; k < kT; ++k) bad[k] = UINT64_MAX;
  parallel_chunks(np, 4096, kT, [&](size_t q0, size_t q1, int k) {
    uint64_t c = 0;
    for (size_t q = q0; q < q1; ++q) {
      const Pass& p = P->passes[q];
      if (p.kind != PK_MYERS) continue;
      if (!myers_class_ok(p.m)) {
        bad[k] = q;
        break;
      }
      ++c;
    }
    nmy[k + 1] = c;
  });
  for (int k = 0; k < kT; ++k) {
    if (bad[k] != UINT64_MAX) {
      int b = 1, l = 1;
      return choose_myers_class(P->passes[bad[k]].m, b, l);  // sets the error
    }
    nmy[k + 1] += nmy[k];
  }
  P->slot.resize(np);
  parallel_chunks(np, 4096, kT, [&](size_t q0, size_t q1, int k) {
    uint64_t my = nmy[k];
    for (size_t q = q0; q < q1; ++q)
      P->slot[q] = (uint32_t)(P->passes[q].kind == PK_MYERS ? my++ : q - my);
  });
  const size_t n_myers = nmy[kT];
  const size_t n_affine = np - n_myers;
  mj.resize(n_myers);
  dj.resize(n_affine);
  dp.resize(n_affine);
  tj.resize(n_affine);
  cls.resize(n_affine);
  auto& pass_work = S.pass_work;
  auto& pass_lat = S.pass_lat;
  auto& tb_need = S.tb_need;
  auto& ops_need = S.ops_need;
  auto& per = S.per;
  auto& has_item = S.has_item;
  // Every entry below is written for its pass by `describe`.
  pass_work.resize(np);
  pass_lat.resize(np);
  tb_need.resize(n_affine);
  ops_need.resize(n_affine);
  per.resize(np);
  has_item.resize(np);
  constexpr int kMaxThreads = 8;
  uint64_t scratch_max[kMaxThreads] = {};
  // Descriptors of passes [q0, q1), each written at its slot.
  auto describe = [&](size_t q0, size_t q1, int worker) {
    // The tune table's answers, memoised per class (a batch has few classes).
    struct TuneMemo {
      ClassKey key;
      int c, lanes;
    };
    std::vector<TuneMemo> memo;
    auto tuned = [&](int kind, int& c, bool wide, bool tb, int& lanes) {
      if (!tune || tune->empty()) return;
      const ClassKey k{kind, c, wide ? 1 : 0, tb ? 1 : 0, lanes};
      for (size_t u = memo.size(); u-- > 0;)
        if (memo[u].key == k) {
          c = memo[u].c;
          lanes = memo[u].lanes;
          return;
        }
      apply_tune(tune, kind, c, wide, tb, lanes);
      memo.push_back(TuneMemo{k, c, lanes});
    };
    for (size_t q = q0; q < q1; ++q) {
      const Pass& p = P->passes[q];
      const uint32_t sl = P->slot[q];
      if (p.kind == PK_MYERS) {
        int b = 1, lanes = 1;
        (void)choose_myers_class(p.m, b, lanes);
        tuned(PK_MYERS, b, false, false, lanes);
        MJob& m = mj[sl];
        m = MJob{};
        m.p_word = word_of[2 * q];
        m.t_word = word_of[2 * q + 1];
        m.m = p.m;
        m.n = p.n;
        m.mode = p.mode;
        m.k = p.k;
        per[q] = {Key2{PK_MYERS, b, 0, 0, lanes},
                  Item{sl, (uint64_t)p.n, ((uint64_t)p.n + (uint64_t)lanes) * (4u * (uint64_t)b + 4u)}};
        has_item[q] = 1;
        pass_work[q] = pass_lat[q] = 0;
        continue;
      }
      uint32_t flags = 0;
      DJob j = make_djob(p, flags);
      j.p_word = word_of[2 * q];
      j.t_word = word_of[2 * q + 1];
      j.p_byte = p.p_off & kOffMask;
      const int64_t wmax = band_wmax(j, flags);
      int c = 4;
      bool wide = false;
      PassKind kind = PK_AFFINE;
      int ln = 32;
      classify_affine(p, flags, wmax, use16, kind, c, wide, ln, lanes16);
      const bool tb = p.want_cigar && p.kind != PK_LOCAL;
      if (!wide) tuned(kind, c, false, tb, ln);
      TJob t{};
      if (tb) {
        flags |= F_TB;
        const int64_t chunks = wide ? wide_chunks(c, wmax) : 1;
        tb_need[sl] = (uint64_t)p.m * (tb_row_words(c, chunks) * (uint64_t)ln / 32);
        const uint64_t cap = (uint64_t)p.m + p.n + 2;
        ops_need[sl] = cap;
        t.ops_cap = (uint32_t)std::min<uint64_t>(cap, 0xffffffffull);
        t.kind = p.tb_kind;
        t.end_bonus = p.end_bonus;
      } else {
        tb_need[sl] = ops_need[sl] = 0;
      }
      if (wide)
        scratch_max[worker] =
            std::max<uint64_t>(scratch_max[worker], (uint64_t)wide_chunks(c, wmax) * 32 * c);
      DParams pr{};
      pr.flags = flags;
      pr.xdrop = p.xdrop;
      pr.bonus0 = p.bonus0;
      pr.bonus1 = p.bonus1;
      pr.mat = p.sc.mat;
      pr.mis = p.sc.mis;
      pr.open = p.sc.open;
      pr.ext = p.sc.ext;
      const uint64_t work = (uint64_t)std::max<uint32_t>(p.m, 1) * (uint64_t)std::max<int64_t>(wmax, 1);
      pass_work[q] = work;
      const uint64_t row_cost = (uint64_t)c * (wide ? (uint64_t)wide_chunks(c, wmax) : 1u) + 8u;
      pass_lat[q] = (uint64_t)std::max<uint32_t>(p.m, 1) * row_cost;
      has_item[q] = !P->chained[q];
      if (has_item[q]) per[q] = {Key2{kind, c, wide, tb, ln}, Item{sl, work, pass_lat[q]}};
      dj[sl] = j;
      dp[sl] = pr;
      tj[sl] = t;
      cls[sl] = (uint16_t)(c | (wide ? 0x100 : 0) | (kind == PK_AFFINE16 ? 0x200 : 0));
    }
  };
  parallel_chunks(np, 2048, kMaxThreads, describe);
  uint64_t scratch_cells = 0;
  for (int w = 0; w < kMaxThreads; ++w) scratch_cells = std::max(scratch_cells, scratch_max[w]);
  P->scratch_cells = scratch_cells;
  return SF_OK;
}

// Offsets in pass order: traceback words, CIGAR slots, the walk list; then the passes' work
// items (S.items).
void lay_out_outputs(sf_plan* P, BuildScratch& S) {
  const size_t np = P->passes.size(), na = S.dj.size();
  auto& dj = S.dj;
  auto& tj = S.tj;
  auto& wlist = S.wlist;
  auto& items = S.items;
  // Two passes over the same chunks: each chunk's totals, then its entries at their places.
  constexpr int kT = 8;
  struct Sums {
    uint64_t tb = 0, ops = 0, walks = 0;
  } sum[kT + 1];
  parallel_chunks(na, 4096, kT, [&](size_t s0, size_t s1, int k) {
    Sums z;
    for (size_t sl = s0; sl < s1; ++sl) {
      if (!(S.dp[sl].flags & F_TB)) continue;
      z.tb += S.tb_need[sl];
      z.ops += S.ops_need[sl];
      z.walks++;
    }
    sum[k + 1] = z;
  });
  for (int k = 0; k < kT; ++k) {
    sum[k + 1].tb += sum[k].tb;
    sum[k + 1].ops += sum[k].ops;
    sum[k + 1].walks += sum[k].walks;
  }
  wlist.resize(sum[kT].walks);
  parallel_chunks(na, 4096, kT, [&](size_t s0, size_t s1, int k) {
    Sums z = sum[k];
    for (size_t sl = s0; sl < s1; ++sl) {
      if (!(S.dp[sl].flags & F_TB)) continue;
      dj[sl].tb_word = z.tb;
      z.tb += S.tb_need[sl];
      tj[sl].ops_off = z.ops;
      z.ops += S.ops_need[sl];
      wlist[z.walks++] = (uint32_t)sl;
    }
  });
  uint64_t cnt[kT + 1] = {};
  parallel_chunks(np, 4096, kT, [&](size_t q0, size_t q1, int k) {
    uint64_t c = 0;
    for (size_t q = q0; q < q1; ++q) c += S.has_item[q];
    cnt[k + 1] = c;
  });
  for (int k = 0; k < kT; ++k) cnt[k + 1] += cnt[k];
  items.resize(cnt[kT]);
  parallel_chunks(np, 4096, kT, [&](size_t q0, size_t q1, int k) {
    uint64_t at = cnt[k];
    for (size_t q = q0; q < q1; ++q)
      if (S.has_item[q]) items[at++] = S.per[q];
  });
  P->tb_words = sum[kT].tb;
  P->ops_words = sum[kT].ops;
}

// Chains: one work item each (longest first, as passes); per chained job its link; per
// chain its snapshot rows, the sorted distinct resume rows (align.rs:2244-2246), and a slot
// for each.
void build_chains(sf_plan* P, BuildScratch& S) {
  auto& chains = S.chains;
  auto& links = S.links;
  auto& want = S.want;
  chains.clear();
  links.clear();
  want.clear();
  uint64_t snap_words = 0;
  uint32_t n_chained = 0;
  for (const ChainSub& sb : S.subs) {
    if (links.empty()) links.assign(S.dj.size(), DLink{});
    DChain ch{};
    ch.first = P->slot[sb.first];
    ch.count = sb.count;
    ch.want = (uint32_t)want.size();
    ch.snap_word = snap_words;
    std::vector<uint32_t> rows;
    uint64_t work = 0, lat = 0;
    for (size_t u = sb.first; u < sb.first + sb.count; ++u) {
      if (u > sb.first) rows.push_back(P->passes[u].resume);
      work += S.pass_work[u];
      lat += S.pass_lat[u];
    }
    std::sort(rows.begin(), rows.end());
    rows.erase(std::unique(rows.begin(), rows.end()), rows.end());
    ch.n_want = (uint32_t)rows.size();
    for (size_t u = sb.first; u < sb.first + sb.count; ++u) {
      const Pass& p = P->passes[u];
      DLink& L = links[P->slot[u]];
      L.resume = u > sb.first ? p.resume : 0;
      L.slot = L.resume ? (uint32_t)(std::lower_bound(rows.begin(), rows.end(), L.resume) - rows.begin()) : 0;
      L.lcp = p.lcp;
      L.same_shape = p.same_shape ? 1u : 0u;
    }
    want.insert(want.end(), rows.begin(), rows.end());
    snap_words += rows.size() * snap_slot_words(sb.c / 2);
    S.items.push_back({BucketKey{PK_CHAIN16, sb.c, 0, 0, 32},
                       BucketItem{(uint32_t)chains.size(), work, lat}});
    chains.push_back(ch);
    n_chained += sb.count;
  }
  S.snap_words = snap_words;
  P->n_chains = (uint32_t)chains.size();
  P->n_chained = n_chained;
}

// Buckets of S.items by key, their launch order, shapes and streams (P->buckets), and the
// execution order of the work items (S.order).
void build_buckets(sf_plan* P, BuildScratch& S) {
  using Key2 = BucketKey;
  const sf_context* ctx = P->ctx;
  const auto& items = S.items;
  const size_t ni = items.size();
  constexpr int kT = 8;
  // Buckets in key order; within a bucket, longest work first (ties in job order).
  // Each item's bucket first: keys pack into 18-bit codes ordered as the keys are (kind < 8,
  // C < 128, lanes < 64), so a bit set of the codes present lists the buckets in order and a
  // code's bucket is the number of codes below it.  Keys outside those bounds (never built)
  // take a search instead.
  auto& kid = S.kid;
  kid.resize(ni);
  std::vector<Key2> keys;  // the buckets' keys, in order
  {
    constexpr uint32_t kWords = (1u << 18) / 64;
    auto fits = [](const Key2& k) {
      return k.kind >= 0 && k.kind < 8 && k.c >= 0 && k.c < 128 && (k.wide & ~1) == 0 &&
             (k.tb & ~1) == 0 && k.lanes >= 0 && k.lanes < 64;
    };
    auto& bits = S.code_bits;
    const size_t nt = chunks_for(ni, 4096, kT);  // the chunks below: each its own bit set
    bits.assign(nt * kWords, 0);
    bool packed[kT];
    std::fill(packed, packed + kT, true);
    parallel_chunks(ni, 4096, kT, [&](size_t q0, size_t q1, int k) {
      uint64_t* w = bits.data() + (size_t)k * kWords;
      for (size_t q = q0; q < q1; ++q) {
        const Key2& key = items[q].first;
        if (!fits(key)) {
          packed[k] = false;
          return;
        }
        const uint32_t c = (uint32_t)key.kind << 15 | (uint32_t)key.c << 8 |
                           (uint32_t)key.wide << 7 | (uint32_t)key.tb << 6 | (uint32_t)key.lanes;
        kid[q] = c;
        w[c >> 6] |= uint64_t(1) << (c & 63);
      }
    });
    if (std::all_of(packed, packed + kT, [](bool x) { return x; })) {
      std::vector<uint32_t> below(kWords + 1, 0);
      for (uint32_t w = 0; w < kWords; ++w) {
        uint64_t x = 0;
        for (size_t k = 0; k < nt; ++k) x |= bits[k * kWords + w];
        bits[w] = x;
        below[w + 1] = below[w] + (uint32_t)__builtin_popcountll(x);
        for (; x; x &= x - 1) {
          const int c = (int)(w * 64 + (uint32_t)__builtin_ctzll(x));
          keys.push_back(Key2{c >> 15, (c >> 8) & 127, (c >> 7) & 1, (c >> 6) & 1, c & 63});
        }
      }
      parallel_chunks(ni, 4096, kT, [&](size_t q0, size_t q1, int) {
        for (size_t q = q0; q < q1; ++q) {
          const uint32_t c = kid[q];
          kid[q] = below[c >> 6] + (uint32_t)__builtin_popcountll(bits[c >> 6] & ((uint64_t(1) << (c & 63)) - 1));
        }
      });
    } else {
      for (const auto& it : items) keys.push_back(it.first);
      std::sort(keys.begin(), keys.end());
      keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
      for (size_t q = 0; q < ni; ++q)
        kid[q] = (uint32_t)(std::lower_bound(keys.begin(), keys.end(), items[q].first) - keys.begin());
    }
  }
  // A stable counting sort by bucket: each chunk's items and work per bucket, then the
  // chunks' places (bucket-major, chunk-minor) and a second pass over the same chunks.
  const size_t nb = keys.size();
  std::vector<uint64_t> at((size_t)kT * nb, 0), wsum((size_t)kT * nb, 0);
  parallel_chunks(ni, 4096, kT, [&](size_t q0, size_t q1, int k) {
    uint64_t* c = at.data() + (size_t)k * nb;
    uint64_t* ws = wsum.data() + (size_t)k * nb;
    for (size_t q = q0; q < q1; ++q) {
      c[kid[q]]++;
      ws[kid[q]] += items[q].second.work;
    }
  });
  std::vector<uint64_t> start(nb + 1, 0), bwork(nb, 0);
  {
    uint64_t acc = 0;
    for (size_t u = 0; u < nb; ++u) {
      start[u] = acc;
      for (int k = 0; k < kT; ++k) {
        const uint64_t c = at[(size_t)k * nb + u];
        at[(size_t)k * nb + u] = acc;
        acc += c;
        bwork[u] += wsum[(size_t)k * nb + u];
      }
    }
    start[nb] = acc;
  }
  auto& byb = S.byb;  // (work, job order) by bucket
  byb.resize(ni);
  parallel_chunks(ni, 4096, kT, [&](size_t q0, size_t q1, int k) {
    uint64_t* a = at.data() + (size_t)k * nb;
    for (size_t q = q0; q < q1; ++q) byb[a[kid[q]]++] = {items[q].second.work, (uint32_t)q};
  });
  auto& order = S.order;
  order.resize(ni);
  P->buckets.assign(nb, Bucket{});
  for (size_t u = 0; u < nb; ++u) {
    Bucket& b = P->buckets[u];
    b.kind = (PassKind)keys[u].kind;
    b.c = keys[u].c;
    b.wide = keys[u].wide;
    b.tb = keys[u].tb;
    b.lanes = keys[u].lanes;
    b.first = (uint32_t)start[u];
    b.count = (uint32_t)(start[u + 1] - start[u]);
    b.work = bwork[u];
  }
  // Longest first within a bucket, by work rounded to 1/16 of its power of two (a stable
  // counting sort: equal rounded work keeps job order).  Buckets of many items sort on the
  // host pool one at a time; the others sort side by side.
  auto wbin = [](uint64_t w) -> uint32_t {
    if (w < 16) return (uint32_t)w;
    const int e = 63 - __builtin_clzll(w);  // w in [2^e, 2^(e+1))
    return (uint32_t)(16 * (e - 3) + ((w >> (e - 4)) & 15));
  };
  constexpr uint32_t kBins = 16 * 61 + 16;
  constexpr size_t kBig = 4096;
  auto& tmp = S.byb_tmp;
  std::vector<uint64_t> bin_at((size_t)kT * kBins);
  for (size_t u = 0; u < nb; ++u) {
    Bucket& b = P->buckets[u];
    if (b.count < kBig) continue;
    const auto* src = byb.data() + b.first;
    const size_t n = b.count;
    std::fill(bin_at.begin(), bin_at.end(), 0);
    parallel_chunks(n, 2048, kT, [&](size_t e0, size_t e1, int k) {
      uint64_t* c = bin_at.data() + (size_t)k * kBins;
      for (size_t e = e0; e < e1; ++e) c[kBins - 1 - wbin(src[e].first)]++;
    });
    uint64_t acc = 0;
    uint32_t bins_used = 0;
    for (uint32_t v = 0; v < kBins; ++v) {
      const uint64_t a0 = acc;
      for (int k = 0; k < kT; ++k) {
        const uint64_t c = bin_at[(size_t)k * kBins + v];
        bin_at[(size_t)k * kBins + v] = acc;
        acc += c;
      }
      bins_used += acc > a0;
    }
    // One bin (work alike): job order is the order.
    const std::pair<uint64_t, uint32_t>* sorted = src;
    if (bins_used > 1) {
      tmp.resize(n);
      parallel_chunks(n, 2048, kT, [&](size_t e0, size_t e1, int k) {
        uint64_t* a = bin_at.data() + (size_t)k * kBins;
        for (size_t e = e0; e < e1; ++e) tmp[a[kBins - 1 - wbin(src[e].first)]++] = src[e];
      });
      sorted = tmp.data();
    }
    uint64_t lat[kT] = {};
    parallel_chunks(n, 2048, kT, [&](size_t e0, size_t e1, int k) {
      uint64_t l = 0;
      for (size_t e = e0; e < e1; ++e) {
        const BucketItem& it = items[sorted[e].second].second;
        order[b.first + e] = it.slot;
        l = std::max(l, it.lat);
      }
      lat[k] = l;
    });
    b.lat = *std::max_element(lat, lat + kT);
  }
  parallel_chunks(nb, ni >= 16384 ? 1 : nb + 1, kT, [&](size_t u0, size_t u1, int) {
    std::vector<uint32_t> bin_n(kBins + 1);
    std::vector<std::pair<uint64_t, uint32_t>> part;
    for (size_t u = u0; u < u1; ++u) {
      Bucket& b = P->buckets[u];
      if (b.count >= kBig) continue;
      auto b0 = byb.begin() + (ptrdiff_t)b.first, b1 = b0 + (ptrdiff_t)b.count;
      std::fill(bin_n.begin(), bin_n.end(), 0u);
      for (auto it = b0; it != b1; ++it) bin_n[kBins - 1 - wbin(it->first) + 1]++;
      for (uint32_t k = 0; k < kBins; ++k) bin_n[k + 1] += bin_n[k];
      part.assign(b0, b1);
      for (const auto& e : part) *(b0 + bin_n[kBins - 1 - wbin(e.first)]++) = e;
      for (auto it = b0; it != b1; ++it) {
        order[(size_t)(it - byb.begin())] = items[it->second].second.slot;
        b.lat = std::max(b.lat, items[it->second].second.lat);
      }
    }
  });
  // Launch order: the buckets whose longest pass takes longest first, so that a few long
  // passes (a small grid) run beside the bulk instead of after it.
  std::stable_sort(P->buckets.begin(), P->buckets.end(),
                   [](const Bucket& x, const Bucket& y) { return x.lat > y.lat; });
  // Launch shapes: persistent grids, at most what fits the device at once.  Wide buckets
  // may run concurrently (fan-out streams), so each gets its own scratch slice.
  int wide_warps = 0;
  uint64_t scratch_total = 0;
  for (auto& b : P->buckets) {
    if (b.kind == PK_MYERS) {
      b.block = b.c <= 4 ? 128 : (b.c <= 8 ? 64 : 32);
      const uint64_t per_warp = (uint64_t)(32 / b.lanes);
      const uint64_t warps = (b.count + per_warp - 1) / per_warp;
      const uint64_t wpb = (uint64_t)b.block / 32;
      b.grid = (int)std::min<uint64_t>((warps + wpb - 1) / wpb, (uint64_t)ctx->sms * (2048 / b.block));
    } else {
      b.block = 128;
      const uint64_t per_block = b.lanes == 16 ? 8 : 4;  // passes (chains) a 4-warp block holds
      const uint64_t blocks = (b.count + per_block - 1) / per_block;
      const uint64_t cap = b.wide ? (uint64_t)ctx->sms * 2 : (uint64_t)ctx->sms * 16;
      b.grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(blocks, cap));
      if (b.wide) {
        wide_warps += b.grid * 4;
        b.scratch_off = scratch_total;
        scratch_total += (uint64_t)b.grid * 4 * 4 * P->scratch_cells;
      }
    }
  }
  P->wide_warps = wide_warps;
  S.scratch_total = scratch_total;
  // Streams: round robin over the buckets in launch order, so that their tails overlap.
  for (size_t u = 0; u < P->buckets.size(); ++u) P->buckets[u].stream = (int)(u % sf_context::kAux);
}

// Device buffers sized for the plan, and its descriptors copied there.
int upload_plan(sf_plan* P, BuildScratch& S) {
  sf_context* ctx = P->ctx;
  const auto& dj = S.dj;
  const auto& dp = S.dp;
  const auto& tj = S.tj;
  const auto& cls = S.cls;
  const auto& mj = S.mj;
  const auto& wlist = S.wlist;
  const auto& order = S.order;
  const auto& chains = S.chains;
  const auto& links = S.links;
  const auto& want = S.want;
  const uint64_t tb_words = P->tb_words, ops_words = P->ops_words;
  const uint64_t scratch_total = S.scratch_total, snap_words = S.snap_words;
  int rc;
  if (!P->bytes_from && (rc = P->d_bytes.ensure(std::max<uint64_t>(P->pool_bytes, 16)))) return rc;
  if ((rc = P->d_pool.ensure(P->pool_words * 4))) return rc;
  const size_t nseq = P->seq_boff.size();
  if ((rc = P->d_seq.ensure(nseq * 20 + 64))) return rc;
  if ((rc = P->d_djobs.ensure(dj.size() * sizeof(DJob) + 64))) return rc;
  if ((rc = P->d_params.ensure(dp.size() * sizeof(DParams) + 64))) return rc;
  if ((rc = P->d_res.ensure(dj.size() * sizeof(DRes) + 64))) return rc;
  if ((rc = P->d_tjobs.ensure(tj.size() * sizeof(TJob) + 64))) return rc;
  if ((rc = P->d_tres.ensure(tj.size() * sizeof(TRes) + 64))) return rc;
  if ((rc = P->d_cls.ensure(cls.size() * 2 + 64))) return rc;
  if ((rc = P->d_mjobs.ensure(mj.size() * sizeof(MJob) + 64))) return rc;
  if ((rc = P->d_mout.ensure(mj.size() * 4 + 64))) return rc;
  if ((rc = P->d_tb.ensure(tb_words * 4 + 64))) return rc;
  if ((rc = P->d_ops.ensure(ops_words * 4 + 64))) return rc;
  if ((rc = P->d_opsc.ensure(ops_words * 4 + 64))) return rc;
  if ((rc = P->d_offs.ensure(wlist.size() * 8 + 64))) return rc;
  if ((rc = P->d_total.ensure(64))) return rc;
  if ((rc = P->d_order.ensure(order.size() * 4 + 64))) return rc;
  if ((rc = P->d_counters.ensure(P->buckets.size() * 4 + 64))) return rc;
  if ((rc = P->d_wlist.ensure(wlist.size() * 4 + 64))) return rc;
  if ((rc = P->d_scratch.ensure(scratch_total * 4 + 64))) return rc;
  if ((rc = P->d_chains.ensure(chains.size() * sizeof(DChain) + 64))) return rc;
  if ((rc = P->d_links.ensure(links.size() * sizeof(DLink) + 64))) return rc;
  if ((rc = P->d_want.ensure(want.size() * 4 + 64))) return rc;
  if ((rc = P->d_snap.ensure(snap_words * 4 + 64))) return rc;
  // Descriptors -> device (one pinned staging area, one stream).  Every array goes into the
  // staging (on host threads, in pieces), then one copy per device buffer.  The sequence
  // table is byte offsets, word offsets (both 8-byte aligned), then lengths.
  struct Part {
    const void* src;
    size_t bytes, at;
  };
  struct Copy {
    DevBuf* d;
    size_t at, bytes;
  };
  std::vector<Part> parts;
  std::vector<Copy> copies;
  size_t at = 0;
  auto put = [&](DevBuf& d, std::initializer_list<std::pair<const void*, size_t>> srcs) {
    size_t bytes = 0;
    for (const auto& sp : srcs) {
      if (sp.second) parts.push_back(Part{sp.first, sp.second, at + bytes});
      bytes += sp.second;
    }
    if (!bytes) return;
    copies.push_back(Copy{&d, at, bytes});
    at += (bytes + 15) & ~size_t(15);
  };
  put(P->d_seq, {{P->seq_boff.data(), nseq * 8}, {P->seq_woff.data(), nseq * 8},
                 {P->seq_len.data(), nseq * 4}});
  put(P->d_djobs, {{dj.data(), dj.size() * sizeof(DJob)}});
  put(P->d_params, {{dp.data(), dp.size() * sizeof(DParams)}});
  put(P->d_tjobs, {{tj.data(), tj.size() * sizeof(TJob)}});
  put(P->d_cls, {{cls.data(), cls.size() * 2}});
  put(P->d_mjobs, {{mj.data(), mj.size() * sizeof(MJob)}});
  put(P->d_order, {{order.data(), order.size() * 4}});
  put(P->d_wlist, {{wlist.data(), wlist.size() * 4}});
  put(P->d_chains, {{chains.data(), chains.size() * sizeof(DChain)}});
  put(P->d_links, {{links.data(), links.size() * sizeof(DLink)}});
  put(P->d_want, {{want.data(), want.size() * 4}});
  if ((rc = stage_wait(P))) return rc;
  if ((rc = P->h_stage.ensure(at + 16))) return rc;
  uint8_t* h = P->h_stage.as<uint8_t>();
  {
    constexpr size_t kPiece = size_t(256) << 10;
    std::vector<std::pair<uint32_t, size_t>> pieces;  // (part, offset)
    for (size_t u = 0; u < parts.size(); ++u)
      for (size_t o = 0; o < parts[u].bytes; o += kPiece) pieces.push_back({(uint32_t)u, o});
    parallel_chunks(pieces.size(), 2, 8, [&](size_t k0, size_t k1, int) {
      for (size_t k = k0; k < k1; ++k) {
        const Part& pt = parts[pieces[k].first];
        const size_t o = pieces[k].second, n = std::min(kPiece, pt.bytes - o);
        std::memcpy(h + pt.at + o, static_cast<const uint8_t*>(pt.src) + o, n);
      }
    });
  }
  for (const Copy& c : copies)
    CK(cudaMemcpyAsync(c.d->p, h + c.at, c.bytes, cudaMemcpyHostToDevice, ctx->s));
  // The pool's slack words stay zero.
  CK(cudaMemsetAsync(P->d_pool.p, 0, P->pool_words * 4, ctx->s));
  if ((rc = stage_done(P))) return rc;
  if (P->graph) {
    cudaGraphExecDestroy(P->graph);
    P->graph = nullptr;
  }
  P->graph_tried = false;
  return SF_OK;
}

// The plan's description (sf_plan_describe): its buckets and arena sizes, as JSON.
void describe_plan(sf_plan* P, const BuildScratch& S) {
  std::string d = "{\"buckets\": [";
  for (size_t q = 0; q < P->buckets.size(); ++q) {
    const Bucket& b = P->buckets[q];
    char buf[256];
    std::snprintf(buf, sizeof buf,
                  "%s{\"kind\": \"%s\", \"c\": %d, \"wide\": %s, \"traceback\": %s, \"lanes\": %d, "
                  "\"jobs\": %u, \"grid\": %d, \"block\": %d, \"work\": %llu}",
                  q ? ", " : "",
                  b.kind == PK_MYERS     ? "myers"
                  : b.kind == PK_LOCAL   ? "local"
                  : b.kind == PK_AFFINE16 ? "affine16"
                  : b.kind == PK_CHAIN16 ? "chain16"
                                         : "affine",
                  b.c,
                  b.wide ? "true" : "false", b.tb ? "true" : "false", b.lanes, b.count, b.grid,
                  b.block, (unsigned long long)b.work);
    d += buf;
  }
  d += "], \"chains\": " + std::to_string(P->n_chains) +
       ", \"chained_passes\": " + std::to_string(P->n_chained) +
       ", \"snapshot_bytes\": " + std::to_string(S.snap_words * 4) +
       ", \"pool_words\": " + std::to_string(P->pool_words) +
       ", \"traceback_bytes\": " + std::to_string(P->tb_words * 4) + "}";
  P->desc = d;
}

int plan_build(sf_plan* P) {
  if (!P->scratch) P->scratch.reset(new BuildScratch);
  BuildScratch& S = *P->scratch;
  sf_context* ctx = P->ctx;
  CK(cudaSetDevice(ctx->dev));
  if (P->passes.size() > 0xffffffffull / 2) return fail(SF_ERR_INVALID, "too many jobs");
  int rc;
  if ((rc = build_sequences(P, S))) return rc;
  P->store = ctx->store;
  const bool use16 = allow16();
  choose_chains(P, S, use16);
  if ((rc = describe_passes(P, S, use16))) return rc;
  lay_out_outputs(P, S);
  build_chains(P, S);
  P->n_aff = (uint32_t)S.dj.size();
  P->n_my = (uint32_t)S.mj.size();
  P->n_walk = (uint32_t)S.wlist.size();
  build_buckets(P, S);
  if ((rc = upload_plan(P, S))) return rc;
  describe_plan(P, S);
  return SF_OK;
}

// The device copy of the plan's byte pool: its own, or the one it borrows.
const uint8_t* plan_dev_bytes(const sf_plan* P) {
  return P->bytes_from ? P->bytes_from : P->d_bytes.as<uint8_t>();
}

// With `evs`, records an event on `s` (per-stage timing).
int mark_stage(std::vector<cudaEvent_t>* evs, cudaStream_t s) {
  if (!evs) return SF_OK;
  cudaEvent_t e;
  CK(cudaEventCreate(&e));
  evs->push_back(e);
  CK(cudaEventRecord(e, s));
  return SF_OK;
}

// The first part of an execute: the pack on `s`, then the buckets, fanned out over the
// auxiliary streams so that their tails overlap (bucket u on stream (u + soff) mod kAux;
// also a single bucket with `fan_one`).  `used` collects the auxiliary streams launched on.
// With `evs`, everything runs in order on `s` with an event after each stage.
int plan_launch_buckets(sf_plan* P, cudaStream_t s, std::vector<cudaEvent_t>* evs, int soff,
                        bool fan_one, bool* used) {
  sf_context* ctx = P->ctx;
  uint64_t launches = 0;
  int mrc;
  if ((mrc = mark_stage(evs, s))) return mrc;
  CK(cudaMemsetAsync(P->d_counters.p, 0, P->buckets.size() * 4 + 4, s));
  {
    const size_t nseq = P->seq_boff.size();
    sfk::PackLaunch pl;
    pl.bytes = plan_dev_bytes(P);
    pl.byte_off = P->d_seq.as<uint64_t>();
    pl.word_off = reinterpret_cast<const uint64_t*>(P->d_seq.as<uint8_t>() + nseq * 8);
    pl.len = reinterpret_cast<const uint32_t*>(P->d_seq.as<uint8_t>() + nseq * 16);
    pl.nseq = (uint32_t)nseq;
    pl.pool = P->d_pool.as<uint32_t>();
    pl.store = P->store ? P->store->words.as<uint32_t>() : nullptr;
    CK(sfk::launch_pack(pl, s));
    launches += nseq ? 1 : 0;
  }
  if ((mrc = mark_stage(evs, s))) return mrc;
  const int nb = (int)P->buckets.size();
  const bool fan = !evs && (nb > 1 || (fan_one && nb == 1));
  bool mine[sf_context::kAux] = {};
  if (fan) CK(cudaEventRecord(ctx->fork, s));
  for (int q = 0; q < nb; ++q) {
    const Bucket& b = P->buckets[q];
    cudaStream_t bs = s;
    if (fan) {
      const int si = (b.stream + soff) % sf_context::kAux;
      bs = ctx->aux[si];
      if (!mine[si]) CK(cudaStreamWaitEvent(bs, ctx->fork, 0));
      mine[si] = used[si] = true;
    }
    uint32_t* counter = P->d_counters.as<uint32_t>() + q;
    const uint32_t* order = P->d_order.as<uint32_t>() + b.first;
    if (b.kind == PK_MYERS) {
      sfk::MyersLaunch ml;
      ml.jobs = P->d_mjobs.as<MJob>();
      ml.order = order;
      ml.njobs = b.count;
      ml.counter = counter;
      ml.pool = P->d_pool.as<uint32_t>();
      ml.out = P->d_mout.as<uint32_t>();
      ml.lanes = b.lanes;
      CK(sfk::launch_myers(b.c, ml, b.grid, b.block, bs));
    } else {
      sfk::AffLaunch al;
      al.jobs = P->d_djobs.as<DJob>();
      al.params = P->d_params.as<DParams>();
      al.order = order;
      al.njobs = b.count;
      al.counter = counter;
      al.pool = P->d_pool.as<uint32_t>();
      al.bytes = plan_dev_bytes(P);
      al.out = P->d_res.as<DRes>();
      al.tb = P->d_tb.as<uint32_t>();
      al.scratch = P->d_scratch.as<int32_t>() + b.scratch_off;
      al.scratch_cells = P->scratch_cells;
      al.tjobs = P->d_tjobs.as<TJob>();
      al.ops = P->d_ops.as<uint32_t>();
      al.tres = P->d_tres.as<TRes>();
      al.chains = P->d_chains.as<DChain>();
      al.links = P->d_links.as<DLink>();
      al.want = P->d_want.as<uint32_t>();
      al.snap = P->d_snap.as<uint32_t>();
      if (b.kind == PK_CHAIN16)
        CK(sfk::launch_affine16_chain(b.c, al, b.grid, b.block, bs));
      else if (b.kind == PK_AFFINE16 && b.lanes == 16)
        CK(sfk::launch_affine16h(b.c, b.tb, al, b.grid, b.block, bs));
      else if (b.kind == PK_AFFINE16)
        CK(sfk::launch_affine16(b.c, b.tb, al, b.grid, b.block, bs));
      else
        CK(sfk::launch_affine(b.c, b.wide, b.tb, b.kind == PK_LOCAL, al, b.grid, b.block, bs));
    }
    launches++;
    if ((mrc = mark_stage(evs, s))) return mrc;
  }
  P->launches = launches;
  return SF_OK;
}

// The auxiliary streams in `used` joined back into `s`.
int join_aux(sf_context* ctx, cudaStream_t s, const bool* used) {
  for (int i = 0; i < sf_context::kAux; ++i) {
    if (!used[i]) continue;
    CK(cudaEventRecord(ctx->join[i], ctx->aux[i]));
    CK(cudaStreamWaitEvent(s, ctx->join[i], 0));
  }
  return SF_OK;
}

// The last part of an execute, after its buckets: the passes walked their own paths
// (sf_walk.cuh); the CIGARs are compacted.
int plan_launch_compact(sf_plan* P, cudaStream_t s, std::vector<cudaEvent_t>* evs) {
  if (P->n_walk) {
    CK(sfk::launch_compact(P->d_tres.as<TRes>(), P->d_tjobs.as<TJob>(), P->d_wlist.as<uint32_t>(),
                           P->n_walk, P->d_offs.as<uint64_t>(), P->d_ops.as<uint32_t>(),
                           P->d_opsc.as<uint32_t>(), P->d_total.as<uint64_t>(), s));
    P->launches += 2;
  }
  return mark_stage(evs, s);
}

// Launches one execute on `s`.  With `evs`, everything runs in order on `s` with an event
// recorded after each stage (pack, each bucket, walk + compaction) for per-stage timing.
int plan_launch(sf_plan* P, cudaStream_t s, std::vector<cudaEvent_t>* evs = nullptr) {
  bool used[sf_context::kAux] = {};
  int rc;
  if ((rc = plan_launch_buckets(P, s, evs, 0, false, used))) return rc;
  if ((rc = join_aux(P->ctx, s, used))) return rc;
  return plan_launch_compact(P, s, evs);
}

int plan_execute(sf_plan* P, bool use_graph) {
  sf_context* ctx = P->ctx;
  CK(cudaSetDevice(ctx->dev));
  if (use_graph && !P->graph && !P->graph_tried) {
    P->graph_tried = true;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(ctx->s, cudaStreamCaptureModeThreadLocal));
    int rc = plan_launch(P, ctx->s);
    cudaError_t e = cudaStreamEndCapture(ctx->s, &g);
    if (rc != SF_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return fail(SF_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&P->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      P->graph = nullptr;
      return fail(SF_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
  }
  if (use_graph && P->graph) {
    CK(cudaGraphLaunch(P->graph, ctx->s));
    return SF_OK;
  }
  return plan_launch(P, ctx->s);
}

int plan_upload_from(sf_plan* P, const uint8_t* pool) {
  sf_context* ctx = P->ctx;
  CK(cudaSetDevice(ctx->dev));
  if (!P->pool_bytes) return SF_OK;
  if (!pool) return fail(SF_ERR_INVALID, "null pool");
  cudaPointerAttributes at{};
  cudaError_t e = cudaPointerGetAttributes(&at, pool);
  if (e != cudaSuccess) (void)cudaGetLastError();
  CK(cudaMemcpyAsync(P->d_bytes.p, pool, P->pool_bytes, cudaMemcpyHostToDevice, ctx->s));
  return SF_OK;
}

// Results -> host pinned buffers (and compacted ops), then the caller's arrays.
int plan_fetch(sf_plan* P) {
  sf_context* ctx = P->ctx;
  int rc;
  if ((rc = P->h_res.ensure(P->n_aff * sizeof(DRes) + 64))) return rc;
  if ((rc = P->h_mout.ensure(P->n_my * 4 + 64))) return rc;
  if ((rc = P->h_tres.ensure(P->n_aff * sizeof(TRes) + 64))) return rc;
  if (P->n_aff) CK(cudaMemcpyAsync(P->h_res.p, P->d_res.p, P->n_aff * sizeof(DRes), cudaMemcpyDeviceToHost, ctx->s));
  if (P->n_my) CK(cudaMemcpyAsync(P->h_mout.p, P->d_mout.p, P->n_my * 4, cudaMemcpyDeviceToHost, ctx->s));
  if (P->n_walk) {
    CK(cudaMemcpyAsync(P->h_tres.p, P->d_tres.p, P->n_aff * sizeof(TRes), cudaMemcpyDeviceToHost, ctx->s));
    if ((rc = P->h_total.ensure(64))) return rc;
    CK(cudaMemcpyAsync(P->h_total.p, P->d_total.p, 8, cudaMemcpyDeviceToHost, ctx->s));
  }
  CK(cudaStreamSynchronize(ctx->s));
  return SF_OK;
}

struct Fetched {
  uint64_t ops_total = 0;
};

int plan_fetch_ops(sf_plan* P, uint64_t& total) {
  sf_context* ctx = P->ctx;
  total = 0;
  if (!P->n_walk) return SF_OK;
  CK(cudaMemcpy(&total, P->d_total.p, 8, cudaMemcpyDeviceToHost));
  int rc;
  if ((rc = P->h_ops.ensure(total * 4 + 64))) return rc;
  if (total) CK(cudaMemcpyAsync(P->h_ops.p, P->d_opsc.p, total * 4, cudaMemcpyDeviceToHost, ctx->s));
  CK(cudaStreamSynchronize(ctx->s));
  return SF_OK;
}

// ---- one-call entry points --------------------------------------------------------------

struct OneCall {
  int device = -1;
  sf_plan plan;
  std::vector<uint8_t> dummy;
  ~OneCall() { plan.ctx = nullptr; }
};

thread_local std::unique_ptr<sf_context> t_ctx;
thread_local std::unique_ptr<OneCall> t_one;
thread_local int t_device = -1;

int one_ctx(sf_plan*& P) {
  if (!t_ctx) {
    int dev = t_device;
    if (dev < 0) {
      cudaError_t e = cudaGetDevice(&dev);
      if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return fail(SF_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
      }
    }
    sf_context* c = nullptr;
    int rc = make_context(dev, &c);
    if (rc) return rc;
    t_ctx.reset(c);
    t_one.reset(new OneCall);
    t_one->plan.ctx = c;
  }
  P = &t_one->plan;
  return SF_OK;
}

// Sequences of one call: gathered into pinned staging as one pool.
struct Gather {
  std::vector<std::pair<const uint8_t*, uint64_t>> parts;
  uint64_t bytes = 0;
  uint64_t add(const uint8_t* p, uint64_t n) {
    const uint64_t off = bytes;
    parts.push_back({p, n});
    bytes += n;
    return off;
  }
};

// Runs the passes of one call; res/mout/tres filled per pass (by pass index).
int run_passes(std::vector<Pass>& passes, const Gather& g, std::vector<DRes>* res,
               std::vector<uint32_t>* mout, std::vector<TRes>* tres, std::vector<uint32_t>* ops,
               std::vector<uint64_t>* ops_at) {
  sf_plan* P = nullptr;
  int rc = one_ctx(P);
  if (rc) return rc;
  for (const Pass& p : passes)
    if (p.m >= 0x7fffffffu || p.n >= 0x7fffffffu) return fail(SF_ERR_TOO_LONG, "sequence too long");
  P->passes = passes;
  P->pool_bytes = g.bytes;
  if ((rc = plan_build(P))) return rc;
  // Pool: gather into pinned staging, then one copy.
  if (g.bytes) {
    // The staging is the build's too: its descriptor copies end first.
    if ((rc = stage_wait(P))) return rc;
    if ((rc = P->h_stage.ensure(g.bytes))) return rc;
    uint8_t* h = P->h_stage.as<uint8_t>();
    uint64_t at = 0;
    for (auto& pr : g.parts) {
      if (pr.second) std::memcpy(h + at, pr.first, pr.second);
      at += pr.second;
    }
    CK(cudaMemcpyAsync(P->d_bytes.p, h, g.bytes, cudaMemcpyHostToDevice, P->ctx->s));
    if ((rc = stage_done(P))) return rc;
  }
  if ((rc = plan_execute(P, false))) return rc;
  if ((rc = plan_fetch(P))) return rc;
  uint64_t total = 0;
  if ((rc = plan_fetch_ops(P, total))) return rc;
  const size_t np = passes.size();
  if (res) res->assign(np, DRes{});
  if (mout) mout->assign(np, 0);
  if (tres) tres->assign(np, TRes{});
  if (ops_at) ops_at->assign(np, 0);
  std::vector<uint64_t> offs;
  if (ops && P->n_walk) {
    // Compacted order = walk-list order; recompute offsets on the host.
    offs.assign(P->n_aff, 0);
    uint64_t acc = 0;
    const TRes* tr = P->h_tres.as<TRes>();
    for (size_t q = 0; q < np; ++q) {
      const Pass& p = passes[q];
      if (p.kind == PK_MYERS || !p.want_cigar) continue;
      const uint32_t s = P->slot[q];
      offs[s] = acc;
      if (tr[s].status == 0) acc += tr[s].n_ops;
    }
    ops->assign(P->h_ops.as<uint32_t>(), P->h_ops.as<uint32_t>() + total);
  }
  for (size_t q = 0; q < np; ++q) {
    const uint32_t s = P->slot[q];
    if (passes[q].kind == PK_MYERS) {
      if (mout) (*mout)[q] = P->h_mout.as<uint32_t>()[s];
    } else {
      if (res) (*res)[q] = P->h_res.as<DRes>()[s];
      if (tres && passes[q].want_cigar) (*tres)[q] = P->h_tres.as<TRes>()[s];
      if (ops_at && passes[q].want_cigar && !offs.empty()) (*ops_at)[q] = offs[s];
    }
  }
  return SF_OK;
}

void count_dp(const std::vector<Pass>& passes, const std::vector<DRes>& res) {
  for (size_t q = 0; q < passes.size(); ++q)
    if (passes[q].kind == PK_AFFINE) {
      g_dp_cells += res[q].cells;
      g_dp_rows += res[q].rows;
    }
}

bool ok_mode(int mode) { return mode == SF_INFIX || mode == SF_PREFIX || mode == SF_GLOBAL; }
bool ok_sc(const sf_affine_t* sc) {
  // align.rs:2504 debug_assert!(open >= 0 && ext >= 0).
  return sc && sc->open >= 0 && sc->ext >= 0;
}

Pass affine_pass(uint64_t p_off, uint64_t m, uint64_t t_off, uint64_t n, int mode,
                 const sf_affine_t* sc, uint64_t band) {
  Pass p;
  p.kind = PK_AFFINE;
  p.mode = (uint8_t)mode;
  p.p_off = p_off;
  p.t_off = t_off;
  p.m = (uint32_t)m;
  p.n = (uint32_t)n;
  p.band = band;
  p.geom = n;
  p.sc = *sc;
  return p;
}

// align.rs:2229-2243: passes [q0, q0 + count) of `ps` hold one pattern against sorted texts
// with one mode, band, clip and geometry rule.  Marks them as one sorted call and sets, per
// pass, the rows it shares with the previous text's pass (rows i read text bases below
// i + above, so rows with i + above <= the common prefix agree; the last row is always
// computed), the common prefix and whether both bands have the same shape.  text(u) gives
// pass u's text bytes.  Unbanded passes share nothing.
template <class F>
void link_sorted(std::vector<Pass>& ps, size_t q0, size_t count, F text) {
  if (count < 2) return;
  if (ps[q0].mode == SF_INFIX || ps[q0].band == SF_NOLIMIT) return;
  auto shape = [](const Pass& p) {
    return std::make_pair(usat_add(p.band, usat_sub(p.m, p.geom)),
                          usat_add(p.band, usat_sub(p.geom, p.m)));
  };
  ps[q0].chain = (uint32_t)count;
  for (size_t k = 1; k < count; ++k) {
    Pass& p = ps[q0 + k];
    const Pass& pp = ps[q0 + k - 1];
    const uint8_t* a = text(q0 + k);
    const uint8_t* b = text(q0 + k - 1);
    const uint64_t lim = std::min<uint64_t>(p.n, pp.n);
    uint64_t l = 0;
    while (l < lim && a[l] == b[l]) ++l;
    p.lcp = (uint32_t)l;
    p.same_shape = shape(p) == shape(pp);
    p.resume = p.same_shape
                   ? (uint32_t)std::min<uint64_t>(usat_sub(l, shape(p).second), usat_sub(p.m, 1))
                   : 0;
  }
}

// align.rs:2248-2310 with 2571-2576: the DP work the reference counts for one sorted call,
// from its passes' whole-pass results res(u) (every result equals the separate pass's).  A
// pass takes the previous text's result when that pass read nothing the two texts differ in
// (with clip) or stopped within the rows they share, and counts nothing; else it counts the
// rows after its resume row.
template <class R>
void count_sorted(const std::vector<Pass>& ps, size_t q0, size_t count, R res) {
  const bool full = count && (ps[q0].mode == SF_INFIX || ps[q0].band == SF_NOLIMIT);
  size_t src = q0;  // the pass whose result the previous text took
  for (size_t k = 0; k < count; ++k) {
    const Pass& p = ps[q0 + k];
    if (k > 0) {
      const DRes& o = res(src);
      const uint32_t tr = o.text_read;
      const bool same = p.clip && !full && p.same_shape && tr < ps[q0 + k - 1].n && tr < p.n &&
                        tr <= p.lcp;
      if (same || (p.resume > 0 && o.last_row <= p.resume)) continue;
    }
    src = q0 + k;
    const DRes& d = res(src);
    uint32_t flags = 0;
    const DJob j = make_djob(p, flags);
    g_dp_rows += d.rows - p.resume;
    g_dp_cells += d.cells - band_cells(p.resume, j.below, j.above, p.n);
  }
}

// One job's pass, or the job's error (recorded for the calling thread).
int job_to_pass(const sf_job_t& j, const sf_affine_t* scores, uint32_t n_scores,
                uint64_t pool_bytes, const sf_store* store, Pass& p) {
  p = Pass{};
  p.p_off = j.p_off;
  p.t_off = j.t_off;
  p.m = j.m;
  p.n = j.n;
  if (j.m >= 0x7fffffffu || j.n >= 0x7fffffffu) return fail(SF_ERR_TOO_LONG, "sequence too long");
  if (j.text_src > SF_TEXT_STORE_REV) return fail(SF_ERR_INVALID, "bad text source");
  if (j.p_off > pool_bytes || j.m > pool_bytes - j.p_off)
    return fail(SF_ERR_INVALID, "job sequence outside the pool");
  if (j.text_src == SF_TEXT_STORE || j.text_src == SF_TEXT_STORE_REV) {
    if (!store) return fail(SF_ERR_INVALID, "store text but the context uses no store");
    if (j.t_off > store->bases || j.n > store->bases - j.t_off)
      return fail(SF_ERR_INVALID, "text window outside the store");
    p.t_off = kStoreFlag | (j.text_src == SF_TEXT_STORE_REV ? kRevFlag : 0) |
              (j.t_off + kStorePad);
  } else if (j.t_off > pool_bytes || j.n > pool_bytes - j.t_off) {
    return fail(SF_ERR_INVALID, "job sequence outside the pool");
  }
  if (j.kind != SF_JOB_MYERS) {
    if (j.sc_index >= n_scores || !ok_sc(&scores[j.sc_index]))
      return fail(SF_ERR_INVALID, "bad scoring index");
    p.sc = scores[j.sc_index];
  }
  switch (j.kind) {
    case SF_JOB_MYERS:
      if (!ok_mode(j.mode)) return fail(SF_ERR_INVALID, "bad mode");
      p.kind = PK_MYERS;
      p.mode = j.mode;
      p.k = j.k;
      break;
    case SF_JOB_AFFINE:
      if (!ok_mode(j.mode)) return fail(SF_ERR_INVALID, "bad mode");
      p.kind = PK_AFFINE;
      p.mode = j.mode;
      p.band = j.band;
      p.geom = j.n;
      p.want_cigar = j.want_cigar != 0;
      p.tb_kind = 0;
      break;
    case SF_JOB_EXTEND_WINDOW:
      p.kind = PK_AFFINE;
      p.mode = SF_PREFIX;
      p.band = j.band;
      p.geom = std::max<uint64_t>(j.window, j.n);
      p.clip = true;
      p.cell = true;
      p.xdrop = j.xdrop;
      p.end_bonus = j.end_bonus;
      p.want_cigar = j.want_cigar != 0;
      p.tb_kind = 1;
      break;
    case SF_JOB_LOCAL:
      p.kind = PK_LOCAL;
      p.dlo = j.dlo;
      p.dhi = j.dhi;
      p.bonus0 = j.end_bonus;
      p.bonus1 = j.end_bonus2;
      break;
    default:
      return fail(SF_ERR_INVALID, "bad job kind");
  }
  return SF_OK;
}

int jobs_to_passes(const sf_job_t* jobs, uint64_t count, const sf_affine_t* scores,
                          uint32_t n_scores, uint64_t pool_bytes, std::vector<Pass>& ps,
                          const sf_store* store) {
  ps.resize(count);
  // Chunks in parallel; each stops at its first bad job, and the first bad job of all is
  // converted again here, so that its error is the calling thread's.
  constexpr int kMaxThreads = 8;
  uint64_t first_bad[kMaxThreads];
  for (int w = 0; w < kMaxThreads; ++w) first_bad[w] = UINT64_MAX;
  parallel_chunks(count, 2048, kMaxThreads, [&](size_t q0, size_t q1, int w) {
    for (size_t q = q0; q < q1; ++q)
      if (job_to_pass(jobs[q], scores, n_scores, pool_bytes, store, ps[q]) != SF_OK) {
        first_bad[w] = std::min<uint64_t>(first_bad[w], q);
        return;
      }
  });
  uint64_t bad = UINT64_MAX;
  for (int w = 0; w < kMaxThreads; ++w) bad = std::min(bad, first_bad[w]);
  if (bad != UINT64_MAX) {
    Pass p;
    const int rc = job_to_pass(jobs[bad], scores, n_scores, pool_bytes, store, p);
    ps.clear();
    return rc;
  }
  return SF_OK;
}

// Fills `results` from the fetched per-pass records; with `copy_ops`, also copies the CIGARs
// fetched into h_ops to `ops` (sf_plan_download copies them straight from the device).
int plan_results(sf_plan* P, sf_result_t* results, uint32_t* ops, uint64_t ops_cap,
                 uint64_t total, bool copy_ops, uint64_t ops_base) {
  if (total && (!ops || ops_cap < total)) {
    return fail(SF_ERR_CAPACITY, "ops buffer smaller than the CIGARs");
  }
  if (total && copy_ops) std::memcpy(ops, P->h_ops.p, total * 4);
  const DRes* rs = P->h_res.as<DRes>();
  const TRes* tr = P->h_tres.as<TRes>();
  const uint32_t* mo = P->h_mout.as<uint32_t>();
  const size_t np = P->passes.size();
  // Compacted op order = walk-list order = pass order among CIGAR passes: each chunk's ops
  // counted while its results convert, then its passes' offsets.
  constexpr int kT = 8;
  uint64_t ops_of[kT + 1] = {};
  auto has_ops = [](const Pass& p) {
    return p.want_cigar && p.kind != PK_LOCAL && p.kind != PK_MYERS;
  };
  parallel_chunks(np, 2048, kT, [&](size_t q0, size_t q1, int k) {
    uint64_t n_ops = 0;
    for (size_t q = q0; q < q1; ++q) {
      const Pass& p = P->passes[q];
      sf_result_t& o = results[q];
      std::memset(&o, 0, sizeof o);
      const uint32_t s = P->slot[q];
      if (p.kind == PK_MYERS) {
        o.distance = mo[s];
        o.score = 0;
        o.cells = (uint64_t)p.m * p.n;
        continue;
      }
      const DRes& d = rs[s];
      o.distance = SF_NONE;
      o.cells = d.cells;
      o.text_read = d.text_read;
      if (p.kind == PK_LOCAL) {
        o.score = d.score;
      } else if (p.tb_kind == 1) {
        const int32_t whole = sat_add32(d.score, p.end_bonus);
        if (d.clip_best >= whole) {
          o.score = d.clip_best;
          o.pattern_end = d.clip_i;
          o.text_end = d.clip_j;
        } else {
          o.score = whole;
          o.pattern_end = p.m;
          o.text_end = d.score_col;
        }
      } else {
        o.score = d.score;
        o.pattern_end = p.m;
        o.text_end = d.score_col;
      }
      if (p.want_cigar && p.kind != PK_LOCAL) {
        const TRes& t = tr[s];
        o.status = t.status;
        o.text_start = t.text_start;
        o.n_ops = t.status == 0 ? t.n_ops : 0;
        n_ops += o.n_ops;
      }
    }
    ops_of[k + 1] = n_ops;
  });
  ops_of[0] = ops_base;
  for (int k = 0; k < kT; ++k) ops_of[k + 1] += ops_of[k];
  parallel_chunks(np, 2048, kT, [&](size_t q0, size_t q1, int k) {
    uint64_t acc = ops_of[k];
    for (size_t q = q0; q < q1; ++q) {
      if (!has_ops(P->passes[q])) continue;
      results[q].cigar_off = acc;
      acc += results[q].n_ops;
    }
  });
  return SF_OK;
}

uint64_t plan_bytes_held(const sf_plan* P) {
  const DevBuf* bufs[] = {&P->d_bytes, &P->d_pool, &P->d_seq, &P->d_djobs, &P->d_params,
                          &P->d_res, &P->d_mjobs, &P->d_mout, &P->d_tjobs, &P->d_tres,
                          &P->d_tb, &P->d_ops, &P->d_opsc, &P->d_offs, &P->d_order,
                          &P->d_counters, &P->d_wlist, &P->d_cls, &P->d_scratch, &P->d_total};
  uint64_t b = 0;
  for (const DevBuf* d : bufs) b += d->cap;
  return b;
}

uint64_t plan_bytes_estimate(const std::vector<Pass>& passes, uint64_t pool_bytes) {
  // Mirrors plan_build's sizes: byte pool, packed pool, descriptors, results, traceback
  // arena, CIGAR slots (twice: slots and compacted), wide-row scratch; DevBuf keeps 25%
  // headroom on each.
  uint64_t b = pool_bytes + 256 * 4 + 4096;
  uint64_t scratch = 0;
  const bool use16 = allow16();
  for (const Pass& p : passes) {
    b += (uint64_t)(p.m + p.n + 34) / 4 + 40 + 200;
    if (p.kind == PK_MYERS) continue;
    uint32_t flags = 0;
    DJob j = make_djob(p, flags);
    const int64_t wmax = band_wmax(j, flags);
    int c = 4;
    bool wide = false;
    PassKind kind = PK_AFFINE;
    int ln = 32;
    classify_affine(p, flags, wmax, use16, kind, c, wide, ln);
    if (p.want_cigar && p.kind != PK_LOCAL) {
      b += (uint64_t)p.m * tb_row_words(c, wide ? wide_chunks(c, wmax) : 1) * 4;
      b += 2 * ((uint64_t)p.m + p.n + 2) * 4;
    }
    if (wide) scratch = std::max<uint64_t>(scratch, (uint64_t)wide_chunks(c, wmax) * 32 * c);
  }
  // Wide buckets (with and without traceback): up to 2 blocks/SM x 4 warps x 4 rows each.
  b += scratch * 4 * 2 * 304 * 4 * 4 * 2;
  return b + b / 4;
}

}  // namespace sfe

int sf_internal_set_error(int code, const char* msg) { return fail(code, msg); }

// ---- C ABI ------------------------------------------------------------------------------

extern "C" {

const char* sf_last_error(void) { return g_err.c_str(); }

const char* sf_version(void) {
  return "spearfish_gb300 sf_align 0.1 (sm_103a; affine C={4,6,8,9,10,11,12,14,16,20,24,28,32,40,48}+wide; "
         "myers B={1,2,3,4,6,8,12,16})";
}

int sf_set_device(int device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    (void)cudaGetLastError();
    return fail(SF_ERR_INVALID, "no such device");
  }
  if (t_device != device) {
    t_one.reset();
    t_ctx.reset();
    t_device = device;
  }
  return SF_OK;
}

int sf_context_create(int device, sf_context** out) {
  if (!out) return fail(SF_ERR_INVALID, "null out");
  return make_context(device, out);
}

void sf_context_destroy(sf_context* ctx) { delete ctx; }

int sf_distance(const uint8_t* pattern, uint64_t m, const uint8_t* text, uint64_t n, int mode,
                uint32_t k, uint32_t* out) {
  if (!out || !ok_mode(mode) || (m && !pattern) || (n && !text)) return fail(SF_ERR_INVALID, "bad argument");
  Gather g;
  Pass p;
  p.kind = PK_MYERS;
  p.mode = (uint8_t)mode;
  p.k = k;
  p.p_off = g.add(pattern, m);
  p.t_off = g.add(text, n);
  p.m = (uint32_t)m;
  p.n = (uint32_t)n;
  std::vector<Pass> ps{p};
  std::vector<uint32_t> mo;
  int rc = run_passes(ps, g, nullptr, &mo, nullptr, nullptr, nullptr);
  if (rc) return rc;
  *out = mo[0];
  return SF_OK;
}

int sf_infix_distance(const uint8_t* pattern, uint64_t m, const uint8_t* text, uint64_t n,
                      uint32_t* out) {
  return sf_distance(pattern, m, text, n, SF_INFIX, SF_NONE, out);
}

int sf_batch_distances(const uint8_t* pattern, uint64_t m, const uint8_t* const* texts,
                       const uint64_t* lens, uint64_t count, int mode, uint32_t k,
                       uint32_t* out) {
  if (!ok_mode(mode) || (count && (!texts || !lens || !out)) || (m && !pattern))
    return fail(SF_ERR_INVALID, "bad argument");
  if (!count) return SF_OK;
  Gather g;
  const uint64_t po = g.add(pattern, m);
  std::vector<Pass> ps;
  ps.reserve(count);
  for (uint64_t q = 0; q < count; ++q) {
    if (lens[q] && !texts[q]) return fail(SF_ERR_INVALID, "null text");
    Pass p;
    p.kind = PK_MYERS;
    p.mode = (uint8_t)mode;
    p.k = k;
    p.p_off = po;
    p.m = (uint32_t)m;
    p.t_off = g.add(texts[q], lens[q]);
    p.n = (uint32_t)lens[q];
    ps.push_back(p);
  }
  std::vector<uint32_t> mo;
  int rc = run_passes(ps, g, nullptr, &mo, nullptr, nullptr, nullptr);
  if (rc) return rc;
  std::memcpy(out, mo.data(), count * 4);
  return SF_OK;
}

int sf_affine(const uint8_t* pattern, uint64_t m, const uint8_t* text, uint64_t n, int mode,
              const sf_affine_t* sc, uint64_t band, int32_t* out) {
  if (!out || !ok_mode(mode) || !ok_sc(sc) || (m && !pattern) || (n && !text))
    return fail(SF_ERR_INVALID, "bad argument");
  Gather g;
  const uint64_t po = g.add(pattern, m), to = g.add(text, n);
  std::vector<Pass> ps{affine_pass(po, m, to, n, mode, sc, band)};
  std::vector<DRes> r;
  int rc = run_passes(ps, g, &r, nullptr, nullptr, nullptr, nullptr);
  if (rc) return rc;
  count_dp(ps, r);
  *out = r[0].score;
  return SF_OK;
}

int sf_affine_extend(const uint8_t* pattern, uint64_t m, const uint8_t* text, uint64_t n,
                     const sf_affine_t* sc, uint64_t band, int32_t end_bonus, int32_t xdrop,
                     int32_t* out) {
  if (!out || !ok_sc(sc) || (m && !pattern) || (n && !text)) return fail(SF_ERR_INVALID, "bad argument");
  Gather g;
  const uint64_t po = g.add(pattern, m), to = g.add(text, n);
  Pass p = affine_pass(po, m, to, n, SF_PREFIX, sc, band);
  p.clip = true;
  p.xdrop = xdrop;
  p.cell = false;
  std::vector<Pass> ps{p};
  std::vector<DRes> r;
  int rc = run_passes(ps, g, &r, nullptr, nullptr, nullptr, nullptr);
  if (rc) return rc;
  count_dp(ps, r);
  // align.rs:728
  *out = std::max(r[0].clip_best, sat_add32(r[0].score, end_bonus));
  return SF_OK;
}

int sf_affine_extend_window(const uint8_t* pattern, uint64_t m, const uint8_t* text, uint64_t n,
                            uint64_t window, const sf_affine_t* sc, uint64_t band,
                            int32_t end_bonus, int32_t xdrop, sf_extend_t* out) {
  if (!out || !ok_sc(sc) || (m && !pattern) || (n && !text)) return fail(SF_ERR_INVALID, "bad argument");
  Gather g;
  const uint64_t po = g.add(pattern, m), to = g.add(text, n);
  Pass p = affine_pass(po, m, to, n, SF_PREFIX, sc, band);
  p.clip = true;
  p.cell = true;
  p.xdrop = xdrop;
  p.geom = std::max<uint64_t>(window, n);
  std::vector<Pass> ps{p};
  std::vector<DRes> r;
  int rc = run_passes(ps, g, &r, nullptr, nullptr, nullptr, nullptr);
  if (rc) return rc;
  count_dp(ps, r);
  // align.rs:975-981
  const DRes& d = r[0];
  const int32_t whole = sat_add32(d.score, end_bonus);
  std::memset(out, 0, sizeof *out);
  if (d.clip_best >= whole) {
    out->score = d.clip_best;
    out->pattern_bases = d.clip_i;
    out->text_bases = d.clip_j;
  } else {
    out->score = whole;
    out->pattern_bases = m;
    out->text_bases = d.score_col;
  }
  out->text_read = d.text_read;
  return SF_OK;
}

int sf_affine_sorted(const uint8_t* pattern, uint64_t m, const uint8_t* const* texts,
                     const uint64_t* lens, uint64_t count, int mode, const sf_affine_t* sc,
                     uint64_t band, int32_t* out) {
  if (!ok_mode(mode) || !ok_sc(sc) || (count && (!texts || !lens || !out)) || (m && !pattern))
    return fail(SF_ERR_INVALID, "bad argument");
  if (!count) return SF_OK;
  Gather g;
  const uint64_t po = g.add(pattern, m);
  std::vector<Pass> ps;
  for (uint64_t q = 0; q < count; ++q) {
    const uint64_t to = g.add(texts[q], lens[q]);
    ps.push_back(affine_pass(po, m, to, lens[q], mode, sc, band));
  }
  link_sorted(ps, 0, count, [&](size_t u) { return texts[u]; });
  std::vector<DRes> r;
  int rc = run_passes(ps, g, &r, nullptr, nullptr, nullptr, nullptr);
  if (rc) return rc;
  count_sorted(ps, 0, count, [&](size_t u) -> const DRes& { return r[u]; });
  for (uint64_t q = 0; q < count; ++q) out[q] = r[q].score;
  return SF_OK;
}

int sf_affine_extend_sorted_cut_bonus(const uint8_t* pattern, uint64_t m,
                                      const uint8_t* const* texts, const uint64_t* lens,
                                      uint64_t count, const sf_affine_t* sc, uint64_t band,
                                      int32_t end_bonus, int32_t xdrop, int diagonal,
                                      uint64_t window, uint64_t cut, int track_cut,
                                      int bonus_within_cut, sf_cut_t* out) {
  if (!ok_sc(sc) || (count && (!texts || !lens || !out)) || (m && !pattern))
    return fail(SF_ERR_INVALID, "bad argument");
  if (!count) return SF_OK;
  Gather g;
  const uint64_t po = g.add(pattern, m);
  std::vector<Pass> ps;
  for (uint64_t q = 0; q < count; ++q) {
    const uint64_t n = lens[q];
    const uint64_t to = g.add(texts[q], n);
    Pass p = affine_pass(po, m, to, n, SF_PREFIX, sc, band);
    // align.rs:917-928
    p.geom = diagonal ? std::min<uint64_t>(m, n) : std::max<uint64_t>(n, window);
    p.clip = true;
    p.xdrop = xdrop;
    p.cell = track_cut && cut != SF_NOLIMIT;
    p.cut = cut;
    ps.push_back(p);
  }
  link_sorted(ps, 0, count, [&](size_t u) { return texts[u]; });
  std::vector<DRes> r;
  int rc = run_passes(ps, g, &r, nullptr, nullptr, nullptr, nullptr);
  if (rc) return rc;
  count_sorted(ps, 0, count, [&](size_t u) -> const DRes& { return r[u]; });
  for (uint64_t q = 0; q < count; ++q) {
    // align.rs:929-948
    const DRes& d = r[q];
    const int32_t end = (bonus_within_cut && cut != SF_NOLIMIT)
                            ? std::max(d.score, sat_add32(d.cut_score, end_bonus))
                            : sat_add32(d.score, end_bonus);
    const int32_t whole = std::max(d.clip_best, end);
    out[q].whole = whole;
    out[q].cols = d.clip_best >= end ? d.clip_j : d.score_col;
    out[q].cut = cut == SF_NOLIMIT ? whole : std::max(d.cut_best, sat_add32(d.cut_score, end_bonus));
  }
  return SF_OK;
}

int sf_affine_extend_sorted_cut(const uint8_t* pattern, uint64_t m, const uint8_t* const* texts,
                                const uint64_t* lens, uint64_t count, const sf_affine_t* sc,
                                uint64_t band, int32_t end_bonus, int32_t xdrop, int diagonal,
                                uint64_t window, uint64_t cut, sf_cut_t* out) {
  // align.rs:891-900
  return sf_affine_extend_sorted_cut_bonus(pattern, m, texts, lens, count, sc, band, end_bonus,
                                           xdrop, diagonal, window, cut, 1, 0, out);
}

int sf_local_band_ends(const uint8_t* read, uint64_t m, const uint8_t* text, uint64_t n,
                       const sf_affine_t* sc, int64_t dlo, int64_t dhi, int32_t bonus_start,
                       int32_t bonus_end, int32_t* out) {
  if (!out || !ok_sc(sc) || (m && !read) || (n && !text)) return fail(SF_ERR_INVALID, "bad argument");
  if (m == 0 || dlo > dhi) {  // align.rs:791-793
    *out = 0;
    return SF_OK;
  }
  Gather g;
  Pass p;
  p.kind = PK_LOCAL;
  p.p_off = g.add(read, m);
  p.t_off = g.add(text, n);
  p.m = (uint32_t)m;
  p.n = (uint32_t)n;
  p.dlo = dlo;
  p.dhi = dhi;
  p.bonus0 = bonus_start;
  p.bonus1 = bonus_end;
  p.sc = *sc;
  std::vector<Pass> ps{p};
  std::vector<DRes> r;
  int rc = run_passes(ps, g, &r, nullptr, nullptr, nullptr, nullptr);
  if (rc) return rc;
  *out = r[0].score;
  return SF_OK;
}

int sf_local_band(const uint8_t* read, uint64_t m, const uint8_t* text, uint64_t n,
                  const sf_affine_t* sc, int64_t dlo, int64_t dhi, int32_t end_bonus,
                  int32_t* out) {
  return sf_local_band_ends(read, m, text, n, sc, dlo, dhi, end_bonus, end_bonus, out);
}

void sf_dp_work(uint64_t* cells, uint64_t* rows) {
  if (cells) *cells = g_dp_cells;
  if (rows) *rows = g_dp_rows;
}

static int cigar_call(Pass p, const Gather& g, uint32_t* ops, uint64_t cap, sf_cigar_t* out,
                      int32_t score_adjust_bonus) {
  (void)score_adjust_bonus;
  p.want_cigar = true;
  std::vector<Pass> ps{p};
  std::vector<DRes> r;
  std::vector<TRes> t;
  std::vector<uint32_t> o;
  std::vector<uint64_t> at;
  int rc = run_passes(ps, g, &r, nullptr, &t, &o, &at);
  if (rc) return rc;
  count_dp(ps, r);
  std::memset(out, 0, sizeof *out);
  out->score = t[0].score;
  out->status = t[0].status;
  out->pattern_end = t[0].end_i;
  out->text_start = t[0].text_start;
  out->text_end = t[0].end_j;
  out->n_ops = t[0].n_ops;
  if (t[0].status == 0) {
    if (t[0].n_ops > cap) {
      out->status = -1;
      return fail(SF_ERR_CAPACITY, "CIGAR longer than the ops buffer");
    }
    if (t[0].n_ops) std::memcpy(ops, o.data() + at[0], t[0].n_ops * 4);
  }
  return SF_OK;
}

int sf_affine_cigar(const uint8_t* pattern, uint64_t m, const uint8_t* text, uint64_t n,
                    int mode, const sf_affine_t* sc, uint64_t band, uint32_t* ops, uint64_t cap,
                    sf_cigar_t* out) {
  if (!out || !ok_mode(mode) || !ok_sc(sc) || (m && !pattern) || (n && !text) || (cap && !ops))
    return fail(SF_ERR_INVALID, "bad argument");
  Gather g;
  const uint64_t po = g.add(pattern, m), to = g.add(text, n);
  Pass p = affine_pass(po, m, to, n, mode, sc, band);
  p.tb_kind = 0;
  return cigar_call(p, g, ops, cap, out, 0);
}

int sf_affine_extend_window_cigar(const uint8_t* pattern, uint64_t m, const uint8_t* text,
                                  uint64_t n, uint64_t window, const sf_affine_t* sc,
                                  uint64_t band, int32_t end_bonus, int32_t xdrop, uint32_t* ops,
                                  uint64_t cap, sf_cigar_t* out) {
  if (!out || !ok_sc(sc) || (m && !pattern) || (n && !text) || (cap && !ops))
    return fail(SF_ERR_INVALID, "bad argument");
  Gather g;
  const uint64_t po = g.add(pattern, m), to = g.add(text, n);
  Pass p = affine_pass(po, m, to, n, SF_PREFIX, sc, band);
  p.clip = true;
  p.cell = true;
  p.xdrop = xdrop;
  p.geom = std::max<uint64_t>(window, n);
  p.tb_kind = 1;
  p.end_bonus = end_bonus;
  return cigar_call(p, g, ops, cap, out, end_bonus);
}

// ---- plans ------------------------------------------------------------------------------

int sf_plan_create(sf_context* ctx, const sf_job_t* jobs, uint64_t count, const sf_affine_t* scores,
                   uint32_t n_scores, uint64_t pool_bytes, sf_plan** out) {
  if (!ctx || !out || (count && !jobs)) return fail(SF_ERR_INVALID, "bad argument");
  std::unique_ptr<sf_plan> P(new sf_plan);
  P->ctx = ctx;
  P->pool_bytes = pool_bytes;
  int rc = jobs_to_passes(jobs, count, scores, n_scores, pool_bytes, P->passes, ctx->store);
  if (rc) return rc;
  if ((rc = plan_build(P.get()))) return rc;
  *out = P.release();
  return SF_OK;
}

void sf_plan_destroy(sf_plan* plan) { delete plan; }

int sf_plan_upload(sf_plan* plan, const uint8_t* pool) {
  if (!plan) return fail(SF_ERR_INVALID, "null plan");
  return plan_upload_from(plan, pool);
}

int sf_plan_execute(sf_plan* plan) {
  if (!plan) return fail(SF_ERR_INVALID, "null plan");
  return plan_execute(plan, true);
}

int sf_plan_sync(sf_plan* plan) {
  if (!plan) return fail(SF_ERR_INVALID, "null plan");
  CK(cudaSetDevice(plan->ctx->dev));
  CK(cudaStreamSynchronize(plan->ctx->s));
  return SF_OK;
}

void* sf_plan_stream(sf_plan* plan) { return plan ? (void*)plan->ctx->s : nullptr; }

uint64_t sf_plan_launches(const sf_plan* plan) { return plan ? plan->launches : 0; }

const char* sf_plan_describe(sf_plan* plan) { return plan ? plan->desc.c_str() : ""; }

int sf_plan_download(sf_plan* P, sf_result_t* results, uint32_t* ops, uint64_t ops_cap,
                     uint64_t* ops_used) {
  if (!P || (!results && !P->passes.empty())) return fail(SF_ERR_INVALID, "bad argument");
  CK(cudaSetDevice(P->ctx->dev));
  int rc = plan_fetch(P);
  if (rc) return rc;
  // The CIGARs go from the device straight into the caller's buffer (a DMA when it is pinned).
  const uint64_t total = P->n_walk ? *P->h_total.as<uint64_t>() : 0;
  if (ops_used) *ops_used = total;
  if (total && (!ops || ops_cap < total)) return fail(SF_ERR_CAPACITY, "ops buffer smaller than the CIGARs");
  if (total) {
    CK(cudaMemcpyAsync(ops, P->d_opsc.p, total * 4, cudaMemcpyDeviceToHost, P->ctx->s));
    CK(cudaStreamSynchronize(P->ctx->s));
  }
  return plan_results(P, results, ops, ops_cap, total, false);
}

// ---- tie-break batching (map/src/lib.rs:851-911 `Mapper::banded`) ------------------------

namespace {

uint32_t sat_add_u32(uint32_t a, uint32_t b) { return a > UINT32_MAX - b ? UINT32_MAX : a + b; }

// A read's texts: which are first occurrences, and each repeat's first occurrence.  The
// reference keys texts by their bytes (lib.rs:858-877); here by an FNV-1a hash, equal
// hashes compared byte by byte.
void dedup_texts(const uint8_t* const* tx, const uint64_t* len, uint64_t count, bool distinct,
                 std::vector<uint32_t>& first_of, std::vector<uint8_t>& is_first) {
  first_of.resize(count);
  is_first.resize(count);
  if (distinct) {
    for (uint64_t q = 0; q < count; ++q) {
      first_of[q] = (uint32_t)q;
      is_first[q] = 1;
    }
    return;
  }
  std::unordered_map<uint64_t, std::vector<uint32_t>> seen;
  for (uint64_t q = 0; q < count; ++q) {
    uint64_t h = 1469598103934665603ull ^ len[q];
    for (uint64_t i = 0; i < len[q]; ++i) {
      h ^= tx[q][i];
      h *= 1099511628211ull;
    }
    auto& v = seen[h];
    int64_t hit = -1;
    for (uint32_t u : v)
      if (len[u] == len[q] && (len[q] == 0 || std::memcmp(tx[u], tx[q], len[q]) == 0)) {
        hit = u;
        break;
      }
    if (hit < 0) {
      v.push_back((uint32_t)q);
      first_of[q] = (uint32_t)q;
      is_first[q] = 1;
    } else {
      first_of[q] = (uint32_t)hit;
      is_first[q] = 0;
    }
  }
}

// lib.rs:880-909: in text order, k = best so far + cap; a first occurrence's distance is
// exact when <= k, else k + 1 (the batch kernel's distances are exact, so the threshold is
// applied here); a repeat takes its first occurrence's value re-capped at the current k.
void banded_finish(uint64_t count, const std::vector<uint32_t>& first_of,
                   const std::vector<uint8_t>& is_first, const uint32_t* dist, uint32_t cap,
                   uint32_t* out) {
  std::vector<uint32_t> val(count, 0);
  uint32_t best = UINT32_MAX;
  for (uint64_t q = 0; q < count; ++q) {
    const uint32_t k = sat_add_u32(best, cap);
    if (!is_first[q]) {
      const uint32_t d = val[first_of[q]];
      out[q] = d <= k ? d : sat_add_u32(k, 1);
      continue;
    }
    const uint32_t d = dist[q] <= k ? dist[q] : sat_add_u32(k, 1);
    best = std::min(best, d);
    val[q] = d;
    out[q] = d;
  }
}

}  // namespace

int sf_banded(const uint8_t* read, uint64_t m, const uint8_t* const* texts, const uint64_t* lens,
              uint64_t count, int mode, uint32_t cap, int distinct, uint32_t* out) {
  if (!ok_mode(mode) || (count && (!texts || !lens || !out)) || (m && !read))
    return fail(SF_ERR_INVALID, "bad argument");
  if (!count) return SF_OK;
  for (uint64_t q = 0; q < count; ++q)
    if (lens[q] && !texts[q]) return fail(SF_ERR_INVALID, "null text");
  std::vector<uint32_t> first_of;
  std::vector<uint8_t> is_first;
  dedup_texts(texts, lens, count, distinct != 0, first_of, is_first);
  Gather g;
  const uint64_t po = g.add(read, m);
  std::vector<Pass> ps;
  std::vector<uint64_t> text_of;
  for (uint64_t q = 0; q < count; ++q) {
    if (!is_first[q]) continue;
    Pass p;
    p.kind = PK_MYERS;
    p.mode = (uint8_t)mode;
    p.k = SF_NONE;
    p.p_off = po;
    p.m = (uint32_t)m;
    p.t_off = g.add(texts[q], lens[q]);
    p.n = (uint32_t)lens[q];
    ps.push_back(p);
    text_of.push_back(q);
  }
  std::vector<uint32_t> mo;
  int rc = run_passes(ps, g, nullptr, &mo, nullptr, nullptr, nullptr);
  if (rc) return rc;
  std::vector<uint32_t> dist(count, 0);
  for (size_t u = 0; u < text_of.size(); ++u) dist[text_of[u]] = mo[u];
  banded_finish(count, first_of, is_first, dist.data(), cap, out);
  return SF_OK;
}

int sf_banded_batch(sf_context* ctx, const uint8_t* pool, uint64_t pool_bytes,
                    const sf_banded_read_t* reads, uint64_t n_reads, const sf_span_t* texts,
                    uint64_t n_texts, uint32_t* out) {
  if (!ctx || (n_reads && !reads) || (n_texts && (!texts || !out)) || (pool_bytes && !pool))
    return fail(SF_ERR_INVALID, "bad argument");
  // Per read: its distinct texts become Myers jobs of the one batch.
  std::vector<std::vector<uint32_t>> first_of(n_reads);
  std::vector<std::vector<uint8_t>> is_first(n_reads);
  std::vector<sf_job_t> jobs;
  std::vector<uint64_t> job_text;  // the text index of each job
  std::vector<const uint8_t*> tp;
  std::vector<uint64_t> tl;
  for (uint64_t r = 0; r < n_reads; ++r) {
    const sf_banded_read_t& R = reads[r];
    if (!ok_mode((int)R.mode)) return fail(SF_ERR_INVALID, "bad mode");
    if (R.first > n_texts || R.count > n_texts - R.first)
      return fail(SF_ERR_INVALID, "read's texts outside the text list");
    if (R.p_off > pool_bytes || R.m > pool_bytes - R.p_off)
      return fail(SF_ERR_INVALID, "read outside the pool");
    tp.resize(R.count);
    tl.resize(R.count);
    for (uint64_t q = 0; q < R.count; ++q) {
      const sf_span_t& t = texts[R.first + q];
      if (t.off > pool_bytes || t.len > pool_bytes - t.off)
        return fail(SF_ERR_INVALID, "text outside the pool");
      tp[q] = pool + t.off;
      tl[q] = t.len;
    }
    dedup_texts(tp.data(), tl.data(), R.count, R.distinct != 0, first_of[r], is_first[r]);
    for (uint64_t q = 0; q < R.count; ++q) {
      if (!is_first[r][q]) continue;
      sf_job_t j{};
      j.kind = SF_JOB_MYERS;
      j.mode = (uint8_t)R.mode;
      j.k = SF_NONE;
      j.band = SF_NOLIMIT;
      j.p_off = R.p_off;
      j.m = R.m;
      j.t_off = texts[R.first + q].off;
      j.n = (uint32_t)texts[R.first + q].len;
      if (texts[R.first + q].len >= 0x7fffffffu) return fail(SF_ERR_TOO_LONG, "sequence too long");
      jobs.push_back(j);
      job_text.push_back(R.first + q);
    }
  }
  std::vector<uint32_t> dist(n_texts, 0);
  if (!jobs.empty()) {
    if (!ctx->cache) {
      ctx->cache.reset(new sf_plan);
      ctx->cache->ctx = ctx;
    }
    sf_plan* P = ctx->cache.get();
    int rc = jobs_to_passes(jobs.data(), jobs.size(), nullptr, 0, pool_bytes, P->passes);
    if (rc) return rc;
    P->pool_bytes = pool_bytes;
    if ((rc = plan_build(P))) return rc;
    if ((rc = plan_upload_from(P, pool))) return rc;
    if ((rc = plan_execute(P, false))) return rc;
    if ((rc = plan_fetch(P))) return rc;
    const uint32_t* mo = P->h_mout.as<uint32_t>();
    for (size_t u = 0; u < jobs.size(); ++u) dist[job_text[u]] = mo[P->slot[u]];
  }
  for (uint64_t r = 0; r < n_reads; ++r)
    banded_finish(reads[r].count, first_of[r], is_first[r], dist.data() + reads[r].first,
                  reads[r].cap, out + reads[r].first);
  return SF_OK;
}

// ---- span-end extensions (map/src/lib.rs:2020-2114 `extend_ends`, `right_reach`) -------

int sf_extend_ends_batch(sf_context* ctx, const uint8_t* pool, uint64_t pool_bytes,
                         const sf_ends_t* e, sf_hit_t* hits, uint64_t n) {
  if (!ctx || !e || (n && !hits) || (pool_bytes && !pool)) return fail(SF_ERR_INVALID, "bad argument");
  if (!ctx->store) return fail(SF_ERR_INVALID, "extensions read their flanks from the store");
  if (e->pad_div == 0 || !ok_sc(&e->sc)) return fail(SF_ERR_INVALID, "bad extension parameters");
  const sf_store* store = ctx->store;
  // lib.rs:2021: the transcript flank searched: the read flank plus pad + flank / pad_div.
  auto window = [&](uint32_t x) { return (uint64_t)x + e->pad + x / e->pad_div; };
  std::vector<Pass> ps;
  std::vector<std::pair<uint64_t, int>> slot;  // (hit, 0 left / 1 right) per pass
  for (uint64_t q = 0; q < n; ++q) {
    const sf_hit_t& h = hits[q];
    if (h.read_off > pool_bytes || h.read_len > pool_bytes - h.read_off)
      return fail(SF_ERR_INVALID, "read outside the pool");
    if (h.tx_start > store->bases || h.tx_len > store->bases - h.tx_start)
      return fail(SF_ERR_INVALID, "transcript outside the store");
    if (h.qstart > h.qend || h.qend > h.read_len || h.tstart > h.tend || h.tend > h.tx_len)
      return fail(SF_ERR_INVALID, "bad hit span");
    Pass p;
    p.kind = PK_AFFINE;
    p.mode = SF_PREFIX;
    p.band = e->band;
    p.clip = true;
    p.cell = true;
    p.xdrop = e->xdrop;
    p.end_bonus = e->end_bonus;
    p.tb_kind = 1;
    p.sc = e->sc;
    if (h.qstart > 0 && h.tstart > 0) {
      // lib.rs:2022-2031: the read prefix and the transcript flank before tstart, backwards.
      const uint64_t w = window(h.qstart);
      const uint64_t lo = h.tstart > w ? h.tstart - w : 0;
      Pass L = p;
      L.p_off = kRevFlag | h.read_off;
      L.m = h.qstart;
      L.t_off = kStoreFlag | kRevFlag | (h.tx_start + lo + kStorePad);
      L.n = (uint32_t)(h.tstart - lo);
      L.geom = std::max<uint64_t>(w, L.n);
      ps.push_back(L);
      slot.push_back({q, 0});
    }
    const uint32_t rest = h.read_len - h.qend;
    if (rest > 0 && h.tend < h.tx_len) {
      // lib.rs:2046-2073: the read suffix and the flank after tend, cut at the transcript's end.
      const uint64_t w = window(rest);
      const uint64_t hi = std::min<uint64_t>(h.tend + w, h.tx_len);
      Pass R = p;
      R.p_off = h.read_off + h.qend;
      R.m = rest;
      R.t_off = kStoreFlag | (h.tx_start + h.tend + kStorePad);
      R.n = (uint32_t)(hi - h.tend);
      R.geom = std::max<uint64_t>(w, R.n);
      ps.push_back(R);
      slot.push_back({q, 1});
    }
  }
  if (ps.empty()) return SF_OK;
  if (!ctx->cache) {
    ctx->cache.reset(new sf_plan);
    ctx->cache->ctx = ctx;
  }
  sf_plan* P = ctx->cache.get();
  P->passes = std::move(ps);
  P->pool_bytes = pool_bytes;
  int rc;
  if ((rc = plan_build(P))) return rc;
  if ((rc = plan_upload_from(P, pool))) return rc;
  if ((rc = plan_execute(P, false))) return rc;
  if ((rc = plan_fetch(P))) return rc;
  std::vector<sf_result_t> res(P->passes.size());
  if ((rc = plan_results(P, res.data(), nullptr, 0, 0, false))) return rc;
  // lib.rs:2029-2032 (left: the span starts qi / tj bases earlier) and 2072 (right).
  for (size_t u = 0; u < res.size(); ++u) {
    sf_hit_t& h = hits[slot[u].first];
    if (slot[u].second == 0) {
      h.qstart -= (uint32_t)res[u].pattern_end;
      h.tstart -= (uint32_t)res[u].text_end;
    } else {
      h.qend += (uint32_t)res[u].pattern_end;
      h.tend += (uint32_t)res[u].text_end;
    }
  }
  return SF_OK;
}

// ---- sorted calls in a batch (the DP of map/src/lib.rs:1294-1884 `segmented`) ---------

int sf_sorted_batch(sf_context* ctx, const uint8_t* pool, uint64_t pool_bytes,
                    const sf_affine_t* scores, uint32_t n_scores, const sf_sorted_call_t* calls,
                    uint64_t n_calls, const sf_span_t* texts, uint64_t n_texts, sf_cut_t* out) {
  if (!ctx || (n_calls && !calls) || (n_texts && (!texts || !out)) || (pool_bytes && !pool) ||
      (n_scores && !scores))
    return fail(SF_ERR_INVALID, "bad argument");
  std::vector<Pass> ps;
  std::vector<uint64_t> text_of;
  for (uint64_t c = 0; c < n_calls; ++c) {
    const sf_sorted_call_t& k = calls[c];
    if (k.sc_index >= n_scores || !ok_sc(&scores[k.sc_index]))
      return fail(SF_ERR_INVALID, "bad scoring index");
    if (k.kind > SF_SORTED_EXTEND_CUT) return fail(SF_ERR_INVALID, "bad sorted call kind");
    if (k.kind == SF_SORTED_AFFINE && !ok_mode((int)k.mode)) return fail(SF_ERR_INVALID, "bad mode");
    if (k.first > n_texts || k.count > n_texts - k.first)
      return fail(SF_ERR_INVALID, "call's texts outside the text list");
    if (k.p_off > pool_bytes || k.m > pool_bytes - k.p_off)
      return fail(SF_ERR_INVALID, "pattern outside the pool");
    if (k.m >= 0x7fffffffu) return fail(SF_ERR_TOO_LONG, "sequence too long");
    const sf_affine_t* sc = &scores[k.sc_index];
    const size_t q0 = ps.size();
    for (uint64_t q = 0; q < k.count; ++q) {
      const sf_span_t& t = texts[k.first + q];
      if (t.off > pool_bytes || t.len > pool_bytes - t.off)
        return fail(SF_ERR_INVALID, "text outside the pool");
      if (t.len >= 0x7fffffffu) return fail(SF_ERR_TOO_LONG, "sequence too long");
      if (k.kind == SF_SORTED_AFFINE) {
        // align.rs:854-861 `affine_sorted`: one Global/Prefix/Infix pass per text.
        ps.push_back(affine_pass(k.p_off, k.m, t.off, t.len, (int)k.mode, sc, k.band));
      } else {
        // align.rs:903-949 `affine_extend_sorted_cut_bonus` (the passes of 917-928).
        Pass p = affine_pass(k.p_off, k.m, t.off, t.len, SF_PREFIX, sc, k.band);
        p.geom = k.diagonal ? std::min<uint64_t>(k.m, t.len) : std::max<uint64_t>(t.len, k.window);
        p.clip = true;
        p.xdrop = k.xdrop;
        p.cell = k.track_cut && k.cut != SF_NOLIMIT;
        p.cut = k.cut;
        ps.push_back(p);
      }
      text_of.push_back(k.first + q);
    }
    link_sorted(ps, q0, k.count, [&](size_t u) { return pool + texts[text_of[u]].off; });
  }
  if (ps.empty()) return SF_OK;
  if (!ctx->cache) {
    ctx->cache.reset(new sf_plan);
    ctx->cache->ctx = ctx;
  }
  sf_plan* P = ctx->cache.get();
  P->passes = std::move(ps);
  P->pool_bytes = pool_bytes;
  int rc;
  if ((rc = plan_build(P))) return rc;
  if ((rc = plan_upload_from(P, pool))) return rc;
  if ((rc = plan_execute(P, false))) return rc;
  if ((rc = plan_fetch(P))) return rc;
  const DRes* rs = P->h_res.as<DRes>();
  size_t u = 0;
  for (uint64_t c = 0; c < n_calls; ++c) {
    const sf_sorted_call_t& k = calls[c];
    count_sorted(P->passes, u, k.count, [&](size_t v) -> const DRes& { return rs[P->slot[v]]; });
    for (uint64_t q = 0; q < k.count; ++q, ++u) {
      const DRes& d = rs[P->slot[u]];
      sf_cut_t& o = out[text_of[u]];
      if (k.kind == SF_SORTED_AFFINE) {
        // lib.rs:1442-1445: an affine_sorted score stands for whole and cut, no columns.
        o.whole = o.cut = d.score;
        o.cols = 0;
        continue;
      }
      // align.rs:929-948
      const int32_t end = (k.bonus_within_cut && k.cut != SF_NOLIMIT)
                              ? std::max(d.score, sat_add32(d.cut_score, k.end_bonus))
                              : sat_add32(d.score, k.end_bonus);
      o.whole = std::max(d.clip_best, end);
      o.cols = d.clip_best >= end ? d.clip_j : d.score_col;
      o.cut = k.cut == SF_NOLIMIT ? o.whole : std::max(d.cut_best, sat_add32(d.cut_score, k.end_bonus));
    }
  }
  return SF_OK;
}

namespace {

// Jobs per segment of a batch: a batch of fewer than twice this runs as one plan.
constexpr uint64_t kSegJobs = 4096;

// Whether a batch's jobs are even enough to run in segments: no job's estimated work above
// 8x the mean.  A long pass in a late segment starts only when the earlier segments' blocks
// have left the device, so it would end after the rest; one plan starts it first.  Work is
// band cells for affine jobs and matrix cells / 24 for Myers (its cells cost about 1/24 of
// an affine cell).
bool batch_even(const sf_job_t* jobs, uint64_t count) {
  constexpr int kT = 8;
  double sum[kT] = {}, mx[kT] = {};
  parallel_chunks(count, 4096, kT, [&](size_t q0, size_t q1, int k) {
    double s = 0, x = 0;
    for (size_t q = q0; q < q1; ++q) {
      const sf_job_t& j = jobs[q];
      const double m = j.m, n = j.n;
      double w;
      if (j.kind == SF_JOB_MYERS) {
        w = m * n / 24.0;
      } else {
        const double band = j.band == SF_NOLIMIT ? n + 1 : 2.0 * (double)j.band + 1;
        w = m * std::min(n + 1, band);
      }
      s += w;
      x = std::max(x, w);
    }
    sum[k] = s;
    mx[k] = x;
  });
  double s = 0, x = 0;
  for (int k = 0; k < kT; ++k) {
    s += sum[k];
    x = std::max(x, mx[k]);
  }
  return count > 0 && x <= 8.0 * (s / (double)count);
}

// A large batch in segments of consecutive jobs, each its own plan: the host converts and
// builds segment k + 1 while the device runs segment k, and each segment's buckets start on
// the auxiliary streams after the last segment's, so that one segment's tail overlaps the
// next one's start.  The pool goes to the device once, into the first segment's plan, which
// the later segments read.  Errors are found in job order as in one plan: segment k's jobs
// are checked before segment k + 1's are converted.
int batch_run_segments(sf_context* ctx, int nseg, const uint8_t* pool, uint64_t pool_bytes,
                       const sf_job_t* jobs, uint64_t count, const sf_affine_t* scores,
                       uint32_t n_scores, sf_result_t* results, uint32_t* ops, uint64_t ops_cap,
                       uint64_t* ops_used) {
  sf_plan* seg[sf_context::kSegs];
  seg[0] = ctx->cache.get();
  for (int k = 1; k < nseg; ++k) {
    auto& sp = ctx->segs[k - 1];
    if (!sp) {
      sp.reset(new sf_plan);
      sp->ctx = ctx;
    }
    seg[k] = sp.get();
  }
  uint64_t lo[sf_context::kSegs + 1];
  for (int k = 0; k <= nseg; ++k) lo[k] = count * (uint64_t)k / (uint64_t)nseg;
  CK(cudaSetDevice(ctx->dev));
  sf_plan* P0 = seg[0];
  P0->bytes_from = nullptr;
  P0->pool_bytes = pool_bytes;
  int rc;
  if ((rc = P0->d_bytes.ensure(std::max<uint64_t>(pool_bytes, 16)))) return rc;
  if ((rc = plan_upload_from(P0, pool))) return rc;
  bool used[sf_context::kAux] = {};
  int soff = 0;
  for (int k = 0; k < nseg; ++k) {
    sf_plan* P = seg[k];
    rc = jobs_to_passes(jobs + lo[k], lo[k + 1] - lo[k], scores, n_scores, pool_bytes, P->passes,
                        ctx->store);
    if (rc == SF_OK) {
      P->pool_bytes = pool_bytes;
      P->bytes_from = k ? P0->d_bytes.as<uint8_t>() : nullptr;
      rc = plan_build(P);
    }
    if (rc == SF_OK) rc = plan_launch_buckets(P, ctx->s, nullptr, soff, true, used);
    if (rc != SF_OK) {
      // Earlier segments' kernels end before the call returns: the next call reuses their
      // buffers.  The first error stays the reported one.
      const std::string msg = last_error();
      (void)join_aux(ctx, ctx->s, used);
      (void)cudaStreamSynchronize(ctx->s);
      return fail(rc, msg);
    }
    soff = (soff + (int)std::max<size_t>(P->buckets.size(), 1)) % sf_context::kAux;
  }
  if ((rc = join_aux(ctx, ctx->s, used))) return rc;
  for (int k = 0; k < nseg; ++k)
    if ((rc = plan_launch_compact(seg[k], ctx->s, nullptr))) return rc;
  // Results: each segment's records, its CIGARs after the earlier segments' ones.
  uint64_t base[sf_context::kSegs + 1] = {};
  for (int k = 0; k < nseg; ++k) {
    if ((rc = plan_fetch(seg[k]))) return rc;
    base[k + 1] = base[k] + (seg[k]->n_walk ? *seg[k]->h_total.as<uint64_t>() : 0);
  }
  const uint64_t total = base[nseg];
  if (ops_used) *ops_used = total;
  if (total && (!ops || ops_cap < total)) return fail(SF_ERR_CAPACITY, "ops buffer smaller than the CIGARs");
  for (int k = 0; k < nseg; ++k) {
    const uint64_t n = base[k + 1] - base[k];
    if (n) CK(cudaMemcpyAsync(ops + base[k], seg[k]->d_opsc.p, n * 4, cudaMemcpyDeviceToHost, ctx->s));
  }
  if (total) CK(cudaStreamSynchronize(ctx->s));
  for (int k = 0; k < nseg; ++k) {
    const uint64_t n = base[k + 1] - base[k];
    if ((rc = plan_results(seg[k], results + lo[k], n ? ops + base[k] : nullptr, n, n, false,
                           base[k])))
      return rc;
  }
  return SF_OK;
}

}  // namespace

int sf_batch_run(sf_context* ctx, const uint8_t* pool, uint64_t pool_bytes, const sf_job_t* jobs,
                 uint64_t count, const sf_affine_t* scores, uint32_t n_scores,
                 sf_result_t* results, uint32_t* ops, uint64_t ops_cap, uint64_t* ops_used) {
  if (!ctx || (count && (!jobs || !results))) return fail(SF_ERR_INVALID, "bad argument");
  // The context keeps one plan whose device and pinned buffers grow and are reused, so a
  // stream of batches allocates only when a batch outgrows the last.
  if (!ctx->cache) {
    ctx->cache.reset(new sf_plan);
    ctx->cache->ctx = ctx;
  }
  const int nseg = (int)std::min<uint64_t>(count / kSegJobs, sf_context::kSegs);
  if (nseg >= 2 && batch_segments_on() && batch_even(jobs, count))
    return batch_run_segments(ctx, nseg, pool, pool_bytes, jobs, count, scores, n_scores, results,
                              ops, ops_cap, ops_used);
  sf_plan* P = ctx->cache.get();
  P->bytes_from = nullptr;
  int rc = jobs_to_passes(jobs, count, scores, n_scores, pool_bytes, P->passes, ctx->store);
  if (rc) return rc;
  P->pool_bytes = pool_bytes;
  // The pool's copy runs while the host builds the plan.
  CK(cudaSetDevice(ctx->dev));
  if ((rc = P->d_bytes.ensure(std::max<uint64_t>(pool_bytes, 16)))) return rc;
  if ((rc = plan_upload_from(P, pool))) return rc;
  if ((rc = plan_build(P))) return rc;
  if ((rc = plan_execute(P, false))) return rc;
  return sf_plan_download(P, results, ops, ops_cap, ops_used);
}

namespace {

// A pass's class before any override, and the Myers blocks it needs.
int default_class(const Pass& p, bool use16, ClassKey& key, int64_t& blocks) {
  if (p.kind == PK_MYERS) {
    int b = 1, lanes = 1;
    int rc = choose_myers_class(p.m, b, lanes);
    if (rc) return rc;
    key = ClassKey{PK_MYERS, b, 0, 0, lanes};
    blocks = ((int64_t)p.m + 63) / 64;
    return SF_OK;
  }
  uint32_t flags = 0;
  DJob j = make_djob(p, flags);
  const int64_t wmax = band_wmax(j, flags);
  int c = 4, lanes = 32;
  bool wide = false;
  PassKind kind = PK_AFFINE;
  classify_affine(p, flags, wmax, use16, kind, c, wide, lanes, default_lanes16());
  const bool tb = p.want_cigar && p.kind != PK_LOCAL;
  key = ClassKey{kind, c, wide ? 1 : 0, tb ? 1 : 0, lanes};
  blocks = wmax;  // affine: the group's widest row
  return SF_OK;
}

// The classes a group of passes may run in instead of its default: Myers, every
// (blocks per lane, lanes per pair) that covers the group's longest pattern; affine
// register rows, the default C and the next two classes of the same kernel.
std::vector<ClassChoice> tune_candidates(const ClassKey& key, int64_t blocks) {
  std::vector<ClassChoice> out;
  out.push_back(ClassChoice{key.c, key.lanes});
  if (key.kind == PK_MYERS) {
    for (int q = 0; q < sfk::kMyersNB; ++q) {
      const int b = sfk::kMyersB[q];
      int lanes = 1;
      while ((int64_t)lanes * b < blocks) lanes <<= 1;
      if (lanes > 32) continue;
      bool dup = false;
      for (const auto& c : out) dup = dup || (c.c == b && c.lanes == lanes);
      if (!dup) out.push_back(ClassChoice{b, lanes});
    }
  } else if (!key.wide) {
    const bool half = key.kind == PK_AFFINE16 && key.lanes == 16;
    const int* cs = key.kind == PK_AFFINE16 ? (half ? sfk::kAffine16HC : sfk::kAffine16C)
                                            : sfk::kAffineC;
    const int nc = key.kind == PK_AFFINE16 ? (half ? sfk::kAffine16HNC : sfk::kAffine16NC)
                                           : sfk::kAffineNC;
    for (int q = 0; q < nc; ++q)
      if (cs[q] > key.c && (int)out.size() < 3) out.push_back(ClassChoice{cs[q], key.lanes});
    // 16-bit rows: the other lane count per pass (two passes per warp, or one), its two
    // narrowest classes that hold the group's widest row (`blocks` carries it here).
    const int other = half ? 32 : 16;
    const int* os = half ? sfk::kAffine16C : sfk::kAffine16HC;
    const int no = half ? sfk::kAffine16NC : sfk::kAffine16HNC;
    int added = 0;
    if (key.kind == PK_AFFINE16)
      for (int q = 0; q < no && added < 2; ++q)
        if ((int64_t)other * os[q] >= blocks) {
          out.push_back(ClassChoice{os[q], other});
          ++added;
        }
  }
  return out;
}

}  // namespace

int sf_plan_tune(sf_plan* P, const uint8_t* pool, uint32_t reps, char* report, uint64_t cap) {
  if (!P || (P->pool_bytes && !pool)) return fail(SF_ERR_INVALID, "bad argument");
  sf_context* ctx = P->ctx;
  CK(cudaSetDevice(ctx->dev));
  if (reps == 0) reps = 1;
  const auto t0 = std::chrono::steady_clock::now();
  const bool use16 = allow16();
  // Group the passes by their default class.
  std::map<ClassKey, std::vector<size_t>> groups;
  std::map<ClassKey, int64_t> gblocks;
  for (size_t q = 0; q < P->passes.size(); ++q) {
    ClassKey k;
    int64_t blocks = 0;
    int rc = default_class(P->passes[q], use16, k, blocks);
    if (rc) return rc;
    groups[k].push_back(q);
    gblocks[k] = std::max(gblocks[k], blocks);
  }
  sf_plan S;  // trial plan, its buffers reused across trials
  S.ctx = ctx;
  S.pool_bytes = P->pool_bytes;
  void* uploaded = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  std::string rep = "{\"groups\": [";
  int rc = SF_OK;
  size_t gi = 0;
  for (auto& g : groups) {
    const ClassKey& key = g.first;
    const std::vector<ClassChoice> cands = tune_candidates(key, gblocks[key]);
    S.passes.clear();
    for (size_t q : g.second) S.passes.push_back(P->passes[q]);
    float best_ms = -1;
    ClassChoice best = cands[0];
    std::string tried;
    for (size_t ci = 0; ci < cands.size() && rc == SF_OK; ++ci) {
      TuneTable t1;
      t1[key] = cands[ci];
      S.tune_override = &t1;
      if ((rc = plan_build(&S))) break;
      if (S.d_bytes.p != uploaded) {
        if ((rc = plan_upload_from(&S, pool))) break;
        uploaded = S.d_bytes.p;
      }
      if ((rc = plan_launch(&S, ctx->s))) break;  // warm-up
      CK(cudaEventRecord(e0, ctx->s));
      for (uint32_t r = 0; r < reps && rc == SF_OK; ++r) rc = plan_launch(&S, ctx->s);
      CK(cudaEventRecord(e1, ctx->s));
      CK(cudaEventSynchronize(e1));
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      ms /= (float)reps;
      char buf[96];
      std::snprintf(buf, sizeof buf, "%s{\"c\": %d, \"lanes\": %d, \"ms\": %.4f}", ci ? ", " : "",
                    cands[ci].c, cands[ci].lanes, ms);
      tried += buf;
      if (best_ms < 0 || ms < best_ms) {
        best_ms = ms;
        best = cands[ci];
      }
    }
    S.tune_override = nullptr;
    if (rc) break;
    if (best.c == key.c && best.lanes == key.lanes)
      ctx->tune.erase(key);
    else
      ctx->tune[key] = best;
    char buf[256];
    std::snprintf(buf, sizeof buf,
                  "%s{\"kind\": \"%s\", \"c\": %d, \"wide\": %s, \"traceback\": %s, \"lanes\": %d, "
                  "\"jobs\": %zu, \"chosen\": {\"c\": %d, \"lanes\": %d}, \"tried\": [",
                  gi++ ? ", " : "",
                  key.kind == PK_MYERS ? "myers"
                                       : (key.kind == PK_LOCAL ? "local"
                                                               : (key.kind == PK_AFFINE16 ? "affine16" : "affine")),
                  key.c, key.wide ? "true" : "false", key.tb ? "true" : "false", key.lanes,
                  g.second.size(), best.c, best.lanes);
    rep += buf + tried + "]}";
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  // The plan itself now runs with the chosen classes.
  if ((rc = plan_build(P))) return rc;
  if ((rc = plan_upload_from(P, pool))) return rc;
  const double secs =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  char tail[64];
  std::snprintf(tail, sizeof tail, "], \"seconds\": %.3f}", secs);
  rep += tail;
  if (report && cap) {
    const size_t n = std::min<size_t>(rep.size(), cap - 1);
    std::memcpy(report, rep.data(), n);
    report[n] = 0;
    if (rep.size() >= cap) return fail(SF_ERR_CAPACITY, "report longer than its buffer");
  }
  return SF_OK;
}

int sf_context_untune(sf_context* ctx) {
  if (!ctx) return fail(SF_ERR_INVALID, "null context");
  ctx->tune.clear();
  return SF_OK;
}

// ---- transcript store ---------------------------------------------------------------

int sf_store_create(sf_context* ctx, const uint8_t* codes, const uint64_t* lens, uint64_t count,
                    sf_store** out) {
  if (!ctx || !out || (count && !lens)) return fail(SF_ERR_INVALID, "bad argument");
  uint64_t bases = 0;
  for (uint64_t q = 0; q < count; ++q) bases += lens[q];
  if (bases && !codes) return fail(SF_ERR_INVALID, "null codes");
  CK(cudaSetDevice(ctx->dev));
  std::unique_ptr<sf_store> S(new sf_store);
  S->dev = ctx->dev;
  S->bases = bases;
  const uint64_t nwords = (bases + 15) / 16 + 1;
  int rc = S->words.ensure((nwords + 64) * 4);
  if (rc) return rc;
  CK(cudaMemsetAsync(S->words.p, 0, (nwords + 64) * 4, ctx->s));
  if (bases) {
    DevBuf staging;
    if ((rc = staging.ensure(bases))) return rc;
    CK(cudaMemcpyAsync(staging.p, codes, bases, cudaMemcpyHostToDevice, ctx->s));
    CK(sfk::launch_store_pack(staging.as<uint8_t>(), bases, S->words.as<uint32_t>(), ctx->s));
    CK(cudaStreamSynchronize(ctx->s));
  } else {
    CK(cudaStreamSynchronize(ctx->s));
  }
  *out = S.release();
  return SF_OK;
}

int sf_store_create_packed(sf_context* ctx, const uint64_t* tx_seq, uint64_t bases,
                           sf_store** out) {
  if (!ctx || !out || (bases && !tx_seq)) return fail(SF_ERR_INVALID, "bad argument");
  CK(cudaSetDevice(ctx->dev));
  std::unique_ptr<sf_store> S(new sf_store);
  S->dev = ctx->dev;
  S->bases = bases;
  const uint64_t nwords = (bases + 15) / 16 + 1;
  int rc = S->words.ensure((nwords + 64) * 4);
  if (rc) return rc;
  CK(cudaMemsetAsync(S->words.p, 0, (nwords + 64) * 4, ctx->s));
  // 32 bases per u64, read as two little-endian u32 words of 16: the store's own order.
  if (bases)
    CK(cudaMemcpyAsync(S->words.as<uint32_t>() + kStorePad / 16, tx_seq, (bases + 31) / 32 * 8,
                       cudaMemcpyHostToDevice, ctx->s));
  CK(cudaStreamSynchronize(ctx->s));
  *out = S.release();
  return SF_OK;
}

void sf_store_destroy(sf_store* store) {
  if (!store) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(store->dev);
  delete store;
  cudaSetDevice(prev);
}

uint64_t sf_store_bases(const sf_store* store) { return store ? store->bases : 0; }

int sf_context_use_store(sf_context* ctx, sf_store* store) {
  if (!ctx) return fail(SF_ERR_INVALID, "null context");
  if (store && store->dev != ctx->dev) return fail(SF_ERR_INVALID, "store on another device");
  ctx->store = store;
  return SF_OK;
}

int sf_plan_profile(sf_plan* P, float* ms, uint32_t cap, uint32_t* n_stages) {
  if (!P || !n_stages || (cap && !ms)) return fail(SF_ERR_INVALID, "bad argument");
  CK(cudaSetDevice(P->ctx->dev));
  std::vector<cudaEvent_t> evs;
  int rc = plan_launch(P, P->ctx->s, &evs);
  cudaError_t e = cudaStreamSynchronize(P->ctx->s);
  const uint32_t n = evs.empty() ? 0 : (uint32_t)evs.size() - 1;
  *n_stages = n;
  for (uint32_t q = 0; q < n && q < cap && rc == SF_OK && e == cudaSuccess; ++q) {
    float t = 0;
    cudaEventElapsedTime(&t, evs[q], evs[q + 1]);
    ms[q] = t;
  }
  for (cudaEvent_t x : evs) cudaEventDestroy(x);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(SF_ERR_CUDA, cudaGetErrorString(e));
  return n > cap ? fail(SF_ERR_CAPACITY, "more stages than ms slots") : SF_OK;
}

int sf_int_peak(int device, double* tops, double* ms) {
  if (!tops) return fail(SF_ERR_INVALID, "bad argument");
  CK(cudaSetDevice(device));
  int sms = 0;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  DevBuf out;
  int rc = out.ensure((size_t)sms * 8 * 256 * 4);
  if (rc) return rc;
  double best = 0, best_ms = 0;
  for (int rep = 0; rep < 4; ++rep) {
    float t = 0;
    uint64_t ops = 0;
    CK(sfk::run_int_peak(sms, out.as<int32_t>(), &t, &ops));
    const double r = (double)ops / (t * 1e-3) / 1e12;
    if (rep > 0 && r > best) {  // the first run warms up clocks and caches
      best = r;
      best_ms = t;
    }
  }
  *tops = best;
  if (ms) *ms = best_ms;
  return SF_OK;
}

}  // extern "C"
