// Batch plans: device contexts, kernel classes, the plan build (sequences, pass descriptors,
// length buckets, HBM layout, descriptor upload), the launches of one execute (persistent
// grids over auxiliary streams, CIGAR compaction, CUDA graph) and the conversion of jobs
// and results at the C ABI (include/sf_align.h).
#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "sf_engine.h"
#include "sf_hostpool.h"

namespace sfe {

thread_local std::string g_err;

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
  CK(cudaStreamCreateWithFlags(&c->tail, cudaStreamNonBlocking));
  for (auto& ev : c->seg_done) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
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

// Lanes per 16-bit pass by default: 32 (with 64 for rows wider than 32 x 40 cells), or with
// SF_AFFINE16_LANES in the environment 16 (two passes per warp) or 64 (two warps per pass,
// every pass a 64-lane class holds); the autotuner chooses per length bucket either way.
int default_lanes16() {
  const char* env = std::getenv("SF_AFFINE16_LANES");
  if (env && env[0] == '1' && env[1] == '6') return 16;
  if (env && env[0] == '6' && env[1] == '4') return 64;
  return 32;
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

// Capped Global and Prefix Myers pairs stop at the first column wholly past their cap
// (sf_myers.cu); SF_MYERS_STOP=0 in the environment runs them to the end (same results).
bool allow_myers_stop() {
  const char* env = std::getenv("SF_MYERS_STOP");
  return !(env && env[0] == '0');
}

bool allow_chains() {
  const char* env = std::getenv("SF_SORTED_CHAINS");
  return env && env[0] == '1';
}

// Two-warp 16-bit passes (64 lanes) for rows wider than 32 x 40 cells: such passes are long
// and bound by their own row latency on one warp.  SF_AFFINE16_W64=0 in the environment keeps
// one warp a pass (the autotuner may still choose either per length bucket); read per plan.
bool allow_w64() {
  const char* env = std::getenv("SF_AFFINE16_W64");
  return !(env && env[0] == '0');
}

// Kernel class of an affine or local pass: the packed 16-bit kernel when the pass fits it,
// else the 32-bit register kernel, else (rows wider than 32 * 48 cells) the wide-row kernel.
void classify_affine(const Pass& p, uint32_t flags, int64_t wmax, bool use16, PassKind& kind,
                     int& c, bool& wide, int& lanes, int lanes16) {
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
    if ((wmax > 32 * 40 && allow_w64()) || lanes16 == 64)
      for (int q = 0; q < sfk::kAffine16WNC; ++q)
        if (64 * (int64_t)sfk::kAffine16WC[q] >= wmax) {
          kind = PK_AFFINE16;
          c = sfk::kAffine16WC[q];
          lanes = 64;
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
  constexpr int kChunks = 16;
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
  constexpr int kT = 16;
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
  constexpr int kMaxThreads = 16;
  uint64_t scratch_max[kMaxThreads] = {};
  bool kcut[kMaxThreads] = {};
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
        if (p.mode != SF_INFIX && (uint64_t)p.k < (uint64_t)p.m + p.n) kcut[worker] = true;
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
  P->myers_kcut = allow_myers_stop() && std::any_of(kcut, kcut + kMaxThreads, [](bool v) { return v; });
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
  constexpr int kT = 16;
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
  constexpr int kT = 16;
  // Buckets in key order; within a bucket, longest work first (ties in job order).
  // Each item's bucket first: keys pack into 15-bit codes ordered as the keys are (kind < 8,
  // C < 128, lanes a power of two up to 64, coded by its log2), so a bit set of the codes
  // present lists the buckets in order and a code's bucket is the number of codes below it.
  // Keys outside those bounds (never built) take a search instead.
  auto& kid = S.kid;
  kid.resize(ni);
  std::vector<Key2> keys;  // the buckets' keys, in order
  {
    constexpr uint32_t kWords = (1u << 15) / 64;
    auto fits = [](const Key2& k) {
      return k.kind >= 0 && k.kind < 8 && k.c >= 0 && k.c < 128 && (k.wide & ~1) == 0 &&
             (k.tb & ~1) == 0 && k.lanes >= 1 && k.lanes <= 64 && (k.lanes & (k.lanes - 1)) == 0;
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
        const uint32_t c = (uint32_t)key.kind << 12 | (uint32_t)key.c << 5 |
                           (uint32_t)key.wide << 4 | (uint32_t)key.tb << 3 |
                           (uint32_t)__builtin_ctz((uint32_t)key.lanes);
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
          keys.push_back(Key2{(int)(c >> 12), (int)((c >> 5) & 127), (int)((c >> 4) & 1),
                              (int)((c >> 3) & 1), 1 << (c & 7)});
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
  // counting sort: equal rounded work keeps job order).  A bucket of a quarter of the items
  // or more sorts on the host pool by itself; the others sort side by side, one thread to a
  // bucket (config 3's 22 buckets: 1.6 -> 0.8 ms, against three pool dispatches a bucket).
  auto wbin = [](uint64_t w) -> uint32_t {
    if (w < 16) return (uint32_t)w;
    const int e = 63 - __builtin_clzll(w);  // w in [2^e, 2^(e+1))
    return (uint32_t)(16 * (e - 3) + ((w >> (e - 4)) & 15));
  };
  constexpr uint32_t kBins = 16 * 61 + 16;
  const size_t big = std::max<size_t>(4096, ni / 4);
  auto& tmp = S.byb_tmp;
  std::vector<uint64_t> bin_at((size_t)kT * kBins);
  for (size_t u = 0; u < nb; ++u) {
    Bucket& b = P->buckets[u];
    if (b.count < big) continue;
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
      if (b.count >= big) continue;
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
      // Two-warp passes: one pass per 64-thread block; otherwise a 4-warp block holds 4
      // passes (chains), or 8 with 16 lanes a pass.
      b.block = b.lanes == 64 ? 64 : 128;
      const uint64_t per_block = b.lanes == 64 ? 1 : (b.lanes == 16 ? 8 : 4);
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
  // Streams.  The first buckets (in launch order) of fewer warps than the device has SMs -- a
  // few long passes: the widest rows, the longest patterns -- take a side stream each, so
  // that no bucket queues behind their long run; the others go round robin over the main
  // streams in launch order, so that their tails overlap.  Measured on 100,000 uneven pairs:
  // 87.5 -> 86.8 ms an execute; every bucket on a stream of its own (16 or 32 streams) took
  // 106-112 ms, the long passes then starting late among the other kernels' blocks.
  int nmain = 0, nside = 0;
  for (auto& b : P->buckets) {
    if ((int64_t)b.grid * (b.block / 32) < ctx->sms && nside < sf_context::kSide)
      b.stream = sf_context::kMain + nside++;
    else
      b.stream = nmain++ % sf_context::kMain;
  }
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

// Each job's bucket, as its index in the plan's description (sf_plan_job_buckets);
// SF_NONE for a pass that a row-sharing chain runs.
int plan_job_buckets(const sf_plan* P, uint32_t* out, uint64_t count) {
  const size_t np = P->passes.size();
  if (count < np) return fail(SF_ERR_INVALID, "job_buckets: output shorter than the plan's jobs");
  if (!P->scratch || P->scratch->per.size() != np) return fail(SF_ERR_INVALID, "job_buckets: plan not built");
  const BuildScratch& S = *P->scratch;
  std::vector<BucketKey> keys(P->buckets.size());
  for (size_t u = 0; u < keys.size(); ++u) {
    const Bucket& b = P->buckets[u];
    keys[u] = BucketKey{(int)b.kind, b.c, b.wide ? 1 : 0, b.tb ? 1 : 0, b.lanes};
  }
  for (size_t q = 0; q < np; ++q) {
    out[q] = SF_NONE;
    if (!S.has_item[q]) continue;
    for (size_t u = 0; u < keys.size(); ++u)
      if (keys[u] == S.per[q].first) {
        out[q] = (uint32_t)u;
        break;
      }
  }
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
// auxiliary streams so that their tails overlap (each bucket on its stream, the main ones
// rotated by `soff`; also a single bucket with `fan_one`).  `used` collects the auxiliary
// streams launched on.
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
      const int si = b.stream < sf_context::kMain ? (b.stream + soff) % sf_context::kMain : b.stream;
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
      ml.kcut = P->myers_kcut ? 1 : 0;
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
      else if (b.kind == PK_AFFINE16 && b.lanes == 64)
        CK(sfk::launch_affine16w(b.c, b.tb, al, b.grid, b.block, bs));
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
int plan_launch(sf_plan* P, cudaStream_t s, std::vector<cudaEvent_t>* evs) {
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
  CK(cudaMemcpyAsync(P->d_bytes.p, pool, P->pool_bytes, cudaMemcpyHostToDevice, ctx->s));
  return SF_OK;
}

// Results -> host pinned buffers (and compacted ops), then the caller's arrays.
int plan_fetch_async(sf_plan* P, cudaStream_t s) {
  int rc;
  if ((rc = P->h_res.ensure(P->n_aff * sizeof(DRes) + 64))) return rc;
  if ((rc = P->h_mout.ensure(P->n_my * 4 + 64))) return rc;
  if ((rc = P->h_tres.ensure(P->n_aff * sizeof(TRes) + 64))) return rc;
  if (P->n_aff) CK(cudaMemcpyAsync(P->h_res.p, P->d_res.p, P->n_aff * sizeof(DRes), cudaMemcpyDeviceToHost, s));
  if (P->n_my) CK(cudaMemcpyAsync(P->h_mout.p, P->d_mout.p, P->n_my * 4, cudaMemcpyDeviceToHost, s));
  if (P->n_walk) {
    CK(cudaMemcpyAsync(P->h_tres.p, P->d_tres.p, P->n_aff * sizeof(TRes), cudaMemcpyDeviceToHost, s));
    if ((rc = P->h_total.ensure(64))) return rc;
    CK(cudaMemcpyAsync(P->h_total.p, P->d_total.p, 8, cudaMemcpyDeviceToHost, s));
  }
  return SF_OK;
}

int plan_fetch(sf_plan* P) {
  int rc;
  if ((rc = plan_fetch_async(P, P->ctx->s))) return rc;
  CK(cudaStreamSynchronize(P->ctx->s));
  return SF_OK;
}

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

bool ok_mode(int mode) { return mode == SF_INFIX || mode == SF_PREFIX || mode == SF_GLOBAL; }
bool ok_sc(const sf_affine_t* sc) {
  // align.rs:2504 debug_assert!(open >= 0 && ext >= 0).
  return sc && sc->open >= 0 && sc->ext >= 0;
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
  constexpr int kMaxThreads = 16;
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
  constexpr int kT = 16;
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
  const int lanes16 = default_lanes16();
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
    classify_affine(p, flags, wmax, use16, kind, c, wide, ln, lanes16);
    if (p.want_cigar && p.kind != PK_LOCAL) {
      b += (uint64_t)p.m * tb_row_words(c, wide ? wide_chunks(c, wmax) : 1) * 4 * ln / 32;
      b += 2 * ((uint64_t)p.m + p.n + 2) * 4;
    }
    if (wide) scratch = std::max<uint64_t>(scratch, (uint64_t)wide_chunks(c, wmax) * 32 * c);
  }
  // Wide buckets (with and without traceback): up to 2 blocks/SM x 4 warps x 4 rows each.
  b += scratch * 4 * 2 * 304 * 4 * 4 * 2;
  return b + b / 4;
}

}  // namespace sfe
