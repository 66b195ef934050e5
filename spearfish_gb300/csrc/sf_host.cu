// The C ABI's entry points (include/sf_align.h): the one-call functions that mirror
// crates/map/src/align.rs on a per-thread context, batch runs (tie-break batches, span-end
// extensions, sorted calls, sf_batch_run in segments), the autotuner, the transcript store
// and the measurement helpers.  Plans themselves are built and launched in sf_plan.cu.
#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "sf_engine.h"
#include "sf_hostpool.h"

using namespace sfe;

namespace sfe {

thread_local uint64_t g_dp_cells = 0, g_dp_rows = 0;

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

}  // namespace sfe

int sf_internal_set_error(int code, const char* msg) { return fail(code, msg); }

// ---- C ABI ------------------------------------------------------------------------------

extern "C" {

const char* sf_last_error(void) { return last_error().c_str(); }

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

int sf_plan_job_buckets(const sf_plan* plan, uint32_t* buckets, uint64_t count) {
  if (!plan || (!buckets && count)) return fail(SF_ERR_INVALID, "bad argument");
  return plan_job_buckets(plan, buckets, count);
}

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

// The end of the furthest pool byte the jobs read (patterns, and texts in the pool), at most
// pool_bytes.
uint64_t pool_reach(const sf_job_t* jobs, uint64_t count, uint64_t pool_bytes) {
  constexpr int kT = 16;
  uint64_t mx[kT] = {};
  auto end = [&](uint64_t off, uint64_t len) {
    return off >= pool_bytes || len > pool_bytes - off ? pool_bytes : off + len;
  };
  parallel_chunks(count, 4096, kT, [&](size_t q0, size_t q1, int k) {
    uint64_t x = 0;
    for (size_t q = q0; q < q1; ++q) {
      const sf_job_t& j = jobs[q];
      x = std::max(x, end(j.p_off, j.m));
      if (j.text_src == SF_TEXT_POOL) x = std::max(x, end(j.t_off, j.n));
    }
    mx[k] = x;
  });
  return *std::max_element(mx, mx + kT);
}

// Whether a batch's jobs are even enough to run in segments: no job's estimated work above
// 8x the mean.  A long pass in a late segment starts only when the earlier segments' blocks
// have left the device, so it would end after the rest; one plan starts it first.  Work is
// band cells for affine jobs and matrix cells / 24 for Myers (its cells cost about 1/24 of
// an affine cell).
bool batch_even(const sf_job_t* jobs, uint64_t count) {
  constexpr int kT = 16;
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
// next one's start.  Each segment's CIGAR compaction and copies back run on the context's
// tail stream as soon as its buckets end, and the host converts its results while later
// segments run.  The pool goes to the device once, into the first segment's plan, which the
// later segments read.  Errors are found in job order as in one plan: segment k's jobs are
// checked before segment k + 1's are converted.
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
  if (pool_bytes && !pool) return fail(SF_ERR_INVALID, "null pool");
  sf_plan* P0 = seg[0];
  P0->bytes_from = nullptr;
  P0->pool_bytes = pool_bytes;
  int rc;
  if ((rc = P0->d_bytes.ensure(std::max<uint64_t>(pool_bytes, 16)))) return rc;
  bool used[sf_context::kAux] = {};
  int soff = 0;
  uint64_t up = 0;  // pool bytes copied so far
  for (int k = 0; k < nseg; ++k) {
    sf_plan* P = seg[k];
    // The pool goes up in prefixes: before a segment, the bytes up to the furthest one its
    // jobs read (in a pool laid out in job order, about a segment's share).
    const uint64_t reach = pool_reach(jobs + lo[k], lo[k + 1] - lo[k], pool_bytes);
    if (reach > up) {
      CK(cudaMemcpyAsync(P0->d_bytes.as<uint8_t>() + up, pool + up, reach - up,
                         cudaMemcpyHostToDevice, ctx->s));
      up = reach;
    }
    rc = jobs_to_passes(jobs + lo[k], lo[k + 1] - lo[k], scores, n_scores, pool_bytes, P->passes,
                        ctx->store);
    if (rc == SF_OK) {
      P->pool_bytes = pool_bytes;
      P->bytes_from = k ? P0->d_bytes.as<uint8_t>() : nullptr;
      rc = plan_build(P);
    }
    bool mine[sf_context::kAux] = {};
    if (rc == SF_OK) rc = plan_launch_buckets(P, ctx->s, nullptr, soff, true, mine);
    for (int i = 0; i < sf_context::kAux; ++i) used[i] = used[i] || mine[i];
    // The segment's tail on the tail stream, while later segments run: its buckets joined,
    // its CIGARs compacted, its records copied back.
    if (rc == SF_OK) rc = join_aux(ctx, ctx->tail, mine);
    if (rc == SF_OK) rc = plan_launch_compact(P, ctx->tail, nullptr);
    if (rc == SF_OK) rc = plan_fetch_async(P, ctx->tail);
    if (rc == SF_OK && cudaEventRecord(ctx->seg_done[k], ctx->tail) != cudaSuccess)
      rc = fail(SF_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
    if (rc != SF_OK) {
      // Earlier segments' kernels and tails end before the call returns: the next call
      // reuses their buffers.  The first error stays the reported one.
      const std::string msg = last_error();
      (void)join_aux(ctx, ctx->s, used);
      (void)cudaStreamSynchronize(ctx->s);
      (void)cudaStreamSynchronize(ctx->tail);
      return fail(rc, msg);
    }
    soff = (soff + (int)std::max<size_t>(P->buckets.size(), 1)) % sf_context::kMain;
  }
  // Results, segment by segment as their tails end: the records converted while later
  // segments run, the CIGARs copied to the caller after the earlier segments' ones.
  uint64_t base[sf_context::kSegs + 1] = {};
  bool fits = true;
  for (int k = 0; k < nseg && rc == SF_OK; ++k) {
    if (cudaEventSynchronize(ctx->seg_done[k]) != cudaSuccess) {
      rc = fail(SF_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
      break;
    }
    const uint64_t n = seg[k]->n_walk ? *seg[k]->h_total.as<uint64_t>() : 0;
    base[k + 1] = base[k] + n;
    if (!fits || (n && (!ops || base[k + 1] > ops_cap))) {
      fits = false;  // the remaining totals are still counted for ops_used
      continue;
    }
    // On the main stream (idle by now): the tail stream still holds later segments' tails.
    if (n && cudaMemcpyAsync(ops + base[k], seg[k]->d_opsc.p, n * 4, cudaMemcpyDeviceToHost,
                             ctx->s) != cudaSuccess) {
      rc = fail(SF_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
      break;
    }
    rc = plan_results(seg[k], results + lo[k], n ? ops + base[k] : nullptr, n, n, false, base[k]);
  }
  // Every copy into the caller's buffers, and all of the call's device work, has ended when
  // the call returns.
  cudaError_t e = cudaStreamSynchronize(ctx->tail);
  const cudaError_t e2 = cudaStreamSynchronize(ctx->s);
  if (e == cudaSuccess) e = e2;
  if (rc != SF_OK) return rc;
  if (e != cudaSuccess) return fail(SF_ERR_CUDA, cudaGetErrorString(e));
  if (ops_used) *ops_used = base[nseg];
  if (!fits) return fail(SF_ERR_CAPACITY, "ops buffer smaller than the CIGARs");
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
    // The 16-bit classes for 16, 32 and 64 lanes a pass.
    auto classes16 = [](int lanes, const int*& cs, int& nc) {
      cs = lanes == 16 ? sfk::kAffine16HC : (lanes == 64 ? sfk::kAffine16WC : sfk::kAffine16C);
      nc = lanes == 16 ? sfk::kAffine16HNC : (lanes == 64 ? sfk::kAffine16WNC : sfk::kAffine16NC);
    };
    const int* cs = sfk::kAffineC;
    int nc = sfk::kAffineNC;
    if (key.kind == PK_AFFINE16) classes16(key.lanes, cs, nc);
    for (int q = 0; q < nc; ++q)
      if (cs[q] > key.c && (int)out.size() < 3) out.push_back(ClassChoice{cs[q], key.lanes});
    // 16-bit rows: other lane counts per pass, the narrowest classes that hold the group's
    // widest row (`blocks` carries it here) -- two passes per warp or one (16 <-> 32 lanes,
    // two classes), and one warp or two (32 <-> 64 lanes, one class, rows over 1,280 cells).
    // Two warps are offered for the widest rows only: timed alone a group of 1,025-1,280
    // cell rows can run faster on them, but among the other buckets of a batch its barriers
    // wait on busy SMs (config 3's passes over 4.8 kb: 33.5 ms a step on one warp each,
    // 55 ms on two).
    auto add_other = [&](int lanes, int most) {
      const int* os;
      int no;
      classes16(lanes, os, no);
      int added = 0;
      for (int q = 0; q < no && added < most; ++q)
        if ((int64_t)lanes * os[q] >= blocks) {
          out.push_back(ClassChoice{os[q], lanes});
          ++added;
        }
    };
    if (key.kind == PK_AFFINE16) {
      if (key.lanes == 16) add_other(32, 2);
      if (key.lanes == 32) add_other(16, 2);
      if (key.lanes == 32 && blocks > 32 * 40) add_other(64, 1);
      if (key.lanes == 64) add_other(32, 1);
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
