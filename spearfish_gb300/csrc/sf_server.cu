// Serving loop: continuous batching of alignment requests on one GPU.
//
// A request is a read batch's jobs (sf_job_t) over a byte pool the caller keeps alive until
// the request is waited for.  Requests queue in arrival order; a dispatcher thread admits the
// oldest one as soon as a slot is free and the device memory the request needs fits the
// server's HBM budget (the budget defaults to 90% of the device memory free when the server
// starts, cudaMemGetInfo).  Each slot owns a context (its CUDA streams) and a plan whose
// device and pinned buffers grow and are reused, so requests on different slots run their
// bucketed persistent kernels concurrently on the device while the dispatcher prepares the
// next.  A finished request's results are copied to host memory and released by
// sf_server_wait, whose waits are bounded by the caller's timeout.  Results depend only on the
// request's own jobs: a request computes the same alone as in any mix.
//
// The device side holds no waits: admission, completion (cudaEventQuery) and hand-off all
// happen on the host, so no kernel ever spins on a flag another kernel or the host must set.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "sf_engine.h"

using namespace sfe;

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

enum ReqState { R_PENDING, R_RUNNING, R_DONE };

struct Request {
  uint64_t ticket = 0;
  const uint8_t* pool = nullptr;
  uint64_t pool_bytes = 0;
  std::vector<Pass> passes;
  uint64_t estimate = 0;
  ReqState state = R_PENDING;
  int rc = SF_OK;
  std::string msg;  // the failure's message (set on the dispatcher thread)
  int slot = -1;
  Clock::time_point t_submit, t_admit, t_done;
  std::vector<sf_result_t> results;
  std::vector<uint32_t> ops;
  uint64_t cells = 0;
};

struct Slot {
  sf_context* ctx = nullptr;
  std::unique_ptr<sf_plan> plan;
  cudaEvent_t done = nullptr;
  std::shared_ptr<Request> req;  // running request
  bool busy = false;
  uint64_t held = 0;  // device bytes the slot's plan holds (updated under the lock)
};

}  // namespace

struct sf_server {
  int dev = 0;
  uint64_t budget = 0;
  sf_store* store = nullptr;  // transcript store for SF_TEXT_STORE texts
  std::vector<sf_affine_t> scores;
  std::vector<Slot> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> pending;
  std::unordered_map<uint64_t, std::shared_ptr<Request>> requests;
  uint64_t next_ticket = 1;
  uint64_t submitted = 0, completed = 0, failed = 0, cells = 0;
  bool stop = false;
  std::thread dispatcher;
  int init_rc = SF_OK;
};

namespace {

uint64_t held_bytes(sf_server* S) {
  uint64_t b = 0;
  for (auto& sl : S->slots) b += sl.held;
  return b;
}

// Runs on the dispatcher thread: plan, upload and launch `req` on slot `si`.
int start_request(sf_server* S, int si, const std::shared_ptr<Request>& req) {
  Slot& sl = S->slots[si];
  sf_plan* P = sl.plan.get();
  P->passes = std::move(req->passes);
  P->pool_bytes = req->pool_bytes;
  int rc = plan_build(P);
  if (rc == SF_OK) rc = plan_upload_from(P, req->pool);
  if (rc == SF_OK) rc = plan_execute(P, false);
  if (rc == SF_OK) {
    const cudaError_t e = cudaEventRecord(sl.done, sl.ctx->s);
    if (e != cudaSuccess) rc = fail(SF_ERR_CUDA, cudaGetErrorString(e));
  }
  return rc;
}

// Runs on the dispatcher thread: results of slot `si`'s finished request to host memory.
int finish_request(sf_server* S, int si, Request& req) {
  sf_plan* P = S->slots[si].plan.get();
  int rc = plan_fetch(P);
  uint64_t total = 0;
  if (rc == SF_OK) rc = plan_fetch_ops(P, total);
  if (rc == SF_OK) {
    req.results.resize(P->passes.size());
    req.ops.resize(total);
    rc = plan_results(P, req.results.data(), req.ops.data(), total, total);
    uint64_t c = 0;
    for (const auto& r : req.results) c += r.cells;
    req.cells = c;
  }
  return rc;
}

void dispatch_loop(sf_server* S) {
  cudaSetDevice(S->dev);
  std::unique_lock<std::mutex> lk(S->mu);
  while (!S->stop) {
    bool progressed = false;
    // Completions.
    for (int si = 0; si < (int)S->slots.size(); ++si) {
      Slot& sl = S->slots[si];
      if (!sl.busy) continue;
      const cudaError_t q = cudaEventQuery(sl.done);
      if (q == cudaErrorNotReady) continue;
      std::shared_ptr<Request> req = sl.req;
      lk.unlock();
      int rc = q == cudaSuccess ? finish_request(S, si, *req)
                                : fail(SF_ERR_CUDA, cudaGetErrorString(q));
      const std::string msg = rc ? last_error() : std::string();
      lk.lock();
      req->rc = rc;
      req->msg = msg;
      req->t_done = Clock::now();
      req->state = R_DONE;
      sl.busy = false;
      sl.req.reset();
      if (rc == SF_OK) {
        S->completed++;
        S->cells += req->cells;
      } else {
        S->failed++;
      }
      progressed = true;
      S->cv_done.notify_all();
    }
    // Admissions: the oldest pending request, when a slot and the memory it needs are free.
    while (!S->pending.empty()) {
      std::shared_ptr<Request> req = S->pending.front();
      const uint64_t held = held_bytes(S);
      int best = -1;
      for (int si = 0; si < (int)S->slots.size(); ++si) {
        Slot& sl = S->slots[si];
        if (sl.busy) continue;
        const uint64_t have = sl.held;
        const uint64_t grow = req->estimate > have ? req->estimate - have : 0;
        if (held + grow > S->budget) continue;
        if (best < 0 || grow == 0) best = si;
        if (grow == 0) break;
      }
      if (best < 0) {
        bool any_busy = false;
        for (auto& sl : S->slots) any_busy |= sl.busy;
        if (any_busy) break;  // wait for memory to free up
        // Nothing runs and it still does not fit: it never will.
        S->pending.pop_front();
        req->rc = SF_ERR_NOMEM;
        req->msg = "request needs more device memory than the server's budget";
        req->state = R_DONE;
        req->t_done = Clock::now();
        S->failed++;
        S->cv_done.notify_all();
        progressed = true;
        continue;
      }
      S->pending.pop_front();
      Slot& sl = S->slots[best];
      sl.busy = true;
      sl.req = req;
      req->slot = best;
      req->state = R_RUNNING;
      req->t_admit = Clock::now();
      lk.unlock();
      const int rc = start_request(S, best, req);
      const uint64_t now_held = plan_bytes_held(sl.plan.get());
      const std::string msg = rc ? last_error() : std::string();
      lk.lock();
      sl.held = now_held;
      if (rc != SF_OK) {
        req->rc = rc;
        req->msg = msg;
        req->state = R_DONE;
        req->t_done = Clock::now();
        sl.busy = false;
        sl.req.reset();
        S->failed++;
        S->cv_done.notify_all();
      }
      progressed = true;
    }
    if (!progressed) {
      bool any_busy = false;
      for (auto& sl : S->slots) any_busy |= sl.busy;
      // Poll running work every 20 us; sleep until a submission otherwise.
      if (any_busy)
        S->cv_work.wait_for(lk, std::chrono::microseconds(20));
      else
        S->cv_work.wait_for(lk, std::chrono::milliseconds(50));
    }
  }
}

}  // namespace

extern "C" {

int sf_server_create(const sf_server_opts* opts, sf_server** out) {
  if (!opts || !out || (opts->n_scores && !opts->scores))
    return fail(SF_ERR_INVALID, "bad argument");
  std::unique_ptr<sf_server> S(new sf_server);
  S->dev = opts->device;
  if (opts->store && opts->store->dev != opts->device)
    return fail(SF_ERR_INVALID, "store on another device");
  S->store = opts->store;
  const uint32_t slots = opts->slots ? std::min<uint32_t>(opts->slots, 64) : 8;
  for (uint32_t q = 0; q < opts->n_scores; ++q) S->scores.push_back(opts->scores[q]);
  if (S->scores.empty()) S->scores.push_back(sf_affine_t{2, 4, 4, 2});
  for (uint32_t q = 0; q < slots; ++q) {
    Slot sl;
    int rc = make_context(S->dev, &sl.ctx);
    if (rc) return rc;
    sl.ctx->store = S->store;
    sl.plan.reset(new sf_plan);
    sl.plan->ctx = sl.ctx;
    sl.plan->owns_ctx = true;
    CK(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
    S->slots.push_back(std::move(sl));
  }
  size_t free_b = 0, total_b = 0;
  CK(cudaMemGetInfo(&free_b, &total_b));
  S->budget = opts->hbm_budget ? opts->hbm_budget : (uint64_t)(0.9 * (double)free_b);
  sf_server* raw = S.get();
  S->dispatcher = std::thread(dispatch_loop, raw);
  *out = S.release();
  return SF_OK;
}

void sf_server_destroy(sf_server* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_work.notify_all();
  if (S->dispatcher.joinable()) S->dispatcher.join();
  cudaSetDevice(S->dev);
  for (auto& sl : S->slots) {
    if (sl.ctx) cudaStreamSynchronize(sl.ctx->s);
    if (sl.done) cudaEventDestroy(sl.done);
    sl.plan.reset();  // owns and deletes the slot's context
  }
  delete S;
}

int sf_server_submit(sf_server* S, const uint8_t* pool, uint64_t pool_bytes, const sf_job_t* jobs,
                     uint64_t count, uint64_t* ticket) {
  if (!S || !ticket || (count && !jobs) || (pool_bytes && !pool))
    return fail(SF_ERR_INVALID, "bad argument");
  auto req = std::make_shared<Request>();
  int rc = jobs_to_passes(jobs, count, S->scores.data(), (uint32_t)S->scores.size(), pool_bytes,
                          req->passes, S->store);
  if (rc) return rc;
  req->pool = pool;
  req->pool_bytes = pool_bytes;
  req->estimate = plan_bytes_estimate(req->passes, pool_bytes);
  if (req->estimate > S->budget)
    return fail(SF_ERR_NOMEM, "request needs more device memory than the server's budget");
  req->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    req->ticket = S->next_ticket++;
    S->requests[req->ticket] = req;
    S->pending.push_back(req);
    S->submitted++;
    *ticket = req->ticket;
  }
  S->cv_work.notify_all();
  return SF_OK;
}

int sf_server_wait(sf_server* S, uint64_t ticket, int32_t timeout_ms, sf_result_t* results,
                   uint32_t* ops, uint64_t ops_cap, uint64_t* ops_used, sf_request_stats* stats) {
  if (!S) return fail(SF_ERR_INVALID, "bad argument");
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->requests.find(ticket);
  if (it == S->requests.end()) return fail(SF_ERR_INVALID, "unknown ticket");
  std::shared_ptr<Request> req = it->second;
  const auto deadline = Clock::now() + std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
  while (req->state != R_DONE) {
    if (S->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && req->state != R_DONE)
      return fail(SF_ERR_TIMEOUT, "request not finished within the timeout");
  }
  if (ops_used) *ops_used = req->ops.size();
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    stats->queue_ms = req->slot >= 0 ? ms_between(req->t_submit, req->t_admit) : 0.0;
    stats->run_ms = req->slot >= 0 ? ms_between(req->t_admit, req->t_done) : 0.0;
    stats->total_ms = ms_between(req->t_submit, req->t_done);
    stats->cells = req->cells;
    stats->slot = (uint32_t)req->slot;
    stats->status = req->rc;
  }
  if (req->rc != SF_OK) {
    const int rc = req->rc;
    const std::string msg = req->msg;
    S->requests.erase(it);
    return fail(rc, msg);
  }
  if (!req->results.empty() && !results) return fail(SF_ERR_INVALID, "null results");
  if (!req->ops.empty() && (!ops || ops_cap < req->ops.size()))
    return fail(SF_ERR_CAPACITY, "ops buffer smaller than the request's CIGARs");
  if (!req->results.empty())
    std::memcpy(results, req->results.data(), req->results.size() * sizeof(sf_result_t));
  if (!req->ops.empty()) std::memcpy(ops, req->ops.data(), req->ops.size() * 4);
  S->requests.erase(it);
  return SF_OK;
}

int sf_server_query(sf_server* S, sf_server_stats* out) {
  if (!S || !out) return fail(SF_ERR_INVALID, "bad argument");
  std::lock_guard<std::mutex> lk(S->mu);
  std::memset(out, 0, sizeof *out);
  out->submitted = S->submitted;
  out->completed = S->completed;
  out->failed = S->failed;
  out->cells = S->cells;
  out->hbm_budget = S->budget;
  out->hbm_held = held_bytes(S);
  out->pending = (uint32_t)S->pending.size();
  for (auto& sl : S->slots) out->busy_slots += sl.busy ? 1 : 0;
  out->slots = (uint32_t)S->slots.size();
  return SF_OK;
}

}  // extern "C"
