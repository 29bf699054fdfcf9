// Request loop: many Davidson solves on one GPU at once.
//
// An SQD-style caller emits diagonalisation requests of uneven sizes.  The
// server keeps a queue of them and a fixed set of worker threads, each with
// its own context and CUDA stream, so that the kernels of several solves run
// on the device at the same time (continuous batching: a request that arrives
// while others run starts as soon as a worker and enough HBM are free).
//
// Admission is by HBM footprint.  At submission a request reserves an upper
// bound of its device memory (solve_footprint with every other string counted
// as a possible excitation); once its tables are built the reservation shrinks
// to the bound with the real table sizes, which lets queued requests in.  A
// worker takes the first queued request that fits; a request that has been
// passed over max_bypass times blocks the ones behind it, so a large request
// is not starved by a stream of small ones.  Each worker context's own budget
// equals its request's reservation, so a request can never use more memory
// than it reserved (it fails with SBDGB_E_NOMEM instead).
//
// Device memory comes from one stream-ordered pool shared by the workers
// (allocation and release synchronise nothing beyond the worker's stream);
// sigma tile shapes come from the problem size, not from timing runs, since
// timings taken while other solves run are not meaningful.
//
// Small requests are batched: a worker that takes a request of at most
// kBatchMaxN determinants also takes the other queued small requests with the
// same solver options (up to kBatchMax, within the HBM left) and solves them
// together with sbdgb_batch_davidson, all in lock step, one graph launch per
// Davidson iteration.  That is the same algorithm as sbdgb_davidson (the
// mixed form is the two-phase one), so a request's energies agree with a lone
// solve to rounding (~1e-13), and its result does not otherwise depend on what
// else runs.
//
// Each solve is the same computation as sbdgb_davidson on a lone problem: the
// result of a request does not depend on what else runs.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <thread>
#include <unordered_map>

#include "common.cuh"

namespace {

using Clock = std::chrono::steady_clock;

double secs(Clock::time_point a, Clock::time_point b) { return std::chrono::duration<double>(b - a).count(); }

// Upper bound of one spin's excitation-table entries before the tables exist:
// per bra string at most the other strings of the list, and at most the
// strings at Hamming distance 2 (singles) or 4 (doubles).
uint64_t entry_bound(size_t n, int norb, int nocc) {
  const double s = (double)nocc * (norb - nocc);
  const double d = 0.25 * nocc * (nocc - 1) * (double)(norb - nocc) * (norb - nocc - 1);
  const double per = std::min<double>(n ? (double)(n - 1) : 0.0, s + d);
  return (uint64_t)(per * (double)n);
}

constexpr size_t kSlack = size_t(1) << 20;  // allocation rounding and small staging buffers
constexpr uint64_t kBatchMaxN = 300000;      // requests up to this many determinants are batched
constexpr int kBatchMax = 64;                // requests per batched solve

struct Request {
  uint64_t ticket = 0;
  int norb = 0;
  std::vector<uint64_t> a, b;
  std::vector<double> h1, eri;
  double ecore = 0.0;
  sbdgb_davidson_opts o{};
  double *X = nullptr;
  size_t reserve = 0;
  int bypassed = 0;
  Clock::time_point t_submit, t_start, t_end;
  sbdgb_result res{};
  bool done = false;
};

void set_message(sbdgb_result &r, const std::string &m) {
  std::strncpy(r.message, m.c_str(), sizeof(r.message) - 1);
  r.message[sizeof(r.message) - 1] = 0;
}

}  // namespace

struct sbdgb_server {
  int device = 0;
  size_t budget = 0, reserved = 0, peak_reserved = 0;
  int running = 0, peak_running = 0, max_bypass = 8;
  cudaMemPool_t pool = nullptr;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
  uint64_t next = 1, submitted = 0, completed = 0, failed = 0, launches = 0, batched = 0;
  bool stop = false;
  std::vector<sbdgb_ctx *> ctxs;
  std::vector<std::thread> threads;
  std::string last_error;
};

namespace {

// First queued request that fits the budget (called with the lock held).
Request *admit(sbdgb_server *S) {
  for (size_t i = 0; i < S->queue.size(); ++i) {
    Request *r = S->queue[i];
    if (S->reserved + r->reserve <= S->budget) {
      for (size_t j = 0; j < i; ++j) S->queue[j]->bypassed++;
      S->queue.erase(S->queue.begin() + (long)i);
      return r;
    }
    if (r->bypassed >= S->max_bypass) return nullptr;  // nothing may pass an aged request
  }
  return nullptr;
}

// Whether a request can join a batched solve (the batched solver's options:
// start on the lowest diagonal, subspace <= 32, no time limit, and for the
// mixed precision the two-phase form).
bool batchable(const Request *r) {
  const sbdgb_davidson_opts &o = r->o;
  return (uint64_t)r->a.size() * r->b.size() <= kBatchMaxN && o.init == 1 && o.max_nb <= 32 && o.max_time <= 0.0 &&
         (o.precision == SBDGB_FP64 || (o.precision == SBDGB_MIXED && o.refine_every == 0));
}

bool same_opts(const Request *x, const Request *y) {
  const sbdgb_davidson_opts &a = x->o, &b = y->o;
  return a.nroots == b.nroots && a.max_nb == b.max_nb && a.max_it == b.max_it && a.eps == b.eps &&
         a.precision == b.precision && a.refine_every == b.refine_every && a.init == b.init;
}

// The queued requests that can join r's batched solve (called with the lock
// held; r is admitted already).  Stops at an aged request that does not join.
void gather(sbdgb_server *S, Request *r, std::vector<Request *> &group) {
  group.assign(1, r);
  if (!batchable(r)) return;
  size_t reserved = S->reserved + r->reserve;
  for (size_t i = 0; i < S->queue.size() && (int)group.size() < kBatchMax;) {
    Request *q = S->queue[i];
    if (batchable(q) && same_opts(q, r) && reserved + q->reserve <= S->budget) {
      reserved += q->reserve;
      group.push_back(q);
      S->queue.erase(S->queue.begin() + (long)i);
      continue;
    }
    if (q->bypassed >= S->max_bypass) break;
    ++i;
  }
}

void finish_result(Request *r, int status, const std::string &msg, const double *E, const sbdgb_report &rep,
                   int wid) {
  sbdgb_result &res = r->res;
  res.status = status;
  if (status != SBDGB_OK) set_message(res, msg);
  res.nroots = r->o.nroots;
  for (int j = 0; j < r->o.nroots && j < 8; ++j) {
    res.energies[j] = E ? E[j] : 0.0;
    res.resid[j] = rep.resid[j];
  }
  res.iterations = rep.iterations;
  res.sigma_calls = rep.sigma_calls;
  res.converged = rep.converged;
  res.worker = wid;
  res.reserved_bytes = r->reserve;
  res.ndet = (uint64_t)r->a.size() * r->b.size();
}

// Several small requests in one batched solve on the worker's context.
void run_batch(sbdgb_server *S, std::vector<Request *> &group, sbdgb_ctx *ctx, int wid) {
  sbdgb::Ctx &c = ctx->c;
  const uint64_t launches0 = c.launches;
  size_t budget = 0;
  for (Request *r : group) budget += r->reserve;
  c.budget = budget;
  std::vector<sbdgb_problem *> ps;
  std::vector<Request *> live;
  for (Request *r : group) {
    sbdgb_problem *p = nullptr;
    int rc = sbdgb_problem_create(ctx, r->norb, r->a.data(), r->a.size(), r->b.data(), r->b.size(), r->h1.data(),
                                  r->eri.data(), r->ecore, &p);
    if (rc == SBDGB_OK) rc = sbdgb_build_tables(p);
    if (rc == SBDGB_OK) rc = sbdgb_diag_terms(p, nullptr);
    if (rc != SBDGB_OK) {
      finish_result(r, rc, c.last_error, nullptr, sbdgb_report{}, wid);
      if (p) sbdgb_problem_destroy(p);
      continue;
    }
    ps.push_back(p);
    live.push_back(r);
  }
  if (!live.empty()) {
    const int k = live[0]->o.nroots, n = (int)live.size();
    std::vector<double> E((size_t)n * k);
    std::vector<sbdgb_report> reps(n);
    std::vector<double *> X(n);
    bool any_x = false;
    for (int i = 0; i < n; ++i) {
      X[i] = live[i]->X;
      any_x = any_x || X[i];
    }
    const int rc = sbdgb_batch_davidson(ctx, ps.data(), n, &live[0]->o, E.data(), reps.data(),
                                        any_x ? X.data() : nullptr);
    for (int i = 0; i < n; ++i)
      finish_result(live[i], rc, c.last_error, E.data() + (size_t)i * k, rc == SBDGB_OK ? reps[i] : sbdgb_report{},
                    wid);
  }
  for (sbdgb_problem *p : ps) sbdgb_problem_destroy(p);
  cudaStreamSynchronize(c.stream);  // the pool frees are done before the reservations go
  cudaGetLastError();
  c.in_use = 0;
  std::lock_guard<std::mutex> lk(S->mu);
  S->launches += c.launches - launches0;
}

void run_request(sbdgb_server *S, Request *r, sbdgb_ctx *ctx, int wid) {
  sbdgb::Ctx &c = ctx->c;
  sbdgb_result &res = r->res;
  const uint64_t launches0 = c.launches;
  c.budget = r->reserve;
  sbdgb_problem *p = nullptr;
  int rc = sbdgb_problem_create(ctx, r->norb, r->a.data(), r->a.size(), r->b.data(), r->b.size(), r->h1.data(),
                                r->eri.data(), r->ecore, &p);
  if (rc == SBDGB_OK) rc = sbdgb_build_tables(p);
  if (rc == SBDGB_OK) {
    // shrink (or, if the bound was too small, grow) the reservation to the real table sizes
    const size_t need = sbdgb::solve_footprint(r->norb, r->a.size(), r->b.size(), r->o, p->p.A.ns + p->p.A.nd,
                                               p->p.B.ns + p->p.B.nd) + kSlack;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      if (need <= r->reserve) {
        S->reserved -= r->reserve - need;
        r->reserve = need;
      } else if (S->reserved + (need - r->reserve) <= S->budget) {
        S->reserved += need - r->reserve;
        r->reserve = need;
        S->peak_reserved = std::max(S->peak_reserved, S->reserved);
      } else {
        rc = SBDGB_E_NOMEM;
        c.last_error = "excitation tables larger than the HBM left for the request";
      }
      c.budget = r->reserve;
    }
    S->cv_work.notify_all();
  }
  if (rc == SBDGB_OK) rc = sbdgb_diag_terms(p, nullptr);
  double E[16] = {};
  sbdgb_report rep{};
  if (rc == SBDGB_OK) rc = sbdgb_davidson(p, &r->o, E, r->X, &rep);
  res.status = rc;
  if (rc != SBDGB_OK) set_message(res, c.last_error);
  res.nroots = r->o.nroots;
  for (int j = 0; j < r->o.nroots && j < 8; ++j) {
    res.energies[j] = E[j];
    res.resid[j] = rep.resid[j];
  }
  res.iterations = rep.iterations;
  res.sigma_calls = rep.sigma_calls;
  res.converged = rep.converged;
  res.worker = wid;
  res.reserved_bytes = r->reserve;
  res.ndet = (uint64_t)r->a.size() * r->b.size();
  if (p) sbdgb_problem_destroy(p);
  cudaStreamSynchronize(c.stream);  // the pool frees are done before the reservation goes
  cudaGetLastError();
  c.in_use = 0;
  std::lock_guard<std::mutex> lk(S->mu);
  S->launches += c.launches - launches0;
}

void worker_loop(sbdgb_server *S, int wid) {
  sbdgb_ctx *ctx = S->ctxs[(size_t)wid];
  cudaSetDevice(S->device);
  std::vector<Request *> group;
  for (;;) {
    Request *r = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_work.wait(lk, [&] { return S->stop || (r = admit(S)) != nullptr; });
      if (!r) return;  // stopping, nothing admitted
      gather(S, r, group);
      const auto now = Clock::now();
      for (Request *q : group) {
        S->reserved += q->reserve;
        q->t_start = now;
      }
      S->peak_reserved = std::max(S->peak_reserved, S->reserved);
      S->running += (int)group.size();
      if (group.size() > 1) S->batched += group.size();
      S->peak_running = std::max(S->peak_running, S->running);
    }
    if (group.size() == 1)
      run_request(S, r, ctx, wid);
    else
      run_batch(S, group, ctx, wid);
    {
      std::lock_guard<std::mutex> lk(S->mu);
      const auto now = Clock::now();
      for (Request *q : group) {
        q->t_end = now;
        q->res.queue_seconds = secs(q->t_submit, q->t_start);
        q->res.run_seconds = secs(q->t_start, q->t_end);
        q->res.total_seconds = secs(q->t_submit, q->t_end);
        S->reserved -= q->reserve;
        S->running--;
        S->completed++;
        if (q->res.status != SBDGB_OK) S->failed++;
        q->done = true;
      }
    }
    S->cv_done.notify_all();
    S->cv_work.notify_all();
  }
}

}  // namespace

extern "C" {

int sbdgb_server_create(int device, int workers, size_t hbm_budget_bytes, sbdgb_server **out) {
  if (!out || workers < 1 || workers > 64) return SBDGB_E_INPUT;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    return SBDGB_E_CUDA;
  }
  auto S = std::make_unique<sbdgb_server>();
  S->device = device;
  S->max_bypass = 2 * workers;
  if (cudaSetDevice(device) != cudaSuccess) return SBDGB_E_CUDA;
  size_t freeb = 0, total = 0;
  if (cudaMemGetInfo(&freeb, &total) != cudaSuccess) return SBDGB_E_CUDA;
  S->budget = hbm_budget_bytes ? std::min(hbm_budget_bytes, freeb) : freeb / 10 * 9;
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  if (cudaMemPoolCreate(&S->pool, &props) != cudaSuccess) {
    cudaGetLastError();
    return SBDGB_E_CUDA;
  }
  // keep released memory in the pool; never make one worker's stream wait for another's frees
  uint64_t keep = ~0ull;
  int no = 0;
  cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  cudaMemPoolSetAttribute(S->pool, cudaMemPoolReuseAllowInternalDependencies, &no);
  for (int w = 0; w < workers; ++w) {
    sbdgb_ctx *ctx = nullptr;
    int rc = sbdgb_ctx_create(&ctx, device, 0);
    if (rc != SBDGB_OK) {
      for (sbdgb_ctx *c : S->ctxs) sbdgb_ctx_destroy(c);
      cudaMemPoolDestroy(S->pool);
      return rc;
    }
    ctx->c.pool = S->pool;
    ctx->c.autotune = false;
    S->ctxs.push_back(ctx);
  }
  sbdgb_server *raw = S.release();
  for (int w = 0; w < workers; ++w) raw->threads.emplace_back(worker_loop, raw, w);
  *out = raw;
  return SBDGB_OK;
}

int sbdgb_server_submit(sbdgb_server *S, const sbdgb_request *q, uint64_t *ticket) {
  if (!S || !q || !ticket) return SBDGB_E_INPUT;
  auto fail = [&](int st, const std::string &m) {
    std::lock_guard<std::mutex> lk(S->mu);
    S->last_error = m;
    return st;
  };
  if (q->norb < 1 || q->norb > 64) return fail(SBDGB_E_UNSUPPORTED, "norb must be in [1, 64]");
  if (!q->astr || !q->bstr || !q->h1 || !q->eri_packed || q->na == 0 || q->nb == 0)
    return fail(SBDGB_E_INPUT, "null or empty request input");
  if (q->opts.nroots < 1 || q->opts.nroots > 8) return fail(SBDGB_E_UNSUPPORTED, "nroots must be in [1, 8]");
  auto r = std::make_unique<Request>();
  r->norb = q->norb;
  r->o = q->opts;
  r->o.verbose = 0;
  r->X = q->vectors_out;
  const int nocc_a = __builtin_popcountll(q->astr[0]), nocc_b = __builtin_popcountll(q->bstr[0]);
  r->reserve = sbdgb::solve_footprint(q->norb, q->na, q->nb, r->o, entry_bound(q->na, q->norb, nocc_a),
                                      entry_bound(q->nb, q->norb, nocc_b)) +
               kSlack;
  if (r->reserve > S->budget)
    return fail(SBDGB_E_NOMEM, "request needs up to " + std::to_string(r->reserve) + " bytes; the budget is " +
                                   std::to_string(S->budget));
  const size_t L = (size_t)q->norb, npair = L * (L + 1) / 2;
  r->a.assign(q->astr, q->astr + q->na);
  r->b.assign(q->bstr, q->bstr + q->nb);
  r->h1.assign(q->h1, q->h1 + L * L);
  r->eri.assign(q->eri_packed, q->eri_packed + npair * (npair + 1) / 2);
  r->ecore = q->ecore;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) {
      S->last_error = "server is shutting down";
      return SBDGB_E_STATE;
    }
    r->ticket = S->next++;
    r->t_submit = Clock::now();
    *ticket = r->ticket;
    S->queue.push_back(r.get());
    S->reqs.emplace(r->ticket, std::move(r));
    S->submitted++;
  }
  S->cv_work.notify_one();
  return SBDGB_OK;
}

int sbdgb_server_poll(sbdgb_server *S, uint64_t ticket, int *done) {
  if (!S || !done) return SBDGB_E_INPUT;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) return SBDGB_E_INPUT;
  *done = it->second->done ? 1 : 0;
  return SBDGB_OK;
}

int sbdgb_server_wait(sbdgb_server *S, uint64_t ticket, double timeout_seconds, sbdgb_result *out) {
  if (!S) return SBDGB_E_INPUT;
  std::unique_lock<std::mutex> lk(S->mu);
  auto ready = [&] {
    auto it = S->reqs.find(ticket);
    return it == S->reqs.end() || it->second->done;
  };
  if (timeout_seconds < 0)
    S->cv_done.wait(lk, ready);
  else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_seconds), ready))
    return SBDGB_E_TIMEOUT;
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) {
    S->last_error = "unknown or already collected ticket";
    return SBDGB_E_INPUT;
  }
  if (out) *out = it->second->res;
  S->reqs.erase(it);
  return SBDGB_OK;
}

int sbdgb_server_stats(sbdgb_server *S, sbdgb_serve_stats *st) {
  if (!S || !st) return SBDGB_E_INPUT;
  std::lock_guard<std::mutex> lk(S->mu);
  st->submitted = S->submitted;
  st->completed = S->completed;
  st->failed = S->failed;
  st->launches = S->launches;
  st->budget_bytes = S->budget;
  st->reserved_bytes = S->reserved;
  st->peak_reserved_bytes = S->peak_reserved;
  st->workers = (int)S->threads.size();
  st->running = S->running;
  st->peak_running = S->peak_running;
  st->queued = (int)S->queue.size();
  st->batched = S->batched;
  return SBDGB_OK;
}

const char *sbdgb_server_last_error(const sbdgb_server *S) { return S ? S->last_error.c_str() : "null server"; }

void sbdgb_server_destroy(sbdgb_server *S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    for (Request *r : S->queue) {
      r->res.status = SBDGB_E_STATE;
      set_message(r->res, "server shut down before the request started");
      r->done = true;
      S->failed++;
    }
    S->queue.clear();
  }
  S->cv_work.notify_all();
  S->cv_done.notify_all();
  for (auto &t : S->threads) t.join();
  for (sbdgb_ctx *c : S->ctxs) sbdgb_ctx_destroy(c);
  cudaSetDevice(S->device);
  cudaMemPoolDestroy(S->pool);
  delete S;
}

}  // extern "C"
