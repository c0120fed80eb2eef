// Request server for steady heat-conduction solves (assemble + PCG), the
// serving form of solveTemperature (src/heat.jl:1020-1084).
//
// Two forms share the request queue, admission and result hand-off:
//
// Continuous batching (llf_server_create_batched).  Preparation threads,
// each with its own context, take requests in arrival order as the memory
// budget allows, upload the mesh, build the pattern, assemble and run the
// first CG steps (llf_engine::prepare).  One engine thread owns the CG
// iterations of every prepared request: the requests live in the slots of
// a device-resident engine (engine.h) that replays one captured graph of
// 16 iterations over all admitted systems; between replays it retires the
// converged ones (result to the host, memory released) and admits those
// that became ready meanwhile, so a request that arrives while others
// iterate joins the next replay.  A request's iterates are those of a lone
// llf_pcg solve bit for bit.
//
// Worker pool (llf_server_create).  N worker threads, each with its own
// llf_ctx (one CUDA stream).  Submitted
// requests are copied into the server and queued in arrival order; a worker
// takes the oldest request whose device-memory estimate fits in what is left
// of the budget (admission by HBM footprint), so small requests keep flowing
// while a large one waits for memory.  Requests in flight on different
// workers overlap on the device.  Every kernel of the pipeline is
// deterministic, so a request's result does not depend on what else is in
// flight.  Completion is signalled per ticket; latency is measured from
// submission to the moment the result is on the host.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/llfem_gb300.h"
#include "engine.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t ticket = 0;
  int dim = 0, family = 0, order = 0, npe = 0, ptype = 0, precond = 0;
  int64_t non = 0, nel = 0, maxiter = 0;
  double k = 0.0, thickness = 1.0, reltol = 1e-10;
  std::vector<double> xyz, rhs, x;
  std::vector<int64_t> conn;
  std::vector<uint8_t> fixed;
  int64_t footprint = 0;
  Clock::time_point submitted;
};

struct Result {
  bool done = false;
  int status = 0;
  std::string error;
  std::vector<double> x;
  int64_t iters = 0;
  double relres = 0.0, latency_s = 0.0, service_s = 0.0;
};

}  // namespace

namespace {
// A prepared request waiting for (or holding) an engine slot.
struct Job {
  std::unique_ptr<Request> req;
  llf_mesh *mesh = nullptr;
  llf_pattern *pat = nullptr;
  llf_matrix *K = nullptr;
  llf_engine::System *sys = nullptr;
  Clock::time_point started;
};
}  // namespace

struct llf_server {
  int device = 0;
  int64_t budget = 0, in_use = 0;
  bool stopping = false;
  int64_t next_ticket = 1;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_engine;
  std::deque<std::unique_ptr<Request>> queue;
  std::map<int64_t, Result> results;
  std::vector<std::thread> workers;
  int64_t served = 0, peak_in_use = 0;
  // continuous batching
  bool batched = false;
  int max_systems = 0;
  int preparing = 0;                // requests taken by preparation threads, not yet handed over
  std::deque<std::unique_ptr<Job>> ready;
  std::thread engine;
  // where the time goes (seconds summed over threads)
  double t_prep = 0.0, t_step = 0.0, t_collect = 0.0, t_idle = 0.0;
  int64_t replays = 0, admitted_sum = 0;
};

namespace {

// Device bytes of one request: mesh (with the affine geometry kept on it,
// 81 bytes per element), pattern (node adjacency bounded by nel*npe^2
// blocks, and its stored layout), values, stored form and the CG vectors.
int64_t estimate_footprint(const Request &r) {
  const int64_t nnz_bound = std::min<int64_t>(r.nel * (int64_t)r.npe * r.npe, r.non * r.non);
  return r.non * 24 + r.nel * r.npe * 16 + r.nel * 88 + nnz_bound * (4 + 8 + 16 + 8) +
         r.nel * (int64_t)r.npe * r.npe * 8 + r.non * 8 * 13 + (64 << 20);
}

void finish(llf_server *s, int64_t ticket, Result &&res, int64_t footprint) {
  std::lock_guard<std::mutex> lock(s->mu);
  s->in_use -= footprint;
  s->served++;
  s->results[ticket] = std::move(res);
  s->cv_done.notify_all();
  s->cv_work.notify_all();
}

void serve_one(llf_ctx *ctx, Request &r, Result &res) {
  llf_mesh *mesh = nullptr;
  llf_pattern *pat = nullptr;
  llf_matrix *K = nullptr;
  int64_t nnz = 0;
  int rc = llf_mesh_upload(ctx, r.dim, r.non, r.xyz.data(), r.nel, r.npe, r.conn.data(), r.family, r.order, &mesh);
  if (rc == LLF_OK) rc = llf_pattern_build(ctx, mesh, 1, &nnz, &pat);
  if (rc == LLF_OK) rc = llf_assemble_heat(ctx, mesh, pat, r.ptype, &r.k, 1, r.thickness, LLF_FP64, &K);
  if (rc == LLF_OK) {
    res.x = r.x;
    rc = llf_pcg(ctx, K, r.rhs.data(), res.x.data(), r.fixed.data(), r.precond, r.reltol, r.maxiter, &res.iters,
                 &res.relres);
  }
  res.status = rc;
  if (rc != LLF_OK) res.error = llf_last_error(ctx);
  llf_matrix_destroy(ctx, K);
  llf_pattern_destroy(ctx, pat);
  llf_mesh_destroy(ctx, mesh);
}

// Take the oldest queued request that fits the remaining budget (an
// oversized one runs once nothing else holds memory); null when stopping.
std::unique_ptr<Request> take_request(llf_server *s) {
  std::unique_lock<std::mutex> lock(s->mu);
  for (;;) {
    if (s->stopping && s->queue.empty()) return nullptr;
    auto it = std::find_if(s->queue.begin(), s->queue.end(), [&](const std::unique_ptr<Request> &q) {
      return s->in_use + q->footprint <= s->budget || s->in_use == 0;
    });
    if (it != s->queue.end()) {
      std::unique_ptr<Request> req = std::move(*it);
      s->queue.erase(it);
      s->in_use += req->footprint;
      s->peak_in_use = std::max(s->peak_in_use, s->in_use);
      if (s->batched) s->preparing++;
      return req;
    }
    s->cv_work.wait(lock);
  }
}

void destroy_job_objects(llf_ctx *ctx, Job &j) {
  llf_matrix_destroy(ctx, j.K);
  llf_pattern_destroy(ctx, j.pat);
  llf_mesh_destroy(ctx, j.mesh);
  j.K = nullptr;
  j.pat = nullptr;
  j.mesh = nullptr;
}

// Preparation thread of the batched server: mesh, pattern, assembly and the
// first CG steps on its own context; the job then goes to the engine.
void prep_main(llf_server *s) {
  llf_ctx *ctx = nullptr;
  int crc = llf_ctx_create(s->device, &ctx);
  for (;;) {
    std::unique_ptr<Request> req = take_request(s);
    if (!req) break;
    auto job = std::make_unique<Job>();
    job->started = Clock::now();
    Request &r = *req;
    int rc = crc;
    int64_t nnz = 0;
    if (rc == LLF_OK)
      rc = llf_mesh_upload(ctx, r.dim, r.non, r.xyz.data(), r.nel, r.npe, r.conn.data(), r.family, r.order,
                           &job->mesh);
    if (rc == LLF_OK) rc = llf_pattern_build(ctx, job->mesh, 1, &nnz, &job->pat);
    if (rc == LLF_OK) rc = llf_assemble_heat(ctx, job->mesh, job->pat, r.ptype, &r.k, 1, r.thickness, LLF_FP64, &job->K);
    if (rc == LLF_OK)
      rc = llf_engine::prepare(ctx, job->K, r.rhs.data(), r.x.data(), r.fixed.data(), r.precond, r.reltol,
                               r.maxiter, &job->sys);
    if (rc != LLF_OK) {
      Result res;
      res.done = true;
      res.status = rc;
      res.error = crc != LLF_OK ? "preparation thread has no CUDA context" : llf_last_error(ctx);
      auto t1 = Clock::now();
      res.service_s = std::chrono::duration<double>(t1 - job->started).count();
      res.latency_s = std::chrono::duration<double>(t1 - r.submitted).count();
      if (ctx) destroy_job_objects(ctx, *job);
      {
        std::lock_guard<std::mutex> lock(s->mu);
        s->preparing--;
      }
      finish(s, r.ticket, std::move(res), r.footprint);
      s->cv_engine.notify_all();
      continue;
    }
    job->req = std::move(req);
    {
      std::lock_guard<std::mutex> lock(s->mu);
      s->preparing--;
      s->t_prep += std::chrono::duration<double>(Clock::now() - job->started).count();
      s->ready.push_back(std::move(job));
    }
    s->cv_engine.notify_all();
  }
  if (ctx) llf_ctx_destroy(ctx);
}

// The engine thread: admits ready jobs between replays, replays, retires.
void engine_main(llf_server *s) {
  llf_ctx *ctx = nullptr;
  llf_engine::Engine *eng = nullptr;
  int crc = llf_ctx_create(s->device, &ctx);
  if (crc == LLF_OK) crc = llf_engine::create(ctx, s->max_systems, (int64_t)1 << 20, &eng);
  std::string cerr = crc == LLF_OK ? "" : (ctx ? llf_last_error(ctx) : "engine has no CUDA context");
  std::deque<std::unique_ptr<Job>> pending;
  std::map<int64_t, std::unique_ptr<Job>> inflight;
  auto fail_job = [&](std::unique_ptr<Job> &j, int rc, const std::string &msg) {
    Result res;
    res.done = true;
    res.status = rc;
    res.error = msg;
    if (ctx) {
      if (j->sys) llf_engine::release(ctx, j->sys);
      j->sys = nullptr;
      destroy_job_objects(ctx, *j);
    }
    finish(s, j->req->ticket, std::move(res), j->req->footprint);
  };
  for (;;) {
    {
      std::unique_lock<std::mutex> lock(s->mu);
      const auto w0 = Clock::now();
      for (;;) {
        while (!s->ready.empty()) {
          pending.push_back(std::move(s->ready.front()));
          s->ready.pop_front();
        }
        if (!pending.empty() || !inflight.empty()) break;
        if (s->stopping && s->queue.empty() && s->preparing == 0) break;
        s->cv_engine.wait(lock);
      }
      s->t_idle += std::chrono::duration<double>(Clock::now() - w0).count();
      if (pending.empty() && inflight.empty()) break;
    }
    if (crc != LLF_OK) {
      while (!pending.empty()) {
        fail_job(pending.front(), crc, cerr);
        pending.pop_front();
      }
      continue;
    }
    // admit in arrival order while slots and chunk room last
    while (!pending.empty()) {
      std::unique_ptr<Job> &j = pending.front();
      const int a = llf_engine::admit(eng, j->sys, j->req->ticket);
      if (a < 0) {
        fail_job(j, a, llf_last_error(ctx));
        pending.pop_front();
        continue;
      }
      if (a == 0) break;
      j->sys = nullptr;   // owned by the engine now
      inflight[j->req->ticket] = std::move(j);
      pending.pop_front();
    }
    if (inflight.empty()) continue;
    std::vector<llf_engine::Done> done;
    const auto t0 = Clock::now();
    const int nadm = llf_engine::admitted(eng);
    int rc = llf_engine::step(eng);
    const auto t1 = Clock::now();
    if (rc == LLF_OK) rc = llf_engine::collect(eng, done);
    {
      std::lock_guard<std::mutex> lock(s->mu);
      s->t_step += std::chrono::duration<double>(t1 - t0).count();
      s->t_collect += std::chrono::duration<double>(Clock::now() - t1).count();
      s->replays++;
      s->admitted_sum += nadm;
    }
    if (rc != LLF_OK) {  // a device error: fail everything in flight and start a fresh engine
      const std::string msg = llf_last_error(ctx);
      llf_engine::destroy(eng);
      eng = nullptr;
      for (auto &kv : inflight) fail_job(kv.second, rc, msg);
      inflight.clear();
      crc = llf_engine::create(ctx, s->max_systems, (int64_t)1 << 20, &eng);
      if (crc != LLF_OK) cerr = llf_last_error(ctx);
      continue;
    }
    for (auto &d : done) {
      auto it = inflight.find(d.tag);
      if (it == inflight.end()) continue;
      std::unique_ptr<Job> j = std::move(it->second);
      inflight.erase(it);
      Result res;
      res.done = true;
      res.status = d.status;
      if (d.status == LLF_ERR_NUMERIC)
        res.error = "pcg: breakdown (u.Au <= 0): matrix not positive definite on the free DoFs";
      else if (d.status == LLF_ERR_NOT_CONVERGED)
        res.error = "pcg: not converged after " + std::to_string(d.iters) + " iterations";
      res.x = std::move(d.x);
      res.iters = d.iters;
      res.relres = d.relres;
      auto t1 = Clock::now();
      res.service_s = std::chrono::duration<double>(t1 - j->started).count();
      res.latency_s = std::chrono::duration<double>(t1 - j->req->submitted).count();
      destroy_job_objects(ctx, *j);
      finish(s, j->req->ticket, std::move(res), j->req->footprint);
    }
  }
  if (eng) llf_engine::destroy(eng);
  if (ctx) llf_ctx_destroy(ctx);
}

void worker_main(llf_server *s) {
  llf_ctx *ctx = nullptr;
  int crc = llf_ctx_create(s->device, &ctx);
  for (;;) {
    std::unique_ptr<Request> req = take_request(s);
    if (!req) break;
    Result res;
    auto t0 = Clock::now();
    if (crc != LLF_OK) {
      res.status = crc;
      res.error = "worker has no CUDA context";
    } else {
      serve_one(ctx, *req, res);
    }
    auto t1 = Clock::now();
    res.done = true;
    res.service_s = std::chrono::duration<double>(t1 - t0).count();
    res.latency_s = std::chrono::duration<double>(t1 - req->submitted).count();
    finish(s, req->ticket, std::move(res), req->footprint);
  }
  if (ctx) llf_ctx_destroy(ctx);
}

}  // namespace

extern "C" {

int llf_server_create(int device, int nworkers, int64_t mem_budget_bytes, llf_server **out) {
  if (!out || nworkers < 1 || nworkers > 64 || mem_budget_bytes <= 0) return LLF_ERR_ARG;
  auto *s = new llf_server();
  s->device = device;
  s->budget = mem_budget_bytes;
  for (int i = 0; i < nworkers; ++i) s->workers.emplace_back(worker_main, s);
  *out = s;
  return LLF_OK;
}

int llf_server_create_batched(int device, int nprep, int max_systems, int64_t mem_budget_bytes, llf_server **out) {
  if (!out || nprep < 1 || nprep > 64 || max_systems < 1 || max_systems > 65536 || mem_budget_bytes <= 0)
    return LLF_ERR_ARG;
  auto *s = new llf_server();
  s->device = device;
  s->budget = mem_budget_bytes;
  s->batched = true;
  s->max_systems = max_systems;
  s->engine = std::thread(engine_main, s);
  for (int i = 0; i < nprep; ++i) s->workers.emplace_back(prep_main, s);
  *out = s;
  return LLF_OK;
}

int llf_server_submit_heat(llf_server *s, int dim, int64_t non, const double *xyz, int64_t nel, int npe,
                           const int64_t *conn, int family, int order, double k, double thickness,
                           const double *rhs, const double *x0, const uint8_t *fixed, int precond,
                           double reltol, int64_t maxiter, int64_t *ticket) {
  if (!s || !xyz || !conn || !x0 || !fixed || !ticket || non <= 0 || nel <= 0 || npe <= 0 || (dim != 2 && dim != 3))
    return LLF_ERR_ARG;
  auto r = std::make_unique<Request>();
  r->dim = dim;
  r->non = non;
  r->nel = nel;
  r->npe = npe;
  r->family = family;
  r->order = order;
  r->k = k;
  r->thickness = thickness;
  r->ptype = dim == 3 ? LLF_HEAT_CONDUCTION : LLF_PLANE_HEAT_CONDUCTION;
  r->precond = precond;
  r->reltol = reltol;
  r->maxiter = maxiter > 0 ? maxiter : 20 * non;
  r->xyz.assign(xyz, xyz + 3 * non);
  r->conn.assign(conn, conn + nel * npe);
  r->x.assign(x0, x0 + non);
  r->fixed.assign(fixed, fixed + non);
  r->rhs.assign(non, 0.0);
  if (rhs) std::memcpy(r->rhs.data(), rhs, sizeof(double) * non);
  r->footprint = estimate_footprint(*r);
  r->submitted = Clock::now();
  std::lock_guard<std::mutex> lock(s->mu);
  r->ticket = s->next_ticket++;
  *ticket = r->ticket;
  s->results[r->ticket] = Result{};
  s->queue.push_back(std::move(r));
  s->cv_work.notify_one();
  s->cv_engine.notify_all();
  return LLF_OK;
}

// Wait (up to timeout_s; < 0 = forever) for a ticket and take its result:
// x[non] solution, iters, relres, latency (submission -> result on host) and
// service time (worker start -> result).  Returns LLF_ERR_STATE on timeout
// or unknown ticket, else the request's own status.
int llf_server_wait(llf_server *s, int64_t ticket, double timeout_s, double *x, int64_t *iters, double *relres,
                    double *latency_s, double *service_s, char *err, int64_t errlen) {
  if (!s) return LLF_ERR_ARG;
  std::unique_lock<std::mutex> lock(s->mu);
  auto ready = [&] {
    auto it = s->results.find(ticket);
    return it == s->results.end() || it->second.done;
  };
  if (timeout_s < 0)
    s->cv_done.wait(lock, ready);
  else if (!s->cv_done.wait_for(lock, std::chrono::duration<double>(timeout_s), ready))
    return LLF_ERR_STATE;
  auto it = s->results.find(ticket);
  if (it == s->results.end()) return LLF_ERR_STATE;
  Result r = std::move(it->second);
  s->results.erase(it);
  lock.unlock();
  if (x && !r.x.empty()) std::memcpy(x, r.x.data(), sizeof(double) * r.x.size());
  if (iters) *iters = r.iters;
  if (relres) *relres = r.relres;
  if (latency_s) *latency_s = r.latency_s;
  if (service_s) *service_s = r.service_s;
  if (err && errlen > 0) {
    size_t n = std::min((size_t)(errlen - 1), r.error.size());
    std::memcpy(err, r.error.data(), n);
    err[n] = 0;
  }
  return r.status;
}

int llf_server_stats(llf_server *s, int64_t *queued, int64_t *served, int64_t *bytes_in_use, int64_t *peak_bytes) {
  if (!s) return LLF_ERR_ARG;
  std::lock_guard<std::mutex> lock(s->mu);
  if (queued) *queued = (int64_t)s->queue.size();
  if (served) *served = s->served;
  if (bytes_in_use) *bytes_in_use = s->in_use;
  if (peak_bytes) *peak_bytes = s->peak_in_use;
  return LLF_OK;
}

int llf_server_timing(llf_server *s, double *prep_s, double *step_s, double *collect_s, double *idle_s,
                      int64_t *replays, double *mean_admitted) {
  if (!s) return LLF_ERR_ARG;
  std::lock_guard<std::mutex> lock(s->mu);
  if (prep_s) *prep_s = s->t_prep;
  if (step_s) *step_s = s->t_step;
  if (collect_s) *collect_s = s->t_collect;
  if (idle_s) *idle_s = s->t_idle;
  if (replays) *replays = s->replays;
  if (mean_admitted) *mean_admitted = s->replays ? (double)s->admitted_sum / (double)s->replays : 0.0;
  return LLF_OK;
}

int llf_server_destroy(llf_server *s) {
  if (!s) return LLF_OK;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stopping = true;
    s->cv_work.notify_all();
  }
  for (auto &t : s->workers) t.join();
  if (s->engine.joinable()) {
    s->cv_engine.notify_all();
    s->engine.join();
  }
  delete s;
  return LLF_OK;
}

}  // extern "C"
