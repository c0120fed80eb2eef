// Request server for steady heat-conduction solves (assemble + PCG), the
// serving form of solveTemperature (src/heat.jl:1020-1084).
//
// N worker threads, each with its own llf_ctx (one CUDA stream).  Submitted
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

struct llf_server {
  int device = 0;
  int64_t budget = 0, in_use = 0;
  bool stopping = false;
  int64_t next_ticket = 1;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::unique_ptr<Request>> queue;
  std::map<int64_t, Result> results;
  std::vector<std::thread> workers;
  int64_t served = 0, peak_in_use = 0;
};

namespace {

// Device bytes of one request: mesh, pattern (node adjacency bounded by
// nel*npe^2 blocks), values, stored form and the CG vectors.
int64_t estimate_footprint(const Request &r) {
  const int64_t nnz_bound = std::min<int64_t>(r.nel * (int64_t)r.npe * r.npe, r.non * r.non);
  return r.non * 24 + r.nel * r.npe * 16 + nnz_bound * (4 + 8 + 16 + 8) + r.nel * (int64_t)r.npe * r.npe * 8 +
         r.non * 8 * 12 + (64 << 20);
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

void worker_main(llf_server *s) {
  llf_ctx *ctx = nullptr;
  int crc = llf_ctx_create(s->device, &ctx);
  for (;;) {
    std::unique_ptr<Request> req;
    {
      std::unique_lock<std::mutex> lock(s->mu);
      for (;;) {
        if (s->stopping && s->queue.empty()) break;
        // oldest request that fits the remaining budget; an oversized request
        // runs alone once nothing else holds memory
        auto it = std::find_if(s->queue.begin(), s->queue.end(), [&](const std::unique_ptr<Request> &q) {
          return s->in_use + q->footprint <= s->budget || s->in_use == 0;
        });
        if (it != s->queue.end()) {
          req = std::move(*it);
          s->queue.erase(it);
          s->in_use += req->footprint;
          s->peak_in_use = std::max(s->peak_in_use, s->in_use);
          break;
        }
        s->cv_work.wait(lock);
      }
    }
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

int llf_server_destroy(llf_server *s) {
  if (!s) return LLF_OK;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stopping = true;
    s->cv_work.notify_all();
  }
  for (auto &t : s->workers) t.join();
  delete s;
  return LLF_OK;
}

}  // extern "C"
