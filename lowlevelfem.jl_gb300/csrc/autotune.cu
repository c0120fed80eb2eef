// Launch-schedule autotuner of the assembly (the element-tile and gather
// schedules; the reference's counterpart is the automatic element chunk
// size of its threaded assembly, src/multifield.jl:2645, :3029-3033).
//
// Knobs, none of which changes a result bit (each element matrix and each
// column sum is computed by the same code in the same order whatever the
// schedule): the element kernels' CTAs per SM, the gather's degree-class
// threshold (which column nodes run in the launch with the smaller
// accumulator) and the gather's warps per CTA.  llf_autotune_stiffness
// times the assembly of the caller's own mesh and pattern under candidate
// schedules by coordinate descent (one knob at a time, the others at their
// best so far; a candidate replaces the best only when it is more than 1 %
// faster, so timing noise does not move the schedule), checks that every candidate's stored CSC equals the first
// one's bit for bit, keeps the fastest on the pattern, and remembers it for
// every later pattern of the same shape (element family, order, nodes per
// element, DoFs per node, operator, arithmetic form, log2 of the element
// count) in this process and, when LLF_TUNE_FILE names a file, across
// processes (one line per shape).
#include "common.cuh"

#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

namespace {

std::mutex g_tune_mu;
std::map<std::string, llf_pattern::Tune> g_tune;
bool g_tune_loaded = false;

std::string tune_key(const llf_pattern *pat, int kind, int form) {
  const llf_mesh *m = pat->mesh;
  int cls = 0;
  for (int64_t n = m->nel; n > 1; n >>= 1) ++cls;
  std::ostringstream o;
  o << "f" << m->family << "o" << m->order << "n" << m->npe << "p" << pat->pdim << "k" << kind << "a" << form
    << "s" << cls;
  return o.str();
}

void load_file_locked() {
  g_tune_loaded = true;
  const char *path = getenv("LLF_TUNE_FILE");
  if (!path) return;
  FILE *f = fopen(path, "r");
  if (!f) return;
  char key[128];
  int cap, thr, wpb;
  while (fscanf(f, "%127s %d %d %d", key, &cap, &thr, &wpb) == 4) {
    llf_pattern::Tune t;
    t.elem_cap = cap;
    t.gather_thr = thr;
    t.gather_wpb = wpb;
    t.from_tuner = true;
    g_tune[key] = t;
  }
  fclose(f);
}

void save_entry_locked(const std::string &key, const llf_pattern::Tune &t) {
  const char *path = getenv("LLF_TUNE_FILE");
  if (!path) return;
  FILE *f = fopen(path, "a");
  if (!f) return;
  fprintf(f, "%s %d %d %d\n", key.c_str(), t.elem_cap, t.gather_thr, t.gather_wpb);
  fclose(f);
}

// Bits of two arrays differ: count (device).
__global__ void k_count_diff(const unsigned long long *__restrict__ a, const unsigned long long *__restrict__ b,
                             int64_t n, unsigned long long *cnt) {
  unsigned long long c = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    c += a[i] != b[i];
  if (c) atomicAdd(cnt, c);
}

void apply(llf_ctx *ctx, llf_pattern *pat, const llf_pattern::Tune &t) {
  if (t.gather_thr != pat->tune.gather_thr) tune_reset_split(ctx, pat);
  pat->tune = t;
}

}  // namespace

void tune_reset_split(llf_ctx *ctx, llf_pattern *pat) {
  dfree(ctx, pat->d_gather_nodes);
  pat->gather_split_done = false;
  pat->gather_n_low = 0;
  pat->gather_md_low = 0;
}

void tune_lookup(llf_pattern *pat, int kind, int form) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  if (!g_tune_loaded) load_file_locked();
  auto it = g_tune.find(tune_key(pat, kind, form));
  if (it == g_tune.end()) return;
  // a pattern whose column classes were already split keeps that split
  if (pat->gather_split_done && it->second.gather_thr != pat->tune.gather_thr) return;
  pat->tune = it->second;
}

namespace {

// One schedule: a warm assembly, then `trials` timed ones (CUDA events on
// the context's stream); the best time, and the last matrix in *keep.
int time_schedule(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int kind, int ptype, const double *c1,
                  const double *c2, int nmat, int form, int trials, double *best_ms, llf_matrix **keep) {
  cudaEvent_t a = nullptr, b = nullptr;
  LLF_CUDA_TRY(ctx, cudaEventCreate(&a));
  LLF_CUDA_TRY(ctx, cudaEventCreate(&b));
  *best_ms = 1e30;
  int rc = LLF_OK;
  for (int t = 0; t <= trials && rc == LLF_OK; ++t) {
    auto *m = new llf_matrix();
    m->pat = pat;
    cudaEventRecord(a, ctx->stream);
    rc = assemble_impl(ctx, mesh, pat, kind, ptype, c1, c2, nmat, form, 0, m);
    cudaEventRecord(b, ctx->stream);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (t > 0 && ms < *best_ms) *best_ms = ms;
    if (t == trials && rc == LLF_OK) {
      *keep = m;
    } else {
      llf_matrix_destroy(ctx, m);
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return rc;
}

int same_result(llf_ctx *ctx, const llf_matrix *x, const llf_matrix *y, bool *same) {
  *same = x->nnz_s == y->nnz_s;
  if (!*same) return LLF_OK;
  unsigned long long *cnt = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &cnt, 1));
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), ctx->stream));
  const unsigned g = (unsigned)(ctx->num_sms * 8);
  k_count_diff<<<g, 256, 0, ctx->stream>>>((const unsigned long long *)x->d_colptr_s,
                                           (const unsigned long long *)y->d_colptr_s, x->pat->ndof + 1, cnt);
  k_count_diff<<<g, 256, 0, ctx->stream>>>((const unsigned long long *)x->d_rowval_s,
                                           (const unsigned long long *)y->d_rowval_s, x->nnz_s, cnt);
  k_count_diff<<<g, 256, 0, ctx->stream>>>((const unsigned long long *)x->d_nzval_s,
                                           (const unsigned long long *)y->d_nzval_s, x->nnz_s, cnt);
  ctx->launches += 3;
  unsigned long long h = 0;
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  dfree(ctx, cnt);
  *same = h == 0;
  return LLF_OK;
}

std::string describe(const llf_pattern::Tune &t) {
  std::ostringstream o;
  o << "{\"elem_ctas_per_sm\": " << t.elem_cap << ", \"gather_threshold_pct\": " << t.gather_thr
    << ", \"gather_warps_per_cta\": " << t.gather_wpb << "}";
  return o.str();
}

}  // namespace

int autotune_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int kind, int ptype, const double *c1,
                  const double *c2, int nmat, int form, int trials, std::string *report) {
  if (trials < 1) trials = 1;
  const llf_pattern::Tune start = pat->tune;
  llf_pattern::Tune best = start;
  best.from_tuner = true;
  llf_matrix *ref = nullptr;
  double best_ms = 0.0;
  std::ostringstream rep;
  rep << "{\"key\": \"" << tune_key(pat, kind, form) << "\", \"trials\": [";
  apply(ctx, pat, best);
  int rc = time_schedule(ctx, mesh, pat, kind, ptype, c1, c2, nmat, form, trials, &best_ms, &ref);
  if (rc != LLF_OK) {
    apply(ctx, pat, start);
    return rc;
  }
  rep << "{\"schedule\": " << describe(best) << ", \"ms\": " << best_ms << "}";
  const std::vector<int> caps = {0, 1, 2, 3, 4}, thrs = {0, 50, 60, 70, 80, 90}, wpbs = {2, 4, 8};
  for (int knob = 0; knob < 3 && rc == LLF_OK; ++knob) {
    const std::vector<int> &vals = knob == 0 ? caps : (knob == 1 ? thrs : wpbs);
    const llf_pattern::Tune base = best;
    for (int v : vals) {
      llf_pattern::Tune t = base;
      int &slot = knob == 0 ? t.elem_cap : (knob == 1 ? t.gather_thr : t.gather_wpb);
      if (slot == v) continue;
      slot = v;
      apply(ctx, pat, t);
      double ms = 0.0;
      llf_matrix *m = nullptr;
      rc = time_schedule(ctx, mesh, pat, kind, ptype, c1, c2, nmat, form, trials, &ms, &m);
      if (rc != LLF_OK) break;
      bool same = false;
      rc = same_result(ctx, ref, m, &same);
      llf_matrix_destroy(ctx, m);
      if (rc != LLF_OK) break;
      if (!same) {
        rc = llf_fail(ctx, LLF_ERR_STATE, "autotune: schedule " + describe(t) + " changed the assembled values");
        break;
      }
      rep << ", {\"schedule\": " << describe(t) << ", \"ms\": " << ms << "}";
      if (ms < 0.99 * best_ms) {   // a change of schedule must win by more than timing noise
        best_ms = ms;
        best = t;
      }
    }
  }
  llf_matrix_destroy(ctx, ref);
  if (rc != LLF_OK) {
    apply(ctx, pat, start);
    return rc;
  }
  apply(ctx, pat, best);
  rep << "], \"chosen\": " << describe(best) << ", \"ms\": " << best_ms << "}";
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    if (!g_tune_loaded) load_file_locked();
    const std::string key = tune_key(pat, kind, form);
    g_tune[key] = best;
    save_entry_locked(key, best);
  }
  if (report) *report = rep.str();
  return LLF_OK;
}
