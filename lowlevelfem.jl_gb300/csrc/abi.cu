// extern "C" entry points of libllfem_gb300.so (declared in
// include/llfem_gb300.h).  Argument checking, object lifetime, host<->device
// copies and error text live here; the arithmetic lives in the kernels.
#include <cstdio>
#include <cstring>
#include <new>
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "tables.h"

#define LLF_VERSION "0.1.0"

int llf_fail(llf_ctx *ctx, int code, const std::string &msg) {
  if (ctx) ctx->err = msg;
  return code;
}
int llf_ok(llf_ctx *ctx) {
  if (ctx) ctx->err.clear();
  return LLF_OK;
}

void prof_resolve(llf_ctx *ctx) {
  for (auto &p : ctx->pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      auto it = std::find_if(ctx->prof.begin(), ctx->prof.end(),
                             [&](const std::pair<std::string, ProfAcc> &x) { return x.first == p.name; });
      if (it == ctx->prof.end()) {
        ctx->prof.push_back({p.name, ProfAcc{}});
        it = ctx->prof.end() - 1;
      }
      it->second.ms += ms;
      it->second.launches += 1;
    }
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  ctx->pending.clear();
}

int llf_check_status(llf_ctx *ctx, const char *what) {
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(unsigned),
                                    cudaMemcpyDeviceToHost, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  unsigned st = *ctx->h_status;
  if (st == 0) return LLF_OK;
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof(unsigned), ctx->stream));
  std::string w(what);
  if (st & ST_BAD_NODE) return llf_fail(ctx, LLF_ERR_MESH, w + ": connectivity refers to a node tag outside 1..non");
  if (st & ST_BAD_JACOBIAN) return llf_fail(ctx, LLF_ERR_MESH, w + ": non-positive Jacobian determinant (inverted or degenerate element)");
  if (st & ST_CAPACITY) return llf_fail(ctx, LLF_ERR_LIMIT, w + ": node neighbourhood exceeds the pattern buffer");
  if (st & ST_NONFINITE) return llf_fail(ctx, LLF_ERR_NUMERIC, w + ": NaN or Inf in an input array");
  if (st & ST_PATTERN) return llf_fail(ctx, LLF_ERR_STATE, w + ": pattern entry without a contributing element (mesh and pattern disagree)");
  if (st & ST_BREAKDOWN) return llf_fail(ctx, LLF_ERR_NUMERIC, w + ": breakdown");
  if (st & ST_TIMEOUT) return llf_fail(ctx, LLF_ERR_CUDA, w + ": a bounded wait on the tensor cores timed out");
  return llf_fail(ctx, LLF_ERR_CUDA, w + ": unknown device status");
}

namespace {

int upload_tables(llf_ctx *ctx, llf_mesh *m, int nip, const double *w, const double *N,
                  const double *dN) {
  dfree(ctx, m->d_w);
  dfree(ctx, m->d_N);
  dfree(ctx, m->d_dN);
  dfree(ctx, m->d_wf);
  dfree(ctx, m->d_Nf);
  dfree(ctx, m->d_dNf);
  dfree(ctx, m->d_nref);
  dfree(ctx, m->d_Rp);
  dfree(ctx, m->d_Mp);
  dfree(ctx, m->d_Rpf);
  dfree(ctx, m->d_Mpf);
  m->nip = nip;
  const size_t nn = (size_t)nip * m->npe;
  m->h_w.assign(w, w + nip);
  m->h_N.assign(nn, 0.0);
  if (N) std::memcpy(m->h_N.data(), N, sizeof(double) * nn);
  m->h_dN.assign(dN, dN + nn * 3);
  LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_w, nip));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_N, nn));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_dN, nn * 3));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(m->d_w, m->h_w.data(), sizeof(double) * nip,
                                    cudaMemcpyHostToDevice, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(m->d_N, m->h_N.data(), sizeof(double) * nn,
                                    cudaMemcpyHostToDevice, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(m->d_dN, m->h_dN.data(), sizeof(double) * nn * 3,
                                    cudaMemcpyHostToDevice, ctx->stream));
  // FP32 copies for the precision form
  std::vector<float> wf(w, w + nip), Nf(m->h_N.begin(), m->h_N.end()),
      dNf(m->h_dN.begin(), m->h_dN.end());
  LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_wf, nip));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_Nf, nn));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_dNf, nn * 3));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(m->d_wf, wf.data(), sizeof(float) * nip,
                                    cudaMemcpyHostToDevice, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(m->d_Nf, Nf.data(), sizeof(float) * nn,
                                    cudaMemcpyHostToDevice, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(m->d_dNf, dNf.data(), sizeof(float) * nn * 3,
                                    cudaMemcpyHostToDevice, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  m->tables_version++;
  return LLF_OK;
}

// Affine-element tables of the current rule (contract of the oracle):
// R_ab[k][l] = fma chain over q of (w_q dN_a,k) dN_b,l and Mref_ab = fma chain
// of (w_q N_a) N_b.  Stored for the pairs a <= b in a-major order: 9 values
// per pair, the symmetric components S_kl = (R_kl + R_lk) * 0.5 (k <= l;
// 3D 00 11 22 01 02 12, 2D 00 11 01) first, the antisymmetric components
// A_kl = (R_kl - R_lk) * 0.5 (off-diagonal, same order) from index 6.
int upload_affine(llf_ctx *ctx, llf_mesh *m, const double *node_ref) {
  static const int sym3[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  static const int sym2[3][2] = {{0, 0}, {1, 1}, {0, 1}};
  const int dim = m->dim;
  const int ns = dim == 3 ? 6 : 3, na = dim == 3 ? 3 : 1;
  const int(*sym)[2] = dim == 3 ? sym3 : sym2;
  const int npe = m->npe, nip = m->nip;
  const size_t npairs = (size_t)npe * (npe + 1) / 2;
  std::vector<double> Rp(npairs * 9, 0.0), Mp(npairs);
  const double *w = m->h_w.data(), *N = m->h_N.data(), *dN = m->h_dN.data();
  size_t pi = 0;
  for (int a = 0; a < npe; ++a)
    for (int b = a; b < npe; ++b, ++pi) {
      double R[9];
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) {
          double acc = 0.0;
          for (int q = 0; q < nip; ++q)
            acc = std::fma(w[q] * dN[((size_t)q * npe + a) * 3 + k], dN[((size_t)q * npe + b) * 3 + l], acc);
          R[k * 3 + l] = acc;
        }
      for (int n = 0; n < ns; ++n) {
        const int k = sym[n][0], l = sym[n][1];
        Rp[pi * 9 + n] = k == l ? R[k * 3 + k] : (R[k * 3 + l] + R[l * 3 + k]) * 0.5;
      }
      for (int n = 0; n < na; ++n) {
        const int k = sym[dim + n][0], l = sym[dim + n][1];
        Rp[pi * 9 + 6 + n] = (R[k * 3 + l] - R[l * 3 + k]) * 0.5;
      }
      double acc = 0.0;
      for (int q = 0; q < nip; ++q) acc = std::fma(w[q] * N[(size_t)q * npe + a], N[(size_t)q * npe + b], acc);
      Mp[pi] = acc;
    }
  LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_nref, (size_t)npe * 3));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_Rp, npairs * 9));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_Mp, npairs));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(m->d_nref, node_ref, sizeof(double) * npe * 3, cudaMemcpyHostToDevice,
                                    ctx->stream));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(m->d_Rp, Rp.data(), sizeof(double) * npairs * 9, cudaMemcpyHostToDevice,
                                    ctx->stream));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(m->d_Mp, Mp.data(), sizeof(double) * npairs, cudaMemcpyHostToDevice,
                                    ctx->stream));
  // FP32 copy at 12 floats per pair (16-byte rows for the precision form's loads)
  std::vector<float> Rpf((size_t)npairs * 12, 0.f), Mpf(Mp.begin(), Mp.end());
  for (size_t pi = 0; pi < (size_t)npairs; ++pi)
    for (int k = 0; k < 9; ++k) Rpf[pi * 12 + k] = (float)Rp[pi * 9 + k];
  LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_Rpf, npairs * 12));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_Mpf, npairs));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(m->d_Rpf, Rpf.data(), sizeof(float) * npairs * 12, cudaMemcpyHostToDevice,
                                    ctx->stream));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(m->d_Mpf, Mpf.data(), sizeof(float) * npairs, cudaMemcpyHostToDevice,
                                    ctx->stream));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return LLF_OK;
}

// Lame constants, written exactly as the oracle writes them: elastic_constants
// (src/general.jl:142-203) and constitutive_matrix (src/linear.jl:154-188) in
// Lame form; b = thickness for plane stress only (:176-179, :186).
void lame(int ptype, double E, double nu, double thickness, double *lamb, double *mub) {
  double mu = E / (2.0 * (1.0 + nu));
  double lam, b = 1.0;
  if (ptype == LLF_PLANE_STRESS) {
    lam = E * nu / ((1.0 - nu) * (1.0 + nu));
    b = thickness;
  } else {
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  }
  *lamb = lam * b;
  *mub = mu * b;
}

bool valid_ptype(int p) { return p >= LLF_SOLID && p <= LLF_PLANE_HEAT_CONDUCTION; }

int pattern_dim_check(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int ptype) {
  if (!mesh || !pat) return llf_fail(ctx, LLF_ERR_ARG, "null mesh or pattern");
  if (pat->mesh != mesh) return llf_fail(ctx, LLF_ERR_STATE, "pattern was built on another mesh");
  if (ptype_dim(ptype) != mesh->dim)
    return llf_fail(ctx, LLF_ERR_STATE, "problem type dimension differs from the mesh dimension");
  return LLF_OK;
}

}  // namespace

extern "C" {

const char *llf_version(void) { return LLF_VERSION; }

int llf_ctx_create(int device, llf_ctx **out) {
  if (!out) return LLF_ERR_ARG;
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) return LLF_ERR_CUDA;
  if (device < 0 || device >= count) return LLF_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return LLF_ERR_CUDA;
  llf_ctx *c = new (std::nothrow) llf_ctx();
  if (!c) return LLF_ERR_LIMIT;
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc((void **)&c->d_status, sizeof(unsigned)) != cudaSuccess ||
      cudaMallocHost((void **)&c->h_status, sizeof(unsigned)) != cudaSuccess ||
      cudaMemset(c->d_status, 0, sizeof(unsigned)) != cudaSuccess ||
      cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
    delete c;
    return LLF_ERR_CUDA;
  }
  // keep freed stream-ordered memory in the pool between calls
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  *out = c;
  return LLF_OK;
}

int llf_ctx_destroy(llf_ctx *ctx) {
  if (!ctx) return LLF_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->d_status) cudaFree(ctx->d_status);
  if (ctx->h_status) cudaFreeHost(ctx->h_status);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return LLF_OK;
}

const char *llf_last_error(const llf_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int llf_ctx_sync(llf_ctx *ctx) {
  if (!ctx) return LLF_ERR_ARG;
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return llf_ok(ctx);
}

int llf_ctx_stream(llf_ctx *ctx, void **stream) {
  if (!ctx || !stream) return LLF_ERR_ARG;
  *stream = (void *)ctx->stream;
  return LLF_OK;
}

int llf_profile_enable(llf_ctx *ctx, int on) {
  if (!ctx) return LLF_ERR_ARG;
  prof_resolve(ctx);
  ctx->profiling = on != 0;
  return LLF_OK;
}

int llf_profile_reset(llf_ctx *ctx) {
  if (!ctx) return LLF_ERR_ARG;
  prof_resolve(ctx);
  ctx->prof.clear();
  ctx->launches = 0;
  return LLF_OK;
}

int llf_profile_report(llf_ctx *ctx, char *buf, int64_t len, int64_t *needed) {
  if (!ctx) return LLF_ERR_ARG;
  prof_resolve(ctx);
  std::string s = "{";
  for (size_t i = 0; i < ctx->prof.size(); ++i) {
    char tmp[256];
    std::snprintf(tmp, sizeof(tmp), "%s\"%s\": {\"launches\": %lld, \"ms\": %.6f}", i ? ", " : "",
                  ctx->prof[i].first.c_str(), ctx->prof[i].second.launches, ctx->prof[i].second.ms);
    s += tmp;
  }
  s += "}";
  if (needed) *needed = (int64_t)s.size() + 1;
  if (buf && len > 0) {
    size_t n = std::min((size_t)(len - 1), s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = 0;
  }
  return LLF_OK;
}

int llf_launch_count(llf_ctx *ctx, int64_t *launches) {
  if (!ctx || !launches) return LLF_ERR_ARG;
  *launches = ctx->launches;
  return LLF_OK;
}

int llf_alloc_count(llf_ctx *ctx, int64_t *allocs) {
  if (!ctx || !allocs) return LLF_ERR_ARG;
  *allocs = ctx->allocs;
  return LLF_OK;
}

int llf_builtin_rule(int family, int order, int *nip, int *npe, double *xi, double *w,
                     double *N, double *dN, double *node_ref) {
  llf::Rule r;
  if (!llf::build_rule(family, order, r)) return LLF_ERR_UNSUPPORTED;
  if (nip) *nip = r.nip;
  if (npe) *npe = r.npe;
  if (xi) std::memcpy(xi, r.xi.data(), sizeof(double) * r.xi.size());
  if (w) std::memcpy(w, r.w.data(), sizeof(double) * r.w.size());
  if (N) std::memcpy(N, r.N.data(), sizeof(double) * r.N.size());
  if (dN) std::memcpy(dN, r.dN.data(), sizeof(double) * r.dN.size());
  if (node_ref) std::memcpy(node_ref, r.node_ref.data(), sizeof(double) * r.node_ref.size());
  return LLF_OK;
}

int llf_builtin_node_gradients(int family, int order, double *dNn) {
  llf::Rule r;
  if (!llf::build_rule(family, order, r)) return LLF_ERR_UNSUPPORTED;
  if (dNn) std::memcpy(dNn, r.dN_nodes.data(), sizeof(double) * r.dN_nodes.size());
  return LLF_OK;
}

int llf_mesh_upload(llf_ctx *ctx, int dim, int64_t non, const double *xyz, int64_t nel,
                    int npe, const int64_t *conn, int family, int order, llf_mesh **out) {
  if (!ctx || !out) return LLF_ERR_ARG;
  *out = nullptr;
  if (dim < 1 || dim > 3 || non <= 0 || nel < 0 || npe <= 0 || !xyz || (!conn && nel > 0))
    return llf_fail(ctx, LLF_ERR_ARG, "llf_mesh_upload: bad sizes or null arrays");
  if (non > INT32_MAX || nel > INT32_MAX)
    return llf_fail(ctx, LLF_ERR_LIMIT, "llf_mesh_upload: node and element counts must fit in int32");
  llf::Rule rule;
  if (!llf::build_rule(family, order, rule))
    return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "llf_mesh_upload: element family/order not built (orders 1-4 of line, tri, quad, tet, hex)");
  if (rule.npe != npe)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_mesh_upload: npe does not match family/order");
  if (rule.dim != dim && rule.dim != dim - 1)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_mesh_upload: element dimension does not match dim");
  cudaSetDevice(ctx->device);
  llf_mesh *m = new (std::nothrow) llf_mesh();
  if (!m) return llf_fail(ctx, LLF_ERR_LIMIT, "out of host memory");
  m->dim = rule.dim;
  m->family = family;
  m->order = order;
  m->npe = npe;
  m->non = non;
  m->nel = nel;
  int64_t *d_conn64 = nullptr;
  cudaError_t e;
  if ((e = dalloc(ctx, &m->d_xyz, 3 * non)) != cudaSuccess ||
      (e = dalloc(ctx, &m->d_conn, (size_t)npe * nel)) != cudaSuccess ||
      (e = dalloc(ctx, &d_conn64, (size_t)npe * nel)) != cudaSuccess) {
    delete m;
    return llf_fail(ctx, LLF_ERR_CUDA, std::string("llf_mesh_upload: ") + cudaGetErrorString(e));
  }
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(m->d_xyz, xyz, sizeof(double) * 3 * non,
                                    cudaMemcpyHostToDevice, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d_conn64, conn, sizeof(int64_t) * npe * nel,
                                    cudaMemcpyHostToDevice, ctx->stream));
  int rc = mesh_convert_conn(ctx, m, d_conn64);
  if (rc == LLF_OK) rc = check_finite(ctx, m->d_xyz, 3 * non);
  dfree(ctx, d_conn64);
  if (rc == LLF_OK) rc = upload_tables(ctx, m, rule.nip, rule.w.data(), rule.N.data(), rule.dN.data());
  if (rc == LLF_OK) rc = upload_affine(ctx, m, rule.node_ref.data());
  if (rc == LLF_OK) {
    LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_dNn, rule.dN_nodes.size()));
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(m->d_dNn, rule.dN_nodes.data(), sizeof(double) * rule.dN_nodes.size(),
                                      cudaMemcpyHostToDevice, ctx->stream));
  }
  if (rc == LLF_OK) rc = llf_check_status(ctx, "llf_mesh_upload");
  if (rc != LLF_OK) {
    llf_mesh_destroy(ctx, m);
    return rc;
  }
  *out = m;
  return llf_ok(ctx);
}

int llf_mesh_update(llf_ctx *ctx, llf_mesh *m, const double *xyz, const int64_t *conn) {
  if (!ctx || !m || !xyz) return LLF_ERR_ARG;
  m->geo_version++;
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(m->d_xyz, xyz, sizeof(double) * 3 * m->non,
                                    cudaMemcpyHostToDevice, ctx->stream));
  if (conn) {
    int64_t *d_conn64 = nullptr;
    LLF_CUDA_TRY(ctx, dalloc(ctx, &d_conn64, (size_t)m->npe * m->nel));
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d_conn64, conn, sizeof(int64_t) * m->npe * m->nel,
                                      cudaMemcpyHostToDevice, ctx->stream));
    bool changed = false;
    int rc = mesh_update_conn(ctx, m, d_conn64, &changed);
    dfree(ctx, d_conn64);
    if (rc != LLF_OK) return rc;
    if (changed) m->conn_version++;  // patterns built before no longer match
  }
  int rc = check_finite(ctx, m->d_xyz, 3 * m->non);
  if (rc != LLF_OK) return rc;
  rc = llf_check_status(ctx, "llf_mesh_update");
  return rc == LLF_OK ? llf_ok(ctx) : rc;
}

int llf_mesh_set_materials(llf_ctx *ctx, llf_mesh *m, const int32_t *elem_mat) {
  if (!ctx || !m) return LLF_ERR_ARG;
  m->geo_version++;
  dfree(ctx, m->d_emat);
  if (elem_mat) {
    LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_emat, m->nel));
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(m->d_emat, elem_mat, sizeof(int32_t) * m->nel,
                                      cudaMemcpyHostToDevice, ctx->stream));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return llf_ok(ctx);
}

int llf_tables_upload(llf_ctx *ctx, llf_mesh *m, int nip, const double *w, const double *N,
                      const double *dN) {
  if (!ctx || !m || nip <= 0 || !w || !dN) return ctx ? llf_fail(ctx, LLF_ERR_ARG, "llf_tables_upload: bad arguments") : LLF_ERR_ARG;
  int rc = upload_tables(ctx, m, nip, w, N, dN);
  return rc == LLF_OK ? llf_ok(ctx) : rc;
}

int llf_mesh_destroy(llf_ctx *ctx, llf_mesh *m) {
  if (!m) return LLF_OK;
  if (ctx) {
    dfree(ctx, m->d_xyz); dfree(ctx, m->d_conn); dfree(ctx, m->d_emat);
    dfree(ctx, m->d_w); dfree(ctx, m->d_N); dfree(ctx, m->d_dN); dfree(ctx, m->d_dNn);
    dfree(ctx, m->d_nref); dfree(ctx, m->d_Rp); dfree(ctx, m->d_Mp);
    dfree(ctx, m->d_Rpf); dfree(ctx, m->d_Mpf);
    dfree(ctx, m->d_wf); dfree(ctx, m->d_Nf); dfree(ctx, m->d_dNf);
    dfree(ctx, m->d_aflag); dfree(ctx, m->d_ageo);
    cudaStreamSynchronize(ctx->stream);
  }
  delete m;
  return LLF_OK;
}

int llf_pattern_build(llf_ctx *ctx, llf_mesh *mesh, int pdim, int64_t *nnz_out,
                      llf_pattern **out) {
  if (!ctx || !mesh || !out) return LLF_ERR_ARG;
  *out = nullptr;
  if (pdim < 1 || pdim > 3) return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "llf_pattern_build: pdim must be 1, 2 or 3");
  llf_pattern *p = new (std::nothrow) llf_pattern();
  if (!p) return llf_fail(ctx, LLF_ERR_LIMIT, "out of host memory");
  int rc = pattern_build_impl(ctx, mesh, pdim, p);
  if (rc != LLF_OK) {
    llf_pattern_destroy(ctx, p);
    return rc;
  }
  if (nnz_out) *nnz_out = p->nnz;
  *out = p;
  return llf_ok(ctx);
}

namespace {
__global__ void k_pattern_rows(const int64_t *__restrict__ colptr, const int64_t *__restrict__ nptr,
                               const int32_t *__restrict__ nadj, int64_t ndof, int P,
                               int64_t *__restrict__ rowval) {
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  for (int64_t c = (int64_t)blockIdx.x * wpb + (threadIdx.x >> 5); c < ndof;
       c += (int64_t)gridDim.x * wpb) {
    const int64_t s = colptr[c], e = colptr[c + 1], r0 = nptr[c / P];
    for (int64_t k = s + lane; k < e; k += 32) {
      int64_t loc = k - s;
      rowval[k] = (int64_t)P * nadj[r0 + loc / P] + loc % P + 1;
    }
  }
}
__global__ void k_plus1(const int64_t *__restrict__ a, int64_t n, int64_t *__restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = a[i] + 1;
}
}  // namespace

int llf_pattern_copy(llf_ctx *ctx, const llf_pattern *pat, int64_t *colptr, int64_t *rowval) {
  if (!ctx || !pat) return LLF_ERR_ARG;
  cudaStream_t s = ctx->stream;
  if (colptr) {
    int64_t *tmp = nullptr;
    LLF_CUDA_TRY(ctx, dalloc(ctx, &tmp, pat->ndof + 1));
    k_plus1<<<ctx->num_sms * 4, 256, 0, s>>>(pat->d_colptr, pat->ndof + 1, tmp);
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(colptr, tmp, sizeof(int64_t) * (pat->ndof + 1),
                                      cudaMemcpyDeviceToHost, s));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    dfree(ctx, tmp);
  }
  if (rowval) {
    int64_t *tmp = nullptr;
    LLF_CUDA_TRY(ctx, dalloc(ctx, &tmp, pat->nnz));
    k_pattern_rows<<<ctx->num_sms * 8, 256, 0, s>>>(pat->d_colptr, pat->d_nptr, pat->d_nadj,
                                                    pat->ndof, pat->pdim, tmp);
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(rowval, tmp, sizeof(int64_t) * pat->nnz,
                                      cudaMemcpyDeviceToHost, s));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    dfree(ctx, tmp);
  }
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  return llf_ok(ctx);
}

int llf_pattern_info(const llf_pattern *pat, int64_t *ndof, int64_t *nnz, int *pdim) {
  if (!pat) return LLF_ERR_ARG;
  if (ndof) *ndof = pat->ndof;
  if (nnz) *nnz = pat->nnz;
  if (pdim) *pdim = pat->pdim;
  return LLF_OK;
}

int llf_pattern_destroy(llf_ctx *ctx, llf_pattern *p) {
  if (!p) return LLF_OK;
  if (ctx) {
    dfree(ctx, p->d_n2e_ptr); dfree(ctx, p->d_n2e); dfree(ctx, p->d_nptr);
    dfree(ctx, p->d_nadj); dfree(ctx, p->d_diagpos); dfree(ctx, p->d_colptr);
    dfree(ctx, p->d_pos);
    dfree(ctx, p->d_gather_nodes);
    dfree(ctx, p->d_keep_prev);
    pattern_free_layouts(ctx, p);
    ic0_coloring_free(ctx, p);
    cudaStreamSynchronize(ctx->stream);
  }
  delete p;
  return LLF_OK;
}

static int new_matrix(llf_ctx *ctx, llf_pattern *pat, llf_matrix **out, llf_matrix **m) {
  if (!out) return llf_fail(ctx, LLF_ERR_ARG, "null output");
  *out = nullptr;
  *m = new (std::nothrow) llf_matrix();
  if (!*m) return llf_fail(ctx, LLF_ERR_LIMIT, "out of host memory");
  (*m)->pat = pat;
  return LLF_OK;
}

static int finish_matrix(llf_ctx *ctx, int rc, llf_matrix *m, llf_matrix **out) {
  if (rc != LLF_OK) {
    std::string keep = ctx->err;
    llf_matrix_destroy(ctx, m);
    ctx->err = keep;
    return rc;
  }
  *out = m;
  return llf_ok(ctx);
}

int llf_assemble_stiffness(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int ptype,
                           const double *E, const double *nu, int nmat, double thickness,
                           int form, llf_matrix **out) {
  if (!ctx) return LLF_ERR_ARG;
  if (!valid_ptype(ptype) || ptype == LLF_HEAT_CONDUCTION || ptype == LLF_PLANE_HEAT_CONDUCTION)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_assemble_stiffness: ptype must be SOLID, PLANE_STRESS or PLANE_STRAIN");
  int rc = pattern_dim_check(ctx, mesh, pat, ptype);
  if (rc) return rc;
  if (pat->pdim != mesh->dim) return llf_fail(ctx, LLF_ERR_STATE, "stiffness needs a pattern with pdim == dim");
  if (!E || !nu || nmat < 1) return llf_fail(ctx, LLF_ERR_ARG, "material arrays");
  if (form != LLF_FP64 && form != LLF_FP32Q) return llf_fail(ctx, LLF_ERR_ARG, "form");
  std::vector<double> c1(nmat), c2(nmat);
  for (int i = 0; i < nmat; ++i) lame(ptype, E[i], nu[i], thickness, &c1[i], &c2[i]);
  llf_matrix *m;
  if ((rc = new_matrix(ctx, pat, out, &m))) return rc;
  rc = assemble_impl(ctx, mesh, pat, KIND_ELASTIC, ptype, c1.data(), c2.data(), nmat, form, 0, m);
  return finish_matrix(ctx, rc, m, out);
}

int llf_autotune_stiffness(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int ptype, const double *E,
                           const double *nu, int nmat, double thickness, int form, int trials, char *report,
                           int64_t report_len, int64_t *needed) {
  if (!ctx) return LLF_ERR_ARG;
  if (!valid_ptype(ptype) || ptype == LLF_HEAT_CONDUCTION || ptype == LLF_PLANE_HEAT_CONDUCTION)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_autotune_stiffness: ptype must be SOLID, PLANE_STRESS or PLANE_STRAIN");
  int rc = pattern_dim_check(ctx, mesh, pat, ptype);
  if (rc) return rc;
  if (pat->pdim != mesh->dim) return llf_fail(ctx, LLF_ERR_STATE, "stiffness needs a pattern with pdim == dim");
  if (!E || !nu || nmat < 1) return llf_fail(ctx, LLF_ERR_ARG, "material arrays");
  if (form != LLF_FP64 && form != LLF_FP32Q) return llf_fail(ctx, LLF_ERR_ARG, "form");
  std::vector<double> c1(nmat), c2(nmat);
  for (int i = 0; i < nmat; ++i) lame(ptype, E[i], nu[i], thickness, &c1[i], &c2[i]);
  std::string rep;
  rc = autotune_impl(ctx, mesh, pat, KIND_ELASTIC, ptype, c1.data(), c2.data(), nmat, form, trials, &rep);
  if (rc != LLF_OK) return rc;
  if (needed) *needed = (int64_t)rep.size();
  if (report && report_len > 0) {
    const size_t n = std::min((size_t)(report_len - 1), rep.size());
    std::memcpy(report, rep.data(), n);
    report[n] = 0;
  }
  return llf_ok(ctx);
}

int llf_assemble_stiffness_csc(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int ptype, const double *E,
                               const double *nu, int nmat, double thickness, int form, int64_t capacity,
                               int64_t *colptr, int64_t *rowval, double *nzval, int64_t *nnz) {
  if (!ctx) return LLF_ERR_ARG;
  if (!valid_ptype(ptype) || ptype == LLF_HEAT_CONDUCTION || ptype == LLF_PLANE_HEAT_CONDUCTION)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_assemble_stiffness_csc: ptype must be SOLID, PLANE_STRESS or PLANE_STRAIN");
  int rc = pattern_dim_check(ctx, mesh, pat, ptype);
  if (rc) return rc;
  if (pat->pdim != mesh->dim) return llf_fail(ctx, LLF_ERR_STATE, "stiffness needs a pattern with pdim == dim");
  if (!E || !nu || nmat < 1) return llf_fail(ctx, LLF_ERR_ARG, "material arrays");
  if (form != LLF_FP64 && form != LLF_FP32Q) return llf_fail(ctx, LLF_ERR_ARG, "form");
  if (!colptr || !rowval || !nzval || !nnz) return llf_fail(ctx, LLF_ERR_ARG, "llf_assemble_stiffness_csc: null output");
  if (capacity < pat->nnz)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_assemble_stiffness_csc: capacity must be at least the structural nnz");
  std::vector<double> c1(nmat), c2(nmat);
  for (int i = 0; i < nmat; ++i) lame(ptype, E[i], nu[i], thickness, &c1[i], &c2[i]);
  rc = assemble_to_host_impl(ctx, mesh, pat, KIND_ELASTIC, c1.data(), c2.data(), nmat, form, capacity, colptr,
                             rowval, nzval, nnz);
  return rc == LLF_OK ? llf_ok(ctx) : rc;
}

int llf_assemble_stiffness_values(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int ptype, const double *E,
                                  const double *nu, int nmat, double thickness, int form, int64_t capacity,
                                  int64_t *colptr, double *nzval, uint32_t *keep, int64_t *nnz,
                                  int *keep_changed) {
  if (!ctx) return LLF_ERR_ARG;
  if (!valid_ptype(ptype) || ptype == LLF_HEAT_CONDUCTION || ptype == LLF_PLANE_HEAT_CONDUCTION)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_assemble_stiffness_values: ptype must be SOLID, PLANE_STRESS or PLANE_STRAIN");
  int rc = pattern_dim_check(ctx, mesh, pat, ptype);
  if (rc) return rc;
  if (pat->pdim != mesh->dim) return llf_fail(ctx, LLF_ERR_STATE, "stiffness needs a pattern with pdim == dim");
  if (!E || !nu || nmat < 1) return llf_fail(ctx, LLF_ERR_ARG, "material arrays");
  if (form != LLF_FP64 && form != LLF_FP32Q) return llf_fail(ctx, LLF_ERR_ARG, "form");
  if (!colptr || !nzval || !keep || !nnz)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_assemble_stiffness_values: null output");
  if (capacity < pat->nnz)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_assemble_stiffness_values: capacity must be at least the structural nnz");
  std::vector<double> c1(nmat), c2(nmat);
  for (int i = 0; i < nmat; ++i) lame(ptype, E[i], nu[i], thickness, &c1[i], &c2[i]);
  rc = assemble_to_host_impl(ctx, mesh, pat, KIND_ELASTIC, c1.data(), c2.data(), nmat, form, capacity, colptr,
                             nullptr, nzval, nnz, keep, keep_changed);
  return rc == LLF_OK ? llf_ok(ctx) : rc;
}

int64_t llf_rowval_from_keep(int64_t nnz_structural, const int64_t *rowval_structural, const uint32_t *keep,
                             int64_t *rowval) {
  if (nnz_structural < 0 || !rowval_structural || !keep || !rowval) return LLF_ERR_ARG;
  int64_t o = 0;
  for (int64_t w = 0; w * 32 < nnz_structural; ++w) {
    uint32_t bits = keep[w];
    const int64_t base = w * 32;
    if (bits == 0xffffffffu && base + 32 <= nnz_structural) {
      std::memcpy(rowval + o, rowval_structural + base, sizeof(int64_t) * 32);
      o += 32;
      continue;
    }
    while (bits) {
      const int b = __builtin_ctz(bits);
      if (base + b >= nnz_structural) break;
      rowval[o++] = rowval_structural[base + b];
      bits &= bits - 1u;
    }
  }
  return o;
}

int llf_assemble_mass(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int ptype,
                      const double *rho, int nmat, double thickness, int lumped, int form,
                      llf_matrix **out) {
  if (!ctx) return LLF_ERR_ARG;
  if (!valid_ptype(ptype)) return llf_fail(ctx, LLF_ERR_ARG, "llf_assemble_mass: ptype");
  int rc = pattern_dim_check(ctx, mesh, pat, ptype);
  if (rc) return rc;
  if (!rho || nmat < 1) return llf_fail(ctx, LLF_ERR_ARG, "material arrays");
  // massMatrixSolid: b = thickness for plane stress, 1 otherwise (src/linear.jl:1873-1879)
  double b = (ptype == LLF_PLANE_STRESS) ? thickness : 1.0;
  std::vector<double> c1(nmat);
  for (int i = 0; i < nmat; ++i) c1[i] = rho[i] * b;
  llf_matrix *m;
  if ((rc = new_matrix(ctx, pat, out, &m))) return rc;
  rc = assemble_impl(ctx, mesh, pat, KIND_MASS, ptype, c1.data(), nullptr, nmat, form, lumped, m);
  return finish_matrix(ctx, rc, m, out);
}

int llf_assemble_support(llf_ctx *ctx, llf_pattern *pat, llf_mesh *bmesh, const double *k_elem,
                         const double *k_elem_nodal, double thickness, llf_matrix **out) {
  if (!ctx) return LLF_ERR_ARG;
  if (!pat || !bmesh || !out || (!k_elem == !k_elem_nodal))
    return llf_fail(ctx, LLF_ERR_ARG, "llf_assemble_support: give exactly one of k_elem and k_elem_nodal");
  if (bmesh->non != pat->mesh->non || bmesh->dim != pat->mesh->dim - 1)
    return llf_fail(ctx, LLF_ERR_ARG,
                    "llf_assemble_support: the boundary mesh must have dimension dim-1 on the volume mesh's nodes");
  if (pat->conn_version != pat->mesh->conn_version)
    return llf_fail(ctx, LLF_ERR_STATE, "the mesh connectivity changed after the pattern was built; rebuild it");
  const size_t n = (size_t)std::max<int64_t>(bmesh->nel, 1) * pat->pdim * (k_elem_nodal ? bmesh->npe : 1);
  double *dk = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &dk, n));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(dk, k_elem ? k_elem : k_elem_nodal,
                                    sizeof(double) * (size_t)bmesh->nel * pat->pdim * (k_elem_nodal ? bmesh->npe : 1),
                                    cudaMemcpyHostToDevice, ctx->stream));
  llf_matrix *m;
  int rc = new_matrix(ctx, pat, out, &m);
  if (rc == LLF_OK) {
    rc = support_impl(ctx, pat, bmesh, k_elem ? dk : nullptr, k_elem_nodal ? dk : nullptr, thickness, m);
    rc = finish_matrix(ctx, rc, m, out);
  }
  dfree(ctx, dk);
  return rc;
}

int llf_assemble_form(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int form_kind, const double *c1,
                      const double *c2, int nmat, const llf_matrix *accumulate, int form, llf_matrix **out) {
  if (!ctx) return LLF_ERR_ARG;
  if (!mesh || !pat || !out || !c1 || nmat < 1) return llf_fail(ctx, LLF_ERR_ARG, "llf_assemble_form: null argument");
  if (pat->mesh != mesh) return llf_fail(ctx, LLF_ERR_STATE, "llf_assemble_form: the pattern belongs to another mesh");
  if (form != LLF_FP64 && form != LLF_FP32Q) return llf_fail(ctx, LLF_ERR_ARG, "llf_assemble_form: form");
  int kind;
  if (form_kind == LLF_FORM_SYMGRAD_D_SYMGRAD) {
    if (pat->pdim != mesh->dim || !c2)
      return llf_fail(ctx, LLF_ERR_ARG, "∫(SymGrad⋅D⋅SymGrad): a vector field with pdim == dim and lambda, mu");
    kind = KIND_ELASTIC;
  } else if (form_kind == LLF_FORM_GRAD_K_GRAD) {
    if (pat->pdim != 1) return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "∫(Grad⋅k⋅Grad): only scalar fields are accelerated");
    kind = KIND_HEAT;
  } else if (form_kind == LLF_FORM_ID_C_ID) {
    kind = KIND_MASS;
  } else {
    return llf_fail(ctx, LLF_ERR_ARG, "llf_assemble_form: form_kind");
  }
  if (accumulate && accumulate->pat == pat && !accumulate->diagonal_only) {
    const int rc = matrix_ensure_nz(ctx, accumulate);
    if (rc != LLF_OK) return rc;
  }
  if (accumulate && (accumulate->pat != pat || accumulate->diagonal_only || !accumulate->d_nz))
    return llf_fail(ctx, LLF_ERR_STATE, "llf_assemble_form: csc_matrix must be a full matrix on the same pattern");
  llf_matrix *m;
  int rc;
  if ((rc = new_matrix(ctx, pat, out, &m))) return rc;
  m->keep_pattern = accumulate != nullptr;
  rc = assemble_impl(ctx, mesh, pat, kind, mesh->dim == 3 ? LLF_SOLID : LLF_PLANE_STRAIN, c1, c2, nmat, form, 0, m,
                     accumulate ? accumulate->d_nz : nullptr);
  return finish_matrix(ctx, rc, m, out);
}

int llf_matrix_zero_pattern(llf_ctx *ctx, llf_pattern *pat, llf_matrix **out) {
  if (!ctx) return LLF_ERR_ARG;
  if (!pat || !out) return llf_fail(ctx, LLF_ERR_ARG, "llf_matrix_zero_pattern: null argument");
  llf_matrix *m;
  int rc;
  if ((rc = new_matrix(ctx, pat, out, &m))) return rc;
  m->keep_pattern = true;
  cudaError_t e = dalloc(ctx, &m->d_nz, pat->nnz);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->d_nz, 0, sizeof(double) * pat->nnz, ctx->stream);
  rc = e == cudaSuccess ? matrix_finalize(ctx, m, nullptr) : llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
  return finish_matrix(ctx, rc, m, out);
}

int llf_assemble_heat(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int ptype,
                      const double *k, int nmat, double thickness, int form,
                      llf_matrix **out) {
  if (!ctx) return LLF_ERR_ARG;
  if (ptype != LLF_HEAT_CONDUCTION && ptype != LLF_PLANE_HEAT_CONDUCTION)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_assemble_heat: ptype must be HEAT_CONDUCTION or PLANE_HEAT_CONDUCTION");
  int rc = pattern_dim_check(ctx, mesh, pat, ptype);
  if (rc) return rc;
  if (pat->pdim != 1) return llf_fail(ctx, LLF_ERR_STATE, "heat conduction needs a pdim 1 pattern");
  if (!k || nmat < 1) return llf_fail(ctx, LLF_ERR_ARG, "material arrays");
  // heatCondMatrixSolid: b = problem.thickness in 2D and 3D (src/heat.jl:49)
  std::vector<double> c1(nmat);
  for (int i = 0; i < nmat; ++i) c1[i] = k[i] * thickness;
  llf_matrix *m;
  if ((rc = new_matrix(ctx, pat, out, &m))) return rc;
  rc = assemble_impl(ctx, mesh, pat, KIND_HEAT, ptype, c1.data(), nullptr, nmat, form, 0, m);
  return finish_matrix(ctx, rc, m, out);
}

int llf_tl_material_tangent(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, const double *Felem,
                            int law, const double *params, int nparams, llf_matrix **out) {
  if (!ctx) return LLF_ERR_ARG;
  if (!mesh || !pat || !Felem || pat->mesh != mesh || mesh->dim != 3 || pat->pdim != 3)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_tl_material_tangent: needs a 3D mesh, a pdim 3 pattern and F (problem.dim == 3 && pdim == 3, src/nonlinear.jl:2094)");
  size_t nF = (size_t)9 * mesh->npe * mesh->nel;
  double *dF = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &dF, nF));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(dF, Felem, sizeof(double) * nF, cudaMemcpyHostToDevice, ctx->stream));
  llf_matrix *m;
  int rc;
  if ((rc = new_matrix(ctx, pat, out, &m))) { dfree(ctx, dF); return rc; }
  rc = tl_material_tangent_impl(ctx, mesh, pat, dF, law, params, nparams, m);
  dfree(ctx, dF);
  return finish_matrix(ctx, rc, m, out);
}

int llf_tl_tangent(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, const double *Felem, int law,
                   const double *params, int nparams, llf_matrix **out) {
  if (!ctx) return LLF_ERR_ARG;
  if (!mesh || !pat || !Felem || pat->mesh != mesh || mesh->dim != 3 || pat->pdim != 3)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_tl_tangent: needs a 3D mesh, its pdim 3 pattern and F");
  size_t nF = (size_t)9 * mesh->npe * mesh->nel;
  double *dF = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &dF, nF));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(dF, Felem, sizeof(double) * nF, cudaMemcpyHostToDevice, ctx->stream));
  llf_matrix *m;
  int rc;
  if ((rc = new_matrix(ctx, pat, out, &m))) { dfree(ctx, dF); return rc; }
  rc = tl_tangent_impl(ctx, mesh, pat, dF, law, params, nparams, m);
  dfree(ctx, dF);
  return finish_matrix(ctx, rc, m, out);
}

int llf_tl_tangent_form(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, const double *Felem, int law,
                        const double *params, int nparams, int form, llf_matrix **out) {
  if (!ctx) return LLF_ERR_ARG;
  if (form == LLF_FP64) return llf_tl_tangent(ctx, mesh, pat, Felem, law, params, nparams, out);
  if (form != LLF_TF32X3) return llf_fail(ctx, LLF_ERR_ARG, "llf_tl_tangent_form: form must be LLF_FP64 or LLF_TF32X3");
  if (!mesh || !pat || !Felem || pat->mesh != mesh || mesh->dim != 3 || pat->pdim != 3)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_tl_tangent_form: needs a 3D mesh, its pdim 3 pattern and F");
  size_t nF = (size_t)9 * mesh->npe * mesh->nel;
  double *dF = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &dF, nF));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(dF, Felem, sizeof(double) * nF, cudaMemcpyHostToDevice, ctx->stream));
  llf_matrix *m;
  int rc;
  if ((rc = new_matrix(ctx, pat, out, &m))) { dfree(ctx, dF); return rc; }
  rc = tl_tangent_tc_impl(ctx, mesh, pat, dF, law, params, nparams, m);
  dfree(ctx, dF);
  return finish_matrix(ctx, rc, m, out);
}

int llf_tl_initial_stress(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, const double *Selem,
                          const double *Celem, int law, const double *params, int nparams,
                          llf_matrix **out) {
  if (!ctx) return LLF_ERR_ARG;
  if (!mesh || !pat || pat->mesh != mesh || pat->pdim != mesh->dim)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_tl_initial_stress: mesh/pattern mismatch");
  if ((Selem == nullptr) == (Celem == nullptr))
    return llf_fail(ctx, LLF_ERR_ARG, "llf_tl_initial_stress: give exactly one of S or C (src/nonlinear.jl:2429)");
  size_t nT = (size_t)9 * mesh->npe * mesh->nel;
  double *dT = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &dT, nT));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(dT, Selem ? Selem : Celem, sizeof(double) * nT,
                                    cudaMemcpyHostToDevice, ctx->stream));
  llf_matrix *m;
  int rc;
  if ((rc = new_matrix(ctx, pat, out, &m))) { dfree(ctx, dT); return rc; }
  rc = tl_initial_stress_impl(ctx, mesh, pat, Selem ? dT : nullptr, Celem ? dT : nullptr, law,
                              params, nparams, m);
  dfree(ctx, dT);
  return finish_matrix(ctx, rc, m, out);
}

int llf_tl_internal_force(llf_ctx *ctx, llf_mesh *mesh, const double *Pelem, const double *Felem,
                          int law, const double *params, int nparams, double *f_int) {
  if (!ctx) return LLF_ERR_ARG;
  if (!mesh || !f_int || mesh->dim != 3)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_tl_internal_force: needs a 3D mesh (src/nonlinear.jl:2760)");
  if ((Pelem == nullptr) == (Felem == nullptr))
    return llf_fail(ctx, LLF_ERR_ARG, "llf_tl_internal_force: give exactly one of P or F (src/nonlinear.jl:2750)");
  size_t nT = (size_t)9 * mesh->npe * mesh->nel;
  double *dT = nullptr, *df = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &dT, nT));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &df, 3 * mesh->non));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(dT, Pelem ? Pelem : Felem, sizeof(double) * nT,
                                    cudaMemcpyHostToDevice, ctx->stream));
  int rc = tl_internal_force_impl(ctx, mesh, Pelem ? dT : nullptr, Felem ? dT : nullptr, law,
                                  params, nparams, df);
  if (rc == LLF_OK) {
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(f_int, df, sizeof(double) * 3 * mesh->non,
                                      cudaMemcpyDeviceToHost, ctx->stream));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  dfree(ctx, dT);
  dfree(ctx, df);
  return rc == LLF_OK ? llf_ok(ctx) : rc;
}

int llf_grad_elementwise(llf_ctx *ctx, llf_mesh *mesh, const double *u, int add_identity,
                         double *out) {
  if (!ctx) return LLF_ERR_ARG;
  if (!mesh || !u || !out || mesh->dim != 3)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_grad_elementwise: needs a 3D mesh and arrays");
  size_t nT = (size_t)9 * mesh->npe * mesh->nel;
  double *du = nullptr, *dout = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &du, 3 * mesh->non));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &dout, nT));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(du, u, sizeof(double) * 3 * mesh->non, cudaMemcpyHostToDevice,
                                    ctx->stream));
  int rc = grad_elementwise_impl(ctx, mesh, du, add_identity, dout);
  if (rc == LLF_OK) {
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(out, dout, sizeof(double) * nT, cudaMemcpyDeviceToHost,
                                      ctx->stream));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  dfree(ctx, du);
  dfree(ctx, dout);
  return rc == LLF_OK ? llf_ok(ctx) : rc;
}

int llf_load_vector(llf_ctx *ctx, llf_mesh *bmesh, int problem_dim, int pdim, const double *t_const,
                    const double *t_nodal, double thickness, double *f, int64_t ndof) {
  if (!ctx) return LLF_ERR_ARG;
  if (!bmesh || !f || pdim < 1 || pdim > 3 || (!t_const && !t_nodal) ||
      bmesh->dim != problem_dim - 1)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_load_vector: bad arguments (boundary mesh must have dimension problem_dim-1)");
  if (ndof != (int64_t)pdim * bmesh->non)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_load_vector: ndof must be pdim * non");
  double *df = nullptr, *dtn = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &df, ndof));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(df, f, sizeof(double) * ndof, cudaMemcpyHostToDevice, ctx->stream));
  if (t_nodal) {
    LLF_CUDA_TRY(ctx, dalloc(ctx, &dtn, ndof));
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(dtn, t_nodal, sizeof(double) * ndof, cudaMemcpyHostToDevice,
                                      ctx->stream));
  }
  int rc = load_vector_impl(ctx, bmesh, problem_dim, pdim, t_const, dtn, thickness, nullptr, df, ndof);
  if (rc == LLF_OK) {
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(f, df, sizeof(double) * ndof, cudaMemcpyDeviceToHost, ctx->stream));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  dfree(ctx, df);
  dfree(ctx, dtn);
  return rc == LLF_OK ? llf_ok(ctx) : rc;
}

int llf_load_vector_follower(llf_ctx *ctx, llf_mesh *bmesh, const double *F_nodal, const double *t_const,
                             const double *t_nodal, double *f, int64_t ndof) {
  if (!ctx) return LLF_ERR_ARG;
  if (!bmesh || !f || !F_nodal || (!t_const && !t_nodal) || bmesh->dim != 2)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_load_vector_follower: needs F, a traction and a face mesh of a 3D body");
  if (ndof != 3 * bmesh->non) return llf_fail(ctx, LLF_ERR_ARG, "llf_load_vector_follower: ndof must be 3 * non");
  double *df = nullptr, *dtn = nullptr, *dF = nullptr;
  int rc = LLF_OK;
  cudaError_t e = dalloc(ctx, &df, ndof);
  if (e == cudaSuccess) e = dalloc(ctx, &dF, (size_t)9 * bmesh->non);
  if (e == cudaSuccess && t_nodal) e = dalloc(ctx, &dtn, ndof);
  if (e == cudaSuccess) e = cudaMemcpyAsync(df, f, sizeof(double) * ndof, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dF, F_nodal, sizeof(double) * 9 * bmesh->non, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess && t_nodal)
    e = cudaMemcpyAsync(dtn, t_nodal, sizeof(double) * ndof, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
  if (rc == LLF_OK) rc = load_vector_impl(ctx, bmesh, 3, 3, t_const, dtn, 1.0, dF, df, ndof);
  if (rc == LLF_OK) {
    e = cudaMemcpyAsync(f, df, sizeof(double) * ndof, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
  }
  dfree(ctx, df);
  dfree(ctx, dtn);
  dfree(ctx, dF);
  return rc == LLF_OK ? llf_ok(ctx) : rc;
}

int llf_follower_tangent(llf_ctx *ctx, llf_pattern *pat, llf_mesh *bmesh, const double *F_nodal,
                         const double *t_elem, const double *t_elem_nodal, llf_matrix **out) {
  if (!ctx) return LLF_ERR_ARG;
  if (!pat || !bmesh || !out || !F_nodal || (!t_elem == !t_elem_nodal))
    return llf_fail(ctx, LLF_ERR_ARG, "llf_follower_tangent: needs F and exactly one of t_elem, t_elem_nodal");
  if (pat->pdim != 3 || pat->mesh->dim != 3 || bmesh->dim != 2 || bmesh->non != pat->mesh->non)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_follower_tangent: a pdim 3 pattern of a 3D mesh and a face mesh on its nodes");
  if (pat->conn_version != pat->mesh->conn_version)
    return llf_fail(ctx, LLF_ERR_STATE, "the mesh connectivity changed after the pattern was built; rebuild it");
  const size_t nt = (size_t)bmesh->nel * 3 * (t_elem_nodal ? bmesh->npe : 1);
  double *dF = nullptr, *dt = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &dF, (size_t)9 * bmesh->non));
  cudaError_t e = dalloc(ctx, &dt, std::max<size_t>(nt, 1));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dF, F_nodal, sizeof(double) * 9 * bmesh->non, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dt, t_elem ? t_elem : t_elem_nodal, sizeof(double) * nt, cudaMemcpyHostToDevice, ctx->stream);
  int rc = e == cudaSuccess ? LLF_OK : llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
  llf_matrix *m = nullptr;
  if (rc == LLF_OK) rc = new_matrix(ctx, pat, out, &m);
  if (rc == LLF_OK) {
    rc = follower_tangent_impl(ctx, pat, bmesh, dF, t_elem ? dt : nullptr, t_elem_nodal ? dt : nullptr, m);
    rc = finish_matrix(ctx, rc, m, out);
  }
  dfree(ctx, dF);
  dfree(ctx, dt);
  return rc;
}

int llf_elements_to_nodes(llf_ctx *ctx, llf_mesh *mesh, int ncomp, const double *elem_values, double *nodal) {
  if (!ctx) return LLF_ERR_ARG;
  if (!mesh || !elem_values || !nodal || ncomp < 1)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_elements_to_nodes: bad arguments");
  const size_t ne = (size_t)mesh->nel * mesh->npe * ncomp, nn = (size_t)mesh->non * ncomp;
  double *dE = nullptr, *dN = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &dE, std::max<size_t>(ne, 1)));
  cudaError_t e = dalloc(ctx, &dN, nn);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dE, elem_values, sizeof(double) * ne, cudaMemcpyHostToDevice, ctx->stream);
  int rc = e == cudaSuccess ? LLF_OK : llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
  if (rc == LLF_OK) rc = elements_to_nodes_impl(ctx, mesh, ncomp, dE, dN);
  if (rc == LLF_OK) {
    e = cudaMemcpyAsync(nodal, dN, sizeof(double) * nn, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
  }
  dfree(ctx, dE);
  dfree(ctx, dN);
  return rc == LLF_OK ? llf_ok(ctx) : rc;
}

int llf_matrix_nnz(llf_ctx *ctx, const llf_matrix *m, int64_t *nnz) {
  if (!ctx || !m || !nnz) return LLF_ERR_ARG;
  *nnz = m->nnz_s;
  return llf_ok(ctx);
}

int llf_matrix_copy_csc(llf_ctx *ctx, const llf_matrix *m, int64_t *colptr, int64_t *rowval,
                        double *nzval) {
  if (!ctx || !m) return LLF_ERR_ARG;
  cudaStream_t s = ctx->stream;
  const int64_t n = m->pat->ndof;
  if (colptr)
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(colptr, m->d_colptr_s, sizeof(int64_t) * (n + 1),
                                      cudaMemcpyDeviceToHost, s));
  if (rowval && m->nnz_s)
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(rowval, m->d_rowval_s, sizeof(int64_t) * m->nnz_s,
                                      cudaMemcpyDeviceToHost, s));
  if (nzval && m->nnz_s)
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(nzval, m->d_nzval_s, sizeof(double) * m->nnz_s,
                                      cudaMemcpyDeviceToHost, s));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  return llf_ok(ctx);
}

int llf_matrix_prepare(llf_ctx *ctx, llf_matrix *m) {
  if (!ctx) return LLF_ERR_ARG;
  if (!m) return llf_fail(ctx, LLF_ERR_ARG, "llf_matrix_prepare: null matrix");
  const int rc = matrix_ensure_nz(ctx, m);
  return rc == LLF_OK ? llf_ok(ctx) : rc;
}

int llf_matrix_copy_structural(llf_ctx *ctx, const llf_matrix *m, double *nzval) {
  if (!ctx || !m || !nzval) return LLF_ERR_ARG;
  if (m->diagonal_only)
    return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "lumped matrix has no structural values");
  {
    const int rc = matrix_ensure_nz(ctx, m);
    if (rc != LLF_OK) return rc;
  }
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(nzval, m->d_nz, sizeof(double) * m->pat->nnz,
                                    cudaMemcpyDeviceToHost, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return llf_ok(ctx);
}

int llf_matrix_from_structural(llf_ctx *ctx, llf_pattern *pat, const double *nzval,
                               llf_matrix **out) {
  if (!ctx) return LLF_ERR_ARG;
  if (!pat || !nzval || !out) return llf_fail(ctx, LLF_ERR_ARG, "llf_matrix_from_structural: null argument");
  llf_matrix *m;
  int rc;
  if ((rc = new_matrix(ctx, pat, out, &m))) return rc;
  cudaError_t e = dalloc(ctx, &m->d_nz, pat->nnz);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(m->d_nz, nzval, sizeof(double) * pat->nnz, cudaMemcpyHostToDevice, ctx->stream);
  rc = (e == cudaSuccess) ? check_finite(ctx, m->d_nz, pat->nnz)
                          : llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
  if (rc == LLF_OK) rc = llf_check_status(ctx, "llf_matrix_from_structural");
  if (rc == LLF_OK) rc = matrix_finalize(ctx, m, nullptr);
  return finish_matrix(ctx, rc, m, out);
}

int llf_matrix_axpby(llf_ctx *ctx, double a, const llf_matrix *A, double b, const llf_matrix *B,
                     llf_matrix **out) {
  if (!ctx) return LLF_ERR_ARG;
  if (!A || !B || !out) return llf_fail(ctx, LLF_ERR_ARG, "llf_matrix_axpby: null argument");
  llf_matrix *m;
  int rc;
  if ((rc = new_matrix(ctx, A->pat, out, &m))) return rc;
  rc = matrix_axpby_impl(ctx, a, A, b, B, m);
  return finish_matrix(ctx, rc, m, out);
}

int llf_matrix_spmv(llf_ctx *ctx, const llf_matrix *m, const double *x, double *y) {
  if (!ctx || !m || !x || !y) return LLF_ERR_ARG;
  const int64_t n = m->pat->ndof;
  double *dx = nullptr, *dy = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &dx, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &dy, n));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  int rc = spmv_impl(ctx, m, dx, dy);
  if (rc == LLF_OK) {
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(y, dy, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  dfree(ctx, dx);
  dfree(ctx, dy);
  return rc == LLF_OK ? llf_ok(ctx) : rc;
}

int llf_matrix_destroy(llf_ctx *ctx, llf_matrix *m) {
  if (!m) return LLF_OK;
  if (ctx) {
    dfree(ctx, m->d_nz); dfree(ctx, m->d_diag); dfree(ctx, m->d_colptr_s);
    dfree(ctx, m->d_rowval_s); dfree(ctx, m->d_nzval_s);
    cudaStreamSynchronize(ctx->stream);
  }
  delete m;
  return LLF_OK;
}

int llf_pcg(llf_ctx *ctx, const llf_matrix *m, const double *b, double *x, const uint8_t *fixed,
            int precond, double reltol, int64_t maxiter, int64_t *iters, double *relres) {
  if (!ctx) return LLF_ERR_ARG;
  if (!m || !b || !x || !fixed) return llf_fail(ctx, LLF_ERR_ARG, "llf_pcg: null argument");
  if (precond < LLF_PRECOND_NONE || precond > LLF_PRECOND_IC0)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_pcg: unknown preconditioner");
  const int64_t n = m->pat->ndof;
  double *db = nullptr, *dx = nullptr;
  uint8_t *df = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &db, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &dx, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &df, n));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(db, b, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(df, fixed, n, cudaMemcpyHostToDevice, ctx->stream));
  int64_t it = 0;
  double rr = 0.0;
  int rc = pcg_impl(ctx, m, db, dx, df, precond, reltol, maxiter, &it, &rr);
  if (iters) *iters = it;
  if (relres) *relres = rr;
  if (rc == LLF_OK || rc == LLF_ERR_NOT_CONVERGED) {
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(x, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  dfree(ctx, db);
  dfree(ctx, dx);
  dfree(ctx, df);
  cudaStreamSynchronize(ctx->stream);
  return rc == LLF_OK ? llf_ok(ctx) : rc;
}

int llf_heat_fdm(llf_ctx *ctx, const llf_matrix *K, const llf_matrix *C, const double *q, int q_steps, double *T,
                 const uint8_t *fixed, int64_t nsteps, double dt, double theta, int precond, double reltol,
                 int64_t maxiter, int64_t *iters_total) {
  if (!ctx) return LLF_ERR_ARG;
  if (!K || !C || !q || !T || !fixed) return llf_fail(ctx, LLF_ERR_ARG, "FDM: null argument");
  if (K->pat != C->pat) return llf_fail(ctx, LLF_ERR_STATE, "FDM: K and C must belong to the same model.");
  if (K->diagonal_only) return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "FDM: K must be a full matrix");
  if (nsteps < 2) return llf_fail(ctx, LLF_ERR_ARG, "FDM: n must be at least 2.");
  if (q_steps != 1 && q_steps != nsteps) return llf_fail(ctx, LLF_ERR_ARG, "FDM: number of time steps in q must be 1 or n.");
  if (!(dt > 0)) return llf_fail(ctx, LLF_ERR_ARG, "FDM: Δt must be positive.");
  if (!(theta >= 0.0 && theta <= 1.0)) return llf_fail(ctx, LLF_ERR_ARG, "FDM: ϑ must be between 0 and 1.");
  if (precond < LLF_PRECOND_NONE || precond > LLF_PRECOND_IC0)
    return llf_fail(ctx, LLF_ERR_ARG, "FDM: unknown preconditioner");
  const int64_t n = K->pat->ndof;
  double *dq = nullptr, *dT = nullptr;
  uint8_t *df = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &dq, n * q_steps));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &dT, n * nsteps));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &df, n));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(dq, q, sizeof(double) * n * q_steps, cudaMemcpyHostToDevice, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(dT, T, sizeof(double) * n * nsteps, cudaMemcpyHostToDevice, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(df, fixed, n, cudaMemcpyHostToDevice, ctx->stream));
  int64_t it = 0;
  int rc = heat_fdm_impl(ctx, K, C, dq, q_steps, dT, df, nsteps, dt, theta, precond, reltol, maxiter, &it);
  if (iters_total) *iters_total = it;
  if (rc == LLF_OK) {
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(T, dT, sizeof(double) * n * nsteps, cudaMemcpyDeviceToHost, ctx->stream));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  dfree(ctx, dq);
  dfree(ctx, dT);
  dfree(ctx, df);
  cudaStreamSynchronize(ctx->stream);
  return rc == LLF_OK ? llf_ok(ctx) : rc;
}

int llf_pcg_noalloc(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x,
                    const uint8_t *d_fixed, int precond, double reltol, int64_t maxiter,
                    int64_t *iters, double *relres) {
  if (!ctx) return LLF_ERR_ARG;
  if (!m || !d_b || !d_x || !d_fixed)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_pcg_noalloc: null argument");
  if (precond == LLF_PRECOND_IC0)
    return llf_fail(ctx, LLF_ERR_UNSUPPORTED,
                    "llf_pcg_noalloc: IC(0) is not supported on the allocation-free path (its factor and colouring "
                    "need device memory sized by the matrix); use none, Jacobi or block Jacobi, or llf_pcg");
  if (precond < LLF_PRECOND_NONE || precond > LLF_PRECOND_BJACOBI)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_pcg_noalloc: unknown preconditioner");
  int64_t it = 0;
  double rr = 0.0;
  int rc = pcg_noalloc_impl(ctx, m, d_b, d_x, d_fixed, precond, reltol, maxiter, &it, &rr);
  if (iters) *iters = it;
  if (relres) *relres = rr;
  return rc == LLF_OK ? llf_ok(ctx) : rc;
}

static int pcg_batched_host(llf_ctx *ctx, const llf_matrix *m, const double *b, double *x, const uint8_t *fixed,
                            int nseg, const int64_t *seg_off, int precond, double reltol, int64_t maxiter,
                            int64_t *iters, double *relres, bool mixed) {
  if (!ctx) return LLF_ERR_ARG;
  if (!m || !b || !x || !fixed || !seg_off || !iters || !relres || nseg < 1)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_pcg_batched/llf_pcg_mixed: null argument or nseg < 1");
  if (precond < LLF_PRECOND_NONE || precond > LLF_PRECOND_IC0)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_pcg_batched/llf_pcg_mixed: unknown preconditioner");
  const int64_t n = m->pat->ndof;
  if (seg_off[0] != 0 || seg_off[nseg] != n)
    return llf_fail(ctx, LLF_ERR_ARG, "llf_pcg_batched/llf_pcg_mixed: seg_off must run from 0 to the DoF count");
  for (int g = 0; g < nseg; ++g)
    if (seg_off[g + 1] < seg_off[g] || (seg_off[g] % m->pat->pdim) != 0)
      return llf_fail(ctx, LLF_ERR_ARG, "llf_pcg_batched/llf_pcg_mixed: seg_off must be non-decreasing node boundaries");
  double *db = nullptr, *dx = nullptr;
  uint8_t *df = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &db, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &dx, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &df, n));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(db, b, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(df, fixed, n, cudaMemcpyHostToDevice, ctx->stream));
  int rc = pcg_batched_impl(ctx, m, db, dx, df, nseg, seg_off, precond, reltol, maxiter, iters, relres, mixed);
  if (rc == LLF_OK || rc == LLF_ERR_NOT_CONVERGED) {
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(x, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  dfree(ctx, db);
  dfree(ctx, dx);
  dfree(ctx, df);
  cudaStreamSynchronize(ctx->stream);
  return rc == LLF_OK ? llf_ok(ctx) : rc;
}

int llf_pcg_batched(llf_ctx *ctx, const llf_matrix *m, const double *b, double *x, const uint8_t *fixed,
                    int nseg, const int64_t *seg_off, int precond, double reltol, int64_t maxiter,
                    int64_t *iters, double *relres) {
  return pcg_batched_host(ctx, m, b, x, fixed, nseg, seg_off, precond, reltol, maxiter, iters, relres, false);
}

int llf_pcg_mixed(llf_ctx *ctx, const llf_matrix *m, const double *b, double *x, const uint8_t *fixed,
                  int nseg, const int64_t *seg_off, int precond, double reltol, int64_t maxiter,
                  int64_t *iters, double *relres) {
  return pcg_batched_host(ctx, m, b, x, fixed, nseg, seg_off, precond, reltol, maxiter, iters, relres, true);
}

}  // extern "C"
