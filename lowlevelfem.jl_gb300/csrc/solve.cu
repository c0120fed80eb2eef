// Sparse matrix-vector product and preconditioned CG.
//
// SpMV works on the structural node-block CSC: column c = P*B + j is the
// contiguous run nz[colptr[c] .. colptr[c+1]) whose k-th entry sits in row
// P*nadj[nptr[B] + k/P] + k%P.  The assembled operators are symmetric bit
// for bit (element blocks are mirrored, per-entry sums run over the same
// elements in the same order), so y = A x is computed column-wise as
// y_c = sum_k A[row_k, c] x[row_k] — one warp per column, no atomics, a fixed
// shuffle tree per column: results are identical run to run.
//
// PCG restates IterativeSolvers.cg (0.9.4) as called by solveDisplacement /
// solveTemperature / solveField (src/linear.jl:3827-3833): x0 = 0 on the
// free DoFs, per iteration c = Pl\r, rho = c.r, u = c + (rho/rho_prev) u,
// c = A u, alpha = rho/(u.c), x += alpha u, r -= alpha c, stop when
// ||r|| <= reltol*||r0|| or after maxiter products.  Dirichlet elimination
// (K[free,free], f_kin = K[:,fixed] u[fixed], src/linear.jl:3819-3826) is done
// by masking: search directions and products are zeroed on fixed DoFs.
// Scalars live on the device; every reduction is two-stage with a fixed
// order (per-block partials, then one block), so the iteration is
// deterministic.  The host enqueues iterations in chunks and polls a
// device "done" flag between chunks; iterations after convergence are no-ops,
// so the stopping iteration is exactly IterativeSolvers'.
#include "common.cuh"

#include <cmath>

namespace {

constexpr int CG_THREADS = 256;

struct CGState {
  double rho_prev, rho, alpha, res, res0, tol;
  long long it, maxiter;
  int done, breakdown;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, off));
  return v;
}

// Block-wide sum with a fixed tree; result valid in thread 0.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double ws[CG_THREADS / 32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) ws[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

template <int P, bool MASK, bool DOT>
__global__ void __launch_bounds__(CG_THREADS)
k_spmv(const double *__restrict__ nz, const int64_t *__restrict__ colptr,
       const int64_t *__restrict__ nptr, const int32_t *__restrict__ nadj,
       const double *__restrict__ x, const uint8_t *__restrict__ fixed,
       double *__restrict__ y, int64_t ndof, double *__restrict__ partial,
       const CGState *st) {
  if (st && st->done) return;
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  double dot = 0.0;
  for (int64_t c = (int64_t)blockIdx.x * wpb + (threadIdx.x >> 5); c < ndof;
       c += (int64_t)gridDim.x * wpb) {
    const int64_t s = colptr[c], e = colptr[c + 1];
    const int64_t r0 = nptr[c / P];
    double acc = 0.0;
    for (int64_t k = s + lane; k < e; k += 32) {
      const int64_t loc = k - s;
      const int64_t row = (int64_t)P * nadj[r0 + loc / P] + loc % P;
      acc = __fma_rn(nz[k], x[row], acc);
    }
    acc = warp_sum(acc);
    if (MASK && fixed[c]) acc = 0.0;
    if (lane == 0) {
      y[c] = acc;
      if (DOT) dot = __fma_rn(x[c], acc, dot);
    }
  }
  if (DOT) {
    double b = block_sum(dot);
    if (threadIdx.x == 0) partial[blockIdx.x] = b;
  }
}

__global__ void k_diag_scale(const double *__restrict__ d, const double *__restrict__ x,
                             double *__restrict__ y, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = __dmul_rn(d[i], x[i]);
}

// Preconditioner setup: Jacobi 1/diag, or the inverse of each node's P x P
// diagonal block (fixed DoFs replaced by identity rows/columns).
template <int P>
__global__ void k_precond_setup(const double *__restrict__ nz, const int64_t *__restrict__ colptr,
                                const int32_t *__restrict__ diagpos, const uint8_t *__restrict__ fixed,
                                int64_t non, int mode, double *__restrict__ pinv) {
  for (int64_t B = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; B < non;
       B += (int64_t)gridDim.x * blockDim.x) {
    double D[P][P];
    const int dp = diagpos[B];
#pragma unroll
    for (int j = 0; j < P; ++j) {
      const int64_t cs = colptr[P * B + j];
#pragma unroll
      for (int i = 0; i < P; ++i) D[i][j] = dp >= 0 ? nz[cs + (int64_t)P * dp + i] : 0.0;
    }
    if (mode == LLF_PRECOND_BJACOBI) {
#pragma unroll
      for (int i = 0; i < P; ++i)
        if (fixed[P * B + i]) {
#pragma unroll
          for (int j = 0; j < P; ++j) { D[i][j] = 0.0; D[j][i] = 0.0; }
          D[i][i] = 1.0;
        }
      // Gauss-Jordan with partial pivoting
      double Inv[P][P];
#pragma unroll
      for (int i = 0; i < P; ++i)
#pragma unroll
        for (int j = 0; j < P; ++j) Inv[i][j] = (i == j) ? 1.0 : 0.0;
      bool ok = true;
      for (int k = 0; k < P; ++k) {
        int piv = k;
        for (int i = k + 1; i < P; ++i)
          if (fabs(D[i][k]) > fabs(D[piv][k])) piv = i;
        if (D[piv][k] == 0.0) { ok = false; break; }
        if (piv != k)
          for (int j = 0; j < P; ++j) {
            double t = D[k][j]; D[k][j] = D[piv][j]; D[piv][j] = t;
            t = Inv[k][j]; Inv[k][j] = Inv[piv][j]; Inv[piv][j] = t;
          }
        double r = 1.0 / D[k][k];
        for (int j = 0; j < P; ++j) { D[k][j] *= r; Inv[k][j] *= r; }
        for (int i = 0; i < P; ++i)
          if (i != k) {
            double f = D[i][k];
            for (int j = 0; j < P; ++j) {
              D[i][j] -= f * D[k][j];
              Inv[i][j] -= f * Inv[k][j];
            }
          }
      }
#pragma unroll
      for (int i = 0; i < P; ++i)
#pragma unroll
        for (int j = 0; j < P; ++j)
          pinv[(size_t)B * P * P + i * P + j] = ok ? Inv[i][j] : (i == j ? 1.0 : 0.0);
    } else {
#pragma unroll
      for (int i = 0; i < P; ++i) {
        double d = D[i][i];
        pinv[P * B + i] = (mode == LLF_PRECOND_JACOBI && d != 0.0) ? 1.0 / d : 1.0;
      }
    }
  }
}

// z = Pl \ r on free DoFs (0 on fixed) and the partial sums of z.r and r.r.
template <int P>
__device__ __forceinline__ double apply_prec(const double *__restrict__ pinv, int mode,
                                             const double *__restrict__ r, int64_t c) {
  if (mode == LLF_PRECOND_BJACOBI) {
    const int64_t B = c / P;
    const int i = (int)(c % P);
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < P; ++j) acc = __fma_rn(pinv[(size_t)B * P * P + i * P + j], r[P * B + j], acc);
    return acc;
  }
  return __dmul_rn(pinv[c], r[c]);
}

// r = fixed ? 0 : b - y; x = 0; u = 0; z = Pl\r; partials (z.r, r.r).
template <int P>
__global__ void __launch_bounds__(CG_THREADS)
k_cg_init(const double *__restrict__ b, const double *__restrict__ y,
          const uint8_t *__restrict__ fixed, double *__restrict__ r, double *__restrict__ xw,
          double *__restrict__ u, int64_t n, double *__restrict__ part_zr,
          double *__restrict__ part_rr) {
  double rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double ri = fixed[i] ? 0.0 : __dsub_rn(b[i], y[i]);
    r[i] = ri;
    xw[i] = 0.0;
    u[i] = 0.0;
    rr = __fma_rn(ri, ri, rr);
  }
  double s = block_sum(rr);
  if (threadIdx.x == 0) part_rr[blockIdx.x] = s;
  (void)part_zr;
}

template <int P>
__global__ void __launch_bounds__(CG_THREADS)
k_cg_prec(const double *__restrict__ pinv, int mode, const double *__restrict__ r,
          const uint8_t *__restrict__ fixed, double *__restrict__ z, int64_t n,
          double *__restrict__ part_zr, const CGState *st) {
  if (st->done) return;
  double zr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double zi = fixed[i] ? 0.0 : apply_prec<P>(pinv, mode, r, i);
    z[i] = zi;
    zr = __fma_rn(zi, r[i], zr);
  }
  double s = block_sum(zr);
  if (threadIdx.x == 0) part_zr[blockIdx.x] = s;
}

__device__ __forceinline__ double sum_partials(const double *p, int n) {
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v = __dadd_rn(v, p[i]);
  return block_sum(v);
}

// Single block: initial residual and tolerance.
__global__ void k_cg_start(const double *part_rr, int np, double reltol, long long maxiter,
                           CGState *st) {
  double rr = sum_partials(part_rr, np);
  if (threadIdx.x == 0) {
    st->res0 = sqrt(rr);
    st->res = st->res0;
    st->tol = reltol * st->res0;
    st->rho_prev = 1.0;
    st->rho = 0.0;
    st->alpha = 0.0;
    st->it = 0;
    st->maxiter = maxiter;
    st->breakdown = 0;
    st->done = (st->res <= st->tol) || (maxiter <= 0);
  }
}

// Single block: rho = z.r of this iteration.
__global__ void k_cg_rho(const double *part_zr, int np, CGState *st) {
  if (st->done) return;
  double zr = sum_partials(part_zr, np);
  if (threadIdx.x == 0) st->rho = zr;
}

// u = z + (rho/rho_prev) u
__global__ void k_cg_dir(const double *__restrict__ z, double *__restrict__ u, int64_t n,
                         const CGState *st) {
  if (st->done) return;
  const double beta = st->rho / st->rho_prev;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    u[i] = __fma_rn(beta, u[i], z[i]);
}

// Single block: alpha = rho / (u.Au)
__global__ void k_cg_alpha(const double *part_uc, int np, CGState *st) {
  if (st->done) return;
  double uc = sum_partials(part_uc, np);
  if (threadIdx.x == 0) {
    if (!(uc > 0.0) || !isfinite(uc)) {
      st->breakdown = 1;
      st->done = 1;
      st->alpha = 0.0;
    } else {
      st->alpha = st->rho / uc;
    }
  }
}

// x += alpha u; r -= alpha c; partial r.r
__global__ void __launch_bounds__(CG_THREADS)
k_cg_update(double *__restrict__ xw, double *__restrict__ r, const double *__restrict__ u,
            const double *__restrict__ c, int64_t n, double *__restrict__ part_rr,
            const CGState *st) {
  if (st->done) return;
  const double alpha = st->alpha;
  double rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    xw[i] = __fma_rn(alpha, u[i], xw[i]);
    double ri = __fma_rn(-alpha, c[i], r[i]);
    r[i] = ri;
    rr = __fma_rn(ri, ri, rr);
  }
  double s = block_sum(rr);
  if (threadIdx.x == 0) part_rr[blockIdx.x] = s;
}

// Single block: residual norm, iteration count, stopping test.
__global__ void k_cg_finish(const double *part_rr, int np, CGState *st) {
  if (st->done) return;
  double rr = sum_partials(part_rr, np);
  if (threadIdx.x == 0) {
    st->res = sqrt(rr);
    st->rho_prev = st->rho;
    st->it += 1;
    if (st->res <= st->tol || st->it >= st->maxiter) st->done = 1;
  }
}

__global__ void k_cg_merge(const double *__restrict__ xw, const uint8_t *__restrict__ fixed,
                           double *__restrict__ x, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    if (!fixed[i]) x[i] = xw[i];
}

__global__ void k_keep_fixed(const double *__restrict__ x, const uint8_t *__restrict__ fixed,
                             double *__restrict__ xc, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    xc[i] = fixed[i] ? x[i] : 0.0;
}

template <int P, bool MASK, bool DOT>
void launch_spmv(llf_ctx *ctx, const llf_matrix *m, const double *x, const uint8_t *fixed,
                 double *y, double *partial, const CGState *st, unsigned grid) {
  const llf_pattern *pat = m->pat;
  KernelScope ks(ctx, "k_spmv");
  k_spmv<P, MASK, DOT><<<grid, CG_THREADS, 0, ctx->stream>>>(
      m->d_nz, pat->d_colptr, pat->d_nptr, pat->d_nadj, x, fixed, y, pat->ndof, partial, st);
}

template <int P>
int pcg_typed(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x,
              const uint8_t *d_fixed, int precond, double reltol, int64_t maxiter,
              int64_t *iters, double *relres) {
  const llf_pattern *pat = m->pat;
  const int64_t n = pat->ndof;
  cudaStream_t s = ctx->stream;
  const unsigned grid = (unsigned)(ctx->num_sms * 4);
  double *r, *z, *u, *c, *xw, *pinv, *part_a, *part_b;
  CGState *st;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &r, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &z, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &u, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &c, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &xw, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &pinv, precond == LLF_PRECOND_BJACOBI ? n * P : n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &part_a, grid));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &part_b, grid));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &st, 1));

  { KernelScope ks_(ctx, "k_precond_setup");

  k_precond_setup<P><<<(unsigned)((pat->mesh->non + 127) / 128), 128, 0, s>>>(
      m->d_nz, pat->d_colptr, pat->d_diagpos, d_fixed, pat->mesh->non, precond, pinv); }
  // f_kin = A x_c
  { KernelScope ks_(ctx, "k_keep_fixed");
  k_keep_fixed<<<grid, CG_THREADS, 0, s>>>(d_x, d_fixed, xw, n); }
  launch_spmv<P, false, false>(ctx, m, xw, d_fixed, c, nullptr, nullptr, grid);
  { KernelScope ks_(ctx, "k_cg_init");
  k_cg_init<P><<<grid, CG_THREADS, 0, s>>>(d_b, c, d_fixed, r, xw, u, n, part_a, part_b); }
  { KernelScope ks_(ctx, "k_cg_start");
  k_cg_start<<<1, CG_THREADS, 0, s>>>(part_b, (int)grid, reltol, (long long)maxiter, st); }
  LLF_CUDA_TRY(ctx, cudaGetLastError());

  CGState hst{};
  const int chunk = 16;
  for (;;) {
    for (int k = 0; k < chunk; ++k) {
      { KernelScope ks_(ctx, "k_cg_prec");
      k_cg_prec<P><<<grid, CG_THREADS, 0, s>>>(pinv, precond, r, d_fixed, z, n, part_a, st); }
      { KernelScope ks_(ctx, "k_cg_rho");
      k_cg_rho<<<1, CG_THREADS, 0, s>>>(part_a, (int)grid, st); }
      { KernelScope ks_(ctx, "k_cg_dir");
      k_cg_dir<<<grid, CG_THREADS, 0, s>>>(z, u, n, st); }
      launch_spmv<P, true, true>(ctx, m, u, d_fixed, c, part_b, st, grid);
      { KernelScope ks_(ctx, "k_cg_alpha");
      k_cg_alpha<<<1, CG_THREADS, 0, s>>>(part_b, (int)grid, st); }
      { KernelScope ks_(ctx, "k_cg_update");
      k_cg_update<<<grid, CG_THREADS, 0, s>>>(xw, r, u, c, n, part_a, st); }
      { KernelScope ks_(ctx, "k_cg_finish");
      k_cg_finish<<<1, CG_THREADS, 0, s>>>(part_a, (int)grid, st); }
    }
    LLF_CUDA_TRY(ctx, cudaGetLastError());
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(&hst, st, sizeof(CGState), cudaMemcpyDeviceToHost, s));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    if (hst.done) break;
  }
  { KernelScope ks_(ctx, "k_cg_merge");
  k_cg_merge<<<grid, CG_THREADS, 0, s>>>(xw, d_fixed, d_x, n); }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  dfree(ctx, r); dfree(ctx, z); dfree(ctx, u); dfree(ctx, c); dfree(ctx, xw);
  dfree(ctx, pinv); dfree(ctx, part_a); dfree(ctx, part_b); dfree(ctx, st);
  *iters = hst.it;
  *relres = hst.res0 > 0 ? hst.res / hst.res0 : 0.0;
  if (hst.breakdown)
    return llf_fail(ctx, LLF_ERR_NUMERIC, "pcg: breakdown (u.Au <= 0): matrix not positive definite on the free DoFs");
  if (!(hst.res <= hst.tol))
    return llf_fail(ctx, LLF_ERR_NOT_CONVERGED,
                    "pcg: not converged after " + std::to_string(hst.it) +
                        " iterations, relative residual " + std::to_string(*relres));
  return LLF_OK;
}

}  // namespace

int spmv_impl(llf_ctx *ctx, const llf_matrix *m, const double *d_x, double *d_y) {
  const int64_t n = m->pat->ndof;
  const unsigned grid = (unsigned)(ctx->num_sms * 4);
  if (m->diagonal_only) {
    KernelScope ks(ctx, "k_diag_scale");
    k_diag_scale<<<grid, CG_THREADS, 0, ctx->stream>>>(m->d_diag, d_x, d_y, n);
  } else {
    switch (m->pat->pdim) {
      case 1: launch_spmv<1, false, false>(ctx, m, d_x, nullptr, d_y, nullptr, nullptr, grid); break;
      case 2: launch_spmv<2, false, false>(ctx, m, d_x, nullptr, d_y, nullptr, nullptr, grid); break;
      case 3: launch_spmv<3, false, false>(ctx, m, d_x, nullptr, d_y, nullptr, nullptr, grid); break;
      default: return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "pdim must be 1, 2 or 3");
    }
  }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  return LLF_OK;
}

int pcg_impl(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x,
             const uint8_t *d_fixed, int precond, double reltol, int64_t maxiter,
             int64_t *iters, double *relres) {
  if (m->diagonal_only)
    return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "pcg on a lumped (diagonal) matrix");
  switch (m->pat->pdim) {
    case 1: return pcg_typed<1>(ctx, m, d_b, d_x, d_fixed, precond, reltol, maxiter, iters, relres);
    case 2: return pcg_typed<2>(ctx, m, d_b, d_x, d_fixed, precond, reltol, maxiter, iters, relres);
    case 3: return pcg_typed<3>(ctx, m, d_b, d_x, d_fixed, precond, reltol, maxiter, iters, relres);
  }
  return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "pdim must be 1, 2 or 3");
}
