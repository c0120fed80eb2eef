// Sparse matrix-vector product and (batched) preconditioned CG.
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
//
// Batched form: the system is block diagonal with nseg independent
// segments (instances assembled together on one pattern, e.g. many meshes
// of one batch).  Every segment runs its own CG — own scalars, own stopping
// test — inside the same launches.  DoFs are cut into fixed chunks that never
// straddle a segment; every reduction is per chunk (block tree), then per
// segment over its chunks in order, so results do not depend on the launch
// shape or on what else is in the batch.  One CG iteration is seven
// launches; the host captures a run of iterations into a CUDA graph once and
// replays it, polling the count of still-active segments between replays.
// Iterations after a segment converged are no-ops for that segment, so every
// segment stops exactly where IterativeSolvers would.
#include "common.cuh"
#include "engine.h"

#include <algorithm>
#include <cmath>
#include <mutex>

namespace {

constexpr int CG_THREADS = 256;
constexpr int CHUNK = 768;  // DoFs per reduction chunk (a multiple of every pdim: chunks hold whole nodes)
constexpr int CHUNK_PER_THREAD = CHUNK / CG_THREADS;  // a chunk's DoFs per thread of its block
static_assert(CHUNK % CG_THREADS == 0, "a chunk is whole rounds of a block");

// Work vectors of the mixed-precision CG (FP32 matrix copy and vectors, the
// FP64 right-hand side minus the prescribed values' product).
struct MixedBufs {
  float *nz32 = nullptr, *r = nullptr, *z = nullptr, *u = nullptr, *c = nullptr;
  double *rb = nullptr;
};

struct SegState {
  double rho_prev, rho, alpha, res, res0, tol;
  long long it, maxiter;
  int done, breakdown;
  double rmax;  // mixed precision: true residual at the last reliable update
  int upd, pad;  // mixed precision: a reliable update is due
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

// Products of the P columns of node B by x, summed over SPMV_G lanes: the
// node's columns are P contiguous runs of deg*P values (entry (t, i) of
// column j at (j*deg + t)*P + i); group lane g takes positions g, g+G, ...
// of all P columns at once, the x value of a position being shared by the
// P columns.  On GB300 the FP64 pipe, not HBM, bounds this product (one DFMA
// per stored value), so a warp serves 32/G nodes and the reduction is
// log2(G) shuffle-adds per column shared by those nodes.  After the call
// every lane of the group holds the P sums.
constexpr int SPMV_G = 4;

template <int P>
__device__ __forceinline__ void node_columns_at(const double *__restrict__ nz, const int32_t *__restrict__ nadj,
                                                const double *__restrict__ x, int64_t r0, int64_t r1, bool valid,
                                                int g, double (&acc)[P]) {
#pragma unroll
  for (int j = 0; j < P; ++j) acc[j] = 0.0;
  if (valid) {
    const int n = (int)(r1 - r0) * P;  // entries per column
    const double *col = nz + (int64_t)P * r0 * P;
    int k = g;
    // the row nodes of the step's two entries, loaded a step ahead so that
    // only the gather of x waits on a load
    int32_t ra = k < n ? nadj[r0 + k / P] : 0, rb = k + SPMV_G < n ? nadj[r0 + (k + SPMV_G) / P] : 0;
    for (; k + SPMV_G < n; k += 2 * SPMV_G) {
      const int k2 = k + SPMV_G, kn = k + 2 * SPMV_G;
      double v[P], v2[P];
#pragma unroll
      for (int j = 0; j < P; ++j) {
        v[j] = col[(int64_t)j * n + k];
        v2[j] = col[(int64_t)j * n + k2];
      }
      const double xa = x[(int64_t)P * ra + k % P];
      const double xb = x[(int64_t)P * rb + k2 % P];
      ra = kn < n ? nadj[r0 + kn / P] : 0;
      rb = kn + SPMV_G < n ? nadj[r0 + (kn + SPMV_G) / P] : 0;
#pragma unroll
      for (int j = 0; j < P; ++j) acc[j] = __fma_rn(v2[j], xb, __fma_rn(v[j], xa, acc[j]));
    }
    if (k < n) {
      const double xa = x[(int64_t)P * ra + k % P];
#pragma unroll
      for (int j = 0; j < P; ++j) acc[j] = __fma_rn(col[(int64_t)j * n + k], xa, acc[j]);
    }
  }
#pragma unroll
  for (int off = SPMV_G / 2; off > 0; off >>= 1)
#pragma unroll
    for (int j = 0; j < P; ++j) acc[j] = __dadd_rn(acc[j], __shfl_xor_sync(0xffffffffu, acc[j], off));
}

// The same for node B, whose row nodes are nadj[nptr[B] .. nptr[B+1]).
template <int P>
__device__ __forceinline__ void node_columns(const double *__restrict__ nz, const int64_t *__restrict__ nptr,
                                             const int32_t *__restrict__ nadj, const double *__restrict__ x,
                                             int64_t B, bool valid, int g, double (&acc)[P]) {
  const int64_t r0 = valid ? nptr[B] : 0, r1 = valid ? nptr[B + 1] : 0;
  node_columns_at<P>(nz, nadj, x, r0, r1, valid, g, acc);
}

// y = A x for all columns (plain product, llf_matrix_spmv), SPMV_G lanes per
// column node.
template <int P>
__global__ void __launch_bounds__(CG_THREADS)
k_spmv(const double *__restrict__ nz, const int64_t *__restrict__ colptr,
       const int64_t *__restrict__ nptr, const int32_t *__restrict__ nadj,
       const double *__restrict__ x, double *__restrict__ y, int64_t ndof) {
  (void)colptr;
  constexpr int NPW = 32 / SPMV_G;  // nodes per warp
  const int lane = threadIdx.x & 31, g = lane % SPMV_G, wpb = blockDim.x >> 5;
  const int64_t non = ndof / P;
  const int64_t stride = (int64_t)gridDim.x * wpb * NPW;
  for (int64_t B0 = ((int64_t)blockIdx.x * wpb + (threadIdx.x >> 5)) * NPW; B0 < non; B0 += stride) {
    const int64_t B = B0 + lane / SPMV_G;
    double acc[P];
    node_columns<P>(nz, nptr, nadj, x, B, B < non, g, acc);
    if (B < non && g < P) {
      double v = acc[0];
#pragma unroll
      for (int j = 1; j < P; ++j) v = g == j ? acc[j] : v;
      y[P * B + g] = v;
    }
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
      double Inv[P][P];
#pragma unroll
      for (int i = 0; i < P; ++i)
#pragma unroll
        for (int j = 0; j < P; ++j) Inv[i][j] = (i == j) ? 1.0 : 0.0;
      bool ok = true;
      for (int k = 0; k < P; ++k) {  // Gauss-Jordan with partial pivoting
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

// ---------------------------------------------------------------- batched CG
struct Seg {
  const int64_t *cbeg, *cend;  // per chunk DoF range
  const int32_t *cseg;         // per chunk segment
  const int64_t *sfirst;       // per segment first chunk (nseg+1)
  int64_t nchunks;
  int nseg;
  SegState *st;
  int *active;
  int *arrive;                 // 3*nseg arrival counters of the fused reductions (zero between uses;
                               // [0, nseg) the product's u.c, [nseg, 2nseg) the update's,
                               // [2nseg, 3nseg) the IC(0) z.r's)
  const int16_t *perm;         // per node position: the product's node order within its chunk (or null)
};

// One block per chunk for the kernels of a CG iteration (direction, product,
// update, z.r): a chunk is three DoFs per thread, so its state and data
// loads are latency that only more chunks in flight hide, and the block
// scheduler balances the products' uneven chunks.
inline unsigned chunk_grid(const Seg &S) { return (unsigned)std::max<int64_t>(1, S.nchunks); }

// Last-block-done segment reduction: after a chunk's partial is written,
// thread 0 fences and counts the chunk in; the block that brings in the
// segment's last chunk sees every partial (fence, then L2 loads) and sums
// them in chunk order — the same order and result as a separate reduction
// kernel.  Block-uniform; the counter is reset by that last block.
__device__ __forceinline__ bool arrive_last(int *cnt, int64_t nch) {
  __shared__ int last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = (int64_t)atomicAdd(cnt, 1) == nch - 1;
    if (last) {
      __threadfence();
      *cnt = 0;
    }
  }
  __syncthreads();
  return last != 0;
}

// y = fixed ? 0 : b - A x_c; r = y; x = 0; u = 0; partial r.r per chunk.
__global__ void __launch_bounds__(CG_THREADS)
k_seg_init(Seg S, const double *__restrict__ b, const double *__restrict__ y,
           const uint8_t *__restrict__ fixed, double *__restrict__ r, double *__restrict__ xw,
           double *__restrict__ u, double *__restrict__ part) {
  for (int64_t ch = blockIdx.x; ch < S.nchunks; ch += gridDim.x) {
    double rr = 0.0;
    for (int64_t i = S.cbeg[ch] + threadIdx.x; i < S.cend[ch]; i += blockDim.x) {
      double ri = fixed[i] ? 0.0 : __dsub_rn(b[i], y[i]);
      r[i] = ri;
      xw[i] = 0.0;
      u[i] = 0.0;
      rr = __fma_rn(ri, ri, rr);
    }
    double s = block_sum(rr);
    if (threadIdx.x == 0) part[ch] = s;
  }
}

__device__ __forceinline__ double seg_total(const Seg &S, int s, const double *part) {
  double v = 0.0;
  for (int64_t ch = S.sfirst[s] + threadIdx.x; ch < S.sfirst[s + 1]; ch += blockDim.x) v = __dadd_rn(v, part[ch]);
  return block_sum(v);
}

// The same sum read through L2 (partials written by other blocks of the
// same launch).
__device__ __forceinline__ double seg_total_l2(const Seg &S, int s, const double *part) {
  double v = 0.0;
  for (int64_t ch = S.sfirst[s] + threadIdx.x; ch < S.sfirst[s + 1]; ch += blockDim.x)
    v = __dadd_rn(v, __ldcg(part + ch));
  return block_sum(v);
}

// Segment state after the alpha reduction (u.c) / the residual reduction.
__device__ __forceinline__ void seg_set_alpha(const Seg &S, int s, double uc) {
  SegState &q = S.st[s];
  if (!(uc > 0.0) || !isfinite(uc)) {
    q.breakdown = 1;
    q.done = 1;
    q.alpha = 0.0;
    atomicSub(S.active, 1);
  } else {
    q.alpha = q.rho / uc;
  }
}
__device__ __forceinline__ bool seg_set_finish(const Seg &S, int s, double rr) {
  SegState &q = S.st[s];
  q.res = sqrt(rr);
  q.rho_prev = q.rho;
  q.it += 1;
  if (q.res <= q.tol || q.it >= q.maxiter) {
    q.done = 1;
    atomicSub(S.active, 1);
    return true;
  }
  return false;
}

__global__ void k_seg_start(Seg S, const double *part, double reltol, long long maxiter) {
  for (int s = blockIdx.x; s < S.nseg; s += gridDim.x) {
    double rr = seg_total(S, s, part);
    if (threadIdx.x == 0) {
      SegState &q = S.st[s];
      q.res0 = sqrt(rr);
      q.res = q.res0;
      q.tol = reltol * q.res0;
      q.rho_prev = 1.0;
      q.rho = 0.0;
      q.alpha = 0.0;
      q.it = 0;
      q.maxiter = maxiter;
      q.breakdown = 0;
      q.rmax = q.res0;
      q.upd = 0;
      q.done = (q.res <= q.tol) || (maxiter <= 0);
      if (!q.done) atomicAdd(S.active, 1);
    }
  }
}

template <int P>
__global__ void __launch_bounds__(CG_THREADS)
k_seg_prec(Seg S, const double *__restrict__ pinv, int mode, const double *__restrict__ r,
           const uint8_t *__restrict__ fixed, double *__restrict__ z, double *__restrict__ part) {
  for (int64_t ch = blockIdx.x; ch < S.nchunks; ch += gridDim.x) {
    if (S.st[S.cseg[ch]].done) continue;
    double zr = 0.0;
    for (int64_t i = S.cbeg[ch] + threadIdx.x; i < S.cend[ch]; i += blockDim.x) {
      double zi = fixed[i] ? 0.0 : apply_prec<P>(pinv, mode, r, i);
      z[i] = zi;
      zr = __fma_rn(zi, r[i], zr);
    }
    double s = block_sum(zr);
    if (threadIdx.x == 0) part[ch] = s;
  }
}

__global__ void k_seg_rho(Seg S, const double *part) {
  for (int s = blockIdx.x; s < S.nseg; s += gridDim.x) {
    if (S.st[s].done) continue;
    double v = seg_total(S, s, part);
    if (threadIdx.x == 0) S.st[s].rho = v;
  }
}

__global__ void k_seg_dir(Seg S, const double *__restrict__ z, double *__restrict__ u) {
  for (int64_t ch = blockIdx.x; ch < S.nchunks; ch += gridDim.x) {
    const SegState &q = S.st[S.cseg[ch]];
    if (q.done) continue;
    const double beta = q.rho / q.rho_prev;
    const int64_t b = S.cbeg[ch], e = S.cend[ch];
#pragma unroll
    for (int k = 0; k < CHUNK_PER_THREAD; ++k) {
      const int64_t i = b + threadIdx.x + (int64_t)k * CG_THREADS;
      if (i < e) u[i] = __fma_rn(beta, u[i], z[i]);
    }
  }
}

// c = A u on the chunk's columns (masked) and partial u.c.  SPMV_G lanes per
// node column B (chunks start and end on node boundaries), the chunk's nodes
// taken in the order S.perm gives (decreasing degree: the eight nodes of a
// warp have lists of similar length, so few lanes idle in the FP64 products).
// A column's sums do not depend on the order; the partial u.c takes its
// nodes in that fixed order.  The block that brings in a segment's last
// chunk sums the partials (chunk order) and sets alpha = rho / u.c.
template <int P>
__global__ void __launch_bounds__(CG_THREADS)
k_seg_spmv(Seg S, const double *__restrict__ nz, const int64_t *__restrict__ nptr,
           const int32_t *__restrict__ nadj, const double *__restrict__ u,
           const uint8_t *__restrict__ fixed, double *__restrict__ c, double *__restrict__ part) {
  constexpr int NPW = 32 / SPMV_G;  // nodes per warp
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5, w = threadIdx.x >> 5, g = lane % SPMV_G;
  for (int64_t ch = blockIdx.x; ch < S.nchunks; ch += gridDim.x) {
    if (S.st[S.cseg[ch]].done) continue;
    double dot = 0.0;
    const int64_t b0 = S.cbeg[ch] / P;
    const int nb = (int)(S.cend[ch] / P - b0);
    const int step = wpb * NPW;
    // this lane group's node of the round and of the next one, with its row
    // range loaded a round ahead
    auto node_of = [&](int r) -> int64_t { return b0 + (r < nb ? (S.perm ? (int)S.perm[b0 + r] : r) : 0); };
    int r = w * NPW + lane / SPMV_G;
    int64_t B = node_of(r);
    int64_t q0 = r < nb ? nptr[B] : 0, q1 = r < nb ? nptr[B + 1] : 0;
    for (int r0 = w * NPW; r0 < nb; r0 += step, r += step) {
      const bool valid = r < nb;
      const int64_t Bn = node_of(r + step);
      const bool vn = r + step < nb;
      const int64_t q0n = vn ? nptr[Bn] : 0, q1n = vn ? nptr[Bn + 1] : 0;
      double acc[P];
      node_columns_at<P>(nz, nadj, u, q0, q1, valid, g, acc);
      if (valid && g == 0) {
#pragma unroll
        for (int j = 0; j < P; ++j) {
          const int64_t d = P * B + j;
          const double v = fixed[d] ? 0.0 : acc[j];
          c[d] = v;
          dot = __fma_rn(u[d], v, dot);
        }
      }
      B = Bn;
      q0 = q0n;
      q1 = q1n;
    }
    double s = block_sum(dot);
    if (threadIdx.x == 0) part[ch] = s;
    const int sg = S.cseg[ch];
    if (arrive_last(S.arrive + sg, S.sfirst[sg + 1] - S.sfirst[sg])) {
      const double uc = seg_total_l2(S, sg, part);
      if (threadIdx.x == 0) seg_set_alpha(S, sg, uc);
    }
  }
}

// The product's node order of every chunk: decreasing degree, then index.
// perm[b0 + r] = offset in the chunk (first node b0) of its r-th node.  A
// block ranks one chunk's degrees in shared memory (a chunk has at most
// CHUNK nodes).
__global__ void __launch_bounds__(CG_THREADS)
k_chunk_perm(Seg S, const int64_t *__restrict__ nptr, int P, int16_t *__restrict__ perm) {
  __shared__ int deg[CHUNK];
  for (int64_t ch = blockIdx.x; ch < S.nchunks; ch += gridDim.x) {
    const int64_t b0 = S.cbeg[ch] / P;
    const int nb = (int)(S.cend[ch] / P - b0);
    for (int i = threadIdx.x; i < nb; i += blockDim.x) deg[i] = (int)(nptr[b0 + i + 1] - nptr[b0 + i]);
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
      const int di = deg[i];
      int rank = 0;
      for (int k = 0; k < nb; ++k) rank += deg[k] > di || (deg[k] == di && k < i);
      perm[b0 + rank] = (int16_t)i;
    }
    __syncthreads();
  }
}



// x += alpha u, r -= alpha c and the residual check; with a local
// preconditioner (mode NONE, JACOBI, BJACOBI) also z = M^-1 r and rho = z.r
// for the next iteration — one launch where there were four.
template <int P>
__global__ void __launch_bounds__(CG_THREADS)
k_seg_update_fused(Seg S, double *__restrict__ xw, double *__restrict__ r, const double *__restrict__ u,
                   const double *__restrict__ c, double *__restrict__ part, double *__restrict__ part2,
                   const double *__restrict__ pinv, int mode, bool local_prec, const uint8_t *__restrict__ fixed,
                   double *__restrict__ z) {
  for (int64_t ch = blockIdx.x; ch < S.nchunks; ch += gridDim.x) {
    const int sg = S.cseg[ch];
    const SegState &q = S.st[sg];
    if (q.done) continue;
    const double alpha = q.alpha;
    double rr = 0.0, zr = 0.0;
    const int64_t b = S.cbeg[ch], e = S.cend[ch];
#pragma unroll
    for (int k = 0; k < CHUNK_PER_THREAD; ++k) {
      const int64_t i = b + threadIdx.x + (int64_t)k * CG_THREADS;
      if (i < e) {
        xw[i] = __fma_rn(alpha, u[i], xw[i]);
        const double ri = __fma_rn(-alpha, c[i], r[i]);
        r[i] = ri;
        rr = __fma_rn(ri, ri, rr);
      }
    }
    if (local_prec) {  // the block-Jacobi blocks stay within the chunk (whole nodes): own r only
      __syncthreads();
      for (int64_t i = S.cbeg[ch] + threadIdx.x; i < S.cend[ch]; i += blockDim.x) {
        const double zi = fixed[i] ? 0.0 : apply_prec<P>(pinv, mode, r, i);
        z[i] = zi;
        zr = __fma_rn(zi, r[i], zr);
      }
    }
    const double s1 = block_sum(rr);
    const double s2 = local_prec ? block_sum(zr) : 0.0;
    if (threadIdx.x == 0) {
      part[ch] = s1;
      if (local_prec) part2[ch] = s2;
    }
    if (arrive_last(S.arrive + S.nseg + sg, S.sfirst[sg + 1] - S.sfirst[sg])) {
      const double trr = seg_total_l2(S, sg, part);
      const double tzr = local_prec ? seg_total_l2(S, sg, part2) : 0.0;
      if (threadIdx.x == 0) {
        const bool done = seg_set_finish(S, sg, trr);
        if (local_prec && !done) S.st[sg].rho = tzr;
      }
    }
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

// IC(0) application z = (L L^T)^-1 r in FP32, one colour per launch, eight
// lanes per node over the node's packed neighbour list; nodes of converged
// systems are skipped.  y and z share one FP32 vector (the backward sweep
// overwrites y_i by z_i once every later z_j is known).  The factor, its
// list pointers, L_jj^-1 and the node -> system map are in colour order (a
// colour's nodes by decreasing degree), so a launch reads one contiguous run
// of each and the four nodes of a warp have lists of similar length; lane g
// of a node takes list positions g, g + 8, ... two at a time (the same order
// as one at a time, so the sums do not change).
constexpr int IC_G = 8;  // lanes per node

// Programmatic dependent launch: a sweep launched with programmatic stream
// serialisation starts while the previous sweep finishes, loads what no
// sweep writes (node data, lists, factor blocks, system states), then waits
// for the previous grid before it reads y / z.  It releases its own
// dependent only after that wait, so a launch never overlaps more than its
// predecessor.  Without the launch attribute both instructions are no-ops.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void grid_dep_release() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// The next two list positions of a lane (q and q + IC_G, both before q1):
// neighbour indices and blocks, loaded ahead of the products that need them.
template <int P>
struct IcPair {
  bool one = false, two = false;
  int64_t k1 = 0, k2 = 0;
  float L1[P * P], L2[P * P];
  __device__ __forceinline__ void load(bool live, int64_t q, int64_t q1, const int32_t *__restrict__ lk,
                                       const float *__restrict__ Lv) {
    constexpr int PP = P * P;
    one = live && q < q1;
    two = one && q + IC_G < q1;
    if (one) {
      k1 = lk[q];
#pragma unroll
      for (int e = 0; e < PP; ++e) L1[e] = Lv[q * PP + e];
    }
    k2 = k1;
    if (two) {
      k2 = lk[q + IC_G];
#pragma unroll
      for (int e = 0; e < PP; ++e) L2[e] = Lv[(q + IC_G) * PP + e];
    }
  }
};

// The forward sweep of one colour (t: position in colour order, first = the
// colour's first position).  LAST: the last colour, whose backward step
// z_j = L_jj^-T y_j needs no later neighbour and is done here as well.
template <int P, bool LAST, class RT>
__global__ void __launch_bounds__(CG_THREADS)
k_ic0_forward(const int32_t *__restrict__ nodes, int64_t first, int count, const int64_t *__restrict__ fptr,
              const int32_t *__restrict__ fk, const float *__restrict__ Lf, const float *__restrict__ Ldf,
              const int32_t *__restrict__ segc, const SegState *__restrict__ st,
              const RT *__restrict__ r, float *__restrict__ y) {
  constexpr int PP = P * P;
  const int lane = threadIdx.x & 31, gl = lane & (IC_G - 1);
  const int per_warp = 32 / IC_G;
  const int wg = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * per_warp;
  const int stride = gridDim.x * (blockDim.x >> 5) * per_warp;
  bool waited = false;
  for (int base = wg; base < count; base += stride) {
    const int idx = base + (lane / IC_G);
    const int64_t t = first + idx;
    int64_t j = -1, q0 = 0, q1 = 0;
    if (idx < count) {
      j = nodes[t];
      q0 = fptr[t];
      q1 = fptr[t + 1];
      if (st[segc[t]].done) j = -1;
    }
    float acc[P];
#pragma unroll
    for (int a = 0; a < P; ++a) acc[a] = 0.f;
    IcPair<P> pr;
    int64_t q = q0 + gl;
    pr.load(j >= 0, q, q1, fk, Lf);
    if (!waited) {  // y of earlier colours: written by the previous launches
      grid_dep_wait();
      grid_dep_release();
      waited = true;
    }
    while (pr.one) {
      float y1[P], y2[P];
#pragma unroll
      for (int m = 0; m < P; ++m) {
        y1[m] = y[P * pr.k1 + m];
        y2[m] = y[P * pr.k2 + m];
      }
#pragma unroll
      for (int a = 0; a < P; ++a)
#pragma unroll
        for (int m = 0; m < P; ++m) acc[a] = fmaf(pr.L1[a * P + m], y1[m], acc[a]);
      if (pr.two) {
#pragma unroll
        for (int a = 0; a < P; ++a)
#pragma unroll
          for (int m = 0; m < P; ++m) acc[a] = fmaf(pr.L2[a * P + m], y2[m], acc[a]);
      }
      q += 2 * IC_G;
      pr.load(true, q, q1, fk, Lf);
    }
#pragma unroll
    for (int a = 0; a < P; ++a)
#pragma unroll
      for (int off = IC_G / 2; off > 0; off >>= 1) acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], off);
    if (j >= 0 && gl == 0) {
      float D[PP], v[P], w[P];
#pragma unroll
      for (int e = 0; e < PP; ++e) D[e] = Ldf[t * PP + e];
#pragma unroll
      for (int a = 0; a < P; ++a) v[a] = (float)r[P * j + a] - acc[a];
#pragma unroll
      for (int a = 0; a < P; ++a) {
        float s = 0.f;
#pragma unroll
        for (int m = 0; m <= a; ++m) s = fmaf(D[a * P + m], v[m], s);
        w[a] = s;
      }
      if (LAST) {  // y_j - 0 then L_jj^-T, as the backward sweep would
#pragma unroll
        for (int b = 0; b < P; ++b) v[b] = w[b] - 0.f;
#pragma unroll
        for (int b = 0; b < P; ++b) {
          float s = 0.f;
#pragma unroll
          for (int m = b; m < P; ++m) s = fmaf(D[m * P + b], v[m], s);
          w[b] = s;
        }
      }
#pragma unroll
      for (int a = 0; a < P; ++a) y[P * j + a] = w[a];
    }
  }
}

template <int P>
__global__ void __launch_bounds__(CG_THREADS)
k_ic0_backward(const int32_t *__restrict__ nodes, int64_t first, int count, const int64_t *__restrict__ bptr,
               const int32_t *__restrict__ bk, const float *__restrict__ Lb, const float *__restrict__ Ldf,
               const int32_t *__restrict__ segc, const SegState *__restrict__ st, float *__restrict__ z) {
  constexpr int PP = P * P;
  const int lane = threadIdx.x & 31, gl = lane & (IC_G - 1);
  const int per_warp = 32 / IC_G;
  const int wg = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * per_warp;
  const int stride = gridDim.x * (blockDim.x >> 5) * per_warp;
  bool waited = false;
  for (int base = wg; base < count; base += stride) {
    const int idx = base + (lane / IC_G);
    const int64_t t = first + idx;
    int64_t i = -1, q0 = 0, q1 = 0;
    if (idx < count) {
      i = nodes[t];
      q0 = bptr[t];
      q1 = bptr[t + 1];
      if (st[segc[t]].done) i = -1;
    }
    float acc[P];
#pragma unroll
    for (int b = 0; b < P; ++b) acc[b] = 0.f;
    IcPair<P> pr;  // blocks L_{jn,i}
    int64_t q = q0 + gl;
    pr.load(i >= 0, q, q1, bk, Lb);
    if (!waited) {  // z of later colours: written by the previous launches
      grid_dep_wait();
      grid_dep_release();
      waited = true;
    }
    while (pr.one) {
      float z1[P], z2[P];
#pragma unroll
      for (int a = 0; a < P; ++a) {
        z1[a] = z[P * pr.k1 + a];
        z2[a] = z[P * pr.k2 + a];
      }
#pragma unroll
      for (int b = 0; b < P; ++b)
#pragma unroll
        for (int a = 0; a < P; ++a) acc[b] = fmaf(pr.L1[a * P + b], z1[a], acc[b]);
      if (pr.two) {
#pragma unroll
        for (int b = 0; b < P; ++b)
#pragma unroll
          for (int a = 0; a < P; ++a) acc[b] = fmaf(pr.L2[a * P + b], z2[a], acc[b]);
      }
      q += 2 * IC_G;
      pr.load(true, q, q1, bk, Lb);
    }
#pragma unroll
    for (int b = 0; b < P; ++b)
#pragma unroll
      for (int off = IC_G / 2; off > 0; off >>= 1) acc[b] += __shfl_xor_sync(0xffffffffu, acc[b], off);
    if (i >= 0 && gl == 0) {
      float D[PP], v[P];
#pragma unroll
      for (int e = 0; e < PP; ++e) D[e] = Ldf[t * PP + e];
#pragma unroll
      for (int b = 0; b < P; ++b) v[b] = z[P * i + b] - acc[b];  // y_i, from an earlier launch
#pragma unroll
      for (int b = 0; b < P; ++b) {
        float s = 0.f;
#pragma unroll
        for (int m = b; m < P; ++m) s = fmaf(D[m * P + b], v[m], s);
        z[P * i + b] = s;
      }
    }
  }
}

// z = (double) zf and the partial z.r per chunk (after an IC(0) application).
__global__ void __launch_bounds__(CG_THREADS)
k_seg_zr(Seg S, const float *__restrict__ zf, const double *__restrict__ r, double *__restrict__ z,
         double *__restrict__ part) {
  for (int64_t ch = blockIdx.x; ch < S.nchunks; ch += gridDim.x) {
    if (S.st[S.cseg[ch]].done) continue;
    double zr = 0.0;
    const int64_t b = S.cbeg[ch], e = S.cend[ch];
#pragma unroll
    for (int k = 0; k < CHUNK_PER_THREAD; ++k) {
      const int64_t i = b + threadIdx.x + (int64_t)k * CG_THREADS;
      if (i < e) {
        const double zi = (double)zf[i];
        z[i] = zi;
        zr = __fma_rn(zi, r[i], zr);
      }
    }
    double s = block_sum(zr);
    if (threadIdx.x == 0) part[ch] = s;
    const int sg = S.cseg[ch];
    if (arrive_last(S.arrive + 2 * S.nseg + sg, S.sfirst[sg + 1] - S.sfirst[sg])) {  // rho = z.r
      const double t = seg_total_l2(S, sg, part);
      if (threadIdx.x == 0) S.st[sg].rho = t;
    }
  }
}

// IC(0) state of one solve: the factor and the node -> system map.
struct IcApply {
  const Ic0Factor *f = nullptr;
  float *zf = nullptr;  // FP32 work vector (ndof)
};

// The colour sweeps of one IC(0) application, z (in ic.zf, FP32) from r.
template <int P, class RT>
void enqueue_ic0_sweeps(llf_ctx *ctx, const Seg &S, const IcApply &ic, const RT *r) {
  const Ic0Factor &f = *ic.f;
  cudaStream_t s = ctx->stream;
  auto grid = [&](int count) {
    const int64_t warps = (count + 32 / IC_G - 1) / (32 / IC_G);
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((warps + 7) / 8, (int64_t)ctx->num_sms * 16));
  };
  // forward sweeps; the last colour's launch also does its backward step.
  // Every sweep but the first follows another sweep and starts early (PDL).
  const int C = f.ncolors;
  bool after_sweep = false;
  auto launch = [&](auto kern, int count, auto... args) {
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid(count));
    cfg.blockDim = dim3(CG_THREADS);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = after_sweep ? 1 : 0;
    after_sweep = true;
    return cudaLaunchKernelEx(&cfg, kern, args...);
  };
  for (int c = 0; c < C; ++c) {
    const int count = (int)(f.color_ptr[c + 1] - f.color_ptr[c]);
    if (!count) continue;
    KernelScope k(ctx, "k_ic0_forward");
    const int64_t t0 = f.color_ptr[c];
    if (c == C - 1)
      launch(k_ic0_forward<P, true, RT>, count, (const int32_t *)f.d_nodes, t0, count,
             (const int64_t *)f.fptr, (const int32_t *)f.fk, (const float *)f.Lf, (const float *)f.Ldf,
             (const int32_t *)f.segc, (const SegState *)S.st, r, ic.zf);
    else
      launch(k_ic0_forward<P, false, RT>, count, (const int32_t *)f.d_nodes, t0, count,
             (const int64_t *)f.fptr, (const int32_t *)f.fk, (const float *)f.Lf, (const float *)f.Ldf,
             (const int32_t *)f.segc, (const SegState *)S.st, r, ic.zf);
  }
  for (int c = C - 2; c >= 0; --c) {
    const int count = (int)(f.color_ptr[c + 1] - f.color_ptr[c]);
    if (!count) continue;
    KernelScope k(ctx, "k_ic0_backward");
    launch(k_ic0_backward<P>, count, (const int32_t *)f.d_nodes, (int64_t)f.color_ptr[c], count,
           (const int64_t *)f.bptr, (const int32_t *)f.bk, (const float *)f.Lb, (const float *)f.Ldf,
           (const int32_t *)f.segc, (const SegState *)S.st, ic.zf);
  }
}

template <int P>
void enqueue_ic0(llf_ctx *ctx, const Seg &S, const llf_matrix *m, const IcApply &ic, const double *r, double *z,
                 double *part) {
  (void)m;
  enqueue_ic0_sweeps<P, double>(ctx, S, ic, r);
  { KernelScope k(ctx, "k_seg_zr"); k_seg_zr<<<chunk_grid(S), CG_THREADS, 0, ctx->stream>>>(S, ic.zf, r, z, part); }
}

// z = M^-1 r and rho = z.r of the first iteration.
template <int P>
void enqueue_first_prec(llf_ctx *ctx, const Seg &S, const llf_matrix *m, const double *pinv, int precond,
                        double *r, double *z, const uint8_t *fixed, double *part, unsigned gch, unsigned gseg,
                        const IcApply &ic) {
  cudaStream_t s = ctx->stream;
  if (precond == LLF_PRECOND_IC0) {
    enqueue_ic0<P>(ctx, S, m, ic, r, z, part);  // its z.r sets rho
    return;
  }
  { KernelScope k(ctx, "k_seg_prec"); k_seg_prec<P><<<gch, CG_THREADS, 0, s>>>(S, pinv, precond, r, fixed, z, part); }
  { KernelScope k(ctx, "k_seg_rho"); k_seg_rho<<<gseg, CG_THREADS, 0, s>>>(S, part); }
}

// One CG iteration: u = z + beta u; c = A u with alpha = rho / u.c made by
// each segment's last product block (u.c partials in part3); x and r
// updated with the residual check, then the next z and rho (fused for the
// local preconditioners, the IC(0) sweeps after the update otherwise).
template <int P>
void enqueue_iteration(llf_ctx *ctx, const Seg &S, const llf_matrix *m, const double *pinv, int precond,
                       double *r, double *z, double *u, double *c, double *xw, const uint8_t *fixed,
                       double *part, double *part2, double *part3, const IcApply &ic) {
  const llf_pattern *pat = m->pat;
  cudaStream_t s = ctx->stream;
  const bool local = precond != LLF_PRECOND_IC0;
  { KernelScope k(ctx, "k_seg_dir"); k_seg_dir<<<chunk_grid(S), CG_THREADS, 0, s>>>(S, z, u); }
  { KernelScope k(ctx, "k_seg_spmv");
    k_seg_spmv<P><<<chunk_grid(S), CG_THREADS, 0, s>>>(S, m->d_nz, pat->d_nptr, pat->d_nadj, u, fixed, c, part3); }
  { KernelScope k(ctx, "k_seg_update");
    k_seg_update_fused<P><<<chunk_grid(S), CG_THREADS, 0, s>>>(S, xw, r, u, c, part, part2, pinv, precond, local,
                                                               fixed, z); }
  if (!local) enqueue_ic0<P>(ctx, S, m, ic, r, z, part);
}

template <int P>
int pcg_core(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x, const uint8_t *d_fixed,
             const Seg &S, double *r, double *z, double *u, double *c, double *xw, double *pinv,
             double *part, double *part2, double *part3, int precond, double reltol, int64_t maxiter, bool use_graph,
             SegState *hst, const IcApply &ic = IcApply());
int pcg_outcome(llf_ctx *ctx, int nseg, const SegState *hst, int64_t *iters, double *relres);
template <int P>
int pcg_mixed_core(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x, const uint8_t *d_fixed,
                   const Seg &S, const MixedBufs &B, double *xw, double *tmp, double *pinv, double *part,
                   double *part2, double *part3, int precond, double reltol, int64_t maxiter, bool use_graph,
                   SegState *hst, const IcApply &ic);

// Buffers, chunking and preconditioner of the segmented PCG for one matrix
// and one set of fixed DoFs, built once and reused by every solve with them
// (the theta-method's time steps solve with the same matrix each step).
template <int P>
struct PcgPlan {
  std::vector<int64_t> cb, ce, sf;
  std::vector<int32_t> cs;
  int64_t *d_cb = nullptr, *d_ce = nullptr, *d_sf = nullptr;
  int32_t *d_cs = nullptr;
  int *d_active = nullptr;
  SegState *d_st = nullptr;
  double *r = nullptr, *z = nullptr, *u = nullptr, *c = nullptr, *xw = nullptr, *pinv = nullptr, *part = nullptr;
  double *part2 = nullptr, *part3 = nullptr;
  int *d_arrive = nullptr;
  int16_t *d_perm = nullptr;
  Ic0Factor icf;
  IcApply ic;
  int32_t *d_node_seg = nullptr;
  int precond = 0, nseg = 0;
  bool mixed = false;  // FP32 iterations with FP64 reliable updates (pcg_mixed_core)
  MixedBufs mb;
  Seg S{};
  std::vector<SegState> hst;

  int create(llf_ctx *ctx, const llf_matrix *m, const uint8_t *d_fixed, int nseg_, const int64_t *seg_off,
             int precond_, bool mixed_ = false) {
    precond = precond_;
    nseg = nseg_;
    mixed = mixed_;
    const llf_pattern *pat = m->pat;
    const int64_t n = pat->ndof;
    cudaStream_t s = ctx->stream;
    // chunks that never straddle a segment
    sf.assign(nseg + 1, 0);
    for (int g = 0; g < nseg; ++g) {
      sf[g] = (int64_t)cb.size();
      for (int64_t i = seg_off[g]; i < seg_off[g + 1]; i += CHUNK) {
        cb.push_back(i);
        ce.push_back(std::min(i + CHUNK, seg_off[g + 1]));
        cs.push_back(g);
      }
    }
    sf[nseg] = (int64_t)cb.size();
    const int64_t nch = (int64_t)cb.size();
    LLF_CUDA_TRY(ctx, dalloc(ctx, &d_cb, nch));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &d_ce, nch));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &d_cs, nch));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &d_sf, nseg + 1));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &d_active, 1));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &d_st, nseg));
    if (mixed) {
      LLF_CUDA_TRY(ctx, dalloc(ctx, &mb.nz32, pat->nnz));
      LLF_CUDA_TRY(ctx, dalloc(ctx, &mb.r, n));
      LLF_CUDA_TRY(ctx, dalloc(ctx, &mb.z, n));
      LLF_CUDA_TRY(ctx, dalloc(ctx, &mb.u, n));
      LLF_CUDA_TRY(ctx, dalloc(ctx, &mb.c, n));
      LLF_CUDA_TRY(ctx, dalloc(ctx, &mb.rb, n));
    } else {
      LLF_CUDA_TRY(ctx, dalloc(ctx, &r, n));
      LLF_CUDA_TRY(ctx, dalloc(ctx, &z, n));
      LLF_CUDA_TRY(ctx, dalloc(ctx, &u, n));
    }
    LLF_CUDA_TRY(ctx, dalloc(ctx, &c, n));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &xw, n));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &pinv, precond == LLF_PRECOND_BJACOBI ? n * P : n));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &part, nch));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &part2, nch));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &part3, nch));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &d_arrive, 3 * (int64_t)nseg));
    LLF_CUDA_TRY(ctx, cudaMemsetAsync(d_arrive, 0, sizeof(int) * 3 * nseg, s));
    if (nch) {
      LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d_cb, cb.data(), sizeof(int64_t) * nch, cudaMemcpyHostToDevice, s));
      LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d_ce, ce.data(), sizeof(int64_t) * nch, cudaMemcpyHostToDevice, s));
      LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d_cs, cs.data(), sizeof(int32_t) * nch, cudaMemcpyHostToDevice, s));
    }
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d_sf, sf.data(), sizeof(int64_t) * (nseg + 1), cudaMemcpyHostToDevice, s));
    LLF_CUDA_TRY(ctx, cudaMemsetAsync(d_active, 0, sizeof(int), s));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &d_perm, pat->mesh->non));
    S = Seg{d_cb, d_ce, d_cs, d_sf, nch, nseg, d_st, d_active, d_arrive, d_perm};
    if (nch) {
      KernelScope k(ctx, "k_chunk_perm");
      k_chunk_perm<<<chunk_grid(S), CG_THREADS, 0, s>>>(S, pat->d_nptr, P, d_perm);
    }
    hst.assign(nseg, SegState{});
    // IC(0): factor of A with the fixed DoFs as identity rows, node -> system map
    if (precond == LLF_PRECOND_IC0) {
      const int64_t non = pat->mesh->non;
      std::vector<int32_t> ns(non, 0);
      std::vector<int64_t> seg_nodes(nseg + 1);
      for (int g = 0; g < nseg; ++g) {
        seg_nodes[g] = seg_off[g] / P;
        for (int64_t b = seg_off[g] / P; b < seg_off[g + 1] / P; ++b) ns[b] = g;
      }
      seg_nodes[nseg] = non;
      LLF_CUDA_TRY(ctx, dalloc(ctx, &d_node_seg, non));
      LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d_node_seg, ns.data(), sizeof(int32_t) * non, cudaMemcpyHostToDevice, s));
      int rc = ic0_factor(ctx, m, d_fixed, seg_nodes, d_node_seg, &icf);
      if (rc != LLF_OK) return rc;
      if (dalloc(ctx, &ic.zf, n) != cudaSuccess)
        return llf_fail(ctx, LLF_ERR_CUDA, "pcg: out of device memory for the IC(0) work vector");
      ic.f = &icf;
    }
    return LLF_OK;
  }

  int solve(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x, const uint8_t *d_fixed,
            double reltol, int64_t maxiter, int64_t *iters, double *relres) {
    int rc = mixed ? pcg_mixed_core<P>(ctx, m, d_b, d_x, d_fixed, S, mb, xw, c, pinv, part, part2, part3, precond,
                                       reltol, maxiter, !ctx->profiling, hst.data(), ic)
                   : pcg_core<P>(ctx, m, d_b, d_x, d_fixed, S, r, z, u, c, xw, pinv, part, part2, part3, precond,
                                 reltol, maxiter, !ctx->profiling, hst.data(), ic);
    if (rc != LLF_OK) return rc;
    return pcg_outcome(ctx, nseg, hst.data(), iters, relres);
  }

  void destroy(llf_ctx *ctx) {
    if (precond == LLF_PRECOND_IC0) {
      ic0_release(ctx, &icf);
      dfree(ctx, d_node_seg);
      dfree(ctx, ic.zf);
    }
    dfree(ctx, d_cb); dfree(ctx, d_ce); dfree(ctx, d_cs); dfree(ctx, d_sf); dfree(ctx, d_active);
    dfree(ctx, d_st); dfree(ctx, r); dfree(ctx, z); dfree(ctx, u); dfree(ctx, c); dfree(ctx, xw);
    dfree(ctx, pinv); dfree(ctx, part); dfree(ctx, part2); dfree(ctx, part3); dfree(ctx, d_arrive);
    dfree(ctx, d_perm);
    dfree(ctx, mb.nz32); dfree(ctx, mb.r); dfree(ctx, mb.z); dfree(ctx, mb.u); dfree(ctx, mb.c); dfree(ctx, mb.rb);
  }
};

template <int P>
int pcg_segments(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x,
                 const uint8_t *d_fixed, int nseg, const int64_t *seg_off, int precond,
                 double reltol, int64_t maxiter, int64_t *iters, double *relres, bool mixed = false) {
  PcgPlan<P> plan;
  int rc = plan.create(ctx, m, d_fixed, nseg, seg_off, precond, mixed);
  if (rc == LLF_OK) rc = plan.solve(ctx, m, d_b, d_x, d_fixed, reltol, maxiter, iters, relres);
  plan.destroy(ctx);
  return rc;
}

// Runs the CG of every segment of S to completion with caller-provided
// device buffers (r, z, u, c, xw of ndof doubles, pinv of ndof or ndof*P,
// part of nchunks) and copies the final per-segment states into hst.
// Allocates no device memory; with use_graph the iteration runs are captured
// once into a CUDA graph and replayed.
template <int P>
int pcg_core(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x, const uint8_t *d_fixed,
             const Seg &S, double *r, double *z, double *u, double *c, double *xw, double *pinv,
             double *part, double *part2, double *part3, int precond, double reltol, int64_t maxiter, bool use_graph,
             SegState *hst, const IcApply &ic) {
  const llf_pattern *pat = m->pat;
  const int64_t n = pat->ndof;
  const int64_t nch = S.nchunks;
  const int nseg = S.nseg;
  cudaStream_t s = ctx->stream;
  int *d_active = S.active;
  const unsigned gch = (unsigned)std::max<int64_t>(1, std::min<int64_t>(nch, (int64_t)ctx->num_sms * 8));
  const unsigned gseg = (unsigned)std::max(1, std::min(nseg, ctx->num_sms * 8));
  const unsigned gv = (unsigned)(ctx->num_sms * 4);

  if (precond != LLF_PRECOND_IC0) {
    KernelScope k(ctx, "k_precond_setup");
    k_precond_setup<P><<<(unsigned)((pat->mesh->non + 127) / 128), 128, 0, s>>>(
        m->d_nz, pat->d_colptr, pat->d_diagpos, d_fixed, pat->mesh->non, precond, pinv);
  }
  { KernelScope k(ctx, "k_keep_fixed"); k_keep_fixed<<<gv, CG_THREADS, 0, s>>>(d_x, d_fixed, xw, n); }
  { KernelScope k(ctx, "k_spmv"); k_spmv<P><<<gv, CG_THREADS, 0, s>>>(m->d_nz, pat->d_colptr, pat->d_nptr, pat->d_nadj, xw, c, n); }
  { KernelScope k(ctx, "k_seg_init"); k_seg_init<<<gch, CG_THREADS, 0, s>>>(S, d_b, c, d_fixed, r, xw, u, part); }
  { KernelScope k(ctx, "k_seg_start"); k_seg_start<<<gseg, CG_THREADS, 0, s>>>(S, part, reltol, (long long)maxiter); }
  enqueue_first_prec<P>(ctx, S, m, pinv, precond, r, z, d_fixed, part, gch, gseg, ic);
  LLF_CUDA_TRY(ctx, cudaGetLastError());

  // capture a run of iterations once, replay until every segment is done
  const int per_graph = 16;
  long long launches_per_graph = 0;
  cudaGraphExec_t exec = nullptr;
  bool graph_ok = use_graph;
  if (graph_ok) {
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const long long saved = ctx->launches;
      for (int k = 0; k < per_graph; ++k) enqueue_iteration<P>(ctx, S, m, pinv, precond, r, z, u, c, xw, d_fixed, part, part2, part3, ic);
      launches_per_graph = ctx->launches - saved;
      ctx->launches = saved;
      if (cudaStreamEndCapture(s, &graph) != cudaSuccess ||
          cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
        graph_ok = false;
      if (graph) cudaGraphDestroy(graph);
    } else {
      graph_ok = false;
    }
    cudaGetLastError();
  }
  int active = 1;
  int *h_active = (int *)ctx->h_status;  // pinned word, free between status checks
  while (active > 0) {
    if (graph_ok) {
      LLF_CUDA_TRY(ctx, cudaGraphLaunch(exec, s));
      ctx->launches += launches_per_graph;
    } else {
      for (int k = 0; k < per_graph; ++k) enqueue_iteration<P>(ctx, S, m, pinv, precond, r, z, u, c, xw, d_fixed, part, part2, part3, ic);
    }
    LLF_CUDA_TRY(ctx, cudaGetLastError());
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(h_active, d_active, sizeof(int), cudaMemcpyDeviceToHost, s));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    active = *h_active;
  }
  *h_active = 0;
  if (exec) cudaGraphExecDestroy(exec);
  { KernelScope k(ctx, "k_cg_merge"); k_cg_merge<<<gv, CG_THREADS, 0, s>>>(xw, d_fixed, d_x, n); }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(hst, S.st, sizeof(SegState) * nseg, cudaMemcpyDeviceToHost, s));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  return LLF_OK;
}


// ---------------------------------------------------------------- mixed CG
// Mixed-precision PCG: the iterations run in FP32 — an FP32 copy of the
// matrix values, FP32 vectors, FP32 products on the FP32 pipe, the
// preconditioner applied into FP32 — while the solution is accumulated in
// FP64 and the residual is replaced by the true FP64 residual
// r = (b - A x_c) - A x of the FP64 matrix whenever the FP32 recurrence
// residual has fallen by MX_DELTA since the last replacement, when it meets
// the tolerance, and at maxiter (reliable updates; the search direction is
// kept across a replacement).  A system is done only when its true FP64
// residual meets ||r|| <= reltol ||r0||.  Scalars (rho, alpha, the dot
// products) are FP64.  Every system of a batch still runs its own CG and
// reductions per chunk and then per system in chunk order, so a system
// gives the same result alone and in a batch.
constexpr double MX_DELTA = 1e-2;

__global__ void k_f64_to_f32(const double *__restrict__ a, float *__restrict__ b, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = __double2float_rn(a[i]);
}

// FP32 products of the P columns of a node (node_columns_at in FP32).
template <int P>
__device__ __forceinline__ void node_columns32_at(const float *__restrict__ nz, const int32_t *__restrict__ nadj,
                                                  const float *__restrict__ x, int64_t r0, int64_t r1, bool valid,
                                                  int g, float (&acc)[P]) {
#pragma unroll
  for (int j = 0; j < P; ++j) acc[j] = 0.f;
  if (valid) {
    const int n = (int)(r1 - r0) * P;
    const float *col = nz + (int64_t)P * r0 * P;
    int k = g;
    int32_t ra = k < n ? nadj[r0 + k / P] : 0, rb = k + SPMV_G < n ? nadj[r0 + (k + SPMV_G) / P] : 0;
    for (; k + SPMV_G < n; k += 2 * SPMV_G) {
      const int k2 = k + SPMV_G, kn = k + 2 * SPMV_G;
      float v[P], v2[P];
#pragma unroll
      for (int j = 0; j < P; ++j) {
        v[j] = col[(int64_t)j * n + k];
        v2[j] = col[(int64_t)j * n + k2];
      }
      const float xa = x[(int64_t)P * ra + k % P];
      const float xb = x[(int64_t)P * rb + k2 % P];
      ra = kn < n ? nadj[r0 + kn / P] : 0;
      rb = kn + SPMV_G < n ? nadj[r0 + (kn + SPMV_G) / P] : 0;
#pragma unroll
      for (int j = 0; j < P; ++j) acc[j] = fmaf(v2[j], xb, fmaf(v[j], xa, acc[j]));
    }
    if (k < n) {
      const float xa = x[(int64_t)P * ra + k % P];
#pragma unroll
      for (int j = 0; j < P; ++j) acc[j] = fmaf(col[(int64_t)j * n + k], xa, acc[j]);
    }
  }
#pragma unroll
  for (int off = SPMV_G / 2; off > 0; off >>= 1)
#pragma unroll
    for (int j = 0; j < P; ++j) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], off);
}

// z_c = M^-1 r at DoF c with an FP32 residual (FP64 arithmetic, FP32 result).
template <int P>
__device__ __forceinline__ float apply_prec32(const double *__restrict__ pinv, int mode, const float *__restrict__ r,
                                              int64_t c) {
  if (mode == LLF_PRECOND_BJACOBI) {
    const int64_t B = c / P;
    const int i = (int)(c % P);
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < P; ++j) acc = __fma_rn(pinv[(size_t)B * P * P + i * P + j], (double)r[P * B + j], acc);
    return __double2float_rn(acc);
  }
  return __double2float_rn(__dmul_rn(pinv[c], (double)r[c]));
}

// rb = r64 = fixed ? 0 : b - A x_c; r = (float) r64; x = 0; u = 0; partial r.r.
__global__ void __launch_bounds__(CG_THREADS)
k_mx_init(Seg S, const double *__restrict__ b, const double *__restrict__ y, const uint8_t *__restrict__ fixed,
          double *__restrict__ rb, float *__restrict__ r, double *__restrict__ xw, float *__restrict__ u,
          double *__restrict__ part) {
  for (int64_t ch = blockIdx.x; ch < S.nchunks; ch += gridDim.x) {
    double rr = 0.0;
    for (int64_t i = S.cbeg[ch] + threadIdx.x; i < S.cend[ch]; i += blockDim.x) {
      const double ri = fixed[i] ? 0.0 : __dsub_rn(b[i], y[i]);
      rb[i] = ri;
      r[i] = __double2float_rn(ri);
      xw[i] = 0.0;
      u[i] = 0.f;
      rr = __fma_rn(ri, ri, rr);
    }
    const double sm = block_sum(rr);
    if (threadIdx.x == 0) part[ch] = sm;
  }
}

// First z = M^-1 r (local preconditioners) and partial z.r.
template <int P>
__global__ void __launch_bounds__(CG_THREADS)
k_mx_prec(Seg S, const double *__restrict__ pinv, int mode, const float *__restrict__ r,
          const uint8_t *__restrict__ fixed, float *__restrict__ z, double *__restrict__ part) {
  for (int64_t ch = blockIdx.x; ch < S.nchunks; ch += gridDim.x) {
    if (S.st[S.cseg[ch]].done) continue;
    double zr = 0.0;
    for (int64_t i = S.cbeg[ch] + threadIdx.x; i < S.cend[ch]; i += blockDim.x) {
      const float zi = fixed[i] ? 0.f : apply_prec32<P>(pinv, mode, r, i);
      z[i] = zi;
      zr = __fma_rn((double)zi, (double)r[i], zr);
    }
    const double sm = block_sum(zr);
    if (threadIdx.x == 0) part[ch] = sm;
  }
}

__global__ void __launch_bounds__(CG_THREADS) k_mx_dir(Seg S, const float *__restrict__ z, float *__restrict__ u) {
  for (int64_t ch = blockIdx.x; ch < S.nchunks; ch += gridDim.x) {
    const SegState &q = S.st[S.cseg[ch]];
    if (q.done) continue;
    const float beta = __double2float_rn(q.rho / q.rho_prev);
    const int64_t b = S.cbeg[ch], e = S.cend[ch];
#pragma unroll
    for (int k = 0; k < CHUNK_PER_THREAD; ++k) {
      const int64_t i = b + threadIdx.x + (int64_t)k * CG_THREADS;
      if (i < e) u[i] = fmaf(beta, u[i], z[i]);
    }
  }
}

// c = A32 u (masked) and alpha = rho / u.c (u.c in FP64) — k_seg_spmv in FP32.
template <int P>
__global__ void __launch_bounds__(CG_THREADS)
k_mx_spmv(Seg S, const float *__restrict__ nz, const int64_t *__restrict__ nptr, const int32_t *__restrict__ nadj,
          const float *__restrict__ u, const uint8_t *__restrict__ fixed, float *__restrict__ c,
          double *__restrict__ part) {
  constexpr int NPW = 32 / SPMV_G;
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5, w = threadIdx.x >> 5, g = lane % SPMV_G;
  for (int64_t ch = blockIdx.x; ch < S.nchunks; ch += gridDim.x) {
    if (S.st[S.cseg[ch]].done) continue;
    double dot = 0.0;
    const int64_t b0 = S.cbeg[ch] / P;
    const int nb = (int)(S.cend[ch] / P - b0);
    const int step = wpb * NPW;
    auto node_of = [&](int rr) -> int64_t { return b0 + (rr < nb ? (S.perm ? (int)S.perm[b0 + rr] : rr) : 0); };
    int rr = w * NPW + lane / SPMV_G;
    int64_t B = node_of(rr);
    int64_t q0 = rr < nb ? nptr[B] : 0, q1 = rr < nb ? nptr[B + 1] : 0;
    for (int r0 = w * NPW; r0 < nb; r0 += step, rr += step) {
      const bool valid = rr < nb;
      const int64_t Bn = node_of(rr + step);
      const bool vn = rr + step < nb;
      const int64_t q0n = vn ? nptr[Bn] : 0, q1n = vn ? nptr[Bn + 1] : 0;
      float acc[P];
      node_columns32_at<P>(nz, nadj, u, q0, q1, valid, g, acc);
      if (valid && g == 0) {
#pragma unroll
        for (int j = 0; j < P; ++j) {
          const int64_t d = P * B + j;
          const float v = fixed[d] ? 0.f : acc[j];
          c[d] = v;
          dot = __fma_rn((double)u[d], (double)v, dot);
        }
      }
      B = Bn;
      q0 = q0n;
      q1 = q1n;
    }
    const double sm = block_sum(dot);
    if (threadIdx.x == 0) part[ch] = sm;
    const int sg = S.cseg[ch];
    if (arrive_last(S.arrive + sg, S.sfirst[sg + 1] - S.sfirst[sg])) {
      const double uc = seg_total_l2(S, sg, part);
      if (threadIdx.x == 0) seg_set_alpha(S, sg, uc);
    }
  }
}

// x += alpha u (FP64), r -= alpha c (FP32), with a local preconditioner the
// next z and z.r; the segment's last block decides whether a reliable update
// is due (recurrence residual below MX_DELTA of the last true one, at the
// tolerance, or at maxiter) and otherwise moves rho on.
template <int P>
__global__ void __launch_bounds__(CG_THREADS)
k_mx_update(Seg S, double *__restrict__ xw, float *__restrict__ r, const float *__restrict__ u,
            const float *__restrict__ c, double *__restrict__ part, double *__restrict__ part2,
            const double *__restrict__ pinv, int mode, bool local_prec, const uint8_t *__restrict__ fixed,
            float *__restrict__ z) {
  for (int64_t ch = blockIdx.x; ch < S.nchunks; ch += gridDim.x) {
    const int sg = S.cseg[ch];
    const SegState &q = S.st[sg];
    if (q.done) continue;
    const double alpha = q.alpha;
    const float af = __double2float_rn(alpha);
    double rr = 0.0, zr = 0.0;
    const int64_t b = S.cbeg[ch], e = S.cend[ch];
#pragma unroll
    for (int k = 0; k < CHUNK_PER_THREAD; ++k) {
      const int64_t i = b + threadIdx.x + (int64_t)k * CG_THREADS;
      if (i < e) {
        xw[i] = __fma_rn(alpha, (double)u[i], xw[i]);
        const float ri = fmaf(-af, c[i], r[i]);
        r[i] = ri;
        rr = __fma_rn((double)ri, (double)ri, rr);
      }
    }
    if (local_prec) {
      __syncthreads();
      for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const float zi = fixed[i] ? 0.f : apply_prec32<P>(pinv, mode, r, i);
        z[i] = zi;
        zr = __fma_rn((double)zi, (double)r[i], zr);
      }
    }
    const double s1 = block_sum(rr);
    const double s2 = local_prec ? block_sum(zr) : 0.0;
    if (threadIdx.x == 0) {
      part[ch] = s1;
      if (local_prec) part2[ch] = s2;
    }
    if (arrive_last(S.arrive + S.nseg + sg, S.sfirst[sg + 1] - S.sfirst[sg])) {
      const double trr = seg_total_l2(S, sg, part);
      const double tzr = local_prec ? seg_total_l2(S, sg, part2) : 0.0;
      if (threadIdx.x == 0) {
        SegState &w = S.st[sg];
        const double res32 = sqrt(trr);
        w.it += 1;
        w.rho_prev = w.rho;
        if (res32 <= w.tol || res32 <= MX_DELTA * w.rmax || w.it >= w.maxiter || !isfinite(res32)) {
          w.upd = 1;
        } else if (local_prec) {
          w.rho = tzr;
        }
      }
    }
  }
}

// Reliable update of the systems that asked for one: r64 = rb - A64 x (FP64
// product, masked), r = (float) r64, with a local preconditioner z = M^-1 r
// and z.r; the system's last block takes the true residual: done when it
// meets the tolerance (or at maxiter), otherwise it becomes the new
// reference of the update test.
template <int P>
__global__ void __launch_bounds__(CG_THREADS)
k_mx_true(Seg S, const double *__restrict__ nz, const int64_t *__restrict__ nptr, const int32_t *__restrict__ nadj,
          const double *__restrict__ xw, const double *__restrict__ rb, const uint8_t *__restrict__ fixed,
          float *__restrict__ r, const double *__restrict__ pinv, int mode, bool local_prec, float *__restrict__ z,
          double *__restrict__ part, double *__restrict__ part2) {
  constexpr int NPW = 32 / SPMV_G;
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5, w = threadIdx.x >> 5, g = lane % SPMV_G;
  for (int64_t ch = blockIdx.x; ch < S.nchunks; ch += gridDim.x) {
    const int sg = S.cseg[ch];
    {
      const SegState &q = S.st[sg];
      if (q.done || !q.upd) continue;
    }
    double rr = 0.0, zr = 0.0;
    const int64_t b0 = S.cbeg[ch] / P;
    const int nb = (int)(S.cend[ch] / P - b0);
    for (int r0 = w * NPW; r0 < nb; r0 += wpb * NPW) {
      const int rr_idx = r0 + lane / SPMV_G;
      const bool valid = rr_idx < nb;
      const int64_t B = b0 + (valid ? rr_idx : 0);
      double acc[P];
      node_columns<P>(nz, nptr, nadj, xw, B, valid, g, acc);
      if (valid && g == 0) {
        float rn[P];
#pragma unroll
        for (int j = 0; j < P; ++j) {
          const int64_t d = P * B + j;
          const double v = fixed[d] ? 0.0 : __dsub_rn(rb[d], acc[j]);
          rn[j] = __double2float_rn(v);
          r[d] = rn[j];
          rr = __fma_rn(v, v, rr);
        }
        if (local_prec) {
#pragma unroll
          for (int j = 0; j < P; ++j) {
            const int64_t d = P * B + j;
            float zi = 0.f;
            if (!fixed[d]) {
              if (mode == LLF_PRECOND_BJACOBI) {
                double a = 0.0;
#pragma unroll
                for (int k = 0; k < P; ++k) a = __fma_rn(pinv[(size_t)B * P * P + j * P + k], (double)rn[k], a);
                zi = __double2float_rn(a);
              } else {
                zi = __double2float_rn(__dmul_rn(pinv[d], (double)rn[j]));
              }
            }
            z[d] = zi;
            zr = __fma_rn((double)zi, (double)rn[j], zr);
          }
        }
      }
    }
    const double s1 = block_sum(rr);
    const double s2 = local_prec ? block_sum(zr) : 0.0;
    if (threadIdx.x == 0) {
      part[ch] = s1;
      if (local_prec) part2[ch] = s2;
    }
    if (arrive_last(S.arrive + 2 * S.nseg + sg, S.sfirst[sg + 1] - S.sfirst[sg])) {
      const double trr = seg_total_l2(S, sg, part);
      const double tzr = local_prec ? seg_total_l2(S, sg, part2) : 0.0;
      if (threadIdx.x == 0) {
        SegState &q = S.st[sg];
        q.res = sqrt(trr);
        q.upd = 0;
        if (q.res <= q.tol || q.it >= q.maxiter || !isfinite(q.res)) {
          if (!isfinite(q.res)) q.breakdown = 1;
          q.done = 1;
          atomicSub(S.active, 1);
        } else {
          q.rmax = q.res;
          if (local_prec) q.rho = tzr;
        }
      }
    }
  }
}

// z.r after an IC(0) application in the mixed CG (z in FP32).
__global__ void __launch_bounds__(CG_THREADS)
k_mx_zr(Seg S, const float *__restrict__ zf, const float *__restrict__ r, double *__restrict__ part) {
  for (int64_t ch = blockIdx.x; ch < S.nchunks; ch += gridDim.x) {
    if (S.st[S.cseg[ch]].done) continue;
    double zr = 0.0;
    const int64_t b = S.cbeg[ch], e = S.cend[ch];
#pragma unroll
    for (int k = 0; k < CHUNK_PER_THREAD; ++k) {
      const int64_t i = b + threadIdx.x + (int64_t)k * CG_THREADS;
      if (i < e) zr = __fma_rn((double)zf[i], (double)r[i], zr);
    }
    const double sm = block_sum(zr);
    if (threadIdx.x == 0) part[ch] = sm;
    const int sg = S.cseg[ch];
    if (arrive_last(S.arrive + 2 * S.nseg + sg, S.sfirst[sg + 1] - S.sfirst[sg])) {
      const double t = seg_total_l2(S, sg, part);
      if (threadIdx.x == 0) S.st[sg].rho = t;
    }
  }
}


template <int P>
void enqueue_iteration_mixed(llf_ctx *ctx, const Seg &S, const llf_matrix *m, const double *pinv, int precond,
                             const MixedBufs &B, double *xw, const uint8_t *fixed, double *part, double *part2,
                             double *part3, const IcApply &ic) {
  const llf_pattern *pat = m->pat;
  cudaStream_t s = ctx->stream;
  const bool local = precond != LLF_PRECOND_IC0;
  float *z = local ? B.z : ic.zf;
  { KernelScope k(ctx, "k_mx_dir"); k_mx_dir<<<chunk_grid(S), CG_THREADS, 0, s>>>(S, z, B.u); }
  { KernelScope k(ctx, "k_mx_spmv");
    k_mx_spmv<P><<<chunk_grid(S), CG_THREADS, 0, s>>>(S, B.nz32, pat->d_nptr, pat->d_nadj, B.u, fixed, B.c, part3); }
  { KernelScope k(ctx, "k_mx_update");
    k_mx_update<P><<<chunk_grid(S), CG_THREADS, 0, s>>>(S, xw, B.r, B.u, B.c, part, part2, pinv, precond, local,
                                                        fixed, z); }
  { KernelScope k(ctx, "k_mx_true");
    k_mx_true<P><<<chunk_grid(S), CG_THREADS, 0, s>>>(S, m->d_nz, pat->d_nptr, pat->d_nadj, xw, B.rb, fixed, B.r,
                                                      pinv, precond, local, z, part, part2); }
  if (!local) {
    enqueue_ic0_sweeps<P, float>(ctx, S, ic, B.r);
    { KernelScope k(ctx, "k_mx_zr"); k_mx_zr<<<chunk_grid(S), CG_THREADS, 0, s>>>(S, ic.zf, B.r, part); }
  }
}

// The mixed CG of every segment of S to completion (caller's buffers; no
// allocation); the final per-segment states go to hst.
template <int P>
int pcg_mixed_core(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x, const uint8_t *d_fixed,
                   const Seg &S, const MixedBufs &B, double *xw, double *tmp, double *pinv, double *part,
                   double *part2, double *part3, int precond, double reltol, int64_t maxiter, bool use_graph,
                   SegState *hst, const IcApply &ic) {
  const llf_pattern *pat = m->pat;
  const int64_t n = pat->ndof;
  const int64_t nch = S.nchunks;
  const int nseg = S.nseg;
  cudaStream_t s = ctx->stream;
  const unsigned gch = (unsigned)std::max<int64_t>(1, std::min<int64_t>(nch, (int64_t)ctx->num_sms * 8));
  const unsigned gseg = (unsigned)std::max(1, std::min(nseg, ctx->num_sms * 8));
  const unsigned gv = (unsigned)(ctx->num_sms * 4);
  const bool local = precond != LLF_PRECOND_IC0;
  if (local) {
    KernelScope k(ctx, "k_precond_setup");
    k_precond_setup<P><<<(unsigned)((pat->mesh->non + 127) / 128), 128, 0, s>>>(
        m->d_nz, pat->d_colptr, pat->d_diagpos, d_fixed, pat->mesh->non, precond, pinv);
  }
  { KernelScope k(ctx, "k_f64_to_f32");
    k_f64_to_f32<<<(unsigned)(ctx->num_sms * 8), CG_THREADS, 0, s>>>(m->d_nz, B.nz32, pat->nnz); }
  { KernelScope k(ctx, "k_keep_fixed"); k_keep_fixed<<<gv, CG_THREADS, 0, s>>>(d_x, d_fixed, xw, n); }
  { KernelScope k(ctx, "k_spmv"); k_spmv<P><<<gv, CG_THREADS, 0, s>>>(m->d_nz, pat->d_colptr, pat->d_nptr, pat->d_nadj, xw, tmp, n); }
  { KernelScope k(ctx, "k_mx_init"); k_mx_init<<<gch, CG_THREADS, 0, s>>>(S, d_b, tmp, d_fixed, B.rb, B.r, xw, B.u, part); }
  { KernelScope k(ctx, "k_seg_start"); k_seg_start<<<gseg, CG_THREADS, 0, s>>>(S, part, reltol, (long long)maxiter); }
  if (local) {
    { KernelScope k(ctx, "k_mx_prec"); k_mx_prec<P><<<gch, CG_THREADS, 0, s>>>(S, pinv, precond, B.r, d_fixed, B.z, part); }
    { KernelScope k(ctx, "k_seg_rho"); k_seg_rho<<<gseg, CG_THREADS, 0, s>>>(S, part); }
  } else {
    enqueue_ic0_sweeps<P, float>(ctx, S, ic, B.r);
    { KernelScope k(ctx, "k_mx_zr"); k_mx_zr<<<chunk_grid(S), CG_THREADS, 0, s>>>(S, ic.zf, B.r, part); }
  }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  const int per_graph = 16;
  long long launches_per_graph = 0;
  cudaGraphExec_t exec = nullptr;
  bool graph_ok = use_graph;
  if (graph_ok) {
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const long long saved = ctx->launches;
      for (int k = 0; k < per_graph; ++k)
        enqueue_iteration_mixed<P>(ctx, S, m, pinv, precond, B, xw, d_fixed, part, part2, part3, ic);
      launches_per_graph = ctx->launches - saved;
      ctx->launches = saved;
      if (cudaStreamEndCapture(s, &graph) != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
        graph_ok = false;
      if (graph) cudaGraphDestroy(graph);
    } else {
      graph_ok = false;
    }
    cudaGetLastError();
  }
  int active = 1;
  int *h_active = (int *)ctx->h_status;
  while (active > 0) {
    if (graph_ok) {
      LLF_CUDA_TRY(ctx, cudaGraphLaunch(exec, s));
      ctx->launches += launches_per_graph;
    } else {
      for (int k = 0; k < per_graph; ++k)
        enqueue_iteration_mixed<P>(ctx, S, m, pinv, precond, B, xw, d_fixed, part, part2, part3, ic);
    }
    LLF_CUDA_TRY(ctx, cudaGetLastError());
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(h_active, S.active, sizeof(int), cudaMemcpyDeviceToHost, s));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    active = *h_active;
  }
  *h_active = 0;
  if (exec) cudaGraphExecDestroy(exec);
  { KernelScope k(ctx, "k_cg_merge"); k_cg_merge<<<gv, CG_THREADS, 0, s>>>(xw, d_fixed, d_x, n); }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(hst, S.st, sizeof(SegState) * nseg, cudaMemcpyDeviceToHost, s));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  return LLF_OK;
}

// Per-segment iteration counts and residuals; error for breakdown or
// non-convergence (first offending system named).
int pcg_outcome(llf_ctx *ctx, int nseg, const SegState *hst, int64_t *iters, double *relres) {
  int rc = LLF_OK;
  int worst = -1;
  for (int g = 0; g < nseg; ++g) {
    iters[g] = hst[g].it;
    relres[g] = hst[g].res0 > 0 ? hst[g].res / hst[g].res0 : 0.0;
    if (hst[g].breakdown) {
      rc = LLF_ERR_NUMERIC;
      worst = g;
    } else if (!(hst[g].res <= hst[g].tol) && rc == LLF_OK) {
      rc = LLF_ERR_NOT_CONVERGED;
      worst = g;
    }
  }
  if (rc == LLF_ERR_NUMERIC)
    return llf_fail(ctx, rc, "pcg: breakdown (u.Au <= 0) in system " + std::to_string(worst) +
                                 ": matrix not positive definite on the free DoFs");
  if (rc == LLF_ERR_NOT_CONVERGED)
    return llf_fail(ctx, rc, "pcg: not converged after " + std::to_string(iters[worst]) +
                                 " iterations (system " + std::to_string(worst) + "), relative residual " +
                                 std::to_string(relres[worst]));
  return LLF_OK;
}

// ---------------------------------------------------------------- no-alloc PCG
// Fixed device scratch for llf_pcg_noalloc: every work vector of one CG of
// at most LLF_NOALLOC_MAX_DOFS unknowns, the chunk descriptors of a single
// system and its state word.  Each GPU that loads the library holds this
// array until the process exits.  Regions are 256-byte aligned.
constexpr int64_t NA_N = LLF_NOALLOC_MAX_DOFS;
constexpr int64_t NA_CH = (NA_N + CHUNK - 1) / CHUNK;
constexpr size_t na_round(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t NA_VEC = na_round(sizeof(double) * NA_N);
constexpr size_t NA_OFF_PINV = 5 * NA_VEC;                       // r, z, u, c, xw
constexpr size_t NA_OFF_PART = NA_OFF_PINV + 3 * NA_VEC;         // pinv (up to 3 per DoF)
constexpr size_t NA_OFF_CB = NA_OFF_PART + na_round(sizeof(double) * NA_CH);
constexpr size_t NA_OFF_CE = NA_OFF_CB + na_round(sizeof(int64_t) * NA_CH);
constexpr size_t NA_OFF_SF = NA_OFF_CE + na_round(sizeof(int64_t) * NA_CH);
constexpr size_t NA_OFF_CS = NA_OFF_SF + na_round(sizeof(int64_t) * 2);
constexpr size_t NA_OFF_ST = NA_OFF_CS + na_round(sizeof(int32_t) * NA_CH);
constexpr size_t NA_OFF_ACT = NA_OFF_ST + na_round(sizeof(SegState));  // active counter, then 3 arrival counters
constexpr size_t NA_OFF_PART2 = NA_OFF_ACT + 256;
constexpr size_t NA_OFF_PART3 = NA_OFF_PART2 + na_round(sizeof(double) * NA_CH);
constexpr size_t NA_OFF_PERM = NA_OFF_PART3 + na_round(sizeof(double) * NA_CH);
constexpr size_t NA_BYTES = NA_OFF_PERM + na_round(sizeof(int16_t) * NA_N);  // the product's node order (<= NA_N nodes)

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

namespace {

// Uniform chunks of one system of n DoFs (chunk count nch <= NA_CH).
__global__ void k_na_chunks(int64_t *cb, int64_t *ce, int32_t *cs, int64_t *sf, int64_t n, int64_t nch) {
  for (int64_t ch = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ch < nch;
       ch += (int64_t)gridDim.x * blockDim.x) {
    cb[ch] = ch * CHUNK;
    ce[ch] = (ch + 1) * CHUNK < n ? (ch + 1) * CHUNK : n;
    cs[ch] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sf[0] = 0;
    sf[1] = nch;
  }
}

// Device address of the scratch array, looked up once per device with that
// device current (host code must not use the symbol itself as an address).
std::mutex g_na_mutex;
unsigned char *g_na_ptr[128] = {nullptr};

int noalloc_scratch(llf_ctx *ctx, unsigned char **out) {
  if (ctx->device < 0 || ctx->device >= 128) return llf_fail(ctx, LLF_ERR_ARG, "device index");
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_ptr[ctx->device]) {
    // the lookup needs the context's device current; the caller's current
    // device is put back afterwards, on the error path too
    int prev = -1;
    LLF_CUDA_TRY(ctx, cudaGetDevice(&prev));
    LLF_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    cudaError_t e2 = cudaSetDevice(prev);
    if (e != cudaSuccess || !p)
      return llf_fail(ctx, LLF_ERR_CUDA, std::string("llf_pcg_noalloc: cudaGetSymbolAddress of the scratch array failed: ") +
                                             cudaGetErrorString(e));
    if (e2 != cudaSuccess)
      return llf_fail(ctx, LLF_ERR_CUDA, std::string("llf_pcg_noalloc: restoring the current device failed: ") +
                                             cudaGetErrorString(e2));
    g_na_ptr[ctx->device] = (unsigned char *)p;
  }
  *out = g_na_ptr[ctx->device];
  return LLF_OK;
}

template <int P>
int pcg_noalloc_typed(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x,
                      const uint8_t *d_fixed, int precond, double reltol, int64_t maxiter,
                      int64_t *iters, double *relres) {
  const int64_t n = m->pat->ndof;
  unsigned char *base = nullptr;
  int rc = noalloc_scratch(ctx, &base);
  if (rc != LLF_OK) return rc;
  double *r = (double *)(base + 0 * NA_VEC), *z = (double *)(base + 1 * NA_VEC);
  double *u = (double *)(base + 2 * NA_VEC), *c = (double *)(base + 3 * NA_VEC);
  double *xw = (double *)(base + 4 * NA_VEC), *pinv = (double *)(base + NA_OFF_PINV);
  double *part = (double *)(base + NA_OFF_PART);
  int64_t *cb = (int64_t *)(base + NA_OFF_CB), *ce = (int64_t *)(base + NA_OFF_CE);
  int64_t *sf = (int64_t *)(base + NA_OFF_SF);
  int32_t *cs = (int32_t *)(base + NA_OFF_CS);
  SegState *st = (SegState *)(base + NA_OFF_ST);
  int *active = (int *)(base + NA_OFF_ACT);
  int *arrive = active + 1;
  double *part2 = (double *)(base + NA_OFF_PART2), *part3 = (double *)(base + NA_OFF_PART3);
  int16_t *perm = (int16_t *)(base + NA_OFF_PERM);
  const int64_t nch = (n + CHUNK - 1) / CHUNK;
  // the array keeps the previous call's contents: the active-system counter
  // and the three arrival counters must start at zero; every other region
  // is written before it is read
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(active, 0, sizeof(int) * 4, ctx->stream));
  k_na_chunks<<<1, 64, 0, ctx->stream>>>(cb, ce, cs, sf, n, nch);
  ctx->launches++;
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  Seg S{cb, ce, cs, sf, nch, 1, st, active, arrive, perm};
  if (nch) {  // the same node order as llf_pcg's plan, so the same sums
    KernelScope k(ctx, "k_chunk_perm");
    k_chunk_perm<<<chunk_grid(S), CG_THREADS, 0, ctx->stream>>>(S, m->pat->d_nptr, P, perm);
  }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  SegState hst[1];
  rc = pcg_core<P>(ctx, m, d_b, d_x, d_fixed, S, r, z, u, c, xw, pinv, part, part2, part3, precond, reltol, maxiter,
                   false, hst);
  if (rc != LLF_OK) return rc;
  return pcg_outcome(ctx, 1, hst, iters, relres);
}

}  // namespace

int pcg_noalloc_impl(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x,
                     const uint8_t *d_fixed, int precond, double reltol, int64_t maxiter,
                     int64_t *iters, double *relres) {
  if (!m->d_nz && !m->diagonal_only)
    return llf_fail(ctx, LLF_ERR_STATE,
                    "llf_pcg_noalloc: the matrix's structural values are not expanded yet (its assembly wrote the "
                    "stored CSC only); run llf_pcg or llf_matrix_spmv on it once first");
  if (m->diagonal_only)
    return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "llf_pcg_noalloc: lumped (diagonal) matrix");
  const int64_t n = m->pat->ndof;
  if (n > LLF_NOALLOC_MAX_DOFS)
    return llf_fail(ctx, LLF_ERR_LIMIT, "llf_pcg_noalloc: the system has " + std::to_string(n) +
                                            " unknowns; the fixed scratch array holds at most " +
                                            std::to_string((long long)LLF_NOALLOC_MAX_DOFS) +
                                            " (use llf_pcg for larger systems)");
  switch (m->pat->pdim) {
    case 1: return pcg_noalloc_typed<1>(ctx, m, d_b, d_x, d_fixed, precond, reltol, maxiter, iters, relres);
    case 2: return pcg_noalloc_typed<2>(ctx, m, d_b, d_x, d_fixed, precond, reltol, maxiter, iters, relres);
    case 3: return pcg_noalloc_typed<3>(ctx, m, d_b, d_x, d_fixed, precond, reltol, maxiter, iters, relres);
  }
  return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "pdim must be 1, 2 or 3");
}

int spmv_impl(llf_ctx *ctx, const llf_matrix *m, const double *d_x, double *d_y) {
  {
    const int rc = matrix_ensure_nz(ctx, m);
    if (rc != LLF_OK) return rc;
  }
  const int64_t n = m->pat->ndof;
  const unsigned grid = (unsigned)(ctx->num_sms * 4);
  if (m->diagonal_only) {
    KernelScope ks(ctx, "k_diag_scale");
    k_diag_scale<<<grid, CG_THREADS, 0, ctx->stream>>>(m->d_diag, d_x, d_y, n);
  } else {
    KernelScope ks(ctx, "k_spmv");
    const llf_pattern *p = m->pat;
    switch (p->pdim) {
      case 1: k_spmv<1><<<grid, CG_THREADS, 0, ctx->stream>>>(m->d_nz, p->d_colptr, p->d_nptr, p->d_nadj, d_x, d_y, n); break;
      case 2: k_spmv<2><<<grid, CG_THREADS, 0, ctx->stream>>>(m->d_nz, p->d_colptr, p->d_nptr, p->d_nadj, d_x, d_y, n); break;
      case 3: k_spmv<3><<<grid, CG_THREADS, 0, ctx->stream>>>(m->d_nz, p->d_colptr, p->d_nptr, p->d_nadj, d_x, d_y, n); break;
      default: return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "pdim must be 1, 2 or 3");
    }
  }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  return LLF_OK;
}

int pcg_batched_impl(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x,
                     const uint8_t *d_fixed, int nseg, const int64_t *seg_off, int precond,
                     double reltol, int64_t maxiter, int64_t *iters, double *relres, bool mixed) {
  {
    const int rc = matrix_ensure_nz(ctx, m);
    if (rc != LLF_OK) return rc;
  }
  if (m->diagonal_only)
    return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "pcg on a lumped (diagonal) matrix");
  switch (m->pat->pdim) {
    case 1: return pcg_segments<1>(ctx, m, d_b, d_x, d_fixed, nseg, seg_off, precond, reltol, maxiter, iters, relres, mixed);
    case 2: return pcg_segments<2>(ctx, m, d_b, d_x, d_fixed, nseg, seg_off, precond, reltol, maxiter, iters, relres, mixed);
    case 3: return pcg_segments<3>(ctx, m, d_b, d_x, d_fixed, nseg, seg_off, precond, reltol, maxiter, iters, relres, mixed);
  }
  return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "pdim must be 1, 2 or 3");
}

int pcg_impl(llf_ctx *ctx, const llf_matrix *m, const double *d_b, double *d_x,
             const uint8_t *d_fixed, int precond, double reltol, int64_t maxiter,
             int64_t *iters, double *relres) {
  {
    const int rc = matrix_ensure_nz(ctx, m);
    if (rc != LLF_OK) return rc;
  }
  const int64_t off[2] = {0, m->pat->ndof};
  return pcg_batched_impl(ctx, m, d_b, d_x, d_fixed, 1, off, precond, reltol, maxiter, iters, relres);
}

// ---------------------------------------------------------------- FDM
// Transient heat by the theta-method — FDM, src/heat.jl:1466-1616.  T holds
// nsteps columns of ndof values on the device: column 0 the initial state,
// the fixed entries of every column the prescribed values.
//  * theta == 0 with a lumped (diagonal) C: the reference's explicit branch,
//    T1_f = T0_f + (1/c_f) (dt (q^n - K T^n)_f), fixed entries kept;
//  * otherwise (C + theta dt K) T^{n+1} = (C - (1-theta) dt K) T^n
//    + dt q^{n+theta} on the free DoFs, with q^{n+theta} = q when q holds one
//    column and (1-theta) q^n + theta q^{n+1} otherwise; the fixed-DoF
//    couplings (-A_fc Tc^{n+1} + B_fc Tc^n) come from the masked PCG, which
//    solves A_ff x_f = b_f - A_fc x_c with b = B T^n + dt q^{n+theta}.  The
//    reference factorises A once (lu) and back-substitutes each step; here
//    the PCG plan (buffers, chunking, IC(0) factor) is built once and each
//    step starts from the previous state.
namespace {

__global__ void k_fdm_explicit(const double *__restrict__ T0, const double *__restrict__ y,
                               const double *__restrict__ q, const double *__restrict__ cdiag,
                               const uint8_t *__restrict__ fixed, double dt, int64_t n, double *__restrict__ T1) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (!fixed[i])
      T1[i] = __dadd_rn(T0[i], __dmul_rn(__drcp_rn(cdiag[i]), __dmul_rn(dt, __dsub_rn(q[i], y[i]))));
}

__global__ void k_fdm_rhs(const double *__restrict__ y, const double *__restrict__ q0,
                          const double *__restrict__ q1, double theta, double dt, int64_t n,
                          double *__restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double qt = q1 ? __fma_rn(theta, q1[i], __dmul_rn(1.0 - theta, q0[i])) : q0[i];
    b[i] = __fma_rn(dt, qt, y[i]);
  }
}

__global__ void k_fdm_start(const double *__restrict__ Tprev, const uint8_t *__restrict__ fixed, int64_t n,
                            double *__restrict__ Tnext) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (!fixed[i]) Tnext[i] = Tprev[i];
}

__global__ void k_diag_of(const double *__restrict__ nz, const int64_t *__restrict__ colptr,
                          const int32_t *__restrict__ diagpos, int P, int64_t n, double *__restrict__ d) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t B = c / P;
    const int j = (int)(c - B * P);
    d[c] = nz[colptr[c] + (int64_t)P * diagpos[B] + j];
  }
}

__global__ void k_fdm_check_diag(const double *__restrict__ d, const uint8_t *__restrict__ fixed, int64_t n,
                                 int *bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (!fixed[i] && !(d[i] > 0.0)) atomicAdd(bad, 1);
}

void free_matrix_arrays(llf_ctx *ctx, llf_matrix *m) {
  dfree(ctx, m->d_nz); dfree(ctx, m->d_diag); dfree(ctx, m->d_colptr_s);
  dfree(ctx, m->d_rowval_s); dfree(ctx, m->d_nzval_s);
}

template <int P>
int fdm_typed(llf_ctx *ctx, const llf_matrix *K, const llf_matrix *C, const double *d_q, int nq, double *d_T,
              const uint8_t *d_fixed, int64_t nsteps, double dt, double theta, int precond, double reltol,
              int64_t maxiter, int64_t *iters_total) {
  const llf_pattern *pat = K->pat;
  const int64_t n = pat->ndof;
  cudaStream_t s = ctx->stream;
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 16));
  double *cd = nullptr, *y = nullptr, *b = nullptr;
  int rc = LLF_OK;
  *iters_total = 0;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &cd, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &y, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &b, n));
  // diag(C_ff) > 0 (the reference's check on the free DoFs)
  if (C->diagonal_only)
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(cd, C->d_diag, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  else
    k_diag_of<<<g, 256, 0, s>>>(C->d_nz, pat->d_colptr, pat->d_diagpos, P, n, cd);
  {
    int *d_bad = nullptr, h_bad = 0;
    LLF_CUDA_TRY(ctx, dalloc(ctx, &d_bad, 1));
    LLF_CUDA_TRY(ctx, cudaMemsetAsync(d_bad, 0, sizeof(int), s));
    k_fdm_check_diag<<<g, 256, 0, s>>>(cd, d_fixed, n, d_bad);
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(&h_bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    dfree(ctx, d_bad);
    if (h_bad) rc = llf_fail(ctx, LLF_ERR_NUMERIC, "FDM: non-positive diagonal entry detected in Cff on free DOFs.");
  }
  if (rc == LLF_OK && theta == 0.0 && C->diagonal_only) {
    for (int64_t i = 1; i < nsteps && rc == LLF_OK; ++i) {
      const double *T0 = d_T + (i - 1) * n;
      rc = spmv_impl(ctx, K, T0, y);
      if (rc != LLF_OK) break;
      KernelScope ks(ctx, "k_fdm_explicit");
      k_fdm_explicit<<<g, 256, 0, s>>>(T0, y, d_q + (nq == 1 ? 0 : (i - 1) * n), cd, d_fixed, dt, n, d_T + i * n);
    }
  } else if (rc == LLF_OK) {
    llf_matrix A, Bm;
    A.pat = Bm.pat = K->pat;
    rc = matrix_axpby_impl(ctx, 1.0, C, theta * dt, K, &A);
    if (rc == LLF_OK) rc = matrix_axpby_impl(ctx, 1.0, C, -((1.0 - theta) * dt), K, &Bm);
    PcgPlan<P> plan;
    const int64_t off[2] = {0, n};
    bool planned = false;
    if (rc == LLF_OK) {
      rc = plan.create(ctx, &A, d_fixed, 1, off, precond);
      planned = true;
    }
    for (int64_t i = 1; i < nsteps && rc == LLF_OK; ++i) {
      const double *T0 = d_T + (i - 1) * n;
      double *T1 = d_T + i * n;
      rc = spmv_impl(ctx, &Bm, T0, y);
      if (rc != LLF_OK) break;
      {
        KernelScope ks(ctx, "k_fdm_rhs");
        k_fdm_rhs<<<g, 256, 0, s>>>(y, d_q + (nq == 1 ? 0 : (i - 1) * n), nq == 1 ? nullptr : d_q + i * n, theta,
                                    dt, n, b);
        k_fdm_start<<<g, 256, 0, s>>>(T0, d_fixed, n, T1);
      }
      int64_t it = 0;
      double rr = 0.0;
      rc = plan.solve(ctx, &A, b, T1, d_fixed, reltol, maxiter, &it, &rr);
      *iters_total += it;
    }
    if (planned) plan.destroy(ctx);
    free_matrix_arrays(ctx, &A);
    free_matrix_arrays(ctx, &Bm);
  }
  dfree(ctx, cd);
  dfree(ctx, y);
  dfree(ctx, b);
  if (rc == LLF_OK) LLF_CUDA_TRY(ctx, cudaGetLastError());
  return rc;
}

}  // namespace

int heat_fdm_impl(llf_ctx *ctx, const llf_matrix *K, const llf_matrix *C, const double *d_q, int nq, double *d_T,
                  const uint8_t *d_fixed, int64_t nsteps, double dt, double theta, int precond, double reltol,
                  int64_t maxiter, int64_t *iters_total) {
  {
    int rc = matrix_ensure_nz(ctx, K);
    if (rc == LLF_OK) rc = matrix_ensure_nz(ctx, C);
    if (rc != LLF_OK) return rc;
  }
  switch (K->pat->pdim) {
    case 1: return fdm_typed<1>(ctx, K, C, d_q, nq, d_T, d_fixed, nsteps, dt, theta, precond, reltol, maxiter, iters_total);
    case 2: return fdm_typed<2>(ctx, K, C, d_q, nq, d_T, d_fixed, nsteps, dt, theta, precond, reltol, maxiter, iters_total);
    case 3: return fdm_typed<3>(ctx, K, C, d_q, nq, d_T, d_fixed, nsteps, dt, theta, precond, reltol, maxiter, iters_total);
  }
  return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "pdim must be 1, 2 or 3");
}

// ---------------------------------------------------------------- engine
// Device-resident continuous batching (engine.h): the CG iterations of many
// independent systems, each with its own matrix and vectors, in the same
// launches.  A slot describes one admitted system; the chunk table lists the
// chunks of all admitted systems, each system's chunks contiguous and in its
// own DoF order.  The kernels loop over the table (its length is read from
// device memory), so one captured graph serves whatever is admitted.
#include "engine.h"

namespace {

struct EngSlot {
  const double *nz;
  const int64_t *nptr;
  const int32_t *nadj;
  const uint8_t *fixed;
  const int16_t *perm;
  const double *pinv;
  double *xw, *r, *z, *u, *c;
  int mode, pad;
};

struct EngTab {
  const EngSlot *slot;
  SegState *st;
  int *arrive;                 // 2 per slot: product, update
  const int32_t *cslot;        // per chunk: slot
  const int64_t *cbeg, *cend;  // per chunk: DoF range within its system
  const int64_t *sfirst;       // per slot: first chunk in the table
  const int64_t *snch;         // per slot: chunk count
  const int64_t *nchunks;      // chunks in the table (device)
  double *part, *part2, *part3;
};

__device__ __forceinline__ double eng_total(const EngTab &T, int sl, const double *part) {
  double v = 0.0;
  const int64_t f = T.sfirst[sl], n = T.snch[sl];
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) v = __dadd_rn(v, __ldcg(part + f + k));
  return block_sum(v);
}

// The chunks of a launch are handed out in table order from a counter (one
// per launch, cleared at the start of every replay): the systems' chunks
// differ in cost by more than an order of magnitude (P1 triangles to P4
// tetrahedra), so a fixed assignment would leave blocks idle.
__device__ __forceinline__ int64_t eng_next(unsigned *ctr) {
  __shared__ unsigned long long s_ch;
  __syncthreads();
  if (threadIdx.x == 0) s_ch = atomicAdd(ctr, 1u);
  __syncthreads();
  return (int64_t)s_ch;
}

// u = z + beta u (k_seg_dir on a slot's vectors).
__global__ void __launch_bounds__(CG_THREADS) k_eng_dir(EngTab T, unsigned *ctr) {
  const int64_t nch = *T.nchunks;
  for (int64_t ch = eng_next(ctr); ch < nch; ch = eng_next(ctr)) {
    const int sl = T.cslot[ch];
    const SegState &q = T.st[sl];
    if (q.done) continue;
    const EngSlot &S = T.slot[sl];
    const double beta = q.rho / q.rho_prev;
    const int64_t b = T.cbeg[ch], e = T.cend[ch];
#pragma unroll
    for (int k = 0; k < CHUNK_PER_THREAD; ++k) {
      const int64_t i = b + threadIdx.x + (int64_t)k * CG_THREADS;
      if (i < e) S.u[i] = __fma_rn(beta, S.u[i], S.z[i]);
    }
  }
}

// c = A u and alpha (k_seg_spmv on a slot's matrix and vectors).
template <int P>
__global__ void __launch_bounds__(CG_THREADS) k_eng_spmv(EngTab T, unsigned *ctr) {
  constexpr int NPW = 32 / SPMV_G;
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5, w = threadIdx.x >> 5, g = lane % SPMV_G;
  const int64_t nch = *T.nchunks;
  for (int64_t ch = eng_next(ctr); ch < nch; ch = eng_next(ctr)) {
    const int sl = T.cslot[ch];
    if (T.st[sl].done) continue;
    const EngSlot &S = T.slot[sl];
    double dot = 0.0;
    const int64_t b0 = T.cbeg[ch] / P;
    const int nb = (int)(T.cend[ch] / P - b0);
    const int step = wpb * NPW;
    auto node_of = [&](int r) -> int64_t { return b0 + (r < nb ? (int)S.perm[b0 + r] : 0); };
    int r = w * NPW + lane / SPMV_G;
    int64_t B = node_of(r);
    int64_t q0 = r < nb ? S.nptr[B] : 0, q1 = r < nb ? S.nptr[B + 1] : 0;
    for (int r0 = w * NPW; r0 < nb; r0 += step, r += step) {
      const bool valid = r < nb;
      const int64_t Bn = node_of(r + step);
      const bool vn = r + step < nb;
      const int64_t q0n = vn ? S.nptr[Bn] : 0, q1n = vn ? S.nptr[Bn + 1] : 0;
      double acc[P];
      node_columns_at<P>(S.nz, S.nadj, S.u, q0, q1, valid, g, acc);
      if (valid && g == 0) {
#pragma unroll
        for (int j = 0; j < P; ++j) {
          const int64_t d = P * B + j;
          const double v = S.fixed[d] ? 0.0 : acc[j];
          S.c[d] = v;
          dot = __fma_rn(S.u[d], v, dot);
        }
      }
      B = Bn;
      q0 = q0n;
      q1 = q1n;
    }
    const double s = block_sum(dot);
    if (threadIdx.x == 0) T.part3[ch] = s;
    if (arrive_last(T.arrive + 2 * sl, T.snch[sl])) {
      const double uc = eng_total(T, sl, T.part3);
      if (threadIdx.x == 0) {
        SegState &q = T.st[sl];
        if (!(uc > 0.0) || !isfinite(uc)) {
          q.breakdown = 1;
          q.done = 1;
          q.alpha = 0.0;
        } else {
          q.alpha = q.rho / uc;
        }
      }
    }
  }
}

// x += alpha u, r -= alpha c, the residual check, the next z and rho
// (k_seg_update_fused with a local preconditioner on a slot's vectors).
template <int P>
__global__ void __launch_bounds__(CG_THREADS) k_eng_update(EngTab T, unsigned *ctr) {
  const int64_t nch = *T.nchunks;
  for (int64_t ch = eng_next(ctr); ch < nch; ch = eng_next(ctr)) {
    const int sl = T.cslot[ch];
    const SegState &q = T.st[sl];
    if (q.done) continue;
    const EngSlot &S = T.slot[sl];
    const double alpha = q.alpha;
    double rr = 0.0, zr = 0.0;
    const int64_t b = T.cbeg[ch], e = T.cend[ch];
#pragma unroll
    for (int k = 0; k < CHUNK_PER_THREAD; ++k) {
      const int64_t i = b + threadIdx.x + (int64_t)k * CG_THREADS;
      if (i < e) {
        S.xw[i] = __fma_rn(alpha, S.u[i], S.xw[i]);
        const double ri = __fma_rn(-alpha, S.c[i], S.r[i]);
        S.r[i] = ri;
        rr = __fma_rn(ri, ri, rr);
      }
    }
    __syncthreads();
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
      const double zi = S.fixed[i] ? 0.0 : apply_prec<P>(S.pinv, S.mode, S.r, i);
      S.z[i] = zi;
      zr = __fma_rn(zi, S.r[i], zr);
    }
    const double s1 = block_sum(rr);
    const double s2 = block_sum(zr);
    if (threadIdx.x == 0) {
      T.part[ch] = s1;
      T.part2[ch] = s2;
    }
    if (arrive_last(T.arrive + 2 * sl + 1, T.snch[sl])) {
      const double trr = eng_total(T, sl, T.part);
      const double tzr = eng_total(T, sl, T.part2);
      if (threadIdx.x == 0) {
        SegState &w = T.st[sl];
        w.res = sqrt(trr);
        w.rho_prev = w.rho;
        w.it += 1;
        if (w.res <= w.tol || w.it >= w.maxiter) w.done = 1;
        else w.rho = tzr;
      }
    }
  }
}

}  // namespace

namespace llf_engine {

struct System {
  const llf_matrix *K = nullptr;
  int P = 1, precond = 0;
  int64_t ndof = 0, nch = 0;
  double *b = nullptr, *x = nullptr, *xw = nullptr, *r = nullptr, *z = nullptr, *u = nullptr, *c = nullptr;
  double *pinv = nullptr;
  uint8_t *fixed = nullptr;
  int16_t *perm = nullptr;
  SegState st{};
};

struct Engine {
  llf_ctx *ctx = nullptr;
  int max_systems = 0;
  int64_t max_chunks = 0;
  std::vector<System *> sys;      // per slot (nullptr: free)
  std::vector<int64_t> tag;
  EngSlot *d_slot = nullptr;
  SegState *d_st = nullptr;
  int *d_arrive = nullptr;
  int32_t *d_cslot = nullptr;
  int64_t *d_cbeg = nullptr, *d_cend = nullptr, *d_sfirst = nullptr, *d_snch = nullptr, *d_nch = nullptr;
  double *d_part = nullptr, *d_part2 = nullptr, *d_part3 = nullptr;
  unsigned *d_ctr = nullptr;       // chunk counters, 3 per iteration of a replay
  std::vector<SegState> hst;
  cudaGraphExec_t exec[3] = {nullptr, nullptr, nullptr};  // per P
  long long launches_per_graph = 0;
  bool table_dirty = true;
};

namespace {

template <int P>
int prepare_t(llf_ctx *ctx, const llf_matrix *K, const double *hb, const double *hx0, const uint8_t *hfixed,
              int precond, double reltol, int64_t maxiter, System *sy) {
  const llf_pattern *pat = K->pat;
  const int64_t n = pat->ndof, non = pat->mesh->non;
  cudaStream_t s = ctx->stream;
  sy->P = P;
  sy->precond = precond;
  sy->ndof = n;
  const int64_t nch = (n + CHUNK - 1) / CHUNK;
  sy->nch = nch;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &sy->b, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &sy->x, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &sy->xw, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &sy->r, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &sy->z, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &sy->u, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &sy->c, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &sy->pinv, precond == LLF_PRECOND_BJACOBI ? n * P : n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &sy->fixed, n));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &sy->perm, non));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(sy->b, hb, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(sy->x, hx0, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(sy->fixed, hfixed, n, cudaMemcpyHostToDevice, s));
  // the first steps of pcg_core on a one-system chunking (the same chunks,
  // kernels and node order as llf_pcg)
  std::vector<int64_t> cb(nch), ce(nch), sf{0, nch};
  std::vector<int32_t> cs(nch, 0);
  for (int64_t k = 0; k < nch; ++k) {
    cb[k] = k * CHUNK;
    ce[k] = std::min<int64_t>((k + 1) * CHUNK, n);
  }
  int64_t *d_cb = nullptr, *d_ce = nullptr, *d_sf = nullptr;
  int32_t *d_cs = nullptr;
  int *d_active = nullptr, *d_arrive = nullptr;
  SegState *d_st = nullptr;
  double *part = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &d_cb, nch));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &d_ce, nch));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &d_cs, nch));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &d_sf, 2));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &d_active, 1));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &d_arrive, 3));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &d_st, 1));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &part, nch));
  if (nch) {
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d_cb, cb.data(), sizeof(int64_t) * nch, cudaMemcpyHostToDevice, s));
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d_ce, ce.data(), sizeof(int64_t) * nch, cudaMemcpyHostToDevice, s));
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d_cs, cs.data(), sizeof(int32_t) * nch, cudaMemcpyHostToDevice, s));
  }
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d_sf, sf.data(), sizeof(int64_t) * 2, cudaMemcpyHostToDevice, s));
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(d_active, 0, sizeof(int), s));
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(d_arrive, 0, sizeof(int) * 3, s));
  Seg S{d_cb, d_ce, d_cs, d_sf, nch, 1, d_st, d_active, d_arrive, sy->perm};
  const unsigned gch = (unsigned)std::max<int64_t>(1, std::min<int64_t>(nch, (int64_t)ctx->num_sms * 8));
  const unsigned gv = (unsigned)(ctx->num_sms * 4);
  if (nch) {
    KernelScope k(ctx, "k_chunk_perm");
    k_chunk_perm<<<chunk_grid(S), CG_THREADS, 0, s>>>(S, pat->d_nptr, P, sy->perm);
  }
  { KernelScope k(ctx, "k_precond_setup");
    k_precond_setup<P><<<(unsigned)((non + 127) / 128), 128, 0, s>>>(K->d_nz, pat->d_colptr, pat->d_diagpos, sy->fixed,
                                                                     non, precond, sy->pinv); }
  { KernelScope k(ctx, "k_keep_fixed"); k_keep_fixed<<<gv, CG_THREADS, 0, s>>>(sy->x, sy->fixed, sy->xw, n); }
  { KernelScope k(ctx, "k_spmv");
    k_spmv<P><<<gv, CG_THREADS, 0, s>>>(K->d_nz, pat->d_colptr, pat->d_nptr, pat->d_nadj, sy->xw, sy->c, n); }
  { KernelScope k(ctx, "k_seg_init"); k_seg_init<<<gch, CG_THREADS, 0, s>>>(S, sy->b, sy->c, sy->fixed, sy->r, sy->xw, sy->u, part); }
  { KernelScope k(ctx, "k_seg_start"); k_seg_start<<<1, CG_THREADS, 0, s>>>(S, part, reltol, (long long)maxiter); }
  { KernelScope k(ctx, "k_seg_prec"); k_seg_prec<P><<<gch, CG_THREADS, 0, s>>>(S, sy->pinv, precond, sy->r, sy->fixed, sy->z, part); }
  { KernelScope k(ctx, "k_seg_rho"); k_seg_rho<<<1, CG_THREADS, 0, s>>>(S, part); }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(&sy->st, d_st, sizeof(SegState), cudaMemcpyDeviceToHost, s));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  dfree(ctx, d_cb); dfree(ctx, d_ce); dfree(ctx, d_cs); dfree(ctx, d_sf); dfree(ctx, d_active);
  dfree(ctx, d_arrive); dfree(ctx, d_st); dfree(ctx, part);
  return LLF_OK;
}

template <int P>
void enqueue_engine_iteration(Engine *e, const EngTab &T, unsigned *ctr) {
  cudaStream_t s = e->ctx->stream;
  const unsigned grid = (unsigned)(e->ctx->num_sms * 8);
  { KernelScope k(e->ctx, "k_eng_dir"); k_eng_dir<<<grid, CG_THREADS, 0, s>>>(T, ctr); }
  { KernelScope k(e->ctx, "k_eng_spmv"); k_eng_spmv<P><<<grid, CG_THREADS, 0, s>>>(T, ctr + 1); }
  { KernelScope k(e->ctx, "k_eng_update"); k_eng_update<P><<<grid, CG_THREADS, 0, s>>>(T, ctr + 2); }
}

EngTab tab_of(Engine *e) {
  return EngTab{e->d_slot, e->d_st, e->d_arrive, e->d_cslot, e->d_cbeg, e->d_cend, e->d_sfirst, e->d_snch,
                e->d_nch, e->d_part, e->d_part2, e->d_part3};
}

// Chunk table of the admitted systems (slot order), uploaded on the stream.
int upload_table(Engine *e) {
  llf_ctx *ctx = e->ctx;
  std::vector<int32_t> cslot;
  std::vector<int64_t> cbeg, cend, sfirst(e->max_systems, 0), snch(e->max_systems, 0);
  for (int sl = 0; sl < e->max_systems; ++sl) {
    System *sy = e->sys[sl];
    if (!sy) continue;
    sfirst[sl] = (int64_t)cslot.size();
    snch[sl] = sy->nch;
    for (int64_t k = 0; k < sy->nch; ++k) {
      cslot.push_back(sl);
      cbeg.push_back(k * CHUNK);
      cend.push_back(std::min<int64_t>((k + 1) * CHUNK, sy->ndof));
    }
  }
  const int64_t nch = (int64_t)cslot.size();
  cudaStream_t s = ctx->stream;
  if (nch) {
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(e->d_cslot, cslot.data(), sizeof(int32_t) * nch, cudaMemcpyHostToDevice, s));
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(e->d_cbeg, cbeg.data(), sizeof(int64_t) * nch, cudaMemcpyHostToDevice, s));
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(e->d_cend, cend.data(), sizeof(int64_t) * nch, cudaMemcpyHostToDevice, s));
  }
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(e->d_sfirst, sfirst.data(), sizeof(int64_t) * e->max_systems,
                                    cudaMemcpyHostToDevice, s));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(e->d_snch, snch.data(), sizeof(int64_t) * e->max_systems, cudaMemcpyHostToDevice, s));
  // the host vectors must outlive the copies
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(e->d_nch, &nch, sizeof(int64_t), cudaMemcpyHostToDevice, s));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  e->table_dirty = false;
  return LLF_OK;
}

int64_t chunks_in_use(const Engine *e) {
  int64_t n = 0;
  for (System *sy : e->sys)
    if (sy) n += sy->nch;
  return n;
}

}  // namespace

int prepare(llf_ctx *ctx, const llf_matrix *K, const double *b, const double *x0, const uint8_t *fixed,
            int precond, double reltol, int64_t maxiter, System **out) {
  if (!ctx || !K || !b || !x0 || !fixed || !out) return LLF_ERR_ARG;
  if (K->diagonal_only) return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "engine: lumped (diagonal) matrix");
  {
    const int rc = matrix_ensure_nz(ctx, K);
    if (rc != LLF_OK) return rc;
  }
  if (precond < LLF_PRECOND_NONE || precond > LLF_PRECOND_BJACOBI)
    return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "engine: preconditioner must be none, Jacobi or block Jacobi");
  auto *sy = new System();
  sy->K = K;
  int rc = LLF_ERR_UNSUPPORTED;
  switch (K->pat->pdim) {
    case 1: rc = prepare_t<1>(ctx, K, b, x0, fixed, precond, reltol, maxiter, sy); break;
    case 2: rc = prepare_t<2>(ctx, K, b, x0, fixed, precond, reltol, maxiter, sy); break;
    case 3: rc = prepare_t<3>(ctx, K, b, x0, fixed, precond, reltol, maxiter, sy); break;
  }
  if (rc != LLF_OK) {
    release(ctx, sy);
    return rc;
  }
  *out = sy;
  return LLF_OK;
}

void release(llf_ctx *ctx, System *sy) {
  if (!sy) return;
  dfree(ctx, sy->b); dfree(ctx, sy->x); dfree(ctx, sy->xw); dfree(ctx, sy->r); dfree(ctx, sy->z);
  dfree(ctx, sy->u); dfree(ctx, sy->c); dfree(ctx, sy->pinv); dfree(ctx, sy->fixed); dfree(ctx, sy->perm);
  delete sy;
}

int create(llf_ctx *ctx, int max_systems, int64_t max_chunks, Engine **out) {
  if (!ctx || !out || max_systems < 1 || max_chunks < 1) return LLF_ERR_ARG;
  auto *e = new Engine();
  e->ctx = ctx;
  e->max_systems = max_systems;
  e->max_chunks = max_chunks;
  e->sys.assign(max_systems, nullptr);
  e->tag.assign(max_systems, 0);
  e->hst.assign(max_systems, SegState{});
  cudaStream_t s = ctx->stream;
  auto fail = [&](cudaError_t err) {
    destroy(e);
    return llf_fail(ctx, LLF_ERR_CUDA, std::string("engine: ") + cudaGetErrorString(err));
  };
  cudaError_t err = dalloc(ctx, &e->d_slot, max_systems);
  if (err == cudaSuccess) err = dalloc(ctx, &e->d_st, max_systems);
  if (err == cudaSuccess) err = dalloc(ctx, &e->d_arrive, 2 * (int64_t)max_systems);
  if (err == cudaSuccess) err = dalloc(ctx, &e->d_cslot, max_chunks);
  if (err == cudaSuccess) err = dalloc(ctx, &e->d_cbeg, max_chunks);
  if (err == cudaSuccess) err = dalloc(ctx, &e->d_cend, max_chunks);
  if (err == cudaSuccess) err = dalloc(ctx, &e->d_sfirst, max_systems);
  if (err == cudaSuccess) err = dalloc(ctx, &e->d_snch, max_systems);
  if (err == cudaSuccess) err = dalloc(ctx, &e->d_nch, 1);
  if (err == cudaSuccess) err = dalloc(ctx, &e->d_part, max_chunks);
  if (err == cudaSuccess) err = dalloc(ctx, &e->d_part2, max_chunks);
  if (err == cudaSuccess) err = dalloc(ctx, &e->d_part3, max_chunks);
  if (err == cudaSuccess) err = dalloc(ctx, &e->d_ctr, 3 * 16);
  if (err == cudaSuccess) err = cudaMemsetAsync(e->d_arrive, 0, sizeof(int) * 2 * max_systems, s);
  if (err == cudaSuccess) err = cudaMemsetAsync(e->d_st, 0, sizeof(SegState) * max_systems, s);
  if (err == cudaSuccess) err = cudaMemsetAsync(e->d_slot, 0, sizeof(EngSlot) * max_systems, s);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) return fail(err);
  int rc = upload_table(e);
  if (rc != LLF_OK) {
    destroy(e);
    return rc;
  }
  *out = e;
  return LLF_OK;
}

void destroy(Engine *e) {
  if (!e) return;
  llf_ctx *ctx = e->ctx;
  for (int sl = 0; sl < e->max_systems; ++sl)
    if (e->sys[sl]) release(ctx, e->sys[sl]);
  for (auto &x : e->exec)
    if (x) cudaGraphExecDestroy(x);
  dfree(ctx, e->d_slot); dfree(ctx, e->d_st); dfree(ctx, e->d_arrive); dfree(ctx, e->d_cslot);
  dfree(ctx, e->d_cbeg); dfree(ctx, e->d_cend); dfree(ctx, e->d_sfirst); dfree(ctx, e->d_snch);
  dfree(ctx, e->d_nch); dfree(ctx, e->d_part); dfree(ctx, e->d_part2); dfree(ctx, e->d_part3);
  dfree(ctx, e->d_ctr);
  cudaStreamSynchronize(ctx->stream);
  delete e;
}

int admitted(const Engine *e) {
  int n = 0;
  for (System *sy : e->sys) n += sy != nullptr;
  return n;
}

int admit(Engine *e, System *sy, int64_t tag) {
  llf_ctx *ctx = e->ctx;
  if (!sy) return llf_fail(ctx, LLF_ERR_ARG, "engine: null system");
  for (int sl = 0; sl < e->max_systems; ++sl)
    if (e->sys[sl] && e->sys[sl]->P != sy->P)
      return llf_fail(ctx, LLF_ERR_STATE, "engine: all admitted systems must have the same DoFs per node");
  if (chunks_in_use(e) + sy->nch > e->max_chunks) return 0;
  int sl = -1;
  for (int k = 0; k < e->max_systems; ++k)
    if (!e->sys[k]) { sl = k; break; }
  if (sl < 0) return 0;
  const llf_pattern *pat = sy->K->pat;
  EngSlot d{sy->K->d_nz, pat->d_nptr, pat->d_nadj, sy->fixed, sy->perm, sy->pinv,
            sy->xw, sy->r, sy->z, sy->u, sy->c, sy->precond, 0};
  cudaStream_t s = ctx->stream;
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(e->d_slot + sl, &d, sizeof(EngSlot), cudaMemcpyHostToDevice, s));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(e->d_st + sl, &sy->st, sizeof(SegState), cudaMemcpyHostToDevice, s));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  e->sys[sl] = sy;
  e->tag[sl] = tag;
  e->hst[sl] = sy->st;
  e->table_dirty = true;
  return 1;
}

int step(Engine *e) {
  llf_ctx *ctx = e->ctx;
  if (e->table_dirty) {
    int rc = upload_table(e);
    if (rc != LLF_OK) return rc;
  }
  int P = 0;
  for (System *sy : e->sys)
    if (sy) { P = sy->P; break; }
  if (!P) return LLF_OK;
  cudaStream_t s = ctx->stream;
  const EngTab T = tab_of(e);
  const int per_graph = 16;
  auto enqueue = [&]() {
    cudaMemsetAsync(e->d_ctr, 0, sizeof(unsigned) * 3 * per_graph, s);
    for (int k = 0; k < per_graph; ++k) {
      unsigned *ctr = e->d_ctr + 3 * k;
      if (P == 1) enqueue_engine_iteration<1>(e, T, ctr);
      else if (P == 2) enqueue_engine_iteration<2>(e, T, ctr);
      else enqueue_engine_iteration<3>(e, T, ctr);
    }
  };
  cudaGraphExec_t &exec = e->exec[P - 1];
  if (!exec && !ctx->profiling) {
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const long long saved = ctx->launches;
      enqueue();
      e->launches_per_graph = ctx->launches - saved;
      ctx->launches = saved;
      if (cudaStreamEndCapture(s, &graph) != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
        exec = nullptr;
      if (graph) cudaGraphDestroy(graph);
    }
    cudaGetLastError();
  }
  if (exec && !ctx->profiling) {
    LLF_CUDA_TRY(ctx, cudaGraphLaunch(exec, s));
    ctx->launches += e->launches_per_graph;
  } else {
    enqueue();
  }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(e->hst.data(), e->d_st, sizeof(SegState) * e->max_systems,
                                    cudaMemcpyDeviceToHost, s));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  return LLF_OK;
}

int collect(Engine *e, std::vector<Done> &out) {
  llf_ctx *ctx = e->ctx;
  cudaStream_t s = ctx->stream;
  const unsigned gv = (unsigned)(ctx->num_sms * 4);
  std::vector<int> fin;
  for (int sl = 0; sl < e->max_systems; ++sl)
    if (e->sys[sl] && e->hst[sl].done) fin.push_back(sl);
  if (fin.empty()) return LLF_OK;
  const size_t base = out.size();
  for (int sl : fin) {
    System *sy = e->sys[sl];
    Done d;
    d.tag = e->tag[sl];
    d.x.resize(sy->ndof);
    { KernelScope k(ctx, "k_cg_merge"); k_cg_merge<<<gv, CG_THREADS, 0, s>>>(sy->xw, sy->fixed, sy->x, sy->ndof); }
    LLF_CUDA_TRY(ctx, cudaGetLastError());
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d.x.data(), sy->x, sizeof(double) * sy->ndof, cudaMemcpyDeviceToHost, s));
    out.push_back(std::move(d));
  }
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  for (size_t k = 0; k < fin.size(); ++k) {
    const int sl = fin[k];
    const SegState &q = e->hst[sl];
    Done &d = out[base + k];
    d.iters = q.it;
    d.relres = q.res0 > 0 ? q.res / q.res0 : 0.0;
    d.status = q.breakdown ? LLF_ERR_NUMERIC : (q.res <= q.tol ? LLF_OK : LLF_ERR_NOT_CONVERGED);
    release(ctx, e->sys[sl]);
    e->sys[sl] = nullptr;
    e->table_dirty = true;
  }
  return LLF_OK;
}

}  // namespace llf_engine
