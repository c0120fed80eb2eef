// Multicolour node-block incomplete Cholesky, IC(0), for the PCG (the
// preconditioner the reference leaves to the caller's `preconditioner=`
// keyword of solveDisplacement / solveField, src/linear.jl:3711-3743 and
// src/poisson.jl:1432-1546).
//
// Ordering.  The node graph of the pattern is coloured once per pattern
// (Jones-Plassmann rounds with degree-then-hash priorities, first-fit colours: nodes
// coloured in one round are pairwise non-adjacent), and the unknowns are
// ordered colour by colour (within a colour by decreasing degree, which no
// result depends on).  Within a colour no two nodes are coupled, so
// every step of the factorisation and of both triangular solves is
// parallel over the nodes of one colour.
//
// Factor.  L is block lower triangular (p x p blocks on the node pattern,
// zero fill):  for node j of colour c and each neighbour i of an earlier
// colour (colour by colour),
//     L_ji = (A'_ji - sum_k L_jk L_ik^T) L_ii^-T,   k earlier than i, k ~ i, k ~ j
//     L_jj = chol(A'_jj - sum_k L_jk L_jk^T)
// where A' is A with the fixed DoFs' rows and columns replaced by identity.
// L_ji is kept twice: with node j's row list (forward solve) and with node
// i's list (backward solve).  A non-positive pivot sets a flag; the host
// then refactors A + alpha diag(A) with growing alpha.
//
// Apply.  z = (L L^T)^-1 r: forward colour sweep y_j = L_jj^-1 (r_j -
// sum L_jk y_k), backward sweep z_i = L_ii^-T (y_i - sum L_ji^T z_j).  The
// factor is computed in FP64 and applied in FP32 (blocks packed per node in
// forward and backward neighbour lists, eight lanes per node, fixed tree
// reductions, so the result is deterministic): the preconditioner only
// steers the CG directions, whose residuals stay FP64.
#include "common.cuh"

#include <algorithm>
#include <cstdlib>
#include <vector>

namespace {

constexpr int IC_THREADS = 256;
constexpr int MAX_COLORS = 256;

__device__ __forceinline__ uint32_t jp_hash(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// One Jones-Plassmann round: an uncoloured node whose priority (its degree,
// then the hash of its index within its system, then that index) is the
// largest among its uncoloured neighbours takes the smallest colour none of
// its coloured neighbours has.  Degree first (largest-degree-first) needs
// fewer colours than the hash alone (tet10: 15 against 18), so the sweeps
// make fewer launches.  Priorities relative to the system's first node make the
// colouring of a system the same alone and inside a batch.  Reads cin,
// writes cout (a copy of cin plus this round's colours); counts the nodes
// left uncoloured.
__global__ void k_jp_round(const int64_t *__restrict__ nptr, const int32_t *__restrict__ nadj, int64_t non,
                           const int32_t *__restrict__ node_seg, const int64_t *__restrict__ seg_nbeg,
                           const int16_t *__restrict__ cin, int16_t *__restrict__ cout, int *remaining,
                           unsigned *status) {
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  for (int64_t B = (int64_t)blockIdx.x * wpb + (threadIdx.x >> 5); B < non; B += (int64_t)gridDim.x * wpb) {
    const int16_t cb = cin[B];
    if (cb >= 0) {
      if (lane == 0) cout[B] = cb;
      continue;
    }
    const int64_t base = seg_nbeg[node_seg[B]];
    const uint32_t lb = (uint32_t)(B - base), hb = jp_hash(lb);
    const int64_t c0 = nptr[B];
    const int deg = (int)(nptr[B + 1] - c0);
    bool beaten = false;
    uint32_t used[MAX_COLORS / 32];
#pragma unroll
    for (int w = 0; w < MAX_COLORS / 32; ++w) used[w] = 0u;
    for (int t = lane; t < deg; t += 32) {
      const int32_t A = nadj[c0 + t];
      if (A == B) continue;
      const int16_t ca = cin[A];
      if (ca >= 0) {
        used[ca >> 5] |= 1u << (ca & 31);
      } else {
        const uint32_t la = (uint32_t)(A - base), ha = jp_hash(la);  // A is in B's system
        const int dega = (int)(nptr[A + 1] - nptr[A]);
        if (dega > deg || (dega == deg && (ha > hb || (ha == hb && la > lb)))) beaten = true;
      }
    }
    beaten = __any_sync(0xffffffffu, beaten);
    if (beaten) {
      if (lane == 0) {
        cout[B] = -1;
        atomicAdd(remaining, 1);
      }
      continue;
    }
#pragma unroll
    for (int w = 0; w < MAX_COLORS / 32; ++w)
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) used[w] |= __shfl_xor_sync(0xffffffffu, used[w], off);
    if (lane == 0) {
      int c = -1;
      for (int w = 0; w < MAX_COLORS / 32 && c < 0; ++w)
        if (~used[w]) c = w * 32 + __ffs(~used[w]) - 1;
      if (c < 0) {
        atomicOr(status, ST_CAPACITY);
        c = MAX_COLORS - 1;
      }
      cout[B] = (int16_t)c;
    }
  }
}

__device__ __forceinline__ int bsearch_row(const int32_t *__restrict__ rows, int deg, int32_t key) {
  int lo = 0, hi = deg - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (rows[mid] < key) lo = mid + 1; else hi = mid;
  }
  return (deg > 0 && rows[lo] == key) ? lo : -1;
}

// A' entry (row DoF (jr), column DoF (ic)) from the structural values: the
// column (i, cc) of node i holds the row node j at position t of i's list.
template <int P>
__device__ __forceinline__ double a_prime(const double *__restrict__ nz, int64_t ci0, int degi, int ti, int r,
                                          int cc, int64_t j, int64_t i, const uint8_t *__restrict__ fixed) {
  const bool fj = fixed[P * j + r], fi = fixed[P * i + cc];
  if (fj || fi) return (j == i && r == cc) ? 1.0 : 0.0;
  return nz[(size_t)P * P * ci0 + (size_t)cc * P * degi + (size_t)P * ti + r];
}

// The factorisation's arithmetic in FT (FP64, or FP32 for the FP32 factor):
// correctly rounded IEEE operations, no contraction.
__device__ __forceinline__ double xfma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float xfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float xsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double xsqrt(double a) { return __dsqrt_rn(a); }
__device__ __forceinline__ float xsqrt(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double xrcp(double a) { return __drcp_rn(a); }
__device__ __forceinline__ float xrcp(float a) { return __frcp_rn(a); }

// Factorisation of the nodes of one colour, a warp per node j.  The blocks
// L_ji of row j are made in colour order of i (L_ji needs the L_jk of
// colours before i's), a group of up to IcFac<P>::SLOTS neighbours i of one
// colour at a time:
//   1. all lanes go over j's list: the common neighbours k of j and i of an
//      earlier colour than i (and j's place in i's list) are found by binary
//      search in i's list and kept, in j's list order, in shared memory;
//   2. lane (slot, a, b) sums entry (a, b) of S = sum_k L_jk L_ik^T over
//      them (the FMA order of a lane doing all P*P entries), forms
//      A'_ji - S and, with the other lanes of its row a, entry (a, b) of
//      (A'_ji - S) L_ii^-T.
// Every lane of a slot takes the same path, so the FP64 instructions run
// with P*P lanes per pair (the GB300's FP64 pipe is spent per warp
// instruction, however few lanes take part).
template <int P>
struct IcFac {
  static constexpr int PP = P * P;
  static constexpr int SLOTS = 32 / PP < 8 ? 32 / PP : 8;  // pairs per group
};

template <int P, class FT>
__global__ void __launch_bounds__(IC_THREADS)
k_ic0_factor(const int32_t *__restrict__ nodes, const int64_t *__restrict__ fptr, const int32_t *__restrict__ fk,
             const int32_t *__restrict__ fsrc, const int32_t *__restrict__ fcol, int count, int max_deg,
             const int64_t *__restrict__ nptr, const int32_t *__restrict__ nadj,
             const int32_t *__restrict__ diagpos, const int16_t *__restrict__ color, const double *__restrict__ nz,
             const uint8_t *__restrict__ fixed, double shift, FT *__restrict__ Lrow,
             FT *__restrict__ Lcol, FT *__restrict__ Ldinv, int *fail) {
  constexpr int PP = P * P, NS = IcFac<P>::SLOTS;
  extern __shared__ int16_t ic_fac_smem[];  // per warp: NS lists of max_deg (u, v) pairs
  __shared__ int s_nm[IC_THREADS / 32][NS], s_tj[IC_THREADS / 32][NS];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  int16_t *mu = ic_fac_smem + (size_t)wib * NS * max_deg * 2, *mv = mu + (size_t)NS * max_deg;
  const int slot = lane / PP, e = lane % PP, ea = e / P, eb = e % P;
  for (int w = blockIdx.x * wpb + wib; w < count; w += gridDim.x * wpb) {
    const int64_t j = nodes[w];
    const int64_t c0 = nptr[j];
    const int deg = (int)(nptr[j + 1] - c0);
    const int32_t *rj = nadj + c0;
    const int cj = color[j];
    const int64_t pe = fptr[w + 1];
    for (int64_t p = fptr[w]; p < pe;) {
      const int cp = color[fk[fcol[p]]];
      int n = 1;
      while (n < NS && p + n < pe && color[fk[fcol[p + n]]] == cp) ++n;
      // 1. common neighbours of an earlier colour, in j's list order
      for (int sl = 0; sl < n; ++sl) {
        const int64_t i = fk[fcol[p + sl]];
        const int64_t ci0 = nptr[i];
        const int degi = (int)(nptr[i + 1] - ci0);
        const int32_t *ri = nadj + ci0;
        int cnt = 0, tj = -1;
        for (int ub = 0; ub < deg; ub += 32) {
          const int u = ub + lane;
          int v = -1;
          bool self = false;
          if (u < deg) {
            const int32_t k = rj[u];
            self = k == (int32_t)j;
            if (self || color[k] < cp) v = bsearch_row(ri, degi, k);
          }
          const bool hit = v >= 0 && !self;
          const unsigned bh = __ballot_sync(0xffffffffu, hit);
          if (hit) {
            const int at = cnt + __popc(bh & ((1u << lane) - 1u));
            mu[sl * max_deg + at] = (int16_t)u;
            mv[sl * max_deg + at] = (int16_t)v;
          }
          cnt += __popc(bh);
          const unsigned bj = __ballot_sync(0xffffffffu, self && v >= 0);
          if (bj) tj = __shfl_sync(0xffffffffu, v, __ffs(bj) - 1);
        }
        if (lane == 0) {
          s_nm[wib][sl] = cnt;
          s_tj[wib][sl] = tj;
        }
      }
      __syncwarp();
      // 2. entry (ea, eb) of pair `slot`
      const bool act = slot < n;
      int64_t i = 0, ci0 = 0;
      int degi = 0, tj = -1, t = 0;
      FT S = 0;
      if (act) {
        const int32_t q = fcol[p + slot];
        i = fk[q];
        t = (int)(fsrc[q] - c0);
        ci0 = nptr[i];
        degi = (int)(nptr[i + 1] - ci0);
        tj = s_tj[wib][slot];
        const int nm = s_nm[wib][slot];
        for (int h = 0; h < nm; ++h) {
          const FT *Ljk = Lrow + (size_t)(c0 + mu[slot * max_deg + h]) * PP + ea * P;
          const FT *Lik = Lrow + (size_t)(ci0 + mv[slot * max_deg + h]) * PP + eb * P;
#pragma unroll
          for (int m = 0; m < P; ++m) S = xfma(Ljk[m], Lik[m], S);
        }
      }
      const FT Bm = act && tj >= 0 ? xsub((FT)a_prime<P>(nz, ci0, degi, tj, ea, eb, j, i, fixed), S) : (FT)0;
      FT X = 0;
#pragma unroll
      for (int m = 0; m < P; ++m) {
        const FT bm = __shfl_sync(0xffffffffu, Bm, (slot * PP + ea * P + m) & 31);  // entry (ea, m)
        if (act) X = xfma(bm, Ldinv[(size_t)i * PP + eb * P + m], X);
      }
      if (act) {
        if (tj < 0) {  // the node pattern is symmetric; a miss means corrupt input
          if (e == 0) atomicOr((unsigned *)fail, 2u);
        } else {
          Lrow[(size_t)(c0 + t) * PP + e] = X;
          Lcol[(size_t)(ci0 + tj) * PP + e] = X;
        }
      }
      __syncwarp();
      p += n;
    }
    // diagonal block
    FT D[P][P];
#pragma unroll
    for (int a = 0; a < P; ++a)
#pragma unroll
      for (int b = 0; b < P; ++b) D[a][b] = 0;
    for (int t = lane; t < deg; t += 32) {
      const int32_t k = rj[t];
      if (color[k] >= cj) continue;
      const FT *Ljk = Lrow + (size_t)(c0 + t) * PP;
#pragma unroll
      for (int a = 0; a < P; ++a)
#pragma unroll
        for (int b = 0; b < P; ++b)
#pragma unroll
          for (int m = 0; m < P; ++m) D[a][b] = xfma(Ljk[a * P + m], Ljk[b * P + m], D[a][b]);
    }
#pragma unroll
    for (int a = 0; a < P; ++a)
#pragma unroll
      for (int b = 0; b < P; ++b)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) D[a][b] = xadd(D[a][b], __shfl_xor_sync(0xffffffffu, D[a][b], off));
    if (lane == 0) {
      const int dp = diagpos[j];
      FT Aj[P][P];
#pragma unroll
      for (int a = 0; a < P; ++a)
#pragma unroll
        for (int b = 0; b < P; ++b) {
          FT v = (FT)(dp >= 0 ? a_prime<P>(nz, c0, deg, dp, a, b, j, j, fixed) : (a == b ? 1.0 : 0.0));
          if (a == b) v = xmul(v, (FT)(1.0 + shift));
          Aj[a][b] = xsub(v, D[a][b]);
        }
      // Cholesky Aj = L L^T, then L^-1 (both lower)
      FT L[P][P], Li[P][P];
      bool ok = true;
#pragma unroll
      for (int a = 0; a < P; ++a)
#pragma unroll
        for (int b = 0; b < P; ++b) { L[a][b] = 0; Li[a][b] = 0; }
#pragma unroll
      for (int b = 0; b < P; ++b) {
        FT d = Aj[b][b];
#pragma unroll
        for (int m = 0; m < b; ++m) d = xfma(-L[b][m], L[b][m], d);
        if (!(d > (FT)0)) { ok = false; d = 1; }
        const FT lb = xsqrt(d);
        L[b][b] = lb;
        const FT rl = xrcp(lb);
#pragma unroll
        for (int a = b + 1; a < P; ++a) {
          FT v = Aj[a][b];
#pragma unroll
          for (int m = 0; m < b; ++m) v = xfma(-L[a][m], L[b][m], v);
          L[a][b] = xmul(v, rl);
        }
      }
#pragma unroll
      for (int b = 0; b < P; ++b) {
        Li[b][b] = xrcp(L[b][b]);
#pragma unroll
        for (int a = b + 1; a < P; ++a) {
          FT v = 0;
#pragma unroll
          for (int m = b; m < a; ++m) v = xfma(L[a][m], Li[m][b], v);
          Li[a][b] = xmul(-v, xrcp(L[a][a]));
        }
      }
      if (!ok) atomicOr((unsigned *)fail, 1u);
      FT *ld = Ldinv + (size_t)j * PP;
#pragma unroll
      for (int a = 0; a < P; ++a)
#pragma unroll
        for (int b = 0; b < P; ++b) ld[a * P + b] = Li[a][b];
    }
    __syncwarp();
  }
}

// Earlier / later neighbour counts of every node, in colour order (thread
// per position of the colour-sorted node list).
__global__ void k_ic0_count(const int32_t *__restrict__ nodes, const int64_t *__restrict__ nptr,
                            const int32_t *__restrict__ nadj, const int16_t *__restrict__ color, int64_t non,
                            int64_t *__restrict__ fcnt, int64_t *__restrict__ bcnt) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < non; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = nodes[t];
    const int16_t cj = color[j];
    int64_t f = 0, b = 0;
    for (int64_t q = nptr[j]; q < nptr[j + 1]; ++q) {
      const int16_t ck = color[nadj[q]];
      f += ck < cj;
      b += ck > cj;
    }
    fcnt[t] = f;
    bcnt[t] = b;
  }
}

// Packed neighbour lists in colour order: for the node at position t of the
// colour-sorted list, its earlier neighbours (forward solve) and later
// neighbours (backward solve), each with the position of the block in the
// node's adjacency list.  One colour's lists are then one contiguous run.
// fcol orders each node's forward list by the neighbours' colour (then list
// order): the factorisation takes the blocks of row t in that order.
__global__ void k_ic0_lists(const int32_t *__restrict__ nodes, const int64_t *__restrict__ nptr,
                            const int32_t *__restrict__ nadj, const int16_t *__restrict__ color, int64_t non,
                            const int64_t *__restrict__ fptr, const int64_t *__restrict__ bptr,
                            int32_t *__restrict__ fk, int32_t *__restrict__ fsrc, int32_t *__restrict__ bk,
                            int32_t *__restrict__ bsrc, int32_t *__restrict__ fcol) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < non; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = nodes[t];
    const int16_t cj = color[j];
    int64_t f = fptr[t], b = bptr[t];
    for (int64_t q = nptr[j]; q < nptr[j + 1]; ++q) {
      const int32_t k = nadj[q];
      const int16_t ck = color[k];
      if (ck < cj) {
        fk[f] = k;
        fsrc[f++] = (int32_t)q;
      } else if (ck > cj) {
        bk[b] = k;
        bsrc[b++] = (int32_t)q;
      }
    }
    int64_t o = fptr[t];
    for (int16_t cc = 0; cc < cj; ++cc)
      for (int64_t u = fptr[t]; u < f; ++u)
        if (color[fk[u]] == cc) fcol[o++] = (int32_t)u;
  }
}

// out[t] = v[nodes[t]]: a per-node int32 array in colour order.
__global__ void k_ic0_by_color(const int32_t *__restrict__ nodes, const int32_t *__restrict__ v, int64_t non,
                               int32_t *__restrict__ out) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < non; t += (int64_t)gridDim.x * blockDim.x)
    out[t] = v[nodes[t]];
}

// FP32 copies of the factor in packed order (blocks of L with the forward
// and backward lists, and L_jj^-1).
template <class FT>
__global__ void k_ic0_pack(const FT *__restrict__ src, const int32_t *__restrict__ idx, int64_t count, int pp,
                           float *__restrict__ dst) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < count * pp;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = t / pp;
    const int e = (int)(t - q * pp);
    dst[t] = (float)src[(idx ? (int64_t)idx[q] : q) * pp + e];
  }
}

}  // namespace

// ---------------------------------------------------------------- host side
struct IcColoring {
  std::vector<int64_t> seg_nodes;  // first node of every system the colouring was made for (+ end)
  int ncolors = 0;
  std::vector<int64_t> ptr;      // colour c: nodes [ptr[c], ptr[c+1]) of d_nodes
  int16_t *d_color = nullptr;    // non
  int32_t *d_nodes = nullptr;    // non, sorted by (colour, decreasing degree, index)
  // packed neighbour lists: earlier (f) and later (b) neighbours of every
  // node, indexed by the node's position in d_nodes (colour order)
  int64_t *d_fptr = nullptr, *d_bptr = nullptr;     // non + 1
  int32_t *d_fk = nullptr, *d_fsrc = nullptr;       // neighbour, position in the adjacency
  int32_t *d_bk = nullptr, *d_bsrc = nullptr;
  int32_t *d_fcol = nullptr;                        // forward-list positions by colour (factorisation order)
  int64_t nf = 0, nb = 0;
};

void ic0_coloring_free(llf_ctx *ctx, llf_pattern *pat) {
  if (!pat->ic_coloring) return;
  IcColoring *cl = (IcColoring *)pat->ic_coloring;
  dfree(ctx, cl->d_color);
  dfree(ctx, cl->d_nodes);
  dfree(ctx, cl->d_fptr); dfree(ctx, cl->d_bptr);
  dfree(ctx, cl->d_fk); dfree(ctx, cl->d_fsrc);
  dfree(ctx, cl->d_bk); dfree(ctx, cl->d_bsrc);
  dfree(ctx, cl->d_fcol);
  delete cl;
  pat->ic_coloring = nullptr;
}

static int ic0_coloring(llf_ctx *ctx, llf_pattern *pat, const std::vector<int64_t> &seg_nodes,
                        const int32_t *d_node_seg, IcColoring **out) {
  if (pat->ic_coloring) {
    if (((IcColoring *)pat->ic_coloring)->seg_nodes == seg_nodes) {
      *out = (IcColoring *)pat->ic_coloring;
      return LLF_OK;
    }
    ic0_coloring_free(ctx, pat);
  }
  const int64_t non = pat->mesh->non;
  cudaStream_t s = ctx->stream;
  int16_t *ca = nullptr, *cb = nullptr;
  int *d_rem = nullptr;
  int64_t *d_nbeg = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &ca, non));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &cb, non));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &d_rem, 1));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &d_nbeg, seg_nodes.size()));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d_nbeg, seg_nodes.data(), sizeof(int64_t) * seg_nodes.size(),
                                    cudaMemcpyHostToDevice, s));
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(ca, 0xff, sizeof(int16_t) * non, s));
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((non + 7) / 8, (int64_t)ctx->num_sms * 16));
  int remaining = 1, rounds = 0;
  while (remaining > 0) {
    LLF_CUDA_TRY(ctx, cudaMemsetAsync(d_rem, 0, sizeof(int), s));
    {
      KernelScope ks(ctx, "k_jp_round");
      k_jp_round<<<grid, IC_THREADS, 0, s>>>(pat->d_nptr, pat->d_nadj, non, d_node_seg, d_nbeg, ca, cb, d_rem,
                                             ctx->d_status);
    }
    LLF_CUDA_TRY(ctx, cudaGetLastError());
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(&remaining, d_rem, sizeof(int), cudaMemcpyDeviceToHost, s));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    std::swap(ca, cb);
    if (++rounds > 100000) {
      remaining = -1;
      break;
    }
  }
  dfree(ctx, cb);
  dfree(ctx, d_rem);
  dfree(ctx, d_nbeg);
  int rc = llf_check_status(ctx, "IC(0) colouring");
  if (rc == LLF_OK && remaining < 0) rc = llf_fail(ctx, LLF_ERR_LIMIT, "IC(0) colouring did not finish");
  if (rc != LLF_OK) {
    dfree(ctx, ca);
    return rc == LLF_ERR_LIMIT ? rc : llf_fail(ctx, LLF_ERR_LIMIT, "IC(0): more than 256 colours needed");
  }
  std::vector<int16_t> h(non);
  std::vector<int64_t> hptr(non + 1);
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(h.data(), ca, sizeof(int16_t) * non, cudaMemcpyDeviceToHost, s));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(hptr.data(), pat->d_nptr, sizeof(int64_t) * (non + 1), cudaMemcpyDeviceToHost, s));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  IcColoring *cl = new IcColoring;
  cl->seg_nodes = seg_nodes;
  for (int64_t i = 0; i < non; ++i) cl->ncolors = std::max(cl->ncolors, (int)h[i] + 1);
  cl->ptr.assign(cl->ncolors + 1, 0);
  for (int64_t i = 0; i < non; ++i) cl->ptr[h[i] + 1]++;
  for (int c = 0; c < cl->ncolors; ++c) cl->ptr[c + 1] += cl->ptr[c];
  // within a colour, nodes by decreasing degree (then index): the rows that
  // one warp of a sweep serves have lists of similar length
  int64_t maxdeg = 0;
  for (int64_t i = 0; i < non; ++i) maxdeg = std::max(maxdeg, hptr[i + 1] - hptr[i]);
  std::vector<int64_t> dcnt(maxdeg + 2, 0);
  for (int64_t i = 0; i < non; ++i) dcnt[maxdeg - (hptr[i + 1] - hptr[i]) + 1]++;
  for (int64_t d = 0; d <= maxdeg; ++d) dcnt[d + 1] += dcnt[d];
  std::vector<int32_t> bydeg(non), nodes(non);
  for (int64_t i = 0; i < non; ++i) bydeg[dcnt[maxdeg - (hptr[i + 1] - hptr[i])]++] = (int32_t)i;
  std::vector<int64_t> fill(cl->ptr.begin(), cl->ptr.end() - 1);
  for (int64_t i : bydeg) nodes[fill[h[i]]++] = (int32_t)i;
  cl->d_color = ca;
  cudaError_t e = dalloc(ctx, &cl->d_nodes, non);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(cl->d_nodes, nodes.data(), sizeof(int32_t) * non, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    dfree(ctx, cl->d_color);
    dfree(ctx, cl->d_nodes);
    delete cl;
    return llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
  }
  pat->ic_coloring = cl;
  // packed forward / backward neighbour lists
  if (pat->nnzb >= (int64_t)1 << 31) return llf_fail(ctx, LLF_ERR_LIMIT, "IC(0): more than 2^31 node blocks");
  int64_t *fcnt = nullptr, *bcnt = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &fcnt, non + 1));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &bcnt, non + 1));
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(fcnt + non, 0, sizeof(int64_t), s));
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(bcnt + non, 0, sizeof(int64_t), s));
  const unsigned gt = (unsigned)std::max<int64_t>(1, std::min<int64_t>((non + 127) / 128, (int64_t)ctx->num_sms * 16));
  k_ic0_count<<<gt, 128, 0, s>>>(cl->d_nodes, pat->d_nptr, pat->d_nadj, cl->d_color, non, fcnt, bcnt);
  LLF_CUDA_TRY(ctx, dalloc(ctx, &cl->d_fptr, non + 1));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &cl->d_bptr, non + 1));
  LLF_CUDA_TRY(ctx, exclusive_scan_i64(ctx, fcnt, cl->d_fptr, non + 1, &cl->nf));
  LLF_CUDA_TRY(ctx, exclusive_scan_i64(ctx, bcnt, cl->d_bptr, non + 1, &cl->nb));
  dfree(ctx, fcnt);
  dfree(ctx, bcnt);
  LLF_CUDA_TRY(ctx, dalloc(ctx, &cl->d_fk, cl->nf));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &cl->d_fsrc, cl->nf));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &cl->d_bk, cl->nb));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &cl->d_bsrc, cl->nb));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &cl->d_fcol, cl->nf));
  k_ic0_lists<<<gt, 128, 0, s>>>(cl->d_nodes, pat->d_nptr, pat->d_nadj, cl->d_color, non, cl->d_fptr, cl->d_bptr,
                                 cl->d_fk, cl->d_fsrc, cl->d_bk, cl->d_bsrc, cl->d_fcol);
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  *out = cl;
  return LLF_OK;
}

template <int P, class FT>
static int ic0_factor_tt(llf_ctx *ctx, const llf_matrix *m, const uint8_t *d_fixed,
                        const std::vector<int64_t> &seg_nodes, const int32_t *d_node_seg, Ic0Factor *f) {
  const llf_pattern *pat = m->pat;
  const int64_t non = pat->mesh->non;
  cudaStream_t s = ctx->stream;
  IcColoring *cl = nullptr;
  int rc = ic0_coloring(ctx, (llf_pattern *)pat, seg_nodes, d_node_seg, &cl);
  if (rc != LLF_OK) return rc;
  f->ncolors = cl->ncolors;
  f->color_ptr = cl->ptr;
  f->d_color = cl->d_color;
  f->d_nodes = cl->d_nodes;
  FT *Lrow = nullptr, *Lcol = nullptr, *Ldinv = nullptr;
  f->fp32 = sizeof(FT) == sizeof(float);
  LLF_CUDA_TRY(ctx, dalloc(ctx, &Lrow, (size_t)pat->nnzb * P * P));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &Lcol, (size_t)pat->nnzb * P * P));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &Ldinv, (size_t)non * P * P));
  f->Lrow = Lrow;
  f->Lcol = Lcol;
  f->Ldinv = Ldinv;
  int *d_fail = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &d_fail, 1));
  // the factorisation's per-warp match lists: NS x max_deg (u, v) pairs of int16
  const int md = std::max(1, pat->max_deg);
  if (md > 32767) return llf_fail(ctx, LLF_ERR_LIMIT, "IC(0): a node has more than 32767 neighbours");
  const size_t per_warp = (size_t)IcFac<P>::SLOTS * md * 2 * sizeof(int16_t);
  const int fwpb = (int)std::min<size_t>(IC_THREADS / 32, (48 * 1024) / per_warp);
  if (fwpb < 1) return llf_fail(ctx, LLF_ERR_LIMIT, "IC(0): node degree too large for the factorisation");
  const size_t fsmem = per_warp * fwpb;
  const double shifts[] = {0.0, 1e-4, 1e-3, 1e-2, 1e-1, 1.0};
  int fail = 1;
  for (double shift : shifts) {
    LLF_CUDA_TRY(ctx, cudaMemsetAsync(d_fail, 0, sizeof(int), s));
    LLF_CUDA_TRY(ctx, cudaMemsetAsync(Lrow, 0, sizeof(FT) * pat->nnzb * P * P, s));
    LLF_CUDA_TRY(ctx, cudaMemsetAsync(Lcol, 0, sizeof(FT) * pat->nnzb * P * P, s));
    for (int c = 0; c < cl->ncolors; ++c) {
      const int count = (int)(cl->ptr[c + 1] - cl->ptr[c]);
      if (count == 0) continue;
      const unsigned grid = (unsigned)std::max<int64_t>(
          1, std::min<int64_t>((count + fwpb - 1) / fwpb, (int64_t)ctx->num_sms * 32));
      KernelScope ks(ctx, "k_ic0_factor");
      k_ic0_factor<P, FT><<<grid, 32 * fwpb, fsmem, s>>>(cl->d_nodes + cl->ptr[c], cl->d_fptr + cl->ptr[c], cl->d_fk,
                                                     cl->d_fsrc, cl->d_fcol, count, md, pat->d_nptr, pat->d_nadj,
                                                     pat->d_diagpos, cl->d_color, m->d_nz, d_fixed, shift, Lrow,
                                                     Lcol, Ldinv, d_fail);
    }
    LLF_CUDA_TRY(ctx, cudaGetLastError());
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(&fail, d_fail, sizeof(int), cudaMemcpyDeviceToHost, s));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    f->shift = shift;
    if (!fail || (fail & 2)) break;
  }
  dfree(ctx, d_fail);
  if (fail & 2) return llf_fail(ctx, LLF_ERR_STATE, "IC(0): the node pattern is not symmetric");
  if (fail) return llf_fail(ctx, LLF_ERR_NUMERIC, "IC(0): non-positive pivot even with a diagonal shift of 1");
  // FP32 copies in packed order for the triangular solves; the FP64 factor goes
  f->fptr = cl->d_fptr; f->fk = cl->d_fk;
  f->bptr = cl->d_bptr; f->bk = cl->d_bk;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &f->Lf, (size_t)cl->nf * P * P));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &f->Lb, (size_t)cl->nb * P * P));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &f->Ldf, (size_t)non * P * P));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &f->segc, non));
  const unsigned gp = (unsigned)(ctx->num_sms * 16);
  {
    KernelScope ks(ctx, "k_ic0_pack");
    k_ic0_pack<FT><<<gp, 256, 0, s>>>(Lrow, cl->d_fsrc, cl->nf, P * P, f->Lf);
    k_ic0_pack<FT><<<gp, 256, 0, s>>>(Lcol, cl->d_bsrc, cl->nb, P * P, f->Lb);
    k_ic0_pack<FT><<<gp, 256, 0, s>>>(Ldinv, cl->d_nodes, non, P * P, f->Ldf);
    k_ic0_by_color<<<gp, 256, 0, s>>>(cl->d_nodes, d_node_seg, non, f->segc);
  }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  dfree(ctx, Lrow);
  dfree(ctx, Lcol);
  dfree(ctx, Ldinv);
  f->Lrow = f->Lcol = f->Ldinv = nullptr;
  return LLF_OK;
}

// The factor's arithmetic: FP32 (FP64 when LLF_IC0_FP32=0).  The factor is
// applied in FP32 either way; the FP32 factorisation runs on the FP32 pipe
// instead of GB300's narrow FP64 one (the 512-instance batch: the same CG
// iteration counts, 22.5 -> 22.8 solves/s).
static bool ic0_fp32_factor() {
  const char *e = getenv("LLF_IC0_FP32");
  return !(e && e[0] == '0');
}

int ic0_factor(llf_ctx *ctx, const llf_matrix *m, const uint8_t *d_fixed, const std::vector<int64_t> &seg_nodes,
               const int32_t *d_node_seg, Ic0Factor *f) {
  {
    const int rc = matrix_ensure_nz(ctx, m);
    if (rc != LLF_OK) return rc;
  }
  const bool f32 = ic0_fp32_factor();
  switch (m->pat->pdim * 2 + (f32 ? 1 : 0)) {
    case 2: return ic0_factor_tt<1, double>(ctx, m, d_fixed, seg_nodes, d_node_seg, f);
    case 3: return ic0_factor_tt<1, float>(ctx, m, d_fixed, seg_nodes, d_node_seg, f);
    case 4: return ic0_factor_tt<2, double>(ctx, m, d_fixed, seg_nodes, d_node_seg, f);
    case 5: return ic0_factor_tt<2, float>(ctx, m, d_fixed, seg_nodes, d_node_seg, f);
    case 6: return ic0_factor_tt<3, double>(ctx, m, d_fixed, seg_nodes, d_node_seg, f);
    case 7: return ic0_factor_tt<3, float>(ctx, m, d_fixed, seg_nodes, d_node_seg, f);
  }
  return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "pdim must be 1, 2 or 3");
}

void ic0_release(llf_ctx *ctx, Ic0Factor *f) {
  dfree(ctx, f->Lrow);
  dfree(ctx, f->Lcol);
  dfree(ctx, f->Ldinv);
  dfree(ctx, f->Lf);
  dfree(ctx, f->Lb);
  dfree(ctx, f->Ldf);
  dfree(ctx, f->segc);
}
