// Element-operator assembly into the reference's CSC layout.
//
// Pipeline (one call of llf_assemble_*):
//   geometry      k_affine_geometry, once per mesh geometry (kept on the
//                 device mesh): which elements are affine images of the
//                 reference element (and which of those are axis-aligned
//                 bricks), with their J^-1 and det;
//   k_elem_affine meshes whose elements are all affine: one CTA per element
//                 at a time (persistent), the node-pair blocks formed from
//                 the reference pair tables into a shared-memory image of the
//                 element matrix, which one bulk store writes out;
//   k_elem_fp64   other meshes: one CTA per element at a time, element node
//                 coordinates gathered into shared memory, the reference
//                 shape gradients staged in shared memory for the CTA's
//                 lifetime (read from global memory for elements whose tables
//                 do not fit), Jacobian / inverse / physical gradients per
//                 integration point (the affine form for affine elements),
//                 then the upper-triangle node-pair blocks, each written
//                 twice (block and mirror).  Both kernels leave the element
//                 matrix whole in the layout Kf[element][column node b][row
//                 node a][block];
//   k_colgather   one warp per column node B: walks the elements around B in
//                 ascending order; for each, the lanes read the element's
//                 column b = local(B) — one contiguous run of npe blocks — and
//                 add every block into a shared-memory accumulator of the
//                 column at the row position the pattern's element-to-column
//                 map gives.  Each entry is thus summed over its elements in
//                 element order, the order SparseArrays.sparse combines the
//                 reference's triplets (src/linear.jl:314-323).  The column is
//                 written out coalesced together with its non-zero count, or,
//                 when the pattern kept the stored layout of an earlier
//                 assembly of the same operator and form, compacted straight
//                 into it (dropzeros!, every column's count checked);
//   finalize      otherwise dropzeros! (src/linear.jl:324): scan of the
//                 counts, then compaction into 1-based Int64 SparseMatrixCSC
//                 arrays, whose column starts the pattern keeps.
// Every floating-point operation of the FP64 form is an explicit IEEE
// intrinsic (__dmul_rn, __dadd_rn, __fma_rn, __drcp_rn), so no contraction
// or reassociation can move the result away from the CPU oracle's.
#include "common.cuh"
#include "affine.cuh"

#include <algorithm>

namespace {

constexpr int ELEM_THREADS = 128;

struct ElemArgs {
  const double *xyz;
  const int32_t *conn;
  const int32_t *emat;
  int64_t nel;
  int npe, nip, npairs;
  const double *w, *N, *dN;  // device tables
  const double *c1, *c2;     // per-material coefficients
  double *Kf;                // nel * npe * colstride (full element matrices)
  int64_t colstride;         // doubles per element-matrix column (16-byte multiple)
  double *scratch;           // per-CTA global scratch for G, S (large elements)
  int64_t scratch_stride;    // doubles per CTA
  unsigned *status;
  // affine-element form: per-element flag and invJ/det (k_affine_geometry;
  // aflag null = none), and per upper-triangle node pair in pair order the
  // symmetric [0,NS) and antisymmetric [6,6+NA) parts of R_ab, and Mref_ab
  const uint8_t *aflag;
  const double *ageo, *Rp, *Mp;
  int cta_cap;               // host side: CTAs per SM at most (0: as many as fit)
  bool all_affine;           // host side: k_affine_geometry counted no non-affine element
};

__device__ __forceinline__ int pair_offset(int a, int npe) {
  return a * npe - (a * (a - 1)) / 2;
}
__device__ __forceinline__ void pair_decode(int pi, int npe, int &a, int &b) {
  int lo = 0, hi = npe - 1;
  while (lo < hi) {  // largest a with pair_offset(a) <= pi
    int mid = (lo + hi + 1) >> 1;
    if (pair_offset(mid, npe) <= pi) lo = mid; else hi = mid - 1;
  }
  a = lo;
  b = a + (pi - pair_offset(a, npe));
}

// Geometry at one point (contract of the oracle): returns det, fills inv
// (row-major invJ[i][j]).  dNq(a, j) is the reference gradient of node a.
template <int DIM, class Tab>
__device__ __forceinline__ double geom_point(const double *sX, Tab dNq, int npe, double *inv) {
  double J[3][3];
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      double acc = 0.0;
      for (int a = 0; a < npe; ++a) acc = __fma_rn(sX[a * DIM + i], dNq(a, j), acc);
      J[i][j] = acc;
    }
  return jac_inverse<DIM>(J, inv);
}

// Store block (a,b) (a <= b) of the element matrix and its mirror (b,a) in
// the column-major-by-node layout Kf[e][col node][row node][i*P+j].
template <int P, int BS>
__device__ __forceinline__ void store_pair(double *Ke, int64_t cs, int a, int b, const double *blk) {
  double *ab = Ke + (size_t)b * cs + (size_t)a * BS;  // rows of node a, columns of node b
#pragma unroll
  for (int k = 0; k < BS; ++k) ab[k] = blk[k];
  if (a != b) {
    double *ba = Ke + (size_t)a * cs + (size_t)b * BS;
    if (BS == 1) {
      ba[0] = blk[0];
    } else {
#pragma unroll
      for (int i = 0; i < P; ++i)
#pragma unroll
        for (int j = 0; j < P; ++j) ba[j * P + i] = blk[i * P + j];
    }
  }
}

// Node-pair blocks of an affine element (contract of the oracle): per pair
// the symmetric part S (NS values) and antisymmetric part A (NA values) of
// R_ab; elasticity Ksym = W S, Kanti = U A (a != b), heat (c1 trV) . S, mass
// (c1 det) Mref_ab.
// ALIGNED (axis-aligned elements, flag 2 of k_affine_geometry, whose
// coefficients affine_stage_aligned forms): elasticity through the
// collapsed Lame combination of the oracle's orc_element_aligned, 15 FP64
// operations per node pair in 3D instead of 51; heat leaves the mixed
// components, whose coefficients are exact zeros there, out of its fma
// chain (a left-out fma(+-0, s, acc) returns acc whenever acc is non-zero,
// so the value is the full chain's up to the sign of a zero result, and
// zeros are dropped from the stored CSC and add nothing to a non-zero sum).
// Rp, Mp: the pair tables in global memory (read through the read-only
// path) or, with TAB_SMEM, in shared memory.
template <bool TAB_SMEM>
__device__ __forceinline__ double ld_tab(const double *p) {
  if (TAB_SMEM) return *p;
  return __ldg(p);
}

template <int KIND, int DIM, int P, int BS, bool ALIGNED, bool TAB_SMEM = false>
__device__ __forceinline__ void affine_pairs(const ElemArgs &A, const double *sAff, double *Ke,
                                             const double *Rp, const double *Mp) {
  constexpr int NS = DIM == 3 ? 6 : 3, NA = DIM == 3 ? 3 : 1;
  const int npe = A.npe;
  if (KIND == KIND_MASS) {
    const double cm = sAff[AF_M];
    for (int pi = threadIdx.x; pi < A.npairs; pi += blockDim.x) {
      int a, b;
      pair_decode(pi, npe, a, b);
      double blk[BS];
      blk[0] = __dmul_rn(cm, ld_tab<TAB_SMEM>(Mp + pi));
      store_pair<P, BS>(Ke, A.colstride, a, b, blk);
    }
  } else if (KIND == KIND_HEAT) {
    double Q[NS];
#pragma unroll
    for (int n = 0; n < NS; ++n) Q[n] = (!ALIGNED || n < DIM) ? sAff[AF_Q + n] : 0.0;
    for (int pi = threadIdx.x; pi < A.npairs; pi += blockDim.x) {
      int a, b;
      pair_decode(pi, npe, a, b);
      const double *sp = Rp + (size_t)pi * 9;
      double acc = 0.0;
#pragma unroll
      for (int n = 0; n < (ALIGNED ? DIM : NS); ++n) acc = __fma_rn(Q[n], ld_tab<TAB_SMEM>(sp + n), acc);
      double blk[BS];
      blk[0] = acc;
      store_pair<P, BS>(Ke, A.colstride, a, b, blk);
    }
  } else if (ALIGNED) {
    // axis-aligned elasticity (contract of the oracle's orc_element_aligned):
    // g = sum beta_n S_n, K_ii = fma(alpha_i, S_i, g), h = b_m A_m,
    // K_ij = fma(a_m, S_m, h), K_ji = fma(a_m, S_m, -h); a == b: a_m S_m
    double al[DIM], be[DIM], am[NA], bm[NA];
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      al[i] = sAff[AF_W + i];
      be[i] = sAff[AF_W + DIM + i];
    }
#pragma unroll
    for (int m = 0; m < NA; ++m) {
      am[m] = sAff[AF_W + 2 * DIM + m];
      bm[m] = sAff[AF_W + 2 * DIM + NA + m];
    }
    for (int pi = threadIdx.x; pi < A.npairs; pi += blockDim.x) {
      int a, b;
      pair_decode(pi, npe, a, b);
      const double *sp = Rp + (size_t)pi * 9;
      double sv[NS], av[NA];
#pragma unroll
      for (int n = 0; n < NS; ++n) sv[n] = ld_tab<TAB_SMEM>(sp + n);
#pragma unroll
      for (int n = 0; n < NA; ++n) av[n] = ld_tab<TAB_SMEM>(sp + 6 + n);
      double g = __dmul_rn(be[0], sv[0]);
#pragma unroll
      for (int n = 1; n < DIM; ++n) g = __fma_rn(be[n], sv[n], g);
      double blk[BS];
#pragma unroll
      for (int i = 0; i < DIM; ++i) blk[i * DIM + i] = __fma_rn(al[i], sv[i], g);
#pragma unroll
      for (int m = 0; m < NA; ++m) {
        const int i = sym_k<DIM>(DIM + m), j = sym_l<DIM>(DIM + m);
        if (a != b) {
          const double h = __dmul_rn(bm[m], av[m]);
          blk[i * DIM + j] = __fma_rn(am[m], sv[DIM + m], h);
          blk[j * DIM + i] = __fma_rn(am[m], sv[DIM + m], -h);
        } else {
          const double v = __dmul_rn(am[m], sv[DIM + m]);
          blk[i * DIM + j] = v;
          blk[j * DIM + i] = v;
        }
      }
      store_pair<P, BS>(Ke, A.colstride, a, b, blk);
    }
  } else {
    double W[NS * NS], U[NA * NA];
#pragma unroll
    for (int t = 0; t < NS * NS; ++t) W[t] = sAff[AF_W + t];
#pragma unroll
    for (int t = 0; t < NA * NA; ++t) U[t] = sAff[AF_U + t];
    for (int pi = threadIdx.x; pi < A.npairs; pi += blockDim.x) {
      int a, b;
      pair_decode(pi, npe, a, b);
      const double *sp = Rp + (size_t)pi * 9;
      double sv[NS], av[NA];
#pragma unroll
      for (int n = 0; n < NS; ++n) sv[n] = ld_tab<TAB_SMEM>(sp + n);
#pragma unroll
      for (int n = 0; n < NA; ++n) av[n] = ld_tab<TAB_SMEM>(sp + 6 + n);
      double ks[NS];
#pragma unroll
      for (int m = 0; m < NS; ++m) {
        double acc = 0.0;
#pragma unroll
        for (int n = 0; n < NS; ++n) acc = __fma_rn(W[m * NS + n], sv[n], acc);
        ks[m] = acc;
      }
      double blk[BS];
#pragma unroll
      for (int i = 0; i < DIM; ++i) blk[i * DIM + i] = ks[i];
      if (a != b) {
#pragma unroll
        for (int m = 0; m < NA; ++m) {
          double acc = 0.0;
#pragma unroll
          for (int n = 0; n < NA; ++n) acc = __fma_rn(U[m * NA + n], av[n], acc);
          const int i = sym_k<DIM>(DIM + m), j = sym_l<DIM>(DIM + m);
          blk[i * DIM + j] = __dadd_rn(ks[DIM + m], acc);
          blk[j * DIM + i] = __dsub_rn(ks[DIM + m], acc);
        }
      } else {
#pragma unroll
        for (int m = 0; m < NA; ++m) {
          const int i = sym_k<DIM>(DIM + m), j = sym_l<DIM>(DIM + m);
          blk[i * DIM + j] = ks[DIM + m];
          blk[j * DIM + i] = ks[DIM + m];
        }
      }
      store_pair<P, BS>(Ke, A.colstride, a, b, blk);
    }
  }
}

// Shared-memory layout of k_elem_fp64 (doubles):
//   [SMEM] sdN [nip*npe*DIM] | sw [nip] | sN [nip*npe] (mass) |
//   sX [npe*DIM] | sWd [nip] | sInv [nip*9] | sAff [32] | [SMEM] G, S (each nip*npe*gsw)
// Without SMEM the tables are read from global memory (stride 3) and G, S
// live in a per-CTA global scratch slot (L2 resident).
template <int KIND, int DIM, bool SMEM>
__global__ void __launch_bounds__(ELEM_THREADS)
k_elem_fp64(ElemArgs A) {
  extern __shared__ double smem[];
  const int npe = A.npe, nip = A.nip;
  constexpr int gsw = (KIND == KIND_MASS) ? 1 : DIM;
  double *sdN = smem;
  double *sw = sdN + (SMEM ? (size_t)nip * npe * DIM : 0);
  double *sN = sw + (SMEM ? nip : 0);
  double *sX = sN + ((SMEM && KIND == KIND_MASS) ? (size_t)nip * npe : 0);
  double *sWd = sX + (size_t)npe * DIM;
  double *sInv = sWd + nip;
  double *sAff = sInv + (size_t)nip * 9;  // affine-form scratch (AF_* offsets)
  double *G = SMEM ? (sAff + AFF_DOUBLES) : (A.scratch + (size_t)blockIdx.x * A.scratch_stride);
  double *S = G + (size_t)nip * npe * gsw;
  // table accessors
  const int tstride = SMEM ? DIM : 3;
  const double *tdN = SMEM ? sdN : A.dN;
  const double *tw = SMEM ? sw : A.w;
  const double *tN = SMEM ? sN : A.N;

  if (SMEM) {
    for (int t = threadIdx.x; t < nip * npe * DIM; t += blockDim.x) {
      int j = t % DIM, qa = t / DIM;
      sdN[t] = A.dN[(size_t)qa * 3 + j];
    }
    for (int t = threadIdx.x; t < nip; t += blockDim.x) sw[t] = A.w[t];
    if (KIND == KIND_MASS)
      for (int t = threadIdx.x; t < nip * npe; t += blockDim.x) sN[t] = A.N[t];
    __syncthreads();
  }

  constexpr int BS = (KIND == KIND_ELASTIC) ? DIM * DIM : 1;
  constexpr int P = (KIND == KIND_ELASTIC) ? DIM : 1;
  for (int64_t e = blockIdx.x; e < A.nel; e += gridDim.x) {
    const int mat = A.emat ? A.emat[e] : 0;
    if (mat < 0) continue;  // uniform across the CTA
    const double c1 = A.c1[mat];
    const double c2 = (KIND == KIND_ELASTIC) ? A.c2[mat] : 0.0;
    double *Ke = A.Kf + (size_t)e * npe * A.colstride;
    if (A.aflag && A.aflag[e]) {  // uniform across the CTA
      const bool aligned = A.aflag[e] == 2;   // uniform across the CTA
      if (threadIdx.x < 32) {
        if (aligned)
          affine_stage_aligned<DIM>(A.ageo + (size_t)e * 10, c1, c2, sAff, A.status, threadIdx.x);
        else
          affine_stage<DIM>(A.ageo + (size_t)e * 10, c1, c2, sAff, A.status, threadIdx.x);
      }
      __syncthreads();
      if (aligned)
        affine_pairs<KIND, DIM, P, BS, true>(A, sAff, Ke, A.Rp, A.Mp);
      else
        affine_pairs<KIND, DIM, P, BS, false>(A, sAff, Ke, A.Rp, A.Mp);
    } else {
      for (int t = threadIdx.x; t < npe * DIM; t += blockDim.x) {
        int a = t / DIM, i = t % DIM;
        sX[t] = A.xyz[(size_t)A.conn[e * npe + a] * 3 + i];
      }
      __syncthreads();
      for (int q = threadIdx.x; q < nip; q += blockDim.x) {
        double inv[9];
        const double *dq = tdN + (size_t)q * npe * tstride;
        double det = geom_point<DIM>(sX, [&](int a, int j) { return dq[a * tstride + j]; }, npe, inv);
        if (!(det > 0.0)) atomicOr(A.status, ST_BAD_JACOBIAN);
        sWd[q] = __dmul_rn(det, tw[q]);
#pragma unroll
        for (int k = 0; k < 9; ++k) sInv[q * 9 + k] = inv[k];
      }
      __syncthreads();
      if (KIND == KIND_MASS) {
        for (int t = threadIdx.x; t < nip * npe; t += blockDim.x) S[t] = __dmul_rn(sWd[t / npe], tN[t]);
      } else {
        for (int t = threadIdx.x; t < nip * npe; t += blockDim.x) {
          const int q = t / npe;
          const double *inv = sInv + q * 9;
          const double *d = tdN + (size_t)t * tstride;
          const double wd = sWd[q];
#pragma unroll
          for (int i = 0; i < DIM; ++i) {
            double acc = 0.0;
#pragma unroll
            for (int j = 0; j < DIM; ++j) acc = __fma_rn(inv[3 * j + i], d[j], acc);
            G[(size_t)t * DIM + i] = acc;
            S[(size_t)t * DIM + i] = __dmul_rn(wd, acc);
          }
        }
      }
      __syncthreads();

      for (int pi = threadIdx.x; pi < A.npairs; pi += blockDim.x) {
        int a, b;
        pair_decode(pi, npe, a, b);
        double blk[BS];
        if (KIND == KIND_ELASTIC) {
          double O[DIM][DIM];
#pragma unroll
          for (int i = 0; i < DIM; ++i)
#pragma unroll
            for (int j = 0; j < DIM; ++j) O[i][j] = 0.0;
          if (a != b) {
            for (int q = 0; q < nip; ++q) {
              const double *sa = S + ((size_t)q * npe + a) * DIM;
              const double *gb = G + ((size_t)q * npe + b) * DIM;
              double s_[DIM], g_[DIM];
#pragma unroll
              for (int i = 0; i < DIM; ++i) { s_[i] = sa[i]; g_[i] = gb[i]; }
#pragma unroll
              for (int i = 0; i < DIM; ++i)
#pragma unroll
                for (int j = 0; j < DIM; ++j) O[i][j] = __fma_rn(s_[i], g_[j], O[i][j]);
            }
          } else {
            for (int q = 0; q < nip; ++q) {
              const double *sa = S + ((size_t)q * npe + a) * DIM;
              const double *ga = G + ((size_t)q * npe + a) * DIM;
              double s_[DIM], g_[DIM];
#pragma unroll
              for (int i = 0; i < DIM; ++i) { s_[i] = sa[i]; g_[i] = ga[i]; }
#pragma unroll
              for (int i = 0; i < DIM; ++i)
#pragma unroll
                for (int j = i; j < DIM; ++j) O[i][j] = __fma_rn(s_[i], g_[j], O[i][j]);
            }
#pragma unroll
            for (int i = 0; i < DIM; ++i)
#pragma unroll
              for (int j = 0; j < i; ++j) O[i][j] = O[j][i];
          }
          double tr = __dadd_rn(O[0][0], O[1 % DIM][1 % DIM]);
          if (DIM == 3) tr = __dadd_rn(tr, O[2 % DIM][2 % DIM]);
#pragma unroll
          for (int i = 0; i < DIM; ++i)
#pragma unroll
            for (int j = 0; j < DIM; ++j) {
              double t = __fma_rn(c2, O[j][i], __dmul_rn(c1, O[i][j]));
              if (i == j) t = __fma_rn(c2, tr, t);
              blk[i * DIM + j] = t;
            }
        } else if (KIND == KIND_HEAT) {
          double acc = 0.0;
          for (int q = 0; q < nip; ++q) {
            const double *sa = S + ((size_t)q * npe + a) * DIM;
            const double *gb = G + ((size_t)q * npe + b) * DIM;
#pragma unroll
            for (int i = 0; i < DIM; ++i) acc = __fma_rn(sa[i], gb[i], acc);
          }
          blk[0] = __dmul_rn(c1, acc);
        } else {  // mass
          double acc = 0.0;
          for (int q = 0; q < nip; ++q)
            acc = __fma_rn(S[(size_t)q * npe + a], tN[(size_t)q * npe + b], acc);
          blk[0] = __dmul_rn(c1, acc);
        }
        store_pair<P, BS>(Ke, A.colstride, a, b, blk);
      }

    }
    __syncthreads();
  }
}

// Affine-element kernel with staged stores, for meshes whose elements are
// all affine (k_affine_geometry counted no other): one CTA per element at a
// time (grid-stride, persistent).  The pair table (the parts of R_ab, or
// Mref_ab) is copied into shared memory once per CTA by a bulk copy
// (cp.async.bulk completing on an mbarrier; a bounded wait).  Each element
// matrix is built in a shared-memory image of its Kf run (the same layout,
// column padding included) and leaves with one bulk store (cp.async.bulk
// global <- shared), which drains while the CTA forms the next element's
// coefficients; the warp that forms them rotates from element to element.
// The arithmetic is affine_pairs', so Kf holds what k_elem_fp64 writes.
// Shared memory: image [npe * colstride] | table [tab_n, even] | sAff |
// mbarrier.
__device__ __forceinline__ uint32_t sh_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait on an mbarrier phase (2 s); false on timeout.
__device__ __forceinline__ bool bar_wait(uint64_t *bar, unsigned parity) {
  const uint64_t t0 = now_ns();
  for (;;) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(sh_addr(bar)), "r"(parity) : "memory");
    if (ok) return true;
    if (now_ns() - t0 > 2000000000ull) return false;
  }
}

constexpr int AFFK_MAX_THREADS = 256;

template <int KIND, int DIM>
__global__ void __launch_bounds__(AFFK_MAX_THREADS)
k_elem_affine(ElemArgs A, int tab_n) {
  extern __shared__ __align__(128) double smem_a[];
  constexpr int BS = (KIND == KIND_ELASTIC) ? DIM * DIM : 1;
  constexpr int P = (KIND == KIND_ELASTIC) ? DIM : 1;
  const int64_t kelems = (int64_t)A.npe * A.colstride;
  const unsigned ke_bytes = (unsigned)(kelems * 8);
  double *sKe = smem_a;
  double *sTab = sKe + kelems;
  double *sAff = sTab + ((tab_n + 1) & ~1);
  uint64_t *bar = reinterpret_cast<uint64_t *>(sAff + AFF_DOUBLES);
  const double *gTab = KIND == KIND_MASS ? A.Mp : A.Rp;
  const unsigned tab_bytes = (unsigned)tab_n * 8u;
  if ((tab_bytes & 15u) == 0 && ((uintptr_t)gTab & 15u) == 0) {
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sh_addr(bar)), "r"(1u) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sh_addr(bar)), "r"(tab_bytes)
                   : "memory");
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                   ::"r"(sh_addr(sTab)), "l"(gTab), "r"(tab_bytes), "r"(sh_addr(bar))
                   : "memory");
    }
    const bool ok = bar_wait(bar, 0);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) atomicOr(A.status, ST_TIMEOUT);
      return;
    }
  } else {
    for (int t = threadIdx.x; t < tab_n; t += blockDim.x) sTab[t] = gTab[t];
    __syncthreads();
  }
  const int nwarps = (int)(blockDim.x >> 5);
  unsigned iter = 0;
  for (int64_t e = blockIdx.x; e < A.nel; e += gridDim.x, ++iter) {
    const int mat = A.emat ? A.emat[e] : 0;
    if (mat < 0) continue;  // uniform across the CTA
    const double c1 = A.c1[mat];
    const double c2 = (KIND == KIND_ELASTIC) ? A.c2[mat] : 0.0;
    const bool aligned = A.aflag[e] == 2;
    if ((int)(threadIdx.x >> 5) == (int)((blockIdx.x + iter) % (unsigned)nwarps)) {
      const int lane = threadIdx.x & 31;
      if (aligned)
        affine_stage_aligned<DIM>(A.ageo + (size_t)e * 10, c1, c2, sAff, A.status, lane);
      else
        affine_stage<DIM>(A.ageo + (size_t)e * 10, c1, c2, sAff, A.status, lane);
    }
    // the previous element's store has read the image
    if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    __syncthreads();
    if (aligned)
      affine_pairs<KIND, DIM, P, BS, true, true>(A, sAff, sKe, sTab, sTab);
    else
      affine_pairs<KIND, DIM, P, BS, false, true>(A, sAff, sKe, sTab, sTab);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
      double *Ke = A.Kf + (size_t)e * kelems;
      asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(Ke), "r"(sh_addr(sKe)),
                   "r"(ke_bytes)
                   : "memory");
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    }
  }
  if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// Column-node gather.  T = double (FP64 form) or float (precision form);
// FP64 sums in element order in both.  Per warp: the column's row-node list
// (deg ints) and its accumulator (deg * P * P doubles) in shared memory.
// Exact FP32 -> FP64 widening on the integer pipe (sign, exponent rebias,
// mantissa shift; subnormals normalised by their leading-zero count; Inf and
// NaN keep their payload): the precision form's gather widens every element
// value, and GB300's FP64 pipe is kept for the additions.
__device__ __forceinline__ double widen(double x) { return x; }
__device__ __forceinline__ double widen(unsigned long long b) { return __longlong_as_double((long long)b); }
// The gather holds FP64 values it only moves as their bit patterns (64-bit
// integers), so that moving, selecting and storing them takes no FP64
// instruction: GB300 spends its FP64 pipe per warp instruction.
template <class T> struct GatherWord { using type = T; };
template <> struct GatherWord<double> { using type = unsigned long long; };
__device__ __forceinline__ unsigned long long value_bits(unsigned long long b) { return b; }
__device__ __forceinline__ unsigned long long value_bits(float f) {
  return (unsigned long long)__double_as_longlong(widen(f));
}
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  if (e - 1u < 254u) {  // normal: in 32-bit halves, exponent + (1023 - 127), mantissa << 29
    const unsigned hi = (u & 0x80000000u) | (((u & 0x7fffffffu) >> 3) + 0x38000000u);
    return __hiloint2double((int)hi, (int)(u << 29));
  }
  unsigned long long bits;
  if (e != 0u) {
    const unsigned long long ed = e == 0xffu ? 0x7ffull : (unsigned long long)(e + 896u);
    bits = (ed << 52) | ((unsigned long long)m << 29);
  } else if (m != 0u) {
    const int p = 31 - __clz((int)m);
    bits = ((unsigned long long)(p + 874) << 52) | (((unsigned long long)m << (52 - p)) & 0xfffffffffffffull);
  } else {
    bits = 0ull;
  }
  return __longlong_as_double((long long)(((unsigned long long)(u >> 31) << 63) | bits));
}

// The accumulator holds P planes, one per DoF column j of the column node,
// ps doubles apart; plane j holds the column's entries (row node t,
// component i) at P*t + i, the order they are written out in.
template <int P, bool BLOCKVAL, bool FIRST, class W>
__device__ __forceinline__ void add_block(double *acc, int t, const W *v, int ps) {
  double *dst = acc + (size_t)t * P;
  unsigned long long *dstb = reinterpret_cast<unsigned long long *>(dst);
#pragma unroll
  for (int i = 0; i < P; ++i)
#pragma unroll
    for (int j = 0; j < P; ++j) {
      if (FIRST) {  // the first block of the position: its bits
        dstb[j * ps + i] = BLOCKVAL ? value_bits(v[i * P + j]) : (i == j ? value_bits(v[0]) : 0ull);
      } else {
        const double x = BLOCKVAL ? widen(v[i * P + j]) : (i == j ? widen(v[0]) : 0.0);
        dst[j * ps + i] = __dadd_rn(dst[j * ps + i], x);
      }
    }
}

// Non-zero test on the bit pattern (integer pipe): every value but +-0.
__device__ __forceinline__ int nonzero_bits(double v) {
  return ((unsigned long long)__double_as_longlong(v) << 1) != 0ull;
}

// Column-node gather.  One warp per column node B: its accumulator
// (deg*P*P doubles) lives in shared memory, starting at -0.0 (the identity
// of IEEE addition).  The elements of B are walked in ascending order; lane
// a reads block (a, b) of the element's column b = local(B) (one contiguous
// run of npe blocks, 16-byte padded) and the block's row position from the
// pattern's element-to-column map, both prefetched one element ahead, and
// adds the block into the accumulator.  A byte per row position records
// whether the position has a value yet: the first block that reaches a
// position is stored, later ones are added, and positions that no element
// reaches are written as -0.0 (the identity of IEEE addition).  Every entry
// thus equals the reference's combination of its triplets (first value,
// then + each later one), signed zeros included, with one FP64 addition per
// contribution after the first only.  With init (values to accumulate into)
// the accumulator starts from them and every block is added.  The column is
// written out coalesced with its non-zero count: column (B,j) holds the
// entries (row node t, component i) at P*t + i.
// all_touched: every row position of a column receives a block (a gather
// over the pattern's own element lists), so the marks are not read when the
// column is written out.
// With spec.ptr0 the column is compacted (dropzeros!) straight into the
// stored CSC at the layout of an earlier assembly: each DoF column's
// non-zeros go, in row order, to [ptr0[c], ptr0[c+1]) (writes stay inside
// that range), and a column whose count differs sets *spec.mismatch; the
// structural values are then written only if nz is given.
template <int P, bool BLOCKVAL, class T>
__global__ void k_colgather(const int64_t *__restrict__ nptr, const int64_t *__restrict__ n2e_ptr,
                            const int2 *__restrict__ n2e, const uint16_t *__restrict__ pos,
                            const T *__restrict__ Kf, int64_t cs, int npe, int64_t non, int max_deg,
                            const double *__restrict__ init, double *__restrict__ nz,
                            int64_t *__restrict__ cnt, const int32_t *__restrict__ list,
                            const int32_t *__restrict__ nadj, StoredSpec spec, int all_touched,
                            int first_marked) {
  extern __shared__ double cg_smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  constexpr int BS = BLOCKVAL ? P * P : 1;
  constexpr int BSTR = kf_bstride(P, BLOCKVAL, (int)sizeof(T));  // stored block stride
  constexpr bool VEC = sizeof(T) == 4 && BSTR % 4 == 0;           // 16-byte block loads
  using W = typename GatherWord<T>::type;
  double *acc = cg_smem + (size_t)wib * max_deg * P * P;
  unsigned long long *accb = reinterpret_cast<unsigned long long *>(acc);
  const int ps = max_deg * P;  // accumulator plane stride
  unsigned char *has = reinterpret_cast<unsigned char *>(cg_smem + (size_t)wpb * max_deg * P * P) +
                       (size_t)wib * ((max_deg + 7) & ~7);
  const int nw = (int)non, wstride = (int)gridDim.x * wpb;  // node counts fit int32 (nadj holds int32 nodes)
  for (int w = (int)blockIdx.x * wpb + wib; w < nw; w += wstride) {
    const int64_t B = list ? (int64_t)__ldg(list + w) : (int64_t)w;  // column node (non: nodes of the list)
    const int64_t c0 = nptr[B];
    const int deg = (int)(nptr[B + 1] - c0);
    const int64_t s = n2e_ptr[B];
    const int nb = (int)(n2e_ptr[B + 1] - s);
    if (init) {  // accumulate into existing structural values (same layout as the output)
      const double *src = init + (size_t)P * P * c0;
      for (int idx = lane; idx < deg * P * P; idx += 32) {
        const int j = idx / (P * deg), r = idx - j * P * deg;
        accb[(size_t)j * ps + r] = reinterpret_cast<const unsigned long long *>(src)[idx];
      }
    } else if (!first_marked) {
      for (int t = lane; t < deg; t += 32) has[t] = 0;
    }
    const bool store_first = init == nullptr;
    __syncwarp();
    if (npe <= 32) {
      const bool act = lane < npe;
      W cur[BSTR], nxt[BSTR];
      unsigned tc = 0xffffu, tn = 0xffffu;
      auto load_block = [&](const T *v, W *dst) {
        if constexpr (VEC) {
#pragma unroll
          for (int m = 0; m < BSTR; m += 4) {
            const float4 f = __ldg(reinterpret_cast<const float4 *>(v + m));
            dst[m] = f.x; dst[m + 1] = f.y; dst[m + 2] = f.z; dst[m + 3] = f.w;
          }
        } else {
          const W *vw = reinterpret_cast<const W *>(v);
#pragma unroll
          for (int m = 0; m < BS; ++m) dst[m] = vw[m];
        }
      };
      if (nb > 0 && act) {
        const int2 el = n2e[s];
        load_block(Kf + ((size_t)el.x * npe + el.y) * cs + (size_t)lane * BSTR, cur);
        tc = pos[s * npe + lane];
      }
      for (int k = 0; k < nb; ++k) {  // elements of B, ascending
        if (k + 1 < nb && act) {
          const int2 el = n2e[s + k + 1];
          load_block(Kf + ((size_t)el.x * npe + el.y) * cs + (size_t)lane * BSTR, nxt);
          tn = pos[(s + k + 1) * npe + lane];
        }
        if (act && tc != 0xffffu) {  // the lanes of one element hold distinct positions
          if (first_marked) {  // the map marks each position's first block
            if (store_first && (tc & 0x8000u))
              add_block<P, BLOCKVAL, true>(acc, (int)(tc & 0x7fffu), cur, ps);
            else
              add_block<P, BLOCKVAL, false>(acc, (int)(tc & 0x7fffu), cur, ps);
          } else if (store_first && !has[tc]) {
            add_block<P, BLOCKVAL, true>(acc, (int)tc, cur, ps);
            has[tc] = 1;
          } else {
            add_block<P, BLOCKVAL, false>(acc, (int)tc, cur, ps);
          }
        }
        __syncwarp();
#pragma unroll
        for (int m = 0; m < BSTR; ++m) cur[m] = nxt[m];
        tc = tn;
      }
    } else {
      for (int k = 0; k < nb; ++k) {
        const int2 el = n2e[s + k];
        const T *col = Kf + ((size_t)el.x * npe + el.y) * cs;
        for (int a = lane; a < npe; a += 32) {
          const unsigned raw = pos[(s + k) * npe + a];
          const unsigned t = (first_marked && raw != 0xffffu) ? (raw & 0x7fffu) : raw;
          if (raw != 0xffffu) {
            if (first_marked) {
              if (store_first && (raw & 0x8000u))
                add_block<P, BLOCKVAL, true>(acc, (int)t, reinterpret_cast<const W *>(col + (size_t)a * BSTR), ps);
              else
                add_block<P, BLOCKVAL, false>(acc, (int)t, reinterpret_cast<const W *>(col + (size_t)a * BSTR), ps);
            } else if (store_first && !has[t]) {
              add_block<P, BLOCKVAL, true>(acc, (int)t, reinterpret_cast<const W *>(col + (size_t)a * BSTR), ps);
              has[t] = 1;
            } else {
              add_block<P, BLOCKVAL, false>(acc, (int)t, reinterpret_cast<const W *>(col + (size_t)a * BSTR), ps);
            }
          }
        }
        __syncwarp();
      }
    }
#pragma unroll
    for (int j = 0; j < P; ++j) {
      double *out = nz ? nz + (size_t)P * P * c0 + (size_t)j * P * deg : nullptr;
      if (spec.ptr0) {
        const int64_t o = spec.ptr0[B * P + j], oend = spec.ptr0[B * P + j + 1];
        const int32_t *rn = nadj + c0;
        int64_t run = 0;
        const unsigned below = (1u << lane) - 1u;
        // warp-uniform chunks of 64 entries, two consecutive ones per lane
        for (int i0 = 0; i0 < P * deg; i0 += 64) {
          const int idx = i0 + 2 * lane;
          unsigned long long v[2] = {0ull, 0ull};   // value bits
          bool keep[2];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const bool valid = idx + h < P * deg;
            if (valid) {
              v[h] = (!store_first || all_touched || has[(idx + h) / P]) ? accb[(size_t)j * ps + idx + h]
                                                                         : 0x8000000000000000ull;   // -0.0
              if (nz) reinterpret_cast<unsigned long long *>(out)[idx + h] = v[h];
            }
            keep[h] = valid && (v[h] << 1) != 0ull;
          }
          const unsigned b0 = __ballot_sync(0xffffffffu, keep[0]), b1 = __ballot_sync(0xffffffffu, keep[1]);
          int64_t at = o + run + __popc(b0 & below) + __popc(b1 & below);   // the lanes before, both entries
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            if (keep[h]) {
              if (at < oend) {
                const int t = (idx + h) / P, i = (idx + h) % P;
                spec.rowval_s[at] = (int64_t)P * rn[t] + i + 1;
                reinterpret_cast<unsigned long long *>(spec.nzval_s)[at] = v[h];
              }
              ++at;
            }
          }
          run += __popc(b0) + __popc(b1);
        }
        if (lane == 0 && run != oend - o) atomicOr(spec.mismatch, 1u);
      } else {
        int n = 0;
        for (int idx = lane; idx < P * deg; idx += 32) {
          const int t = idx / P, i = idx % P;
          const unsigned long long v =
              (!store_first || all_touched || has[t]) ? accb[(size_t)j * ps + idx] : 0x8000000000000000ull;
          reinterpret_cast<unsigned long long *>(out)[idx] = v;
          n += (v << 1) != 0ull;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) n += __shfl_xor_sync(0xffffffffu, n, off);
        if (lane == 0 && cnt) cnt[B * P + j] = n;
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- dropzeros
// Structural entry count of every column (a matrix that keeps its pattern).
__global__ void k_count_struct(const int64_t *__restrict__ colptr, int64_t ndof, int64_t *__restrict__ cnt) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ndof; c += (int64_t)gridDim.x * blockDim.x)
    cnt[c] = colptr[c + 1] - colptr[c];
}

__global__ void k_count_nz(const double *__restrict__ nz, const int64_t *__restrict__ colptr,
                           int64_t ndof, int64_t *__restrict__ cnt) {
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  for (int64_t c = (int64_t)blockIdx.x * wpb + (threadIdx.x >> 5); c < ndof;
       c += (int64_t)gridDim.x * wpb) {
    int64_t s = colptr[c], e = colptr[c + 1];
    int n = 0;
    for (int64_t k = s + lane; k < e; k += 32) n += nonzero_bits(nz[k]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) n += __shfl_xor_sync(0xffffffffu, n, off);
    if (lane == 0) cnt[c] = n;
  }
}

// One warp per DoF column; four 32-entry chunks loaded (values and row
// nodes) before their ballots so that each warp keeps 2 KB in flight.
// rowval_s may be null (values only); keepbits (or null) receives one bit
// per structural entry, set when the entry is stored (the array must start
// zeroed; chunk boundaries do not fall on word boundaries, so the words are
// or-ed in).
template <int P, bool KEEP>
__global__ void k_compact(const double *__restrict__ nz, const int64_t *__restrict__ colptr,
                          const int64_t *__restrict__ nptr, const int32_t *__restrict__ nadj,
                          int64_t ndof, const int64_t *__restrict__ outptr,
                          int64_t *__restrict__ rowval_s, double *__restrict__ nzval_s,
                          unsigned *__restrict__ keepbits = nullptr) {
  constexpr int U = 4;
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  for (int64_t c = (int64_t)blockIdx.x * wpb + (threadIdx.x >> 5); c < ndof;
       c += (int64_t)gridDim.x * wpb) {
    const int64_t s = colptr[c];
    const int len = (int)(colptr[c + 1] - s);
    const int32_t *rn = nadj + nptr[c / P];
    int64_t o = outptr[c];
    for (int l0 = 0; l0 < len; l0 += 32 * U) {
      double v[U];
      int64_t row[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int l = l0 + u * 32 + lane;
        v[u] = l < len ? nz[s + l] : 0.0;
        row[u] = l < len ? (int64_t)P * rn[l / P] + l % P : 0;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const bool keep = (l0 + u * 32 + lane < len) && (KEEP || nonzero_bits(v[u]));
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        if (keep) {
          const int off = __popc(bal & ((1u << lane) - 1u));
          if (rowval_s) rowval_s[o + off] = row[u] + 1;
          nzval_s[o + off] = v[u];
        }
        if (keepbits && lane == 0 && bal) {
          const int64_t sidx = s + l0 + u * 32;
          const int sh = (int)(sidx & 31);
          atomicOr(keepbits + (sidx >> 5), bal << sh);
          if (sh) atomicOr(keepbits + (sidx >> 5) + 1, bal >> (32 - sh));
        }
        o += __popc(bal);
      }
    }
  }
}

// Number of differing 32-bit words of two arrays (device counter).
__global__ void k_words_differ(const unsigned *__restrict__ a, const unsigned *__restrict__ b, int64_t n,
                               unsigned long long *cnt) {
  unsigned long long c = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    c += a[i] != b[i];
  if (c) atomicAdd(cnt, c);
}

__global__ void k_colptr_1based(const int64_t *__restrict__ in, int64_t n,
                                int64_t *__restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = in[i] + 1;
}

// Row sums of a symmetric matrix = column sums in row order, from 0.0
// (sum(M, dims=2) walks columns in order; M[R,C] == M[C,R] bit for bit).
__global__ void k_lump(const double *__restrict__ nz, const int64_t *__restrict__ colptr,
                       int64_t ndof, double *__restrict__ diag) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ndof;
       c += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int64_t k = colptr[c]; k < colptr[c + 1]; ++k) acc = __dadd_rn(acc, nz[k]);
    diag[c] = acc;
  }
}

__global__ void k_diag_stored(const double *__restrict__ diag, int64_t ndof,
                              int64_t *__restrict__ cnt) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ndof;
       c += (int64_t)gridDim.x * blockDim.x)
    cnt[c] = nonzero_bits(diag[c]);
}

__global__ void k_diag_compact(const double *__restrict__ diag, int64_t ndof,
                               const int64_t *__restrict__ outptr,
                               int64_t *__restrict__ rowval_s, double *__restrict__ nzval_s) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ndof;
       c += (int64_t)gridDim.x * blockDim.x)
    if (nonzero_bits(diag[c])) {
      rowval_s[outptr[c]] = c + 1;
      nzval_s[outptr[c]] = diag[c];
    }
}

__global__ void k_axpby(double a, const double *__restrict__ x, double b,
                        const double *__restrict__ y, double *__restrict__ z, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    z[i] = __fma_rn(b, y[i], __dmul_rn(a, x[i]));
}

inline unsigned grid_1d(int64_t n, int threads, int sms) {
  int64_t b = (n + threads - 1) / threads;
  int64_t cap = (int64_t)sms * 16;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

template <int KIND, int DIM, bool SM>
int launch_elem(llf_ctx *ctx, const ElemArgs &a, size_t smem, unsigned grid) {
  auto fn = k_elem_fp64<KIND, DIM, SM>;
  if (smem > 48 * 1024)
    LLF_CUDA_TRY(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
  KernelScope ks(ctx, "k_elem_fp64");
  fn<<<grid, ELEM_THREADS, smem, ctx->stream>>>(a);
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  return LLF_OK;
}

// The staged affine kernel when every element is affine, the element has
// enough node pairs to fill a CTA and two CTAs fit on an SM; *done = false
// otherwise.  Threads: the node pairs in as few rounds of at most 256 as
// possible, rounded up to whole warps (hex27: 378 pairs, 2 rounds of 192).
template <int KIND, int DIM>
int run_elem_affine(llf_ctx *ctx, const ElemArgs &a, bool *done) {
  *done = false;
  const int npairs = a.npairs;
  if (!a.all_affine || !a.aflag || npairs < 32) return LLF_OK;
  const int tab_n = KIND == KIND_MASS ? npairs : npairs * 9;
  const size_t smem = sizeof(double) * ((size_t)a.npe * a.colstride + ((tab_n + 1) & ~1) + AFF_DOUBLES) + 16;
  if (smem > 110 * 1024) return LLF_OK;
  const int rounds = (npairs + AFFK_MAX_THREADS - 1) / AFFK_MAX_THREADS;
  const int threads = ((npairs + rounds - 1) / rounds + 31) / 32 * 32;
  auto fn = k_elem_affine<KIND, DIM>;
  if (smem > 48 * 1024)
    LLF_CUDA_TRY(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  LLF_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
  if (per_sm < 1) return LLF_OK;
  if (a.cta_cap > 0 && per_sm > a.cta_cap) per_sm = a.cta_cap;
  int64_t grid = (int64_t)ctx->num_sms * per_sm;
  if (grid > a.nel) grid = a.nel;
  KernelScope ks(ctx, "k_elem_affine");
  fn<<<(unsigned)grid, threads, smem, ctx->stream>>>(a, tab_n);
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  *done = true;
  return LLF_OK;
}

template <int KIND, int DIM>
int run_elem(llf_ctx *ctx, ElemArgs a) {
  {
    bool done = false;
    const int rc = run_elem_affine<KIND, DIM>(ctx, a, &done);
    if (rc != LLF_OK || done) return rc;
  }
  const int npe = a.npe, nip = a.nip;
  const int gsw = (KIND == KIND_MASS) ? 1 : DIM;
  const size_t tables = sizeof(double) * ((size_t)nip * npe * DIM + nip +
                                          (KIND == KIND_MASS ? (size_t)nip * npe : 0));
  const size_t local = sizeof(double) * ((size_t)npe * DIM + nip + (size_t)nip * 9 + AFF_DOUBLES);
  const size_t gs = sizeof(double) * 2 * (size_t)nip * npe * gsw;
  const bool in_smem = tables + local + gs <= 96 * 1024;
  const size_t smem = in_smem ? tables + local + gs : local;
  if (smem > 200 * 1024) return llf_fail(ctx, LLF_ERR_LIMIT, "element exceeds shared memory");
  // the dynamic shared-memory limit is raised before the occupancy query:
  // above 48 KB the query answers 0 for a kernel still at the default limit
  int per_sm = 0;
  if (in_smem) {
    if (smem > 48 * 1024)
      LLF_CUDA_TRY(ctx, cudaFuncSetAttribute(k_elem_fp64<KIND, DIM, true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    LLF_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                          &per_sm, k_elem_fp64<KIND, DIM, true>, ELEM_THREADS, smem));
  } else {
    if (smem > 48 * 1024)
      LLF_CUDA_TRY(ctx, cudaFuncSetAttribute(k_elem_fp64<KIND, DIM, false>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    LLF_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                          &per_sm, k_elem_fp64<KIND, DIM, false>, ELEM_THREADS, smem));
  }
  if (per_sm < 1) per_sm = 1;
  if (a.cta_cap > 0 && per_sm > a.cta_cap) per_sm = a.cta_cap;
  int64_t grid = (int64_t)ctx->num_sms * per_sm;
  if (grid > a.nel) grid = a.nel > 0 ? a.nel : 1;
  double *scratch = nullptr;
  if (!in_smem) {
    a.scratch_stride = (int64_t)(gs / sizeof(double));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &scratch, (size_t)grid * a.scratch_stride));
    a.scratch = scratch;
  }
  int rc = in_smem ? launch_elem<KIND, DIM, true>(ctx, a, smem, (unsigned)grid)
                   : launch_elem<KIND, DIM, false>(ctx, a, smem, (unsigned)grid);
  dfree(ctx, scratch);
  return rc;
}

// Gather over explicit node -> element lists and element-to-column map (the
// pattern's own, or those of another element set on the same nodes).
// The column nodes of the pattern in two degree classes, once per pattern:
// when at least 60 % of the nodes have a degree of at most 0.7 of the
// largest, those nodes form the low class (ascending), the rest follow.
// The low class then runs with a smaller accumulator and so with more warps
// per SM (hex27: degree <= 75 against 125 for 7/8 of the nodes).  Each
// column is summed the same way whichever launch takes it.
static int gather_split(llf_ctx *ctx, llf_pattern *pat) {
  if (pat->gather_split_done) return LLF_OK;
  pat->gather_split_done = true;
  const int64_t non = pat->mesh->non;
  const int thr = pat->tune.gather_thr;   // percent of the largest degree
  if (non < 1024 || pat->max_deg < 16 || thr <= 0) return LLF_OK;
  std::vector<int64_t> h(non + 1);
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(h.data(), pat->d_nptr, sizeof(int64_t) * (non + 1), cudaMemcpyDeviceToHost,
                                    ctx->stream));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<int64_t> hist(pat->max_deg + 1, 0);
  for (int64_t b = 0; b < non; ++b) hist[h[b + 1] - h[b]]++;
  int md_low = -1;
  int64_t acc = 0;
  for (int d = 0; d <= pat->max_deg; ++d) {
    acc += hist[d];
    if (acc >= (non * 6 + 9) / 10) { md_low = d; break; }
  }
  if (md_low < 1 || md_low * 100 > pat->max_deg * thr) return LLF_OK;
  std::vector<int32_t> order;
  order.reserve(non);
  for (int64_t b = 0; b < non; ++b)
    if (h[b + 1] - h[b] <= md_low) order.push_back((int32_t)b);
  const int64_t n_low = (int64_t)order.size();
  for (int64_t b = 0; b < non; ++b)
    if (h[b + 1] - h[b] > md_low) order.push_back((int32_t)b);
  LLF_CUDA_TRY(ctx, dalloc(ctx, &pat->d_gather_nodes, non));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(pat->d_gather_nodes, order.data(), sizeof(int32_t) * non, cudaMemcpyHostToDevice,
                                    ctx->stream));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  pat->gather_n_low = n_low;
  pat->gather_md_low = md_low;
  return LLF_OK;
}

// Marks, once per pattern, the first block of every row position in the
// pattern's element-to-column map: per column node B (a warp each), its
// elements in ascending order, and the first element whose block reaches a
// row position gets bit 15 of that map entry (positions fit 15 bits).  The
// gather then stores that block and adds the later ones without keeping
// per-position marks of its own.
__global__ void k_mark_first(const int64_t *__restrict__ nptr, const int64_t *__restrict__ n2e_ptr,
                             uint16_t *__restrict__ pos, int npe, int64_t non, int max_deg) {
  extern __shared__ unsigned char mf_has[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  unsigned char *has = mf_has + (size_t)wib * ((max_deg + 7) & ~7);
  for (int64_t B = (int64_t)blockIdx.x * wpb + wib; B < non; B += (int64_t)gridDim.x * wpb) {
    const int deg = (int)(nptr[B + 1] - nptr[B]);
    const int64_t s = n2e_ptr[B];
    const int nb = (int)(n2e_ptr[B + 1] - s);
    for (int t = lane; t < deg; t += 32) has[t] = 0;
    __syncwarp();
    for (int k = 0; k < nb; ++k) {
      for (int a = lane; a < npe; a += 32) {  // the lanes of one element hold distinct positions
        const unsigned raw = pos[(s + k) * npe + a];
        if (raw < 0x8000u && !has[raw]) {
          has[raw] = 1;
          pos[(s + k) * npe + a] = (uint16_t)(raw | 0x8000u);
        }
      }
      __syncwarp();
    }
  }
}

template <int P, bool BV, class T>
int run_colgather(llf_ctx *ctx, llf_pattern *pat, const int64_t *n2e_ptr, const int2 *n2e, const uint16_t *pos,
                  int npe, const T *Kf, int64_t cs, const double *init, double *nz, int64_t *cnt,
                  int64_t B0 = 0, int64_t nB = -1, const StoredSpec *spec = nullptr) {
  const StoredSpec sp = spec ? *spec : StoredSpec{};
  // column nodes [B0, B0 + nB): the node-indexed arrays are offset, the
  // offsets they hold (into n2e, pos, nz) stay absolute
  if (nB < 0) nB = pat->mesh->non - B0;
  if (pat->conn_version != pat->mesh->conn_version)
    return llf_fail(ctx, LLF_ERR_STATE, "the mesh connectivity changed after the pattern was built; rebuild it");
  // the pattern's own map: each position's first block marked (once)
  bool first_marked = false;
  const int mdm = pat->max_deg > 0 ? pat->max_deg : 1;
  if (pos == pat->d_pos && mdm < 0x7fff) {
    if (!pat->pos_first) {
      const int mw = 4;
      const size_t msm = (size_t)mw * ((mdm + 7) & ~7);
      KernelScope ks(ctx, "k_mark_first");
      k_mark_first<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((pat->mesh->non + mw - 1) / mw,
                                                                    (int64_t)ctx->num_sms * 8)),
                     mw * 32, msm, ctx->stream>>>(pat->d_nptr, pat->d_n2e_ptr, pat->d_pos, npe, pat->mesh->non, mdm);
      LLF_CUDA_TRY(ctx, cudaGetLastError());
      pat->pos_first = true;
    }
    first_marked = true;
  }
  auto fn = k_colgather<P, BV, T>;
  // one launch over `count` column nodes (the list's, or [B0, B0 + count))
  // with an accumulator of md row positions per warp
  auto launch = [&](int md, const int32_t *list, int64_t b0, int64_t count) -> int {
    if (count <= 0) return LLF_OK;
    const size_t per_warp = (size_t)md * P * P * sizeof(double) + (size_t)((md + 7) & ~7);
    int wpb = (int)std::min<size_t>(pat->tune.gather_wpb > 0 ? pat->tune.gather_wpb : 4, (200 * 1024) / per_warp);
    if (wpb < 1) wpb = 1;
    size_t smem = (size_t)wpb * per_warp;
    if (smem > 200 * 1024)
      return llf_fail(ctx, LLF_ERR_LIMIT, "a column node has too many neighbours for the gather buffer");
    if (smem > 48 * 1024)
      LLF_CUDA_TRY(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 1;
    LLF_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, wpb * 32, smem));
    int64_t grid = (int64_t)ctx->num_sms * (per_sm < 1 ? 1 : per_sm);
    int64_t need = (count + wpb - 1) / wpb;
    if (grid > need) grid = need > 0 ? need : 1;
    KernelScope ks(ctx, "k_colgather");
    fn<<<(unsigned)grid, wpb * 32, smem, ctx->stream>>>(pat->d_nptr + b0, n2e_ptr + b0, n2e, pos, Kf, cs, npe, count,
                                                        md, init, nz, cnt ? cnt + b0 * P : nullptr, list,
                                                        pat->d_nadj, sp, n2e_ptr == pat->d_n2e_ptr ? 1 : 0,
                                                        first_marked ? 1 : 0);
    LLF_CUDA_TRY(ctx, cudaGetLastError());
    return LLF_OK;
  };
  const int md = pat->max_deg > 0 ? pat->max_deg : 1;
  if (B0 == 0 && nB == pat->mesh->non) {
    int rc = gather_split(ctx, pat);
    if (rc != LLF_OK) return rc;
    if (pat->d_gather_nodes) {
      rc = launch(pat->gather_md_low, pat->d_gather_nodes, 0, pat->gather_n_low);
      if (rc == LLF_OK)
        rc = launch(md, pat->d_gather_nodes + pat->gather_n_low, 0, pat->mesh->non - pat->gather_n_low);
      return rc;
    }
  }
  return launch(md, nullptr, B0, nB);
}

}  // namespace

// ------------------------------------------------------------------ host
template <class T>
int gather_full_t(llf_ctx *ctx, llf_pattern *pat, const int64_t *n2e_ptr, const int2 *n2e, const uint16_t *pos,
                  int npe, const T *Kf, int64_t cs, bool blockval, const double *init, double *nz, int64_t *cnt,
                  StoredSpec *spec = nullptr);

// The gather into a kept stored layout; if a column's count differs, the
// usual gather (structural values and counts) follows.
template <class T>
int gather_spec_t(llf_ctx *ctx, llf_pattern *pat, const T *Kf, int64_t cs, bool blockval, StoredSpec *spec) {
  int rc = gather_full_t<T>(ctx, pat, pat->d_n2e_ptr, pat->d_n2e, pat->d_pos, pat->mesh->npe, Kf, cs, blockval,
                            nullptr, nullptr, nullptr, spec);
  if (rc != LLF_OK) return rc;
  unsigned mis = 1;
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(&mis, spec->mismatch, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (mis == 0) return LLF_OK;
  spec->fell_back = true;
  LLF_CUDA_TRY(ctx, dalloc(ctx, spec->nz_slot, pat->nnz));
  return gather_full_t<T>(ctx, pat, pat->d_n2e_ptr, pat->d_n2e, pat->d_pos, pat->mesh->npe, Kf, cs, blockval,
                          nullptr, *spec->nz_slot, spec->cnt_fallback, nullptr);
}

template <class T>
int gather_full_t(llf_ctx *ctx, llf_pattern *pat, const int64_t *n2e_ptr, const int2 *n2e, const uint16_t *pos,
                  int npe, const T *Kf, int64_t cs, bool blockval, const double *init, double *nz, int64_t *cnt,
                  StoredSpec *spec) {
  switch (pat->pdim * 2 + (blockval ? 1 : 0)) {
    case 2: return run_colgather<1, false, T>(ctx, pat, n2e_ptr, n2e, pos, npe, Kf, cs, init, nz, cnt, 0, -1, spec);
    case 3: return run_colgather<1, true, T>(ctx, pat, n2e_ptr, n2e, pos, npe, Kf, cs, init, nz, cnt, 0, -1, spec);
    case 4: return run_colgather<2, false, T>(ctx, pat, n2e_ptr, n2e, pos, npe, Kf, cs, init, nz, cnt, 0, -1, spec);
    case 5: return run_colgather<2, true, T>(ctx, pat, n2e_ptr, n2e, pos, npe, Kf, cs, init, nz, cnt, 0, -1, spec);
    case 6: return run_colgather<3, false, T>(ctx, pat, n2e_ptr, n2e, pos, npe, Kf, cs, init, nz, cnt, 0, -1, spec);
    case 7: return run_colgather<3, true, T>(ctx, pat, n2e_ptr, n2e, pos, npe, Kf, cs, init, nz, cnt, 0, -1, spec);
  }
  return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "pdim must be 1, 2 or 3");
}

int gather_full(llf_ctx *ctx, llf_pattern *pat, const double *Kf, int64_t colstride, bool blockval,
                double *nz, int64_t *cnt, const double *init, StoredSpec *spec) {
  if (spec) return gather_spec_t<double>(ctx, pat, Kf, colstride, blockval, spec);
  return gather_full_t<double>(ctx, pat, pat->d_n2e_ptr, pat->d_n2e, pat->d_pos, pat->mesh->npe, Kf, colstride,
                               blockval, init, nz, cnt);
}
int gather_full32(llf_ctx *ctx, llf_pattern *pat, const float *Kf, int64_t colstride, bool blockval,
                  double *nz, int64_t *cnt, const double *init, StoredSpec *spec) {
  if (spec) return gather_spec_t<float>(ctx, pat, Kf, colstride, blockval, spec);
  return gather_full_t<float>(ctx, pat, pat->d_n2e_ptr, pat->d_n2e, pat->d_pos, pat->mesh->npe, Kf, colstride,
                              blockval, init, nz, cnt);
}
int gather_full_ext(llf_ctx *ctx, llf_pattern *pat, const int64_t *n2e_ptr, const int2 *n2e, const uint16_t *pos,
                    int npe, const double *Kf, int64_t colstride, bool blockval, double *nz, int64_t *cnt) {
  return gather_full_t<double>(ctx, pat, n2e_ptr, n2e, pos, npe, Kf, colstride, blockval, nullptr, nz, cnt);
}

// Structural values from the stored CSC, one warp per DoF column: the
// column's structural entries are zeroed, then each stored entry finds its
// structural position (its row node by binary search in the column's node
// list, sorted) and is written there.
template <int P>
__global__ void k_expand_nz(const int64_t *__restrict__ colptr, const int64_t *__restrict__ nptr,
                            const int32_t *__restrict__ nadj, int64_t ndof, const int64_t *__restrict__ colptr_s,
                            const int64_t *__restrict__ rowval_s, const double *__restrict__ nzval_s,
                            double *__restrict__ nz, unsigned *__restrict__ status) {
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  for (int64_t c = (int64_t)blockIdx.x * wpb + (threadIdx.x >> 5); c < ndof; c += (int64_t)gridDim.x * wpb) {
    const int64_t s = colptr[c], len = colptr[c + 1] - s;
    const int64_t c0 = nptr[c / P];
    const int deg = (int)(nptr[c / P + 1] - c0);
    for (int64_t l = lane; l < len; l += 32) nz[s + l] = 0.0;
    __syncwarp();
    const int64_t o0 = colptr_s[c] - 1, o1 = colptr_s[c + 1] - 1;
    for (int64_t k = o0 + lane; k < o1; k += 32) {
      const int64_t r = rowval_s[k] - 1;
      const int32_t node = (int32_t)(r / P);
      int lo = 0, hi = deg - 1;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (nadj[c0 + mid] < node) lo = mid + 1; else hi = mid;
      }
      if (deg > 0 && nadj[c0 + lo] == node) {
        nz[s + (int64_t)P * lo + r % P] = nzval_s[k];
      } else {
        atomicOr(status, ST_PATTERN);
      }
    }
  }
}

int matrix_ensure_nz(llf_ctx *ctx, const llf_matrix *cm) {
  llf_matrix *m = const_cast<llf_matrix *>(cm);
  if (m->d_nz || m->diagonal_only) return LLF_OK;
  if (!m->d_colptr_s) return llf_fail(ctx, LLF_ERR_STATE, "matrix has neither structural nor stored values");
  llf_pattern *pat = m->pat;
  const int64_t n = pat->ndof;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_nz, pat->nnz > 0 ? pat->nnz : 1));
  unsigned g = grid_1d(n * 32, 256, ctx->num_sms);
  KernelScope ks(ctx, "k_expand_nz");
  switch (pat->pdim) {
#define LLF_EXPAND(PP)                                                                                          \
  k_expand_nz<PP><<<g, 256, 0, ctx->stream>>>(pat->d_colptr, pat->d_nptr, pat->d_nadj, n, m->d_colptr_s,       \
                                              m->d_rowval_s, m->d_nzval_s, m->d_nz, ctx->d_status)
    case 1: LLF_EXPAND(1); break;
    case 2: LLF_EXPAND(2); break;
    case 3: LLF_EXPAND(3); break;
#undef LLF_EXPAND
    default: return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "pdim must be 1, 2 or 3");
  }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  return llf_check_status(ctx, "structural values from the stored CSC");
}

int matrix_finalize(llf_ctx *ctx, llf_matrix *m, int64_t *counts, int64_t **ptr0_out) {
  llf_pattern *pat = m->pat;
  const int64_t n = pat->ndof;
  cudaStream_t s = ctx->stream;
  int64_t *cnt = counts;
  const bool keep = m->keep_pattern && !m->diagonal_only;
  if (!cnt || m->diagonal_only || keep) {
    cnt = nullptr;
    LLF_CUDA_TRY(ctx, dalloc(ctx, &cnt, n + 1));
    LLF_CUDA_TRY(ctx, cudaMemsetAsync(cnt, 0, sizeof(int64_t) * (n + 1), s));
    if (keep) {
      KernelScope ks(ctx, "k_count_struct");
      k_count_struct<<<grid_1d(n, 256, ctx->num_sms), 256, 0, s>>>(pat->d_colptr, n, cnt);
    } else if (m->diagonal_only) {
      KernelScope ks(ctx, "k_diag_stored");
      k_diag_stored<<<grid_1d(n, 256, ctx->num_sms), 256, 0, s>>>(m->d_diag, n, cnt);
    } else {
      KernelScope ks(ctx, "k_count_nz");
      k_count_nz<<<grid_1d(n * 32, 256, ctx->num_sms), 256, 0, s>>>(m->d_nz, pat->d_colptr, n, cnt);
    }
    LLF_CUDA_TRY(ctx, cudaGetLastError());
  }
  int64_t *ptr0 = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &ptr0, n + 1));
  int64_t total = 0;
  {
    KernelScope ks(ctx, "scan");
    LLF_CUDA_TRY(ctx, exclusive_scan_i64(ctx, cnt, ptr0, n + 1, &total));
  }
  dfree(ctx, m->d_colptr_s);
  dfree(ctx, m->d_rowval_s);
  dfree(ctx, m->d_nzval_s);
  m->nnz_s = total;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_colptr_s, n + 1));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_rowval_s, total));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_nzval_s, total));
  if (m->diagonal_only) {
    KernelScope ks(ctx, "k_diag_compact");
    k_diag_compact<<<grid_1d(n, 256, ctx->num_sms), 256, 0, s>>>(m->d_diag, n, ptr0,
                                                                 m->d_rowval_s, m->d_nzval_s);
  } else {
    unsigned g = grid_1d(n * 32, 256, ctx->num_sms);
    KernelScope ks(ctx, "k_compact");
    switch (pat->pdim) {
#define LLF_COMPACT(PP, KK) \
  k_compact<PP, KK><<<g, 256, 0, s>>>(m->d_nz, pat->d_colptr, pat->d_nptr, pat->d_nadj, n, ptr0, m->d_rowval_s, \
                                      m->d_nzval_s)
      case 1: if (keep) LLF_COMPACT(1, true); else LLF_COMPACT(1, false); break;
      case 2: if (keep) LLF_COMPACT(2, true); else LLF_COMPACT(2, false); break;
      case 3: if (keep) LLF_COMPACT(3, true); else LLF_COMPACT(3, false); break;
#undef LLF_COMPACT
      default: return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "pdim must be 1, 2 or 3");
    }
  }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  {
    KernelScope ks(ctx, "k_colptr_1based");
    k_colptr_1based<<<grid_1d(n + 1, 256, ctx->num_sms), 256, 0, s>>>(ptr0, n + 1, m->d_colptr_s);
  }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  if (cnt != counts) dfree(ctx, cnt);
  if (ptr0_out) {
    *ptr0_out = ptr0;
  } else {
    dfree(ctx, ptr0);
  }
  return LLF_OK;
}

// ------------------------------------------------------- stored layouts
namespace {

llf_pattern::StoredLayout *layout_find(llf_pattern *pat, int kind, int form) {
  for (auto &l : pat->layouts)
    if (l.d_ptr0 && l.kind == kind && l.form == form) return &l;
  return nullptr;
}

// Keep ptr0 (ndof + 1, taken over) as the layout of (kind, form): in the
// slot of the same operator and form, else an empty one, else the least
// recently used.
void layout_store(llf_ctx *ctx, llf_pattern *pat, int kind, int form, int64_t *ptr0, int64_t total) {
  llf_pattern::StoredLayout *slot = layout_find(pat, kind, form);
  if (!slot)
    for (auto &l : pat->layouts)
      if (!l.d_ptr0) { slot = &l; break; }
  if (!slot) {
    slot = &pat->layouts[0];
    for (auto &l : pat->layouts)
      if (l.used < slot->used) slot = &l;
  }
  dfree(ctx, slot->d_ptr0);
  slot->kind = kind;
  slot->form = form;
  slot->total = total;
  slot->d_ptr0 = ptr0;
  slot->used = ++pat->layout_clock;
}

// Stored-layout reuse is on unless LLF_STORED_LAYOUT=0.
bool layout_reuse_enabled() {
  const char *v = getenv("LLF_STORED_LAYOUT");
  return !(v && v[0] == '0');
}

}  // namespace

void pattern_free_layouts(llf_ctx *ctx, llf_pattern *pat) {
  for (auto &l : pat->layouts) {
    dfree(ctx, l.d_ptr0);
    l = llf_pattern::StoredLayout{};
  }
}

int assemble_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int kind, int ptype,
                  const double *c1, const double *c2, int nmat, int form, int lumped,
                  llf_matrix *m, const double *init, GatherSink *sink) {
  (void)ptype;
  if (!pat->tune.from_tuner) tune_lookup(pat, kind, form);
  const int dim = mesh->dim;
  const int npe = mesh->npe;
  const int P = pat->pdim;
  const int BS = (kind == KIND_ELASTIC) ? P * P : 1;
  cudaStream_t s = ctx->stream;

  double *d_c1 = nullptr, *d_c2 = nullptr;
  int64_t *cnt = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &d_c1, nmat));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &d_c2, nmat));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &cnt, pat->ndof + 1));
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(cnt, 0, sizeof(int64_t) * (pat->ndof + 1), s));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d_c1, c1, sizeof(double) * nmat, cudaMemcpyHostToDevice, s));
  LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d_c2, c2 ? c2 : c1, sizeof(double) * nmat,
                                    cudaMemcpyHostToDevice, s));
  // the stored layout of the last assembly of this operator and form on
  // the pattern: the gather then writes the stored CSC itself, and the
  // structural values are left to matrix_ensure_nz
  const bool reuse = !sink && !init && !(kind == KIND_MASS && lumped) && !m->keep_pattern && layout_reuse_enabled();
  llf_pattern::StoredLayout *lay = reuse ? layout_find(pat, kind, form) : nullptr;
  StoredSpec spec;
  unsigned *d_mis = nullptr;
  if (lay) {
    LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_rowval_s, lay->total > 0 ? lay->total : 1));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_nzval_s, lay->total > 0 ? lay->total : 1));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &d_mis, 1));
    LLF_CUDA_TRY(ctx, cudaMemsetAsync(d_mis, 0, sizeof(unsigned), s));
    spec.ptr0 = lay->d_ptr0;
    spec.rowval_s = m->d_rowval_s;
    spec.nzval_s = m->d_nzval_s;
    spec.mismatch = d_mis;
    spec.nz_slot = &m->d_nz;
    spec.cnt_fallback = cnt;
    // the column pointers follow from the layout alone (recomputed if a
    // column's count turns out to differ)
    LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_colptr_s, pat->ndof + 1));
    {
      KernelScope ks(ctx, "k_colptr_1based");
      k_colptr_1based<<<grid_1d(pat->ndof + 1, 256, ctx->num_sms), 256, 0, s>>>(lay->d_ptr0, pat->ndof + 1,
                                                                               m->d_colptr_s);
    }
    LLF_CUDA_TRY(ctx, cudaGetLastError());
  } else if (!sink) {
    LLF_CUDA_TRY(ctx, dalloc(ctx, &m->d_nz, pat->nnz));
  }
  StoredSpec *sp = lay ? &spec : nullptr;
  int64_t *ptr0 = nullptr;   // the stored layout of this assembly, kept on the pattern
  // affine geometry of every element (built-in tables only), kept on the
  // mesh until its coordinates, connectivity, materials or tables change
  uint8_t *aflag = nullptr;
  double *ageo = nullptr;
  bool all_affine = false;
  if (mesh->d_Rp) {
    if (mesh->geo_cached != mesh->geo_version || mesh->geo_cached_tables != mesh->tables_version ||
        !mesh->d_aflag) {
      mesh->geo_cached = -1;
      if (!mesh->d_aflag) {
        LLF_CUDA_TRY(ctx, dalloc(ctx, &mesh->d_aflag, mesh->nel));
        LLF_CUDA_TRY(ctx, dalloc(ctx, &mesh->d_ageo, (size_t)mesh->nel * 10));
      }
      unsigned long long *nonaff = nullptr;   // elements in use that are not affine
      LLF_CUDA_TRY(ctx, dalloc(ctx, &nonaff, 1));
      LLF_CUDA_TRY(ctx, cudaMemsetAsync(nonaff, 0, sizeof(unsigned long long), s));
      {
        KernelScope ks(ctx, "k_affine_geometry");
        const unsigned g = grid_1d(mesh->nel, 128, ctx->num_sms);
        if (dim == 3)
          k_affine_geometry<3><<<g, 128, 0, s>>>(mesh->d_xyz, mesh->d_conn, mesh->d_emat, mesh->nel, npe,
                                                 mesh->d_dN, mesh->d_nref, mesh->d_ageo, mesh->d_aflag, nonaff);
        else
          k_affine_geometry<2><<<g, 128, 0, s>>>(mesh->d_xyz, mesh->d_conn, mesh->d_emat, mesh->nel, npe,
                                                 mesh->d_dN, mesh->d_nref, mesh->d_ageo, mesh->d_aflag, nonaff);
        LLF_CUDA_TRY(ctx, cudaGetLastError());
      }
      unsigned long long h = 1;
      LLF_CUDA_TRY(ctx, cudaMemcpyAsync(&h, nonaff, sizeof(h), cudaMemcpyDeviceToHost, s));
      LLF_CUDA_TRY(ctx, cudaStreamSynchronize(s));
      dfree(ctx, nonaff);
      mesh->geo_all_affine = h == 0;
      mesh->geo_cached = mesh->geo_version;
      mesh->geo_cached_tables = mesh->tables_version;
    }
    aflag = mesh->d_aflag;
    ageo = mesh->d_ageo;
    all_affine = mesh->geo_all_affine;
  }
  int rc = LLF_OK;
  if (form == LLF_FP32Q) {
    rc = assemble_fp32_impl(ctx, mesh, pat, kind, d_c1, d_c2, aflag, ageo, m->d_nz, cnt, init, sink, sp, all_affine);
  } else {
    double *Kf = nullptr;
    const int64_t cs = kf_colstride(npe, BS, (int)sizeof(double));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &Kf, (size_t)mesh->nel * npe * cs));
    ElemArgs a{};
    a.xyz = mesh->d_xyz;
    a.conn = mesh->d_conn;
    a.emat = mesh->d_emat;
    a.nel = mesh->nel;
    a.npe = npe;
    a.nip = mesh->nip;
    a.npairs = npe * (npe + 1) / 2;
    a.w = mesh->d_w;
    a.N = mesh->d_N;
    a.dN = mesh->d_dN;
    a.c1 = d_c1;
    a.c2 = d_c2;
    a.Kf = Kf;
    a.colstride = cs;
    a.status = ctx->d_status;
    a.aflag = aflag;
    a.ageo = ageo;
    a.Rp = mesh->d_Rp;
    a.Mp = mesh->d_Mp;
    a.cta_cap = pat->tune.elem_cap;
    a.all_affine = all_affine;
    // element range [e0, e1): the element-indexed arrays are offset
    auto elems = [&](int64_t e0, int64_t e1) -> int {
      ElemArgs b = a;
      b.conn = a.conn + e0 * npe;
      b.emat = a.emat ? a.emat + e0 : nullptr;
      b.nel = e1 - e0;
      b.Kf = a.Kf + e0 * npe * cs;
      b.aflag = a.aflag ? a.aflag + e0 : nullptr;
      b.ageo = a.ageo ? a.ageo + e0 * 10 : nullptr;
      if (b.nel <= 0) return LLF_OK;
      if (dim == 3) {
        if (kind == KIND_ELASTIC) return run_elem<KIND_ELASTIC, 3>(ctx, b);
        if (kind == KIND_HEAT) return run_elem<KIND_HEAT, 3>(ctx, b);
        return run_elem<KIND_MASS, 3>(ctx, b);
      }
      if (kind == KIND_ELASTIC) return run_elem<KIND_ELASTIC, 2>(ctx, b);
      if (kind == KIND_HEAT) return run_elem<KIND_HEAT, 2>(ctx, b);
      return run_elem<KIND_MASS, 2>(ctx, b);
    };
    if (sink) {
      rc = sink->gather(ctx, pat, Kf, cs, kind == KIND_ELASTIC, elems);
    } else {
      rc = elems(0, mesh->nel);
      if (rc == LLF_OK) rc = gather_full(ctx, pat, Kf, cs, kind == KIND_ELASTIC, m->d_nz, cnt, init, sp);
    }
    dfree(ctx, Kf);
  }
  dfree(ctx, d_c1);
  dfree(ctx, d_c2);
  if (rc == LLF_OK) rc = llf_check_status(ctx, "assembly");
  if (sink) {
    dfree(ctx, cnt);
    return rc;
  }
  if (rc == LLF_OK && kind == KIND_MASS && lumped) {
    m->diagonal_only = true;
    cudaError_t e = dalloc(ctx, &m->d_diag, pat->ndof);
    if (e != cudaSuccess) rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
    if (rc == LLF_OK) {
      KernelScope ks(ctx, "k_lump");
      k_lump<<<grid_1d(pat->ndof, 128, ctx->num_sms), 128, 0, s>>>(m->d_nz, pat->d_colptr,
                                                                   pat->ndof, m->d_diag);
    }
  }
  if (lay && rc == LLF_OK) {
    dfree(ctx, d_mis);
    if (!spec.fell_back) {  // every column's count matched: the stored CSC is complete
      m->nnz_s = lay->total;
      lay->used = ++pat->layout_clock;
      dfree(ctx, cnt);
      return LLF_OK;
    }
    // a column's count differed: the gather ran again the usual way
    dfree(ctx, m->d_rowval_s);
    dfree(ctx, m->d_nzval_s);
    rc = matrix_finalize(ctx, m, cnt, reuse ? &ptr0 : nullptr);
  } else {
    dfree(ctx, d_mis);
    if (rc == LLF_OK)
      rc = matrix_finalize(ctx, m, (kind == KIND_MASS && lumped) ? nullptr : cnt, reuse ? &ptr0 : nullptr);
  }
  if (rc == LLF_OK && ptr0) layout_store(ctx, pat, kind, form, ptr0, m->nnz_s);
  dfree(ctx, cnt);
  return rc;
}

namespace {
// Structural values of a*X + b*D for a lumped (diagonal) D: off the
// diagonal a*x, on it fma(b, d, a*x) — the full-full formula with zeros off
// the diagonal of D.
__global__ void k_axpby_diag(double a, const double *__restrict__ x, double b, const double *__restrict__ d,
                             const int64_t *__restrict__ colptr, const int32_t *__restrict__ diagpos, int P,
                             int64_t ndof, double *__restrict__ z) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ndof; c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t B = c / P;
    const int j = (int)(c - B * P);
    const int64_t k = colptr[c] + (int64_t)P * diagpos[B] + j;
    z[k] = __fma_rn(b, d[c], __dmul_rn(a, x[k]));
  }
}

__global__ void k_scale(double a, const double *__restrict__ x, double *__restrict__ z, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    z[i] = __dmul_rn(a, x[i]);
}
}  // namespace

int matrix_axpby_impl(llf_ctx *ctx, double a, const llf_matrix *A, double b,
                      const llf_matrix *B, llf_matrix *C) {
  if (!A->diagonal_only) {
    const int rc = matrix_ensure_nz(ctx, A);
    if (rc != LLF_OK) return rc;
  }
  if (!B->diagonal_only) {
    const int rc = matrix_ensure_nz(ctx, B);
    if (rc != LLF_OK) return rc;
  }
  if (A->pat != B->pat)
    return llf_fail(ctx, LLF_ERR_STATE, "axpby: matrices live on different patterns");
  C->pat = A->pat;
  if (A->diagonal_only && B->diagonal_only) {  // both lumped: a lumped result
    const int64_t n = A->pat->ndof;
    C->diagonal_only = true;
    LLF_CUDA_TRY(ctx, dalloc(ctx, &C->d_diag, n));
    k_axpby<<<grid_1d(n, 256, ctx->num_sms), 256, 0, ctx->stream>>>(a, A->d_diag, b, B->d_diag, C->d_diag, n);
    LLF_CUDA_TRY(ctx, cudaGetLastError());
    return matrix_finalize(ctx, C, nullptr);
  }
  if (A->diagonal_only || B->diagonal_only) {  // one lumped operand
    const llf_matrix *F = A->diagonal_only ? B : A, *D = A->diagonal_only ? A : B;
    const double af = A->diagonal_only ? b : a, bd = A->diagonal_only ? a : b;
    const llf_pattern *p = A->pat;
    LLF_CUDA_TRY(ctx, dalloc(ctx, &C->d_nz, p->nnz));
    k_scale<<<grid_1d(p->nnz, 256, ctx->num_sms), 256, 0, ctx->stream>>>(af, F->d_nz, C->d_nz, p->nnz);
    k_axpby_diag<<<grid_1d(p->ndof, 256, ctx->num_sms), 256, 0, ctx->stream>>>(
        af, F->d_nz, bd, D->d_diag, p->d_colptr, p->d_diagpos, p->pdim, p->ndof, C->d_nz);
    LLF_CUDA_TRY(ctx, cudaGetLastError());
    return matrix_finalize(ctx, C, nullptr);
  }
  int64_t n = A->pat->nnz;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &C->d_nz, n));
  {
    KernelScope ks(ctx, "k_axpby");
    k_axpby<<<grid_1d(n, 256, ctx->num_sms), 256, 0, ctx->stream>>>(a, A->d_nz, b, B->d_nz,
                                                                    C->d_nz, n);
  }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  return matrix_finalize(ctx, C, nullptr);
}

// ---------------------------------------------------------------- to host
// Assembly straight into host SparseMatrixCSC arrays.  After the element
// kernel the columns are processed in NSLAB node slabs on the compute
// stream: gather (structural values and non-zero counts), scan of the
// counts continued from the previous slab's end (a device-side carry),
// compaction and the 1-based column pointers.  Each slab's end offset is
// copied to pinned host memory behind an event; the host waits for slab s
// only, then copies its compacted rows and values to the caller's arrays
// on a second stream while the GPU works on the slabs after it, so the
// device-to-host copy (the largest cost of the whole call) overlaps all but
// the first slab of the gather and compaction.  The result is the one
// llf_assemble_stiffness + llf_matrix_copy_csc give, bit for bit.
namespace {

__global__ void k_slab_carry(int64_t *__restrict__ outptr, int64_t n, int64_t *__restrict__ carry, int s,
                             const int64_t *__restrict__ slab_total) {
  const int64_t c0 = carry[s];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    outptr[i] += c0;
  if (blockIdx.x == 0 && threadIdx.x == 0) carry[s + 1] = c0 + *slab_total;
}

// d_max[k] = 1 + the largest element index in the lists of the nodes of
// slab k (B[k] <= node < B[k+1]); lists are sorted, so the last entry.
__global__ void k_slab_last_elem(const int64_t *__restrict__ n2e_ptr, const int2 *__restrict__ n2e, int64_t non,
                                 const int64_t *__restrict__ B, int nslab, int64_t *__restrict__ d_max) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < non; v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = n2e_ptr[v + 1];
    if (e == n2e_ptr[v]) continue;
    int k = 0;
    while (k + 1 < nslab && v >= B[k + 1]) ++k;
    atomicMax((unsigned long long *)&d_max[k], (unsigned long long)(n2e[e - 1].x + 1));
  }
}

__global__ void k_colptr_last(const int64_t *__restrict__ carry, int s, int64_t *__restrict__ colptr_last) {
  *colptr_last = carry[s] + 1;
}

struct HostSlabSink : GatherSink {
  static constexpr int NSLAB = 16;
  int64_t capacity = 0;
  int64_t *h_colptr = nullptr, *h_rowval = nullptr;
  double *h_nzval = nullptr;
  unsigned *h_keep = nullptr;   // values-only form: keep bits instead of rowval
  int keep_changed = 1;         // values-only form: the bits differ from the last call's on the pattern
  int64_t nnz = 0;

  template <class T>
  int run(llf_ctx *ctx, llf_pattern *pat, const T *Kf, int64_t cs, bool blockval, const ElemLauncher &elems) {
    const int P = pat->pdim;
    const int64_t non = pat->mesh->non, ndof = pat->ndof;
    cudaStream_t s = ctx->stream;
    double *nz = nullptr, *nzval = nullptr;
    int64_t *cnt = nullptr, *outptr = nullptr, *rowval = nullptr, *colptr = nullptr, *carry = nullptr,
            *totals = nullptr, *h_end = nullptr;
    cudaStream_t cp = nullptr;
    cudaEvent_t ev[NSLAB] = {}, done[NSLAB] = {};
    int rc = LLF_OK;
    unsigned *keep = nullptr;
    const int64_t nwords = pat->nnz / 32 + 2;
    cudaError_t e = dalloc(ctx, &nz, pat->nnz);
    if (e == cudaSuccess && h_keep) e = dalloc(ctx, &keep, nwords);
    if (e == cudaSuccess && h_keep) e = cudaMemsetAsync(keep, 0, sizeof(unsigned) * nwords, s);
    if (e == cudaSuccess) e = dalloc(ctx, &cnt, ndof + 1);
    if (e == cudaSuccess) e = dalloc(ctx, &outptr, ndof + 1);
    if (e == cudaSuccess) e = dalloc(ctx, &colptr, ndof + 1);
    if (e == cudaSuccess && !h_keep) e = dalloc(ctx, &rowval, pat->nnz);
    if (e == cudaSuccess) e = dalloc(ctx, &nzval, pat->nnz);
    if (e == cudaSuccess) e = dalloc(ctx, &carry, NSLAB + 1);
    if (e == cudaSuccess) e = dalloc(ctx, &totals, NSLAB);
    if (e == cudaSuccess) e = cudaMemsetAsync(carry, 0, sizeof(int64_t) * (NSLAB + 1), s);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&h_end, sizeof(int64_t) * (NSLAB + 1));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cp, cudaStreamNonBlocking);
    for (int k = 0; k < NSLAB && e == cudaSuccess; ++k) {
      e = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
    // 1. all slabs on the compute stream, each after the elements it needs
    int64_t B[NSLAB + 1];
    for (int k = 0; k <= NSLAB; ++k) B[k] = non * k / NSLAB;
    if (rc == LLF_OK) rc = slab_elements(ctx, pat, B);
    int64_t e_done = 0;
    for (int k = 0; k < NSLAB && rc == LLF_OK; ++k) {
      const int64_t B0 = B[k], nB = B[k + 1] - B[k], c0 = B0 * P, nc = nB * P;
      const int64_t e_need = pat->slab_elem_end[k];
      if (e_need > e_done) {
        rc = elems(e_done, e_need);
        if (rc != LLF_OK) break;
        e_done = e_need;
      }
      if (nB > 0) {
        switch (P * 2 + (blockval ? 1 : 0)) {
          case 2: rc = run_colgather<1, false, T>(ctx, pat, pat->d_n2e_ptr, pat->d_n2e, pat->d_pos, pat->mesh->npe, Kf, cs, nullptr, nz, cnt, B0, nB); break;
          case 3: rc = run_colgather<1, true, T>(ctx, pat, pat->d_n2e_ptr, pat->d_n2e, pat->d_pos, pat->mesh->npe, Kf, cs, nullptr, nz, cnt, B0, nB); break;
          case 4: rc = run_colgather<2, false, T>(ctx, pat, pat->d_n2e_ptr, pat->d_n2e, pat->d_pos, pat->mesh->npe, Kf, cs, nullptr, nz, cnt, B0, nB); break;
          case 5: rc = run_colgather<2, true, T>(ctx, pat, pat->d_n2e_ptr, pat->d_n2e, pat->d_pos, pat->mesh->npe, Kf, cs, nullptr, nz, cnt, B0, nB); break;
          case 6: rc = run_colgather<3, false, T>(ctx, pat, pat->d_n2e_ptr, pat->d_n2e, pat->d_pos, pat->mesh->npe, Kf, cs, nullptr, nz, cnt, B0, nB); break;
          case 7: rc = run_colgather<3, true, T>(ctx, pat, pat->d_n2e_ptr, pat->d_n2e, pat->d_pos, pat->mesh->npe, Kf, cs, nullptr, nz, cnt, B0, nB); break;
          default: rc = llf_fail(ctx, LLF_ERR_UNSUPPORTED, "pdim must be 1, 2 or 3");
        }
        if (rc != LLF_OK) break;
        {
          KernelScope ks(ctx, "scan");
          e = exclusive_scan_i64_dev(ctx, cnt + c0, outptr + c0, nc, totals + k);
        }
        if (e != cudaSuccess) { rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e)); break; }
      } else {
        cudaMemsetAsync(totals + k, 0, sizeof(int64_t), s);
      }
      k_slab_carry<<<grid_1d(std::max<int64_t>(nc, 1), 256, ctx->num_sms), 256, 0, s>>>(outptr + c0, nc, carry, k,
                                                                                       totals + k);
      if (nc > 0) {
        const unsigned g = grid_1d(nc * 32, 256, ctx->num_sms);
        KernelScope ks(ctx, "k_compact");
#define LLF_SLAB_COMPACT(PP) \
  k_compact<PP, false><<<g, 256, 0, s>>>(nz, pat->d_colptr + c0, pat->d_nptr + B0, pat->d_nadj, nc, outptr + c0, \
                                          rowval, nzval, keep)
        if (P == 1) LLF_SLAB_COMPACT(1); else if (P == 2) LLF_SLAB_COMPACT(2); else LLF_SLAB_COMPACT(3);
#undef LLF_SLAB_COMPACT
        k_colptr_1based<<<grid_1d(nc, 256, ctx->num_sms), 256, 0, s>>>(outptr + c0, nc, colptr + c0);
      }
      if (k == NSLAB - 1) k_colptr_last<<<1, 1, 0, s>>>(carry, NSLAB, colptr + ndof);
      cudaMemcpyAsync(h_end + k + 1, carry + k + 1, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
      cudaEventRecord(ev[k], s);
      e = cudaGetLastError();
      if (e != cudaSuccess) { rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e)); break; }
    }
    // 2. each slab to the host as soon as it is compacted
    h_end[0] = 0;
    for (int k = 0; k < NSLAB && rc == LLF_OK; ++k) {
      e = cudaEventSynchronize(ev[k]);
      if (e != cudaSuccess) { rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e)); break; }
      const int64_t o0 = h_end[k], o1 = h_end[k + 1];
      if (o1 > capacity) { rc = llf_fail(ctx, LLF_ERR_LIMIT, "llf_assemble_stiffness_csc: capacity too small"); break; }
      const int64_t c0 = B[k] * P, nc = (B[k + 1] - B[k]) * P + (k == NSLAB - 1 ? 1 : 0);
      e = cudaStreamWaitEvent(cp, ev[k], 0);
      if (e == cudaSuccess && nc > 0)
        e = cudaMemcpyAsync(h_colptr + c0, colptr + c0, sizeof(int64_t) * nc, cudaMemcpyDeviceToHost, cp);
      if (e == cudaSuccess && o1 > o0 && !h_keep)
        e = cudaMemcpyAsync(h_rowval + o0, rowval + o0, sizeof(int64_t) * (o1 - o0), cudaMemcpyDeviceToHost, cp);
      if (e == cudaSuccess && o1 > o0)
        e = cudaMemcpyAsync(h_nzval + o0, nzval + o0, sizeof(double) * (o1 - o0), cudaMemcpyDeviceToHost, cp);
      if (e == cudaSuccess) e = cudaEventRecord(done[k], cp);
      if (e != cudaSuccess) rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
    }
    // the keep bits once every slab is compacted (the words at slab edges
    // take bits from both neighbours)
    if (rc == LLF_OK && h_keep) {
      const int64_t nw = (pat->nnz + 31) / 32;
      unsigned long long *ndiff = nullptr;
      unsigned long long hdiff = 1;
      e = cudaMemcpyAsync(h_keep, keep, sizeof(unsigned) * nw, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess && pat->d_keep_prev) {   // compare with the last call's bits on the device
        e = dalloc(ctx, &ndiff, 1);
        if (e == cudaSuccess) e = cudaMemsetAsync(ndiff, 0, sizeof(unsigned long long), s);
        if (e == cudaSuccess) {
          KernelScope ks(ctx, "k_words_differ");
          k_words_differ<<<grid_1d(nw, 256, ctx->num_sms), 256, 0, s>>>(keep, pat->d_keep_prev, nw, ndiff);
          e = cudaGetLastError();
        }
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(&hdiff, ndiff, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
      }
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      dfree(ctx, ndiff);
      if (e != cudaSuccess) {
        rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
      } else {
        keep_changed = hdiff != 0;
        dfree(ctx, pat->d_keep_prev);   // this call's bits become the pattern's reference
        pat->d_keep_prev = keep;
        keep = nullptr;
      }
    }
    if (cp) {
      cudaError_t e2 = cudaStreamSynchronize(cp);
      if (rc == LLF_OK && e2 != cudaSuccess) rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e2));
    }
    // the buffers are freed on the compute stream after the copies that read them
    for (int k = 0; k < NSLAB; ++k)
      if (done[k]) cudaStreamWaitEvent(s, done[k], 0);
    if (rc == LLF_OK) nnz = h_end[NSLAB];
    dfree(ctx, nz);
    dfree(ctx, cnt);
    dfree(ctx, outptr);
    dfree(ctx, colptr);
    dfree(ctx, rowval);
    dfree(ctx, nzval);
    dfree(ctx, carry);
    dfree(ctx, totals);
    dfree(ctx, keep);
    cudaStreamSynchronize(s);
    for (int k = 0; k < NSLAB; ++k) {
      if (ev[k]) cudaEventDestroy(ev[k]);
      if (done[k]) cudaEventDestroy(done[k]);
    }
    if (cp) cudaStreamDestroy(cp);
    if (h_end) cudaFreeHost(h_end);
    return rc;
  }
  // pat->slab_elem_end for the node slabs B (once per pattern): prefix
  // maximum over the slabs of the last element in each node's list.
  static int slab_elements(llf_ctx *ctx, llf_pattern *pat, const int64_t *B) {
    if ((int)pat->slab_elem_end.size() == NSLAB) return LLF_OK;
    int64_t *d_B = nullptr, *d_max = nullptr;
    LLF_CUDA_TRY(ctx, dalloc(ctx, &d_B, NSLAB + 1));
    LLF_CUDA_TRY(ctx, dalloc(ctx, &d_max, NSLAB));
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(d_B, B, sizeof(int64_t) * (NSLAB + 1), cudaMemcpyHostToDevice, ctx->stream));
    LLF_CUDA_TRY(ctx, cudaMemsetAsync(d_max, 0, sizeof(int64_t) * NSLAB, ctx->stream));
    k_slab_last_elem<<<grid_1d(pat->mesh->non, 256, ctx->num_sms), 256, 0, ctx->stream>>>(
        pat->d_n2e_ptr, pat->d_n2e, pat->mesh->non, d_B, NSLAB, d_max);
    std::vector<int64_t> h(NSLAB);
    LLF_CUDA_TRY(ctx, cudaMemcpyAsync(h.data(), d_max, sizeof(int64_t) * NSLAB, cudaMemcpyDeviceToHost,
                                      ctx->stream));
    LLF_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    dfree(ctx, d_B);
    dfree(ctx, d_max);
    for (int k = 1; k < NSLAB; ++k) h[k] = std::max(h[k], h[k - 1]);
    pat->slab_elem_end = h;
    return LLF_OK;
  }
  int gather(llf_ctx *ctx, llf_pattern *pat, const double *Kf, int64_t cs, bool blockval,
             const ElemLauncher &elems) override {
    return run<double>(ctx, pat, Kf, cs, blockval, elems);
  }
  int gather(llf_ctx *ctx, llf_pattern *pat, const float *Kf, int64_t cs, bool blockval,
             const ElemLauncher &elems) override {
    return run<float>(ctx, pat, Kf, cs, blockval, elems);
  }
};

}  // namespace

int assemble_to_host_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int kind, const double *c1,
                          const double *c2, int nmat, int form, int64_t capacity, int64_t *colptr,
                          int64_t *rowval, double *nzval, int64_t *nnz, unsigned *keep, int *keep_changed) {
  HostSlabSink sink;
  sink.capacity = capacity;
  sink.h_colptr = colptr;
  sink.h_rowval = rowval;
  sink.h_nzval = nzval;
  sink.h_keep = keep;
  if (keep_changed) *keep_changed = 1;
  llf_matrix scratch;
  scratch.pat = pat;
  int rc = assemble_impl(ctx, mesh, pat, kind, LLF_SOLID, c1, c2, nmat, form, 0, &scratch, nullptr, &sink);
  if (rc == LLF_OK) *nnz = sink.nnz;
  if (rc == LLF_OK && keep_changed) *keep_changed = sink.keep_changed;
  return rc;
}
