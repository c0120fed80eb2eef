// Total Lagrangian operators: material tangent (materialTangentMatrix,
// src/nonlinear.jl:2083-2268), initial-stress (geometric) stiffness
// (initialStressMatrix, :2417-2595) and internal force (internalForceVector,
// :2738-2910), with the hyperelastic laws in closed form (the reference
// differentiates psi with Tensors.jl, ext/LowLevelFEMTensorsExt.jl:9-60).
//
// One CTA per element at a time.  Phase A (threads over integration points):
// Jacobian inverse, weight, interpolated F (or S, C), law -> PK2 stress S and
// 6x6 Voigt tangent D, all kept in shared memory.  Phase B (per point):
// physical gradients g, B(F) (6x3 per node) and T = w D B staged for all
// nodes, then every thread accumulates the 3x3 blocks of its node pairs
// (upper triangle; pairs processed in tiles of PPT per thread so the
// accumulators stay in registers).  Blocks go to the same pair buffer and
// element-ordered gather as the linear operators.
// Arithmetic contract: identical, operation by operation, to the oracle's
// TL restatement (intrinsics only; ln by the atanh series of the oracle).
#include "common.cuh"

namespace {

constexpr int TL_THREADS = 128;
constexpr int QD = 64;  // per-point record: wq, invJ[9], F or S [9], D[36], S[9] (tangent)
enum { TL_KMAT = 0, TL_KGEO_S = 1, TL_KGEO_C = 2, TL_KTAN = 3 };

struct TLArgs {
  const double *xyz;
  const int32_t *conn;
  const int32_t *emat;
  int64_t nel;
  int npe, nip, npairs;
  const double *w, *N, *dN;
  const double *T;  // elementwise nodal tensors, 9*npe per element
  int law;
  double prm[36];
  double *out;      // pair blocks (matrices) or element vectors (force)
  unsigned *status;
};

__device__ __constant__ int VI[6] = {0, 1, 2, 1, 0, 0};
__device__ __constant__ int VJ[6] = {0, 1, 2, 2, 2, 1};

__device__ double tl_ln(double x) {
  int e;
  double m = frexp(x, &e);
  if (m < 0.70710678118654752440) {
    m = __dmul_rn(m, 2.0);
    e = e - 1;
  }
  double s = __ddiv_rn(__dsub_rn(m, 1.0), __dadd_rn(m, 1.0));
  double s2 = __dmul_rn(s, s);
  double p = __ddiv_rn(1.0, 25.0);
  for (int k = 11; k >= 0; --k) p = __fma_rn(p, s2, __ddiv_rn(1.0, __dadd_rn(__dmul_rn(2.0, (double)k), 1.0)));
  return __fma_rn((double)e, 0.69314718055994530942, __dmul_rn(2.0, __dmul_rn(s, p)));
}

// S (3x3) and D (6x6 row-major) from C; false if det C <= 0.
__device__ bool tl_law(int law, const double *prm, const double C[3][3], double S[3][3], double *D) {
  if (law == LLF_LAW_CONSTANT_C) {
    for (int a = 0; a < 6; ++a)
      for (int b = 0; b < 6; ++b) D[a * 6 + b] = prm[b * 6 + a];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) S[i][j] = 0.0;
    return true;
  }
  const double mu = prm[0], lam = prm[1];
  if (law == LLF_LAW_SVK) {
    double E[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) E[i][j] = __dmul_rn(0.5, __dsub_rn(C[i][j], i == j ? 1.0 : 0.0));
    double trE = __dadd_rn(__dadd_rn(E[0][0], E[1][1]), E[2][2]);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) S[i][j] = __fma_rn(lam, i == j ? trE : 0.0, __dmul_rn(__dmul_rn(2.0, mu), E[i][j]));
    for (int a = 0; a < 6; ++a)
      for (int b = 0; b < 6; ++b) {
        int I = VI[a], J = VJ[a], K = VI[b], L = VJ[b];
        double v = __dmul_rn(lam, (I == J && K == L) ? 1.0 : 0.0);
        v = __dadd_rn(v, __dmul_rn(mu, __dadd_rn((I == K && J == L) ? 1.0 : 0.0, (I == L && J == K) ? 1.0 : 0.0)));
        D[a * 6 + b] = v;
      }
    return true;
  }
  double c00 = __dsub_rn(__dmul_rn(C[1][1], C[2][2]), __dmul_rn(C[1][2], C[2][1]));
  double c01 = -__dsub_rn(__dmul_rn(C[1][0], C[2][2]), __dmul_rn(C[1][2], C[2][0]));
  double c02 = __dsub_rn(__dmul_rn(C[1][0], C[2][1]), __dmul_rn(C[1][1], C[2][0]));
  double c10 = -__dsub_rn(__dmul_rn(C[0][1], C[2][2]), __dmul_rn(C[0][2], C[2][1]));
  double c11 = __dsub_rn(__dmul_rn(C[0][0], C[2][2]), __dmul_rn(C[0][2], C[2][0]));
  double c12 = -__dsub_rn(__dmul_rn(C[0][0], C[2][1]), __dmul_rn(C[0][1], C[2][0]));
  double c20 = __dsub_rn(__dmul_rn(C[0][1], C[1][2]), __dmul_rn(C[0][2], C[1][1]));
  double c21 = -__dsub_rn(__dmul_rn(C[0][0], C[1][2]), __dmul_rn(C[0][2], C[1][0]));
  double c22 = __dsub_rn(__dmul_rn(C[0][0], C[1][1]), __dmul_rn(C[0][1], C[1][0]));
  double det = __dadd_rn(__dadd_rn(__dmul_rn(C[0][0], c00), __dmul_rn(C[0][1], c01)), __dmul_rn(C[0][2], c02));
  if (!(det > 0.0)) return false;
  double r = __drcp_rn(det);
  double Ci[3][3] = {{__dmul_rn(c00, r), __dmul_rn(c10, r), __dmul_rn(c20, r)},
                     {__dmul_rn(c01, r), __dmul_rn(c11, r), __dmul_rn(c21, r)},
                     {__dmul_rn(c02, r), __dmul_rn(c12, r), __dmul_rn(c22, r)}};
  double lnJ = __dmul_rn(0.5, tl_ln(det));
  double t = __dmul_rn(lam, lnJ);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      S[i][j] = __fma_rn(t, Ci[i][j], __dmul_rn(mu, __dsub_rn(i == j ? 1.0 : 0.0, Ci[i][j])));
  double m2 = __dsub_rn(mu, t);
  for (int a = 0; a < 6; ++a)
    for (int b = 0; b < 6; ++b) {
      int I = VI[a], J = VJ[a], K = VI[b], L = VJ[b];
      double sym = __dadd_rn(__dmul_rn(Ci[I][K], Ci[J][L]), __dmul_rn(Ci[I][L], Ci[J][K]));
      D[a * 6 + b] = __fma_rn(lam, __dmul_rn(Ci[I][J], Ci[K][L]), __dmul_rn(m2, sym));
    }
  return true;
}

__device__ __forceinline__ int pair_off(int a, int npe) { return a * npe - (a * (a - 1)) / 2; }
__device__ __forceinline__ void pair_dec(int pi, int npe, int &a, int &b) {
  int lo = 0, hi = npe - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (pair_off(mid, npe) <= pi) lo = mid; else hi = mid - 1;
  }
  a = lo;
  b = a + (pi - pair_off(a, npe));
}

// Phase A for one point: wq, invJ, and the tensors the mode needs.
// Layout of rec: [0] wq, [1..9] invJ, [10..18] F (KMAT) or S, [19..54] D.
__device__ void tl_point(const TLArgs &A, int mode, int q, const double *sX, const double *sT,
                         double *rec) {
  const int npe = A.npe;
  const double *dNq = A.dN + (size_t)q * npe * 3;
  double J[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double acc = 0.0;
      for (int a = 0; a < npe; ++a) acc = __fma_rn(sX[a * 3 + i], __ldg(dNq + a * 3 + j), acc);
      J[i][j] = acc;
    }
  double c00 = __dsub_rn(__dmul_rn(J[1][1], J[2][2]), __dmul_rn(J[1][2], J[2][1]));
  double c01 = -__dsub_rn(__dmul_rn(J[1][0], J[2][2]), __dmul_rn(J[1][2], J[2][0]));
  double c02 = __dsub_rn(__dmul_rn(J[1][0], J[2][1]), __dmul_rn(J[1][1], J[2][0]));
  double c10 = -__dsub_rn(__dmul_rn(J[0][1], J[2][2]), __dmul_rn(J[0][2], J[2][1]));
  double c11 = __dsub_rn(__dmul_rn(J[0][0], J[2][2]), __dmul_rn(J[0][2], J[2][0]));
  double c12 = -__dsub_rn(__dmul_rn(J[0][0], J[2][1]), __dmul_rn(J[0][1], J[2][0]));
  double c20 = __dsub_rn(__dmul_rn(J[0][1], J[1][2]), __dmul_rn(J[0][2], J[1][1]));
  double c21 = -__dsub_rn(__dmul_rn(J[0][0], J[1][2]), __dmul_rn(J[0][2], J[1][0]));
  double c22 = __dsub_rn(__dmul_rn(J[0][0], J[1][1]), __dmul_rn(J[0][1], J[1][0]));
  double det = __dadd_rn(__dadd_rn(__dmul_rn(J[0][0], c00), __dmul_rn(J[0][1], c01)), __dmul_rn(J[0][2], c02));
  if (!(det > 0.0)) atomicOr(A.status, ST_BAD_JACOBIAN);
  double r = __drcp_rn(det);
  rec[0] = __dmul_rn(det, __ldg(A.w + q));
  rec[1] = __dmul_rn(c00, r); rec[2] = __dmul_rn(c10, r); rec[3] = __dmul_rn(c20, r);
  rec[4] = __dmul_rn(c01, r); rec[5] = __dmul_rn(c11, r); rec[6] = __dmul_rn(c21, r);
  rec[7] = __dmul_rn(c02, r); rec[8] = __dmul_rn(c12, r); rec[9] = __dmul_rn(c22, r);
  // interpolated nodal tensor (column-major per node)
  const double *Nq = A.N + (size_t)q * npe;
  double Tq[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double acc = 0.0;
      for (int a = 0; a < npe; ++a) acc = __fma_rn(__ldg(Nq + a), sT[9 * a + 3 * j + i], acc);
      Tq[i][j] = acc;
    }
  if (mode == TL_KGEO_S) {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) rec[10 + 3 * i + j] = Tq[i][j];
    return;
  }
  double C[3][3];
  if (mode == TL_KMAT || mode == TL_KTAN) {
    for (int I = 0; I < 3; ++I)
      for (int J2 = 0; J2 < 3; ++J2) {
        double acc = 0.0;
        for (int k = 0; k < 3; ++k) acc = __fma_rn(Tq[k][I], Tq[k][J2], acc);
        C[I][J2] = acc;
      }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) rec[10 + 3 * i + j] = Tq[i][j];  // F
  } else {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) C[i][j] = Tq[i][j];
  }
  double S[3][3];
  if (!tl_law(A.law, A.prm, C, S, rec + 19)) atomicOr(A.status, ST_NONFINITE);
  if (mode == TL_KGEO_C)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) rec[10 + 3 * i + j] = S[i][j];
  if (mode == TL_KTAN)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) rec[55 + 3 * i + j] = S[i][j];
}

template <int MODE, int PPT>
__global__ void __launch_bounds__(TL_THREADS) k_tl_matrix(TLArgs A) {
  extern __shared__ double sm[];
  const int npe = A.npe, nip = A.nip;
  double *sX = sm;                         // npe*3
  double *sT = sX + npe * 3;               // npe*9
  double *qd = sT + npe * 9;               // nip*QD
  double *sG = qd + (size_t)nip * QD;      // npe*3
  double *sB = sG + npe * 3;               // npe*18
  double *sTb = sB + npe * 18;             // npe*18 (KMAT)
  constexpr bool MAT = (MODE == TL_KMAT || MODE == TL_KTAN);
  constexpr int BS = MAT ? 9 : 1;
  for (int64_t e = blockIdx.x; e < A.nel; e += gridDim.x) {
    if (A.emat && A.emat[e] < 0) continue;
    for (int t = threadIdx.x; t < npe * 3; t += blockDim.x)
      sX[t] = A.xyz[(size_t)A.conn[e * npe + t / 3] * 3 + t % 3];
    for (int t = threadIdx.x; t < npe * 9; t += blockDim.x) sT[t] = A.T[(size_t)e * npe * 9 + t];
    __syncthreads();
    for (int q = threadIdx.x; q < nip; q += blockDim.x) tl_point(A, MODE, q, sX, sT, qd + (size_t)q * QD);
    __syncthreads();
    double *Ke = A.out + (size_t)e * npe * npe * BS;  // [column node][row node][block]
    const int tile = blockDim.x * PPT;
    for (int p0 = 0; p0 < A.npairs; p0 += tile) {
      double acc[PPT][BS];
#pragma unroll
      for (int k = 0; k < PPT; ++k)
#pragma unroll
        for (int m = 0; m < BS; ++m) acc[k][m] = 0.0;
      for (int q = 0; q < nip; ++q) {
        const double *rec = qd + (size_t)q * QD;
        // physical gradients of all nodes at q
        for (int t = threadIdx.x; t < npe * 3; t += blockDim.x) {
          int a = t / 3, i = t % 3;
          const double *d = A.dN + ((size_t)q * npe + a) * 3;
          double s = 0.0;
          for (int j = 0; j < 3; ++j) s = __fma_rn(rec[1 + 3 * j + i], __ldg(d + j), s);
          sG[t] = s;
        }
        __syncthreads();
        if (MAT) {
          // B(F) per node (src/nonlinear.jl:2219-2242)
          for (int t = threadIdx.x; t < npe * 3; t += blockDim.x) {
            int b = t / 3, j = t % 3;
            const double *F = rec + 10;  // F[j][k] at 10 + 3j + k
            double v1 = F[3 * j + 0], v2 = F[3 * j + 1], v3 = F[3 * j + 2];
            const double *g = sG + 3 * b;
            double *Bb = sB + b * 18;
            Bb[0 * 3 + j] = __dmul_rn(v1, g[0]);
            Bb[1 * 3 + j] = __dmul_rn(v2, g[1]);
            Bb[2 * 3 + j] = __dmul_rn(v3, g[2]);
            Bb[3 * 3 + j] = __dadd_rn(__dmul_rn(v2, g[2]), __dmul_rn(v3, g[1]));
            Bb[4 * 3 + j] = __dadd_rn(__dmul_rn(v1, g[2]), __dmul_rn(v3, g[0]));
            Bb[5 * 3 + j] = __dadd_rn(__dmul_rn(v1, g[1]), __dmul_rn(v2, g[0]));
          }
          __syncthreads();
          const double *D = rec + 19;
          const double wq = rec[0];
          for (int t = threadIdx.x; t < npe * 18; t += blockDim.x) {
            int b = t / 18, I = (t % 18) / 3, j = t % 3;
            double s = 0.0;
            for (int J2 = 0; J2 < 6; ++J2) s = __fma_rn(D[I * 6 + J2], sB[b * 18 + J2 * 3 + j], s);
            sTb[t] = __dmul_rn(s, wq);
          }
          __syncthreads();
        }
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
          const int pi = p0 + k * blockDim.x + threadIdx.x;
          if (pi >= A.npairs) continue;
          int a, b;
          pair_dec(pi, npe, a, b);
          if (MAT) {
            const double *Ba = sB + a * 18, *Tb = sTb + b * 18;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
              for (int j = 0; j < 3; ++j) {
                if (a == b && j < i) continue;
                double s = acc[k][i * 3 + j];
#pragma unroll
                for (int I = 0; I < 6; ++I) s = __fma_rn(Ba[I * 3 + i], Tb[I * 3 + j], s);
                acc[k][i * 3 + j] = s;
              }
            if (MODE == TL_KTAN) {  // consistent tangent: geometric part from the same S
              const double *S = rec + 55, *ga = sG + 3 * a, *gb = sG + 3 * b;
              double tv[3];
#pragma unroll
              for (int I = 0; I < 3; ++I) {
                double s = 0.0;
#pragma unroll
                for (int J2 = 0; J2 < 3; ++J2) s = __fma_rn(S[3 * I + J2], gb[J2], s);
                tv[I] = s;
              }
              double v = 0.0;
#pragma unroll
              for (int I = 0; I < 3; ++I) v = __fma_rn(ga[I], tv[I], v);
#pragma unroll
              for (int i = 0; i < 3; ++i) acc[k][i * 3 + i] = __fma_rn(v, rec[0], acc[k][i * 3 + i]);
            }
          } else {
            const double *S = rec + 10, *ga = sG + 3 * a, *gb = sG + 3 * b;
            double tv[3];
#pragma unroll
            for (int I = 0; I < 3; ++I) {
              double s = 0.0;
#pragma unroll
              for (int J2 = 0; J2 < 3; ++J2) s = __fma_rn(S[3 * I + J2], gb[J2], s);
              tv[I] = s;
            }
            double v = 0.0;
#pragma unroll
            for (int I = 0; I < 3; ++I) v = __fma_rn(ga[I], tv[I], v);
            acc[k][0] = __fma_rn(v, rec[0], acc[k][0]);
          }
        }
        __syncthreads();
      }
#pragma unroll
      for (int k = 0; k < PPT; ++k) {
        const int pi = p0 + k * blockDim.x + threadIdx.x;
        if (pi >= A.npairs) continue;
        int a, b;
        pair_dec(pi, npe, a, b);
        double *ab = Ke + ((size_t)b * npe + a) * BS;   // block (a,b)
        double *ba = Ke + ((size_t)a * npe + b) * BS;   // mirror (b,a)
        if (MAT) {
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              const double v = (a == b && j < i) ? acc[k][j * 3 + i] : acc[k][i * 3 + j];
              ab[i * 3 + j] = v;
              if (a != b) ba[j * 3 + i] = v;
            }
        } else {
          ab[0] = acc[k][0];
          if (a != b) ba[0] = acc[k][0];
        }
      }
    }
    __syncthreads();
  }
}

// Internal force: element vectors fe[e][a][i].
template <int MODE>  // 0: T = F with law, 1: T = P
__global__ void __launch_bounds__(TL_THREADS) k_tl_force(TLArgs A) {
  extern __shared__ double sm[];
  const int npe = A.npe, nip = A.nip;
  double *sX = sm;
  double *sT = sX + npe * 3;
  double *qd = sT + npe * 9;  // per point: wq, invJ[9], P[9]
  for (int64_t e = blockIdx.x; e < A.nel; e += gridDim.x) {
    for (int t = threadIdx.x; t < npe * 3; t += blockDim.x)
      sX[t] = A.xyz[(size_t)A.conn[e * npe + t / 3] * 3 + t % 3];
    for (int t = threadIdx.x; t < npe * 9; t += blockDim.x) sT[t] = A.T[(size_t)e * npe * 9 + t];
    __syncthreads();
    for (int q = threadIdx.x; q < nip; q += blockDim.x) {
      double *rec = qd + (size_t)q * QD;
      tl_point(A, MODE == 0 ? TL_KMAT : TL_KGEO_S, q, sX, sT, rec);
      // rec[10..18] holds F (MODE 0) or the interpolated P (MODE 1)
      if (MODE == 0) {
        double F[3][3], C[3][3], S[3][3], D[36];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) F[i][j] = rec[10 + 3 * i + j];
        for (int I = 0; I < 3; ++I)
          for (int J2 = 0; J2 < 3; ++J2) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k) acc = __fma_rn(F[k][I], F[k][J2], acc);
            C[I][J2] = acc;
          }
        if (!tl_law(A.law, A.prm, C, S, D)) atomicOr(A.status, ST_NONFINITE);
        for (int i = 0; i < 3; ++i)
          for (int J2 = 0; J2 < 3; ++J2) {
            double s = 0.0;
            for (int K = 0; K < 3; ++K) s = __fma_rn(F[i][K], S[K][J2], s);
            rec[10 + 3 * i + J2] = s;  // P
          }
      }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < npe * 3; t += blockDim.x) {
      const int a = t / 3, i = t % 3;
      double fe = 0.0;
      for (int q = 0; q < nip; ++q) {
        const double *rec = qd + (size_t)q * QD;
        const double *d = A.dN + ((size_t)q * npe + a) * 3;
        double g[3];
        for (int c = 0; c < 3; ++c) {
          double s = 0.0;
          for (int j = 0; j < 3; ++j) s = __fma_rn(rec[1 + 3 * j + c], __ldg(d + j), s);
          g[c] = s;
        }
        double v = 0.0;
        for (int J2 = 0; J2 < 3; ++J2) v = __fma_rn(rec[10 + 3 * i + J2], g[J2], v);
        fe = __fma_rn(v, rec[0], fe);
      }
      A.out[(size_t)e * npe * 3 + t] = fe;
    }
    __syncthreads();
  }
}

size_t tl_smem(int npe, int nip, bool matrix) {
  size_t d = (size_t)npe * 3 + (size_t)npe * 9 + (size_t)nip * QD;
  if (matrix) d += (size_t)npe * 3 + (size_t)npe * 18 * 2;
  return d * sizeof(double);
}

int fill_args(llf_ctx *ctx, llf_mesh *mesh, const double *T, int law, const double *params,
              int nparams, TLArgs &a) {
  a.xyz = mesh->d_xyz;
  a.conn = mesh->d_conn;
  a.emat = mesh->d_emat;
  a.nel = mesh->nel;
  a.npe = mesh->npe;
  a.nip = mesh->nip;
  a.npairs = mesh->npe * (mesh->npe + 1) / 2;
  a.w = mesh->d_w;
  a.N = mesh->d_N;
  a.dN = mesh->d_dN;
  a.T = T;
  a.law = law;
  a.status = ctx->d_status;
  for (int i = 0; i < 36; ++i) a.prm[i] = 0.0;
  if (law == LLF_LAW_CONSTANT_C) {
    if (nparams != 36 || !params) return llf_fail(ctx, LLF_ERR_ARG, "constant tangent needs 36 parameters (6x6)");
  } else if (law == LLF_LAW_NEOHOOKE_COMP || law == LLF_LAW_SVK) {
    if (nparams < 2 || !params) return llf_fail(ctx, LLF_ERR_ARG, "law needs parameters (mu, lambda)");
  } else {
    return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "unknown hyperelastic law");
  }
  for (int i = 0; i < nparams && i < 36; ++i) a.prm[i] = params[i];
  return LLF_OK;
}

template <int MODE>
int launch_matrix(llf_ctx *ctx, TLArgs a, size_t smem) {
  int ppt = (a.npairs + TL_THREADS - 1) / TL_THREADS;
  ppt = ppt <= 1 ? 1 : (ppt <= 2 ? 2 : 4);
  int per_sm = 1;
  auto pick = [&](auto fn) -> int {
    if (smem > 48 * 1024)
      LLF_CUDA_TRY(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    LLF_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, TL_THREADS, smem));
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)ctx->num_sms * per_sm;
    if (grid > a.nel) grid = a.nel > 0 ? a.nel : 1;
    KernelScope ks(ctx, MODE == TL_KMAT ? "k_tl_material" : (MODE == TL_KTAN ? "k_tl_tangent" : "k_tl_geometric"));
    fn<<<(unsigned)grid, TL_THREADS, smem, ctx->stream>>>(a);
    LLF_CUDA_TRY(ctx, cudaGetLastError());
    return LLF_OK;
  };
  if (ppt == 1) return pick(k_tl_matrix<MODE, 1>);
  if (ppt == 2) return pick(k_tl_matrix<MODE, 2>);
  return pick(k_tl_matrix<MODE, 4>);
}

int tl_matrix(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int mode, const double *dT, int law,
              const double *params, int nparams, llf_matrix *m) {
  if (mesh->dim != 3 || pat->pdim != 3)
    return llf_fail(ctx, LLF_ERR_ARG, "Total Lagrangian operators need dim == 3 and pdim == 3");
  TLArgs a{};
  int rc = fill_args(ctx, mesh, dT, law, params, nparams, a);
  if (rc) return rc;
  size_t smem = tl_smem(mesh->npe, mesh->nip, true);
  if (smem > 200 * 1024) return llf_fail(ctx, LLF_ERR_LIMIT, "element too large for the TL kernels");
  const bool mat = (mode == TL_KMAT || mode == TL_KTAN);
  const int BS = mat ? 9 : 1;
  double *Kp = nullptr;
  int64_t *cnt = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &Kp, (size_t)mesh->nel * mesh->npe * mesh->npe * BS));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &cnt, pat->ndof + 1));
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(cnt, 0, sizeof(int64_t) * (pat->ndof + 1), ctx->stream));
  a.out = Kp;
  rc = (mode == TL_KMAT) ? launch_matrix<TL_KMAT>(ctx, a, smem)
       : (mode == TL_KTAN) ? launch_matrix<TL_KTAN>(ctx, a, smem)
       : (mode == TL_KGEO_S ? launch_matrix<TL_KGEO_S>(ctx, a, smem) : launch_matrix<TL_KGEO_C>(ctx, a, smem));
  if (rc == LLF_OK) {
    cudaError_t e = dalloc(ctx, &m->d_nz, pat->nnz);
    rc = (e == cudaSuccess) ? gather_full(ctx, pat, Kp, (int64_t)mesh->npe * BS, mat, m->d_nz, cnt)
                            : llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
  }
  dfree(ctx, Kp);
  if (rc == LLF_OK) rc = llf_check_status(ctx, mat ? "materialTangentMatrix" : "initialStressMatrix");
  if (rc == LLF_OK) rc = matrix_finalize(ctx, m, cnt);
  dfree(ctx, cnt);
  return rc;
}

}  // namespace

int tl_material_tangent_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, const double *d_F,
                             int law, const double *params, int nparams, llf_matrix *m) {
  return tl_matrix(ctx, mesh, pat, TL_KMAT, d_F, law, params, nparams, m);
}

int tl_tangent_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, const double *d_F, int law,
                    const double *params, int nparams, llf_matrix *m) {
  return tl_matrix(ctx, mesh, pat, TL_KTAN, d_F, law, params, nparams, m);
}

int tl_initial_stress_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, const double *d_S,
                           const double *d_C, int law, const double *params, int nparams,
                           llf_matrix *m) {
  if (d_S) {
    double dummy[2] = {0.0, 0.0};
    return tl_matrix(ctx, mesh, pat, TL_KGEO_S, d_S, LLF_LAW_NEOHOOKE_COMP, dummy, 2, m);
  }
  return tl_matrix(ctx, mesh, pat, TL_KGEO_C, d_C, law, params, nparams, m);
}

int tl_internal_force_impl(llf_ctx *ctx, llf_mesh *mesh, const double *d_P, const double *d_F,
                           int law, const double *params, int nparams, double *d_f) {
  TLArgs a{};
  int rc;
  if (d_P) {
    double dummy[2] = {0.0, 0.0};
    rc = fill_args(ctx, mesh, d_P, LLF_LAW_NEOHOOKE_COMP, dummy, 2, a);
  } else {
    rc = fill_args(ctx, mesh, d_F, law, params, nparams, a);
  }
  if (rc) return rc;
  size_t smem = tl_smem(mesh->npe, mesh->nip, false);
  double *fe = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &fe, (size_t)mesh->nel * mesh->npe * 3));
  a.out = fe;
  auto go = [&](auto fn) -> int {
    if (smem > 48 * 1024)
      LLF_CUDA_TRY(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 1;
    LLF_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, TL_THREADS, smem));
    int64_t grid = (int64_t)ctx->num_sms * (per_sm < 1 ? 1 : per_sm);
    if (grid > a.nel) grid = a.nel > 0 ? a.nel : 1;
    KernelScope ks(ctx, "k_tl_force");
    fn<<<(unsigned)grid, TL_THREADS, smem, ctx->stream>>>(a);
    LLF_CUDA_TRY(ctx, cudaGetLastError());
    return LLF_OK;
  };
  rc = d_P ? go(k_tl_force<1>) : go(k_tl_force<0>);
  if (rc == LLF_OK) {
    LLF_CUDA_TRY(ctx, cudaMemsetAsync(d_f, 0, sizeof(double) * 3 * mesh->non, ctx->stream));
    rc = node_gather(ctx, mesh->d_conn, mesh->nel, mesh->npe, mesh->non, 3, fe, d_f);
  }
  dfree(ctx, fe);
  if (rc) return rc;
  return llf_check_status(ctx, "internalForceVector");
}
