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

// ------------------------------------------------------------ tensor-core form
// Consistent tangent on the 5th-generation tensor cores (tcgen05), for
// high-order elements where the element contraction is dense.  Per point q
// the tangent is [B_q; G_q]^T diag(w D_q, w S_q (x) I) [B_q; G_q], with B_q
// the 6 x 3npe matrix B(F) and G_q the 9 x 3npe displacement-gradient
// operator, so the whole element matrix is one GEMM over K = 15 rows per
// point.  One CTA computes a 128 x 192 tile of one element matrix:
//   - the point data (F, w D, w S, physical gradients; FP64 as in the FP64
//     form, rounded to FP32) come from k_tl_points_tc, two points per
//     k-block, fetched by cp.async.bulk one k-block ahead;
//   - per k-block of 2 points (2 x 15 rows, padded to 32) the threads build
//     the A (= [B; G] rows of the tile) and B (= weighted [D B; S G]) tiles
//     in shared memory in the K-major core-matrix layout (8 rows x 16 bytes),
//     each split into TF32 hi and lo parts;
//   - one thread issues tcgen05.mma kind::tf32 (M 128, N 192, K 8) for the
//     three split products hi*hi + hi*lo + lo*hi into an FP32 accumulator in
//     tensor memory and commits to the stage's mbarrier (two stages, the
//     next k-block is built while the tensor cores run);
//   - the epilogue reads the accumulator with tcgen05.ld and writes the
//     element matrix (FP32) in the gather's layout.
// Every mbarrier wait is bounded (2 s): a timeout sets ST_TIMEOUT, the CTA
// skips its epilogue and releases its tensor memory.
constexpr int TC_M = 128, TC_N = 192, TC_KB = 32, TC_PTS = 2, TC_THREADS = 512;
constexpr int TC_TILE_A = TC_M * TC_KB, TC_TILE_B = TC_N * TC_KB;  // floats
constexpr size_t TC_STAGE = (size_t)2 * (TC_TILE_A + TC_TILE_B);   // floats per stage (hi + lo)

struct TcArgs {
  const float *pd;     // nel * nip * tc_pstride(npe) packed point data (k_tl_points_tc)
  const int32_t *emat;
  int64_t nel;
  int npe, nip, n, nstrip, nhalf;
  float *Kf;           // nel * npe * cs
  int64_t cs;
  unsigned *status;
};

__device__ __forceinline__ uint32_t tc_saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, K-major, no swizzle: core matrices of
// 8 rows x 16 bytes, LBO = distance of K-adjacent core matrices (128 B),
// SBO = distance of 8-row groups (TC_KB / 4 core matrices of 128 B).
__device__ __forceinline__ uint64_t tc_desc(const float *p) {
  const uint64_t lbo = 128, sbo = (TC_KB / 4) * 128;
  return (uint64_t)((tc_saddr(p) & 0x3FFFF) >> 4) | ((lbo >> 4) << 16) | ((sbo >> 4) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ int tc_off(int row, int k) {
  return ((row >> 3) * (TC_KB / 4) + (k >> 2)) * 32 + (row & 7) * 4 + (k & 3);
}

__device__ __forceinline__ float tc_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// Row `row`, columns k0 .. k0+15 (k0 a multiple of 4) of a tile: TF32 hi and
// lo parts, one 16-byte store per 4 columns (a core-matrix row).
__device__ __forceinline__ void tc_put16(float *hi, float *lo, int row, int k0, const float *v) {
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float4 h, l;
    h.x = tc_tf32(v[4 * c]);
    h.y = tc_tf32(v[4 * c + 1]);
    h.z = tc_tf32(v[4 * c + 2]);
    h.w = tc_tf32(v[4 * c + 3]);
    l.x = v[4 * c] - h.x;
    l.y = v[4 * c + 1] - h.y;
    l.z = v[4 * c + 2] - h.z;
    l.w = v[4 * c + 3] - h.w;
    const int o = tc_off(row, k0 + 4 * c);
    *reinterpret_cast<float4 *>(hi + o) = h;
    *reinterpret_cast<float4 *>(lo + o) = l;
  }
}

__device__ __forceinline__ uint64_t tc_now() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait on an mbarrier phase (2 s); false on timeout.
__device__ __forceinline__ bool tc_wait(uint64_t *bar, unsigned parity) {
  const uint64_t t0 = tc_now();
  for (;;) {
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(tc_saddr(bar)), "r"(parity) : "memory");
    if (ok) return true;
    if (tc_now() - t0 > 2000000000ull) return false;
  }
}

// Packed FP32 point data of the tensor-core form, one CTA per element: for
// every point q a run of tc_pstride(npe) floats (16-byte multiple)
//   [0,9) F | [9,45) w D | [45,54) w S | [54,56) 0 | [56, 56+3 npe) grad N_a
// computed in FP64 (the FP64 form's point record and gradients) and rounded.
__host__ __device__ __forceinline__ int tc_pstride(int npe) { return (56 + 3 * npe + 3) & ~3; }

__global__ void __launch_bounds__(TL_THREADS) k_tl_points_tc(TLArgs A, float *pd) {
  extern __shared__ double sm[];
  const int npe = A.npe, nip = A.nip, ps = tc_pstride(npe);
  double *sX = sm, *sT = sX + npe * 3, *rec = sT + npe * 9;  // rec: nip * QD
  for (int64_t e = blockIdx.x; e < A.nel; e += gridDim.x) {
    if (A.emat && A.emat[e] < 0) continue;
    for (int t = threadIdx.x; t < npe * 3; t += blockDim.x)
      sX[t] = A.xyz[(size_t)A.conn[e * npe + t / 3] * 3 + t % 3];
    for (int t = threadIdx.x; t < npe * 9; t += blockDim.x) sT[t] = A.T[(size_t)e * npe * 9 + t];
    __syncthreads();
    for (int q = threadIdx.x; q < nip; q += blockDim.x) tl_point(A, TL_KTAN, q, sX, sT, rec + (size_t)q * QD);
    __syncthreads();
    float *out = pd + (size_t)e * nip * ps;
    for (int t = threadIdx.x; t < nip * ps; t += blockDim.x) {
      const int q = t / ps, f = t - q * ps;
      const double *r = rec + (size_t)q * QD;
      double v = 0.0;
      if (f < 9) v = r[10 + f];
      else if (f < 45) v = __dmul_rn(r[0], r[19 + (f - 9)]);
      else if (f < 54) v = __dmul_rn(r[0], r[55 + (f - 45)]);
      else if (f >= 56 && f < 56 + 3 * npe) {
        const int a = (f - 56) / 3, I = (f - 56) % 3;
        const double *d = A.dN + ((size_t)q * npe + a) * 3;
        double g = 0.0;
        for (int J = 0; J < 3; ++J) g = __fma_rn(r[1 + 3 * J + I], d[J], g);
        v = g;
      }
      out[t] = (float)v;
    }
    __syncthreads();
  }
}

__device__ __forceinline__ void tc_bulk(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc_saddr(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(tc_saddr(dst)), "l"(src), "r"(bytes), "r"(tc_saddr(bar))
               : "memory");
}

// Shared memory: 2 stages x (A hi, A lo, B hi, B lo) | 2 point-data buffers
// (TC_PTS points each, fetched by cp.async.bulk one k-block ahead) |
// (TC_N / (TC_THREADS / 128) must be a multiple of 16)
// mbarriers: MMA completion x2, point data x2 | tensor-memory address.
__global__ void __launch_bounds__(TC_THREADS, 1) k_tl_tangent_tc(TcArgs A) {
  extern __shared__ __align__(1024) float tsm[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int per_e = A.nstrip * A.nhalf;
  const int64_t e = blockIdx.x / per_e;
  const int rr = (int)(blockIdx.x - e * per_e);
  const int row0 = (rr / A.nhalf) * TC_M, col0 = (rr % A.nhalf) * TC_N;
  if (e >= A.nel || (A.emat && A.emat[e] < 0)) return;  // uniform across the CTA
  const int npe = A.npe, nip = A.nip, n = A.n, ps = tc_pstride(npe);
  float *pbuf = tsm + 2 * TC_STAGE;                      // 2 x TC_PTS * ps
  uint64_t *bar = (uint64_t *)(pbuf + 2 * TC_PTS * ps);  // [0,2) MMA, [2,4) point data
  uint32_t *tslot = (uint32_t *)(bar + 4);
  const float *pd = A.pd + (size_t)e * nip * ps;
  const int nkb = (nip + TC_PTS - 1) / TC_PTS;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_saddr(tslot)), "r"(256u)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int b = 0; b < 4; ++b)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_saddr(bar + b)), "r"(1u) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    const int np = nip < TC_PTS ? nip : TC_PTS;
    tc_bulk(pbuf, pd, (unsigned)(np * ps * sizeof(float)), bar + 2);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TC_N >> 3) << 17) |
                         ((uint32_t)(TC_M >> 4) << 24);
  bool ok = true;
  int fetched = 1;  // point-data copies issued (k-blocks 0 .. fetched-1)
  for (int kb = 0; kb < nkb; ++kb) {
    const int st = kb & 1;
    float *Ahi = tsm + st * TC_STAGE, *Alo = Ahi + TC_TILE_A, *Bhi = Alo + TC_TILE_A, *Blo = Bhi + TC_TILE_B;
    // tiles of this stage free (MMAs of k-block kb - 2 done) and point data of kb landed
    bool w = kb < 2 || tc_wait(bar + st, (unsigned)((kb - 2) >> 1) & 1u);
    w = w && tc_wait(bar + 2 + st, (unsigned)(kb >> 1) & 1u);
    if (!__syncthreads_and(w)) {
      ok = false;
      break;
    }
    // prefetch the next k-block's point data into the other buffer (its last
    // reader, the tile build of kb - 1, finished before the barrier above)
    if (kb + 1 < nkb) {
      if (tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const int q1 = (kb + 1) * TC_PTS, np = (nip - q1) < TC_PTS ? (nip - q1) : TC_PTS;
        tc_bulk(pbuf + ((kb + 1) & 1) * TC_PTS * ps, pd + (size_t)q1 * ps, (unsigned)(np * ps * sizeof(float)),
                bar + 2 + ((kb + 1) & 1));
      }
      ++fetched;
    }
    const int q0 = kb * TC_PTS;
    const float *pb = pbuf + st * TC_PTS * ps;
    // A tile: rows of the strip, K = (point, 16 rows: B(F) 6, grad 9, pad 1)
    for (int t = tid; t < TC_M * TC_PTS; t += TC_THREADS) {
      const int ql = t / TC_M, i = t - ql * TC_M, gi = row0 + i, q = q0 + ql;
      float v[16];
#pragma unroll
      for (int r = 0; r < 16; ++r) v[r] = 0.f;
      if (gi < n && q < nip) {
        const int a = gi / 3, ci = gi - 3 * (gi / 3);
        const float *P = pb + ql * ps, *g = P + 56 + 3 * a;
        const float v1 = P[3 * ci], v2 = P[3 * ci + 1], v3 = P[3 * ci + 2];
        v[0] = v1 * g[0];
        v[1] = v2 * g[1];
        v[2] = v3 * g[2];
        v[3] = fmaf(v2, g[2], v3 * g[1]);
        v[4] = fmaf(v1, g[2], v3 * g[0]);
        v[5] = fmaf(v1, g[1], v2 * g[0]);
#pragma unroll
        for (int I = 0; I < 3; ++I)
#pragma unroll
          for (int c = 0; c < 3; ++c) v[6 + 3 * I + c] = (c == ci) ? g[I] : 0.f;
      }
      tc_put16(Ahi, Alo, i, ql * 16, v);
    }
    // B tile: columns of the half, weighted by w D and w S
    for (int t = tid; t < TC_N * TC_PTS; t += TC_THREADS) {
      const int ql = t / TC_N, j = t - ql * TC_N, gj = col0 + j, q = q0 + ql;
      float v[16];
#pragma unroll
      for (int r = 0; r < 16; ++r) v[r] = 0.f;
      if (gj < n && q < nip) {
        const int b = gj / 3, cj = gj - 3 * (gj / 3);
        const float *P = pb + ql * ps, *g = P + 56 + 3 * b;
        const float v1 = P[3 * cj], v2 = P[3 * cj + 1], v3 = P[3 * cj + 2];
        float Bv[6];
        Bv[0] = v1 * g[0];
        Bv[1] = v2 * g[1];
        Bv[2] = v3 * g[2];
        Bv[3] = fmaf(v2, g[2], v3 * g[1]);
        Bv[4] = fmaf(v1, g[2], v3 * g[0]);
        Bv[5] = fmaf(v1, g[1], v2 * g[0]);
        const float *wD = P + 9, *wS = P + 45;
#pragma unroll
        for (int r = 0; r < 6; ++r) {
          float sacc = 0.f;
#pragma unroll
          for (int r2 = 0; r2 < 6; ++r2) sacc = fmaf(wD[r * 6 + r2], Bv[r2], sacc);
          v[r] = sacc;
        }
#pragma unroll
        for (int I = 0; I < 3; ++I) {
          float sacc = 0.f;
#pragma unroll
          for (int J = 0; J < 3; ++J) sacc = fmaf(wS[3 * I + J], g[J], sacc);
#pragma unroll
          for (int c = 0; c < 3; ++c) v[6 + 3 * I + c] = (c == cj) ? sacc : 0.f;
        }
      }
      tc_put16(Bhi, Blo, j, ql * 16, v);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int kk = 0; kk < TC_KB / 8; ++kk)
#pragma unroll
        for (int p = 0; p < 3; ++p) {
          const float *Ax = (p == 2 ? Alo : Ahi) + kk * 64, *Bx = (p == 1 ? Blo : Bhi) + kk * 64;
          const uint32_t acc = (kb | kk | p) != 0;
          asm volatile("{\n\t.reg .pred pa;\n\tsetp.ne.b32 pa, %4, 0;\n\t"
                       "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, pa;\n\t}"
                       ::"r"(tmem), "l"(tc_desc(Ax)), "l"(tc_desc(Bx)), "r"(idesc), "r"(acc)
                       : "memory");
        }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       tc_saddr(bar + st))
                   : "memory");
    }
  }
  // the last commit covers every earlier MMA of this thread
  const bool fin = ok ? tc_wait(bar + ((nkb - 1) & 1), (unsigned)((nkb - 1) >> 1) & 1u) : false;
  ok = __syncthreads_and(fin);
  if (!ok && tid == 0) atomicOr(A.status, ST_TIMEOUT);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    // warp w reads TMEM lanes 32 (w % 4) .. +31 (the lanes its position in a
    // warpgroup may access) and one of TC_THREADS / 128 column ranges
    constexpr int NCR = TC_THREADS / 128, CW = TC_N / NCR;
    const int lanes = (warp & 3) * 32, cbeg = (warp >> 2) * CW;
    const int gi = row0 + lanes + lane;
    const int a = gi / 3, ci = gi - 3 * (gi / 3);
    for (int c0 = cbeg; c0 < cbeg + CW; c0 += 16) {
      uint32_t r[16];
      const uint32_t addr = tmem + ((uint32_t)lanes << 16) + (uint32_t)c0;
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                   : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                     "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                     "=r"(r[15])
                   : "r"(addr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (gi < n)
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int gj = col0 + c0 + u;
          if (gj < n) {
            const int b = gj / 3, cj = gj - 3 * (gj / 3);
            A.Kf[((size_t)e * npe + b) * A.cs + a * kf_bstride(3, true, 4) + ci * 3 + cj] = __uint_as_float(r[u]);
          }
        }
    }
  } else {
    // drain this CTA's point-data copies (bounded) before it exits: copy k of
    // buffer k & 1 is that buffer's (k >> 1)-th phase
    for (int k = 0; k < fetched; ++k) tc_wait(bar + 2 + (k & 1), (unsigned)(k >> 1) & 1u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256u) : "memory");
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

// Tensor-core form of the consistent tangent (k_tl_points_tc + k_tl_tangent_tc,
// then the FP32 element matrices summed in FP64 by the gather).
namespace {
// Exact symmetry of the tensor-core element matrices: the tiles above and
// below the diagonal round their FP32 sums differently, so block (b,a) is
// not quite block (a,b)^T.  Each mirrored pair of entries is replaced by
// their mean, so the gathered tangent is symmetric bit for bit (CG relies
// on it; unsymmetric rounding cost it about twice the iterations).  One
// thread per element and node pair a <= b.
__global__ void k_tc_symmetrize(float *__restrict__ Kf, int64_t nel, int npe, int64_t cs) {
  constexpr int BSTR = kf_bstride(3, true, 4);
  const int64_t npairs = (int64_t)npe * (npe + 1) / 2;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nel * npairs;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / npairs;
    int p = (int)(t - e * npairs);
    int a = 0;
    while (p >= npe - a) {  // pair index -> (a, b >= a), row by row
      p -= npe - a;
      ++a;
    }
    const int b = a + p;
    float *X = Kf + ((size_t)e * npe + b) * cs + (size_t)a * BSTR;  // block (a, b)
    float *Y = Kf + ((size_t)e * npe + a) * cs + (size_t)b * BSTR;  // block (b, a)
#pragma unroll
    for (int ci = 0; ci < 3; ++ci)
#pragma unroll
      for (int cj = 0; cj < 3; ++cj) {
        if (a == b && cj <= ci) continue;
        const float m = (X[ci * 3 + cj] + Y[cj * 3 + ci]) * 0.5f;
        X[ci * 3 + cj] = m;
        Y[cj * 3 + ci] = m;
      }
  }
}
}  // namespace

int tl_tangent_tc_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, const double *d_F, int law,
                       const double *params, int nparams, llf_matrix *m) {
  if (mesh->dim != 3 || pat->pdim != 3)
    return llf_fail(ctx, LLF_ERR_ARG, "Total Lagrangian operators need dim == 3 and pdim == 3");
  TLArgs a{};
  int rc = fill_args(ctx, mesh, d_F, law, params, nparams, a);
  if (rc) return rc;
  const int npe = mesh->npe, nip = mesh->nip, n = 3 * npe;
  cudaStream_t s = ctx->stream;
  float *pd = nullptr;
  float *Kf = nullptr;
  int64_t *cnt = nullptr;
  const int ps = tc_pstride(npe);
  const int64_t cs = kf_colstride(npe, kf_bstride(3, true, (int)sizeof(float)), (int)sizeof(float));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &pd, (size_t)mesh->nel * nip * ps));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &Kf, (size_t)mesh->nel * npe * cs));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &cnt, pat->ndof + 1));
  LLF_CUDA_TRY(ctx, cudaMemsetAsync(cnt, 0, sizeof(int64_t) * (pat->ndof + 1), s));
  {
    const size_t smem = sizeof(double) * ((size_t)npe * 12 + (size_t)nip * QD);
    if (smem > 200 * 1024) rc = llf_fail(ctx, LLF_ERR_LIMIT, "tensor-core tangent: element too large");
    if (rc == LLF_OK && smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(k_tl_points_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
    }
    if (rc == LLF_OK) {
      const unsigned grid = (unsigned)std::min<int64_t>(std::max<int64_t>(mesh->nel, 1), (int64_t)ctx->num_sms * 4);
      KernelScope ks(ctx, "k_tl_points_tc");
      k_tl_points_tc<<<grid, TL_THREADS, smem, s>>>(a, pd);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
    }
  }
  TcArgs t{};
  t.pd = pd;
  t.emat = mesh->d_emat;
  t.nel = mesh->nel;
  t.npe = npe;
  t.nip = nip;
  t.n = n;
  t.nstrip = (n + TC_M - 1) / TC_M;
  t.nhalf = (n + TC_N - 1) / TC_N;
  t.Kf = Kf;
  t.cs = cs;
  t.status = ctx->d_status;
  const size_t smem = sizeof(float) * (2 * TC_STAGE + 2 * (size_t)TC_PTS * ps) + 4 * sizeof(uint64_t) + 16;
  if (rc == LLF_OK && smem > 220 * 1024) rc = llf_fail(ctx, LLF_ERR_LIMIT, "tensor-core tangent: element too large");
  const int64_t ctas = mesh->nel * t.nstrip * t.nhalf;
  if (rc == LLF_OK && ctas >= ((int64_t)1 << 31)) rc = llf_fail(ctx, LLF_ERR_LIMIT, "tensor-core tangent: too many tiles");
  if (rc == LLF_OK && ctas > 0) {
    cudaError_t e = cudaFuncSetAttribute(k_tl_tangent_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
    if (rc == LLF_OK) {
      KernelScope ks(ctx, "k_tl_tangent_tc");
      k_tl_tangent_tc<<<(unsigned)ctas, TC_THREADS, smem, s>>>(t);
      e = cudaGetLastError();
      if (e != cudaSuccess) rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
    }
  }
  if (rc == LLF_OK && mesh->nel > 0) {
    KernelScope ks(ctx, "k_tc_symmetrize");
    k_tc_symmetrize<<<(unsigned)(ctx->num_sms * 16), 256, 0, s>>>(Kf, mesh->nel, npe, cs);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
  }
  if (rc == LLF_OK) {
    cudaError_t e = dalloc(ctx, &m->d_nz, pat->nnz);
    rc = (e == cudaSuccess) ? gather_full32(ctx, pat, Kf, cs, true, m->d_nz, cnt)
                            : llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
  }
  dfree(ctx, pd);
  dfree(ctx, Kf);
  if (rc == LLF_OK) rc = llf_check_status(ctx, "tangent (tensor-core form)");
  if (rc == LLF_OK) rc = matrix_finalize(ctx, m, cnt);
  dfree(ctx, cnt);
  return rc;
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
