// Device helpers shared by the FP64 and precision-form element kernels:
// the Jacobian inverse of the geometry contract and the affine-element form
// (affinity test, per-element coefficients).  The operation order is the
// CPU oracle's (llfem_oracle.c: orc_geom, orc_is_affine, orc_element_affine).
#pragma once
#include "common.cuh"

namespace {

// Determinant and row-major inverse of the Jacobian J (contract of the
// oracle's geometry: cofactors, det by the first row, inverse = cofactor^T
// times the rounded reciprocal of det).
template <int DIM>
__device__ __forceinline__ double jac_inverse(const double (&J)[3][3], double *inv) {
  double det, rdet;
  if (DIM == 3) {
    double c00 = __dsub_rn(__dmul_rn(J[1][1], J[2][2]), __dmul_rn(J[1][2], J[2][1]));
    double c01 = -__dsub_rn(__dmul_rn(J[1][0], J[2][2]), __dmul_rn(J[1][2], J[2][0]));
    double c02 = __dsub_rn(__dmul_rn(J[1][0], J[2][1]), __dmul_rn(J[1][1], J[2][0]));
    double c10 = -__dsub_rn(__dmul_rn(J[0][1], J[2][2]), __dmul_rn(J[0][2], J[2][1]));
    double c11 = __dsub_rn(__dmul_rn(J[0][0], J[2][2]), __dmul_rn(J[0][2], J[2][0]));
    double c12 = -__dsub_rn(__dmul_rn(J[0][0], J[2][1]), __dmul_rn(J[0][1], J[2][0]));
    double c20 = __dsub_rn(__dmul_rn(J[0][1], J[1][2]), __dmul_rn(J[0][2], J[1][1]));
    double c21 = -__dsub_rn(__dmul_rn(J[0][0], J[1][2]), __dmul_rn(J[0][2], J[1][0]));
    double c22 = __dsub_rn(__dmul_rn(J[0][0], J[1][1]), __dmul_rn(J[0][1], J[1][0]));
    det = __dadd_rn(__dadd_rn(__dmul_rn(J[0][0], c00), __dmul_rn(J[0][1], c01)),
                    __dmul_rn(J[0][2], c02));
    rdet = __drcp_rn(det);
    inv[0] = __dmul_rn(c00, rdet); inv[1] = __dmul_rn(c10, rdet); inv[2] = __dmul_rn(c20, rdet);
    inv[3] = __dmul_rn(c01, rdet); inv[4] = __dmul_rn(c11, rdet); inv[5] = __dmul_rn(c21, rdet);
    inv[6] = __dmul_rn(c02, rdet); inv[7] = __dmul_rn(c12, rdet); inv[8] = __dmul_rn(c22, rdet);
  } else {
    det = __dsub_rn(__dmul_rn(J[0][0], J[1][1]), __dmul_rn(J[0][1], J[1][0]));
    rdet = __drcp_rn(det);
    inv[0] = __dmul_rn(J[1][1], rdet);
    inv[1] = __dmul_rn(-J[0][1], rdet);
    inv[2] = 0.0;
    inv[3] = __dmul_rn(-J[1][0], rdet);
    inv[4] = __dmul_rn(J[0][0], rdet);
    inv[5] = 0.0; inv[6] = 0.0; inv[7] = 0.0; inv[8] = 0.0;
  }
  return det;
}

// sAff: [0,10) unused | [10,19) invJ | [19] det | [20,56) V | [56,92) W |
// [92,101) U | [101,107) c1*trV | [107] c1*det
constexpr int AFF_DOUBLES = 128;
enum { AF_INV = 10, AF_DET = 19, AF_V = 20, AF_W = 56, AF_U = 92, AF_Q = 101, AF_M = 107 };

// Symmetric components (k,l), k <= l: 3D 00 11 22 01 02 12, 2D 00 11 01; the
// antisymmetric components are the off-diagonal ones, in the same order.
template <int DIM>
__host__ __device__ constexpr int sym_k(int n) {
  return DIM == 3 ? (n < 3 ? n : (n < 5 ? 0 : 1)) : (n < 2 ? n : 0);
}
template <int DIM>
__host__ __device__ constexpr int sym_l(int n) {
  return DIM == 3 ? (n < 3 ? n : (n == 3 ? 1 : 2)) : (n < 2 ? n : 1);
}

// Affine geometry of every element, one thread per element (contract of the
// oracle's orc_is_affine / orc_geom at point 0): J0 = fma chain over nodes of
// X_a,i dN0_a,j; s = max |X|; the element is affine when every node satisfies
// |X_a - X_0 - J0 (xi_a - xi_0)| <= 2^-46 s componentwise (fma chain over j)
// and s > 0.  When every off-diagonal entry of J0 is within the same
// tolerance the element is an axis-aligned brick and those entries are set
// to +0.0 before the inverse (oracle: orc_geom_affine).  For affine elements
// geo[e*10 + 0..8] = invJ (row-major) and geo[e*10 + 9] = det; flag[e] = 2
// for axis-aligned ones, else 1.  Elements with a negative material index
// get flag 0; the others with flag 0 are counted in *nonaffine (if given).
template <int DIM>
__global__ void k_affine_geometry(const double *__restrict__ xyz, const int32_t *__restrict__ conn,
                                  const int32_t *__restrict__ emat, int64_t nel, int npe,
                                  const double *__restrict__ dN0, const double *__restrict__ nref,
                                  double *__restrict__ geo, uint8_t *__restrict__ flag,
                                  unsigned long long *__restrict__ nonaffine) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nel;
       e += (int64_t)gridDim.x * blockDim.x) {
    uint8_t f = 0;
    if (!emat || emat[e] >= 0) {
      const int32_t *cn = conn + e * npe;
      double J[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
      double s = 0.0;
      for (int a = 0; a < npe; ++a) {
        const double *x = xyz + (size_t)cn[a] * 3;
#pragma unroll
        for (int i = 0; i < DIM; ++i) {
          s = fmax(s, fabs(x[i]));
#pragma unroll
          for (int j = 0; j < DIM; ++j) J[i][j] = __fma_rn(x[i], dN0[a * 3 + j], J[i][j]);
        }
      }
      const double tol = __dmul_rn(1.4210854715202004e-14, s);  // 64 * 2^-52
      bool ok = s > 0.0;
      const double *x0 = xyz + (size_t)cn[0] * 3;
      for (int a = 1; a < npe && ok; ++a) {
        const double *x = xyz + (size_t)cn[a] * 3;
#pragma unroll
        for (int i = 0; i < DIM; ++i) {
          double r = __dsub_rn(x[i], x0[i]);
#pragma unroll
          for (int j = 0; j < DIM; ++j) r = __fma_rn(-J[i][j], __dsub_rn(nref[a * 3 + j], nref[j]), r);
          if (!(fabs(r) <= tol)) ok = false;
        }
      }
      if (ok) {
        // axis-aligned up to the rounding of the sums: the off-diagonal
        // entries become +0.0, so every coefficient mixing two axes is an
        // exact zero (flag 2 selects the element kernels' reduced form)
        bool aligned = true;
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
          for (int j = 0; j < DIM; ++j)
            if (i != j && !(fabs(J[i][j]) <= tol)) aligned = false;
        if (aligned) {
#pragma unroll
          for (int i = 0; i < DIM; ++i)
#pragma unroll
            for (int j = 0; j < DIM; ++j)
              if (i != j) J[i][j] = 0.0;
        }
        double inv[9];
        const double det = jac_inverse<DIM>(J, inv);
#pragma unroll
        for (int k = 0; k < 9; ++k) geo[e * 10 + k] = inv[k];
        geo[e * 10 + 9] = det;
        f = aligned ? 2 : 1;
      } else if (nonaffine) {
        atomicAdd(nonaffine, 1ull);
      }
    }
    flag[e] = f;
  }
}

// Stage the element's invJ and det (from k_affine_geometry) and form its
// coefficients: called by warp 0; sAff[AF_INV..AF_DET] then the rest.
template <int DIM>
__device__ __forceinline__ void affine_stage(const double *geo_e, double c1, double c2, double *sAff,
                                             unsigned *status);

// Per-element coefficients of the affine form (contract of the oracle), by
// warp 0 after invJ and det are in sAff: V (symmetric congruence of S),
// W = Lame combination of V, U (antisymmetric congruence times c1 - c2),
// c1*trV (heat) and c1*det (mass).
template <int DIM>
__device__ __forceinline__ void affine_coefficients(double *sAff, double c1, double c2, int lane) {
  constexpr int NS = DIM == 3 ? 6 : 3, NA = DIM == 3 ? 3 : 1;
  const double *inv = sAff + AF_INV;
  const double det = sAff[AF_DET];
  for (int t = lane; t < NS * NS; t += 32) {
    const int m = t / NS, n = t - m * NS;
    const int i = sym_k<DIM>(m), j = sym_l<DIM>(m), k = sym_k<DIM>(n), l = sym_l<DIM>(n);
    sAff[AF_V + t] = k == l ? __dmul_rn(det, __dmul_rn(inv[k * 3 + i], inv[k * 3 + j]))
                            : __dmul_rn(det, __fma_rn(inv[k * 3 + i], inv[l * 3 + j],
                                                      __dmul_rn(inv[l * 3 + i], inv[k * 3 + j])));
  }
  __syncwarp();
  const double cp = __dadd_rn(c1, c2), cm = __dsub_rn(c1, c2);
  for (int t = lane; t < NS * NS; t += 32) {
    const int m = t / NS, n = t - m * NS;
    const double *V = sAff + AF_V;
    double tr = __dadd_rn(V[n], V[NS + n]);
    if (DIM == 3) tr = __dadd_rn(tr, V[2 * NS + n]);
    const double v = __dmul_rn(cp, V[t]);
    sAff[AF_W + t] = m < DIM ? __fma_rn(c2, tr, v) : v;
    if (m == 0) sAff[AF_Q + n] = __dmul_rn(c1, tr);
  }
  if (lane < NA * NA) {
    const int m = lane / NA, n = lane - m * NA;
    const int i = sym_k<DIM>(DIM + m), j = sym_l<DIM>(DIM + m);
    const int k = sym_k<DIM>(DIM + n), l = sym_l<DIM>(DIM + n);
    sAff[AF_U + lane] =
        __dmul_rn(cm, __dmul_rn(det, __fma_rn(inv[k * 3 + i], inv[l * 3 + j],
                                              -__dmul_rn(inv[l * 3 + i], inv[k * 3 + j]))));
  }
  if (lane == 0) sAff[AF_M] = __dmul_rn(c1, det);
}

// The same coefficients by one thread, rounded to FP32 for the precision
// form: every value is formed by exactly the operations of
// affine_coefficients.  out: elastic W[NS*NS] then U[NA*NA]; heat
// (c1 trV)[NS]; mass c1*det.
template <int KIND, int DIM>
__device__ __forceinline__ void affine_coefficients32(const double *geo_e, double c1, double c2, float *out) {
  constexpr int NS = DIM == 3 ? 6 : 3, NA = DIM == 3 ? 3 : 1;
  const double *inv = geo_e;
  const double det = geo_e[9];
  if (KIND == KIND_MASS) {
    out[0] = (float)__dmul_rn(c1, det);
    return;
  }
  const double cp = __dadd_rn(c1, c2), cm = __dsub_rn(c1, c2);
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    const int k = sym_k<DIM>(n), l = sym_l<DIM>(n);
    double V[NS];
#pragma unroll
    for (int m = 0; m < NS; ++m) {
      const int i = sym_k<DIM>(m), j = sym_l<DIM>(m);
      V[m] = k == l ? __dmul_rn(det, __dmul_rn(inv[k * 3 + i], inv[k * 3 + j]))
                    : __dmul_rn(det, __fma_rn(inv[k * 3 + i], inv[l * 3 + j],
                                              __dmul_rn(inv[l * 3 + i], inv[k * 3 + j])));
    }
    double tr = __dadd_rn(V[0], V[1]);
    if (DIM == 3) tr = __dadd_rn(tr, V[2]);
    if (KIND == KIND_HEAT) {
      out[n] = (float)__dmul_rn(c1, tr);
    } else {
#pragma unroll
      for (int m = 0; m < NS; ++m) {
        const double v = __dmul_rn(cp, V[m]);
        out[m * NS + n] = (float)(m < DIM ? __fma_rn(c2, tr, v) : v);
      }
    }
  }
  if (KIND == KIND_ELASTIC) {
#pragma unroll
    for (int t = 0; t < NA * NA; ++t) {
      const int m = t / NA, n = t - m * NA;
      const int i = sym_k<DIM>(DIM + m), j = sym_l<DIM>(DIM + m);
      const int k = sym_k<DIM>(DIM + n), l = sym_l<DIM>(DIM + n);
      out[NS * NS + t] = (float)__dmul_rn(cm, __dmul_rn(det, __fma_rn(inv[k * 3 + i], inv[l * 3 + j],
                                                                     -__dmul_rn(inv[l * 3 + i], inv[k * 3 + j]))));
    }
  }
}

template <int DIM>
__device__ __forceinline__ void affine_stage(const double *geo_e, double c1, double c2, double *sAff,
                                             unsigned *status, int lane) {
  if (lane < 10) sAff[AF_INV + lane] = geo_e[lane];
  __syncwarp();
  if (lane == 0 && !(sAff[AF_DET] > 0.0)) atomicOr(status, ST_BAD_JACOBIAN);
  affine_coefficients<DIM>(sAff, c1, c2, lane);
}

// The coefficients of an axis-aligned element (flag 2: invJ diagonal, its
// other entries exact zeros; d_k = invJ[k][k]), by one warp (contract of
// the oracle's orc_element_aligned): V_n = det (d_k d_l) for the symmetric
// component n = (k,l); elasticity alpha_i = cp V_i, beta_i = c2 V_i (at
// AF_W + i and AF_W + DIM + i), a_m = cp V_m, b_m = cm V_m for the mixed
// components (at AF_W + 2 DIM + m and AF_W + 2 DIM + NA + m); heat
// c1 trV_n = c1 V_n (n < DIM, the general form's value bit for bit: the
// other terms of trV are exact zeros); mass c1 det.
template <int DIM>
__device__ __forceinline__ void affine_stage_aligned(const double *geo_e, double c1, double c2, double *sAff,
                                                     unsigned *status, int lane) {
  constexpr int NS = DIM == 3 ? 6 : 3, NA = DIM == 3 ? 3 : 1;
  const double det = geo_e[9];
  if (lane == 0) {
    sAff[AF_DET] = det;
    if (!(det > 0.0)) atomicOr(status, ST_BAD_JACOBIAN);
  }
  double *Vd = sAff + AF_V;   // V_n, n < NS
  if (lane < NS) {
    const int k = sym_k<DIM>(lane), l = sym_l<DIM>(lane);
    Vd[lane] = __dmul_rn(det, __dmul_rn(geo_e[k * 3 + k], geo_e[l * 3 + l]));
  }
  __syncwarp();
  const double cp = __dadd_rn(c1, c2), cm = __dsub_rn(c1, c2);
  if (lane < DIM) {
    sAff[AF_W + lane] = __dmul_rn(cp, Vd[lane]);
    sAff[AF_W + DIM + lane] = __dmul_rn(c2, Vd[lane]);
    sAff[AF_Q + lane] = __dmul_rn(c1, Vd[lane]);
  } else if (lane < DIM + NA) {
    const int m = lane - DIM;
    sAff[AF_W + 2 * DIM + m] = __dmul_rn(cp, Vd[DIM + m]);
    sAff[AF_W + 2 * DIM + NA + m] = __dmul_rn(cm, Vd[DIM + m]);
  } else if (lane == DIM + NA) {
    sAff[AF_M] = __dmul_rn(c1, det);
  }
}

}  // namespace
