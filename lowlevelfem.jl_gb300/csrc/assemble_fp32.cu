// Precision form of the linear operators: element quadrature in FP32 (node
// coordinates taken relative to the element's first node in FP64 before the
// conversion, so large or offset meshes keep their geometric accuracy),
// FP32 element matrices, and the global CSC accumulation in FP64 (each
// element's FP32 contribution converted exactly to FP64 and summed in
// element order by the same column-node gather as the FP64 form).
// Halves the element-matrix traffic and moves the quadrature off the FP64
// pipe.  Results agree with the FP64 form to FP32 quadrature accuracy
// (~1e-7 relative to the largest entry); the stored (dropzeros!) pattern can
// keep entries that cancel exactly only in FP64.
#include "common.cuh"
#include "affine.cuh"

#include <algorithm>

namespace {

constexpr int E32_THREADS = 128;

struct Elem32Args {
  const double *xyz;
  const int32_t *conn;
  const int32_t *emat;
  int64_t nel;
  int npe, nip, npairs;
  const float *w, *N, *dN;
  const double *c1, *c2;
  float *Kf;
  int64_t colstride;  // floats per element-matrix column (16-byte multiple)
  unsigned *status;
  // affine-element form: per-element flag and FP64 invJ/det (aflag null =
  // none) and the per-pair tables of the FP64 form rounded to FP32
  const uint8_t *aflag;
  const double *ageo;
  const float *Rp, *Mp;
  // per affine element its FP32 coefficients (k_affine_coeff32), CW floats
  const float *coef;
  int affine_elsewhere;  // affine elements are left to k_affine_fp32
  int cta_cap;           // host side: CTAs per SM at most (0: as many as fit)
};

constexpr int CW = 48;  // coefficient floats per element (W 36 + U 9, padded)
constexpr int RPF_STRIDE = 12;  // floats per pair in the FP32 R table (sym 6, anti 3, pad 3)

// Twelve consecutive floats from a 16-byte aligned address.
__device__ __forceinline__ void load12(const float *p, float *r) {
#pragma unroll
  for (int t = 0; t < 12; t += 4) {
    const float4 f = __ldg(reinterpret_cast<const float4 *>(p + t));
    r[t] = f.x; r[t + 1] = f.y; r[t + 2] = f.z; r[t + 3] = f.w;
  }
}

// One thread per affine element: the FP64 form's coefficients rounded to
// FP32 (affine_coefficients32), and the determinant check of the staged form.
template <int KIND, int DIM>
__global__ void k_affine_coeff32(const double *__restrict__ ageo, const uint8_t *__restrict__ aflag,
                                 const int32_t *__restrict__ emat, const double *__restrict__ c1,
                                 const double *__restrict__ c2, int64_t nel, float *__restrict__ coef,
                                 unsigned *status) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nel; e += (int64_t)gridDim.x * blockDim.x) {
    const int mat = emat ? emat[e] : 0;
    if (mat < 0 || !aflag[e]) continue;
    const double *g = ageo + (size_t)e * 10;
    if (!(g[9] > 0.0)) atomicOr(status, ST_BAD_JACOBIAN);
    affine_coefficients32<KIND, DIM>(g, c1[mat], KIND == KIND_ELASTIC ? c2[mat] : 0.0, coef + (size_t)e * CW);
  }
}

__device__ __forceinline__ int poff(int a, int npe) { return a * npe - (a * (a - 1)) / 2; }
__device__ __forceinline__ void pdec(int pi, int npe, int &a, int &b) {
  int lo = 0, hi = npe - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (poff(mid, npe) <= pi) lo = mid; else hi = mid - 1;
  }
  a = lo;
  b = a + (pi - poff(a, npe));
}

// Block (a,b) and its mirror (b,a) at the padded block stride
// kf_bstride(P, BS > 1, 4); blocks of 4 and 12 floats go out as 16-byte
// stores (the column stride is a 16-byte multiple).
template <int P, int BS>
__device__ __forceinline__ void store_pair32(float *Ke, int64_t cs, int a, int b, const float *blk) {
  constexpr int BSTR = kf_bstride(P, BS > 1, 4);
  float *ab = Ke + (size_t)b * cs + (size_t)a * BSTR;
  if constexpr (BSTR % 4 == 0) {
    float t[BSTR];
#pragma unroll
    for (int k = 0; k < BSTR; ++k) t[k] = k < BS ? blk[k] : 0.f;
#pragma unroll
    for (int k = 0; k < BSTR; k += 4)
      *reinterpret_cast<float4 *>(ab + k) = make_float4(t[k], t[k + 1], t[k + 2], t[k + 3]);
    if (a != b) {
      float *ba = Ke + (size_t)a * cs + (size_t)b * BSTR;
#pragma unroll
      for (int i = 0; i < P; ++i)
#pragma unroll
        for (int j = 0; j < P; ++j) t[j * P + i] = blk[i * P + j];
#pragma unroll
      for (int k = 0; k < BSTR; k += 4)
        *reinterpret_cast<float4 *>(ba + k) = make_float4(t[k], t[k + 1], t[k + 2], t[k + 3]);
    }
  } else {
#pragma unroll
    for (int k = 0; k < BS; ++k) ab[k] = blk[k];
    if (a != b) {
      float *ba = Ke + (size_t)a * cs + (size_t)b * BSTR;
      ba[0] = blk[0];
    }
  }
}

// Node-pair blocks of an affine element in FP32: the FP64 form's per-element
// coefficients (from the FP64 invJ and det) rounded to FP32, read from the
// element's coefficient row cf, then Ksym = W S, Kanti = U A per pair as in
// the FP64 form.  No shared memory and no barrier: each thread's pairs only.
// R rows (RPF_STRIDE floats per pair, 16-byte aligned) from global memory
// or from a shared-memory copy; (a, b) decoded from the pair index, or read
// from a shared table packed as a | b << 16.
struct GlobalPairs {
  const float *R, *M;
  int npe;
  __device__ void row(int pi, float *r) const { load12(R + (size_t)pi * RPF_STRIDE, r); }
  __device__ float mass(int pi) const { return __ldg(M + pi); }
  __device__ void ab(int pi, int &a, int &b) const { pdec(pi, npe, a, b); }
};
struct SharedPairs {
  const float *R, *M;
  const uint32_t *AB;
  __device__ void row(int pi, float *r) const {
#pragma unroll
    for (int t = 0; t < RPF_STRIDE; t += 4) {
      const float4 f = *reinterpret_cast<const float4 *>(R + (size_t)pi * RPF_STRIDE + t);
      r[t] = f.x; r[t + 1] = f.y; r[t + 2] = f.z; r[t + 3] = f.w;
    }
  }
  __device__ float mass(int pi) const { return M[pi]; }
  __device__ void ab(int pi, int &a, int &b) const {
    const uint32_t v = AB[pi];
    a = (int)(v & 0xffffu);
    b = (int)(v >> 16);
  }
};

template <int KIND, int DIM, int P, int BS, class Pairs>
__device__ __forceinline__ void affine_pairs32(const Elem32Args &A, const Pairs &T, const float *__restrict__ cf,
                                               float *Ke) {
  constexpr int NS = DIM == 3 ? 6 : 3, NA = DIM == 3 ? 3 : 1;
  if (KIND == KIND_MASS) {
    const float cm = __ldg(cf);
    for (int pi = threadIdx.x; pi < A.npairs; pi += blockDim.x) {
      int a, b;
      T.ab(pi, a, b);
      float blk[BS];
      blk[0] = cm * T.mass(pi);
      store_pair32<P, BS>(Ke, A.colstride, a, b, blk);
    }
  } else if (KIND == KIND_HEAT) {
    float Q[NS];
#pragma unroll
    for (int n = 0; n < NS; ++n) Q[n] = __ldg(cf + n);
    for (int pi = threadIdx.x; pi < A.npairs; pi += blockDim.x) {
      int a, b;
      T.ab(pi, a, b);
      float r[RPF_STRIDE];
      T.row(pi, r);
      float acc = 0.f;
#pragma unroll
      for (int n = 0; n < NS; ++n) acc = fmaf(Q[n], r[n], acc);
      float blk[BS];
      blk[0] = acc;
      store_pair32<P, BS>(Ke, A.colstride, a, b, blk);
    }
  } else {
    float c[CW];
#pragma unroll
    for (int t = 0; t < CW; t += 4) {
      const float4 f = __ldg(reinterpret_cast<const float4 *>(cf + t));
      c[t] = f.x; c[t + 1] = f.y; c[t + 2] = f.z; c[t + 3] = f.w;
    }
    float W[NS * NS], U[NA * NA];
#pragma unroll
    for (int t = 0; t < NS * NS; ++t) W[t] = c[t];
#pragma unroll
    for (int t = 0; t < NA * NA; ++t) U[t] = c[NS * NS + t];
    for (int pi = threadIdx.x; pi < A.npairs; pi += blockDim.x) {
      int a, b;
      T.ab(pi, a, b);
      float r[RPF_STRIDE];
      T.row(pi, r);
      float sv[NS], av[NA];
#pragma unroll
      for (int n = 0; n < NS; ++n) sv[n] = r[n];
#pragma unroll
      for (int n = 0; n < NA; ++n) av[n] = r[6 + n];
      float ks[NS];
#pragma unroll
      for (int m = 0; m < NS; ++m) {
        float acc = 0.f;
#pragma unroll
        for (int n = 0; n < NS; ++n) acc = fmaf(W[m * NS + n], sv[n], acc);
        ks[m] = acc;
      }
      float blk[BS];
#pragma unroll
      for (int i = 0; i < DIM; ++i) blk[i * DIM + i] = ks[i];
#pragma unroll
      for (int m = 0; m < NA; ++m) {
        float acc = 0.f;
        if (a != b)
#pragma unroll
          for (int n = 0; n < NA; ++n) acc = fmaf(U[m * NA + n], av[n], acc);
        const int i = sym_k<DIM>(DIM + m), j = sym_l<DIM>(DIM + m);
        blk[i * DIM + j] = ks[DIM + m] + acc;
        blk[j * DIM + i] = ks[DIM + m] - acc;
      }
      store_pair32<P, BS>(Ke, A.colstride, a, b, blk);
    }
  }
}

template <int KIND, int DIM>
__global__ void __launch_bounds__(E32_THREADS) k_elem_fp32(Elem32Args A) {
  extern __shared__ double sd64[];
  const int npe = A.npe, nip = A.nip;
  constexpr int gsw = (KIND == KIND_MASS) ? 1 : DIM;
  double *sAff = sd64;                              // AFF_DOUBLES (affine form)
  float *sf = (float *)(sAff + AFF_DOUBLES);
  float *sdN = sf;                                  // nip*npe*DIM
  float *sw = sdN + (size_t)nip * npe * DIM;        // nip
  float *sN = sw + nip;                             // nip*npe (mass)
  float *sX = sN + (KIND == KIND_MASS ? (size_t)nip * npe : 0);  // npe*DIM
  float *sWd = sX + (size_t)npe * DIM;              // nip
  float *sInv = sWd + nip;                          // nip*9
  float *G = sInv + (size_t)nip * 9;                // nip*npe*gsw
  float *S = G + (size_t)nip * npe * gsw;           // nip*npe*gsw
  for (int t = threadIdx.x; t < nip * npe * DIM; t += blockDim.x)
    sdN[t] = A.dN[(size_t)(t / DIM) * 3 + t % DIM];
  for (int t = threadIdx.x; t < nip; t += blockDim.x) sw[t] = A.w[t];
  if (KIND == KIND_MASS)
    for (int t = threadIdx.x; t < nip * npe; t += blockDim.x) sN[t] = A.N[t];
  __syncthreads();
  constexpr int BS = (KIND == KIND_ELASTIC) ? DIM * DIM : 1;
  constexpr int P = (KIND == KIND_ELASTIC) ? DIM : 1;
  for (int64_t e = blockIdx.x; e < A.nel; e += gridDim.x) {
    const int mat = A.emat ? A.emat[e] : 0;
    if (mat < 0) continue;
    const float c1 = (float)A.c1[mat];
    const float c2 = (KIND == KIND_ELASTIC) ? (float)A.c2[mat] : 0.f;
    const int32_t *cn = A.conn + e * npe;
    float *Ke = A.Kf + (size_t)e * npe * A.colstride;
    if (A.aflag && A.aflag[e]) {  // uniform across the CTA; no shared state
      if (!A.affine_elsewhere)
        affine_pairs32<KIND, DIM, P, BS>(A, GlobalPairs{A.Rp, A.Mp, npe}, A.coef + (size_t)e * CW, Ke);
      continue;
    }
    for (int t = threadIdx.x; t < npe * DIM; t += blockDim.x) {
      int a = t / DIM, i = t % DIM;
      sX[t] = (float)(A.xyz[(size_t)cn[a] * 3 + i] - A.xyz[(size_t)cn[0] * 3 + i]);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nip; q += blockDim.x) {
      const float *d = sdN + (size_t)q * npe * DIM;
      float J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
      for (int a = 0; a < npe; ++a)
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
          for (int j = 0; j < DIM; ++j) J[i][j] = fmaf(sX[a * DIM + i], d[a * DIM + j], J[i][j]);
      float inv[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      float det;
      if (DIM == 3) {
        float c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        float c01 = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]);
        float c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        float r = 1.0f / det;
        inv[0] = c00 * r;
        inv[1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) * r;
        inv[2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
        inv[3] = c01 * r;
        inv[4] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
        inv[5] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) * r;
        inv[6] = c02 * r;
        inv[7] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) * r;
        inv[8] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
      } else {
        det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        float r = 1.0f / det;
        inv[0] = J[1][1] * r; inv[1] = -J[0][1] * r;
        inv[3] = -J[1][0] * r; inv[4] = J[0][0] * r;
      }
      if (!(det > 0.f)) atomicOr(A.status, ST_BAD_JACOBIAN);
      sWd[q] = det * sw[q];
#pragma unroll
      for (int k = 0; k < 9; ++k) sInv[q * 9 + k] = inv[k];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nip * npe; t += blockDim.x) {
      const int q = t / npe;
      if (KIND == KIND_MASS) {
        S[t] = sWd[q] * sN[t];
      } else {
        const float *inv = sInv + q * 9;
        const float *d = sdN + (size_t)t * DIM;
#pragma unroll
        for (int i = 0; i < DIM; ++i) {
          float acc = 0.f;
#pragma unroll
          for (int j = 0; j < DIM; ++j) acc = fmaf(inv[3 * j + i], d[j], acc);
          G[(size_t)t * DIM + i] = acc;
          S[(size_t)t * DIM + i] = sWd[q] * acc;
        }
      }
    }
    __syncthreads();
    for (int pi = threadIdx.x; pi < A.npairs; pi += blockDim.x) {
      int a, b;
      pdec(pi, npe, a, b);
      float blk[BS];
      if (KIND == KIND_ELASTIC) {
        float O[DIM][DIM];
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
          for (int j = 0; j < DIM; ++j) O[i][j] = 0.f;
        for (int q = 0; q < nip; ++q) {
          const float *sa = S + ((size_t)q * npe + a) * DIM;
          const float *gb = G + ((size_t)q * npe + b) * DIM;
#pragma unroll
          for (int i = 0; i < DIM; ++i)
#pragma unroll
            for (int j = 0; j < DIM; ++j) O[i][j] = fmaf(sa[i], gb[j], O[i][j]);
        }
        if (a == b)
#pragma unroll
          for (int i = 0; i < DIM; ++i)
#pragma unroll
            for (int j = 0; j < i; ++j) O[i][j] = O[j][i];
        float tr = O[0][0] + O[1 % DIM][1 % DIM];
        if (DIM == 3) tr += O[2 % DIM][2 % DIM];
#pragma unroll
        for (int i = 0; i < DIM; ++i)
#pragma unroll
          for (int j = 0; j < DIM; ++j) {
            float t = fmaf(c2, O[j][i], c1 * O[i][j]);
            if (i == j) t = fmaf(c2, tr, t);
            blk[i * DIM + j] = t;
          }
      } else if (KIND == KIND_HEAT) {
        float acc = 0.f;
        for (int q = 0; q < nip; ++q) {
          const float *sa = S + ((size_t)q * npe + a) * DIM;
          const float *gb = G + ((size_t)q * npe + b) * DIM;
#pragma unroll
          for (int i = 0; i < DIM; ++i) acc = fmaf(sa[i], gb[i], acc);
        }
        blk[0] = c1 * acc;
      } else {
        float acc = 0.f;
        for (int q = 0; q < nip; ++q) acc = fmaf(S[(size_t)q * npe + a], sN[(size_t)q * npe + b], acc);
        blk[0] = c1 * acc;
      }
      store_pair32<P, BS>(Ke, A.colstride, a, b, blk);
    }
    __syncthreads();
  }
}

// Every block (a, b) of an affine element, column by column: unit u is
// column b = u / npe, row a = u % npe, so the lanes of a warp write one
// contiguous run of a column and every block is written once.  The block is
// the pair (min, max)'s, transposed when a > b — the values of
// affine_pairs32 and its mirror, bit for bit.
template <int KIND, int DIM, int P, int BS>
__device__ __forceinline__ void affine_units32(const Elem32Args &A, const SharedPairs &T, const float *__restrict__ cf,
                                               float *Ke) {
  constexpr int NS = DIM == 3 ? 6 : 3, NA = DIM == 3 ? 3 : 1;
  constexpr int BSTR = kf_bstride(P, BS > 1, 4);
  const int npe = A.npe, nu = npe * npe;
  float c[CW];
  if (KIND == KIND_ELASTIC) {
#pragma unroll
    for (int t = 0; t < CW; t += 4) {
      const float4 f = __ldg(reinterpret_cast<const float4 *>(cf + t));
      c[t] = f.x; c[t + 1] = f.y; c[t + 2] = f.z; c[t + 3] = f.w;
    }
  } else {
#pragma unroll
    for (int t = 0; t < 8; t += 4) {
      const float4 f = __ldg(reinterpret_cast<const float4 *>(cf + t));
      c[t] = f.x; c[t + 1] = f.y; c[t + 2] = f.z; c[t + 3] = f.w;
    }
  }
  for (int u = threadIdx.x; u < nu; u += blockDim.x) {
    const int b = u / npe, a = u - b * npe;
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    const int pi = lo * npe - (lo * (lo - 1)) / 2 + (hi - lo);
    float *dst = Ke + (size_t)b * A.colstride + (size_t)a * BSTR;
    if (KIND == KIND_MASS) {
      dst[0] = c[0] * T.mass(pi);
    } else if (KIND == KIND_HEAT) {
      float r[RPF_STRIDE];
      T.row(pi, r);
      float acc = 0.f;
#pragma unroll
      for (int n = 0; n < NS; ++n) acc = fmaf(c[n], r[n], acc);
      dst[0] = acc;
    } else {
      float r[RPF_STRIDE];
      T.row(pi, r);
      float ks[NS];
#pragma unroll
      for (int m = 0; m < NS; ++m) {
        float acc = 0.f;
#pragma unroll
        for (int n = 0; n < NS; ++n) acc = fmaf(c[m * NS + n], r[n], acc);
        ks[m] = acc;
      }
      float blk[BSTR];
#pragma unroll
      for (int k = BS; k < BSTR; ++k) blk[k] = 0.f;
#pragma unroll
      for (int i = 0; i < DIM; ++i) blk[i * DIM + i] = ks[i];
#pragma unroll
      for (int m = 0; m < NA; ++m) {
        float acc = 0.f;
        if (lo != hi)
#pragma unroll
          for (int n = 0; n < NA; ++n) acc = fmaf(c[NS * NS + m * NA + n], r[6 + n], acc);
        const int i = sym_k<DIM>(DIM + m), j = sym_l<DIM>(DIM + m);
        // block (lo, hi) holds ks + acc at (i, j) and ks - acc at (j, i); (hi, lo) its transpose
        blk[i * DIM + j] = a <= b ? ks[DIM + m] + acc : ks[DIM + m] - acc;
        blk[j * DIM + i] = a <= b ? ks[DIM + m] - acc : ks[DIM + m] + acc;
      }
      if constexpr (BSTR % 4 == 0) {
#pragma unroll
        for (int k = 0; k < BSTR; k += 4)
          *reinterpret_cast<float4 *>(dst + k) = make_float4(blk[k], blk[k + 1], blk[k + 2], blk[k + 3]);
      } else {
#pragma unroll
        for (int k = 0; k < BS; ++k) dst[k] = blk[k];
      }
    }
  }
}

// Affine elements only: the pair tables (R rows or reference mass, and the
// packed (a, b) of every pair) are copied into shared memory once per CTA
// and stay there; per element a thread reads the element's coefficient row
// and forms its pairs with no further global loads and no barrier.
template <int KIND, int DIM>
__global__ void __launch_bounds__(E32_THREADS) k_affine_fp32(Elem32Args A) {
  extern __shared__ float4 af_smem[];
  constexpr int BS = (KIND == KIND_ELASTIC) ? DIM * DIM : 1;
  constexpr int P = (KIND == KIND_ELASTIC) ? DIM : 1;
  const int np = A.npairs;
  float *sR = reinterpret_cast<float *>(af_smem);                       // np * RPF_STRIDE (elastic, heat)
  float *sM = sR + (KIND == KIND_MASS ? 0 : (size_t)np * RPF_STRIDE);   // np (mass)
  uint32_t *sAB = reinterpret_cast<uint32_t *>(sM + (KIND == KIND_MASS ? np : 0));
  if (KIND == KIND_MASS) {
    for (int t = threadIdx.x; t < np; t += blockDim.x) sM[t] = A.Mp[t];
  } else {
    for (int t = threadIdx.x; t < np * RPF_STRIDE / 4; t += blockDim.x)
      reinterpret_cast<float4 *>(sR)[t] = __ldg(reinterpret_cast<const float4 *>(A.Rp) + t);
  }
  for (int pi = threadIdx.x; pi < np; pi += blockDim.x) {
    int a, b;
    pdec(pi, A.npe, a, b);
    sAB[pi] = (uint32_t)a | ((uint32_t)b << 16);
  }
  __syncthreads();
  const SharedPairs T{sR, sM, sAB};
  for (int64_t e = blockIdx.x; e < A.nel; e += gridDim.x) {
    if (!A.aflag[e] || (A.emat && A.emat[e] < 0)) continue;
    affine_units32<KIND, DIM, P, BS>(A, T, A.coef + (size_t)e * CW, A.Kf + (size_t)e * A.npe * A.colstride);
  }
}

// Shared memory of k_affine_fp32 for npairs pairs.
template <int KIND>
size_t affine_fp32_smem(int npairs) {
  return (KIND == KIND_MASS ? sizeof(float) * npairs : sizeof(float) * (size_t)npairs * RPF_STRIDE) +
         sizeof(uint32_t) * npairs;
}

template <int KIND, int DIM>
int run_affine32(llf_ctx *ctx, const Elem32Args &a) {
  const size_t smem = affine_fp32_smem<KIND>(a.npairs);
  auto fn = k_affine_fp32<KIND, DIM>;
  if (smem > 48 * 1024)
    LLF_CUDA_TRY(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 1;
  LLF_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, E32_THREADS, smem));
  if (a.cta_cap > 0 && per_sm > a.cta_cap) per_sm = a.cta_cap;
  int64_t grid = (int64_t)ctx->num_sms * (per_sm < 1 ? 1 : per_sm);
  if (grid > a.nel) grid = a.nel > 0 ? a.nel : 1;
  KernelScope ks(ctx, "k_affine_fp32");
  fn<<<(unsigned)grid, E32_THREADS, smem, ctx->stream>>>(a);
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  return LLF_OK;
}

template <int KIND, int DIM>
int run_elem32(llf_ctx *ctx, Elem32Args a) {
  const int npe = a.npe, nip = a.nip;
  const int gsw = (KIND == KIND_MASS) ? 1 : DIM;
  size_t smem = sizeof(double) * AFF_DOUBLES +
                sizeof(float) * ((size_t)nip * npe * DIM + nip + (KIND == KIND_MASS ? (size_t)nip * npe : 0) +
                                 (size_t)npe * DIM + nip + (size_t)nip * 9 + 2 * (size_t)nip * npe * gsw);
  if (smem > 200 * 1024)
    return llf_fail(ctx, LLF_ERR_LIMIT, "precision form: element tables exceed shared memory (use the FP64 form)");
  auto fn = k_elem_fp32<KIND, DIM>;
  if (smem > 48 * 1024)
    LLF_CUDA_TRY(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 1;
  LLF_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, E32_THREADS, smem));
  if (a.cta_cap > 0 && per_sm > a.cta_cap) per_sm = a.cta_cap;
  int64_t grid = (int64_t)ctx->num_sms * (per_sm < 1 ? 1 : per_sm);
  if (grid > a.nel) grid = a.nel > 0 ? a.nel : 1;
  KernelScope ks(ctx, "k_elem_fp32");
  fn<<<(unsigned)grid, E32_THREADS, smem, ctx->stream>>>(a);
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  return LLF_OK;
}

}  // namespace

// Precision-form assembly of the structural values into nz (and the
// per-column non-zero counts into cnt).
int assemble_fp32_impl(llf_ctx *ctx, llf_mesh *mesh, llf_pattern *pat, int kind, const double *d_c1,
                       const double *d_c2, const uint8_t *aflag, const double *ageo, double *nz,
                       int64_t *cnt, const double *init, GatherSink *sink, StoredSpec *spec, bool all_affine) {
  const int npe = mesh->npe, P = pat->pdim;
  float *Kf = nullptr;
  const int64_t cs = kf_colstride(npe, kf_bstride(P, kind == KIND_ELASTIC, (int)sizeof(float)), (int)sizeof(float));
  LLF_CUDA_TRY(ctx, dalloc(ctx, &Kf, (size_t)mesh->nel * npe * cs));
  Elem32Args a{};
  a.xyz = mesh->d_xyz;
  a.conn = mesh->d_conn;
  a.emat = mesh->d_emat;
  a.nel = mesh->nel;
  a.npe = npe;
  a.nip = mesh->nip;
  a.npairs = npe * (npe + 1) / 2;
  a.w = mesh->d_wf;
  a.N = mesh->d_Nf;
  a.dN = mesh->d_dNf;
  a.c1 = d_c1;
  a.c2 = d_c2;
  a.Kf = Kf;
  a.colstride = cs;
  a.status = ctx->d_status;
  a.aflag = aflag;
  a.ageo = ageo;
  a.Rp = mesh->d_Rpf;
  a.Mp = mesh->d_Mpf;
  float *coef = nullptr;
  if (aflag) {  // FP32 coefficients of every affine element, one thread each
    LLF_CUDA_TRY(ctx, dalloc(ctx, &coef, (size_t)std::max<int64_t>(mesh->nel, 1) * CW));
    const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((mesh->nel + 127) / 128, (int64_t)ctx->num_sms * 16));
    KernelScope ks(ctx, "k_affine_coeff32");
#define LLF_COEF32(KK, DD) \
  k_affine_coeff32<KK, DD><<<g, 128, 0, ctx->stream>>>(ageo, aflag, mesh->d_emat, d_c1, d_c2, mesh->nel, coef, \
                                                         ctx->d_status)
    if (mesh->dim == 3) {
      if (kind == KIND_ELASTIC) LLF_COEF32(KIND_ELASTIC, 3);
      else if (kind == KIND_HEAT) LLF_COEF32(KIND_HEAT, 3);
      else LLF_COEF32(KIND_MASS, 3);
    } else {
      if (kind == KIND_ELASTIC) LLF_COEF32(KIND_ELASTIC, 2);
      else if (kind == KIND_HEAT) LLF_COEF32(KIND_HEAT, 2);
      else LLF_COEF32(KIND_MASS, 2);
    }
#undef LLF_COEF32
    LLF_CUDA_TRY(ctx, cudaGetLastError());
  }
  a.coef = coef;
  // the affine kernel keeps the pair tables in shared memory; beyond 96 KB
  // (high orders) the general kernel reads them from global memory instead
  const size_t af_smem = kind == KIND_MASS ? affine_fp32_smem<KIND_MASS>(a.npairs)
                                           : affine_fp32_smem<KIND_ELASTIC>(a.npairs);
  a.affine_elsewhere = (aflag && af_smem <= 96 * 1024) ? 1 : 0;
  a.cta_cap = pat->tune.elem_cap;
  // element range [e0, e1): the element-indexed arrays are offset
  auto elems = [&](int64_t e0, int64_t e1) -> int {
    Elem32Args b = a;
    b.conn = a.conn + e0 * npe;
    b.emat = a.emat ? a.emat + e0 : nullptr;
    b.nel = e1 - e0;
    b.Kf = a.Kf + e0 * npe * cs;
    b.aflag = a.aflag ? a.aflag + e0 : nullptr;
    b.ageo = a.ageo ? a.ageo + e0 * 10 : nullptr;
    b.coef = a.coef ? a.coef + e0 * CW : nullptr;
    if (b.nel <= 0) return LLF_OK;
    int r = LLF_OK;
    if (b.affine_elsewhere) {
      if (mesh->dim == 3)
        r = kind == KIND_ELASTIC ? run_affine32<KIND_ELASTIC, 3>(ctx, b)
                                 : (kind == KIND_HEAT ? run_affine32<KIND_HEAT, 3>(ctx, b) : run_affine32<KIND_MASS, 3>(ctx, b));
      else
        r = kind == KIND_ELASTIC ? run_affine32<KIND_ELASTIC, 2>(ctx, b)
                                 : (kind == KIND_HEAT ? run_affine32<KIND_HEAT, 2>(ctx, b) : run_affine32<KIND_MASS, 2>(ctx, b));
      if (r != LLF_OK) return r;
      if (all_affine) return LLF_OK;   // no element left for the general kernel
    }
    if (mesh->dim == 3)
      return kind == KIND_ELASTIC ? run_elem32<KIND_ELASTIC, 3>(ctx, b)
                                  : (kind == KIND_HEAT ? run_elem32<KIND_HEAT, 3>(ctx, b) : run_elem32<KIND_MASS, 3>(ctx, b));
    return kind == KIND_ELASTIC ? run_elem32<KIND_ELASTIC, 2>(ctx, b)
                                : (kind == KIND_HEAT ? run_elem32<KIND_HEAT, 2>(ctx, b) : run_elem32<KIND_MASS, 2>(ctx, b));
  };
  int rc;
  if (sink) {
    rc = sink->gather(ctx, pat, Kf, cs, kind == KIND_ELASTIC, elems);
  } else {
    rc = elems(0, mesh->nel);
    if (rc == LLF_OK) rc = gather_full32(ctx, pat, Kf, cs, kind == KIND_ELASTIC, nz, cnt, init, spec);
  }
  dfree(ctx, coef);
  dfree(ctx, Kf);
  return rc;
}
