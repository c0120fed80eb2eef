// Boundary loads (loadVector) and elementwise nodal gradients (u∘∇).
//
// loadVector, src/linear.jl:3088-3434: per boundary element and point,
//   t1, t2 = columns of the boundary Jacobian (fma chains over the nodes),
//   Ja = |t1| * b (2D edge, :3394-3395) or |t1 x t2| (3D face, :3380-3384),
//   fe[a,i] = fma(N_a t_i, Ja w, fe[a,i]);
// element vectors are buffered and then summed into f node by node in
// element order, the order the reference (and the oracle) adds them.
//
// elasticSupportMatrix / heatConvectionMatrix, src/linear.jl:2859-3005 and
// src/heat.jl:562-567: C = sum over boundary elements and points of
// H^T diag(k) H Ja w with Ja as in the load vector.  One thread per boundary
// element accumulates, for node pairs a <= b and component i, the fma chain
// over the points of ((N_a Ja w) k_i) N_b into the diagonal of block (a,b) of
// a full element matrix in the assembly's column-major-by-node layout; the
// pattern's column gather then sums the element matrices in element order
// into the volume pattern and dropzeros! compacts it.
//
// ∇ (:vector_grad branch), src/nabla.jl:77-311: at every element node k the
// Jacobian and physical gradients of all shape functions are evaluated at
// that node's reference coordinates, T[i,j] = sum_l g_l,j u_l,i (fma chain
// over l), stored column-major per node (9 values); F = I + T on request.
#include "common.cuh"
#include "affine.cuh"

#include <algorithm>
#include <string>

namespace {

// F at a face point: Fq[i][j] = fma chain over the nodes of N_a F_a[i][j],
// F nodal (9 per node, column-major 3x3).
template <int BDIM>
__device__ __forceinline__ void face_F(const double *__restrict__ Fn, const int32_t *c, int npe,
                                       const double *__restrict__ Nq, double (&Fq)[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double acc = 0.0;
      for (int a = 0; a < npe; ++a) acc = __fma_rn(Nq[a], Fn[(size_t)c[a] * 9 + 3 * j + i], acc);
      Fq[i][j] = acc;
    }
}

template <int BDIM>
__global__ void k_load_elem(const double *__restrict__ xyz, const int32_t *__restrict__ conn,
                            int64_t nel, int npe, int nip, const double *__restrict__ w,
                            const double *__restrict__ N, const double *__restrict__ dN, int pdim,
                            double t0, double t1c, double t2c, const double *__restrict__ tn,
                            double thickness, const double *__restrict__ Fn, unsigned *status,
                            double *__restrict__ fe) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nel;
       e += (int64_t)gridDim.x * blockDim.x) {
    double *out = fe + (size_t)e * npe * pdim;
    for (int k = 0; k < npe * pdim; ++k) out[k] = 0.0;
    const int32_t *c = conn + (size_t)e * npe;
    for (int q = 0; q < nip; ++q) {
      double a1[3], a2[3];
      for (int i = 0; i < 3; ++i) {
        double s1 = 0.0, s2 = 0.0;
        for (int a = 0; a < npe; ++a) {
          double xa = xyz[(size_t)c[a] * 3 + i];
          s1 = __fma_rn(xa, dN[((size_t)q * npe + a) * 3 + 0], s1);
          if (BDIM == 2) s2 = __fma_rn(xa, dN[((size_t)q * npe + a) * 3 + 1], s2);
        }
        a1[i] = s1;
        a2[i] = s2;
      }
      double Ja;
      if (BDIM == 1) {
        Ja = __dmul_rn(__dsqrt_rn(__dadd_rn(__dmul_rn(a1[0], a1[0]), __dmul_rn(a1[1], a1[1]))), thickness);
      } else {
        double xy = __dsub_rn(__dmul_rn(a1[0], a2[1]), __dmul_rn(a1[1], a2[0]));
        double yz = __dsub_rn(__dmul_rn(a1[1], a2[2]), __dmul_rn(a1[2], a2[1]));
        double zx = __dsub_rn(__dmul_rn(a1[2], a2[0]), __dmul_rn(a1[0], a2[2]));
        Ja = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(xy, xy), __dmul_rn(yz, yz)), __dmul_rn(zx, zx)));
      }
      double tq[3] = {t0, t1c, t2c};
      if (tn) {
        for (int i = 0; i < pdim; ++i) {
          double acc = 0.0;
          for (int a = 0; a < npe; ++a)
            acc = __fma_rn(N[(size_t)q * npe + a], tn[(size_t)c[a] * pdim + i], acc);
          tq[i] = acc;
        }
      }
      if (BDIM == 2 && Fn) {  // follower traction F_q t_q (3D faces)
        double Fq[3][3], Fi[9];
        face_F<BDIM>(Fn, c, npe, N + (size_t)q * npe, Fq);
        if (!(jac_inverse<3>(Fq, Fi) > 0.0)) atomicOr(status, ST_BAD_JACOBIAN);
        double tg[3];
        for (int i = 0; i < 3; ++i) {
          double acc = 0.0;
          for (int j = 0; j < 3; ++j) acc = __fma_rn(Fq[i][j], tq[j], acc);
          tg[i] = acc;
        }
        for (int i = 0; i < 3; ++i) tq[i] = tg[i];
      }
      const double jw = __dmul_rn(Ja, w[q]);
      for (int a = 0; a < npe; ++a) {
        const double Na = N[(size_t)q * npe + a];
        for (int i = 0; i < pdim; ++i)
          out[a * pdim + i] = __fma_rn(__dmul_rn(Na, tq[i]), jw, out[a * pdim + i]);
      }
    }
  }
}

// Ja of boundary point q (contract of the load vector): |t1| * b for a 2D
// edge, |t1 x t2| for a 3D face; t1, t2 fma chains over the nodes.
template <int BDIM>
__device__ __forceinline__ double boundary_ja(const double *__restrict__ xyz, const int32_t *c, int npe, int q,
                                              const double *__restrict__ dN, double thickness) {
  double a1[3], a2[3];
  for (int i = 0; i < 3; ++i) {
    double s1 = 0.0, s2 = 0.0;
    for (int a = 0; a < npe; ++a) {
      double xa = xyz[(size_t)c[a] * 3 + i];
      s1 = __fma_rn(xa, dN[((size_t)q * npe + a) * 3 + 0], s1);
      if (BDIM == 2) s2 = __fma_rn(xa, dN[((size_t)q * npe + a) * 3 + 1], s2);
    }
    a1[i] = s1;
    a2[i] = s2;
  }
  if (BDIM == 1)
    return __dmul_rn(__dsqrt_rn(__dadd_rn(__dmul_rn(a1[0], a1[0]), __dmul_rn(a1[1], a1[1]))), thickness);
  double xy = __dsub_rn(__dmul_rn(a1[0], a2[1]), __dmul_rn(a1[1], a2[0]));
  double yz = __dsub_rn(__dmul_rn(a1[1], a2[2]), __dmul_rn(a1[2], a2[1]));
  double zx = __dsub_rn(__dmul_rn(a1[2], a2[0]), __dmul_rn(a1[0], a2[2]));
  return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(xy, xy), __dmul_rn(yz, yz)), __dmul_rn(zx, zx)));
}

// Boundary support element matrices: Kf[e][col node b][row node a][i*P+j],
// cs doubles per column; stiffness per element ke[P*e+i], or element-node
// values ken[(npe*e+a)*P+i] interpolated at the points.
template <int BDIM>
__global__ void k_support_elem(const double *__restrict__ xyz, const int32_t *__restrict__ conn, int64_t nel,
                               int npe, int nip, const double *__restrict__ w, const double *__restrict__ N,
                               const double *__restrict__ dN, int P, const double *__restrict__ ke,
                               const double *__restrict__ ken, double thickness, double *__restrict__ Kf,
                               int64_t cs) {
  const int BS = P * P;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nel;
       e += (int64_t)gridDim.x * blockDim.x) {
    double *Ke = Kf + (size_t)e * npe * cs;
    for (int b = 0; b < npe; ++b)
      for (int m = 0; m < npe * BS; ++m) Ke[(size_t)b * cs + m] = 0.0;
    const int32_t *c = conn + (size_t)e * npe;
    for (int q = 0; q < nip; ++q) {
      const double jw = __dmul_rn(boundary_ja<BDIM>(xyz, c, npe, q, dN, thickness), w[q]);
      double kq[3] = {0.0, 0.0, 0.0};
      for (int i = 0; i < P; ++i) {
        if (ken) {
          double acc = 0.0;
          for (int a = 0; a < npe; ++a)
            acc = __fma_rn(N[(size_t)q * npe + a], ken[((size_t)e * npe + a) * P + i], acc);
          kq[i] = acc;
        } else {
          kq[i] = ke[(size_t)e * P + i];
        }
      }
      for (int a = 0; a < npe; ++a) {
        const double naj = __dmul_rn(N[(size_t)q * npe + a], jw);
        for (int b = a; b < npe; ++b) {
          const double Nb = N[(size_t)q * npe + b];
          double *blk = Ke + (size_t)b * cs + (size_t)a * BS;
          for (int i = 0; i < P; ++i) blk[i * P + i] = __fma_rn(__dmul_rn(naj, kq[i]), Nb, blk[i * P + i]);
        }
      }
    }
    for (int a = 0; a < npe; ++a)
      for (int b = a + 1; b < npe; ++b)
        for (int i = 0; i < P; ++i)
          Ke[(size_t)a * cs + (size_t)b * BS + i * P + i] = Ke[(size_t)b * cs + (size_t)a * BS + i * P + i];
  }
}

// externalTangentFollower element matrices (3D faces, P = 3), full and
// unsymmetric: Kf[e][col node b][row node a][ia*3+jb].  Contract of the
// oracle: face Jacobian [t1 t2 n], n = (t1 x t2)/|t1 x t2|, surface
// gradients g_b = Jm^-T (dN/du, dN/dv, 0); per column (b, jb)
// u = alpha tg - s g + c e_jb, dt0 = Jgp Finv^T u, Ke += (N_a jw) dt0.
__global__ void k_follower_elem(const double *__restrict__ xyz, const int32_t *__restrict__ conn, int64_t nel,
                                int npe, int nip, const double *__restrict__ w, const double *__restrict__ N,
                                const double *__restrict__ dN, const double *__restrict__ Fn,
                                const double *__restrict__ te, const double *__restrict__ ten,
                                double *__restrict__ Kf, int64_t cs, unsigned *status) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nel;
       e += (int64_t)gridDim.x * blockDim.x) {
    double *Ke = Kf + (size_t)e * npe * cs;
    for (int b = 0; b < npe; ++b)
      for (int m = 0; m < npe * 9; ++m) Ke[(size_t)b * cs + m] = 0.0;
    const int32_t *c = conn + (size_t)e * npe;
    for (int q = 0; q < nip; ++q) {
      const double *Nq = N + (size_t)q * npe;
      double t1[3], t2[3];
      for (int i = 0; i < 3; ++i) {
        double s1 = 0.0, s2 = 0.0;
        for (int a = 0; a < npe; ++a) {
          const double xa = xyz[(size_t)c[a] * 3 + i];
          s1 = __fma_rn(xa, dN[((size_t)q * npe + a) * 3 + 0], s1);
          s2 = __fma_rn(xa, dN[((size_t)q * npe + a) * 3 + 1], s2);
        }
        t1[i] = s1;
        t2[i] = s2;
      }
      const double xy = __dsub_rn(__dmul_rn(t1[0], t2[1]), __dmul_rn(t1[1], t2[0]));
      const double yz = __dsub_rn(__dmul_rn(t1[1], t2[2]), __dmul_rn(t1[2], t2[1]));
      const double zx = __dsub_rn(__dmul_rn(t1[2], t2[0]), __dmul_rn(t1[0], t2[2]));
      const double da = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(xy, xy), __dmul_rn(yz, yz)), __dmul_rn(zx, zx)));
      const double nrm[3] = {__ddiv_rn(yz, da), __ddiv_rn(zx, da), __ddiv_rn(xy, da)};
      double Jm[3][3], Ji[9], Fq[3][3], Fi[9];
      for (int i = 0; i < 3; ++i) {
        Jm[i][0] = t1[i];
        Jm[i][1] = t2[i];
        Jm[i][2] = nrm[i];
      }
      jac_inverse<3>(Jm, Ji);
      face_F<2>(Fn, c, npe, Nq, Fq);
      const double Jgp = jac_inverse<3>(Fq, Fi);
      if (!(Jgp > 0.0)) atomicOr(status, ST_BAD_JACOBIAN);
      double tq[3], tg[3], tl[3];
      for (int i = 0; i < 3; ++i) {
        if (ten) {
          double acc = 0.0;
          for (int a = 0; a < npe; ++a) acc = __fma_rn(Nq[a], ten[((size_t)e * npe + a) * 3 + i], acc);
          tq[i] = acc;
        } else {
          tq[i] = te[(size_t)e * 3 + i];
        }
      }
      for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int j = 0; j < 3; ++j) acc = __fma_rn(Fq[i][j], tq[j], acc);
        tg[i] = acc;
      }
      for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int j = 0; j < 3; ++j) acc = __fma_rn(Fi[3 * i + j], tg[j], acc);
        tl[i] = acc;
      }
      const double jw = __dmul_rn(da, w[q]);
      for (int b = 0; b < npe; ++b) {
        const double *d = dN + ((size_t)q * npe + b) * 3;
        double g[3];
        for (int i = 0; i < 3; ++i) g[i] = __fma_rn(Ji[3 + i], d[1], __dmul_rn(Ji[i], d[0]));
        double cdot = 0.0;
        for (int i = 0; i < 3; ++i) cdot = __fma_rn(g[i], tl[i], cdot);
        for (int jb = 0; jb < 3; ++jb) {
          double alpha = 0.0, sdot = 0.0;
          for (int i = 0; i < 3; ++i) {
            alpha = __fma_rn(Fi[3 * i + jb], g[i], alpha);
            sdot = __fma_rn(Fi[3 * i + jb], tg[i], sdot);
          }
          double u[3];
          for (int i = 0; i < 3; ++i) u[i] = __dsub_rn(__dmul_rn(alpha, tg[i]), __dmul_rn(sdot, g[i]));
          u[jb] = __dadd_rn(u[jb], cdot);
          double dt0[3];
          for (int i = 0; i < 3; ++i) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k) acc = __fma_rn(Fi[3 * k + i], u[k], acc);
            dt0[i] = __dmul_rn(Jgp, acc);
          }
          double *col = Ke + (size_t)b * cs;
          for (int a = 0; a < npe; ++a) {
            const double nj = __dmul_rn(Nq[a], jw);
            for (int ia = 0; ia < 3; ++ia) {
              double *t = col + (size_t)a * 9 + ia * 3 + jb;
              *t = __fma_rn(nj, dt0[ia], *t);
            }
          }
        }
      }
    }
  }
}

// elementsToNodes: nodal value = (sum of the element-node values of the
// node in element order, from +0) * rcp(count).
__global__ void k_elements_to_nodes(const int64_t *__restrict__ ptr, const int2 *__restrict__ list, int64_t non,
                                    int npe, int ncomp, const double *__restrict__ ev, double *__restrict__ nv) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < non * ncomp;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = t / ncomp;
    const int i = (int)(t - v * ncomp);
    const int64_t s = ptr[v], e = ptr[v + 1];
    double acc = 0.0;
    for (int64_t k = s; k < e; ++k) {
      const int2 el = list[k];
      acc = __dadd_rn(acc, ev[((size_t)el.x * npe + el.y) * ncomp + i]);
    }
    nv[t] = (e > s) ? __dmul_rn(acc, __drcp_rn((double)(e - s))) : 0.0;
  }
}

// f[node*pdim+i] += fe of every element of the node, in element order.
__global__ void k_load_gather(const int64_t *__restrict__ ptr, const int2 *__restrict__ list,
                              int64_t non, int npe, int pdim, const double *__restrict__ fe,
                              double *__restrict__ f) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < non;
       v += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = ptr[v], e = ptr[v + 1];
    if (s == e) continue;
    for (int i = 0; i < pdim; ++i) {
      double acc = f[v * pdim + i];
      for (int64_t k = s; k < e; ++k) {
        const int2 el = list[k];
        acc = __dadd_rn(acc, fe[((size_t)el.x * npe + el.y) * pdim + i]);
      }
      f[v * pdim + i] = acc;
    }
  }
}

// One thread per (element, element node k).
__global__ void k_grad_nodes(const double *__restrict__ xyz, const int32_t *__restrict__ conn,
                             int64_t nel, int npe, const double *__restrict__ dNn,
                             const double *__restrict__ u, int add_identity,
                             double *__restrict__ out, unsigned *status) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nel * npe;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / npe;
    const int k = (int)(t - e * npe);
    const int32_t *c = conn + (size_t)e * npe;
    const double *d = dNn + (size_t)k * npe * 3;
    double J[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double acc = 0.0;
        for (int a = 0; a < npe; ++a) acc = __fma_rn(xyz[(size_t)c[a] * 3 + i], d[a * 3 + j], acc);
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
    double det = __dadd_rn(__dadd_rn(__dmul_rn(J[0][0], c00), __dmul_rn(J[0][1], c01)),
                           __dmul_rn(J[0][2], c02));
    if (!(det > 0.0)) atomicOr(status, ST_BAD_JACOBIAN);
    double r = __drcp_rn(det);
    double inv[9] = {__dmul_rn(c00, r), __dmul_rn(c10, r), __dmul_rn(c20, r),
                     __dmul_rn(c01, r), __dmul_rn(c11, r), __dmul_rn(c21, r),
                     __dmul_rn(c02, r), __dmul_rn(c12, r), __dmul_rn(c22, r)};
    double T[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // T[i][j] = du_i/dX_j
    for (int l = 0; l < npe; ++l) {
      double g[3];
      for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int j = 0; j < 3; ++j) acc = __fma_rn(inv[3 * j + i], d[l * 3 + j], acc);
        g[i] = acc;
      }
      const double *ul = u + (size_t)c[l] * 3;
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) T[i][j] = __fma_rn(g[j], ul[i], T[i][j]);
    }
    double *o = out + (size_t)e * npe * 9 + (size_t)k * 9;
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i)
        o[3 * j + i] = (add_identity && i == j) ? __dadd_rn(T[i][j], 1.0) : T[i][j];
  }
}

inline unsigned grid_1d(int64_t n, int threads, int sms) {
  int64_t b = (n + threads - 1) / threads;
  int64_t cap = (int64_t)sms * 16;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace

int load_vector_impl(llf_ctx *ctx, llf_mesh *bm, int problem_dim, int pdim, const double *t_const,
                     const double *d_tn, double thickness, const double *d_Fn, double *d_f, int64_t ndof) {
  (void)problem_dim;
  (void)ndof;
  cudaStream_t s = ctx->stream;
  double *fe = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &fe, (size_t)bm->nel * bm->npe * pdim));
  double t[3] = {0, 0, 0};
  if (t_const)
    for (int i = 0; i < pdim; ++i) t[i] = t_const[i];
  unsigned g = grid_1d(bm->nel, 128, ctx->num_sms);
  {
    KernelScope ks(ctx, "k_load_elem");
    if (bm->dim == 1)
      k_load_elem<1><<<g, 128, 0, s>>>(bm->d_xyz, bm->d_conn, bm->nel, bm->npe, bm->nip, bm->d_w, bm->d_N,
                                       bm->d_dN, pdim, t[0], t[1], t[2], d_tn, thickness, nullptr, ctx->d_status,
                                       fe);
    else
      k_load_elem<2><<<g, 128, 0, s>>>(bm->d_xyz, bm->d_conn, bm->nel, bm->npe, bm->nip, bm->d_w, bm->d_N,
                                       bm->d_dN, pdim, t[0], t[1], t[2], d_tn, thickness, d_Fn, ctx->d_status,
                                       fe);
  }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  int64_t *ptr = nullptr;
  int2 *list = nullptr;
  int mx = 0;
  int rc = build_n2e(ctx, bm->d_conn, nullptr, bm->nel, bm->npe, bm->non, &ptr, &list, &mx);
  if (rc != LLF_OK) {
    dfree(ctx, fe);
    return rc;
  }
  { KernelScope ks(ctx, "k_load_gather");
  k_load_gather<<<grid_1d(bm->non, 128, ctx->num_sms), 128, 0, s>>>(ptr, list, bm->non, bm->npe, pdim, fe, d_f); }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  dfree(ctx, fe);
  dfree(ctx, ptr);
  dfree(ctx, list);
  return llf_check_status(ctx, "loadVector");
}

// Gather the element matrices Kf (cs doubles per column) of the boundary
// mesh bm into the volume pattern (element order per entry), dropzeros!, and
// free Kf.
static int boundary_matrix_finish(llf_ctx *ctx, llf_pattern *pat, llf_mesh *bm, double *Kf, int64_t cs,
                                  const char *what, llf_matrix *m) {
  int64_t *ptr = nullptr, *cnt = nullptr;
  int2 *list = nullptr;
  uint16_t *pos = nullptr;
  int mx = 0;
  int rc = llf_check_status(ctx, what);
  if (rc == LLF_OK) rc = build_n2e(ctx, bm->d_conn, nullptr, bm->nel, bm->npe, pat->mesh->non, &ptr, &list, &mx);
  if (rc == LLF_OK) rc = row_positions(ctx, pat, bm->d_conn, bm->npe, ptr, list, bm->nel * bm->npe, &pos);
  if (rc == LLF_OK)
    rc = llf_check_status(ctx, (std::string(what) + ": a boundary element pair outside the volume pattern").c_str());
  if (rc == LLF_OK) {
    cudaError_t e = dalloc(ctx, &cnt, pat->ndof + 1);
    if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, sizeof(int64_t) * (pat->ndof + 1), ctx->stream);
    if (e == cudaSuccess) e = dalloc(ctx, &m->d_nz, pat->nnz);
    if (e != cudaSuccess) rc = llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
  }
  if (rc == LLF_OK) rc = gather_full_ext(ctx, pat, ptr, list, pos, bm->npe, Kf, cs, true, m->d_nz, cnt);
  dfree(ctx, Kf);
  dfree(ctx, ptr);
  dfree(ctx, list);
  dfree(ctx, pos);
  if (rc == LLF_OK) rc = llf_check_status(ctx, what);
  if (rc == LLF_OK) rc = matrix_finalize(ctx, m, cnt);
  dfree(ctx, cnt);
  return rc;
}

int support_impl(llf_ctx *ctx, llf_pattern *pat, llf_mesh *bm, const double *d_ke, const double *d_ken,
                 double thickness, llf_matrix *m) {
  const int P = pat->pdim, npe = bm->npe;
  const int64_t cs = kf_colstride(npe, P * P, (int)sizeof(double));
  double *Kf = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &Kf, (size_t)std::max<int64_t>(bm->nel, 1) * npe * cs));
  {
    KernelScope ks(ctx, "k_support_elem");
    const unsigned g = grid_1d(bm->nel, 128, ctx->num_sms);
    if (bm->dim == 1)
      k_support_elem<1><<<g, 128, 0, ctx->stream>>>(bm->d_xyz, bm->d_conn, bm->nel, npe, bm->nip, bm->d_w, bm->d_N,
                                                    bm->d_dN, P, d_ke, d_ken, thickness, Kf, cs);
    else
      k_support_elem<2><<<g, 128, 0, ctx->stream>>>(bm->d_xyz, bm->d_conn, bm->nel, npe, bm->nip, bm->d_w, bm->d_N,
                                                    bm->d_dN, P, d_ke, d_ken, thickness, Kf, cs);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    dfree(ctx, Kf);
    return llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
  }
  return boundary_matrix_finish(ctx, pat, bm, Kf, cs, "elasticSupportMatrix", m);
}

int follower_tangent_impl(llf_ctx *ctx, llf_pattern *pat, llf_mesh *bm, const double *d_Fn, const double *d_te,
                          const double *d_ten, llf_matrix *m) {
  const int npe = bm->npe;
  const int64_t cs = kf_colstride(npe, 9, (int)sizeof(double));
  double *Kf = nullptr;
  LLF_CUDA_TRY(ctx, dalloc(ctx, &Kf, (size_t)std::max<int64_t>(bm->nel, 1) * npe * cs));
  {
    KernelScope ks(ctx, "k_follower_elem");
    k_follower_elem<<<grid_1d(bm->nel, 128, ctx->num_sms), 128, 0, ctx->stream>>>(
        bm->d_xyz, bm->d_conn, bm->nel, npe, bm->nip, bm->d_w, bm->d_N, bm->d_dN, d_Fn, d_te, d_ten, Kf, cs,
        ctx->d_status);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    dfree(ctx, Kf);
    return llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
  }
  return boundary_matrix_finish(ctx, pat, bm, Kf, cs, "externalTangentFollower", m);
}

int elements_to_nodes_impl(llf_ctx *ctx, llf_mesh *mesh, int ncomp, const double *d_ev, double *d_nv) {
  int64_t *ptr = nullptr;
  int2 *list = nullptr;
  int mx = 0;
  int rc = build_n2e(ctx, mesh->d_conn, nullptr, mesh->nel, mesh->npe, mesh->non, &ptr, &list, &mx);
  if (rc != LLF_OK) return rc;
  {
    KernelScope ks(ctx, "k_elements_to_nodes");
    k_elements_to_nodes<<<grid_1d(mesh->non * ncomp, 128, ctx->num_sms), 128, 0, ctx->stream>>>(
        ptr, list, mesh->non, mesh->npe, ncomp, d_ev, d_nv);
  }
  cudaError_t e = cudaGetLastError();
  dfree(ctx, ptr);
  dfree(ctx, list);
  if (e != cudaSuccess) return llf_fail(ctx, LLF_ERR_CUDA, cudaGetErrorString(e));
  return LLF_OK;
}

int node_gather(llf_ctx *ctx, const int32_t *conn, int64_t nel, int npe, int64_t non, int pdim,
                const double *fe, double *f) {
  int64_t *ptr = nullptr;
  int2 *list = nullptr;
  int mx = 0;
  int rc = build_n2e(ctx, conn, nullptr, nel, npe, non, &ptr, &list, &mx);
  if (rc != LLF_OK) return rc;
  {
    KernelScope ks(ctx, "k_node_gather");
    k_load_gather<<<grid_1d(non, 128, ctx->num_sms), 128, 0, ctx->stream>>>(ptr, list, non, npe, pdim, fe, f);
  }
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  dfree(ctx, ptr);
  dfree(ctx, list);
  return LLF_OK;
}

int grad_elementwise_impl(llf_ctx *ctx, llf_mesh *m, const double *d_u, int add_identity,
                          double *d_out) {
  KernelScope ks(ctx, "k_grad_nodes");
  k_grad_nodes<<<grid_1d(m->nel * m->npe, 128, ctx->num_sms), 128, 0, ctx->stream>>>(
      m->d_xyz, m->d_conn, m->nel, m->npe, m->d_dNn, d_u, add_identity, d_out, ctx->d_status);
  LLF_CUDA_TRY(ctx, cudaGetLastError());
  return llf_check_status(ctx, "grad");
}
