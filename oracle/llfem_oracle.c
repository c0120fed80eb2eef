/*
 * llfem_oracle.c — CPU oracle for the operator-assembly + solve hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the algorithms
 * of LowLevelFEM.jl v1.13.31 that the GPU library replaces.  It is used only
 * by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, always
 * as the checker or the timed CPU baseline, never as the product.
 *
 * Parity pins: the oracle is checked against the reference's own published
 * numbers (examples/dev/compare_LLFEM_Ferrite_dealII_Gridap/results.txt:7,
 * test/test_validation.jl, test/test_integration.jl, test/test_dsl.jl
 * resultants, pattern counts of examples/dev/DSL_vs_legacy*.ipynb).
 *
 * Arithmetic contract shared with the CUDA kernels (both compiled without
 * floating-point contraction; every fused multiply-add is an explicit fma):
 *   geometry at an integration point q (element nodes X[a][i]):
 *     J[i][j]  = fma-chain over a of X[a][i] * dN[q][a][j]       (from 0.0)
 *     cofactors c, det = (J00 c00 + J01 c01) + J02 c02 (3D) or
 *                 J00 J11 - J01 J10 (2D);  rdet = 1/det
 *     invJ[i][j] = c[j][i] * rdet
 *     g[a][i]  = fma-chain over j of invJ[j][i] * dN[q][a][j]    (J^-T grad)
 *     wdet     = det * w[q];   s[a][i] = wdet * g[a][i]
 *   node-pair block a <= b:
 *     O[i][j]  = fma-chain over q of s[a][i](q) * g[b][j](q)  (a == b: i <= j
 *                computed, O[j][i] = O[i][j])
 *     elastic  K[i][j] = fma(mub, O[j][i], lamb*O[i][j]) (+ fma(mub, tr, .)
 *              on i == j, tr = O00 + O11 (+ O22))
 *     heat     K = kb * (fma-chain over q, then i, of s[a][i] g[b][i])
 *     mass     M = rb * (fma-chain over q of (wdet N[a]) * N[b]), identity
 *              over the pdim components
 *   the element matrix is exactly symmetric: block (b,a) = block(a,b)^T.
 *   global: contributions to one entry are summed in element order,
 *   left to right, starting from the first one (SparseArrays.sparse's input
 *   order); exact zeros are then removed (dropzeros!).
 * The element formulas are the B^T D B, H^T H and B^T B products of
 * src/linear.jl:154-330, :1854-2004 and src/heat.jl:36-137 written in
 * node-pair form (for isotropic Hooke D: K_ab = lambda g_a g_b^T +
 * mu g_b g_a^T + mu (g_a . g_b) I).  Julia's BLAS summation order inside
 * B^T D B cannot be reproduced on any other machine, so this contract fixes
 * an order of its own; values agree with the reference to rounding.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_ELASTIC 0
#define ORC_HEAT 1
#define ORC_MASS 2

#define PT_SOLID 0
#define PT_PLANE_STRESS 1
#define PT_PLANE_STRAIN 2
#define PT_HEAT 3
#define PT_PLANE_HEAT 4
/* DSL forms (src/multifield.jl): coefficients given as they are (ELASTIC:
 * lambda, mu; HEAT: k; MASS: c), b = 1 */
#define PT_LAME (-1)

/* ------------------------------------------------------------------------ */
/* Material constants: elastic_constants (src/general.jl:142-203) and the    */
/* D matrices of constitutive_matrix (src/linear.jl:154-188) in Lame form.  */
/* ------------------------------------------------------------------------ */
void orc_lame(int ptype, double E, double nu, double thickness, double *lamb,
              double *mub) {
  double mu = E / (2.0 * (1.0 + nu));
  double lam, b = 1.0;
  if (ptype == PT_PLANE_STRESS) {
    lam = E * nu / ((1.0 - nu) * (1.0 + nu));
    b = thickness;
  } else {
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  }
  *lamb = lam * b;
  *mub = mu * b;
}

/* ------------------------------------------------------------------------ */
/* Geometry at one integration point (the shared arithmetic contract).      */
/* Returns det.                                                             */
/* ------------------------------------------------------------------------ */
static double orc_inv3(const double J[3][3], double invJ[9]);

static double orc_geom(int dim, int npe, const double *X, const double *dNq,
                       double invJ[9]) {
  double J[3][3] = {{0}};
  for (int i = 0; i < dim; ++i)
    for (int j = 0; j < dim; ++j) {
      double acc = 0.0;
      for (int a = 0; a < npe; ++a) acc = fma(X[3 * a + i], dNq[3 * a + j], acc);
      J[i][j] = acc;
    }
  if (dim == 3) return orc_inv3(J, invJ);
  double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
  double rdet = 1.0 / det;
  invJ[0] = J[1][1] * rdet;   invJ[1] = -J[0][1] * rdet; invJ[2] = 0.0;
  invJ[3] = -J[1][0] * rdet;  invJ[4] = J[0][0] * rdet;  invJ[5] = 0.0;
  invJ[6] = 0.0; invJ[7] = 0.0; invJ[8] = 0.0;
  return det;
}

/* 3x3 inverse by cofactors, invJ row-major; returns det. */
static double orc_inv3(const double J[3][3], double invJ[9]) {
  double det, rdet;
  {
    double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    double c01 = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]);
    double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    double c10 = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]);
    double c11 = J[0][0] * J[2][2] - J[0][2] * J[2][0];
    double c12 = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]);
    double c20 = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    double c21 = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]);
    double c22 = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    det = (J[0][0] * c00 + J[0][1] * c01) + J[0][2] * c02;
    rdet = 1.0 / det;
    /* invJ[i][j] = c[j][i] * rdet, stored row-major */
    invJ[0] = c00 * rdet; invJ[1] = c10 * rdet; invJ[2] = c20 * rdet;
    invJ[3] = c01 * rdet; invJ[4] = c11 * rdet; invJ[5] = c21 * rdet;
    invJ[6] = c02 * rdet; invJ[7] = c12 * rdet; invJ[8] = c22 * rdet;
  }
  return det;
}

/* Physical gradients g[q][a][i] and weighted s = wdet*g for all points.
 * Returns 0, or -1 on a non-positive Jacobian determinant. */
static int orc_grads(int dim, int npe, int nip, const double *w,
                     const double *dN, const double *X, double *g, double *s,
                     double *wdet) {
  for (int q = 0; q < nip; ++q) {
    double invJ[9];
    double det = orc_geom(dim, npe, X, dN + (size_t)q * npe * 3, invJ);
    if (!(det > 0.0)) return -1;
    double wd = det * w[q];
    wdet[q] = wd;
    for (int a = 0; a < npe; ++a) {
      const double *d = dN + ((size_t)q * npe + a) * 3;
      for (int i = 0; i < dim; ++i) {
        double acc = 0.0;
        for (int j = 0; j < dim; ++j) acc = fma(invJ[3 * j + i], d[j], acc);
        g[((size_t)q * npe + a) * 3 + i] = acc;
        s[((size_t)q * npe + a) * 3 + i] = wd * acc;
      }
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Affine elements.  When the element's nodes are an affine image of the     */
/* reference nodes (every straight-sided element), J is the same at every    */
/* point and the quadrature factors through reference matrices:              */
/*   O_ab = det J^-T R_ab J^-1,  R_ab[k][l] = sum_q w_q dN_a,k dN_b,l,        */
/*   M_ab = det Mref_ab,         Mref_ab    = sum_q w_q N_a N_b.              */
/* Contract: R and Mref are fma chains over q of (w_q * first) * second;     */
/* J0, det, invJ as the geometry contract at point 0; an element is affine   */
/* when every node satisfies |X_a - X_0 - J0 (xi_a - xi_0)| <= 64 eps s      */
/* componentwise (fma chain over j), s the largest |X| of the element.       */
/* ------------------------------------------------------------------------ */
void orc_affine_tables(int npe, int nip, const double *w, const double *N, const double *dN,
                       double *R, double *Mref) {
  for (int a = 0; a < npe; ++a)
    for (int b = 0; b < npe; ++b) {
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) {
          double acc = 0.0;
          for (int q = 0; q < nip; ++q)
            acc = fma(w[q] * dN[((size_t)q * npe + a) * 3 + k], dN[((size_t)q * npe + b) * 3 + l], acc);
          R[((size_t)a * npe + b) * 9 + k * 3 + l] = acc;
        }
      double m = 0.0;
      for (int q = 0; q < nip; ++q) m = fma(w[q] * N[(size_t)q * npe + a], N[(size_t)q * npe + b], m);
      Mref[(size_t)a * npe + b] = m;
    }
}

static int orc_is_affine(int dim, int npe, const double *X, const double *dN0, const double *nref) {
  double J[3][3] = {{0}};
  for (int i = 0; i < dim; ++i)
    for (int j = 0; j < dim; ++j) {
      double acc = 0.0;
      for (int a = 0; a < npe; ++a) acc = fma(X[3 * a + i], dN0[3 * a + j], acc);
      J[i][j] = acc;
    }
  double s = 0.0;
  for (int a = 0; a < npe; ++a)
    for (int i = 0; i < dim; ++i) s = fmax(s, fabs(X[3 * a + i]));
  const double tol = 64.0 * 2.220446049250313e-16 * s;
  for (int a = 0; a < npe; ++a)
    for (int i = 0; i < dim; ++i) {
      double t = X[3 * a + i] - X[i];
      for (int j = 0; j < dim; ++j) t = fma(-J[i][j], nref[3 * a + j] - nref[j], t);
      if (!(fabs(t) <= tol)) return 0;
    }
  return s > 0.0;
}

/* Affine-element matrix; returns -1 for det <= 0.
 * R_ab splits into its symmetric part S (components n = (k,l), k <= l, in the
 * order 00 11 22 01 02 12; 2D: 00 11 01; S_kl = (R_kl + R_lk) * 0.5) and its
 * antisymmetric part A (01 02 12; 2D: 01; A_kl = (R_kl - R_lk) * 0.5).  With
 * O = det J^-T R J^-1 = Os + Oa, the element's coefficients
 *   V[m][n] = det * inv_ki inv_kj                      (k == l)
 *           = det * fma(inv_ki, inv_lj, inv_li inv_kj)  (k <  l)   m = (i,j)
 *   U[m][n] = cm * (det * fma(inv_ki, inv_lj, -(inv_li inv_kj)))
 * (inv_ki = invJ[k][i]) map S and A to Os and Oa, and the Lame combination
 * K = c1 O + c2 O^T + c2 tr(O) I becomes, with cp = c1 + c2, cm = c1 - c2,
 *   Ksym = W S,  W[m][n] = fma(c2, trV[n], cp*V[m][n]) (m diagonal) or cp*V[m][n],
 *   Kanti = U A,  K_ii = Ksym_ii,  K_ij = Ksym_ij + Kanti_ij,  K_ji = Ksym_ij - Kanti_ij
 * (a == b: A = 0, K_ij = K_ji = Ksym_ij); heat: (c1 trV) . S; mass: (c1 det) Mref.
 * Products with W, U, c1 trV are fma chains over n from 0.0. */
static const int ORC_SYM3[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
static const int ORC_SYM2[3][2] = {{0, 0}, {1, 1}, {0, 1}};

void orc_affine_split(int dim, const double *Rab, double *sv, double *av) {
  const int ns = dim == 3 ? 6 : 3, na = dim == 3 ? 3 : 1;
  const int(*sym)[2] = dim == 3 ? ORC_SYM3 : ORC_SYM2;
  for (int n = 0; n < ns; ++n) {
    int k = sym[n][0], l = sym[n][1];
    sv[n] = k == l ? Rab[k * 3 + k] : (Rab[k * 3 + l] + Rab[l * 3 + k]) * 0.5;
  }
  for (int n = 0; n < na; ++n) {
    int k = sym[dim + n][0], l = sym[dim + n][1];
    av[n] = (Rab[k * 3 + l] - Rab[l * 3 + k]) * 0.5;
  }
}

/* Geometry of an affine element: J0 as the geometry contract at point 0;
 * when every off-diagonal entry of J0 is within the affinity tolerance
 * (|J0_ij| <= 64 eps s, s the largest |X| of the element) the element is an
 * axis-aligned brick up to the rounding of the sums, and those entries are
 * set to +0.0 before the inverse, so that invJ and every coefficient below
 * that mixes two axes are exact zeros.  Returns det; *aligned = 1 then. */
static double orc_geom_affine(int dim, int npe, const double *X, const double *dN0, double inv[9],
                              int *aligned) {
  double J[3][3] = {{0}};
  for (int i = 0; i < dim; ++i)
    for (int j = 0; j < dim; ++j) {
      double acc = 0.0;
      for (int a = 0; a < npe; ++a) acc = fma(X[3 * a + i], dN0[3 * a + j], acc);
      J[i][j] = acc;
    }
  double s = 0.0;
  for (int a = 0; a < npe; ++a)
    for (int i = 0; i < dim; ++i) s = fmax(s, fabs(X[3 * a + i]));
  const double tol = 64.0 * 2.220446049250313e-16 * s;
  int al = 1;
  for (int i = 0; i < dim; ++i)
    for (int j = 0; j < dim; ++j)
      if (i != j && !(fabs(J[i][j]) <= tol)) al = 0;
  if (al)
    for (int i = 0; i < dim; ++i)
      for (int j = 0; j < dim; ++j)
        if (i != j) J[i][j] = 0.0;
  *aligned = al;
  if (dim == 3) return orc_inv3(J, inv);
  double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
  double rdet = 1.0 / det;
  inv[0] = J[1][1] * rdet;   inv[1] = -J[0][1] * rdet; inv[2] = 0.0;
  inv[3] = -J[1][0] * rdet;  inv[4] = J[0][0] * rdet;  inv[5] = 0.0;
  inv[6] = 0.0; inv[7] = 0.0; inv[8] = 0.0;
  return det;
}

/* Elasticity on an axis-aligned affine element (invJ diagonal: d_k =
 * invJ[k][k]).  With V_n = det (d_k d_l) for the symmetric component
 * n = (k,l), the Lame combination collapses to
 *   K_ii = (c1 + c2) V_i S_i + c2 sum_n<dim V_n S_n,
 *   K_ij = (c1 + c2) V_m S_m + (c1 - c2) V_m A_m,  K_ji = (c1 + c2) V_m S_m - (c1 - c2) V_m A_m
 * (m = (i,j) mixed; A = 0 when a == b).  Contract: alpha_i = cp V_i,
 * beta_i = c2 V_i, a_m = cp V_m, b_m = cm V_m; per pair
 * g = fma chain over n < dim of beta_n S_n (from beta_0 S_0),
 * K_ii = fma(alpha_i, S_i, g), h_m = b_m A_m, K_ij = fma(a_m, S_m, h_m),
 * K_ji = fma(a_m, S_m, -h_m); a == b: K_ij = K_ji = a_m S_m.
 * 15 FP64 operations per node pair in 3D. */
static int orc_element_aligned(int dim, int npe, const double *inv, double det, const double *R, double c1,
                               double c2, double *Ke) {
  const int ns = dim == 3 ? 6 : 3, na = dim == 3 ? 3 : 1;
  const int(*sym)[2] = dim == 3 ? ORC_SYM3 : ORC_SYM2;
  const size_t nd = (size_t)dim * npe;
  double V[6], alpha[3], beta[3], am[3], bm[3];
  for (int n = 0; n < ns; ++n) {
    int k = sym[n][0], l = sym[n][1];
    V[n] = det * (inv[k * 3 + k] * inv[l * 3 + l]);
  }
  const double cp = c1 + c2, cm = c1 - c2;
  for (int i = 0; i < dim; ++i) {
    alpha[i] = cp * V[i];
    beta[i] = c2 * V[i];
  }
  for (int m = 0; m < na; ++m) {
    am[m] = cp * V[dim + m];
    bm[m] = cm * V[dim + m];
  }
  memset(Ke, 0, sizeof(double) * nd * nd);
  for (int a = 0; a < npe; ++a)
    for (int b = a; b < npe; ++b) {
      double sv[6], av[3], blk[9] = {0};
      orc_affine_split(dim, R + ((size_t)a * npe + b) * 9, sv, av);
      double g = beta[0] * sv[0];
      for (int n = 1; n < dim; ++n) g = fma(beta[n], sv[n], g);
      for (int i = 0; i < dim; ++i) blk[i * dim + i] = fma(alpha[i], sv[i], g);
      for (int m = 0; m < na; ++m) {
        int i = sym[dim + m][0], j = sym[dim + m][1];
        if (a != b) {
          double h = bm[m] * av[m];
          blk[i * dim + j] = fma(am[m], sv[dim + m], h);
          blk[j * dim + i] = fma(am[m], sv[dim + m], -h);
        } else {
          blk[i * dim + j] = blk[j * dim + i] = am[m] * sv[dim + m];
        }
      }
      for (int i = 0; i < dim; ++i)
        for (int j = 0; j < dim; ++j) {
          double v = blk[i * dim + j];
          Ke[((size_t)a * dim + i) * nd + (size_t)b * dim + j] = v;
          Ke[((size_t)b * dim + j) * nd + (size_t)a * dim + i] = v;
        }
    }
  return 0;
}

static int orc_element_affine(int kind, int dim, int pdim, int npe, const double *dN0, const double *X,
                              const double *R, const double *Mref, double c1, double c2, double *Ke) {
  size_t nd = (size_t)pdim * npe;
  double inv[9];
  int aligned = 0;
  double det = orc_geom_affine(dim, npe, X, dN0, inv, &aligned);
  if (!(det > 0.0)) return -1;
  if (aligned && kind == ORC_ELASTIC) return orc_element_aligned(dim, npe, inv, det, R, c1, c2, Ke);
  const int ns = dim == 3 ? 6 : 3, na = dim == 3 ? 3 : 1;
  const int(*sym)[2] = dim == 3 ? ORC_SYM3 : ORC_SYM2;
  double V[6][6], trV[6], W[6][6], U[3][3], Qh[6];
  for (int m = 0; m < ns; ++m)
    for (int n = 0; n < ns; ++n) {
      int i = sym[m][0], j = sym[m][1], k = sym[n][0], l = sym[n][1];
      V[m][n] = k == l ? det * (inv[k * 3 + i] * inv[k * 3 + j])
                       : det * fma(inv[k * 3 + i], inv[l * 3 + j], inv[l * 3 + i] * inv[k * 3 + j]);
    }
  for (int n = 0; n < ns; ++n) trV[n] = dim == 3 ? (V[0][n] + V[1][n]) + V[2][n] : V[0][n] + V[1][n];
  const double cp = c1 + c2, cm = c1 - c2;
  for (int m = 0; m < ns; ++m)
    for (int n = 0; n < ns; ++n) W[m][n] = m < dim ? fma(c2, trV[n], cp * V[m][n]) : cp * V[m][n];
  for (int m = 0; m < na; ++m)
    for (int n = 0; n < na; ++n) {
      int i = sym[dim + m][0], j = sym[dim + m][1], k = sym[dim + n][0], l = sym[dim + n][1];
      U[m][n] = cm * (det * fma(inv[k * 3 + i], inv[l * 3 + j], -(inv[l * 3 + i] * inv[k * 3 + j])));
    }
  for (int n = 0; n < ns; ++n) Qh[n] = c1 * trV[n];
  const double cmass = c1 * det;
  memset(Ke, 0, sizeof(double) * nd * nd);
  for (int a = 0; a < npe; ++a)
    for (int b = a; b < npe; ++b) {
      double blk[9] = {0};
      if (kind == ORC_MASS) {
        double mv = cmass * Mref[(size_t)a * npe + b];
        for (int i = 0; i < pdim; ++i) blk[i * pdim + i] = mv;
      } else {
        double sv[6], av[3];
        orc_affine_split(dim, R + ((size_t)a * npe + b) * 9, sv, av);
        if (kind == ORC_HEAT) {
          double acc = 0.0;
          for (int n = 0; n < ns; ++n) acc = fma(Qh[n], sv[n], acc);
          blk[0] = acc;
        } else {
          double ks[6], ka[3] = {0.0, 0.0, 0.0};
          for (int m = 0; m < ns; ++m) {
            double acc = 0.0;
            for (int n = 0; n < ns; ++n) acc = fma(W[m][n], sv[n], acc);
            ks[m] = acc;
          }
          if (a != b)
            for (int m = 0; m < na; ++m) {
              double acc = 0.0;
              for (int n = 0; n < na; ++n) acc = fma(U[m][n], av[n], acc);
              ka[m] = acc;
            }
          for (int i = 0; i < dim; ++i) blk[i * pdim + i] = ks[i];
          for (int m = 0; m < na; ++m) {
            int i = sym[dim + m][0], j = sym[dim + m][1];
            blk[i * pdim + j] = a != b ? ks[dim + m] + ka[m] : ks[dim + m];
            blk[j * pdim + i] = a != b ? ks[dim + m] - ka[m] : ks[dim + m];
          }
        }
      }
      for (int i = 0; i < pdim; ++i)
        for (int j = 0; j < pdim; ++j) {
          double v = blk[i * pdim + j];
          Ke[((size_t)a * pdim + i) * nd + (size_t)b * pdim + j] = v;
          Ke[((size_t)b * pdim + j) * nd + (size_t)a * pdim + i] = v;
        }
    }
  return 0;
}

/* Element matrix Ke (row-major, (pdim*npe)^2) under the arithmetic contract.
 * kind ORC_ELASTIC: c1 = lamb, c2 = mub; ORC_HEAT: c1 = kb; ORC_MASS: c1 = rb.
 * pdim = dim for elastic, dim for mass (vector problems) or 1, 1 for heat.
 * nref/R/Mref (may be NULL) enable the affine-element form. */
int orc_element_matrix_ex(int kind, int dim, int pdim, int npe, int nip,
                          const double *w, const double *N, const double *dN,
                          const double *X, double c1, double c2, const double *nref,
                          const double *R, const double *Mref, double *Ke);

int orc_element_matrix(int kind, int dim, int pdim, int npe, int nip,
                       const double *w, const double *N, const double *dN,
                       const double *X, double c1, double c2, double *Ke) {
  return orc_element_matrix_ex(kind, dim, pdim, npe, nip, w, N, dN, X, c1, c2, NULL, NULL, NULL, Ke);
}

int orc_element_matrix_ex(int kind, int dim, int pdim, int npe, int nip,
                          const double *w, const double *N, const double *dN,
                          const double *X, double c1, double c2, const double *nref,
                          const double *R, const double *Mref, double *Ke) {
  if (nref && R && Mref && orc_is_affine(dim, npe, X, dN, nref))
    return orc_element_affine(kind, dim, pdim, npe, dN, X, R, Mref, c1, c2, Ke);
  size_t nd = (size_t)pdim * npe;
  double *g = (double *)malloc(sizeof(double) * nip * npe * 3);
  double *s = (double *)malloc(sizeof(double) * nip * npe * 3);
  double *wdet = (double *)malloc(sizeof(double) * nip);
  int rc = orc_grads(dim, npe, nip, w, dN, X, g, s, wdet);
  if (rc) {
    free(g); free(s); free(wdet);
    return rc;
  }
  memset(Ke, 0, sizeof(double) * nd * nd);
  for (int a = 0; a < npe; ++a) {
    for (int b = a; b < npe; ++b) {
      double blk[9] = {0};
      if (kind == ORC_ELASTIC) {
        double O[3][3] = {{0}};
        for (int i = 0; i < dim; ++i)
          for (int j = (a == b ? i : 0); j < dim; ++j) {
            double acc = 0.0;
            for (int q = 0; q < nip; ++q)
              acc = fma(s[((size_t)q * npe + a) * 3 + i],
                        g[((size_t)q * npe + b) * 3 + j], acc);
            O[i][j] = acc;
            if (a == b) O[j][i] = acc;
          }
        double tr = O[0][0] + O[1][1];
        if (dim == 3) tr = tr + O[2][2];
        for (int i = 0; i < dim; ++i)
          for (int j = 0; j < dim; ++j) {
            double t = fma(c2, O[j][i], c1 * O[i][j]);
            if (i == j) t = fma(c2, tr, t);
            blk[i * pdim + j] = t;
          }
      } else if (kind == ORC_HEAT) {
        double acc = 0.0;
        for (int q = 0; q < nip; ++q)
          for (int i = 0; i < dim; ++i)
            acc = fma(s[((size_t)q * npe + a) * 3 + i],
                      g[((size_t)q * npe + b) * 3 + i], acc);
        blk[0] = c1 * acc;
      } else { /* mass */
        double acc = 0.0;
        for (int q = 0; q < nip; ++q)
          acc = fma(wdet[q] * N[(size_t)q * npe + a], N[(size_t)q * npe + b], acc);
        double m = c1 * acc;
        for (int i = 0; i < pdim; ++i) blk[i * pdim + i] = m;
      }
      for (int i = 0; i < pdim; ++i)
        for (int j = 0; j < pdim; ++j) {
          double v = blk[i * pdim + j];
          Ke[((size_t)a * pdim + i) * nd + (size_t)b * pdim + j] = v;
          Ke[((size_t)b * pdim + j) * nd + (size_t)a * pdim + i] = v;
        }
    }
  }
  free(g); free(s); free(wdet);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Structural CSC pattern: build_csc_pattern, src/multifield.jl:2083-2250.   */
/* Node adjacency through shared elements, sorted + unique per node, then   */
/* expanded to pdim components (rows (A-1)*pdim+i sorted inside a column).   */
/* ------------------------------------------------------------------------ */
static int cmp_i64(const void *x, const void *y) {
  int64_t a = *(const int64_t *)x, b = *(const int64_t *)y;
  return (a > b) - (a < b);
}

typedef struct {
  int64_t n, nnz;
  int64_t *colptr; /* 0-based, n+1 */
  int64_t *rowval; /* 0-based      */
  double *nzval;
} orc_csc;

/* node adjacency lists (CSR by column node), 0-based */
static void node_adjacency(int64_t non, int64_t nel, int npe,
                           const int32_t *conn, const int32_t *emat,
                           int64_t **nptr_out, int64_t **nadj_out) {
  /* node -> elements */
  int64_t *cnt = (int64_t *)calloc(non + 1, sizeof(int64_t));
  for (int64_t e = 0; e < nel; ++e) {
    if (emat && emat[e] < 0) continue;
    for (int a = 0; a < npe; ++a) cnt[conn[e * npe + a] + 1]++;
  }
  for (int64_t i = 0; i < non; ++i) cnt[i + 1] += cnt[i];
  int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (non + 1));
  memcpy(fill, cnt, sizeof(int64_t) * (non + 1));
  int64_t *n2e = (int64_t *)malloc(sizeof(int64_t) * (cnt[non] + 1));
  for (int64_t e = 0; e < nel; ++e) {
    if (emat && emat[e] < 0) continue;
    for (int a = 0; a < npe; ++a) n2e[fill[conn[e * npe + a]]++] = e;
  }
  /* adjacency */
  int64_t *nptr = (int64_t *)calloc(non + 1, sizeof(int64_t));
  int64_t cap = 0;
  for (int64_t B = 0; B < non; ++B) {
    int64_t m = (cnt[B + 1] - cnt[B]) * npe;
    if (m > cap) cap = m;
  }
  int64_t *buf = (int64_t *)malloc(sizeof(int64_t) * (cap + 1));
  int64_t total = 0;
  int64_t *adj = NULL;
  for (int pass = 0; pass < 2; ++pass) {
    total = 0;
    for (int64_t B = 0; B < non; ++B) {
      int64_t m = 0;
      for (int64_t k = cnt[B]; k < cnt[B + 1]; ++k) {
        int64_t e = n2e[k];
        for (int a = 0; a < npe; ++a) buf[m++] = conn[e * npe + a];
      }
      qsort(buf, m, sizeof(int64_t), cmp_i64);
      int64_t u = 0;
      for (int64_t k = 0; k < m; ++k)
        if (k == 0 || buf[k] != buf[k - 1]) buf[u++] = buf[k];
      if (pass == 0) {
        nptr[B + 1] = u;
      } else {
        memcpy(adj + nptr[B], buf, sizeof(int64_t) * u);
      }
      total += u;
    }
    if (pass == 0) {
      for (int64_t B = 0; B < non; ++B) nptr[B + 1] += nptr[B];
      adj = (int64_t *)malloc(sizeof(int64_t) * (total + 1));
    }
  }
  free(buf); free(n2e); free(fill); free(cnt);
  *nptr_out = nptr;
  *nadj_out = adj;
}

orc_csc *orc_pattern(int64_t non, int64_t nel, int npe, const int32_t *conn,
                     const int32_t *emat, int pdim) {
  int64_t *nptr, *adj;
  node_adjacency(non, nel, npe, conn, emat, &nptr, &adj);
  orc_csc *m = (orc_csc *)calloc(1, sizeof(orc_csc));
  m->n = non * pdim;
  m->nnz = nptr[non] * pdim * pdim;
  m->colptr = (int64_t *)malloc(sizeof(int64_t) * (m->n + 1));
  m->rowval = (int64_t *)malloc(sizeof(int64_t) * (m->nnz + 1));
  m->nzval = (double *)calloc(m->nnz + 1, sizeof(double));
  int64_t p = 0;
  for (int64_t B = 0; B < non; ++B)
    for (int j = 0; j < pdim; ++j) {
      m->colptr[B * pdim + j] = p;
      for (int64_t k = nptr[B]; k < nptr[B + 1]; ++k)
        for (int i = 0; i < pdim; ++i) m->rowval[p++] = adj[k] * pdim + i;
    }
  m->colptr[m->n] = p;
  free(nptr); free(adj);
  return m;
}

void orc_free(orc_csc *m) {
  if (!m) return;
  free(m->colptr); free(m->rowval); free(m->nzval); free(m);
}
int64_t orc_n(const orc_csc *m) { return m->n; }
int64_t orc_nnz(const orc_csc *m) { return m->nnz; }
void orc_export(const orc_csc *m, int64_t *colptr, int64_t *rowval, double *nzval) {
  if (colptr) memcpy(colptr, m->colptr, sizeof(int64_t) * (m->n + 1));
  if (rowval) memcpy(rowval, m->rowval, sizeof(int64_t) * m->nnz);
  if (nzval) memcpy(nzval, m->nzval, sizeof(double) * m->nnz);
}

/* ------------------------------------------------------------------------ */
/* sparse(I, J, V, n, n) with duplicates combined left-to-right in input     */
/* order (SparseArrays stdlib, as called at src/linear.jl:323), then         */
/* dropzeros! (src/linear.jl:324).  Triplets are streamed element by element */
/* in element order, so the combine order per entry is the element order.    */
/* ------------------------------------------------------------------------ */
typedef struct {
  int64_t n, cap, len;
  int64_t *I, *J;
  double *V;
} coo;

static void coo_push(coo *c, int64_t i, int64_t j, double v) {
  if (c->len == c->cap) {
    c->cap = c->cap ? c->cap * 2 : 1024;
    c->I = (int64_t *)realloc(c->I, sizeof(int64_t) * c->cap);
    c->J = (int64_t *)realloc(c->J, sizeof(int64_t) * c->cap);
    c->V = (double *)realloc(c->V, sizeof(double) * c->cap);
  }
  c->I[c->len] = i;
  c->J[c->len] = j;
  c->V[c->len] = v;
  c->len++;
}

/* Returns CSC with summed duplicates (structural zeros kept). */
static orc_csc *coo_to_csc(coo *c) {
  int64_t n = c->n, L = c->len;
  /* stable bucket by column */
  int64_t *cptr = (int64_t *)calloc(n + 1, sizeof(int64_t));
  for (int64_t k = 0; k < L; ++k) cptr[c->J[k] + 1]++;
  for (int64_t j = 0; j < n; ++j) cptr[j + 1] += cptr[j];
  int64_t *pos = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
  memcpy(pos, cptr, sizeof(int64_t) * (n + 1));
  int64_t *perm = (int64_t *)malloc(sizeof(int64_t) * (L + 1));
  for (int64_t k = 0; k < L; ++k) perm[pos[c->J[k]]++] = k;
  /* combine duplicates per column in input order using a last-touched map */
  int64_t *last = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
  for (int64_t i = 0; i < n; ++i) last[i] = -1;
  orc_csc *m = (orc_csc *)calloc(1, sizeof(orc_csc));
  m->n = n;
  m->colptr = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
  m->rowval = (int64_t *)malloc(sizeof(int64_t) * (L + 1));
  m->nzval = (double *)malloc(sizeof(double) * (L + 1));
  int64_t out = 0;
  for (int64_t j = 0; j < n; ++j) {
    int64_t start = out;
    m->colptr[j] = start;
    for (int64_t t = cptr[j]; t < cptr[j + 1]; ++t) {
      int64_t k = perm[t];
      int64_t i = c->I[k];
      if (last[i] >= start) {
        m->nzval[last[i]] = m->nzval[last[i]] + c->V[k];
      } else {
        last[i] = out;
        m->rowval[out] = i;
        m->nzval[out] = c->V[k];
        out++;
      }
    }
    /* sort rows of this column (values move with rows) */
    int64_t len = out - start;
    for (int64_t a = 1; a < len; ++a) {
      int64_t r = m->rowval[start + a];
      double v = m->nzval[start + a];
      int64_t b = a - 1;
      while (b >= 0 && m->rowval[start + b] > r) {
        m->rowval[start + b + 1] = m->rowval[start + b];
        m->nzval[start + b + 1] = m->nzval[start + b];
        --b;
      }
      m->rowval[start + b + 1] = r;
      m->nzval[start + b + 1] = v;
    }
  }
  m->colptr[n] = out;
  m->nnz = out;
  free(cptr); free(pos); free(perm); free(last);
  return m;
}

/* dropzeros! in place */
void orc_dropzeros(orc_csc *m) {
  int64_t out = 0;
  for (int64_t j = 0; j < m->n; ++j) {
    int64_t s = m->colptr[j], e = m->colptr[j + 1];
    m->colptr[j] = out;
    for (int64_t k = s; k < e; ++k)
      if (m->nzval[k] != 0.0) {
        m->rowval[out] = m->rowval[k];
        m->nzval[out] = m->nzval[k];
        out++;
      }
  }
  m->colptr[m->n] = out;
  m->nnz = out;
}

/* Lumped mass: spdiagm(vec(sum(M, dims=2))) (src/linear.jl:1999-2001);
 * row sums accumulated column by column in column order from 0.0. */
static orc_csc *orc_lump(const orc_csc *M) {
  int64_t n = M->n;
  double *r = (double *)calloc(n + 1, sizeof(double));
  for (int64_t j = 0; j < n; ++j)
    for (int64_t k = M->colptr[j]; k < M->colptr[j + 1]; ++k)
      r[M->rowval[k]] = r[M->rowval[k]] + M->nzval[k];
  orc_csc *D = (orc_csc *)calloc(1, sizeof(orc_csc));
  D->n = n;
  D->nnz = n;
  D->colptr = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
  D->rowval = (int64_t *)malloc(sizeof(int64_t) * (n + 1));
  D->nzval = r;
  for (int64_t j = 0; j <= n; ++j) D->colptr[j] = j;
  for (int64_t j = 0; j < n; ++j) D->rowval[j] = j;
  return D;
}

/* ------------------------------------------------------------------------ */
/* Assembly, restating stiffnessMatrixSolid (src/linear.jl:190-330),         */
/* massMatrixSolid (:1854-2004) and heatCondMatrixSolid (src/heat.jl:36-137): */
/* element loop in element order, per-element matrix, triplets with the      */
/* transposed placement I = dof(l), J = dof(k), V = K1[k,l] (:258-259,       */
/* :314-316), then sparse + dropzeros!.                                      */
/*   params: per material (ELASTIC: E, nu; HEAT: k; MASS: rho), stride np.   */
/* Returns NULL on a non-positive Jacobian (status in *err).                 */
/* ------------------------------------------------------------------------ */
/* With init (a CSC of the full structural pattern, 0-based arrays icp,
 * irv, values inz) its entries go first as triplets and no zeros are
 * dropped: the DSL's ∫(...; csc_matrix=K), which adds into K.nzval in
 * element order and keeps K's pattern (src/multifield.jl:5280-5346). */
orc_csc *orc_assemble_ex(int kind, int ptype, int dim, int pdim, int64_t non,
                         const double *xyz, int64_t nel, int npe,
                         const int32_t *conn, const int32_t *emat, int nip,
                         const double *w, const double *N, const double *dN,
                         const double *params, int nmat, double thickness,
                         int lumped, const double *nref, const int64_t *icp,
                         const int64_t *irv, const double *inz, int *err) {
  (void)nmat;
  size_t nd = (size_t)pdim * npe;
  double *Ke = (double *)malloc(sizeof(double) * nd * nd);
  double *X = (double *)malloc(sizeof(double) * npe * 3);
  double *R = (double *)malloc(sizeof(double) * npe * npe * 9);
  double *Mref = (double *)malloc(sizeof(double) * npe * npe);
  orc_affine_tables(npe, nip, w, N, dN, R, Mref);
  coo c = {0};
  c.n = non * pdim;
  *err = 0;
  if (icp)
    for (int64_t j = 0; j < non * pdim; ++j)
      for (int64_t k = icp[j]; k < icp[j + 1]; ++k) coo_push(&c, irv[k], j, inz[k]);
  for (int64_t e = 0; e < nel; ++e) {
    int mat = emat ? emat[e] : 0;
    if (mat < 0) continue;
    double c1 = 0, c2 = 0;
    double b = (ptype == PT_PLANE_STRESS || ptype == PT_HEAT || ptype == PT_PLANE_HEAT) ? thickness : 1.0;
    if (kind == ORC_ELASTIC && ptype == PT_LAME) {
      c1 = params[2 * mat];
      c2 = params[2 * mat + 1];
    } else if (kind == ORC_ELASTIC) {
      orc_lame(ptype, params[2 * mat], params[2 * mat + 1], thickness, &c1, &c2);
    } else if (kind == ORC_HEAT) {
      c1 = params[mat] * b;
    } else {  /* massMatrixSolid: b = thickness for plane stress only (src/linear.jl:1873-1879);
                 heatCapacityMatrix: b = 1 (src/heat.jl:275-283) */
      c1 = params[mat] * (ptype == PT_PLANE_STRESS ? thickness : 1.0);
    }
    for (int a = 0; a < npe; ++a) {
      int64_t node = conn[e * npe + a];
      for (int i = 0; i < 3; ++i) X[3 * a + i] = xyz[3 * node + i];
    }
    if (orc_element_matrix_ex(kind, dim, pdim, npe, nip, w, N, dN, X, c1, c2, nref, R, Mref, Ke)) {
      *err = -1;
      free(Ke); free(X); free(R); free(Mref); free(c.I); free(c.J); free(c.V);
      return NULL;
    }
    /* column-major walk of K1: k fastest; I = nn2[l], J = nn2[k] */
    for (size_t l = 0; l < nd; ++l)
      for (size_t k = 0; k < nd; ++k) {
        int64_t dl = (int64_t)conn[e * npe + l / pdim] * pdim + (int64_t)(l % pdim);
        int64_t dk = (int64_t)conn[e * npe + k / pdim] * pdim + (int64_t)(k % pdim);
        coo_push(&c, dl, dk, Ke[k * nd + l]);
      }
  }
  orc_csc *m = coo_to_csc(&c);
  free(c.I); free(c.J); free(c.V);
  free(Ke); free(X); free(R); free(Mref);
  if (kind == ORC_MASS && lumped) {
    orc_csc *D = orc_lump(m);
    orc_free(m);
    m = D;
  }
  if (!icp) orc_dropzeros(m);
  return m;
}

orc_csc *orc_assemble(int kind, int ptype, int dim, int pdim, int64_t non,
                      const double *xyz, int64_t nel, int npe,
                      const int32_t *conn, const int32_t *emat, int nip,
                      const double *w, const double *N, const double *dN,
                      const double *params, int nmat, double thickness,
                      int lumped, const double *nref, int *err) {
  return orc_assemble_ex(kind, ptype, dim, pdim, non, xyz, nel, npe, conn, emat, nip, w, N, dN, params, nmat,
                         thickness, lumped, nref, NULL, NULL, NULL, err);
}

/* ------------------------------------------------------------------------ */
/* Threaded direct-CSC assembly, restating the reference's fastest CPU path  */
/* (assemble_csc_worker! + reduce_csc_buffers!, src/multifield.jl:2394-2499, */
/* :2345-2380): structural pattern reused, cyclic element chunks per worker, */
/* one binary search per node pair (find_csc_position, :2260-2283), per-     */
/* worker nzval buffers summed at the end.  Used as the timed CPU baseline.  */
/* `pat` must be the structural pattern of the same mesh; nzval overwritten. */
/* Returns elapsed seconds of the assembly (pattern excluded).               */
/* ------------------------------------------------------------------------ */
static int64_t find_pos(const int64_t *rowval, int64_t lo, int64_t hi, int64_t r) {
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (rowval[mid] < r) lo = mid + 1; else hi = mid;
  }
  return lo;
}

double orc_assemble_csc_threaded(int kind, int ptype, int dim, int pdim,
                                 const double *xyz, int64_t nel, int npe,
                                 const int32_t *conn, int nip, const double *w,
                                 const double *N, const double *dN,
                                 const double *params, double thickness,
                                 orc_csc *pat, int nthreads, int chunk, const double *nref) {
  int64_t nnz = pat->nnz;
  double *R = (double *)malloc(sizeof(double) * npe * npe * 9);
  double *Mref = (double *)malloc(sizeof(double) * npe * npe);
  orc_affine_tables(npe, nip, w, N, dN, R, Mref);
  int T = nthreads > 0 ? nthreads : 1;
#ifdef _OPENMP
  double t0 = omp_get_wtime();
#else
  double t0 = 0;
#endif
  double **bufs = (double **)malloc(sizeof(double *) * T);
#pragma omp parallel num_threads(T)
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
#else
    int tid = 0;
#endif
    double *nz = (double *)calloc(nnz + 1, sizeof(double));
    bufs[tid] = nz;
    size_t nd = (size_t)pdim * npe;
    double *Ke = (double *)malloc(sizeof(double) * nd * nd);
    double *X = (double *)malloc(sizeof(double) * npe * 3);
    double c1 = 0, c2 = 0;
    double b = (ptype == PT_PLANE_STRESS || ptype == PT_HEAT || ptype == PT_PLANE_HEAT) ? thickness : 1.0;
    if (kind == ORC_ELASTIC) orc_lame(ptype, params[0], params[1], thickness, &c1, &c2);
    else if (kind == ORC_HEAT) c1 = params[0] * b;
    else c1 = params[0] * (ptype == PT_PLANE_STRESS ? thickness : 1.0);
    int64_t nchunks = (nel + chunk - 1) / chunk;
    for (int64_t ch = tid; ch < nchunks; ch += T) {
      int64_t e0 = ch * chunk, e1 = e0 + chunk < nel ? e0 + chunk : nel;
      for (int64_t e = e0; e < e1; ++e) {
        for (int a = 0; a < npe; ++a) {
          int64_t node = conn[e * npe + a];
          for (int i = 0; i < 3; ++i) X[3 * a + i] = xyz[3 * node + i];
        }
        orc_element_matrix_ex(kind, dim, pdim, npe, nip, w, N, dN, X, c1, c2, nref, R, Mref, Ke);
        for (int bn = 0; bn < npe; ++bn) {
          int64_t B = conn[e * npe + bn];
          for (int an = 0; an < npe; ++an) {
            int64_t A = conn[e * npe + an];
            int64_t col0 = B * pdim;
            int64_t p0 = find_pos(pat->rowval, pat->colptr[col0], pat->colptr[col0 + 1], A * pdim);
            int64_t off = p0 - pat->colptr[col0];
            for (int j = 0; j < pdim; ++j) {
              int64_t base = pat->colptr[col0 + j] + off;
              for (int i = 0; i < pdim; ++i)
                nz[base + i] += Ke[((size_t)an * pdim + i) * nd + (size_t)bn * pdim + j];
            }
          }
        }
      }
    }
    free(Ke); free(X);
  }
  /* reduce worker buffers */
#pragma omp parallel for num_threads(T) schedule(static)
  for (int64_t k = 0; k < nnz; ++k) {
    double s = 0.0;
    for (int t = 0; t < T; ++t) s += bufs[t][k];
    pat->nzval[k] = s;
  }
  for (int t = 0; t < T; ++t) free(bufs[t]);
  free(bufs);
  free(R);
  free(Mref);
#ifdef _OPENMP
  return omp_get_wtime() - t0;
#else
  return 0.0;
#endif
}

/* ------------------------------------------------------------------------ */
/* y = A x (CSC, sequential).                                               */
/* ------------------------------------------------------------------------ */
void orc_spmv(const orc_csc *A, const double *x, double *y) {
  for (int64_t i = 0; i < A->n; ++i) y[i] = 0.0;
  for (int64_t j = 0; j < A->n; ++j) {
    double xj = x[j];
    for (int64_t k = A->colptr[j]; k < A->colptr[j + 1]; ++k)
      y[A->rowval[k]] += A->nzval[k] * xj;
  }
}

static double dotp(int64_t n, const double *a, const double *b) {
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

/* ------------------------------------------------------------------------ */
/* Condensed Dirichlet solve with IterativeSolvers.cg's recurrence           */
/* (IterativeSolvers 0.9.4, the call at src/linear.jl:3827-3833):            */
/*   f_kin = A[:,fixed] x[fixed]; solve A_ff x_f = b_f - f_kin_f from x_f=0; */
/*   per iteration c = P^-1 r, rho = c.r, u = c + (rho/rho_prev) u,          */
/*   c = A u, alpha = rho/(u.c), x += alpha u, r -= alpha c,                 */
/*   stop when ||r|| <= reltol ||r0|| or after maxiter products.             */
/* precond: 0 identity, 1 Jacobi (diagonal of A_ff).                         */
/* Returns iterations; *relres = ||r||/||r0||.                               */
/* ------------------------------------------------------------------------ */
int64_t orc_cg(const orc_csc *A, const double *b, double *x,
               const uint8_t *fixed, int precond, double reltol,
               int64_t maxiter, double *relres) {
  int64_t n = A->n;
  double *xf = (double *)calloc(n, sizeof(double));
  double *r = (double *)malloc(sizeof(double) * n);
  double *c = (double *)malloc(sizeof(double) * n);
  double *u = (double *)calloc(n, sizeof(double));
  double *dinv = (double *)malloc(sizeof(double) * n);
  for (int64_t i = 0; i < n; ++i) xf[i] = fixed[i] ? x[i] : 0.0;
  orc_spmv(A, xf, c); /* f_kin */
  for (int64_t i = 0; i < n; ++i) r[i] = fixed[i] ? 0.0 : b[i] - c[i];
  for (int64_t j = 0; j < n; ++j) {
    double d = 0.0;
    for (int64_t k = A->colptr[j]; k < A->colptr[j + 1]; ++k)
      if (A->rowval[k] == j) d = A->nzval[k];
    dinv[j] = (precond == 1 && d != 0.0) ? 1.0 / d : 1.0;
  }
  for (int64_t i = 0; i < n; ++i) xf[i] = 0.0;
  double res0 = sqrt(dotp(n, r, r)), res = res0;
  double tol = reltol * res0;
  double rho_prev = 1.0;
  int64_t it = 0;
  while (!(res <= tol) && it < maxiter) {
    for (int64_t i = 0; i < n; ++i) c[i] = fixed[i] ? 0.0 : dinv[i] * r[i];
    double rho = dotp(n, c, r);
    double beta = rho / rho_prev;
    rho_prev = rho;
    for (int64_t i = 0; i < n; ++i) u[i] = c[i] + beta * u[i];
    orc_spmv(A, u, c);
    for (int64_t i = 0; i < n; ++i) if (fixed[i]) c[i] = 0.0;
    double alpha = rho / dotp(n, u, c);
    for (int64_t i = 0; i < n; ++i) {
      xf[i] += alpha * u[i];
      r[i] -= alpha * c[i];
    }
    res = sqrt(dotp(n, r, r));
    ++it;
  }
  for (int64_t i = 0; i < n; ++i) if (!fixed[i]) x[i] = xf[i];
  *relres = res0 > 0 ? res / res0 : 0.0;
  free(xf); free(r); free(c); free(u); free(dinv);
  return it;
}

/* ------------------------------------------------------------------------ */
/* Consistent nodal load of boundary elements, loadVector                    */
/* (src/linear.jl:3088-3434): f1 += H^T t Ja w per point with               */
/* Ja = |t1| b for 2D edges (:3394-3395), |t1 x t2| for 3D faces            */
/* (:3380-3384), t1, t2 the columns of the boundary Jacobian.  Constant     */
/* traction t[pdim] or nodal values tn[pdim*nb] interpolated with H.        */
/* Element contributions are added into f in element order.                 */
/* ------------------------------------------------------------------------ */
/* elasticSupportMatrix / heatConvectionMatrix (src/linear.jl:2859-3005,
 * src/heat.jl:562-567): C = sum over boundary elements and points of
 * H^T diag(k) H Ja w, Ja as in the load vector.  The stiffness k_i at a
 * point of element e is the element's constant ke[pdim*e+i] or, with ken,
 * its element-node values ken[(npe*e+a)*pdim+i] interpolated with H (fma
 * chain over the nodes).  Several support groups are one element list in
 * group order (the reference collects all groups' triplets before its single
 * sparse() call).  Contract: jw = Ja * w_q;
 * for node pairs a <= b and component i, the fma chain over q of
 * ((N_a * jw) * k_i) * N_b is the diagonal entry i of block (a,b), mirrored
 * to (b,a); triplets in the reference's transposed order, sparse
 * (duplicates in input order), dropzeros!. */
orc_csc *orc_support_matrix(int problem_dim, int pdim, int64_t non, const double *xyz, int64_t nelb, int npeb,
                            const int32_t *connb, int nip, const double *w, const double *N, const double *dN,
                            const double *ke, const double *ken, double thickness) {
  int bdim = problem_dim - 1;
  size_t nd = (size_t)pdim * npeb;
  /* acc[(a*npeb+b)*pdim+i]: diagonal entry i of block (a,b), a <= b */
  double *acc = (double *)malloc(sizeof(double) * npeb * npeb * pdim);
  double *Ke = (double *)malloc(sizeof(double) * nd * nd);
  coo c = {0};
  c.n = non * pdim;
  for (int64_t e = 0; e < nelb; ++e) {
    const int32_t *ce = connb + e * npeb;
    for (int k = 0; k < npeb * npeb * pdim; ++k) acc[k] = 0.0;
    for (int q = 0; q < nip; ++q) {
      double t1[3] = {0, 0, 0}, t2[3] = {0, 0, 0};
      for (int i = 0; i < 3; ++i) {
        double a1 = 0.0, a2 = 0.0;
        for (int a = 0; a < npeb; ++a) {
          double xa = xyz[3 * (int64_t)ce[a] + i];
          a1 = fma(xa, dN[((size_t)q * npeb + a) * 3 + 0], a1);
          if (bdim == 2) a2 = fma(xa, dN[((size_t)q * npeb + a) * 3 + 1], a2);
        }
        t1[i] = a1;
        t2[i] = a2;
      }
      double Ja;
      if (bdim == 1) {
        Ja = sqrt(t1[0] * t1[0] + t1[1] * t1[1]) * thickness;
      } else {
        double xy = t1[0] * t2[1] - t1[1] * t2[0];
        double yz = t1[1] * t2[2] - t1[2] * t2[1];
        double zx = t1[2] * t2[0] - t1[0] * t2[2];
        Ja = sqrt(xy * xy + yz * yz + zx * zx);
      }
      double jw = Ja * w[q];
      double kq[3] = {0, 0, 0};
      for (int i = 0; i < pdim; ++i) {
        if (ken) {
          double s = 0.0;
          for (int a = 0; a < npeb; ++a) s = fma(N[(size_t)q * npeb + a], ken[(e * npeb + a) * pdim + i], s);
          kq[i] = s;
        } else {
          kq[i] = ke[e * pdim + i];
        }
      }
      for (int a = 0; a < npeb; ++a) {
        double naj = N[(size_t)q * npeb + a] * jw;
        for (int b = a; b < npeb; ++b)
          for (int i = 0; i < pdim; ++i) {
            double *t = &acc[((size_t)a * npeb + b) * pdim + i];
            *t = fma(naj * kq[i], N[(size_t)q * npeb + b], *t);
          }
      }
    }
    memset(Ke, 0, sizeof(double) * nd * nd);
    for (int a = 0; a < npeb; ++a)
      for (int b = a; b < npeb; ++b)
        for (int i = 0; i < pdim; ++i) {
          double v = acc[((size_t)a * npeb + b) * pdim + i];
          Ke[((size_t)a * pdim + i) * nd + (size_t)b * pdim + i] = v;
          Ke[((size_t)b * pdim + i) * nd + (size_t)a * pdim + i] = v;
        }
    for (size_t l = 0; l < nd; ++l)
      for (size_t k = 0; k < nd; ++k) {
        int64_t dl = (int64_t)ce[l / pdim] * pdim + (int64_t)(l % pdim);
        int64_t dk = (int64_t)ce[k / pdim] * pdim + (int64_t)(k % pdim);
        coo_push(&c, dl, dk, Ke[k * nd + l]);
      }
  }
  orc_csc *out = coo_to_csc(&c);
  free(c.I); free(c.J); free(c.V);
  free(acc); free(Ke);
  orc_dropzeros(out);
  return out;
}

/* ------------------------------------------------------------------------ */
/* Follower loads on boundary faces of a 3D body, F given at the nodes      */
/* (Fn[9*node], column-major 3x3).  Shared contract at a face point q:       */
/*   t1, t2 = fma chains over the nodes of x_a dN_a/du, x_a dN_a/dv;         */
/*   cr = t1 x t2 as (yz, zx, xy), da = sqrt(|cr|^2) (the load vector's Ja); */
/*   F_q[i][j] = fma chain over the nodes of N_a F_a[i][j];                  */
/*   t_q = per-element constant te[3e+i], or fma chain of N_a ten[..];       */
/*   tg = F_q t_q (fma chain over j).                                        */
/* ------------------------------------------------------------------------ */
static void orc_face_point(const double *xyz, const int32_t *ce, int npe, int q, const double *N,
                           const double *dN, const double *Fn, double t1[3], double t2[3], double *da,
                           double Fq[3][3]) {
  for (int i = 0; i < 3; ++i) {
    double a1 = 0.0, a2 = 0.0;
    for (int a = 0; a < npe; ++a) {
      double xa = xyz[3 * (int64_t)ce[a] + i];
      a1 = fma(xa, dN[((size_t)q * npe + a) * 3 + 0], a1);
      a2 = fma(xa, dN[((size_t)q * npe + a) * 3 + 1], a2);
    }
    t1[i] = a1;
    t2[i] = a2;
  }
  double xy = t1[0] * t2[1] - t1[1] * t2[0];
  double yz = t1[1] * t2[2] - t1[2] * t2[1];
  double zx = t1[2] * t2[0] - t1[0] * t2[2];
  *da = sqrt(xy * xy + yz * yz + zx * zx);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double acc = 0.0;
      for (int a = 0; a < npe; ++a) acc = fma(N[(size_t)q * npe + a], Fn[9 * (int64_t)ce[a] + 3 * j + i], acc);
      Fq[i][j] = acc;
    }
}

static void orc_face_traction(int64_t e, const int32_t *ce, int npe, int q, const double *N, const double *te,
                              const double *ten, double tq[3]) {
  (void)ce;
  for (int i = 0; i < 3; ++i) {
    if (ten) {
      double acc = 0.0;
      for (int a = 0; a < npe; ++a) acc = fma(N[(size_t)q * npe + a], ten[(e * npe + a) * 3 + i], acc);
      tq[i] = acc;
    } else {
      tq[i] = te[3 * e + i];
    }
  }
}

/* loadVector(problem, loads; F) (src/linear.jl:3088-3434, follower branch
 * :3333-3372): the traction at a point is F_q t_q, integrated on the
 * reference face, f[3*node+i] += fma(N_a tg_i, da w).  Element vectors are
 * added into f in element order.  Returns 0, or -1 when det F_q <= 0. */
int orc_load_vector_follower(const double *xyz, int64_t nelb, int npeb, const int32_t *connb, int nip,
                             const double *w, const double *N, const double *dN, const double *Fn,
                             const double *te, const double *ten, double *f) {
  double *fe = (double *)malloc(sizeof(double) * npeb * 3);
  int rc = 0;
  for (int64_t e = 0; e < nelb; ++e) {
    const int32_t *ce = connb + e * npeb;
    for (int k = 0; k < npeb * 3; ++k) fe[k] = 0.0;
    for (int q = 0; q < nip; ++q) {
      double t1[3], t2[3], da, Fq[3][3], Fi[9], tq[3], tg[3];
      orc_face_point(xyz, ce, npeb, q, N, dN, Fn, t1, t2, &da, Fq);
      if (!(orc_inv3(Fq, Fi) > 0.0)) rc = -1;
      orc_face_traction(e, ce, npeb, q, N, te, ten, tq);
      for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int j = 0; j < 3; ++j) acc = fma(Fq[i][j], tq[j], acc);
        tg[i] = acc;
      }
      double jw = da * w[q];
      for (int a = 0; a < npeb; ++a) {
        double Na = N[(size_t)q * npeb + a];
        for (int i = 0; i < 3; ++i) fe[a * 3 + i] = fma(Na * tg[i], jw, fe[a * 3 + i]);
      }
    }
    for (int a = 0; a < npeb; ++a)
      for (int i = 0; i < 3; ++i) f[3 * (int64_t)ce[a] + i] += fe[a * 3 + i];
  }
  free(fe);
  return rc;
}

/* externalTangentFollower (src/nonlinear.jl:3053-3258): per face point,
 * the face Jacobian Jm = [t1 t2 n] with n = cr / da (gmsh's completion of a
 * surface Jacobian), jw = da w, grad N_b = Jm^-T (dN_b/du, dN_b/dv, 0) (fma
 * chains), Finv = F_q^-1 and Jgp = det F_q by cofactors, tg = F_q t_q,
 * tl = Finv tg.  For column (b, jb), with g = grad N_b and f = Finv[:,jb]:
 *   u = alpha tg - s g + c e_jb,  alpha = f.g, s = f.tg, c = g.tl
 *   dt0 = Jgp (Finv^T u)  (each dot product an fma chain in index order)
 *   Ke[(a,ia),(b,jb)] = fma(N_a jw, dt0_ia, Ke)
 * which is the reference's Jgp F^-T (alpha I - g f^T) tg + Jgp F^-T e_jb c.
 * Triplets (row (a,ia), column (b,jb), Ke) in element order, sparse,
 * dropzeros!.  *status = -1 when det F_q <= 0 somewhere. */
orc_csc *orc_follower_tangent(int64_t non, const double *xyz, int64_t nelb, int npeb, const int32_t *connb,
                              int nip, const double *w, const double *N, const double *dN, const double *Fn,
                              const double *te, const double *ten, int *status) {
  size_t nd = (size_t)3 * npeb;
  double *Ke = (double *)malloc(sizeof(double) * nd * nd);
  coo c = {0};
  c.n = non * 3;
  *status = 0;
  for (int64_t e = 0; e < nelb; ++e) {
    const int32_t *ce = connb + e * npeb;
    for (size_t k = 0; k < nd * nd; ++k) Ke[k] = 0.0;
    for (int q = 0; q < nip; ++q) {
      double t1[3], t2[3], da, Fq[3][3], Fi[9], tq[3], tg[3], tl[3], Jm[3][3], Ji[9];
      orc_face_point(xyz, ce, npeb, q, N, dN, Fn, t1, t2, &da, Fq);
      double xy = t1[0] * t2[1] - t1[1] * t2[0];
      double yz = t1[1] * t2[2] - t1[2] * t2[1];
      double zx = t1[2] * t2[0] - t1[0] * t2[2];
      double nrm[3] = {yz / da, zx / da, xy / da};
      for (int i = 0; i < 3; ++i) {
        Jm[i][0] = t1[i];
        Jm[i][1] = t2[i];
        Jm[i][2] = nrm[i];
      }
      orc_inv3(Jm, Ji);
      double Jgp = orc_inv3(Fq, Fi);
      if (!(Jgp > 0.0)) *status = -1;
      orc_face_traction(e, ce, npeb, q, N, te, ten, tq);
      for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int j = 0; j < 3; ++j) acc = fma(Fq[i][j], tq[j], acc);
        tg[i] = acc;
      }
      for (int i = 0; i < 3; ++i) {
        double acc = 0.0;
        for (int j = 0; j < 3; ++j) acc = fma(Fi[3 * i + j], tg[j], acc);
        tl[i] = acc;
      }
      double jw = da * w[q];
      for (int b = 0; b < npeb; ++b) {
        const double *d = dN + ((size_t)q * npeb + b) * 3;
        double g[3];
        for (int i = 0; i < 3; ++i) g[i] = fma(Ji[3 + i], d[1], Ji[i] * d[0]);
        double cdot = 0.0;
        for (int i = 0; i < 3; ++i) cdot = fma(g[i], tl[i], cdot);
        for (int jb = 0; jb < 3; ++jb) {
          double alpha = 0.0, sdot = 0.0;
          for (int i = 0; i < 3; ++i) {
            alpha = fma(Fi[3 * i + jb], g[i], alpha);
            sdot = fma(Fi[3 * i + jb], tg[i], sdot);
          }
          double u[3];
          for (int i = 0; i < 3; ++i) u[i] = alpha * tg[i] - sdot * g[i];
          u[jb] += cdot;
          double dt0[3];
          for (int i = 0; i < 3; ++i) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k) acc = fma(Fi[3 * k + i], u[k], acc);
            dt0[i] = Jgp * acc;
          }
          for (int a = 0; a < npeb; ++a) {
            double nj = N[(size_t)q * npeb + a] * jw;
            for (int ia = 0; ia < 3; ++ia) {
              double *t = &Ke[((size_t)a * 3 + ia) * nd + (size_t)b * 3 + jb];
              *t = fma(nj, dt0[ia], *t);
            }
          }
        }
      }
    }
    for (size_t r = 0; r < nd; ++r)
      for (size_t k = 0; k < nd; ++k) {
        int64_t dr = (int64_t)ce[r / 3] * 3 + (int64_t)(r % 3);
        int64_t dk = (int64_t)ce[k / 3] * 3 + (int64_t)(k % 3);
        coo_push(&c, dr, dk, Ke[r * nd + k]);
      }
  }
  orc_csc *out = coo_to_csc(&c);
  free(c.I); free(c.J); free(c.V);
  free(Ke);
  orc_dropzeros(out);
  return out;
}

/* elementsToNodes (src/general.jl:5519-5640): nodal value = (sum of the
 * element-node values in element order) * (1 / count). */
void orc_elements_to_nodes(int64_t non, int64_t nel, int npe, const int32_t *conn, int ncomp, const double *ev,
                           double *nv) {
  int64_t *cnt = (int64_t *)calloc((size_t)non, sizeof(int64_t));
  for (int64_t k = 0; k < non * ncomp; ++k) nv[k] = 0.0;
  for (int64_t e = 0; e < nel; ++e)
    for (int a = 0; a < npe; ++a) {
      int64_t v = conn[e * npe + a];
      cnt[v] += 1;
      for (int i = 0; i < ncomp; ++i) nv[v * ncomp + i] += ev[(e * npe + a) * ncomp + i];
    }
  for (int64_t v = 0; v < non; ++v) {
    if (!cnt[v]) continue;
    double fct = 1.0 / (double)cnt[v];
    for (int i = 0; i < ncomp; ++i) nv[v * ncomp + i] *= fct;
  }
  free(cnt);
}

void orc_load_vector(int problem_dim, int pdim, const double *xyz,
                     int64_t nelb, int npeb, const int32_t *connb, int nip,
                     const double *w, const double *N, const double *dN,
                     const double *t, const double *tn, double thickness,
                     double *f) {
  int bdim = problem_dim - 1;
  double *fe = (double *)malloc(sizeof(double) * npeb * pdim);
  for (int64_t e = 0; e < nelb; ++e) {
    for (int k = 0; k < npeb * pdim; ++k) fe[k] = 0.0;
    for (int q = 0; q < nip; ++q) {
      double t1[3] = {0, 0, 0}, t2[3] = {0, 0, 0};
      for (int i = 0; i < 3; ++i) {
        double a1 = 0.0, a2 = 0.0;
        for (int a = 0; a < npeb; ++a) {
          double xa = xyz[3 * (int64_t)connb[e * npeb + a] + i];
          a1 = fma(xa, dN[((size_t)q * npeb + a) * 3 + 0], a1);
          if (bdim == 2) a2 = fma(xa, dN[((size_t)q * npeb + a) * 3 + 1], a2);
        }
        t1[i] = a1;
        t2[i] = a2;
      }
      double Ja;
      if (bdim == 1) {
        Ja = sqrt(t1[0] * t1[0] + t1[1] * t1[1]) * thickness;
      } else {
        double xy = t1[0] * t2[1] - t1[1] * t2[0];
        double yz = t1[1] * t2[2] - t1[2] * t2[1];
        double zx = t1[2] * t2[0] - t1[0] * t2[2];
        Ja = sqrt(xy * xy + yz * yz + zx * zx);
      }
      double tq[3] = {0, 0, 0};
      for (int i = 0; i < pdim; ++i) {
        if (tn) {
          double acc = 0.0;
          for (int a = 0; a < npeb; ++a)
            acc = fma(N[(size_t)q * npeb + a], tn[(int64_t)connb[e * npeb + a] * pdim + i], acc);
          tq[i] = acc;
        } else {
          tq[i] = t[i];
        }
      }
      double jw = Ja * w[q];
      for (int a = 0; a < npeb; ++a)
        for (int i = 0; i < pdim; ++i)
          fe[a * pdim + i] = fma(N[(size_t)q * npeb + a] * tq[i], jw, fe[a * pdim + i]);
    }
    for (int a = 0; a < npeb; ++a)
      for (int i = 0; i < pdim; ++i)
        f[(int64_t)connb[e * npeb + a] * pdim + i] += fe[a * pdim + i];
  }
  free(fe);
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Elementwise nodal gradient, the :vector_grad branch of ∇ (src/nabla.jl:   */
/* 77-311): at every element node k, J and the physical gradients of all     */
/* shape functions at node k's reference coordinates; T[i][j] = sum_l        */
/* g_l[j] u_l[i] (fma chain over l), stored column-major (9 per node);       */
/* with add_identity the deformation gradient F = I + T.                     */
/* dNn[(k*npe+l)*3+j] = dN_l/dxi_j at node k.                               */
/* ------------------------------------------------------------------------ */
int orc_grad_elementwise(const double *xyz, int64_t nel, int npe, const int32_t *conn,
                         const double *dNn, const double *u, int add_identity,
                         double *out) {
  double *X = (double *)malloc(sizeof(double) * npe * 3);
  int rc = 0;
  for (int64_t e = 0; e < nel; ++e) {
    for (int a = 0; a < npe; ++a)
      for (int i = 0; i < 3; ++i) X[3 * a + i] = xyz[3 * (int64_t)conn[e * npe + a] + i];
    for (int k = 0; k < npe; ++k) {
      const double *d = dNn + (size_t)k * npe * 3;
      double inv[9];
      double det = orc_geom(3, npe, X, d, inv);
      if (!(det > 0.0)) rc = -1;
      double T[3][3] = {{0}};
      for (int l = 0; l < npe; ++l) {
        double g[3];
        for (int i = 0; i < 3; ++i) {
          double acc = 0.0;
          for (int j = 0; j < 3; ++j) acc = fma(inv[3 * j + i], d[l * 3 + j], acc);
          g[i] = acc;
        }
        const double *ul = u + 3 * (int64_t)conn[e * npe + l];
        for (int j = 0; j < 3; ++j)
          for (int i = 0; i < 3; ++i) T[i][j] = fma(g[j], ul[i], T[i][j]);
      }
      double *o = out + (size_t)e * npe * 9 + (size_t)k * 9;
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) o[3 * j + i] = (add_identity && i == j) ? T[i][j] + 1.0 : T[i][j];
    }
  }
  free(X);
  return rc;
}

/* ======================================================================== */
/* Total Lagrangian operators (src/nonlinear.jl:2083-2910).                  */
/* ======================================================================== */
/* Arithmetic contract (shared with the CUDA kernels):
 *   F(q)  = fma-chain over element nodes a of N_a(q) * Fnode_a (per entry)
 *   C     = F^T F, C_IJ = fma-chain over k of F_kI F_kJ
 *   Cinv  = adj(C)/det(C) with the cofactor formulas of the geometry contract
 *   lnJ   = 0.5 * ln(det C), ln by the atanh series below
 *   neo-Hookean psi = mu/2 (I1-3) - mu lnJ + lambda/2 lnJ^2:
 *     S_IJ = fma(lambda lnJ, Cinv_IJ, mu (delta_IJ - Cinv_IJ))
 *     D_ab = fma(lambda, Cinv_IJ Cinv_KL, (mu - lambda lnJ) (Cinv_IK Cinv_JL + Cinv_IL Cinv_JK))
 *   Saint Venant-Kirchhoff psi = lambda/2 tr(E)^2 + mu E:E, E = (C - I)/2:
 *     S_IJ = fma(lambda, trE delta_IJ, 2 mu E_IJ)
 *     D_ab = lambda delta_IJ delta_KL + mu (delta_IK delta_JL + delta_IL delta_JK)
 *   Voigt order (11,22,33,23,13,12), a=(I,J), b=(K,L)
 *   (ext/LowLevelFEMTensorsExt.jl:43-50, no shear factors in D).
 * These are the derivatives S = 2 dpsi/dC and C = 4 d2psi/dC2 that the
 * reference takes by automatic differentiation (ext/LowLevelFEMTensorsExt.jl:
 * 19, :37); they are checked against finite differences of psi in the tests.
 */
#define ORC_LAW_CONST 0
#define ORC_LAW_NEOHOOKE 1
#define ORC_LAW_SVK 2

/* Natural logarithm: x = m 2^e with m in [sqrt(1/2), sqrt(2)),
 * ln x = e ln2 + 2 atanh(s), s = (m-1)/(m+1), atanh by its Taylor series
 * s + s^3/3 + ... (|s| <= 0.1716, 12 terms). */
double orc_ln(double x) {
  int e;
  double m = frexp(x, &e);
  if (m < 0.70710678118654752440) {
    m = m * 2.0;
    e = e - 1;
  }
  double s = (m - 1.0) / (m + 1.0);
  double s2 = s * s;
  double p = 1.0 / 25.0;
  for (int k = 11; k >= 0; --k) p = fma(p, s2, 1.0 / (2.0 * k + 1.0));
  return fma((double)e, 0.69314718055994530942, 2.0 * (s * p));
}

static const int VI[6] = {0, 1, 2, 1, 0, 0};
static const int VJ[6] = {0, 1, 2, 2, 2, 1};

static void sym_inverse(const double C[3][3], double Ci[3][3], double *detC) {
  double c00 = C[1][1] * C[2][2] - C[1][2] * C[2][1];
  double c01 = -(C[1][0] * C[2][2] - C[1][2] * C[2][0]);
  double c02 = C[1][0] * C[2][1] - C[1][1] * C[2][0];
  double c10 = -(C[0][1] * C[2][2] - C[0][2] * C[2][1]);
  double c11 = C[0][0] * C[2][2] - C[0][2] * C[2][0];
  double c12 = -(C[0][0] * C[2][1] - C[0][1] * C[2][0]);
  double c20 = C[0][1] * C[1][2] - C[0][2] * C[1][1];
  double c21 = -(C[0][0] * C[1][2] - C[0][2] * C[1][0]);
  double c22 = C[0][0] * C[1][1] - C[0][1] * C[1][0];
  double det = (C[0][0] * c00 + C[0][1] * c01) + C[0][2] * c02;
  double r = 1.0 / det;
  Ci[0][0] = c00 * r; Ci[0][1] = c10 * r; Ci[0][2] = c20 * r;
  Ci[1][0] = c01 * r; Ci[1][1] = c11 * r; Ci[1][2] = c21 * r;
  Ci[2][0] = c02 * r; Ci[2][1] = c12 * r; Ci[2][2] = c22 * r;
  *detC = det;
}

/* PK2 stress S and Voigt tangent D (6x6 row-major) from C; returns -1 if
 * det C <= 0. */
int orc_law(int law, const double *prm, const double C[3][3], double S[3][3], double *D) {
  if (law == ORC_LAW_CONST) {
    for (int a = 0; a < 6; ++a)
      for (int b = 0; b < 6; ++b) D[a * 6 + b] = prm[b * 6 + a]; /* params column-major */
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) S[i][j] = 0.0;
    return 0;
  }
  double mu = prm[0], lam = prm[1];
  if (law == ORC_LAW_SVK) {
    double E[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) E[i][j] = 0.5 * (C[i][j] - (i == j ? 1.0 : 0.0));
    double trE = (E[0][0] + E[1][1]) + E[2][2];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) S[i][j] = fma(lam, i == j ? trE : 0.0, (2.0 * mu) * E[i][j]);
    for (int a = 0; a < 6; ++a)
      for (int b = 0; b < 6; ++b) {
        int I = VI[a], J = VJ[a], K = VI[b], L = VJ[b];
        double v = lam * ((I == J && K == L) ? 1.0 : 0.0);
        v = v + mu * ((double)((I == K && J == L) ? 1 : 0) + (double)((I == L && J == K) ? 1 : 0));
        D[a * 6 + b] = v;
      }
    return 0;
  }
  double Ci[3][3], detC;
  sym_inverse(C, Ci, &detC);
  if (!(detC > 0.0)) return -1;
  double lnJ = 0.5 * orc_ln(detC);
  double t = lam * lnJ;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) S[i][j] = fma(t, Ci[i][j], mu * ((i == j ? 1.0 : 0.0) - Ci[i][j]));
  double m2 = mu - t;
  for (int a = 0; a < 6; ++a)
    for (int b = 0; b < 6; ++b) {
      int I = VI[a], J = VJ[a], K = VI[b], L = VJ[b];
      double sym = Ci[I][K] * Ci[J][L] + Ci[I][L] * Ci[J][K];
      D[a * 6 + b] = fma(lam, Ci[I][J] * Ci[K][L], m2 * sym);
    }
  return 0;
}

/* 3x3 tensor at point q interpolated from the element's nodal values
 * (column-major 3x3 per node, T[i][j] at 9a + 3j + i). */
static void interp_tensor(int npe, const double *Nq, const double *Tn, double T[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double acc = 0.0;
      for (int a = 0; a < npe; ++a) acc = fma(Nq[a], Tn[9 * a + 3 * j + i], acc);
      T[i][j] = acc;
    }
}

static void right_cauchy_green(const double F[3][3], double C[3][3]) {
  for (int I = 0; I < 3; ++I)
    for (int J = 0; J < 3; ++J) {
      double acc = 0.0;
      for (int k = 0; k < 3; ++k) acc = fma(F[k][I], F[k][J], acc);
      C[I][J] = acc;
    }
}

/* B(F) of node a, 6x3: B[I][i] for Voigt row I and displacement component i
 * (src/nonlinear.jl:2219-2242). */
static void tl_B(const double F[3][3], const double g[3], double B[6][3]) {
  for (int j = 0; j < 3; ++j) {
    double v1 = F[j][0], v2 = F[j][1], v3 = F[j][2];
    B[0][j] = v1 * g[0];
    B[1][j] = v2 * g[1];
    B[2][j] = v3 * g[2];
    B[3][j] = v2 * g[2] + v3 * g[1];
    B[4][j] = v1 * g[2] + v3 * g[0];
    B[5][j] = v1 * g[1] + v2 * g[0];
  }
}

/* Element matrices of the TL operators.  mode 0: material tangent
 * (Felem, law); mode 1: initial stress from nodal S (Telem = S, law ignored);
 * mode 2: initial stress from nodal C with law.  Ke row-major (3 npe)^2. */
static int tl_element(int mode, int npe, int nip, const double *w, const double *N,
                      const double *dN, const double *X, const double *Tn, int law,
                      const double *prm, double *Ke) {
  size_t nd = 3 * (size_t)npe;
  double *g = (double *)malloc(sizeof(double) * npe * 3);
  double *Bs = (double *)malloc(sizeof(double) * npe * 18);
  double *Ts = (double *)malloc(sizeof(double) * npe * 18);
  double *acc = (double *)calloc((size_t)npe * npe * 9, sizeof(double)); /* pair (a,b): 9 */
  int rc = 0;
  for (int q = 0; q < nip && !rc; ++q) {
    double invJ[9];
    double det = orc_geom(3, npe, X, dN + (size_t)q * npe * 3, invJ);
    if (!(det > 0.0)) { rc = -1; break; }
    double wq = det * w[q];
    const double *Nq = N + (size_t)q * npe;
    for (int a = 0; a < npe; ++a) {
      const double *d = dN + ((size_t)q * npe + a) * 3;
      for (int i = 0; i < 3; ++i) {
        double s = 0.0;
        for (int j = 0; j < 3; ++j) s = fma(invJ[3 * j + i], d[j], s);
        g[3 * a + i] = s;
      }
    }
    if (mode == 0 || mode == 3) {
      double F[3][3], C[3][3], S[3][3], D[36];
      interp_tensor(npe, Nq, Tn, F);
      right_cauchy_green(F, C);
      if (orc_law(law, prm, C, S, D)) { rc = -2; break; }
      for (int b = 0; b < npe; ++b) {
        double B[6][3];
        tl_B(F, g + 3 * b, B);
        for (int I = 0; I < 6; ++I)
          for (int j = 0; j < 3; ++j) Bs[b * 18 + I * 3 + j] = B[I][j];
        for (int I = 0; I < 6; ++I)
          for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int J = 0; J < 6; ++J) s = fma(D[I * 6 + J], B[J][j], s);
            Ts[b * 18 + I * 3 + j] = s * wq;
          }
      }
      for (int a = 0; a < npe; ++a)
        for (int b = a; b < npe; ++b) {
          double *A = acc + ((size_t)a * npe + b) * 9;
          for (int i = 0; i < 3; ++i)
            for (int j = (a == b ? i : 0); j < 3; ++j) {
              double s = A[i * 3 + j];
              for (int I = 0; I < 6; ++I) s = fma(Bs[a * 18 + I * 3 + i], Ts[b * 18 + I * 3 + j], s);
              A[i * 3 + j] = s;
            }
          if (mode == 3) {  /* consistent tangent: geometric part from the same S */
            const double *ga = g + 3 * a, *gb = g + 3 * b;
            double t[3];
            for (int I = 0; I < 3; ++I) {
              double s = 0.0;
              for (int J = 0; J < 3; ++J) s = fma(S[I][J], gb[J], s);
              t[I] = s;
            }
            double v = 0.0;
            for (int I = 0; I < 3; ++I) v = fma(ga[I], t[I], v);
            for (int i = 0; i < 3; ++i) A[i * 3 + i] = fma(v, wq, A[i * 3 + i]);
          }
        }
    } else {
      double S[3][3];
      if (mode == 1) {
        interp_tensor(npe, Nq, Tn, S);
      } else {
        double C[3][3], D[36];
        interp_tensor(npe, Nq, Tn, C);
        if (orc_law(law, prm, C, S, D)) { rc = -2; break; }
      }
      for (int a = 0; a < npe; ++a)
        for (int b = a; b < npe; ++b) {
          const double *ga = g + 3 * a, *gb = g + 3 * b;
          double t[3];
          for (int I = 0; I < 3; ++I) {
            double s = 0.0;
            for (int J = 0; J < 3; ++J) s = fma(S[I][J], gb[J], s);
            t[I] = s;
          }
          double v = 0.0;
          for (int I = 0; I < 3; ++I) v = fma(ga[I], t[I], v);
          double *A = acc + ((size_t)a * npe + b) * 9;
          A[0] = fma(v, wq, A[0]);
        }
    }
  }
  if (!rc) {
    memset(Ke, 0, sizeof(double) * nd * nd);
    for (int a = 0; a < npe; ++a)
      for (int b = a; b < npe; ++b) {
        const double *A = acc + ((size_t)a * npe + b) * 9;
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) {
            double v;
            if (mode == 0 || mode == 3)
              v = (a == b && j < i) ? A[j * 3 + i] : A[i * 3 + j];
            else
              v = (i == j) ? A[0] : 0.0;
            Ke[((size_t)a * 3 + i) * nd + (size_t)b * 3 + j] = v;
            Ke[((size_t)b * 3 + j) * nd + (size_t)a * 3 + i] = v;
          }
      }
  }
  free(g); free(Bs); free(Ts); free(acc);
  return rc;
}

/* Global TL matrix in the reference's order: element triplets (row a, col b,
 * Ke[a,b], src/nonlinear.jl:2249-2256), sparse, dropzeros!. */
orc_csc *orc_tl_matrix(int mode, int64_t non, const double *xyz, int64_t nel, int npe,
                       const int32_t *conn, int nip, const double *w, const double *N,
                       const double *dN, const double *Telem, int law, const double *prm,
                       int *err) {
  size_t nd = 3 * (size_t)npe;
  double *Ke = (double *)malloc(sizeof(double) * nd * nd);
  double *X = (double *)malloc(sizeof(double) * npe * 3);
  coo c = {0};
  c.n = non * 3;
  *err = 0;
  for (int64_t e = 0; e < nel; ++e) {
    for (int a = 0; a < npe; ++a)
      for (int i = 0; i < 3; ++i) X[3 * a + i] = xyz[3 * (int64_t)conn[e * npe + a] + i];
    int rc = tl_element(mode, npe, nip, w, N, dN, X, Telem + (size_t)e * 9 * npe, law, prm, Ke);
    if (rc) {
      *err = rc;
      free(Ke); free(X); free(c.I); free(c.J); free(c.V);
      return NULL;
    }
    for (size_t k = 0; k < nd; ++k)
      for (size_t l = 0; l < nd; ++l)
        coo_push(&c, (int64_t)conn[e * npe + k / 3] * 3 + (int64_t)(k % 3),
                 (int64_t)conn[e * npe + l / 3] * 3 + (int64_t)(l % 3), Ke[k * nd + l]);
  }
  orc_csc *m = coo_to_csc(&c);
  free(c.I); free(c.J); free(c.V); free(Ke); free(X);
  orc_dropzeros(m);
  return m;
}

/* Internal force (src/nonlinear.jl:2738-2910): per point P = F S (energy)
 * or P interpolated; fe[a,i] = fma(P_iJ g_aJ chain, w, fe); element vectors
 * added into f in element order. mode 0: Telem = F with law; 1: Telem = P. */
int orc_tl_internal_force(int mode, int64_t non, const double *xyz, int64_t nel, int npe,
                          const int32_t *conn, int nip, const double *w, const double *N,
                          const double *dN, const double *Telem, int law, const double *prm,
                          double *f) {
  double *X = (double *)malloc(sizeof(double) * npe * 3);
  double *fe = (double *)malloc(sizeof(double) * npe * 3);
  int rc = 0;
  for (int64_t i = 0; i < 3 * non; ++i) f[i] = 0.0;
  for (int64_t e = 0; e < nel && !rc; ++e) {
    for (int a = 0; a < npe; ++a)
      for (int i = 0; i < 3; ++i) X[3 * a + i] = xyz[3 * (int64_t)conn[e * npe + a] + i];
    for (int k = 0; k < 3 * npe; ++k) fe[k] = 0.0;
    const double *Tn = Telem + (size_t)e * 9 * npe;
    for (int q = 0; q < nip; ++q) {
      double invJ[9];
      double det = orc_geom(3, npe, X, dN + (size_t)q * npe * 3, invJ);
      if (!(det > 0.0)) { rc = -1; break; }
      double wq = det * w[q];
      const double *Nq = N + (size_t)q * npe;
      double P[3][3];
      if (mode == 1) {
        interp_tensor(npe, Nq, Tn, P);
      } else {
        double F[3][3], C[3][3], S[3][3], D[36];
        interp_tensor(npe, Nq, Tn, F);
        right_cauchy_green(F, C);
        if (orc_law(law, prm, C, S, D)) { rc = -2; break; }
        for (int i = 0; i < 3; ++i)
          for (int J = 0; J < 3; ++J) {
            double s = 0.0;
            for (int K = 0; K < 3; ++K) s = fma(F[i][K], S[K][J], s);
            P[i][J] = s;
          }
      }
      for (int a = 0; a < npe; ++a) {
        const double *d = dN + ((size_t)q * npe + a) * 3;
        double g[3];
        for (int i = 0; i < 3; ++i) {
          double s = 0.0;
          for (int j = 0; j < 3; ++j) s = fma(invJ[3 * j + i], d[j], s);
          g[i] = s;
        }
        for (int i = 0; i < 3; ++i) {
          double v = 0.0;
          for (int J = 0; J < 3; ++J) v = fma(P[i][J], g[J], v);
          fe[3 * a + i] = fma(v, wq, fe[3 * a + i]);
        }
      }
    }
    if (rc) break;
    for (int a = 0; a < npe; ++a)
      for (int i = 0; i < 3; ++i) f[3 * (int64_t)conn[e * npe + a] + i] += fe[3 * a + i];
  }
  free(X); free(fe);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* The reference's own element arithmetic for stiffnessMatrix, threaded:    */
/* the CPU baseline of the benchmark (not a checker of the GPU bits).       */
/*                                                                          */
/* Per element and integration point q (src/linear.jl:190-330):             */
/*   J from the element's coordinates, J = sum_a x_a (x) dN_a(xi_q)          */
/*   (compute_element_geometry!, src/multifield.jl:1666-1743, standing in   */
/*   for gmsh getJacobians); dh[:,a] = inv(J)^T dN_ref[a];                  */
/*   B1 filled as fill_B_matrix! does (src/linear.jl:125-151): rows         */
/*   xx, yy, zz, xy, yz, zx (2D: xx, yy, xy), DoF columns interleaved;      */
/*   K1 += (((B1^T D) B1) b) detJ w, left to right, with D of               */
/*   constitutive_matrix (src/linear.jl:154-188).                           */
/* Global placement is the reference's transposed one (entry (nn2[l],       */
/* nn2[k]) receives K1[k,l]) scattered straight into the structural CSC     */
/* through one binary search per node pair, into one buffer per thread,     */
/* the buffers summed at the end: the reference's threaded direct-CSC       */
/* assembly (assemble_csc_worker! / reduce_csc_buffers!,                    */
/* src/multifield.jl:2394-2499, :2345-2380).  Values agree with             */
/* orc_assemble to rounding, not bit for bit.  Returns elapsed seconds.     */
/* ------------------------------------------------------------------------ */
static void orc_constitutive(int ptype, int dim, double E, double nu, double *D, int *rows) {
  int r = dim == 3 ? 6 : 3;
  *rows = r;
  for (int i = 0; i < r * r; ++i) D[i] = 0.0;
  if (dim == 3) {
    double c = E / ((1.0 + nu) * (1.0 - 2.0 * nu));
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) D[i * 6 + j] = c * (i == j ? 1.0 - nu : nu);
    for (int i = 3; i < 6; ++i) D[i * 6 + i] = c * ((1.0 - 2.0 * nu) / 2.0);
  } else if (ptype == PT_PLANE_STRESS) {
    double c = E / (1.0 - nu * nu);
    D[0] = c; D[1] = c * nu; D[3] = c * nu; D[4] = c; D[8] = c * ((1.0 - nu) / 2.0);
  } else {
    double c = E / ((1.0 + nu) * (1.0 - 2.0 * nu));
    D[0] = c * (1.0 - nu); D[1] = c * nu; D[3] = c * nu; D[4] = c * (1.0 - nu);
    D[8] = c * ((1.0 - 2.0 * nu) / 2.0);
  }
}

double orc_assemble_bdb_threaded(int ptype, int dim, const double *xyz, int64_t nel, int npe,
                                 const int32_t *conn, int nip, const double *w, const double *dN,
                                 double E, double nu, double thickness, orc_csc *pat, int nthreads,
                                 int chunk) {
  const int64_t nnz = pat->nnz;
  const int pdim = dim;
  const int nd = pdim * npe;
  double D[36];
  int rows = 0;
  orc_constitutive(ptype, dim, E, nu, D, &rows);
  const double b = (dim == 2 && ptype == PT_PLANE_STRESS) ? thickness : 1.0;
  int T = nthreads > 0 ? nthreads : 1;
#ifdef _OPENMP
  double t0 = omp_get_wtime();
#else
  double t0 = 0;
#endif
  double **bufs = (double **)malloc(sizeof(double *) * T);
#pragma omp parallel num_threads(T)
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
#else
    int tid = 0;
#endif
    double *nz = (double *)calloc(nnz + 1, sizeof(double));
    bufs[tid] = nz;
    double *X = (double *)malloc(sizeof(double) * npe * 3);
    double *dh = (double *)malloc(sizeof(double) * 3 * npe);
    double *B1 = (double *)malloc(sizeof(double) * rows * nd);
    double *BtD = (double *)malloc(sizeof(double) * nd * rows);
    double *K1 = (double *)malloc(sizeof(double) * nd * nd);
    int64_t nchunks = (nel + chunk - 1) / chunk;
    for (int64_t ch = tid; ch < nchunks; ch += T) {
      int64_t e0 = ch * chunk, e1 = e0 + chunk < nel ? e0 + chunk : nel;
      for (int64_t e = e0; e < e1; ++e) {
        for (int a = 0; a < npe; ++a)
          for (int i = 0; i < 3; ++i) X[3 * a + i] = xyz[3 * (int64_t)conn[e * npe + a] + i];
        memset(K1, 0, sizeof(double) * nd * nd);
        for (int q = 0; q < nip; ++q) {
          const double *dq = dN + (size_t)q * npe * 3;
          double J[3][3] = {{0}};
          for (int i = 0; i < dim; ++i)
            for (int j = 0; j < dim; ++j) {
              double acc = 0.0;
              for (int a = 0; a < npe; ++a) acc += X[3 * a + i] * dq[3 * a + j];
              J[i][j] = acc;
            }
          double iJ[9], det;
          if (dim == 3) {
            det = orc_inv3(J, iJ);
          } else {
            det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
            iJ[0] = J[1][1] / det; iJ[1] = -J[0][1] / det; iJ[3] = -J[1][0] / det; iJ[4] = J[0][0] / det;
          }
          det = fabs(det);
          /* dh[i][a] = sum_j inv(J)^T[i][j] dN[a][j] = sum_j iJ[j][i] dN[a][j] */
          for (int a = 0; a < npe; ++a)
            for (int i = 0; i < dim; ++i) {
              double acc = 0.0;
              for (int j = 0; j < dim; ++j) acc += iJ[j * 3 + i] * dq[3 * a + j];
              dh[i * npe + a] = acc;
            }
          memset(B1, 0, sizeof(double) * rows * nd);
          for (int l = 0; l < npe; ++l) {
            const double h1 = dh[l], h2 = dh[npe + l];
            if (dim == 3) {
              const double h3 = dh[2 * npe + l];
              const int cx = 3 * l, cy = 3 * l + 1, cz = 3 * l + 2;
              B1[0 * nd + cx] = h1; B1[1 * nd + cy] = h2; B1[2 * nd + cz] = h3;
              B1[3 * nd + cx] = h2; B1[3 * nd + cy] = h1;
              B1[4 * nd + cy] = h3; B1[4 * nd + cz] = h2;
              B1[5 * nd + cx] = h3; B1[5 * nd + cz] = h1;
            } else {
              const int cx = 2 * l, cy = 2 * l + 1;
              B1[0 * nd + cx] = h1; B1[1 * nd + cy] = h2;
              B1[2 * nd + cx] = h2; B1[2 * nd + cy] = h1;
            }
          }
          /* (B1^T D): nd x rows */
          for (int k = 0; k < nd; ++k)
            for (int c = 0; c < rows; ++c) {
              double acc = 0.0;
              for (int r = 0; r < rows; ++r) acc += B1[r * nd + k] * D[r * rows + c];
              BtD[k * rows + c] = acc;
            }
          /* ((B1^T D) B1) b detJ w, added to K1 */
          const double wq = w[q];
          for (int k = 0; k < nd; ++k)
            for (int l = 0; l < nd; ++l) {
              double acc = 0.0;
              for (int r = 0; r < rows; ++r) acc += BtD[k * rows + r] * B1[r * nd + l];
              K1[k * nd + l] += ((acc * b) * det) * wq;
            }
        }
        /* transposed placement: column nn2[k], row nn2[l] <- K1[k][l] */
        for (int bn = 0; bn < npe; ++bn) {
          int64_t Bnode = conn[e * npe + bn];
          int64_t col0 = Bnode * pdim;
          for (int an = 0; an < npe; ++an) {
            int64_t A = conn[e * npe + an];
            int64_t p0 = find_pos(pat->rowval, pat->colptr[col0], pat->colptr[col0 + 1], A * pdim);
            int64_t off = p0 - pat->colptr[col0];
            for (int j = 0; j < pdim; ++j) {
              int64_t base = pat->colptr[col0 + j] + off;
              for (int i = 0; i < pdim; ++i) nz[base + i] += K1[((size_t)bn * pdim + j) * nd + an * pdim + i];
            }
          }
        }
      }
    }
    free(X); free(dh); free(B1); free(BtD); free(K1);
  }
#pragma omp parallel for num_threads(T) schedule(static)
  for (int64_t k = 0; k < nnz; ++k) {
    double s = 0.0;
    for (int t = 0; t < T; ++t) s += bufs[t][k];
    pat->nzval[k] = s;
  }
  for (int t = 0; t < T; ++t) free(bufs[t]);
  free(bufs);
#ifdef _OPENMP
  return omp_get_wtime() - t0;
#else
  return 0.0;
#endif
}
