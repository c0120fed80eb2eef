// Built-in quadrature rules and Lagrange shape tables.
//
// These stand in for the gmsh calls the reference makes per element type:
//   getIntegrationPoints(et, "Gauss" * string(2*order+1))   src/linear.jl:235
//   getBasisFunctions(et, ip, "GradLagrange")               src/linear.jl:238
//   getBasisFunctions(et, ip, "Lagrange")                   src/linear.jl:1909
// A caller holding gmsh's own tables passes them with llf_tables_upload
// instead; the kernels never depend on which rule produced the tables.
//
// Rules (all exact to polynomial degree 2*order+1, as "Gauss(2p+1)" is):
//   line / quad / hex : tensor Gauss-Legendre, order+1 points per direction
//                       (the same point count gmsh uses for these shapes);
//   tri / tet         : collapsed (conical product) Gauss-Jacobi rules with
//                       order+1 points per direction, positive weights.
// Nodes/weights come from the Golub-Welsch method: eigenvalues of the
// symmetric tridiagonal Jacobi matrix of the weight (1-x)^a, computed here by
// cyclic Jacobi rotations.
//
// Node order inside an element: vertices, then edge-interior nodes (edge by
// edge, from the first to the second vertex), then face-interior nodes, then
// volume-interior nodes, each interior block ordered recursively as a lower
// order element of the same shape.  With gmsh's vertex/edge/face lists this
// is gmsh's order for orders 1 and 2 (quad4/9, hex8/27, tri3/6, tet4/10).
#include <cmath>
#include <cstring>
#include <vector>
#include <array>
#include <stdexcept>
#include <algorithm>

#include "tables.h"

namespace llf {

namespace {

// Symmetric eigen-decomposition of a small dense matrix by cyclic Jacobi
// rotations.  A (n x n, row-major) is destroyed; eigenvalues in ev, the
// eigenvectors in the columns of V.
void jacobi_eig(int n, std::vector<double> &A, std::vector<double> &ev,
                std::vector<double> &V) {
  V.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i) V[i * n + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) off += A[i * n + j] * A[i * n + j];
    if (off < 1e-300) break;
    for (int p = 0; p < n; ++p) {
      for (int q = p + 1; q < n; ++q) {
        double apq = A[p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        double app = A[p * n + p], aqq = A[q * n + q];
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) /
                   (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // A <- A J
          double akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = c * akp - s * akq;
          A[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // A <- J^T A
          double apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = c * apk - s * aqk;
          A[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = c * vkp - s * vkq;
          V[k * n + q] = s * vkp + c * vkq;
        }
      }
    }
  }
  ev.resize(n);
  for (int i = 0; i < n; ++i) ev[i] = A[i * n + i];
}

// Gauss-Jacobi rule on [0,1] for the weight (1-u)^alpha, n points, sorted
// ascending.  Recurrence coefficients of the Jacobi polynomials P^(alpha,0).
void gauss_jacobi01(int n, int alpha, std::vector<double> &x,
                    std::vector<double> &w) {
  const double a = alpha, b = 0.0;
  std::vector<double> J(n * n, 0.0);
  for (int k = 0; k < n; ++k) {
    double diag;
    if (k == 0) {
      diag = (b - a) / (a + b + 2.0);
    } else {
      double s = 2.0 * k + a + b;
      diag = (b * b - a * a) / (s * (s + 2.0));
    }
    J[k * n + k] = diag;
    if (k >= 1) {
      double s = 2.0 * k + a + b;
      double num = 4.0 * k * (k + a) * (k + b) * (k + a + b);
      double den = s * s * (s + 1.0) * (s - 1.0);
      double off = std::sqrt(num / den);
      J[k * n + k - 1] = off;
      J[(k - 1) * n + k] = off;
    }
  }
  std::vector<double> diag(n), off(n + 1, 0.0);
  for (int k = 0; k < n; ++k) diag[k] = J[k * n + k];
  for (int k = 1; k < n; ++k) off[k] = J[k * n + k - 1];
  std::vector<double> ev, V;
  jacobi_eig(n, J, ev, V);
  // mu0 = int_{-1}^{1} (1-x)^a dx = 2^(a+1)/(a+1)
  double mu0 = std::pow(2.0, a + 1.0) / (a + 1.0);
  // Orthonormal polynomials p_0..p_n by the three-term recurrence of the
  // Jacobi matrix: off[k+1] p_{k+1} = (x - diag[k]) p_k - off[k] p_{k-1}.
  auto orth = [&](double x, double *pn, double *dpn, double *christ) {
    double pm = 0.0, p = 1.0 / std::sqrt(mu0), dpm = 0.0, dp = 0.0, c = p * p;
    for (int k = 0; k < n; ++k) {
      double bnext = (k + 1 < n) ? off[k + 1] : 1.0;
      double pnew = ((x - diag[k]) * p - off[k] * pm) / bnext;
      double dnew = (p + (x - diag[k]) * dp - off[k] * dpm) / bnext;
      pm = p; p = pnew; dpm = dp; dp = dnew;
      if (k + 1 < n) c += p * p;
    }
    *pn = p; *dpn = dp; *christ = c;
  };
  std::vector<std::pair<double, double>> xw(n);
  for (int i = 0; i < n; ++i) {
    double x = ev[i], pn, dpn, c;
    for (int it = 0; it < 3; ++it) {  // Newton polish of the eigenvalue
      orth(x, &pn, &dpn, &c);
      if (dpn != 0.0) x -= pn / dpn;
    }
    orth(x, &pn, &dpn, &c);
    xw[i] = {x, 1.0 / c};  // Christoffel weight
  }
  std::sort(xw.begin(), xw.end());
  x.resize(n);
  w.resize(n);
  // map [-1,1] -> [0,1]: u = (1+x)/2, (1-u)^a du = 2^-(a+1) (1-x)^a dx
  double scale = std::pow(0.5, a + 1.0);
  for (int i = 0; i < n; ++i) {
    x[i] = 0.5 * (1.0 + xw[i].first);
    w[i] = xw[i].second * scale;
  }
}

// Gauss-Legendre on [-1,1].
void gauss_legendre(int n, std::vector<double> &x, std::vector<double> &w) {
  std::vector<double> u, wu;
  gauss_jacobi01(n, 0, u, wu);
  x.resize(n);
  w.resize(n);
  for (int i = 0; i < n; ++i) {
    x[i] = 2.0 * u[i] - 1.0;
    w[i] = 2.0 * wu[i];
  }
  // symmetrise (the rule is symmetric; remove eigen-solver round-off)
  for (int i = 0; i < n / 2; ++i) {
    double xm = 0.5 * (x[n - 1 - i] - x[i]);
    double wm = 0.5 * (w[i] + w[n - 1 - i]);
    x[i] = -xm;
    x[n - 1 - i] = xm;
    w[i] = wm;
    w[n - 1 - i] = wm;
  }
  if (n % 2 == 1) x[n / 2] = 0.0;
}

// ---------------------------------------------------------------- node order
// Integer lattice coordinates of element nodes.  Tensor shapes use indices
// 0..p per direction (reference coordinate -1 + 2 i/p); simplices use
// barycentric-style indices 0..p per coordinate (reference coordinate i/p).
using Pt = std::array<int, 3>;

// Nodes of a quadrilateral of order `len` laid on the lattice points
// o + i*du + j*dv (0 <= i,j <= len), in the recursive vertex/edge/interior
// order.  len==0 is a single point.
void quad_lattice(int len, Pt o, Pt du, Pt dv, std::vector<Pt> &out) {
  auto at = [&](int i, int j) {
    return Pt{o[0] + i * du[0] + j * dv[0], o[1] + i * du[1] + j * dv[1],
              o[2] + i * du[2] + j * dv[2]};
  };
  if (len < 0) return;
  if (len == 0) {
    out.push_back(at(0, 0));
    return;
  }
  const int vi[4] = {0, len, len, 0}, vj[4] = {0, 0, len, len};
  for (int v = 0; v < 4; ++v) out.push_back(at(vi[v], vj[v]));
  for (int e = 0; e < 4; ++e) {
    int a = e, b = (e + 1) % 4;
    for (int s = 1; s < len; ++s) {
      int i = vi[a] + (vi[b] - vi[a]) * s / len;
      int j = vj[a] + (vj[b] - vj[a]) * s / len;
      out.push_back(at(i, j));
    }
  }
  if (len >= 2) {
    Pt o2 = at(1, 1);
    quad_lattice(len - 2, o2, du, dv, out);
  }
}

void hex_lattice(int len, Pt o, std::vector<Pt> &out) {
  auto at = [&](int i, int j, int k) {
    return Pt{o[0] + i, o[1] + j, o[2] + k};
  };
  if (len < 0) return;
  if (len == 0) {
    out.push_back(at(0, 0, 0));
    return;
  }
  const int L = len;
  const int V[8][3] = {{0, 0, 0}, {L, 0, 0}, {L, L, 0}, {0, L, 0},
                       {0, 0, L}, {L, 0, L}, {L, L, L}, {0, L, L}};
  for (int v = 0; v < 8; ++v) out.push_back(at(V[v][0], V[v][1], V[v][2]));
  static const int E[12][2] = {{0, 1}, {0, 3}, {0, 4}, {1, 2}, {1, 5}, {2, 3},
                               {2, 6}, {3, 7}, {4, 5}, {4, 7}, {5, 6}, {6, 7}};
  for (int e = 0; e < 12; ++e) {
    const int *a = V[E[e][0]], *b = V[E[e][1]];
    for (int s = 1; s < L; ++s)
      out.push_back(at(a[0] + (b[0] - a[0]) * s / L, a[1] + (b[1] - a[1]) * s / L,
                       a[2] + (b[2] - a[2]) * s / L));
  }
  static const int F[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {0, 4, 7, 3},
                              {1, 2, 6, 5}, {2, 3, 7, 6}, {4, 5, 6, 7}};
  if (L >= 2) {
    for (int f = 0; f < 6; ++f) {
      const int *v0 = V[F[f][0]], *v1 = V[F[f][1]], *v3 = V[F[f][3]];
      Pt du{(v1[0] - v0[0]) / L, (v1[1] - v0[1]) / L, (v1[2] - v0[2]) / L};
      Pt dv{(v3[0] - v0[0]) / L, (v3[1] - v0[1]) / L, (v3[2] - v0[2]) / L};
      Pt o2{o[0] + v0[0] + du[0] + dv[0], o[1] + v0[1] + du[1] + dv[1],
            o[2] + v0[2] + du[2] + dv[2]};
      quad_lattice(L - 2, o2, du, dv, out);
    }
    hex_lattice(L - 2, Pt{o[0] + 1, o[1] + 1, o[2] + 1}, out);
  }
}

// Triangle of order len on lattice points o + i*du + j*dv (i,j>=0, i+j<=len).
void tri_lattice(int len, Pt o, Pt du, Pt dv, std::vector<Pt> &out) {
  auto at = [&](int i, int j) {
    return Pt{o[0] + i * du[0] + j * dv[0], o[1] + i * du[1] + j * dv[1],
              o[2] + i * du[2] + j * dv[2]};
  };
  if (len < 0) return;
  if (len == 0) {
    out.push_back(at(0, 0));
    return;
  }
  const int vi[3] = {0, len, 0}, vj[3] = {0, 0, len};
  for (int v = 0; v < 3; ++v) out.push_back(at(vi[v], vj[v]));
  for (int e = 0; e < 3; ++e) {
    int a = e, b = (e + 1) % 3;
    for (int s = 1; s < len; ++s)
      out.push_back(at(vi[a] + (vi[b] - vi[a]) * s / len,
                       vj[a] + (vj[b] - vj[a]) * s / len));
  }
  if (len >= 3) {
    Pt o2 = at(1, 1);
    tri_lattice(len - 3, o2, du, dv, out);
  }
}

void tet_lattice(int len, Pt o, std::vector<Pt> &out) {
  auto at = [&](int i, int j, int k) {
    return Pt{o[0] + i, o[1] + j, o[2] + k};
  };
  if (len < 0) return;
  if (len == 0) {
    out.push_back(at(0, 0, 0));
    return;
  }
  const int L = len;
  const int V[4][3] = {{0, 0, 0}, {L, 0, 0}, {0, L, 0}, {0, 0, L}};
  for (int v = 0; v < 4; ++v) out.push_back(at(V[v][0], V[v][1], V[v][2]));
  static const int E[6][2] = {{0, 1}, {1, 2}, {2, 0}, {3, 0}, {3, 2}, {3, 1}};
  for (int e = 0; e < 6; ++e) {
    const int *a = V[E[e][0]], *b = V[E[e][1]];
    for (int s = 1; s < L; ++s)
      out.push_back(at(a[0] + (b[0] - a[0]) * s / L, a[1] + (b[1] - a[1]) * s / L,
                       a[2] + (b[2] - a[2]) * s / L));
  }
  static const int F[4][3] = {{0, 2, 1}, {0, 1, 3}, {0, 3, 2}, {3, 1, 2}};
  if (L >= 3) {
    for (int f = 0; f < 4; ++f) {
      const int *v0 = V[F[f][0]], *v1 = V[F[f][1]], *v2 = V[F[f][2]];
      Pt du{(v1[0] - v0[0]) / L, (v1[1] - v0[1]) / L, (v1[2] - v0[2]) / L};
      Pt dv{(v2[0] - v0[0]) / L, (v2[1] - v0[1]) / L, (v2[2] - v0[2]) / L};
      Pt o2{o[0] + v0[0] + du[0] + dv[0], o[1] + v0[1] + du[1] + dv[1],
            o[2] + v0[2] + du[2] + dv[2]};
      tri_lattice(L - 3, o2, du, dv, out);
    }
    if (L >= 4) tet_lattice(L - 4, Pt{o[0] + 1, o[1] + 1, o[2] + 1}, out);
  }
}

// 1D Lagrange polynomial on equispaced points t_m = -1 + 2m/p, index i;
// value and derivative at x.
void lagrange1d(int p, int i, double x, double &val, double &der) {
  double xi = -1.0 + 2.0 * i / p;
  val = 1.0;
  der = 0.0;
  for (int m = 0; m <= p; ++m) {
    if (m == i) continue;
    double xm = -1.0 + 2.0 * m / p;
    double f = (x - xm) / (xi - xm);
    der = der * f + val / (xi - xm);
    val *= f;
  }
}

// Silvester factor R_k(l) = prod_{s<k} (p l - s)/(s+1) and its derivative.
void silvester(int p, int k, double l, double &val, double &der) {
  val = 1.0;
  der = 0.0;
  for (int s = 0; s < k; ++s) {
    double f = (p * l - s) / (s + 1.0);
    der = der * f + val * (p / (s + 1.0));
    val *= f;
  }
}

}  // namespace

int shape_dim(int family) {
  switch (family) {
    case FAM_LINE: return 1;
    case FAM_TRI: case FAM_QUAD: return 2;
    case FAM_TET: case FAM_HEX: return 3;
  }
  return -1;
}

int num_nodes(int family, int p) {
  switch (family) {
    case FAM_LINE: return p + 1;
    case FAM_QUAD: return (p + 1) * (p + 1);
    case FAM_HEX: return (p + 1) * (p + 1) * (p + 1);
    case FAM_TRI: return (p + 1) * (p + 2) / 2;
    case FAM_TET: return (p + 1) * (p + 2) * (p + 3) / 6;
  }
  return -1;
}

bool node_lattice(int family, int p, std::vector<std::array<int, 3>> &pts) {
  pts.clear();
  switch (family) {
    case FAM_LINE:
      pts.push_back({0, 0, 0});
      if (p >= 1) pts.push_back({p, 0, 0});
      for (int s = 1; s < p; ++s) pts.push_back({s, 0, 0});
      break;
    case FAM_QUAD:
      quad_lattice(p, Pt{0, 0, 0}, Pt{1, 0, 0}, Pt{0, 1, 0}, pts);
      break;
    case FAM_HEX:
      hex_lattice(p, Pt{0, 0, 0}, pts);
      break;
    case FAM_TRI:
      tri_lattice(p, Pt{0, 0, 0}, Pt{1, 0, 0}, Pt{0, 1, 0}, pts);
      break;
    case FAM_TET:
      tet_lattice(p, Pt{0, 0, 0}, pts);
      break;
    default:
      return false;
  }
  return (int)pts.size() == num_nodes(family, p);
}

bool eval_basis(int family, int p, const double *pts, int npts, double *Nout, double *dNout) {
  int d = shape_dim(family);
  std::vector<std::array<int, 3>> lat;
  if (d < 0 || !node_lattice(family, p, lat)) return false;
  const int npe = (int)lat.size();
  const bool tensor = (family == FAM_LINE || family == FAM_QUAD || family == FAM_HEX);
  for (int q = 0; q < npts; ++q) {
    const double *x = pts + 3 * q;
    for (int a = 0; a < npe; ++a) {
      double val = 1.0, g[3] = {0.0, 0.0, 0.0};
      if (tensor) {
        double v1[3] = {1, 1, 1}, d1[3] = {0, 0, 0};
        for (int j = 0; j < d; ++j) lagrange1d(p, lat[a][j], x[j], v1[j], d1[j]);
        val = v1[0] * v1[1] * v1[2];
        g[0] = d1[0] * v1[1] * v1[2];
        if (d >= 2) g[1] = v1[0] * d1[1] * v1[2];
        if (d >= 3) g[2] = v1[0] * v1[1] * d1[2];
      } else {
        int k0 = p;
        for (int j = 0; j < d; ++j) k0 -= lat[a][j];
        double l0 = 1.0;
        for (int j = 0; j < d; ++j) l0 -= x[j];
        double r0, dr0, rj[3], drj[3];
        silvester(p, k0, l0, r0, dr0);
        for (int j = 0; j < d; ++j) silvester(p, lat[a][j], x[j], rj[j], drj[j]);
        val = r0;
        for (int j = 0; j < d; ++j) val *= rj[j];
        for (int m = 0; m < d; ++m) {
          double t1 = -dr0, t2 = r0 * drj[m];
          for (int j = 0; j < d; ++j) {
            t1 *= rj[j];
            if (j != m) t2 *= rj[j];
          }
          g[m] = t1 + t2;
        }
      }
      Nout[(size_t)q * npe + a] = val;
      for (int j = 0; j < 3; ++j) dNout[((size_t)q * npe + a) * 3 + j] = g[j];
    }
  }
  return true;
}

bool build_rule(int family, int p, Rule &r) {
  if (p < 1 || p > 4) return false;
  int d = shape_dim(family);
  if (d < 0) return false;
  std::vector<std::array<int, 3>> lat;
  if (!node_lattice(family, p, lat)) return false;
  r.family = family;
  r.order = p;
  r.dim = d;
  r.npe = (int)lat.size();
  r.node_ref.assign(3 * r.npe, 0.0);
  const bool tensor = (family == FAM_LINE || family == FAM_QUAD || family == FAM_HEX);
  for (int a = 0; a < r.npe; ++a)
    for (int j = 0; j < d; ++j)
      r.node_ref[3 * a + j] = tensor ? (-1.0 + 2.0 * lat[a][j] / p)
                                     : (double)lat[a][j] / p;

  // ---- quadrature
  const int n = p + 1;
  r.xi.clear();
  r.w.clear();
  if (tensor) {
    std::vector<double> x, w;
    gauss_legendre(n, x, w);
    int nz = d >= 3 ? n : 1, ny = d >= 2 ? n : 1;
    for (int k = 0; k < nz; ++k)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < n; ++i) {
          r.xi.push_back(x[i]);
          r.xi.push_back(d >= 2 ? x[j] : 0.0);
          r.xi.push_back(d >= 3 ? x[k] : 0.0);
          double ww = w[i];
          if (d >= 2) ww *= w[j];
          if (d >= 3) ww *= w[k];
          r.w.push_back(ww);
        }
  } else if (family == FAM_TRI) {
    std::vector<double> u, wu, v, wv;
    gauss_jacobi01(n, 1, u, wu);
    gauss_jacobi01(n, 0, v, wv);
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        r.xi.push_back(u[i]);
        r.xi.push_back((1.0 - u[i]) * v[j]);
        r.xi.push_back(0.0);
        r.w.push_back(wu[i] * wv[j]);
      }
  } else {  // TET
    std::vector<double> u, wu, v, wv, t, wt;
    gauss_jacobi01(n, 2, u, wu);
    gauss_jacobi01(n, 1, v, wv);
    gauss_jacobi01(n, 0, t, wt);
    for (int k = 0; k < n; ++k)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          double x = u[i], y = (1.0 - u[i]) * v[j],
                 z = (1.0 - u[i]) * (1.0 - v[j]) * t[k];
          r.xi.push_back(x);
          r.xi.push_back(y);
          r.xi.push_back(z);
          r.w.push_back(wu[i] * wv[j] * wt[k]);
        }
  }
  r.nip = (int)r.w.size();

  // ---- basis values and reference gradients at the points
  r.N.assign((size_t)r.nip * r.npe, 0.0);
  r.dN.assign((size_t)r.nip * r.npe * 3, 0.0);
  eval_basis(family, p, r.xi.data(), r.nip, r.N.data(), r.dN.data());
  // gradients at the element's own nodes (for nodal gradient fields)
  r.dN_nodes.assign((size_t)r.npe * r.npe * 3, 0.0);
  std::vector<double> Nn((size_t)r.npe * r.npe);
  eval_basis(family, p, r.node_ref.data(), r.npe, Nn.data(), r.dN_nodes.data());
  return true;
}

}  // namespace llf
