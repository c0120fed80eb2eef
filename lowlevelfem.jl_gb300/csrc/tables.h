// Built-in quadrature rules and Lagrange shape tables (host side).
#pragma once
#include <array>
#include <vector>

namespace llf {

enum { FAM_LINE = 1, FAM_TRI = 2, FAM_QUAD = 3, FAM_TET = 4, FAM_HEX = 5 };

struct Rule {
  int family = 0, order = 0, dim = 0, npe = 0, nip = 0;
  std::vector<double> xi;        // 3*nip reference coordinates
  std::vector<double> w;         // nip weights
  std::vector<double> N;         // nip*npe values,   N[q*npe+a]
  std::vector<double> dN;        // nip*npe*3 grads,  dN[(q*npe+a)*3+j]
  std::vector<double> node_ref;  // 3*npe reference node coordinates
  std::vector<double> dN_nodes;  // npe*npe*3 grads at the nodes, [(k*npe+a)*3+j]
};

int shape_dim(int family);
int num_nodes(int family, int order);
// Integer lattice coordinates of the element's nodes in element node order.
bool node_lattice(int family, int order, std::vector<std::array<int, 3>> &pts);
bool build_rule(int family, int order, Rule &r);
// Values and reference gradients of the family's basis at npts points (3 coords each).
bool eval_basis(int family, int order, const double *pts, int npts, double *N, double *dN);

}  // namespace llf
