// setup.cpp -- host-side setup layer: structured mesh hierarchies, DOF
// numbering, CSR sparsity pattern, grid-transfer matrices and the reference
// tensors of the element contraction.  This is the part of ParMooN's setup
// (TDomain refinement, TFESpace::ConstructSpace, TStructure, FEDatabase
// prolongation matrices) that the hot path consumes as input; it runs once
// per mesh hierarchy and needs no GPU.
//
// Reference behaviour restated here:
//  * cell order after regular refinement: depth-first over the refinement
//    tree (src/Geometry/It_Finest.C), children and their local vertex order
//    from src/Refinement/RefQuadRegDesc.C:21-22 and RefHexaRegDesc.C:17-21;
//  * DOF numbering (src/FE/FESpace2D.C:83-312, FESpace.C:1863-2099,
//    FEMapper.C:456-600): the FE mapper keeps the smallest (cell, local dof)
//    position of every global DOF as its representative and the final pass
//    numbers representatives in traversal order, inner DOFs first, then
//    non-Dirichlet boundary DOFs, then Dirichlet DOFs.  make_space applies
//    that rule directly;
//  * TStructure (src/Matrix/Structure.C:226-618): full rows also for
//    Dirichlet DOFs, columns sorted ascending;
//  * GridTransfer::Prolongate / DefectRestriction (src/Multigrid/
//    GridTransfer.C:29-410): averaged child-local interpolation and its
//    transpose; written as two CSR matrices.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <unordered_map>

#include "cdg_internal.h"

namespace cdg {

// ---------------------------------------------------------------------------
// quadrature
// ---------------------------------------------------------------------------
void gauss_legendre(int n, double* x, double* w) {
  // roots of P_n by Newton's method from Tricomi's initial guesses, in
  // extended precision; nodes ascending
  for (int i = 0; i < n; ++i) {
    long double th = 3.14159265358979323846264338327950288L * (4 * i + 3) / (4 * n + 2);
    long double z = cosl(th);
    long double dp = 1;
    for (int it = 0; it < 64; ++it) {
      long double p0 = 1, p1 = z;
      for (int k = 2; k <= n; ++k) {
        long double pk = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = pk;
      }
      if (n == 1) { p1 = z; p0 = 1; }
      dp = n * (z * p1 - p0) / (z * z - 1);
      long double dz = p1 / dp;
      z -= dz;
      if (fabsl(dz) < 1e-32L) break;
    }
    x[n - 1 - i] = (double)z;
    w[n - 1 - i] = (double)(2.0L / ((1 - z * z) * dp * dp));
  }
}

int gauss_points_for_degree(int deg) {
  // QuadratureFormulaDatabase.C:41-81 (quad / hexa rules by accuracy)
  if (deg > 17) deg = 17;
  if (deg <= 2) return 2;
  if (deg <= 5) return 3;
  return deg / 2 + 1;
}

// ---------------------------------------------------------------------------
// reference element: tensor-product Lagrange Q1/Q2, local DOF k = k0 +
// (p+1)(k1 + (p+1)k2) at nodes {-1,1} (Q1) or {-1,0,1} (Q2), xi fastest
// (include/FE2D/BF_C_Q_Q{1,2}_2D.h, include/FE3D/BF_C_H_Q{1,2}_3D.h)
// ---------------------------------------------------------------------------
static void line_basis(int p, double t, double* v, double* d, double* dd) {
  if (p == 1) {
    v[0] = 0.5 * (1 - t); v[1] = 0.5 * (1 + t);
    d[0] = -0.5; d[1] = 0.5;
    dd[0] = 0; dd[1] = 0;
  } else {
    v[0] = 0.5 * t * (t - 1); v[1] = (1 - t) * (1 + t); v[2] = 0.5 * t * (t + 1);
    d[0] = t - 0.5; d[1] = -2 * t; d[2] = t + 0.5;
    dd[0] = 1; dd[1] = -2; dd[2] = 1;
  }
}

void local_dof_ref(int dim, int p, int k, double* r) {
  int n1 = p + 1;
  int i[3] = {k % n1, (k / n1) % n1, k / (n1 * n1)};
  for (int a = 0; a < 3; ++a) r[a] = (a < dim) ? -1.0 + (2.0 / p) * i[a] : 0.0;
}

// P1/P2 tetrahedron: local DOFs in the order of include/FE3D/NF_C_T_P2_3D.h
// (vertices 0, 2, 5, 9 and edge midpoints 1 (v0v1), 3 (v0v2), 4 (v1v2),
// 6 (v0v3), 7 (v1v3), 8 (v2v3)); P1: the four vertices
static const double kTetP2Nodes[10][3] = {{0, 0, 0},     {0.5, 0, 0}, {1, 0, 0},     {0, 0.5, 0},
                                          {0.5, 0.5, 0}, {0, 1, 0},   {0, 0, 0.5},   {0.5, 0, 0.5},
                                          {0, 0.5, 0.5}, {0, 0, 1}};
static const double kTetP1Nodes[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

void local_dof_ref_shape(int shape, int order, int k, double* r) {
  if (shape == kTetra) {
    const double* q = order == 1 ? kTetP1Nodes[k] : kTetP2Nodes[k];
    r[0] = q[0];
    r[1] = q[1];
    r[2] = q[2];
    return;
  }
  local_dof_ref(shape == kQuad ? 2 : 3, order, k, r);
}

// barycentric Lagrange basis on the reference tetrahedron, with gradient and
// Hessian (pairs 00,01,02,11,12,22) in reference coordinates
void tetra_basis_point(int order, const double* xi, double* val, double* grad, double* hess) {
  const double l[4] = {1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]};
  // d lambda_v / d xi_a
  auto dl = [](int v, int a) { return v == 0 ? -1.0 : (v - 1 == a ? 1.0 : 0.0); };
  const int nl = order == 1 ? 4 : 10;
  if (order == 1) {
    for (int k = 0; k < 4; ++k) {
      if (val) val[k] = l[k];
      if (grad)
        for (int a = 0; a < 3; ++a) grad[a * nl + k] = dl(k, a);
      if (hess)
        for (int s = 0; s < 6; ++s) hess[s * nl + k] = 0.0;
    }
    return;
  }
  // node k: vertex (va == vb) -> l(2l-1); edge -> 4 la lb
  static const int va[10] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3};
  static const int vb[10] = {0, 1, 1, 2, 2, 2, 3, 3, 3, 3};
  static const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {0, 1, 2, 1, 2, 2};
  for (int k = 0; k < 10; ++k) {
    const int a0 = va[k], b0 = vb[k];
    if (a0 == b0) {
      if (val) val[k] = l[a0] * (2.0 * l[a0] - 1.0);
      if (grad)
        for (int a = 0; a < 3; ++a) grad[a * nl + k] = (4.0 * l[a0] - 1.0) * dl(a0, a);
      if (hess)
        for (int s = 0; s < 6; ++s) hess[s * nl + k] = 4.0 * dl(a0, pa[s]) * dl(a0, pb[s]);
    } else {
      if (val) val[k] = 4.0 * l[a0] * l[b0];
      if (grad)
        for (int a = 0; a < 3; ++a) grad[a * nl + k] = 4.0 * (dl(a0, a) * l[b0] + l[a0] * dl(b0, a));
      if (hess)
        for (int s = 0; s < 6; ++s)
          hess[s * nl + k] = 4.0 * (dl(a0, pa[s]) * dl(b0, pb[s]) + dl(a0, pb[s]) * dl(b0, pa[s]));
    }
  }
}

void cell_point(int shape, int dim, const double* cv, const double* r, double* x) {
  if (shape == kTetra) {
    // TetraAffin: x = v0 + (v1-v0) xi + (v2-v0) eta + (v3-v0) zeta
    for (int c = 0; c < 3; ++c) {
      double s = cv[c];
      for (int a = 0; a < 3; ++a) s += r[a] * (cv[(a + 1) * 3 + c] - cv[c]);
      x[c] = s;
    }
    return;
  }
  // QuadAffin / HexaAffin: x = v0 + sum_a (r_a + 1)/2 (v_{e_a} - v0), e = (1, 3, 4)
  const int e[3] = {1, 3, 4};
  for (int c = 0; c < dim; ++c) {
    double s = cv[c];
    for (int a = 0; a < dim; ++a) s += 0.5 * (r[a] + 1.0) * (cv[e[a] * dim + c] - cv[c]);
    x[c] = s;
  }
}

// TQuadBilinear / THexaTrilinear::GetOrigFromRef: x = sum_v x_v N_v(r) with
// the Q1 vertex functions (vertices 0-3 counterclockwise at zeta = -1, 4-7
// above them); equal to the affine map on parallelograms / parallelepipeds
void cell_point_multilinear(int dim, const double* cv, const double* r, double* x) {
  static const int sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                               {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  const int nv = dim == 2 ? 4 : 8;
  for (int c = 0; c < dim; ++c) x[c] = 0.0;
  for (int v = 0; v < nv; ++v) {
    double n = 1.0;
    for (int a = 0; a < dim; ++a) n *= 0.5 * (1.0 + sg[v][a] * r[a]);
    for (int c = 0; c < dim; ++c) x[c] += n * cv[v * dim + c];
  }
}

// hess: symmetric pairs (a<=b) in order (00,01,11) / (00,01,02,11,12,22)
void ref_basis_point(int dim, int p, const double* xi, double* val, double* grad,
                     double* hess) {
  double v[3][3], d[3][3], dd[3][3];
  for (int a = 0; a < dim; ++a) line_basis(p, xi[a], v[a], d[a], dd[a]);
  int n1 = p + 1;
  int nloc = dim == 2 ? n1 * n1 : n1 * n1 * n1;
  for (int k = 0; k < nloc; ++k) {
    int i[3] = {k % n1, (k / n1) % n1, k / (n1 * n1)};
    // per direction: value, first, second derivative
    auto f = [&](int a, int order) {
      return order == 0 ? v[a][i[a]] : order == 1 ? d[a][i[a]] : dd[a][i[a]];
    };
    auto prod = [&](int o0, int o1, int o2) {
      double r = f(0, o0) * f(1, o1);
      if (dim == 3) r *= f(2, o2);
      return r;
    };
    if (val) val[k] = prod(0, 0, 0);
    if (grad) {
      grad[0 * nloc + k] = prod(1, 0, 0);
      grad[1 * nloc + k] = prod(0, 1, 0);
      if (dim == 3) grad[2 * nloc + k] = prod(0, 0, 1);
    }
    if (hess) {
      int np = dim == 2 ? 3 : 6;
      int pr = 0;
      for (int a = 0; a < dim; ++a)
        for (int b = a; b < dim; ++b) {
          int o[3] = {0, 0, 0};
          o[a] += 1;
          o[b] += 1;
          hess[pr * nloc + k] = prod(o[0], o[1], o[2]);
          ++pr;
        }
      (void)np;
    }
  }
}

// Quadrature on the reference tetrahedron by degree, as the reference picks it
// (QuadratureFormulaDatabase.C:30-37): degree <= 2 P2Tetra, 3-4 P4Tetra, 5-6
// P5Tetra (QuadFormula.C:1693,1739) -- Keast's symmetric rules (P. Keast,
// Moderate-degree tetrahedral quadrature formulas, Comput. Methods Appl. Mech.
// Engrg. 55 (1986) 339-348) with 4, 11 and 15 points.  They are returned as
// the code kTetraRule + degree of the rule; degrees above 6 (no element here
// needs them) take the collapsed Gauss rule below with (degree + 4) / 2
// points per direction.
int tetra_points_for_degree(int degree) {
  if (degree <= 2) return kTetraRule + 2;
  if (degree <= 4) return kTetraRule + 4;
  if (degree <= 6) return kTetraRule + 5;
  return (degree + 4) / 2;
}

int tetra_rule_size(int code) {
  if (code == kTetraRule + 2) return 4;
  if (code == kTetraRule + 4) return 11;
  if (code == kTetraRule + 5) return 15;
  return code * code * code;
}

namespace {
// one orbit of a symmetric rule in barycentric coordinates (l0, l1, l2, l3):
// kind 1 the centroid, kind 4 the permutations of (a, b, b, b), kind 6 those
// of (a, a, b, b); w the weight of each point (the weights sum to 1/6)
struct TetOrbit {
  int kind;
  double a, b, w;
};
void add_orbit(const TetOrbit& o, std::vector<double>& pts, std::vector<double>& wts) {
  auto put = [&](const double l[4]) {
    pts.push_back(l[1]);
    pts.push_back(l[2]);
    pts.push_back(l[3]);
    wts.push_back(o.w);
  };
  if (o.kind == 1) {
    const double l[4] = {0.25, 0.25, 0.25, 0.25};
    put(l);
  } else if (o.kind == 4) {
    for (int i = 0; i < 4; ++i) {
      double l[4] = {o.b, o.b, o.b, o.b};
      l[i] = o.a;
      put(l);
    }
  } else {
    for (int i = 0; i < 4; ++i)
      for (int j = i + 1; j < 4; ++j) {
        double l[4] = {o.b, o.b, o.b, o.b};
        l[i] = l[j] = o.a;
        put(l);
      }
  }
}
}  // namespace

static void keast_rule(int degree, std::vector<double>& pts, std::vector<double>& wts) {
  pts.clear();
  wts.clear();
  if (degree == 2) {
    add_orbit({4, 0.585410196624968454461376050311, 0.138196601125010515179541316563,
               1.0 / 24.0}, pts, wts);
  } else if (degree == 4) {
    add_orbit({1, 0.25, 0.25, -74.0 / 5625.0}, pts, wts);
    add_orbit({4, 11.0 / 14.0, 1.0 / 14.0, 343.0 / 45000.0}, pts, wts);
    add_orbit({6, 0.399403576166799204996102147462, 0.100596423833200795003897852538,
               56.0 / 2250.0}, pts, wts);
  } else {
    add_orbit({4, 0.0, 1.0 / 3.0, 0.602678571428571428571428571428571e-2}, pts, wts);
    add_orbit({1, 0.25, 0.25, 0.302836780970891758063769725577305e-1}, pts, wts);
    add_orbit({4, 8.0 / 11.0, 1.0 / 11.0, 0.116452490860289694108936091443380e-1}, pts, wts);
    add_orbit({6, 0.665501535736642982398804642263025e-1, 0.433449846426335701760119535773697,
               0.109491415613864593456430191124068e-1}, pts, wts);
  }
}

// collapsed (Duffy) Gauss rule on the reference tetrahedron with n points per
// direction: xi = u, eta = v (1-u), zeta = w (1-u)(1-v), exact for degree
// <= 2n-3 (the exact reference tensors take it with n = 5)
static void tetra_rule(int n, std::vector<double>& pts, std::vector<double>& wts) {
  if (n > kTetraRule) {
    keast_rule(n - kTetraRule, pts, wts);
    return;
  }
  double x[kMaxQp1], w[kMaxQp1];
  gauss_legendre(n, x, w);
  pts.clear();
  wts.clear();
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const double u = 0.5 * (x[i] + 1), v = 0.5 * (x[j] + 1), t = 0.5 * (x[k] + 1);
        pts.push_back(u);
        pts.push_back(v * (1 - u));
        pts.push_back(t * (1 - u) * (1 - v));
        wts.push_back(0.125 * w[i] * w[j] * w[k] * (1 - u) * (1 - u) * (1 - v));
      }
}

// quadrature points/weights on the reference cell of `shape`
static void shape_rule(int shape, int n, std::vector<double>& pts, std::vector<double>& wts) {
  if (shape == kTetra) {
    tetra_rule(n, pts, wts);
    return;
  }
  const int dim = shape == kQuad ? 2 : 3;
  double x[kMaxQp1], w[kMaxQp1];
  gauss_legendre(n, x, w);
  pts.clear();
  wts.clear();
  const int nq = dim == 2 ? n * n : n * n * n;
  for (int q = 0; q < nq; ++q) {
    const int qi[3] = {q % n, (q / n) % n, q / (n * n)};
    pts.push_back(x[qi[0]]);
    pts.push_back(x[qi[1]]);
    pts.push_back(dim == 3 ? x[qi[2]] : 0.0);
    wts.push_back(w[qi[0]] * w[qi[1]] * (dim == 3 ? w[qi[2]] : 1.0));
  }
}

static void basis_at(int shape, int p, const double* xi, double* val, double* grad, double* hess) {
  if (shape == kTetra)
    tetra_basis_point(p, xi, val, grad, hess);
  else
    ref_basis_point(shape == kQuad ? 2 : 3, p, xi, val, grad, hess);
}

RefTensors make_ref_tensors(int dim, int p, int shape) {
  RefTensors T;
  T.dim = dim;
  T.shape = shape;
  T.order = p;
  T.nloc = n_local_dofs(shape, p);
  T.n_sym = dim == 2 ? 3 : 6;
  const int nl = T.nloc, ns = T.n_sym;
  T.offC = ns;
  T.offM = ns + dim;
  T.offL = ns + dim + 1;
  T.offD = T.offL + dim * dim;
  T.offT = T.offD + dim;
  T.nterms = T.offT + ns * dim;
  T.R.assign((size_t)T.nterms * nl * nl, 0.0);
  // every integrand is a polynomial of degree <= 5 per direction (Q2: 4 + the
  // linear factor of L); these rules integrate all of them exactly, like the
  // reference's rules do for the terms it assembles
  std::vector<double> pts, wts;
  shape_rule(shape, shape == kTetra ? 5 : 4, pts, wts);
  int pa[6], pb[6];
  {
    int k = 0;
    for (int a = 0; a < dim; ++a)
      for (int b = a; b < dim; ++b) { pa[k] = a; pb[k] = b; ++k; }
  }
  std::vector<double> val(nl), grad(3 * nl), hess(6 * nl);
  const size_t NE = (size_t)nl * nl;
  for (size_t q = 0; q < wts.size(); ++q) {
    const double* xi = &pts[3 * q];
    const double wq = wts[q];
    basis_at(shape, p, xi, val.data(), grad.data(), hess.data());
    for (int i = 0; i < nl; ++i)
      for (int j = 0; j < nl; ++j) {
        const size_t ij = (size_t)i * nl + j;
        for (int s2 = 0; s2 < ns; ++s2) {
          const int a = pa[s2], b = pb[s2];
          double v = grad[a * nl + i] * grad[b * nl + j];
          if (a != b) v += grad[b * nl + i] * grad[a * nl + j];
          T.R[(size_t)s2 * NE + ij] += wq * v;
        }
        for (int a = 0; a < dim; ++a) {
          T.R[(size_t)(T.offC + a) * NE + ij] += wq * val[i] * grad[a * nl + j];
          T.R[(size_t)(T.offD + a) * NE + ij] += wq * grad[a * nl + i] * val[j];
          for (int c = 0; c < dim; ++c)
            T.R[(size_t)(T.offL + a * dim + c) * NE + ij] += wq * val[i] * xi[c] * grad[a * nl + j];
        }
        T.R[(size_t)T.offM * NE + ij] += wq * val[i] * val[j];
        for (int s2 = 0; s2 < ns; ++s2)
          for (int c = 0; c < dim; ++c)
            T.R[(size_t)(T.offT + s2 * dim + c) * NE + ij] +=
                wq * grad[c * nl + i] * hess[s2 * nl + j];
      }
  }
  return T;
}

RefTables make_ref_tables(int dim, int p, int nqp1, int shape) {
  RefTables t;
  t.dim = dim;
  t.order = p;
  t.nloc = n_local_dofs(shape, p);
  t.nqp1 = nqp1;
  std::vector<double> pts, wts;
  shape_rule(shape, nqp1, pts, wts);
  t.nqp = (int)wts.size();
  t.xi = pts;
  t.w = wts;
  t.val.resize((size_t)t.nqp * t.nloc);
  t.grad.resize((size_t)t.nqp * dim * t.nloc);
  for (int q = 0; q < t.nqp; ++q)
    basis_at(shape, p, &pts[3 * q], &t.val[(size_t)q * t.nloc], &t.grad[(size_t)q * dim * t.nloc],
             nullptr);
  return t;
}

// ---------------------------------------------------------------------------
// mesh: root grid of M^d unit-cube cells (lexicographic) refined nref times
// ---------------------------------------------------------------------------
namespace {
// refined-cell vertices as means of parent vertices (regular refinement of a
// quadrangle / hexahedron), and the child cells' vertex lists
const int kQuadNew[9][4] = {{0}, {1}, {2}, {3}, {0, 1}, {1, 2}, {2, 3}, {3, 0}, {0, 1, 2, 3}};
const int kQuadNewN[9] = {1, 1, 1, 1, 2, 2, 2, 2, 4};
const int kQuadChild[4][4] = {{0, 4, 8, 7}, {1, 5, 8, 4}, {2, 6, 8, 5}, {3, 7, 8, 6}};
const int kHexNew[27][8] = {
    {0}, {1}, {2}, {3}, {4}, {5}, {6}, {7}, {0, 1}, {1, 2}, {2, 3}, {3, 0},
    {0, 1, 2, 3}, {1, 5}, {4, 5}, {0, 4}, {0, 4, 5, 1}, {2, 6}, {5, 6},
    {1, 5, 6, 2}, {3, 7}, {6, 7}, {2, 6, 7, 3}, {7, 4}, {0, 3, 7, 4},
    {4, 7, 6, 5}, {0, 1, 2, 3, 4, 5, 6, 7}};
const int kHexNewN[27] = {1, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 4, 2,
                          2, 2, 4, 2, 2, 4, 2, 2, 4, 2, 4, 4, 8};
const int kHexChild[8][8] = {
    {0, 8, 12, 11, 15, 16, 26, 24}, {1, 9, 12, 8, 13, 19, 26, 16},
    {2, 10, 12, 9, 17, 22, 26, 19}, {3, 11, 12, 10, 20, 24, 26, 22},
    {4, 23, 25, 14, 15, 24, 26, 16}, {5, 14, 25, 18, 13, 16, 26, 19},
    {6, 18, 25, 21, 17, 19, 26, 22}, {7, 21, 25, 23, 20, 22, 26, 24}};
}  // namespace

Mesh make_refined_box(int dim, int roots, int nref) {
  // root cells: roots^dim unit-cube cells in lexicographic order (x fastest),
  // each with the standard vertex order; It_Finest visits root cells in order
  // and the refinement tree of each depth-first
  Mesh m;
  m.dim = dim;
  m.shape = dim == 2 ? kQuad : kHexa;
  m.nv = dim == 2 ? 4 : 8;
  m.ncells = dim == 2 ? roots * roots : roots * roots * roots;
  static const double sq[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
  static const double cu[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                  {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  m.verts.resize((size_t)m.ncells * m.nv * dim);
  for (int c = 0; c < m.ncells; ++c) {
    int ijk[3] = {c % roots, (c / roots) % roots, c / (roots * roots)};
    for (int v = 0; v < m.nv; ++v)
      for (int a = 0; a < dim; ++a) {
        double corner = dim == 2 ? sq[v][a] : cu[v][a];
        m.verts[((size_t)c * m.nv + v) * dim + a] = (ijk[a] + corner) / roots;
      }
  }
  for (int r = 0; r < nref; ++r) {
    int nch = dim == 2 ? 4 : 8, nnew = dim == 2 ? 9 : 27;
    std::vector<double> out((size_t)m.ncells * nch * m.nv * dim);
    for (int c = 0; c < m.ncells; ++c) {
      const double* pv = &m.verts[(size_t)c * m.nv * dim];
      double nv[27][3];
      for (int k = 0; k < nnew; ++k) {
        int n = dim == 2 ? kQuadNewN[k] : kHexNewN[k];
        for (int a = 0; a < dim; ++a) {
          double s = 0;
          for (int q = 0; q < n; ++q) s += pv[(dim == 2 ? kQuadNew[k][q] : kHexNew[k][q]) * dim + a];
          nv[k][a] = s / n;
        }
      }
      for (int ch = 0; ch < nch; ++ch)
        for (int v = 0; v < m.nv; ++v) {
          int id = dim == 2 ? kQuadChild[ch][v] : kHexChild[ch][v];
          for (int a = 0; a < dim; ++a)
            out[(((size_t)c * nch + ch) * m.nv + v) * dim + a] = nv[id][a];
        }
    }
    m.verts.swap(out);
    m.ncells *= nch;
  }
  return m;
}

// Bey's regular refinement of a tetrahedron (x0,x1,x2,x3): the four corner
// tetrahedra and the four of the inner octahedron split along x02-x13; with a
// Kuhn-ordered parent every child is a Kuhn tetrahedron of the halved grid
static const int kTetChild[8][4][2] = {
    {{0, 0}, {0, 1}, {0, 2}, {0, 3}}, {{0, 1}, {1, 1}, {1, 2}, {1, 3}},
    {{0, 2}, {1, 2}, {2, 2}, {2, 3}}, {{0, 3}, {1, 3}, {2, 3}, {3, 3}},
    {{0, 1}, {0, 2}, {0, 3}, {1, 3}}, {{0, 1}, {0, 2}, {1, 2}, {1, 3}},
    {{0, 2}, {0, 3}, {1, 3}, {2, 3}}, {{0, 2}, {1, 2}, {1, 3}, {2, 3}}};

Mesh make_kuhn_box(int roots, int nref) {
  Mesh m;
  m.dim = 3;
  m.shape = kTetra;
  m.nv = 4;
  // six tetrahedra per cube, one per permutation of the axes (lexicographic)
  static const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  const int ncube = roots * roots * roots;
  m.ncells = 6 * ncube;
  m.verts.resize((size_t)m.ncells * 12);
  for (int c = 0; c < ncube; ++c) {
    const int ijk[3] = {c % roots, (c / roots) % roots, c / (roots * roots)};
    for (int t = 0; t < 6; ++t) {
      int pt[3] = {ijk[0], ijk[1], ijk[2]};
      double* cv = &m.verts[((size_t)c * 6 + t) * 12];
      for (int a = 0; a < 3; ++a) cv[a] = (double)pt[a] / roots;
      for (int s = 0; s < 3; ++s) {
        pt[perm[t][s]] += 1;
        for (int a = 0; a < 3; ++a) cv[(s + 1) * 3 + a] = (double)pt[a] / roots;
      }
    }
  }
  for (int r = 0; r < nref; ++r) {
    std::vector<double> out((size_t)m.ncells * 8 * 12);
    for (int c = 0; c < m.ncells; ++c) {
      const double* pv = &m.verts[(size_t)c * 12];
      for (int ch = 0; ch < 8; ++ch)
        for (int v = 0; v < 4; ++v)
          for (int a = 0; a < 3; ++a)
            out[(((size_t)c * 8 + ch) * 4 + v) * 3 + a] =
                0.5 * (pv[kTetChild[ch][v][0] * 3 + a] + pv[kTetChild[ch][v][1] * 3 + a]);
    }
    m.verts.swap(out);
    m.ncells *= 8;
  }
  return m;
}

static inline unsigned long long mix64(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

void perturb_interior(Mesh& m, double h, double amplitude, unsigned long long seed) {
  const int dim = m.dim;
  const long res = std::lround(1.0 / h);
  const size_t nvt = (size_t)m.ncells * m.nv;
  for (size_t v = 0; v < nvt; ++v) {
    double* x = &m.verts[v * dim];
    bool boundary = false;
    long key = 0;
    for (int a = dim - 1; a >= 0; --a) {
      const long ia = std::lround(x[a] * res);
      if (ia == 0 || ia == res) boundary = true;
      key = key * (res + 1) + ia;
    }
    if (boundary) continue;
    for (int a = 0; a < dim; ++a) {
      const unsigned long long r = mix64(mix64((unsigned long long)key * 3 + a) ^ seed);
      const double u = (double)(r >> 11) * (1.0 / 9007199254740992.0);   // [0,1)
      x[a] += amplitude * h * (2.0 * u - 1.0);
    }
  }
}

// ---------------------------------------------------------------------------
// DOF numbering
// ---------------------------------------------------------------------------
int boundary_component(int dim, const double* x) {
  const double t = 1e-12;
  if (dim == 2) {
    if (std::fabs(x[1]) < t) return 0;
    if (std::fabs(x[0] - 1) < t) return 1;
    if (std::fabs(x[1] - 1) < t) return 2;
    if (std::fabs(x[0]) < t) return 3;
    return -1;
  }
  if (std::fabs(x[2]) < t) return 0;
  if (std::fabs(x[1]) < t) return 1;
  if (std::fabs(x[0] - 1) < t) return 2;
  if (std::fabs(x[1] - 1) < t) return 3;
  if (std::fabs(x[0]) < t) return 4;
  if (std::fabs(x[2] - 1) < t) return 5;
  return -1;
}

Space make_space(const Mesh& m, int p, int neumann_mask) {
  Space s;
  s.dim = m.dim;
  s.shape = m.shape;
  s.order = p;
  s.nloc = n_local_dofs(m.shape, p);
  const int dim = m.dim, nl = s.nloc;
  // lattice resolution from the first cell's first edge (axis-aligned length h
  // for all meshes built here); DOFs sit on multiples of h/p
  double h = 0;
  for (int a = 0; a < dim; ++a) h += std::fabs(m.verts[dim + a] - m.verts[a]);
  const long nres = std::lround(p / h);
  const long n1l = nres + 1;
  const size_t nkeys = dim == 2 ? (size_t)n1l * n1l : (size_t)n1l * n1l * n1l;
  // class per lattice point: 0 inner, 1 non-Dirichlet boundary, 2 Dirichlet
  std::vector<long> keys((size_t)m.ncells * nl);
  std::vector<signed char> cls((size_t)m.ncells * nl);
  for (int c = 0; c < m.ncells; ++c) {
    const double* cv = &m.verts[(size_t)c * m.nv * dim];
    for (int k = 0; k < nl; ++k) {
      double r[3], x[3];
      local_dof_ref_shape(m.shape, p, k, r);
      cell_point(m.shape, dim, cv, r, x);
      long key = 0;
      for (int a = dim - 1; a >= 0; --a) key = key * n1l + std::lround(x[a] * nres);
      keys[(size_t)c * nl + k] = key;
      int cl = 0;
      const double t = 1e-12;
      for (int a = 0; a < dim; ++a)
        for (int side = 0; side < 2; ++side) {
          if (std::fabs(x[a] - side) >= t) continue;
          double probe[3] = {0.5, 0.5, 0.5};
          probe[a] = side;
          const int comp = boundary_component(dim, probe);
          const int t_ = ((neumann_mask >> comp) & 1) ? 1 : 2;
          cl = std::max(cl, t_);
        }
      cls[(size_t)c * nl + k] = (signed char)cl;
    }
  }
  // number representatives by class, in order of first appearance
  std::vector<int> id(nkeys, -1);
  std::vector<signed char> cls_of_key(nkeys, 0);
  int count[3] = {0, 0, 0};
  for (size_t i = 0; i < keys.size(); ++i) {
    const long key = keys[i];
    if (id[key] < 0) {
      id[key] = count[cls[i]]++;
      cls_of_key[key] = cls[i];
    }
  }
  const int off[3] = {0, count[0], count[0] + count[1]};
  s.gdof.resize(keys.size());
  for (size_t i = 0; i < keys.size(); ++i) s.gdof[i] = off[cls_of_key[keys[i]]] + id[keys[i]];
  s.nactive = count[0] + count[1];
  s.ndof = s.nactive + count[2];
  return s;
}

Pattern make_pattern(const Space& s) {
  Pattern P;
  int n = s.ndof, nl = s.nloc;
  int ncells = (int)(s.gdof.size() / nl);
  std::vector<int> cnt(n + 1, 0);
  for (int c = 0; c < ncells; ++c)
    for (int m = 0; m < nl; ++m) cnt[s.gdof[(size_t)c * nl + m] + 1] += nl;
  for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
  std::vector<int> tmp(cnt[n]), fill(n, 0);
  for (int c = 0; c < ncells; ++c)
    for (int m = 0; m < nl; ++m) {
      int r = s.gdof[(size_t)c * nl + m];
      for (int k = 0; k < nl; ++k) tmp[cnt[r] + fill[r]++] = s.gdof[(size_t)c * nl + k];
    }
  P.nrows = n;
  P.row_ptr.assign(n + 1, 0);
  P.col.reserve(cnt[n] / 2);
  for (int r = 0; r < n; ++r) {
    int* b = tmp.data() + cnt[r];
    std::sort(b, b + fill[r]);
    int* e = std::unique(b, b + fill[r]);
    P.col.insert(P.col.end(), b, e);
    P.row_ptr[r + 1] = (int)P.col.size();
  }
  return P;
}

// ---------------------------------------------------------------------------
// grid transfer (fine <- coarse), parent[f] = coarse cell of fine cell f
// ---------------------------------------------------------------------------
void make_transfer(const Mesh& fm, const Space& fs, const Mesh& cm, const Space& cs,
                   const int* parent, HostCsr* P, HostCsr* R) {
  const int dim = fm.dim, nl = fs.nloc, p = fs.order, shape = fm.shape;
  // child-local interpolation: fine dof k of cell f gets coarse basis l of
  // parent evaluated at the fine node (nodal functionals are point values);
  // the fine node is located in the parent's reference cell through the
  // (unperturbed) geometry
  std::vector<std::unordered_map<int, double>> rows(fs.ndof);
  std::vector<int> mult(fs.ndof, 0);
  std::vector<double> val(nl);
  for (int f = 0; f < fm.ncells; ++f) {
    const int c = parent[f];
    const double* cvf = &fm.verts[(size_t)f * fm.nv * dim];
    const double* cvc = &cm.verts[(size_t)c * cm.nv * dim];
    // coarse affine map x = x0 + J r and its inverse
    double J[3][3], Ji[3][3], x0[3], zero[3] = {0, 0, 0}, unit[3];
    if (shape == kTetra) {
      cell_point(shape, dim, cvc, zero, x0);
    } else {
      const double m1[3] = {-1, -1, -1};
      cell_point(shape, dim, cvc, m1, x0);   // vertex 0 at r = (-1,-1,-1)
    }
    for (int a = 0; a < dim; ++a) {
      for (int b = 0; b < 3; ++b) unit[b] = shape == kTetra ? 0.0 : -1.0;
      unit[a] = 1.0;
      double xa[3];
      cell_point(shape, dim, cvc, unit, xa);
      for (int r = 0; r < dim; ++r) J[r][a] = (xa[r] - x0[r]) / (shape == kTetra ? 1.0 : 2.0);
    }
    if (dim == 2) {
      const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
      Ji[0][0] = J[1][1] / det; Ji[0][1] = -J[0][1] / det;
      Ji[1][0] = -J[1][0] / det; Ji[1][1] = J[0][0] / det;
    } else {
      const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          const int i1 = (j + 1) % 3, i2 = (j + 2) % 3, j1 = (i + 1) % 3, j2 = (i + 2) % 3;
          Ji[i][j] = (J[i1][j1] * J[i2][j2] - J[i1][j2] * J[i2][j1]) / det;
        }
    }
    const double r0 = shape == kTetra ? 0.0 : -1.0;
    for (int k = 0; k < nl; ++k) {
      double r[3], x[3], xi[3] = {0, 0, 0};
      local_dof_ref_shape(shape, p, k, r);
      cell_point(shape, dim, cvf, r, x);
      for (int a = 0; a < dim; ++a) {
        double t = 0;
        for (int rr = 0; rr < dim; ++rr) t += Ji[a][rr] * (x[rr] - x0[rr]);
        xi[a] = r0 + t;
      }
      basis_at(shape, p, xi, val.data(), nullptr, nullptr);
      const int fi = fs.gdof[(size_t)f * nl + k];
      mult[fi] += 1;
      for (int l = 0; l < nl; ++l) {
        if (std::fabs(val[l]) < 1e-14) continue;
        rows[fi][cs.gdof[(size_t)c * nl + l]] += val[l];
      }
    }
  }
  // averaged prolongation (all fine rows) and its transpose (all coarse
  // rows); the multigrid masks non-active rows in the transfer kernels
  P->nrows = fs.ndof;
  P->ncols = cs.ndof;
  P->row_ptr.assign(fs.ndof + 1, 0);
  P->col.clear();
  P->val.clear();
  std::vector<std::vector<std::pair<int, double>>> Rrows(cs.ndof);
  for (int i = 0; i < fs.ndof; ++i) {
    std::vector<std::pair<int, double>> e(rows[i].begin(), rows[i].end());
    std::sort(e.begin(), e.end());
    for (auto& kv : e) {
      double v = kv.second / mult[i];
      P->col.push_back(kv.first);
      P->val.push_back(v);
      Rrows[kv.first].push_back({i, v});
    }
    P->row_ptr[i + 1] = (int)P->col.size();
  }
  R->nrows = cs.ndof;
  R->ncols = fs.ndof;
  R->row_ptr.assign(cs.ndof + 1, 0);
  R->col.clear();
  R->val.clear();
  for (int j = 0; j < cs.ndof; ++j) {
    for (auto& kv : Rrows[j]) {
      R->col.push_back(kv.first);
      R->val.push_back(kv.second);
    }
    R->row_ptr[j + 1] = (int)R->col.size();
  }
}

}  // namespace cdg
