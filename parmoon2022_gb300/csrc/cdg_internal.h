// cdg_internal.h -- host-side data structures shared by the C++ setup layer,
// the CUDA kernels and the C-ABI implementation.  Not part of the public ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace cdg {

constexpr int kMaxLoc = 27;    // Q2 hexahedron
constexpr int kMaxQp1 = 10;    // 1D Gauss points
constexpr int kMaxTerms = 40;  // reference tensors of one element type

// cell shapes
enum Shape : int { kQuad = 0, kHexa = 1, kTetra = 2 };
inline int shape_of(int dim, bool tetra) { return tetra ? kTetra : (dim == 2 ? kQuad : kHexa); }
inline int n_vertices(int shape) { return shape == kHexa ? 8 : 4; }
inline int n_local_dofs(int shape, int order) {
  if (shape == kTetra) return order == 1 ? 4 : 10;
  int n1 = order + 1;
  return shape == kQuad ? n1 * n1 : n1 * n1 * n1;
}

// ---------------------------------------------------------------------------
// mesh hierarchy (the reference's TDomain/TCollection as plain arrays)
// ---------------------------------------------------------------------------
struct Mesh {
  int dim = 2;
  int shape = kQuad;
  int nv = 4;          // vertices per cell
  int ncells = 0;
  std::vector<double> verts;   // ncells * nv * dim, cell-local vertex order
};

// FE space: the reference's TFESpace (GlobalNumbers with uniform BeginIndex)
struct Space {
  int dim = 2, shape = kQuad, order = 1, nloc = 4;
  int ndof = 0, nactive = 0;
  std::vector<int> gdof;       // ncells * nloc
};

// TStructure: CSR pattern, full rows, sorted columns
struct Pattern {
  int nrows = 0;
  std::vector<int> row_ptr, col;
};

// CSR matrix on the host (prolongation / restriction)
struct HostCsr {
  int nrows = 0, ncols = 0;
  std::vector<int> row_ptr, col;
  std::vector<double> val;
};

// ---------------------------------------------------------------------------
// quadrature and reference element data
// ---------------------------------------------------------------------------
void gauss_legendre(int n, double* x, double* w);
int gauss_points_for_degree(int degree);   // quad/hexa accuracy -> points/dir

// Reference tensors of one element type, used by the element-matrix
// contraction A_ij = sum_t g_t(cell) R_t[i][j].  Term blocks in order:
//   S^{ab}  (ns = d(d+1)/2) symmetric gradient pairs d_a phi_i d_b phi_j (+ba)
//   C^a     (d)    phi_i d_a phi_j                 (convection)
//   M       (1)    phi_i phi_j                     (reaction, mass)
//   L^{a,c} (d*d)  phi_i xi_c d_a phi_j            (convection linear in x)
//   D^a     (d)    d_a phi_i phi_j                 (SUPG reaction)
//   T^{(ab),c} (ns*d) d_c phi_i d_ab phi_j         (SUPG diffusion)
struct RefTensors {
  int dim = 2, shape = kQuad, order = 1, nloc = 4, nterms = 0;
  int n_sym = 3;                  // symmetric derivative pairs
  int offC = 0, offM = 0, offL = 0, offD = 0, offT = 0;
  std::vector<double> R;          // nterms * nloc * nloc
};
RefTensors make_ref_tensors(int dim, int order, int shape);

// values / gradients / Hessians of the reference basis at quadrature points
struct RefTables {
  int dim = 2, order = 1, nloc = 4, nqp = 0, nqp1 = 0;
  std::vector<double> xi;   // nqp * 3
  std::vector<double> w;    // nqp
  std::vector<double> val;  // nqp * nloc   phi
  std::vector<double> grad; // nqp * dim * nloc  d_a phi
};
RefTables make_ref_tables(int dim, int order, int nqp1, int shape);
// the reference tetrahedron's quadrature rule for `degree` (above kTetraRule:
// the reference's Keast rule, kTetraRule + its degree; else points per
// direction of a collapsed Gauss rule)
constexpr int kTetraRule = 100;
int tetra_points_for_degree(int degree);
int tetra_rule_size(int code);   // points of that rule

void ref_basis_point(int dim, int order, const double* xi, double* val,
                     double* grad /* dim*nloc */, double* hess /* sym */);
void tetra_basis_point(int order, const double* xi, double* val, double* grad, double* hess);
void local_dof_ref(int dim, int order, int k, double* r);
void local_dof_ref_shape(int shape, int order, int k, double* r);
// x = affine map of the cell (QuadAffin / HexaAffin / TetraAffin) at r
void cell_point(int shape, int dim, const double* cv, const double* r, double* x);
void cell_point_multilinear(int dim, const double* cv, const double* r, double* x);

// ---------------------------------------------------------------------------
// setup: structured meshes, DOF numbering, pattern, grid transfer
// ---------------------------------------------------------------------------
// unit square / cube split into roots^dim cells, each refined nref times;
// children in depth-first order, so parent(fine cell f) = f / 2^dim
Mesh make_refined_box(int dim, int roots, int nref);
// unit cube split into roots^3 cubes of 6 Kuhn tetrahedra each (permutation
// order), refined nref times by Bey's red refinement (children stay Kuhn
// tetrahedra, parent(fine cell f) = f / 8)
Mesh make_kuhn_box(int roots, int nref);
// move every vertex off the boundary by amplitude*h*U(-1,1) per coordinate,
// the same displacement for every cell sharing the vertex (seeded)
void perturb_interior(Mesh& m, double h, double amplitude, unsigned long long seed);
// DOF numbering: inner, then non-Dirichlet boundary, then Dirichlet; each
// class numbered in order of first appearance over (cell, local dof)
Space make_space(const Mesh& m, int order, int neumann_mask);
Pattern make_pattern(const Space& s);
// prolongation fine <- coarse (child-local interpolation averaged by DOF
// multiplicity) and restriction coarse <- fine (its transpose)
void make_transfer(const Mesh& fine_mesh, const Space& fine, const Mesh& coarse_mesh,
                   const Space& coarse, const int* parent, HostCsr* P, HostCsr* R);

int boundary_component(int dim, const double* x);   // -1 inside

}  // namespace cdg
