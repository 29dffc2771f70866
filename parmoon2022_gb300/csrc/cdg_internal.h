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
constexpr int kMaxTerms = 32;  // reference tensors of one element type

// ---------------------------------------------------------------------------
// mesh hierarchy (the reference's TDomain/TCollection as plain arrays)
// ---------------------------------------------------------------------------
struct Mesh {
  int dim = 2;
  int nv = 4;          // vertices per cell
  int ncells = 0;
  std::vector<double> verts;   // ncells * nv * dim, cell-local vertex order
};

// FE space: the reference's TFESpace (GlobalNumbers with uniform BeginIndex)
struct Space {
  int dim = 2, order = 1, nloc = 4;
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

// Reference tensors of one (dim, order) element, used by the element-matrix
// contraction A_ij = sum_t g_t(cell) R_t[i][j].  Term layout (2D sizes in
// brackets): [0..5]  (3) S^{ab}: sym. gradient-gradient pairs
//            [6..8]  (2) C^a:  phi_i d_a phi_j          (convection)
//            [9]     (1) M:    phi_i phi_j              (reaction)
//            [10..12](2) D^a:  d_a phi_i phi_j          (SUPG reaction)
//            [13..30](6) T^{(ab),c}: d_c phi_i d_ab phi_j (SUPG diffusion)
struct RefTensors {
  int dim = 2, order = 1, nloc = 4, nterms = 0;
  int n_sym = 3;                  // symmetric derivative pairs
  std::vector<double> R;          // nterms * nloc * nloc
};
RefTensors make_ref_tensors(int dim, int order);

// values / gradients / Hessians of the reference basis at quadrature points
struct RefTables {
  int dim = 2, order = 1, nloc = 4, nqp = 0, nqp1 = 0;
  std::vector<double> xi;   // nqp * 3
  std::vector<double> w;    // nqp
  std::vector<double> val;  // nqp * nloc   phi
  std::vector<double> grad; // nqp * dim * nloc  d_a phi
};
RefTables make_ref_tables(int dim, int order, int nqp1);

void ref_basis_point(int dim, int order, const double* xi, double* val,
                     double* grad /* dim*nloc */, double* hess /* sym */);
void local_dof_ref(int dim, int order, int k, double* r);

// ---------------------------------------------------------------------------
// setup: structured meshes, DOF numbering, pattern, grid transfer
// ---------------------------------------------------------------------------
// unit square / cube split into roots^dim cells, each refined nref times;
// children in depth-first order, so parent(fine cell f) = f / 2^dim
Mesh make_refined_box(int dim, int roots, int nref);
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
