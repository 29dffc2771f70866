// assemble.cu -- GB300 kernels of the CD assembly: cell geometry, element
// matrices by contraction with reference tensors, CSR scatter through a
// precomputed coupling->slot map, right-hand side with the example's source
// term, Dirichlet rows and data, error norms, and the Crank-Nicolson pieces of
// the time-dependent problem.
//
// Reference path (ParMooN2022): ConvectionDiffusion<d>::call_assembling_
// routine (src/System/ConvectionDiffusion.C:410-452) -> Assemble2D/3D cell
// loop (src/AssembleRoutines/Assemble2D.C:2798-3481, Assemble3D.C:39-917) ->
// FEDatabase::GetOrig (src/FE/FEDatabase.C:1498-1719) -> LocalAssembling::
// GetLocalForms (src/AssembleRoutines/LocalAssembling.C:734-970) ->
// BilinearAssembleGalerkin<d> / BilinearAssemble_SD<d>
// (src/AssembleRoutines/ConvDiff.C:1776-1999), TCDStiff / TCDMass / TCDRhs
// (src/AssembleRoutines/CD_local_assembling_routines.C:9-181) -> scatter by
// row search (Assemble3D.C:257-292, Matrix.C:180-255); time discretisation
// src/TimeDiscRoutines/TimeDiscretizations.C:117-283.
//
// On affine cells (QuadAffin / HexaAffin / TetraAffin, the maps of every cell
// these meshes produce) with cell-constant eps, c and a convection field that
// is constant or linear in x, the per-quadrature-point local forms are
// bilinear in reference-element integrals.  The local matrix is therefore
// A_ij = sum_t g_t(cell) R_t[i][j] with R_t exact reference integrals (the
// reference's Gauss rules integrate these polynomials exactly) and g_t a few
// FP64 geometric/coefficient factors per cell; the quadrature sum of the
// reference becomes one FP64 contraction per entry.  The right-hand side
// keeps a quadrature rule of the reference's degree because f is not
// polynomial.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <mutex>

#include "common.cuh"

namespace cdg {

// ---------------------------------------------------------------------------
// device-side problem data
// ---------------------------------------------------------------------------
struct AsmCoefs {
  int dim, shape, order, nloc, example, supg, sdfem_type, cell_measure, poly_degree,
      neumann_mask, nqp, nqp1, n_sym, linear_b;
  double eps, b[3], bg[9], c, freq, delta0, delta1, t, ic[4];
  int tcd;        // time-dependent assembly (SUPG parameter of the TCD routines)
  double ttau;    // theta1 * time step (Crank-Nicolson: theta1 = 1/2)
  double tau, theta1;   // CURRENTTIMESTEPLENGTH and THETA1 (SDFEM types 9-11)
};

static AsmCoefs make_coefs(const cdg_assembly_params& a, int shape, int order) {
  AsmCoefs k;
  k.shape = shape;
  k.dim = shape == kQuad ? 2 : 3;
  k.order = order;
  k.nloc = n_local_dofs(shape, order);
  k.example = a.example;
  k.supg = a.supg;
  k.tcd = 0;
  k.ttau = 0.0;
  k.tau = 0.0;
  k.theta1 = 0.0;
  k.sdfem_type = a.sdfem_type;
  k.cell_measure = a.cell_measure;
  k.poly_degree = a.poly_degree > 0 ? a.poly_degree : order;
  k.neumann_mask = a.neumann_mask;
  k.eps = a.eps;
  k.linear_b = 0;
  for (int i = 0; i < 3; ++i) k.b[i] = (i < k.dim) ? a.b[i] : 0.0;
  for (int i = 0; i < 9; ++i) {
    const int r = i / 3, c = i % 3;
    k.bg[i] = (r < k.dim && c < k.dim) ? a.b_grad[i] : 0.0;
    if (k.bg[i] != 0.0) k.linear_b = 1;
  }
  k.c = a.c;
  k.freq = a.freq;
  k.delta0 = a.delta0;
  k.delta1 = a.delta1;
  k.t = a.t;
  for (int i = 0; i < 4; ++i) k.ic[i] = a.ic[i];
  const int nterms = a.problem_linear ? 2 : 3;
  const int deg = nterms * order;
  if (shape == kTetra) {
    k.nqp1 = tetra_points_for_degree(deg);   // the reference's rule by degree
    k.nqp = tetra_rule_size(k.nqp1);
  } else {
    k.nqp1 = gauss_points_for_degree(deg);
    k.nqp = k.dim == 2 ? k.nqp1 * k.nqp1 : k.nqp1 * k.nqp1 * k.nqp1;
  }
  k.n_sym = k.dim == 2 ? 3 : 6;
  return k;
}

// convection at x
__device__ __forceinline__ void b_at(const AsmCoefs& k, const double* x, double* bx) {
  for (int i = 0; i < 3; ++i) {
    double s = k.b[i];
    if (k.linear_b)
      for (int j = 0; j < k.dim; ++j) s += k.bg[3 * i + j] * x[j];
    bx[i] = s;
  }
}

// exact solution of the example: u[0] value, u[1..dim] gradient, u[dim+1]
// Laplacian, u[dim+2] time derivative (examples with a known solution;
// CONST_F and BUMP return zeros)
__device__ void ex_exact(const AsmCoefs& k, const double* x, double* u) {
  int d = k.dim;
  for (int i = 0; i < 6; ++i) u[i] = 0.0;
  if (k.example == CDG_EX_SINE_LAPLACE || k.example == CDG_EX_SINE) {
    double w = (k.example == CDG_EX_SINE_LAPLACE ? 1.0 : k.freq) * M_PI;
    double s0 = sin(w * x[0]), c0 = cos(w * x[0]);
    double s1 = sin(w * x[1]), c1 = cos(w * x[1]);
    if (d == 2) {
      u[0] = s0 * s1;
      u[1] = w * c0 * s1;
      u[2] = w * s0 * c1;
      u[3] = -2.0 * w * w * s0 * s1;
    } else {
      double s2 = sin(w * x[2]), c2 = cos(w * x[2]);
      u[0] = s0 * s1 * s2;
      u[1] = w * c0 * s1 * s2;
      u[2] = w * s0 * c1 * s2;
      u[3] = w * s0 * s1 * c2;
      u[4] = -3.0 * w * w * s0 * s1 * s2;
    }
  } else if (k.example == CDG_EX_POLYEXP) {
    double e = exp(x[0]);
    double px = x[0] * (1 - x[0]) * e;
    double px1 = e * (1 - x[0] - x[0] * x[0]);
    double px2 = -e * x[0] * (3 + x[0]);
    double qy = x[1] * (1 - x[1]), qz = x[2] * (1 - x[2]);
    u[0] = px * qy * qz;
    u[1] = px1 * qy * qz;
    u[2] = px * (1 - 2 * x[1]) * qz;
    u[3] = px * qy * (1 - 2 * x[2]);
    u[4] = px2 * qy * qz - 2 * px * qz - 2 * px * qy;
  } else if (k.example == CDG_EX_EXP_SIN) {
    // e^{sin 2 pi t} prod sin(2 pi x_a) (include/Examples/TCD_2D/exp.h)
    const double w = 2.0 * M_PI, e = exp(sin(w * k.t));
    double sn[3], cs[3];
    for (int a = 0; a < d; ++a) {
      sn[a] = sin(w * x[a]);
      cs[a] = cos(w * x[a]);
    }
    const double pr = d == 2 ? sn[0] * sn[1] : sn[0] * sn[1] * sn[2];
    u[0] = e * pr;
    u[1] = e * w * cs[0] * sn[1] * (d == 3 ? sn[2] : 1.0);
    u[2] = e * w * sn[0] * cs[1] * (d == 3 ? sn[2] : 1.0);
    if (d == 3) u[3] = e * w * sn[0] * sn[1] * cs[2];
    u[d + 1] = -d * w * w * e * pr;
    u[d + 2] = w * cos(w * k.t) * e * pr;
  } else if (k.example == CDG_EX_LINEAR_ST) {
    // 1 + 2x + 3ty (+ 4tz) (include/Examples/TCD_3D/linear_space_time.h)
    const double z = d == 3 ? x[2] : 0.0;
    u[0] = 1 + 2 * x[0] + 3 * k.t * x[1] + 4 * k.t * z;
    u[1] = 2;
    u[2] = 3 * k.t;
    if (d == 3) u[3] = 4 * k.t;
    u[d + 2] = 3 * x[1] + 4 * z;
  } else if (k.example == CDG_EX_QUAD_ST) {
    // t^2 (x^2 + yz) (include/Examples/TCD_3D/quadratic_space_time.h)
    const double z = d == 3 ? x[2] : 0.0, t2 = k.t * k.t;
    const double q = x[0] * x[0] + x[1] * z;
    u[0] = t2 * q;
    u[1] = 2 * x[0] * t2;
    u[2] = z * t2;
    if (d == 3) u[3] = x[1] * t2;
    u[d + 1] = 2 * t2;
    u[d + 2] = 2 * k.t * q;
  } else if (k.example == CDG_EX_POLY1 || k.example == CDG_EX_POLY1_T) {
    const double s = k.example == CDG_EX_POLY1_T ? 1.0 + k.t : 1.0;
    const double q = 1 + x[0] + 2 * x[1] + (d == 3 ? 3 * x[2] : 0.0);
    u[0] = s * q;
    u[1] = s;
    u[2] = 2 * s;
    if (d == 3) u[3] = 3 * s;
    if (k.example == CDG_EX_POLY1_T) u[d + 2] = q;
  }
}

// source term f = u_t - eps lap u + b.grad u + c u (the examples' coefficient
// callbacks, e.g. include/Examples/CD_2D/SineLaplace.h BilinearCoeffs)
__device__ double ex_source(const AsmCoefs& k, const double* x) {
  if (k.example == CDG_EX_CONST_F) return 1.0;
  if (k.example == CDG_EX_BUMP) return 0.0;
  double u[6], bx[3];
  ex_exact(k, x, u);
  b_at(k, x, bx);
  int d = k.dim;
  double f = -k.eps * u[d + 1];
  for (int a = 0; a < d; ++a) f += bx[a] * u[1 + a];
  f += k.c * u[0];
  f += u[d + 2];
  return f;
}

// initial condition (interpolated at the nodes) and boundary data
__device__ double ex_initial(const AsmCoefs& k, const double* x) {
  if (k.example == CDG_EX_BUMP) {
    double r2 = 0;
    for (int a = 0; a < k.dim; ++a) r2 += (x[a] - k.ic[a]) * (x[a] - k.ic[a]);
    return exp(-r2 / (2.0 * k.ic[3] * k.ic[3]));
  }
  double u[6];
  ex_exact(k, x, u);
  return u[0];
}

// affine reference map from the cell vertices: x = x0 + J xi
// QuadAffin.C:175- / HexaAffin.C:221-252 (xi in [-1,1]^d along v0->v1,
// v0->v3, v0->v4; x0 the centre) and TetraAffin.C:235-265 (xi in the unit
// tetrahedron, columns v1-v0, v2-v0, v3-v0; x0 = v0)
struct Affine {
  double x0[3], J[3][3], Ji[3][3], det;
};

__device__ void invert_J(int dim, Affine& A) {
  if (dim == 2) {
    double det = A.J[0][0] * A.J[1][1] - A.J[0][1] * A.J[1][0];
    A.det = det;
    A.Ji[0][0] = A.J[1][1] / det;
    A.Ji[0][1] = -A.J[0][1] / det;
    A.Ji[1][0] = -A.J[1][0] / det;
    A.Ji[1][1] = A.J[0][0] / det;
  } else {
    double det = A.J[0][0] * (A.J[1][1] * A.J[2][2] - A.J[1][2] * A.J[2][1]) -
                 A.J[0][1] * (A.J[1][0] * A.J[2][2] - A.J[1][2] * A.J[2][0]) +
                 A.J[0][2] * (A.J[1][0] * A.J[2][1] - A.J[1][1] * A.J[2][0]);
    A.det = det;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        int j1 = (j + 1) % 3, j2 = (j + 2) % 3, i1 = (i + 1) % 3, i2 = (i + 2) % 3;
        A.Ji[i][j] = (A.J[j1][i1] * A.J[j2][i2] - A.J[j1][i2] * A.J[j2][i1]) / det;
      }
  }
}

// x0, J and det only (no inverse): what the Galerkin rhs needs
__device__ void cell_geom_s(int shape, int dim, const double* __restrict__ cv, Affine& A) {
  if (shape == kTetra) {
    for (int r = 0; r < 3; ++r) {
      A.x0[r] = cv[r];
      for (int a = 0; a < 3; ++a) A.J[r][a] = cv[(a + 1) * 3 + r] - cv[r];
    }
  } else {
    const int e[3] = {1, 3, 4};
    for (int r = 0; r < dim; ++r)
      for (int a = 0; a < dim; ++a) A.J[r][a] = (cv[e[a] * dim + r] - cv[r]) * 0.5;
    for (int r = 0; r < dim; ++r) {
      double s = cv[r];
      for (int a = 0; a < dim; ++a) s += A.J[r][a];
      A.x0[r] = s;
    }
  }
  if (dim == 2)
    A.det = A.J[0][0] * A.J[1][1] - A.J[0][1] * A.J[1][0];
  else
    A.det = A.J[0][0] * (A.J[1][1] * A.J[2][2] - A.J[1][2] * A.J[2][1]) -
            A.J[0][1] * (A.J[1][0] * A.J[2][2] - A.J[1][2] * A.J[2][0]) +
            A.J[0][2] * (A.J[1][0] * A.J[2][1] - A.J[1][1] * A.J[2][0]);
}

__device__ void cell_affine_s(int shape, int dim, const double* __restrict__ cv, Affine& A) {
  if (shape == kTetra) {
    for (int r = 0; r < 3; ++r) {
      A.x0[r] = cv[r];
      for (int a = 0; a < 3; ++a) A.J[r][a] = cv[(a + 1) * 3 + r] - cv[r];
    }
  } else {
    const int e[3] = {1, 3, 4};
    for (int r = 0; r < dim; ++r)
      for (int a = 0; a < dim; ++a) A.J[r][a] = (cv[e[a] * dim + r] - cv[r]) * 0.5;
    for (int r = 0; r < dim; ++r) {
      double s = cv[r];
      for (int a = 0; a < dim; ++a) s += A.J[r][a];
      A.x0[r] = s;
    }
  }
  invert_J(dim, A);
}

// Multilinear reference maps of quadrilaterals that are not parallelograms
// and hexahedra that are not parallelepipeds (TQuadBilinear::SetCell,
// QuadBilinear.C:243-263; THexaTrilinear::SetCell, HexaTrilinear.C:225-270):
// x_r(xi) = c0 + c1 xi + c2 eta + c3 xi eta (2D), c0 + c1 xi + c2 eta +
// c3 zeta + c4 xi eta + c5 xi zeta + c6 eta zeta + c7 xi eta zeta (3D), the
// coefficients from the vertices in the reference cells' order
struct MultiMap {
  double c[3][8];
};

__device__ void multilinear_coeffs(int dim, const double* __restrict__ cv, MultiMap& M) {
  if (dim == 2) {
    for (int r = 0; r < 2; ++r) {
      const double v0 = cv[r], v1 = cv[2 + r], v2 = cv[4 + r], v3 = cv[6 + r];
      M.c[r][0] = (v0 + v1 + v2 + v3) * 0.25;
      M.c[r][1] = (-v0 + v1 + v2 - v3) * 0.25;
      M.c[r][2] = (-v0 - v1 + v2 + v3) * 0.25;
      M.c[r][3] = (v0 - v1 + v2 - v3) * 0.25;
    }
    return;
  }
  for (int r = 0; r < 3; ++r) {
    double v[8];
    for (int i = 0; i < 8; ++i) v[i] = cv[3 * i + r];
    M.c[r][0] = (v[0] + v[1] + v[3] + v[2] + v[4] + v[5] + v[7] + v[6]) * 0.125;
    M.c[r][1] = (-v[0] + v[1] - v[3] + v[2] - v[4] + v[5] - v[7] + v[6]) * 0.125;
    M.c[r][2] = (-v[0] - v[1] + v[3] + v[2] - v[4] - v[5] + v[7] + v[6]) * 0.125;
    M.c[r][3] = (-v[0] - v[1] - v[3] - v[2] + v[4] + v[5] + v[7] + v[6]) * 0.125;
    M.c[r][4] = (v[0] - v[1] - v[3] + v[2] + v[4] - v[5] - v[7] + v[6]) * 0.125;
    M.c[r][5] = (v[0] - v[1] + v[3] - v[2] - v[4] + v[5] - v[7] + v[6]) * 0.125;
    M.c[r][6] = (v[0] + v[1] - v[3] - v[2] - v[4] - v[5] + v[7] + v[6]) * 0.125;
    M.c[r][7] = (-v[0] + v[1] + v[3] - v[2] + v[4] - v[5] - v[7] + v[6]) * 0.125;
  }
}

// the map at a reference point: P.x0 = x(xi), P.J = dx/dxi, P.Ji, P.det
// (GetOrigFromRef / GetOrigValues of the two maps)
__device__ void multilinear_at(int dim, const MultiMap& M, const double* xi, Affine& P) {
  if (dim == 2) {
    const double s = xi[0], t = xi[1];
    for (int r = 0; r < 2; ++r) {
      const double* c = M.c[r];
      P.x0[r] = c[0] + c[1] * s + c[2] * t + c[3] * s * t;
      P.J[r][0] = c[1] + c[3] * t;
      P.J[r][1] = c[2] + c[3] * s;
    }
  } else {
    const double s = xi[0], t = xi[1], u = xi[2];
    for (int r = 0; r < 3; ++r) {
      const double* c = M.c[r];
      P.x0[r] = c[0] + c[1] * s + c[2] * t + c[3] * u + c[4] * s * t + c[5] * s * u +
                c[6] * t * u + c[7] * s * t * u;
      P.J[r][0] = c[1] + c[4] * t + c[5] * u + c[7] * t * u;
      P.J[r][1] = c[2] + c[4] * s + c[6] * u + c[7] * s * u;
      P.J[r][2] = c[3] + c[5] * s + c[6] * t + c[7] * s * t;
    }
  }
  invert_J(dim, P);
}

// Laplacian weights of a bilinear quadrilateral at a point
// (TQuadBilinear::GetOrigAllDerivatives, QuadBilinear.C:131-181): with
// G the 5 x 5 matrix taking the physical derivatives (u_x, u_y, u_xx, u_xy,
// u_yy) to the reference ones (u_xi, u_eta, u_xixi, u_xieta, u_etaeta), the
// physical ones are G^-1 times the reference ones, and lap u = (row 2 + row 4
// of G^-1) . (u_xi, u_eta, u_xixi, u_xieta, u_etaeta).  G^-1 by Gaussian
// elimination with partial pivoting (the reference's SolveMultipleSystemsNew
// solves G X = I the same way)
__device__ void bilinear_lap_weights(const MultiMap& M, const double* xi, double* lw) {
  const double s = xi[0], t = xi[1];
  const double xx = M.c[0][1] + M.c[0][3] * t, yx = M.c[1][1] + M.c[1][3] * t;   // d/dxi
  const double xe = M.c[0][2] + M.c[0][3] * s, ye = M.c[1][2] + M.c[1][3] * s;   // d/deta
  double G[5][10];
  const double row[5][5] = {{xx, yx, 0.0, 0.0, 0.0},
                            {xe, ye, 0.0, 0.0, 0.0},
                            {0.0, 0.0, xx * xx, 2.0 * xx * yx, yx * yx},
                            {M.c[0][3], M.c[1][3], xx * xe, yx * xe + xx * ye, yx * ye},
                            {0.0, 0.0, xe * xe, 2.0 * xe * ye, ye * ye}};
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 10; ++j) G[i][j] = j < 5 ? row[i][j] : (j - 5 == i ? 1.0 : 0.0);
  for (int col = 0; col < 5; ++col) {
    int pr = col;
    for (int i = col + 1; i < 5; ++i)
      if (fabs(G[i][col]) > fabs(G[pr][col])) pr = i;
    if (pr != col)
      for (int j = 0; j < 10; ++j) {
        const double tmp = G[col][j];
        G[col][j] = G[pr][j];
        G[pr][j] = tmp;
      }
    const double inv = 1.0 / G[col][col];
    for (int j = 0; j < 10; ++j) G[col][j] *= inv;
    for (int i = 0; i < 5; ++i) {
      if (i == col) continue;
      const double f = G[i][col];
      if (f != 0.0)
        for (int j = 0; j < 10; ++j) G[i][j] -= f * G[col][j];
    }
  }
  for (int k = 0; k < 5; ++k) lw[k] = G[2][5 + k] + G[4][5 + k];
}

// area of a quadrilateral from its two triangles (TQuadrangle::GetMeasure,
// Quadrangle.C:102-117): the cell measure of a bilinear cell
__device__ double quad_measure(const double* __restrict__ cv) {
  const double x1 = cv[0], y1 = cv[1], x2 = cv[2], y2 = cv[3], x3 = cv[4], y3 = cv[5],
               x4 = cv[6], y4 = cv[7];
  return 0.5 * fabs(x2 * y3 - x3 * y2 - x1 * y3 + x3 * y1 + x1 * y2 - x2 * y1) +
         0.5 * fabs(x4 * y3 - x3 * y4 - x1 * y3 + x3 * y1 + x1 * y4 - x4 * y1);
}

// quadrilateral / hexahedron form used by the fixed-scratch error norms
__device__ void cell_affine(int dim, const double* __restrict__ cv, Affine& A) {
  cell_affine_s(dim == 2 ? kQuad : kHexa, dim, cv, A);
}

// cell measure hK (BaseCell.C:102-131; Rectangle.C:12-33; Hexahedron.C:70-121;
// Tetrahedron.C:64-113)
__device__ double cell_hK_s(int shape, int dim, const double* __restrict__ cv, int measure,
                            double det) {
  auto d2 = [&](int i, int j) {
    double s = 0;
    for (int a = 0; a < dim; ++a) {
      double t = cv[i * dim + a] - cv[j * dim + a];
      s += t * t;
    }
    return s;
  };
  if (shape == kTetra) {
    if (measure == 1 || measure == 3) return sqrt(fabs(det) / 6.0);
    double m = d2(0, 1);
    const int pr[5][2] = {{0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
    for (int k = 0; k < 5; ++k)
      m = measure == 2 ? fmin(m, d2(pr[k][0], pr[k][1])) : fmax(m, d2(pr[k][0], pr[k][1]));
    return sqrt(m);
  }
  if (measure == 1 || measure == 3) return sqrt(fabs(det) * (dim == 2 ? 4.0 : 8.0));
  if (dim == 2) {
    if (measure == 2) {
      double l1 = d2(0, 1), l2 = d2(1, 2);
      return l1 < l2 ? sqrt(l1) : sqrt(l2);
    }
    return sqrt(d2(0, 2));
  }
  if (measure == 2) {
    double m = d2(0, 4);
    m = fmin(m, d2(0, 1));
    m = fmin(m, d2(0, 3));
    return sqrt(m);
  }
  double m = d2(0, 6);
  m = fmax(m, d2(1, 7));
  m = fmax(m, d2(2, 4));
  m = fmax(m, d2(3, 5));
  return sqrt(m);
}

__device__ double cell_hK(int dim, const double* __restrict__ cv, int measure, double det) {
  return cell_hK_s(dim == 2 ? kQuad : kHexa, dim, cv, measure, det);
}

// Mesh_size_in_convection_direction (ConvDiff.C:26-254), CELL_MEASURE 4: the
// vertex functions of the cell fitted in physical coordinates -- (1,x,y,xy)
// on quadrilaterals, (1,x,y,z) on tetrahedra, (1,x,y,z,xy,xz,yz,xyz) on
// hexahedra -- and h = 2|b| / sum_i |b.grad phi_i(barycentre)|, hK when the
// sum vanishes.  The inverse of the vertex system by Gauss-Jordan with
// partial pivoting; column i holds the coefficients of phi_i.
__device__ __noinline__ double conv_hK(int shape, int dim, const double* __restrict__ cv, const double* b,
                          double hK) {
  const int n = shape == kHexa ? 8 : 4;
  double a[8][8], x[8][8], sc[3] = {0, 0, 0};
#pragma unroll 1
  for (int i = 0; i < n; ++i) {
    const double* v = cv + i * dim;
    const double px = v[0], py = v[1], pz = dim == 3 ? v[2] : 0.0;
    sc[0] += px / n;
    sc[1] += py / n;
    sc[2] += pz / n;
    double r[8] = {1, px, py, 0, 0, 0, 0, 0};
    if (shape == kQuad) r[3] = px * py;
    else r[3] = pz;
    if (shape == kHexa) {
      r[4] = px * py;
      r[5] = px * pz;
      r[6] = py * pz;
      r[7] = px * py * pz;
    }
#pragma unroll 1
    for (int j = 0; j < n; ++j) {
      a[i][j] = r[j];
      x[i][j] = i == j ? 1.0 : 0.0;
    }
  }
#pragma unroll 1
  for (int c = 0; c < n; ++c) {
    int pr = c;
#pragma unroll 1
    for (int r = c + 1; r < n; ++r)
      if (fabs(a[r][c]) > fabs(a[pr][c])) pr = r;
    if (a[pr][c] == 0.0) return hK;
#pragma unroll 1
    for (int j = 0; j < n; ++j) {
      double t = a[c][j]; a[c][j] = a[pr][j]; a[pr][j] = t;
      t = x[c][j]; x[c][j] = x[pr][j]; x[pr][j] = t;
    }
    const double ip = 1.0 / a[c][c];
#pragma unroll 1
    for (int j = 0; j < n; ++j) {
      a[c][j] *= ip;
      x[c][j] *= ip;
    }
#pragma unroll 1
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const double f = a[r][c];
      if (f == 0.0) continue;
#pragma unroll 1
      for (int j = 0; j < n; ++j) {
        a[r][j] -= f * a[c][j];
        x[r][j] -= f * x[c][j];
      }
    }
  }
  double den = 0.0, nb = 0.0;
#pragma unroll 1
  for (int a2 = 0; a2 < dim; ++a2) nb += b[a2] * b[a2];
  nb = sqrt(nb);
#pragma unroll 1
  for (int i = 0; i < n; ++i) {
    double g[3];
    if (shape == kQuad) {
      g[0] = x[1][i] + x[3][i] * sc[1];
      g[1] = x[2][i] + x[3][i] * sc[0];
      g[2] = 0.0;
    } else if (shape == kTetra) {
      g[0] = x[1][i];
      g[1] = x[2][i];
      g[2] = x[3][i];
    } else {
      g[0] = x[1][i] + x[4][i] * sc[1] + x[5][i] * sc[2] + x[7][i] * sc[1] * sc[2];
      g[1] = x[2][i] + x[4][i] * sc[0] + x[6][i] * sc[2] + x[7][i] * sc[0] * sc[2];
      g[2] = x[3][i] + x[5][i] * sc[0] + x[6][i] * sc[1] + x[7][i] * sc[0] * sc[1];
    }
    double v = 0.0;
#pragma unroll 1
    for (int a2 = 0; a2 < dim; ++a2) v += b[a2] * g[a2];
    den += fabs(v);
  }
  return den < 1e-10 ? hK : 2 * nb / den;
}

// Compute_SDFEM_delta (ConvDiff.C:269-495); h is the cell's Get_hK, replaced
// by the size in convection direction for CELL_MEASURE 4
__device__ double sdfem_delta(const AsmCoefs& k, const double* cv, double h, double eps,
                              const double* b, double react, double linfb) {
  double delta = 0, alpha;
  if (k.cell_measure == 4) h = conv_hK(k.shape, k.dim, cv, b, h);
  if (fabs(eps) < 1e-20) eps = 1e-20;
  double nb = b[0] * b[0] + b[1] * b[1];
  if (k.dim == 3) nb += b[2] * b[2];
  nb = sqrt(nb);
  double reaction = fabs(react);
  switch (k.sdfem_type) {
    case 0:
      delta = (eps < h * nb) ? k.delta0 * h / nb : k.delta1 * h * h / eps;
      break;
    case 1:
    case 2: {
      double nu = 1.0 / k.poly_degree;
      if (nb > 0) {
        alpha = nu * nb * h / (2 * eps);
        delta = nu * h * (1 / tanh(alpha) - 1 / alpha) / (2 * nb);
      } else {
        delta = 0;
      }
      delta *= k.delta0;
      break;
    }
    case 4:
    case 5:
    case 8:
      delta = -1;
      if (k.sdfem_type == 4) {
        if (linfb > 0) delta = h / linfb;
      } else if (nb > 0) {
        delta = h / (2 * nb);
      }
      if (reaction > 0) {
        alpha = 1.0 / reaction;
        if (delta < 0 || alpha < delta) delta = alpha;
      }
      if (eps > 0) {
        alpha = h * h / eps;
        if (delta < 0 || alpha < delta) delta = alpha;
      }
      delta *= k.delta0;
      if (delta < 0) delta = 0;
      break;
    case 6: {
      // Franca/Valentin (2000)
      double r = reaction < 1e-20 ? 1e20 : reaction;
      alpha = 6 * eps / (h * h * r);
      if (alpha <= 1) alpha = 1;
      double alpha2 = h * nb / (3 * eps);
      if (alpha2 <= 1) alpha2 = 1;
      delta = 1 / (r * h * h * alpha + 6 * eps * alpha2);
      delta *= k.delta0 * h * h;
      break;
    }
    case 7:
      delta = k.delta0 * h * h / (4 * eps + 2 * h * nb + h * h * reaction);
      break;
    // the time-dependent estimates of John and Novo
    case 9:
      delta = k.delta0 * k.tau;
      break;
    case 10:
      eps /= (k.theta1 * k.tau);   // the unscaled diffusion of the 2D routines
      delta = eps <= h ? k.delta0 * h : k.delta0 * h * h / eps;
      break;
    case 11:
      nb /= k.tau;
      delta = nb > 0 ? k.delta0 * h * sqrt(k.tau) / nb : 0.0;
      break;
    case 12: {
      const double c_inv = k.delta0;
      delta = 100 * fmin(h / (2. * sqrt(3.0) * c_inv) *
                             fmin(0.25, sqrt(3.0) * h / (8 * eps * c_inv)), 1.);
      break;
    }
    default:
      delta = 0;   // rejected before any launch
  }
  return delta;
}

__device__ double cell_delta(const AsmCoefs& k, const double* cv, const Affine& A) {
  if (!k.supg) return 0.0;
  double h = cell_hK_s(k.shape, k.dim, cv, k.cell_measure, A.det);
  double linfb = fmax(fabs(k.b[0]), fabs(k.b[1]));
  if (k.dim == 3) linfb = fmax(linfb, fabs(k.b[2]));
  if (!k.tcd) return sdfem_delta(k, cv, h, k.eps, k.b, k.c, linfb);
  // TCDStiffSUPG / TCDMassSUPG / TCDRhsSUPG (CD_local_assembling_routines.C:
  // 184-387): in 2D the coefficients are scaled by theta1*tau first (except
  // SDFEM_TYPE 2 and 12, which keep them but take the scaled L_inf norm);
  // then delta *= theta1*tau except for the types 2, 9, 10, 11, 12
  const int ty = k.sdfem_type;
  double delta;
  if (k.dim == 2) {
    const double bs[3] = {k.ttau * k.b[0], k.ttau * k.b[1], 0.0};
    const double bb = fmax(fabs(bs[0]), fabs(bs[1]));
    if (ty != 2 && ty != 12)
      delta = sdfem_delta(k, cv, h, k.ttau * k.eps, bs,
                          ty == 8 ? k.ttau * k.c : 1.0 + k.ttau * k.c, bb);
    else
      delta = sdfem_delta(k, cv, h, k.eps, k.b, k.c, bb);
  } else {
    delta = sdfem_delta(k, cv, h, k.eps, k.b, k.c, linfb);
  }
  if (ty != 2 && ty != 9 && ty != 10 && ty != 11 && ty != 12) delta *= k.ttau;
  return delta;
}

// term blocks of RefTensors: S (ns), C (d), M (1), L (d*d), D (d), T (ns*d)
template <int DIM>
struct Terms {
  static constexpr int NS = DIM == 2 ? 3 : 6;
  static constexpr int offC = NS, offM = NS + DIM, offL = NS + DIM + 1;
  static constexpr int offD = offL + DIM * DIM, offT = offD + DIM;
  static constexpr int NT = offT + NS * DIM;
};

// per-cell factors g_t of the contraction.  mode 0: the stiffness terms;
// mode 1: mass, g = |det J| on M; mode 2: mass with the SUPG mass term of the
// time-dependent problem (TCDMassSUPG): delta (b.grad phi_i) phi_j, the D
// block with factor 1 in place of the reaction
template <int DIM>
__device__ void cell_factors(const AsmCoefs& k, const double* __restrict__ cv, double* g,
                             int mode) {
  using TT = Terms<DIM>;
  Affine A;
  cell_affine_s(k.shape, DIM, cv, A);
  const double adet = fabs(A.det);
  if (mode != 0) {
    for (int t = 0; t < TT::NT; ++t) g[t] = 0.0;
    g[TT::offM] = adet;
    if (mode == 2) {
      const double delta = cell_delta(k, cv, A);
      for (int a = 0; a < DIM; ++a) {
        double s = 0;
        for (int r = 0; r < DIM; ++r) s += A.Ji[a][r] * k.b[r];
        g[TT::offD + a] = adet * delta * s;
      }
    }
    return;
  }
  const double delta = cell_delta(k, cv, A);
  // convection at the map origin and its gradient: b(x0 + J xi) =
  // b(x0) + B J xi, in reference coordinates beta0 = J^-1 b(x0),
  // Gamma = J^-1 B J
  double bx0[3];
  b_at(k, A.x0, bx0);
  double bp[3];
  for (int a = 0; a < DIM; ++a) {
    double s = 0;
    for (int r = 0; r < DIM; ++r) s += A.Ji[a][r] * bx0[r];
    bp[a] = s;
  }
  int s = 0;
  double H[6];
  for (int a = 0; a < DIM; ++a)
    for (int bb = a; bb < DIM; ++bb) {
      double h = 0;
      for (int r = 0; r < DIM; ++r) h += A.Ji[a][r] * A.Ji[bb][r];
      H[s] = h;
      g[s] = adet * (k.eps * h + delta * bp[a] * bp[bb]);
      ++s;
    }
  for (int a = 0; a < DIM; ++a) g[TT::offC + a] = adet * bp[a];
  g[TT::offM] = adet * k.c;
  for (int a = 0; a < DIM; ++a)
    for (int c = 0; c < DIM; ++c) {
      double gam = 0;
      if (k.linear_b)
        for (int r = 0; r < DIM; ++r)
          for (int q = 0; q < DIM; ++q) gam += A.Ji[a][r] * k.bg[3 * r + q] * A.J[q][c];
      g[TT::offL + a * DIM + c] = adet * gam;
    }
  for (int a = 0; a < DIM; ++a) g[TT::offD + a] = adet * delta * k.c * bp[a];
  s = 0;
  for (int a = 0; a < DIM; ++a)
    for (int bb = a; bb < DIM; ++bb) {
      double m = (a == bb) ? 1.0 : 2.0;
      for (int c = 0; c < DIM; ++c)
        g[TT::offT + s * DIM + c] = -adet * delta * k.eps * m * H[s] * bp[c];
      ++s;
    }
}

// the factors of the stationary operator of every cell in FP32, for the
// matrix-free multigrid operator of Q2 hexahedral levels (matfree.cu)
__global__ void k_mf_factors(AsmCoefs k, int ncells, const double* __restrict__ verts,
                             float* __restrict__ fac) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= ncells) return;
  static_assert(Terms<3>::NT == kMfFactors, "factor layout of the matrix-free operator");
  double g[Terms<3>::NT];
  cell_factors<3>(k, verts + (size_t)cell * 8 * 3, g, 0);
  for (int t = 0; t < Terms<3>::NT; ++t) fac[(size_t)cell * kMfFactors + t] = (float)g[t];
}

// Position of every (cell, local DOF) result in the DOF-major array the
// matrix-free gather sums: the entries of active row r occupy
// [dof_rp[r], dof_rp[r+1]) in the order of dof_ent; -1 for non-active DOFs
// (identity rows, never summed)
__global__ void k_mf_pos(int nactive, const int* __restrict__ dof_rp,
                         const int* __restrict__ dof_ent, int* __restrict__ pos) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nactive) return;
  for (int e = dof_rp[r]; e < dof_rp[r + 1]; ++e) pos[dof_ent[e]] = e;
}

// Cells of a refined hexahedral hierarchy carry rotated and reflected local
// frames.  Where every cell is a translate of cell 0 (a uniform mesh, or one
// affine image of it), R = J_0^-1 J_c is a signed permutation: the node of
// cell c at reference point xi sits at R xi in cell 0's frame, so in that
// order the cell has cell 0's element matrix.  Per cell: the DOFs and the
// gather positions in cell 0's order (gdof_c, pos_c); any cell without such
// an R sets *nonuniform (its own order kept).
__global__ void k_mf_canon(int ncells, const double* __restrict__ verts,
                           const int* __restrict__ gdof, const int* __restrict__ pos,
                           int* __restrict__ gdof_c, int* __restrict__ pos_c,
                           int* __restrict__ loc_c, int* __restrict__ nonuniform) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= ncells) return;
  Affine A0, Ac;
  cell_affine(3, verts, A0);
  cell_affine(3, verts + (size_t)cell * 8 * 3, Ac);
  int R[3][3];
  bool ok = true, exact = true;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      double r = 0.0;
      for (int q = 0; q < 3; ++q) r += A0.Ji[a][q] * Ac.J[q][b];
      const double ri = rint(r);
      if (fabs(r - ri) > 1e-9 || fabs(ri) > 1.0) ok = false;
      if (fabs(r - ri) > 1e-13) exact = false;
      R[a][b] = (int)ri;
    }
  for (int a = 0; a < 3 && ok; ++a) {
    int nr = 0, nc = 0;
    for (int b = 0; b < 3; ++b) {
      nr += R[a][b] != 0;
      nc += R[b][a] != 0;
    }
    if (nr != 1 || nc != 1) ok = false;
  }
  const size_t o = (size_t)cell * 27;
  for (int k = 0; k < 27; ++k) {
    const int xi[3] = {k % 3 - 1, (k / 3) % 3 - 1, k / 9 - 1};
    int m = k;
    if (ok) {
      int xp[3];
      for (int a = 0; a < 3; ++a) xp[a] = R[a][0] * xi[0] + R[a][1] * xi[1] + R[a][2] * xi[2];
      m = (xp[0] + 1) + 3 * (xp[1] + 1) + 9 * (xp[2] + 1);
    }
    gdof_c[o + m] = gdof[o + k];
    pos_c[o + m] = pos[o + k];
    loc_c[o + m] = k;
  }
  // bit 0: not translates within 1e-9 (the FP32 operator's test); bit 1: not
  // within 1e-13 (the FP64 matrix from one element matrix must equal the
  // per-cell contraction to round-off)
  if (!ok) atomicOr(nonuniform, 3);
  else if (!exact) atomicOr(nonuniform, 2);
}

// A uniform level's FP64 matrix: every cell's element matrix is cell 0's
// (Ae = sum_t g_t R_t of cell 0, in its local order) with the cell's local
// DOFs listed in cell 0's frame, so one FP64 element matrix is formed and
// scattered into the CSR values through the slot map (entry (i, j) of cell 0's
// frame goes to the cell's local pair (loc_c[i], loc_c[j])), in place of
// ~22k FP64 multiply-adds per cell in the contraction; rows of non-active
// DOFs are skipped as in the contraction
__global__ void k_uniform_element64(AsmCoefs k, const double* __restrict__ verts,
                                    const double* __restrict__ R, double* __restrict__ Ae) {
  __shared__ double g0[Terms<3>::NT];
  if (threadIdx.x == 0) cell_factors<3>(k, verts, g0, 0);
  __syncthreads();
  // the factors outside the operator's term set are zero (no SUPG: delta
  // terms; constant b: the linear-convection block)
  for (int e = threadIdx.x; e < 27 * 27; e += blockDim.x) {
    double a = 0.0;
    for (int t = 0; t < Terms<3>::NT; ++t) a += g0[t] * R[(size_t)t * 729 + e];
    Ae[e] = a;
  }
}

__global__ void __launch_bounds__(256)
k_uniform_scatter(long n, int nactive, const int* __restrict__ gdof, const int* __restrict__ slot,
                  const int* __restrict__ loc_c, const double* __restrict__ Ae,
                  double* __restrict__ val) {
  for (long t = blockIdx.x * 256L + threadIdx.x; t < n; t += (long)gridDim.x * 256) {
    const long cell = t / 729;
    const int e = (int)(t - cell * 729), i = e / 27, j = e - i * 27;
    const int li = __ldg(loc_c + cell * 27 + i), lj = __ldg(loc_c + cell * 27 + j);
    if (__ldg(gdof + cell * 27 + li) >= nactive) continue;
    atomicAdd(val + __ldg(slot + cell * 729 + li * 27 + lj), __ldg(Ae + e));
  }
}

// element matrix of cell 0 in FP32, transposed (AeT[j*27 + i] = A_ij): the
// matrix of every cell of a uniform level, A = sum_t g_t R_t in FP64
__global__ void k_mf_element(AsmCoefs k, const double* __restrict__ verts,
                             const double* __restrict__ R, float* __restrict__ AeT) {
  __shared__ double g0[Terms<3>::NT];
  if (threadIdx.x == 0) cell_factors<3>(k, verts, g0, 0);
  __syncthreads();
  for (int e = threadIdx.x; e < 27 * 27; e += blockDim.x) {
    double a = 0.0;
    for (int t = 0; t < Terms<3>::NT; ++t) a += g0[t] * R[(size_t)t * 729 + e];
    AeT[(e % 27) * 27 + e / 27] = (float)a;
  }
}

// ---------------------------------------------------------------------------
// Element matrices on the tensor pipe, for operators used only in FP32 (the
// mixed-precision multigrid's levels between the finest and the coarsest):
// A(cells x entries) = G(cells x terms) R(terms x entries), the contraction
// of the FP64 kernel above, as one tcgen05 GEMM tile per 128 cells.  G and R
// are split into TF32 pairs (x = hi + lo), and D = Ghi Rhi + Ghi Rlo + Glo Rhi
// accumulates in FP32 in tensor memory: FP32-level accuracy (the lo*lo term,
// ~2^-22 of the product, is dropped).  Operands are staged in shared memory
// in the no-swizzle K-major layout (core matrices of 8 rows x 16 bytes,
// 128 B each; the next core along K at +128 B, along rows at +KP/4 * 128 B);
// one thread issues the MMAs (M = 128, N <= 256, K = 8 per instruction), a
// commit arrives on an mbarrier whose wait is bounded, and 16 warps read the
// tile back with tcgen05.ld (four per tensor-memory lane quarter, each a
// quarter of the columns) and add the entries of active rows into the FP32
// CSR values through the slot map.
// ---------------------------------------------------------------------------
constexpr int kTcCells = 128;
constexpr int kTcThreads = 512;      // four warps per tensor-memory lane quarter
constexpr long kTcSpin = 1L << 26;   // mbarrier polls before the wait counts as lost

__device__ __forceinline__ unsigned tc_smem(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ float tc_tf32(float x) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}
// float index of element (row, k) in the no-swizzle K-major layout with kg
// core matrices along K
__device__ __forceinline__ int tc_off(int row, int k, int kg) {
  return ((row >> 3) * kg + (k >> 2)) * 32 + (row & 7) * 4 + (k & 3);
}
__device__ __forceinline__ unsigned long long tc_desc(unsigned addr, unsigned lbo, unsigned sbo) {
  unsigned long long d = (unsigned long long)((addr & 0x3FFFF) >> 4);
  d |= (unsigned long long)(lbo >> 4) << 16;
  d |= (unsigned long long)(sbo >> 4) << 32;
  d |= 1ull << 46;   // descriptor version; base offset 0, no swizzle
  return d;
}

template <int DIM, int NLOC>
__global__ void __launch_bounds__(kTcThreads)
k_tc_contract(AsmCoefs k, int ncells, int nactive, const double* __restrict__ verts,
              const int* __restrict__ gdof, const int* __restrict__ slot,
              const double* __restrict__ R, float* __restrict__ val32, int* err) {
  using TT = Terms<DIM>;
  constexpr int NE = NLOC * NLOC;
  constexpr int KP = (TT::NT + 7) / 8 * 8;   // terms padded to the MMA's K step
  constexpr int KG = KP / 4;                  // core matrices along K
  constexpr int NV = DIM == 2 ? 4 : (NLOC == 4 || NLOC == 10 ? 4 : 8);
  extern __shared__ __align__(1024) float tsm[];
  float* Ahi = tsm;                    // kTcCells x KP
  float* Alo = Ahi + kTcCells * KP;
  float* Bhi = Alo + kTcCells * KP;    // 256 x KP
  float* Blo = Bhi + 256 * KP;
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ unsigned tbase;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int c0 = blockIdx.x * kTcCells;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;"
                 ::"r"(tc_smem(&tbase)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&mbar)));
  if (tid < kTcCells) {
    // the cell's factors (FP64) as TF32 pairs, one row per thread
    double g[TT::NT];
    const int cell = c0 + tid;
    if (cell < ncells)
      cell_factors<DIM>(k, verts + (size_t)cell * NV * DIM, g, 0);
    else
      for (int t = 0; t < TT::NT; ++t) g[t] = 0.0;
    for (int t = 0; t < KP; ++t) {
      const double x = t < TT::NT ? g[t] : 0.0;
      const float hi = tc_tf32((float)x);
      Ahi[tc_off(tid, t, KG)] = hi;
      Alo[tc_off(tid, t, KG)] = tc_tf32((float)(x - (double)hi));
    }
  }
  // this thread's cell in the epilogue: tensor-memory lane quarter warp % 4,
  // columns interleaved over the four warps of that quarter
  const int quarter = warp & 3, colgrp = warp >> 2;
  const int row = 32 * quarter + lane;
  const int ecell = c0 + row;
  unsigned active = 0;   // bit i: local row i is an active DOF
  if (ecell < ncells)
    for (int i = 0; i < NLOC; ++i)
      if (gdof[(size_t)ecell * NLOC + i] < nactive) active |= 1u << i;
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  const unsigned sbo = KG * 128;
  unsigned phase = 0;
  bool ok = true;
  for (int n0 = 0; n0 < NE; n0 += 256) {
    const int nv = min(256, NE - n0);          // valid entries in this tile
    const int nt = (nv + 15) / 16 * 16;        // MMA N (multiple of 16 for M = 128)
    for (int e = tid; e < nt * KP; e += kTcThreads) {
      const int n = e / KP, t = e - n * KP;
      const double x = (n < nv && t < TT::NT) ? R[(size_t)t * NE + n0 + n] : 0.0;
      const float hi = tc_tf32((float)x);
      Bhi[tc_off(n, t, KG)] = hi;
      Blo[tc_off(n, t, KG)] = tc_tf32((float)(x - (double)hi));
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = tbase;
    if (tid == 0) {
      // D f32, A and B tf32, both K-major, N >> 3 at bit 17, M >> 4 at bit 24
      const unsigned idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((unsigned)(nt >> 3) << 17) |
                             ((unsigned)(kTcCells >> 4) << 24);
      const float* As[3] = {Ahi, Ahi, Alo};
      const float* Bs[3] = {Bhi, Blo, Bhi};
      int acc = 0;
      for (int sp = 0; sp < 3; ++sp)
        for (int ks = 0; ks < KP / 8; ++ks) {
          const unsigned long long ad = tc_desc(tc_smem(As[sp]) + ks * 256, 128, sbo);
          const unsigned long long bd = tc_desc(tc_smem(Bs[sp]) + ks * 256, 128, sbo);
          asm volatile(
              "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
              "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
              ::"r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
          acc = 1;
        }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                   ::"r"(tc_smem(&mbar)) : "memory");
    }
    unsigned done = 0;
    for (long it = 0; it < kTcSpin && !done; ++it)
      asm volatile(
          "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
          "selp.u32 %0, 1, 0, p;\n\t}"
          : "=r"(done) : "r"(tc_smem(&mbar)), "r"(phase) : "memory");
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!done) {
      ok = false;
      if (lane == 0) atomicOr(err, kErrTimeout);
    }
    // uniform over the block: a lost wait in any warp ends the tile loop below
    if (__syncthreads_or(!ok)) {
      ok = false;
      break;
    }
    for (int cc = 16 * colgrp; cc < nt; cc += 64) {
      unsigned r[16];
      const unsigned addr = tmem + ((unsigned)(32 * quarter) << 16) + cc;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
          "%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
            "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
            "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(addr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (ecell < ncells) {
        int sl[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int e = n0 + cc + j;
          sl[j] = (cc + j < nv && ((active >> (e / NLOC)) & 1u))
                      ? __ldg(slot + (size_t)ecell * NE + e) : -1;
        }
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (sl[j] >= 0) atomicAdd(val32 + sl[j], __uint_as_float(r[j]));
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();   // tensor memory and the B tile are reused by the next tile
  }
  if (!ok) {
    // a lost wait: give the MMAs in flight another bounded wait before the
    // tensor memory is released
    unsigned done = 0;
    for (long it = 0; it < kTcSpin && !done; ++it)
      asm volatile(
          "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
          "selp.u32 %0, 1, 0, p;\n\t}"
          : "=r"(done) : "r"(tc_smem(&mbar)), "r"(phase ^ 1u) : "memory");
  }
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tbase));
}

__global__ void k_dirichlet_rows32(int n, int nactive, const int* __restrict__ dslot,
                                   float* __restrict__ val) {
  const int r = nactive + blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) val[dslot[r]] = 1.0f;
}

// inverse diagonal and the Dirichlet-coupling values of an FP32-only level
__global__ void k_finish_matrix32(int n, const int* __restrict__ dslot,
                                  const float* __restrict__ val32, float* __restrict__ invd32,
                                  int ndc, const int* __restrict__ dc_pos,
                                  float* __restrict__ dc_val32, int* err) {
  const long stride = (long)gridDim.x * blockDim.x;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < ndc; t += stride)
    dc_val32[t] = val32[dc_pos[t]];
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += stride) {
    const float d = val32[dslot[r]];
    if (d == 0.0f) atomicOr(err, kErrZeroDiag);
    invd32[r] = d == 0.0f ? 0.0f : 1.0f / d;
  }
}

// ---------------------------------------------------------------------------
// coupling -> CSR slot map (replaces the reference's linear row search)
// ---------------------------------------------------------------------------
__global__ void k_build_slots(int ncells, int nloc, const int* __restrict__ gdof,
                              const int* __restrict__ row_ptr, const int* __restrict__ col,
                              int* __restrict__ slot, int* err) {
  long n = (long)ncells * nloc * nloc;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n;
       t += (long)gridDim.x * blockDim.x) {
    int cell = (int)(t / (nloc * nloc));
    int ij = (int)(t % (nloc * nloc));
    int row = gdof[cell * nloc + ij / nloc];
    int c = gdof[cell * nloc + ij % nloc];
    int lo = row_ptr[row], hi = row_ptr[row + 1] - 1, found = -1;
    while (lo <= hi) {
      int mid = (lo + hi) >> 1;
      int v = col[mid];
      if (v == c) { found = mid; break; }
      if (v < c) lo = mid + 1; else hi = mid - 1;
    }
    slot[t] = found;
    if (found < 0) atomicOr(err, kErrPattern);
  }
}

__global__ void k_diag_slots(int n, const int* __restrict__ row_ptr, const int* __restrict__ col,
                             int* __restrict__ dslot, int* err) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  int lo = row_ptr[r], hi = row_ptr[r + 1] - 1, found = -1;
  while (lo <= hi) {
    int mid = (lo + hi) >> 1;
    int v = col[mid];
    if (v == r) { found = mid; break; }
    if (v < r) lo = mid + 1; else hi = mid - 1;
  }
  dslot[r] = found;
  if (found < 0) atomicOr(err, kErrPattern);
}

// ---------------------------------------------------------------------------
// element matrices: A_ij = sum_t g_t R_t[ij], scattered with FP64 atomics
// ---------------------------------------------------------------------------
// entries per block (EPB) and cell lanes per block: a block of EPB*LANES
// threads holds EPB entries' reference-tensor columns in registers and
// sweeps a tile of cells with LANES cells in flight
template <int NLOC> struct ContractShape;
template <> struct ContractShape<4> {   // Q1 quadrilateral, P1 tetrahedron
  static constexpr int NE = 16, EPB = 16, LANES = 16;
};
template <> struct ContractShape<9> {   // Q2 quadrilateral
  static constexpr int NE = 81, EPB = 81, LANES = 3;
};
template <> struct ContractShape<8> {   // Q1 hexahedron
  static constexpr int NE = 64, EPB = 64, LANES = 4;
};
template <> struct ContractShape<10> {  // P2 tetrahedron
  static constexpr int NE = 100, EPB = 100, LANES = 2;
};
template <> struct ContractShape<27> {  // Q2 hexahedron
  static constexpr int NE = 729, EPB = 243, LANES = 1;
};
template <int NLOC> struct ShapeInfo {
  using S = ContractShape<NLOC>;
  static constexpr int NEB = (S::NE + S::EPB - 1) / S::EPB;   // entry blocks
  static constexpr int THREADS = S::EPB * S::LANES;
};

// cells per block: one thread per cell computes the factors while the block
// waits, so larger tiles amortise that serial FP64 phase; with at least three
// blocks per SM (register cap) another block contracts meanwhile.  Measured on
// GB300: 663,552 P2 tetrahedra 3.36 ms (32 cells, 124 registers) -> 2.78 ms
// (64 cells, 3 blocks/SM); 32^3 Q2 1.57 -> 1.46 ms
constexpr int kCellTile = 64;

// which reference tensors a launch contracts
struct TermList {
  int idx[kMaxTerms];
};

template <int DIM, int NLOC, int NTU>
__global__ void __launch_bounds__(256, 3)
k_element_contract(AsmCoefs k, TermList tl, int mode, int all_rows, int ncells,
                   int nactive, const double* __restrict__ verts, const int* __restrict__ gdof,
                   const int* __restrict__ slot, const double* __restrict__ R,
                   double* __restrict__ val) {
  using S = ContractShape<NLOC>;
  constexpr int NV = DIM == 2 ? 4 : (NLOC == 8 || NLOC == 27 ? 8 : 4);
  constexpr int NT = Terms<DIM>::NT;
  __shared__ double g[kCellTile][NT];
  const int tile0 = blockIdx.x * kCellTile;
  // phase 1: per-cell factors
  for (int c = threadIdx.x; c < kCellTile; c += blockDim.x) {
    int cell = tile0 + c;
    if (cell < ncells) cell_factors<DIM>(k, verts + (size_t)cell * NV * DIM, g[c], mode);
  }
  __syncthreads();
  const int e_local = threadIdx.x % S::EPB;
  const int lane = threadIdx.x / S::EPB;
  const int e = blockIdx.y * S::EPB + e_local;
  if (lane >= S::LANES || e >= S::NE) return;
  double r[NTU];
#pragma unroll
  for (int t = 0; t < NTU; ++t) r[t] = __ldg(R + (size_t)tl.idx[t] * S::NE + e);
  const int i = e / NLOC;
  for (int c = lane; c < kCellTile; c += S::LANES) {
    int cell = tile0 + c;
    if (cell >= ncells) break;
    double acc = 0.0;
#pragma unroll
    for (int t = 0; t < NTU; ++t) acc = fma(g[c][tl.idx[t]], r[t], acc);
    int row = __ldg(gdof + (size_t)cell * NLOC + i);
    if (all_rows || row < nactive) atomicAdd(val + __ldg(slot + (size_t)cell * S::NE + e), acc);
  }
}

// Dirichlet rows: diagonal 1 (Matrix.C:225-233); other entries stay zero
__global__ void k_dirichlet_rows(int n, int nactive, const int* __restrict__ dslot,
                                 double* __restrict__ val) {
  int r = nactive + blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) val[dslot[r]] = 1.0;
}

// FP32 copy of the values and inverse diagonals (Iteration_jacobi.C:14-28);
// sell_val != null: the values of the active rows into the sliced ELLPACK copy
__global__ void k_finish_matrix(int n, int nnz, const int* __restrict__ dslot,
                                const double* __restrict__ val, float* __restrict__ val32,
                                double* __restrict__ invd, float* __restrict__ invd32,
                                const int* __restrict__ sell_pos, double* __restrict__ sell_val,
                                int ndc, const int* __restrict__ dc_pos,
                                double* __restrict__ dc_val, float* __restrict__ dc_val32,
                                int* err) {
  long stride = (long)gridDim.x * blockDim.x;
  // couplings of active rows to non-active columns, contiguous per row (the
  // first smoothing step reads them without the CSR slot indirection)
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < ndc; t += stride) {
    const double v = val[dc_pos[t]];
    dc_val[t] = v;
    dc_val32[t] = (float)v;
  }
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < nnz; t += stride) {
    const double v = val[t];
    val32[t] = (float)v;
    if (sell_val) {
      const int q = sell_pos[t];
      if (q >= 0) sell_val[q] = v;
    }
  }
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += stride) {
    double d = val[dslot[r]];
    if (d == 0.0) {
      atomicOr(err, kErrZeroDiag);
      invd[r] = 0.0;
      invd32[r] = 0.0f;
    } else {
      invd[r] = 1.0 / d;
      invd32[r] = (float)(1.0 / d);
    }
  }
}

// ---------------------------------------------------------------------------
// right-hand side: one warp per cell
// ---------------------------------------------------------------------------
struct RhsTables {
  const double* xi;    // nqp*3
  const double* w;     // nqp
  const double* val;   // nqp*nloc
  const double* grad;  // nqp*dim*nloc
};

__constant__ double c_tet_p2_nodes[10][3] = {
    {0, 0, 0}, {0.5, 0, 0}, {1, 0, 0}, {0, 0.5, 0}, {0.5, 0.5, 0},
    {0, 1, 0}, {0, 0, 0.5}, {0.5, 0, 0.5}, {0, 0.5, 0.5}, {0, 0, 1}};
__constant__ double c_tet_p1_nodes[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

__device__ void ref_node_s(int shape, int dim, int p, int k, double* r) {
  if (shape == kTetra) {
    for (int a = 0; a < 3; ++a) r[a] = p == 1 ? c_tet_p1_nodes[k][a] : c_tet_p2_nodes[k][a];
    return;
  }
  int n1 = p + 1;
  int i[3] = {k % n1, (k / n1) % n1, k / (n1 * n1)};
  for (int a = 0; a < 3; ++a) r[a] = (a < dim) ? -1.0 + (2.0 / p) * i[a] : 0.0;
}

__device__ void ref_node(int dim, int p, int k, double* r) { ref_node_s(dim == 2 ? kQuad : kHexa, dim, p, k, r); }

__device__ void line_basis_d(int p, double t, double* v) {
  if (p == 1) {
    v[0] = 0.5 * (1 - t);
    v[1] = 0.5 * (1 + t);
  } else {
    v[0] = 0.5 * t * (t - 1);
    v[1] = (1 - t) * (1 + t);
    v[2] = 0.5 * t * (t + 1);
  }
}

// value of P1/P2 basis function i at reference point xi of the tetrahedron
// (BF_C_T_P2_3D node order: vertices and edge midpoints by barycentric pairs)
__device__ double tet_basis_val_d(int p, const double* xi, int i) {
  const double l[4] = {1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]};
  if (p == 1) return l[i];
  const int va[10] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3};
  const int vb[10] = {0, 1, 1, 2, 2, 2, 3, 3, 3, 3};
  const int a = va[i], b = vb[i];
  return a == b ? l[a] * (2.0 * l[a] - 1.0) : 4.0 * l[a] * l[b];
}

__device__ int boundary_comp_d(int dim, const double* x) {
  const double t = 1e-12;
  if (dim == 2) {
    if (fabs(x[1]) < t) return 0;
    if (fabs(x[0] - 1) < t) return 1;
    if (fabs(x[1] - 1) < t) return 2;
    if (fabs(x[0]) < t) return 3;
    return -1;
  }
  if (fabs(x[2]) < t) return 0;
  if (fabs(x[1]) < t) return 1;
  if (fabs(x[0] - 1) < t) return 2;
  if (fabs(x[1] - 1) < t) return 3;
  if (fabs(x[0]) < t) return 4;
  if (fabs(x[2] - 1) < t) return 5;
  return -1;
}

// Right-hand side, cell tiles of kRhsTile cells per block.  GB300's FP64 pipe
// issues one warp instruction per 16 cycles per SM whatever the number of
// active lanes, so warp-uniform per-cell work (geometry, delta) runs one cell
// per thread:
//   phase 1  thread per cell: x0, J, |det J| (inverse and delta for SUPG)
//   phase 2  (cell, quadrature point): w |det J| f(x_q)
//   phase 3  (cell, local DOF): F_i = sum_q fw_q (phi_i + delta b.grad phi_i),
//            Dirichlet values at the nodes, Neumann edge integrals (2D) and
//            face integrals (hexahedra, tetrahedra)
constexpr int kRhsTile = 32;
constexpr int kRhsGeo = 18;   // x0[3], J[9], |det|, delta, b'[3]

template <int DIM>
__global__ void __launch_bounds__(256)
k_rhs(AsmCoefs k, int ncells, int nactive, const double* __restrict__ verts,
      const int* __restrict__ gdof, RhsTables tb, double* __restrict__ rhs,
      double* __restrict__ loc) {
  const int NV = k.shape == kHexa ? 8 : 4;
  __shared__ double geo[kRhsTile][kRhsGeo];
  __shared__ double fw[kRhsTile][128];
  const int tile0 = blockIdx.x * kRhsTile;
  const int nt = min(kRhsTile, ncells - tile0);
  const bool need_inv = k.supg || k.neumann_mask;
  if (threadIdx.x < nt) {
    const int c = threadIdx.x;
    const double* cv = verts + (size_t)(tile0 + c) * NV * DIM;
    Affine A;
    if (need_inv)
      cell_affine_s(k.shape, DIM, cv, A);
    else
      cell_geom_s(k.shape, DIM, cv, A);
    double* g = geo[c];
    for (int r = 0; r < 3; ++r) g[r] = r < DIM ? A.x0[r] : 0.0;
    for (int r = 0; r < 3; ++r)
      for (int a = 0; a < 3; ++a) g[3 + 3 * r + a] = (r < DIM && a < DIM) ? A.J[r][a] : 0.0;
    g[12] = fabs(A.det);
    const double delta = k.supg ? cell_delta(k, cv, A) : 0.0;
    g[13] = delta;
    for (int a = 0; a < 3; ++a) {
      double s = 0.0;
      if (delta != 0.0 && a < DIM)
        for (int r = 0; r < DIM; ++r) s += A.Ji[a][r] * k.b[r];
      g[14 + a] = s;
    }
  }
  __syncthreads();
  // an identically zero source (CDG_EX_BUMP) has a zero volume integral: the
  // quadrature would add exact zeros, so it is not run (same bits)
  const bool zero_f = k.example == CDG_EX_BUMP;
  const int nqp = k.nqp, nl = k.nloc;
  if (!zero_f) {
    for (int t = threadIdx.x; t < nt * nqp; t += blockDim.x) {
      const int c = t / nqp, q = t - c * nqp;
      const double* g = geo[c];
      double x[3];
      for (int r = 0; r < DIM; ++r) {
        double s = g[r];
        for (int a = 0; a < DIM; ++a) s += g[3 + 3 * r + a] * tb.xi[q * 3 + a];
        x[r] = s;
      }
      fw[c][q] = tb.w[q] * g[12] * ex_source(k, x);
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nt * nl; t += blockDim.x) {
    const int c = t / nl, i = t - c * nl;
    const int cell = tile0 + c;
    const double* g = geo[c];
    const int row = gdof[(size_t)cell * nl + i];
    if (row >= nactive) {
      // Dirichlet value: nodal functional of Lagrange elements = value at the
      // node (every cell sharing the node writes the same value)
      double r[3], x[3], u[6];
      ref_node_s(k.shape, DIM, k.order, i, r);
      for (int rr = 0; rr < DIM; ++rr) {
        double s = g[rr];
        for (int a = 0; a < DIM; ++a) s += g[3 + 3 * rr + a] * r[a];
        x[rr] = s;
      }
      ex_exact(k, x, u);
      rhs[row] = u[0];
      continue;
    }
    double F = 0.0;
    if (!zero_f) {
      const double delta = g[13];
      if (delta == 0.0) {
        // Galerkin: w f phi_i
        for (int q = 0; q < nqp; ++q) F = fma(fw[c][q], tb.val[q * nl + i], F);
      } else {
        // SUPG: w f (phi_i + delta b.grad phi_i)
        for (int q = 0; q < nqp; ++q) {
          double bg = 0.0;
          for (int a = 0; a < DIM; ++a) bg += g[14 + a] * tb.grad[(q * DIM + a) * nl + i];
          F = fma(fw[c][q], fma(delta, bg, tb.val[q * nl + i]), F);
        }
      }
    }
    // Neumann data on boundary edges (Assemble2D.C:3210-3248), 2D only
    if (DIM == 2 && k.neumann_mask) {
      const double* cv = verts + (size_t)cell * NV * DIM;
      Affine A;
      cell_affine_s(k.shape, DIM, cv, A);
      const double nrm[4][2] = {{0, -1}, {1, 0}, {0, 1}, {-1, 0}};
      for (int j = 0; j < 4; ++j) {
        const double* a0 = cv + 2 * j;
        const double* a1 = cv + 2 * ((j + 1) & 3);
        double ctr[2] = {0.5 * (a0[0] + a1[0]), 0.5 * (a0[1] + a1[1])};
        int comp = boundary_comp_d(2, ctr);
        if (comp < 0 || !((k.neumann_mask >> comp) & 1)) continue;
        int np = k.order + 1;   // line rule of degree 2p
        double lx[3], lw[3];
        if (np == 2) {
          lx[0] = -0.57735026918962576451; lx[1] = 0.57735026918962576451;
          lw[0] = lw[1] = 1.0;
        } else {
          lx[0] = -0.77459666924148337704; lx[1] = 0.0; lx[2] = 0.77459666924148337704;
          lw[0] = lw[2] = 5.0 / 9.0; lw[1] = 8.0 / 9.0;
        }
        double hE = 0.5 * sqrt((a1[0] - a0[0]) * (a1[0] - a0[0]) + (a1[1] - a0[1]) * (a1[1] - a0[1]));
        double G = 0.0;
        for (int l = 0; l < np; ++l) {
          double sp = 0.5 * (lx[l] + 1);
          double x[2] = {a0[0] + sp * (a1[0] - a0[0]), a0[1] + sp * (a1[1] - a0[1])};
          double u[6];
          ex_exact(k, x, u);
          double gval = k.eps * (nrm[comp][0] * u[1] + nrm[comp][1] * u[2]);
          double xi[2];
          for (int a = 0; a < 2; ++a)
            xi[a] = A.Ji[a][0] * (x[0] - A.x0[0]) + A.Ji[a][1] * (x[1] - A.x0[1]);
          double v0[3], v1[3];
          line_basis_d(k.order, xi[0], v0);
          line_basis_d(k.order, xi[1], v1);
          int n1 = k.order + 1;
          G += gval * hE * lw[l] * (v0[i % n1] * v1[i / n1]);
        }
        F += G;
      }
    }
    // Neumann data on boundary faces of hexahedra (Assemble3D.C:552-655):
    // g = eps n.grad(u), tensor Gauss rule of degree 2p on [-1,1]^2 mapped
    // bilinearly through the face's vertices, weight times |dx/ds x dx/dt|
    if (DIM == 3 && k.neumann_mask && k.shape == kHexa) {
      const double* cv = verts + (size_t)cell * NV * DIM;
      const int hf[6][4] = {{0, 1, 2, 3}, {0, 4, 5, 1}, {1, 5, 6, 2},
                            {2, 6, 7, 3}, {0, 3, 7, 4}, {4, 7, 6, 5}};
      const double nrm[6][3] = {{0, 0, -1}, {0, -1, 0}, {1, 0, 0},
                                {0, 1, 0},  {-1, 0, 0}, {0, 0, 1}};
      Affine A;
      cell_affine_s(k.shape, DIM, cv, A);
      const int n1 = k.order + 1;
      const int ia = i % n1, ib = (i / n1) % n1, ic = i / (n1 * n1);
      double lx[3], lw[3];
      if (n1 == 2) {
        lx[0] = -0.57735026918962576451; lx[1] = 0.57735026918962576451;
        lw[0] = lw[1] = 1.0;
      } else {
        lx[0] = -0.77459666924148337704; lx[1] = 0.0; lx[2] = 0.77459666924148337704;
        lw[0] = lw[2] = 5.0 / 9.0; lw[1] = 8.0 / 9.0;
      }
      for (int j = 0; j < 6; ++j) {
        double X[4][3], ctr[3] = {0, 0, 0};
        for (int m = 0; m < 4; ++m)
          for (int a = 0; a < 3; ++a) {
            X[m][a] = cv[hf[j][m] * 3 + a];
            ctr[a] += 0.25 * X[m][a];
          }
        const int comp = boundary_comp_d(3, ctr);
        if (comp < 0 || !((k.neumann_mask >> comp) & 1)) continue;
        double c1[3], c2[3], c3[3];
        for (int a = 0; a < 3; ++a) {
          c1[a] = (-X[0][a] + X[1][a] + X[2][a] - X[3][a]) * 0.25;
          c2[a] = (-X[0][a] - X[1][a] + X[2][a] + X[3][a]) * 0.25;
          c3[a] = (X[0][a] - X[1][a] + X[2][a] - X[3][a]) * 0.25;
        }
        double G = 0.0;
        for (int l1 = 0; l1 < n1; ++l1)
          for (int l2 = 0; l2 < n1; ++l2) {
            const double ps = lx[l1], pt = lx[l2];
            const double t0 = 0.5 * (ps + 1), t1 = 0.5 * (pt + 1);
            const double lc[4] = {(1 - t0) * (1 - t1), t0 * (1 - t1), t0 * t1, (1 - t0) * t1};
            double x[3] = {0, 0, 0};
            for (int m = 0; m < 4; ++m)
              for (int a = 0; a < 3; ++a) x[a] += lc[m] * X[m][a];
            double u[6];
            ex_exact(k, x, u);
            const double gval =
                k.eps * (nrm[comp][0] * u[1] + nrm[comp][1] * u[2] + nrm[comp][2] * u[3]);
            double ta[3], tb[3];
            for (int a = 0; a < 3; ++a) {
              ta[a] = c1[a] + pt * c3[a];
              tb[a] = c2[a] + ps * c3[a];
            }
            const double nx = ta[1] * tb[2] - ta[2] * tb[1];
            const double ny = ta[2] * tb[0] - ta[0] * tb[2];
            const double nz = ta[0] * tb[1] - ta[1] * tb[0];
            double xi[3];
            for (int a = 0; a < 3; ++a)
              xi[a] = A.Ji[a][0] * (x[0] - A.x0[0]) + A.Ji[a][1] * (x[1] - A.x0[1]) +
                      A.Ji[a][2] * (x[2] - A.x0[2]);
            double v0[3], v1[3], v2[3];
            line_basis_d(k.order, xi[0], v0);
            line_basis_d(k.order, xi[1], v1);
            line_basis_d(k.order, xi[2], v2);
            G += gval * lw[l1] * lw[l2] * sqrt(nx * nx + ny * ny + nz * nz) *
                 (v0[ia] * v1[ib] * v2[ic]);
          }
        F += G;
      }
    }
    // Neumann data on boundary faces of tetrahedra (Assemble3D.C:552-655,
    // triangular faces): g = eps n.grad(u) at x = X0 + s (X1-X0) + t (X2-X0),
    // weight times |(X1-X0) x (X2-X0)|; the rule on the reference triangle
    // is the collapsed Gauss rule with p+1 points per direction (degree 2p:
    // s = sigma (1 - tau), t = tau, weight (1 - tau) w_sigma w_tau / 4)
    if (DIM == 3 && k.neumann_mask && k.shape == kTetra) {
      const double* cv = verts + (size_t)cell * NV * DIM;
      const int tf[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
      const double nrm[6][3] = {{0, 0, -1}, {0, -1, 0}, {1, 0, 0},
                                {0, 1, 0},  {-1, 0, 0}, {0, 0, 1}};
      Affine A;
      cell_affine_s(k.shape, DIM, cv, A);
      const int n1 = k.order + 1;
      double lx[3], lw[3];
      if (n1 == 2) {
        lx[0] = -0.57735026918962576451; lx[1] = 0.57735026918962576451;
        lw[0] = lw[1] = 1.0;
      } else {
        lx[0] = -0.77459666924148337704; lx[1] = 0.0; lx[2] = 0.77459666924148337704;
        lw[0] = lw[2] = 5.0 / 9.0; lw[1] = 8.0 / 9.0;
      }
      for (int j = 0; j < 4; ++j) {
        double X[3][3], ctr[3] = {0, 0, 0};
        for (int m = 0; m < 3; ++m)
          for (int a = 0; a < 3; ++a) {
            X[m][a] = cv[tf[j][m] * 3 + a];
            ctr[a] += X[m][a] / 3.0;
          }
        const int comp = boundary_comp_d(3, ctr);
        if (comp < 0 || !((k.neumann_mask >> comp) & 1)) continue;
        double e1[3], e2[3];
        for (int a = 0; a < 3; ++a) {
          e1[a] = X[1][a] - X[0][a];
          e2[a] = X[2][a] - X[0][a];
        }
        const double cx = e1[1] * e2[2] - e1[2] * e2[1];
        const double cy = e1[2] * e2[0] - e1[0] * e2[2];
        const double cz = e1[0] * e2[1] - e1[1] * e2[0];
        const double area2 = sqrt(cx * cx + cy * cy + cz * cz);
        double G = 0.0;
        for (int l1 = 0; l1 < n1; ++l1)
          for (int l2 = 0; l2 < n1; ++l2) {
            const double sg = 0.5 * (lx[l1] + 1), ta = 0.5 * (lx[l2] + 1);
            const double fs = sg * (1 - ta), ft = ta;
            const double w = 0.25 * lw[l1] * lw[l2] * (1 - ta);
            double x[3];
            for (int a = 0; a < 3; ++a) x[a] = X[0][a] + fs * e1[a] + ft * e2[a];
            double u[6];
            ex_exact(k, x, u);
            const double gval =
                k.eps * (nrm[comp][0] * u[1] + nrm[comp][1] * u[2] + nrm[comp][2] * u[3]);
            double xi[3];
            for (int a = 0; a < 3; ++a)
              xi[a] = A.Ji[a][0] * (x[0] - A.x0[0]) + A.Ji[a][1] * (x[1] - A.x0[1]) +
                      A.Ji[a][2] * (x[2] - A.x0[2]);
            G += gval * w * area2 * tet_basis_val_d(k.order, xi, i);
          }
        F += G;
      }
    }
    // local rhs entry; the rows gather them in cell order (no atomics)
    loc[(size_t)cell * nl + i] = F;
  }
}

// rhs of the active rows: sum of the local entries of the row's DOF in
// (cell, local DOF) order -- the scatter of Assemble3D.C:257-292, reordered
// as a gather, deterministic
__global__ void k_rhs_gather(int nactive, const int* __restrict__ dof_rp,
                             const int* __restrict__ dof_ent, const double* __restrict__ loc,
                             double* __restrict__ rhs) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nactive; r += gridDim.x * blockDim.x) {
    double s = 0.0;
    const int e = dof_rp[r + 1];
    for (int q = dof_rp[r]; q < e; ++q) s += loc[__ldg(dof_ent + q)];
    rhs[r] = s;
  }
}

// solution.copy_nonactive(rhs)
__global__ void k_copy_nonactive(int n, int nactive, const double* __restrict__ rhs,
                                 double* __restrict__ sol) {
  int i = nactive + blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) sol[i] = rhs[i];
}

// ---------------------------------------------------------------------------
// error norms (TFEFunction2D/3D::GetErrors + conv_diff_l2_h1_linf_error,
// src/FE/FEFunction2D.C:291-470, src/AssembleRoutines/ConvDiff.C:2124-2183)
// ---------------------------------------------------------------------------
template <int DIM>
__global__ void __launch_bounds__(256)
k_errors(AsmCoefs k, int ncells, const double* __restrict__ verts, const int* __restrict__ gdof,
         const double* __restrict__ sol, RhsTables tb, int multi, double* __restrict__ acc,
         unsigned long long* __restrict__ linf) {
  const int NV = k.shape == kHexa ? 8 : 4;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cell = blockIdx.x * 8 + warp;
  if (cell >= ncells) return;
  const double* cv = verts + (size_t)cell * NV * DIM;
  // the cell's affine map, or its multilinear map evaluated at every point
  Affine A;
  MultiMap MM;
  double hK;
  if (multi) {
    multilinear_coeffs(DIM, cv, MM);
    hK = cell_hK_s(k.shape, DIM, cv, k.cell_measure, DIM == 2 ? quad_measure(cv) * 0.25 : 0.0);
  } else {
    cell_affine_s(k.shape, DIM, cv, A);
    hK = cell_hK_s(k.shape, DIM, cv, k.cell_measure, A.det);
  }
  const int nl = k.nloc;
  double fv = lane < nl ? sol[gdof[(size_t)cell * nl + lane]] : 0.0;
  double e[4] = {0, 0, 0, 0}, emax = 0.0;
  for (int q = 0; q < k.nqp; ++q) {
    // u_h and its gradient at q: warp reduction over local dofs
    double uh = lane < nl ? fv * tb.val[q * nl + lane] : 0.0;
    double gr[3] = {0, 0, 0};
    if (lane < nl)
      for (int a = 0; a < DIM; ++a) gr[a] = fv * tb.grad[(q * DIM + a) * nl + lane];
    for (int o = 16; o > 0; o >>= 1) {
      uh += __shfl_xor_sync(0xffffffffu, uh, o);
      for (int a = 0; a < DIM; ++a) gr[a] += __shfl_xor_sync(0xffffffffu, gr[a], o);
    }
    if (lane == 0) {
      double x[3], u[6], bx[3];
      if (multi) {
        multilinear_at(DIM, MM, tb.xi + q * 3, A);
        for (int r = 0; r < DIM; ++r) x[r] = A.x0[r];
      } else {
        for (int r = 0; r < DIM; ++r) {
          double s = A.x0[r];
          for (int a = 0; a < DIM; ++a) s += A.J[r][a] * tb.xi[q * 3 + a];
          x[r] = s;
        }
      }
      const double adet = fabs(A.det);
      double g[3] = {0, 0, 0};
      for (int r = 0; r < DIM; ++r)
        for (int a = 0; a < DIM; ++a) g[r] += A.Ji[a][r] * gr[a];
      ex_exact(k, x, u);
      b_at(k, x, bx);
      double linfb = fmax(fabs(bx[0]), fabs(bx[1]));
      if (DIM == 3) linfb = fmax(linfb, fabs(bx[2]));
      const double delta = sdfem_delta(k, cv, hK, k.eps, bx, k.c, linfb);
      double w = tb.w[q] * adet;
      double e0 = uh - u[0];
      emax = fmax(emax, fabs(e0));
      double e1 = g[0] - u[1], e2 = g[1] - u[2], e3 = DIM == 2 ? 0.0 : g[2] - u[3];
      e[0] += w * e0 * e0;
      e[1] += w * (e1 * e1 + e2 * e2 + e3 * e3);
      double e4 = bx[0] * e1 + bx[1] * e2 + (DIM == 3 ? bx[2] * e3 : 0.0);
      e[2] += w * (k.eps * (e1 * e1 + e2 * e2 + e3 * e3) + k.c * e0 * e0 + delta * e4 * e4);
      e[3] += w * (k.eps * (e1 * e1 + e2 * e2 + e3 * e3) + (e4 + k.c * e0) * e0);
    }
  }
  if (lane == 0) {
    for (int i = 0; i < 4; ++i) atomicAdd(acc + i, e[i]);
    atomicMax(linf, (unsigned long long)__double_as_longlong(emax));
  }
}

// ---------------------------------------------------------------------------
// time-dependent CD pieces
// ---------------------------------------------------------------------------
// initial condition: nodal interpolation of the example's u0 (every DOF)
__global__ void k_interpolate(AsmCoefs k, int ncells, const double* __restrict__ verts,
                              const int* __restrict__ gdof, double* __restrict__ sol) {
  const int NV = k.shape == kHexa ? 8 : 4;
  const long n = (long)ncells * k.nloc;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n;
       t += (long)gridDim.x * blockDim.x) {
    const int cell = (int)(t / k.nloc), loc = (int)(t % k.nloc);
    const double* cv = verts + (size_t)cell * NV * k.dim;
    Affine A;
    cell_affine_s(k.shape, k.dim, cv, A);
    double r[3], x[3];
    ref_node_s(k.shape, k.dim, k.order, loc, r);
    for (int rr = 0; rr < k.dim; ++rr) {
      double s = A.x0[rr];
      for (int a = 0; a < k.dim; ++a) s += A.J[rr][a] * r[a];
      x[rr] = s;
    }
    sol[gdof[t]] = ex_initial(k, x);   // all cells sharing a node write one value
  }
}

// Right-hand side of one step (TimeDiscretization::prepare_rhs_from_time_disc,
// TimeDiscretizations.C:117-189), on active rows
//   Crank-Nicolson  c_new f_new + c_new f_old + M u - c_new A u   (c_new = tau/2)
//   backward Euler  c_new f_new + M u                             (c_new = tau)
//   BDF2            c_new f_new + 4/3 M u - 1/3 M u2              (c_new = 2/3 tau)
// in the reference's order of additions; non-active rows take f_new (the
// Dirichlet data, copy_nonactive).  Only the operands a scheme uses are read.
template <int TPR, int KIND>
__global__ void __launch_bounds__(256)
k_tcd_rhs(int n, int nactive, const int* __restrict__ rp, const int* __restrict__ col,
          const double* __restrict__ Aval, const double* __restrict__ Mval,
          const double* __restrict__ u, const double* __restrict__ u2,
          const double* __restrict__ fnew, const double* __restrict__ fold, double c_new,
          double* __restrict__ out) {
  constexpr bool kA = KIND == CDG_TIME_CRANK_NICOLSON, kU2 = KIND == CDG_TIME_BDF_TWO;
  const long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int row = (int)(gt / TPR), sub = threadIdx.x % TPR;
  double sa = 0.0, sm = 0.0, sm2 = 0.0;
  if (row < nactive) {
    const int e = rp[row + 1];
    for (int k = rp[row] + sub; k < e; k += TPR) {
      const int c = __ldg(col + k);
      const double m = __ldcs(Mval + k);
      const double x = __ldg(u + c);
      sm = fma(m, x, sm);
      if (kA) sa = fma(__ldcs(Aval + k), x, sa);
      if (kU2) sm2 = fma(m, __ldg(u2 + c), sm2);
    }
  }
#pragma unroll
  for (int o = TPR / 2; o > 0; o >>= 1) {
    sm += __shfl_xor_sync(0xffffffffu, sm, o, TPR);
    if (kA) sa += __shfl_xor_sync(0xffffffffu, sa, o, TPR);
    if (kU2) sm2 += __shfl_xor_sync(0xffffffffu, sm2, o, TPR);
  }
  if (row >= n || sub != 0) return;
  if (row < nactive) {
    double r = c_new * fnew[row];
    if (kA) {
      r += c_new * fold[row];
      r += 1.0 * sm;
      r += -c_new * sa;
    } else if (kU2) {
      r += (4. / 3.) * sm;
      r += (-1. / 3.) * sm2;
    } else {
      r += 1.0 * sm;
    }
    out[row] = r;
  } else {
    out[row] = fnew[row];
  }
}

// system matrix (TimeDiscretization::prepare_system_matrix,
// TimeDiscretizations.C:195-251): active rows theta1 tau A + M, non-active
// rows keep the assembled stiffness rows
__global__ void k_tcd_system(int nactive_entries, int nnz, const double* __restrict__ Aval,
                             const double* __restrict__ Mval, double factor,
                             double* __restrict__ S) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < nnz; t += (long)gridDim.x * blockDim.x)
    S[t] = t < nactive_entries ? Aval[t] * factor + 1.0 * Mval[t] : Aval[t];
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <typename T>
static int dalloc(T** p, size_t n) {
  if (n == 0) n = 1;
  CDG_CUDA(cudaMalloc((void**)p, n * sizeof(T)));
  return CDG_OK;
}

int upload_level(cdg_context* ctx, DevLevel& L) {
  cudaStream_t st = ctx->stream;
  size_t nvd = (size_t)L.ncells * L.nv * L.dim;
  size_t nsl = (size_t)L.ncells * L.nloc * L.nloc;
  CDG_TRY(dalloc(&L.verts, nvd));
  CDG_TRY(dalloc(&L.gdof, (size_t)L.ncells * L.nloc));
  CDG_TRY(dalloc(&L.row_ptr, (size_t)L.ndof + 1));
  CDG_TRY(dalloc(&L.col, (size_t)L.nnz + 4));   // + tail padding of the staged chunks
  CDG_TRY(dalloc(&L.slot, nsl));
  CDG_TRY(dalloc(&L.diag_slot, (size_t)L.ndof));
  CDG_TRY(dalloc(&L.val64, (size_t)L.nnz));
  CDG_TRY(dalloc(&L.val32, (size_t)L.nnz + 4));
  CDG_TRY(dalloc(&L.rhs, (size_t)L.ndof));
  CDG_TRY(dalloc(&L.sol, (size_t)L.ndof));
  CDG_TRY(dalloc(&L.invdiag64, (size_t)L.ndof));
  CDG_TRY(dalloc(&L.invdiag32, (size_t)L.ndof));
  CDG_CUDA(cudaMemcpyAsync(L.verts, L.mesh.verts.data(), nvd * sizeof(double),
                           cudaMemcpyHostToDevice, st));
  CDG_CUDA(cudaMemcpyAsync(L.gdof, L.space.gdof.data(), L.space.gdof.size() * sizeof(int),
                           cudaMemcpyHostToDevice, st));
  CDG_CUDA(cudaMemcpyAsync(L.row_ptr, L.pattern.row_ptr.data(), (L.ndof + 1) * sizeof(int),
                           cudaMemcpyHostToDevice, st));
  CDG_CUDA(cudaMemcpyAsync(L.col, L.pattern.col.data(), (size_t)L.nnz * sizeof(int),
                           cudaMemcpyHostToDevice, st));
  CDG_CUDA(cudaMemsetAsync(L.sol, 0, (size_t)L.ndof * sizeof(double), st));
  CDG_CUDA(cudaMemsetAsync(L.rhs, 0, (size_t)L.ndof * sizeof(double), st));
  {
    std::vector<int> rp(L.nactive + 1, 0), dcol, dpos;
    for (int r = 0; r < L.nactive; ++r) {
      for (int k = L.pattern.row_ptr[r]; k < L.pattern.row_ptr[r + 1]; ++k)
        if (L.pattern.col[k] >= L.nactive) {
          dcol.push_back(L.pattern.col[k]);
          dpos.push_back(k);
        }
      rp[r + 1] = (int)dcol.size();
    }
    std::vector<int> rows;
    for (int r = 0; r < L.nactive; ++r)
      if (rp[r + 1] > rp[r]) rows.push_back(r);
    L.dc_nrows = (int)rows.size();
    CDG_TRY(dalloc(&L.dc_rows, std::max<size_t>(rows.size(), 1)));
    if (!rows.empty())
      CDG_CUDA(cudaMemcpyAsync(L.dc_rows, rows.data(), rows.size() * sizeof(int),
                               cudaMemcpyHostToDevice, st));
    CDG_TRY(dalloc(&L.dc_rp, rp.size()));
    CDG_TRY(dalloc(&L.dc_col, dcol.size()));
    CDG_TRY(dalloc(&L.dc_pos, dpos.size()));
    CDG_TRY(dalloc(&L.dc_val64, dpos.size()));
    CDG_TRY(dalloc(&L.dc_val32, dpos.size()));
    L.dc_n = (int)dpos.size();
    CDG_CUDA(cudaMemcpyAsync(L.dc_rp, rp.data(), rp.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    if (!dcol.empty()) {
      CDG_CUDA(cudaMemcpyAsync(L.dc_col, dcol.data(), dcol.size() * sizeof(int),
                               cudaMemcpyHostToDevice, st));
      CDG_CUDA(cudaMemcpyAsync(L.dc_pos, dpos.data(), dpos.size() * sizeof(int),
                               cudaMemcpyHostToDevice, st));
    }
    CDG_CUDA(cudaStreamSynchronize(st));   // host vectors go out of scope
  }
  {
    // active DOF -> local entries (cell * nloc + i) in increasing order
    std::vector<int> rp(L.nactive + 1, 0);
    const std::vector<int>& g = L.space.gdof;
    for (size_t e = 0; e < g.size(); ++e)
      if (g[e] < L.nactive) rp[g[e] + 1]++;
    for (int r = 0; r < L.nactive; ++r) rp[r + 1] += rp[r];
    std::vector<int> ent(rp[L.nactive]), fill(rp.begin(), rp.end() - 1);
    for (size_t e = 0; e < g.size(); ++e)
      if (g[e] < L.nactive) ent[fill[g[e]]++] = (int)e;
    CDG_TRY(dalloc(&L.dof_rp, rp.size()));
    CDG_TRY(dalloc(&L.dof_ent, ent.size()));
    CDG_TRY(dalloc(&L.rhs_loc, g.size()));
    CDG_CUDA(cudaMemcpyAsync(L.dof_rp, rp.data(), rp.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    if (!ent.empty())
      CDG_CUDA(cudaMemcpyAsync(L.dof_ent, ent.data(), ent.size() * sizeof(int),
                               cudaMemcpyHostToDevice, st));
    CDG_CUDA(cudaStreamSynchronize(st));
  }
  double avg = L.ndof ? (double)L.nnz / L.ndof : 1.0;
  // lanes per CSR row for 8-deep unrolled row sums: 8 * lanes >= avg row length
  L.rows_per_warp_hint = avg > 64 ? 16 : avg > 32 ? 8 : avg > 16 ? 4 : 2;
  return build_slots(ctx, L);
}

__global__ void k_sell_identity(int nd, const long long* __restrict__ q, double* __restrict__ v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nd) v[q[i]] = 1.0;
}

// Sliced ELLPACK layout of the level's pattern (see DevLevel::sell_*).  A
// warp takes one slice of 32/G rows whose lengths agree, so every FP64
// multiply-add has a full warp of useful lanes: CSR rows of 27..125 entries
// (Q2) split over a fixed number of lanes leave half of the FP64 issue slots
// to padding, and the FP64 pipe is what bounds these kernels on GB300.  The G
// lanes of a row take its consecutive entries, whose columns are close, so a
// gather touches few cache lines.  Sorting by length inside 256-row windows
// keeps the padding small and the rows of a slice close together.  (For the
// FP32 multigrid, bound by memory latency rather than the FP32 pipe, the CSR
// kernels measured faster, and it keeps them.)
int build_sell(cdg_context* ctx, DevLevel& L) {
  const int n = L.ndof, na = L.nactive;
  if (n < kSellMinRows) return CDG_OK;
  const std::vector<int>& rp = L.pattern.row_ptr;
  const std::vector<int>& cl = L.pattern.col;
  auto len = [&](int r) { return r < na ? rp[r + 1] - rp[r] : 1; };
  // lanes per row (measured on GB300, FP64 operator: 2 lanes beat 1, 4 and
  // 8 for Q2 hexahedra, 62 entries per row, and P2 tetrahedra, 28), doubled
  // on smaller levels until the launch has enough warps to cover the GPU
  const double avg = (double)L.nnz / n;
  int G = avg > 160 ? 4 : avg > 16 ? 2 : 1;
  while (G < 16 && (long)n * G / 32 < kSellMinWarps) G *= 2;
  if (const char* e = getenv("CDG_SELL_LANES")) {
    const int g = atoi(e);
    if (g == 0) return CDG_OK;                  // CSR kernels
    if (g == 1 || g == 2 || g == 4 || g == 8 || g == 16) G = g;
  }
  // built on the device (the same layout); CDG_SELL_HOST=1 builds it here
  if (!getenv("CDG_SELL_HOST")) {
    const int rc = device_sell(ctx, L, G);
    if (rc != CDG_ERR_LIMIT) return rc;
    return CDG_OK;                              // positions beyond int: keep CSR
  }
  const int R = 32 / G;                         // rows per slice
  const int nslices = (n + R - 1) / R;
  std::vector<int> order(n);
  for (int w0 = 0; w0 < n; w0 += kSellWindow) {
    const int w1 = std::min(n, w0 + kSellWindow);
    for (int r = w0; r < w1; ++r) order[r] = r;
    std::stable_sort(order.begin() + w0, order.begin() + w1,
                     [&](int a, int b) { return len(a) > len(b); });
  }
  std::vector<long long> off(nslices + 1, 0);
  std::vector<int> srow((size_t)nslices * R, -1);
  for (int s = 0; s < nslices; ++s) {
    int steps = 0;
    for (int i = 0; i < R && (long)s * R + i < n; ++i) {
      const int r = order[(size_t)s * R + i];
      srow[(size_t)s * R + i] = r;
      steps = std::max(steps, (len(r) + G - 1) / G);
    }
    off[s + 1] = off[s] + 32LL * steps;
  }
  const long long total = off[nslices];
  if (total >= (1LL << 31)) return CDG_OK;   // positions are int: keep the CSR operator
  std::vector<int> scol((size_t)total, 0), pos((size_t)L.nnz, -1);
  std::vector<long long> ident;
  for (int s = 0; s < nslices; ++s) {
    const int slots = (int)((off[s + 1] - off[s]) / 32) * G;   // per row
    for (int i = 0; i < R; ++i) {
      const int r = srow[(size_t)s * R + i];
      if (r < 0) continue;                      // padding row: column 0, value 0
      const int m = r < na ? rp[r + 1] - rp[r] : 0;
      for (int k = 0; k < slots; ++k) {
        const long long q = off[s] + 32LL * (k / G) + G * i + k % G;
        if (k < m) {
          scol[q] = cl[rp[r] + k];
          pos[rp[r] + k] = (int)q;
        } else {
          scol[q] = r;                          // padding: own row, value 0
        }
      }
      if (r >= na) ident.push_back(off[s] + G * i);   // identity row: 1 at its first slot
    }
  }
  cudaStream_t st = ctx->stream;
  CDG_TRY(dalloc(&L.sell_off, off.size()));
  CDG_TRY(dalloc(&L.sell_row, srow.size()));
  CDG_TRY(dalloc(&L.sell_col, (size_t)total));
  CDG_TRY(dalloc(&L.sell_val, (size_t)total));
  CDG_TRY(dalloc(&L.sell_pos, (size_t)L.nnz));
  CDG_CUDA(cudaMemcpyAsync(L.sell_off, off.data(), off.size() * sizeof(long long),
                           cudaMemcpyHostToDevice, st));
  CDG_CUDA(cudaMemcpyAsync(L.sell_row, srow.data(), srow.size() * sizeof(int),
                           cudaMemcpyHostToDevice, st));
  CDG_CUDA(cudaMemcpyAsync(L.sell_col, scol.data(), (size_t)total * sizeof(int),
                           cudaMemcpyHostToDevice, st));
  CDG_CUDA(cudaMemcpyAsync(L.sell_pos, pos.data(), (size_t)L.nnz * sizeof(int),
                           cudaMemcpyHostToDevice, st));
  CDG_CUDA(cudaMemsetAsync(L.sell_val, 0, (size_t)total * sizeof(double), st));
  if (!ident.empty()) {
    long long* dq = nullptr;
    CDG_TRY(dalloc(&dq, ident.size()));
    CDG_CUDA(cudaMemcpyAsync(dq, ident.data(), ident.size() * sizeof(long long),
                             cudaMemcpyHostToDevice, st));
    CDG_LAUNCH(ctx, k_sell_identity, grid_for<int>((long)ident.size(), 256), 256, 0,
               (int)ident.size(), dq, L.sell_val);
    CDG_CUDA(cudaStreamSynchronize(st));
    CDG_CUDA(cudaFree(dq));
  }
  CDG_CUDA(cudaStreamSynchronize(st));      // host vectors go out of scope
  L.sell_nslices = nslices;
  L.sell_lanes = G;
  L.sell_total = total;
  return CDG_OK;
}

// chunks of consecutive active rows with at most kBulkChunk entries each
int build_bulk(cdg_context* ctx, DevLevel& L) {
  if (L.nactive < kBulkMinRows) return CDG_OK;
  int chunk = kBulkChunk;   // off by default: slower than k_spmv on GB300 (2-3.5x)
  if (const char* e = getenv("CDG_BULK_CHUNK")) {   // 0: register-streaming kernels
    const int c = atoi(e);
    if (c == 0) return CDG_OK;
    if (c == 256 || c == 512 || c == 1024) chunk = c;
  }
  if (chunk == 0) return CDG_OK;
  const std::vector<int>& rp = L.pattern.row_ptr;
  std::vector<int> cr(1, 0);
  for (int r = 0; r < L.nactive; ++r) {
    const int len = rp[r + 1] - rp[r];
    if (len > chunk) return CDG_OK;             // a row beyond a chunk: keep CSR streaming
    if (rp[r + 1] - rp[cr.back()] > chunk) cr.push_back(r);
  }
  cr.push_back(L.nactive);
  CDG_TRY(dalloc(&L.bulk_row, cr.size()));
  CDG_CUDA(cudaMemcpyAsync(L.bulk_row, cr.data(), cr.size() * sizeof(int), cudaMemcpyHostToDevice,
                           ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  L.bulk_nchunks = (int)cr.size() - 1;
  L.bulk_chunk = chunk;
  return CDG_OK;
}

int free_level(DevLevel& L) {
  void* ptrs[] = {L.bulk_row, L.sell_off, L.sell_row, L.sell_col, L.sell_val, L.sell_pos,L.verts, L.gdof, L.row_ptr, L.col, L.slot, L.diag_slot, L.val64, L.val32,
                  L.rhs, L.sol, L.invdiag64, L.invdiag32, L.mg_rhs, L.mg_sol, L.mg_tmp,
                  L.mg_def, L.P_rp, L.P_col, L.P_val, L.P_val32, L.R_rp, L.R_col, L.R_val,
                  L.R_val32, L.coarse_inv, L.coarse_work, L.dc_rp, L.dc_col, L.dc_pos,
                  L.tcd_A, L.tcd_M, L.tcd_f, L.tcd_fold, L.tcd_u2, L.dof_rp, L.dof_ent,
                  L.rhs_loc, L.mf_fac, L.mf_y, L.mf_ae, L.mf_gdof, L.mf_pos, L.mf_pos_c,
                  L.mf_tile_rp, L.mf_tile_gdof, L.mf_ent_loc, L.mf_loc, L.ue64,
                  L.dc_val64, L.dc_val32, L.dc_rows, L.st_map, L.st_coef};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  return CDG_OK;
}

int check_device_error(cdg_context* ctx) {
  int h = 0;
  CDG_CUDA(cudaMemcpyAsync(&h, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (h) {
    CDG_CUDA(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
    if (h & kErrPattern) { set_error("local coupling not in the sparsity pattern"); return CDG_ERR_PATTERN; }
    if (h & kErrZeroDiag) { set_error("zero entry on the diagonal (Jacobi)"); return CDG_ERR_ZERO_DIAG; }
    if (h & kErrSingular) { set_error("singular coarse matrix"); return CDG_ERR_SINGULAR; }
    if (h & kErrBreakdown) { set_error("Unhappy breakdown in flexible gmres"); return CDG_ERR_BREAKDOWN; }
    if (h & kErrLattice) { set_error("a DOF lies off the lattice of the unit square / cube"); return CDG_ERR_ARG; }
    if (h & kErrTimeout) { set_error("a bounded wait for a staged copy ran out"); return CDG_ERR_TIMEOUT; }
    set_error("device error word %d", h);
    return CDG_ERR_CUDA;
  }
  return CDG_OK;
}

int build_slots(cdg_context* ctx, DevLevel& L) {
  long n = (long)L.ncells * L.nloc * L.nloc;
  int grid = (int)std::min<long>((n + 255) / 256, (long)ctx->num_sms * 32);
  CDG_LAUNCH(ctx, k_build_slots, grid, 256, 0, L.ncells, L.nloc, L.gdof, L.row_ptr, L.col,
             L.slot, ctx->d_err);
  CDG_LAUNCH(ctx, k_diag_slots, grid_for<int>(L.ndof, 256), 256, 0, L.ndof, L.row_ptr, L.col,
             L.diag_slot, ctx->d_err);
  return check_device_error(ctx);
}

static int ensure_tables(cdg_context* ctx, cdg_problem* p) {
  if (p->d_tables && p->rt_order == p->order) return CDG_OK;
  RefTensors T = make_ref_tensors(p->dim, p->order, p->shape);
  if (p->d_tables) cudaFree(p->d_tables);
  CDG_TRY(dalloc(&p->d_tables, T.R.size()));
  CDG_CUDA(cudaMemcpyAsync(p->d_tables, T.R.data(), T.R.size() * sizeof(double),
                           cudaMemcpyHostToDevice, ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  p->nterms = T.nterms;
  p->rt_order = p->order;
  return CDG_OK;
}

// contraction of the terms in `tl` (count NTU) into val
template <int DIM, int NLOC, int NTU>
static int launch_terms(cdg_context* ctx, const AsmCoefs& k, DevLevel& L, const double* R,
                        const TermList& tl, int mode, bool all_rows, double* out) {
  using S = ShapeInfo<NLOC>;
  dim3 grid((L.ncells + kCellTile - 1) / kCellTile, S::NEB);
  CDG_LAUNCH(ctx, (k_element_contract<DIM, NLOC, NTU>), grid, S::THREADS, 0, k, tl,
             mode, all_rows ? 1 : 0, L.ncells, L.nactive, L.verts, L.gdof,
             L.slot, R, out);
  return CDG_OK;
}

// term selection: galerkin (S, C, M [, L]), supg (S, C, M, D, T), mass (M),
// mass with the SUPG mass term (M, D)
enum class TermSet { Galerkin, GalerkinLinear, Supg, Mass, MassSupg };

template <int DIM, int NLOC>
static int contract_set(cdg_context* ctx, const AsmCoefs& k, DevLevel& L, const double* R,
                        TermSet set, bool all_rows, double* out) {
  using TT = Terms<DIM>;
  TermList tl{};
  int n = 0;
  if (set == TermSet::Mass) {
    tl.idx[n++] = TT::offM;
    return launch_terms<DIM, NLOC, 1>(ctx, k, L, R, tl, 1, all_rows, out);
  }
  if (set == TermSet::MassSupg) {
    tl.idx[n++] = TT::offM;
    for (int a = 0; a < DIM; ++a) tl.idx[n++] = TT::offD + a;
    return launch_terms<DIM, NLOC, 1 + DIM>(ctx, k, L, R, tl, 2, all_rows, out);
  }
  for (int t = 0; t < TT::offL; ++t) tl.idx[n++] = t;   // S, C, M
  if (set == TermSet::GalerkinLinear) {
    for (int t = TT::offL; t < TT::offD; ++t) tl.idx[n++] = t;
    return launch_terms<DIM, NLOC, TT::offD>(ctx, k, L, R, tl, 0, all_rows, out);
  }
  if (set == TermSet::Supg) {
    for (int t = TT::offD; t < TT::NT; ++t) tl.idx[n++] = t;
    return launch_terms<DIM, NLOC, TT::NT - DIM * DIM>(ctx, k, L, R, tl, 0, all_rows, out);
  }
  return launch_terms<DIM, NLOC, TT::offL>(ctx, k, L, R, tl, 0, all_rows, out);
}

static int contract(cdg_context* ctx, const AsmCoefs& k, DevLevel& L, const double* R,
                    TermSet set, bool all_rows, double* out) {
  if (L.shape == kQuad && L.nloc == 4) return contract_set<2, 4>(ctx, k, L, R, set, all_rows, out);
  if (L.shape == kQuad && L.nloc == 9) return contract_set<2, 9>(ctx, k, L, R, set, all_rows, out);
  if (L.shape == kHexa && L.nloc == 8) return contract_set<3, 8>(ctx, k, L, R, set, all_rows, out);
  if (L.shape == kHexa && L.nloc == 27) return contract_set<3, 27>(ctx, k, L, R, set, all_rows, out);
  if (L.shape == kTetra && L.nloc == 4) return contract_set<3, 4>(ctx, k, L, R, set, all_rows, out);
  if (L.shape == kTetra && L.nloc == 10) return contract_set<3, 10>(ctx, k, L, R, set, all_rows, out);
  set_error("unsupported element");
  return CDG_ERR_ARG;
}

static TermSet stiffness_set(const AsmCoefs& k) {
  if (k.supg) return TermSet::Supg;
  return k.linear_b ? TermSet::GalerkinLinear : TermSet::Galerkin;
}

static int check_coefs(const AsmCoefs& k) {
  if (k.nqp > 128) { set_error("quadrature rule too large"); return CDG_ERR_ARG; }
  if (k.supg) {
    // Compute_SDFEM_delta (ConvDiff.C:290-487): types 0-2 and 4-12; 3 and the
    // rest throw; 100 (a delta field of the finest level) is not taken here
    const int ty = k.sdfem_type;
    if (ty < 0 || ty == 3 || ty > 12) {
      set_error("SDFEM_TYPE %d not implemented", ty);
      return CDG_ERR_ARG;
    }
    if (!k.tcd && ty >= 9 && ty <= 11) {
      set_error("SDFEM_TYPE %d depends on the time step: time-dependent problem only", ty);
      return CDG_ERR_ARG;
    }
  }
  if (k.supg && k.linear_b) {
    set_error("SUPG with a convection field linear in x is not supported");
    return CDG_ERR_ARG;
  }
  return CDG_OK;
}

int contract_only(cdg_context* ctx, cdg_problem* p, DevLevel& L, const cdg_assembly_params& a) {
  CDG_TRY(ensure_tables(ctx, p));
  AsmCoefs k = make_coefs(a, L.shape, L.order);
  CDG_TRY(check_coefs(k));
  return contract(ctx, k, L, p->d_tables, stiffness_set(k), false, L.val64);
}

// reference tables for the rhs / error rules, cached per (device, shape,
// order, rule); shared by every problem and thread, never evicted (a few KB
// per entry, a handful of entries)
struct DevRefTables {
  int device = -1, shape = -1, order = 0, nqp1 = 0;
  double* buf = nullptr;
  RhsTables t{};
};
static DevRefTables g_rt[64];
static std::mutex g_rt_mutex;

static int get_rhs_tables(cdg_context* ctx, int shape, int order, int nqp1, RhsTables* out) {
  std::lock_guard<std::mutex> lock(g_rt_mutex);
  for (auto& e : g_rt)
    if (e.buf && e.device == ctx->device && e.shape == shape && e.order == order &&
        e.nqp1 == nqp1) {
      *out = e.t;
      return CDG_OK;
    }
  const int dim = shape == kQuad ? 2 : 3;
  RefTables T = make_ref_tables(dim, order, nqp1, shape);
  size_t n = T.xi.size() + T.w.size() + T.val.size() + T.grad.size();
  DevRefTables* slot = nullptr;
  for (auto& e : g_rt)
    if (!e.buf) { slot = &e; break; }
  if (!slot) { set_error("reference table cache full"); return CDG_ERR_LIMIT; }
  CDG_TRY(dalloc(&slot->buf, n));
  std::vector<double> h;
  h.reserve(n);
  h.insert(h.end(), T.xi.begin(), T.xi.end());
  h.insert(h.end(), T.w.begin(), T.w.end());
  h.insert(h.end(), T.val.begin(), T.val.end());
  h.insert(h.end(), T.grad.begin(), T.grad.end());
  CDG_CUDA(cudaMemcpyAsync(slot->buf, h.data(), n * sizeof(double), cudaMemcpyHostToDevice,
                           ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  slot->device = ctx->device;
  slot->shape = shape;
  slot->order = order;
  slot->nqp1 = nqp1;
  slot->t.xi = slot->buf;
  slot->t.w = slot->t.xi + T.xi.size();
  slot->t.val = slot->t.w + T.w.size();
  slot->t.grad = slot->t.val + T.val.size();
  *out = slot->t;
  return CDG_OK;
}

static int launch_rhs(cdg_context* ctx, const AsmCoefs& k, DevLevel& L, double* out) {
  RhsTables tb;
  CDG_TRY(get_rhs_tables(ctx, L.shape, L.order, k.nqp1, &tb));
  if (L.dim == 2)
    CDG_LAUNCH(ctx, k_rhs<2>, grid_for<int>(L.ncells, kRhsTile), 256, 0, k, L.ncells,
               L.nactive, L.verts, L.gdof, tb, out, L.rhs_loc);
  else
    CDG_LAUNCH(ctx, k_rhs<3>, grid_for<int>(L.ncells, kRhsTile), 256, 0, k, L.ncells,
               L.nactive, L.verts, L.gdof, tb, out, L.rhs_loc);
  if (L.nactive > 0)
    CDG_LAUNCH(ctx, k_rhs_gather, (int)std::min<long>((L.nactive + 255) / 256, (long)ctx->num_sms * 16),
               256, 0, L.nactive, L.dof_rp, L.dof_ent, L.rhs_loc, out);
  return CDG_OK;
}

// ---------------------------------------------------------------------------
// Assembly with coefficients given per (cell, quadrature point): the
// reference's per-point loop for a CoeffFct2D/3D example (GetLocalForms,
// BilinearAssembleGalerkin and BilinearAssemble_SD, ConvDiff.C:1776-1999,
// with Compute_SDFEM_delta taking the point's coefficients).  The contraction
// above needs cell-constant coefficients; this kernel takes any field.  One
// block per cell (grid-stride), 128 threads: the physical basis values of a
// point (value, gradient, Laplacian through the affine map) go to shared
// memory, every thread accumulates its entries of the local matrix over the
// points, and the entries of active rows are added into the CSR values
// through the slot map.  coef[(cell * nqp + q) * (DIM + 3) + k]: k = 0 eps,
// 1..DIM b, DIM+1 c, DIM+2 f.
// ---------------------------------------------------------------------------
struct QpTables {
  const double* w;      // nqp
  const double* xi;     // nqp * 3
  const double* val;    // nqp * nloc
  const double* grad;   // nqp * dim * nloc
  const double* hess;   // nqp * nsym * nloc (pairs (00,01,11) / (00,01,02,11,12,22))
  int nqp;
};

constexpr int kCoefThreads = 128;

// src 0: coef[(cell * nqp + q) * (DIM + 3) + k] from the caller (k = 0 eps,
// 1..DIM b, DIM+1 c, DIM+2 f); src 1: the example's eps, b(x), c, f(x) at
// the physical point.  multi: the cells' multilinear maps, evaluated at every
// point (J, J^-1, |det J|, the physical point and, in 2D, the Laplacian
// through the bilinear map's second derivatives); otherwise one affine map
// per cell.
template <int DIM>
__global__ void __launch_bounds__(kCoefThreads)
k_coef_element(AsmCoefs k, int ncells, int nactive, const double* __restrict__ verts,
               const int* __restrict__ gdof, const int* __restrict__ slot, QpTables tb,
               const double* __restrict__ coef, int src, int multi, double* __restrict__ val,
               double* __restrict__ rhs, double* __restrict__ loc) {
  constexpr int NSYM = DIM == 2 ? 3 : 6;
  constexpr int NACC = (kMaxLoc * kMaxLoc + kCoefThreads - 1) / kCoefThreads;
  __shared__ double ph[kMaxLoc][DIM + 2];   // phi, grad phi (physical), laplacian
  __shared__ double cq[DIM + 5];            // eps, b, c, f, delta, w |det J|
  __shared__ Affine A;                      // the cell's affine map, or the point's
  __shared__ MultiMap MM;
  __shared__ double lw[5];
  __shared__ double hK;
  const int NV = k.shape == kHexa ? 8 : 4;
  const int nl = k.nloc, ne = nl * nl, tid = threadIdx.x;
  for (int cell = blockIdx.x; cell < ncells; cell += gridDim.x) {
    const double* cv = verts + (size_t)cell * NV * DIM;
    if (tid == 0) {
      if (multi) {
        multilinear_coeffs(DIM, cv, MM);
        // measure-based cell sizes take the cell's area (two triangles in 2D)
        const double det = DIM == 2 ? quad_measure(cv) * 0.25 : 0.0;
        hK = cell_hK_s(k.shape, DIM, cv, k.cell_measure, det);
      } else {
        cell_affine_s(k.shape, DIM, cv, A);
        hK = cell_hK_s(k.shape, DIM, cv, k.cell_measure, A.det);
      }
    }
    __syncthreads();
    double acc[NACC], facc = 0.0;
#pragma unroll
    for (int m = 0; m < NACC; ++m) acc[m] = 0.0;
    for (int q = 0; q < tb.nqp; ++q) {
      if (multi) {
        if (tid == 64) {
          multilinear_at(DIM, MM, tb.xi + q * 3, A);
          if (DIM == 2 && k.supg) bilinear_lap_weights(MM, tb.xi + q * 3, lw);
        }
        __syncthreads();
      }
      if (tid < nl) {
        const int i = tid;
        ph[i][0] = tb.val[q * nl + i];
        for (int r = 0; r < DIM; ++r) {
          double s = 0.0;
          for (int a = 0; a < DIM; ++a) s += A.Ji[a][r] * tb.grad[(q * DIM + a) * nl + i];
          ph[i][1 + r] = s;
        }
        double l = 0.0;
        if (multi) {
          // bilinear map: lap = lw . (u_xi, u_eta, u_xixi, u_xieta, u_etaeta);
          // trilinear maps (Galerkin only) need none
          if (DIM == 2 && k.supg) {
            const double rd[5] = {tb.grad[(q * DIM) * nl + i], tb.grad[(q * DIM + 1) * nl + i],
                                  tb.hess[(q * NSYM) * nl + i], tb.hess[(q * NSYM + 1) * nl + i],
                                  tb.hess[(q * NSYM + 2) * nl + i]};
            for (int a = 0; a < 5; ++a) l += lw[a] * rd[a];
          }
        } else {
          // Laplacian of the affine image: sum_r J^-T H J^-1 (r, r)
          double H[3][3];
          int pr = 0;
          for (int a = 0; a < DIM; ++a)
            for (int b = a; b < DIM; ++b) {
              H[a][b] = H[b][a] = tb.hess[(q * NSYM + pr) * nl + i];
              ++pr;
            }
          for (int r = 0; r < DIM; ++r)
            for (int a = 0; a < DIM; ++a)
              for (int b = 0; b < DIM; ++b) l += A.Ji[a][r] * A.Ji[b][r] * H[a][b];
        }
        ph[i][DIM + 1] = l;
      } else if (tid == 32) {
        double bq[3] = {0.0, 0.0, 0.0}, linfb = 0.0;
        if (src == 0) {
          const double* ci = coef + ((size_t)cell * tb.nqp + q) * (DIM + 3);
          for (int a = 0; a < DIM + 3; ++a) cq[a] = ci[a];
          for (int a = 0; a < DIM; ++a) bq[a] = ci[1 + a];
        } else {
          double x[3] = {0.0, 0.0, 0.0};
          for (int r = 0; r < DIM; ++r) {
            double sx = A.x0[r];
            if (!multi)
              for (int a = 0; a < DIM; ++a) sx += A.J[r][a] * tb.xi[q * 3 + a];
            x[r] = sx;
          }
          b_at(k, x, bq);
          cq[0] = k.eps;
          for (int a = 0; a < DIM; ++a) cq[1 + a] = bq[a];
          cq[DIM + 1] = k.c;
          cq[DIM + 2] = ex_source(k, x);
        }
        for (int a = 0; a < DIM; ++a) linfb = fmax(linfb, fabs(bq[a]));
        cq[DIM + 3] = k.supg ? sdfem_delta(k, cv, hK, cq[0], bq, cq[DIM + 1], linfb) : 0.0;
        cq[DIM + 4] = tb.w[q] * fabs(A.det);
      }
      __syncthreads();
      const double eps = cq[0], c = cq[DIM + 1], f = cq[DIM + 2], delta = cq[DIM + 3];
      const double mult = cq[DIM + 4];
#pragma unroll
      for (int m = 0; m < NACC; ++m) {
        const int e = tid + m * kCoefThreads;
        if (e >= ne) break;
        const int i = e / nl, j = e - i * nl;
        double gg = 0.0, bgj = 0.0, bgi = 0.0;
        for (int r = 0; r < DIM; ++r) {
          gg += ph[i][1 + r] * ph[j][1 + r];
          bgj += cq[1 + r] * ph[j][1 + r];
          bgi += cq[1 + r] * ph[i][1 + r];
        }
        // Galerkin: eps grad phi_j . grad phi_i + (b . grad phi_j) phi_i + c phi_j phi_i
        double v = eps * gg + bgj * ph[i][0] + c * ph[j][0] * ph[i][0];
        // SUPG: delta (-eps lap phi_j + b . grad phi_j + c phi_j) (b . grad phi_i)
        if (delta != 0.0) v += delta * bgi * (-eps * ph[j][DIM + 1] + bgj + c * ph[j][0]);
        acc[m] = fma(mult, v, acc[m]);
      }
      if (tid < nl) {
        double bgi = 0.0;
        for (int r = 0; r < DIM; ++r) bgi += cq[1 + r] * ph[tid][1 + r];
        facc = fma(mult * f, ph[tid][0] + delta * bgi, facc);
      }
      __syncthreads();   // ph, cq and the point's map are rewritten for the next point
    }
#pragma unroll
    for (int m = 0; m < NACC; ++m) {
      const int e = tid + m * kCoefThreads;
      if (e >= ne) break;
      const int row = gdof[(size_t)cell * nl + e / nl];
      if (row < nactive) atomicAdd(val + slot[(size_t)cell * ne + e], acc[m]);
    }
    if (tid < nl) {
      const int row = gdof[(size_t)cell * nl + tid];
      loc[(size_t)cell * nl + tid] = facc;
      if (row >= nactive) {
        // Dirichlet value at the node from the example's boundary data
        double r[3], x[3], u[6];
        ref_node_s(k.shape, DIM, k.order, tid, r);
        if (multi) {
          Affine P;
          multilinear_at(DIM, MM, r, P);
          for (int rr = 0; rr < DIM; ++rr) x[rr] = P.x0[rr];
        } else {
          for (int rr = 0; rr < DIM; ++rr) {
            double sx = A.x0[rr];
            for (int a = 0; a < DIM; ++a) sx += A.J[rr][a] * r[a];
            x[rr] = sx;
          }
        }
        ex_exact(k, x, u);
        rhs[row] = u[0];
      }
    }
    __syncthreads();   // A, MM and hK are rewritten for the next cell
  }
}

static RefTables coef_tables(const DevLevel& L, const AsmCoefs& k, std::vector<double>* hess) {
  RefTables t = make_ref_tables(L.dim, L.order, k.nqp1, L.shape);
  const int nl = t.nloc, ns = L.dim == 2 ? 3 : 6;
  hess->assign((size_t)t.nqp * ns * nl, 0.0);
  std::vector<double> v(nl), g(3 * nl), h(6 * nl);
  for (int q = 0; q < t.nqp; ++q) {
    if (L.shape == kTetra)
      tetra_basis_point(L.order, &t.xi[3 * q], v.data(), g.data(), h.data());
    else
      ref_basis_point(L.dim, L.order, &t.xi[3 * q], v.data(), g.data(), h.data());
    for (int s2 = 0; s2 < ns; ++s2)
      for (int i = 0; i < nl; ++i) (*hess)[((size_t)q * ns + s2) * nl + i] = h[(size_t)s2 * nl + i];
  }
  return t;
}

int level_quadrature_points(const DevLevel& L, const cdg_assembly_params& a, int* nqp,
                            double* x) {
  AsmCoefs k = make_coefs(a, L.shape, L.order);
  RefTables t = make_ref_tables(L.dim, L.order, k.nqp1, L.shape);
  *nqp = t.nqp;
  if (!x) return CDG_OK;
  const int nv = L.mesh.nv, dim = L.dim;
  for (int c = 0; c < L.ncells; ++c)
    for (int q = 0; q < t.nqp; ++q) {
      const double* cv = &L.mesh.verts[(size_t)c * nv * dim];
      double* xq = x + ((size_t)c * t.nqp + q) * dim;
      if (L.multilinear)
        cell_point_multilinear(dim, cv, &t.xi[3 * q], xq);
      else
        cell_point(L.shape, dim, cv, &t.xi[3 * q], xq);
    }
  return CDG_OK;
}

static int finish_matrix(cdg_context* ctx, cdg_problem* p, DevLevel& L) {
  int g = (int)std::min<long>(((long)std::max(L.nnz, L.ndof) + 255) / 256, (long)ctx->num_sms * 16);
  CDG_LAUNCH(ctx, k_finish_matrix, g, 256, 0, L.ndof, L.nnz, L.diag_slot, L.val64, L.val32,
             L.invdiag64, L.invdiag32, L.sell_pos, L.sell_val, L.dc_n, L.dc_pos, L.dc_val64,
             L.dc_val32, p->d_zero_diag);
  return CDG_OK;
}

// once per Q2 hexahedral level: the DOF-major positions of the cells' local
// DOFs and the cells' frames relative to cell 0 (L.mf_geo = 1: every cell a
// translate of cell 0 once its DOFs are listed in cell 0's frame); on such
// levels the one-launch sweep's tiles and the DOF lattice of the stencil sweep
static int mf_geometry(cdg_context* ctx, DevLevel& L) {
  if (L.mf_geo >= 0) return CDG_OK;
  cudaStream_t st = ctx->stream;
  CDG_TRY(mf_ensure(L));
  CDG_CUDA(cudaMemsetAsync(L.mf_pos, 0xff, (size_t)L.ncells * 27 * sizeof(int), st));
  CDG_LAUNCH(ctx, k_mf_pos, grid_for<int>(L.nactive, 256), 256, 0, L.nactive, L.dof_rp,
             L.dof_ent, L.mf_pos);
  int* flag = nullptr;
  CDG_CUDA(cudaMalloc(&flag, sizeof(int)));
  int nonuni = 1;
  cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), st);
  if (e == cudaSuccess) {
    k_mf_canon<<<grid_for<int>(L.ncells, 128), 128, 0, st>>>(
        L.ncells, L.verts, L.gdof, L.mf_pos, L.mf_gdof, L.mf_pos_c, L.mf_loc, flag);
    ++ctx->launches;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&nonuni, flag, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(flag);
  CDG_CUDA(e);
  L.mf_geo = (nonuni & 1) ? 0 : 1;
  L.mf_geo_exact = nonuni == 0 ? 1 : 0;
  if (L.mf_geo == 1) {
    CDG_TRY(mf_build_tiles(ctx, L));
    CDG_TRY(mf_build_lattice(ctx, L));
  }
  return CDG_OK;
}

// the FP64 operator of a uniform level (every cell a translate of cell 0,
// constant coefficients): one element matrix scattered (CDG_UNIFORM_FP64=0
// keeps the per-cell contraction); false when the level does not qualify
static bool uniform_fp64(const DevLevel& L, const AsmCoefs& k) {
  const char* e = std::getenv("CDG_UNIFORM_FP64");
  const bool off = e && e[0] == '0';
  return !off && mf_eligible(L) && L.mf_geo_exact == 1 && !k.linear_b;
}

// the matrix-free FP32 operator takes the same factors (the SUPG term set
// has no linear-convection terms, so that combination keeps the CSR path)
static int mf_prepare(cdg_context* ctx, cdg_problem* p, DevLevel& L, const AsmCoefs& k) {
  L.mf_valid = 0;
  if (mf_eligible(L) && L.mf_mode != 0 && !(k.supg && k.linear_b)) {
    CDG_TRY(mf_geometry(ctx, L));
    // constant coefficients on translated cells: one element matrix;
    // otherwise per-cell factors for the sum-factorised kernel
    L.mf_uniform = L.mf_geo == 1 && !k.linear_b ? 1 : 0;
    if (L.mf_uniform) {
      CDG_LAUNCH(ctx, k_mf_element, 1, 256, 0, k, L.verts, p->d_tables, L.mf_ae);
      CDG_TRY(mf_stencil_coef(ctx, L));
    } else
      CDG_LAUNCH(ctx, k_mf_factors, grid_for<int>(L.ncells, 128), 128, 0, k, L.ncells, L.verts,
                 L.mf_fac);
    L.mf_valid = 1;
    L.mf_lin = k.linear_b;
  }
  return CDG_OK;
}

static int pointwise_assembly(cdg_context* ctx, cdg_problem* p, DevLevel& L, const AsmCoefs& k,
                              const double* coef_host);

int assemble_level(cdg_context* ctx, cdg_problem* p, DevLevel& L, const cdg_assembly_params& a) {
  CDG_TRY(ensure_tables(ctx, p));
  AsmCoefs k = make_coefs(a, L.shape, L.order);
  CDG_TRY(check_coefs(k));
  // cells with multilinear maps: the reference's per-point assembly with the
  // example's coefficients (the contraction needs one Jacobian per cell)
  if (L.multilinear) return pointwise_assembly(ctx, p, L, k, nullptr);
  cudaStream_t st = ctx->stream;
  // block->reset(), rhs.reset()
  CDG_CUDA(cudaMemsetAsync(L.val64, 0, (size_t)L.nnz * sizeof(double), st));
  CDG_CUDA(cudaMemsetAsync(L.rhs, 0, (size_t)L.ndof * sizeof(double), st));
  if (mf_eligible(L)) CDG_TRY(mf_geometry(ctx, L));
  if (uniform_fp64(L, k)) {
    CDG_LAUNCH(ctx, k_uniform_element64, 1, 256, 0, k, L.verts, p->d_tables, L.ue64);
    const long n = (long)L.ncells * 729;
    CDG_LAUNCH(ctx, k_uniform_scatter, (int)std::min<long>((n + 255) / 256, (long)ctx->num_sms * 32),
               256, 0, n, L.nactive, L.gdof, L.slot, L.mf_loc, L.ue64, L.val64);
  } else {
    CDG_TRY(contract(ctx, k, L, p->d_tables, stiffness_set(k), false, L.val64));
  }
  CDG_TRY(mf_prepare(ctx, p, L, k));
  int nd = L.ndof - L.nactive;
  if (nd > 0)
    CDG_LAUNCH(ctx, k_dirichlet_rows, grid_for<int>(nd, 256), 256, 0, L.ndof, L.nactive,
               L.diag_slot, L.val64);
  CDG_TRY(launch_rhs(ctx, k, L, L.rhs));
  if (nd > 0)
    CDG_LAUNCH(ctx, k_copy_nonactive, grid_for<int>(nd, 256), 256, 0, L.ndof, L.nactive, L.rhs,
               L.sol);
  L.fp64_stale = 0;
  return finish_matrix(ctx, p, L);
}

template <int DIM, int NLOC>
static int launch_tc(cdg_context* ctx, const AsmCoefs& k, DevLevel& L, const double* R) {
  constexpr int KP = (Terms<DIM>::NT + 7) / 8 * 8;
  const size_t smem = (size_t)(kTcCells + 256) * KP * 2 * sizeof(float);
  CDG_CUDA(cudaFuncSetAttribute(k_tc_contract<DIM, NLOC>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  CDG_LAUNCH(ctx, (k_tc_contract<DIM, NLOC>), (L.ncells + kTcCells - 1) / kTcCells, kTcThreads,
             smem, k, L.ncells, L.nactive, L.verts, L.gdof, L.slot, R, L.val32, ctx->d_err);
  return CDG_OK;
}

// A level whose operator is used only in FP32 (mixed-precision multigrid,
// between the finest and the coarsest level): its FP32 values from the
// tensor-core contraction, rhs and Dirichlet data as in assemble_level.  The
// FP64 values are not formed; ensure_fp64 forms them when something needs
// them (an FP64 solve, the matrix getter, the FP64 operator).
int assemble_level_tc(cdg_context* ctx, cdg_problem* p, DevLevel& L,
                      const cdg_assembly_params& a) {
  CDG_TRY(ensure_tables(ctx, p));
  AsmCoefs k = make_coefs(a, L.shape, L.order);
  CDG_TRY(check_coefs(k));
  if (k.supg && k.linear_b) return assemble_level(ctx, p, L, a);   // terms differ: FP64 path
  cudaStream_t st = ctx->stream;
  CDG_CUDA(cudaMemsetAsync(L.val32, 0, (size_t)L.nnz * sizeof(float), st));
  CDG_CUDA(cudaMemsetAsync(L.rhs, 0, (size_t)L.ndof * sizeof(double), st));
  int rc = CDG_ERR_ARG;
  if (L.shape == kHexa && L.nloc == 27) rc = launch_tc<3, 27>(ctx, k, L, p->d_tables);
  else if (L.shape == kHexa && L.nloc == 8) rc = launch_tc<3, 8>(ctx, k, L, p->d_tables);
  else if (L.shape == kQuad && L.nloc == 9) rc = launch_tc<2, 9>(ctx, k, L, p->d_tables);
  else if (L.shape == kQuad && L.nloc == 4) rc = launch_tc<2, 4>(ctx, k, L, p->d_tables);
  else if (L.shape == kTetra && L.nloc == 10) rc = launch_tc<3, 10>(ctx, k, L, p->d_tables);
  else if (L.shape == kTetra && L.nloc == 4) rc = launch_tc<3, 4>(ctx, k, L, p->d_tables);
  else set_error("unsupported element");
  CDG_TRY(rc);
  CDG_TRY(mf_prepare(ctx, p, L, k));
  const int nd = L.ndof - L.nactive;
  if (nd > 0)
    CDG_LAUNCH(ctx, k_dirichlet_rows32, grid_for<int>(nd, 256), 256, 0, L.ndof, L.nactive,
               L.diag_slot, L.val32);
  CDG_TRY(launch_rhs(ctx, k, L, L.rhs));
  if (nd > 0)
    CDG_LAUNCH(ctx, k_copy_nonactive, grid_for<int>(nd, 256), 256, 0, L.ndof, L.nactive, L.rhs,
               L.sol);
  const int g = (int)std::min<long>(((long)L.ndof + 255) / 256, (long)ctx->num_sms * 16);
  CDG_LAUNCH(ctx, k_finish_matrix32, g, 256, 0, L.ndof, L.diag_slot, L.val32, L.invdiag32,
             L.dc_n, L.dc_pos, L.dc_val32, p->d_zero_diag);
  L.fp64_stale = 1;
  L.last_a = a;
  return CDG_OK;
}

int ensure_fp64(cdg_context* ctx, cdg_problem* p, DevLevel& L) {
  if (!L.fp64_stale) return CDG_OK;
  return assemble_level(ctx, p, L, L.last_a);
}

// one level with coefficients per (cell, quadrature point) (the generic
// CoeffFct path); the matrix-free operator is not used for such a level
// what the multilinear (per-point) path takes: Dirichlet boundaries; on
// trilinear hexahedra no second derivatives (THexaTrilinear::
// GetOrigAllDerivatives, HexaTrilinear.C:185-222, throws) and the cell sizes
// from vertex distances (CELL_MEASURE 0 or 2)
int check_multilinear(const DevLevel& L, const AsmCoefs& k) {
  if (!L.multilinear) return CDG_OK;
  if (k.neumann_mask) {
    set_error("cells with multilinear maps: Dirichlet boundaries only");
    return CDG_ERR_ARG;
  }
  if (L.dim == 3 && k.supg) {
    set_error("SUPG needs second derivatives on trilinear hexahedra, which are not "
              "transformed (the reference throws here as well)");
    return CDG_ERR_ARG;
  }
  if (L.dim == 3 && k.cell_measure != 0 && k.cell_measure != 2) {
    set_error("trilinear hexahedra take CELL_MEASURE 0 or 2");
    return CDG_ERR_ARG;
  }
  return CDG_OK;
}

// per-point assembly of a level (k_coef_element): coefficients from the
// caller (coef_host, CoeffFct values at level_quadrature_points) or, with
// coef_host null, from the example at the physical points; each level's
// affine or multilinear cell maps
static int pointwise_assembly(cdg_context* ctx, cdg_problem* p, DevLevel& L, const AsmCoefs& k,
                              const double* coef_host) {
  if (k.neumann_mask) {
    set_error("the per-point assembly (CoeffFct coefficients, multilinear cells) handles "
              "Dirichlet boundaries only");
    return CDG_ERR_ARG;
  }
  CDG_TRY(check_multilinear(L, k));
  std::vector<double> hess;
  RefTables t = coef_tables(L, k, &hess);
  const int ncoef = L.dim + 3;
  const size_t ncoefs = coef_host ? (size_t)L.ncells * t.nqp * ncoef : 0;
  const size_t ntab = t.w.size() + t.xi.size() + t.val.size() + t.grad.size() + hess.size();
  cudaStream_t st = ctx->stream;
  double* buf = nullptr;
  CDG_TRY(dalloc(&buf, ntab + ncoefs));
  double* d = buf;
  QpTables tb;
  auto put = [&](const std::vector<double>& v) {
    cudaMemcpyAsync(d, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    const double* r = d;
    d += v.size();
    return r;
  };
  tb.w = put(t.w);
  tb.xi = put(t.xi);
  tb.val = put(t.val);
  tb.grad = put(t.grad);
  tb.hess = put(hess);
  tb.nqp = t.nqp;
  if (coef_host) {
    cudaError_t e = cudaMemcpyAsync(d, coef_host, ncoefs * sizeof(double),
                                    cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
      cudaFree(buf);
      CDG_CUDA(e);
    }
  }
  L.mf_valid = 0;
  L.fp64_stale = 0;
  CDG_CUDA(cudaMemsetAsync(L.val64, 0, (size_t)L.nnz * sizeof(double), st));
  CDG_CUDA(cudaMemsetAsync(L.rhs, 0, (size_t)L.ndof * sizeof(double), st));
  const int g = std::max(1, std::min(L.ncells, ctx->num_sms * 8));
  const int src = coef_host ? 0 : 1;
  if (L.dim == 2)
    CDG_LAUNCH(ctx, k_coef_element<2>, g, kCoefThreads, 0, k, L.ncells, L.nactive, L.verts,
               L.gdof, L.slot, tb, d, src, L.multilinear, L.val64, L.rhs, L.rhs_loc);
  else
    CDG_LAUNCH(ctx, k_coef_element<3>, g, kCoefThreads, 0, k, L.ncells, L.nactive, L.verts,
               L.gdof, L.slot, tb, d, src, L.multilinear, L.val64, L.rhs, L.rhs_loc);
  const int nd = L.ndof - L.nactive;
  if (nd > 0)
    CDG_LAUNCH(ctx, k_dirichlet_rows, grid_for<int>(nd, 256), 256, 0, L.ndof, L.nactive,
               L.diag_slot, L.val64);
  if (L.nactive > 0)
    CDG_LAUNCH(ctx, k_rhs_gather, (int)std::min<long>((L.nactive + 255) / 256, (long)ctx->num_sms * 16),
               256, 0, L.nactive, L.dof_rp, L.dof_ent, L.rhs_loc, L.rhs);
  if (nd > 0)
    CDG_LAUNCH(ctx, k_copy_nonactive, grid_for<int>(nd, 256), 256, 0, L.ndof, L.nactive, L.rhs,
               L.sol);
  CDG_TRY(finish_matrix(ctx, p, L));
  cudaError_t e = cudaStreamSynchronize(st);   // the tables and coefficients are released
  cudaFree(buf);
  CDG_CUDA(e);
  return CDG_OK;
}

int assemble_level_coefficients(cdg_context* ctx, cdg_problem* p, DevLevel& L,
                                const cdg_assembly_params& a, const double* coef_host) {
  AsmCoefs k = make_coefs(a, L.shape, L.order);
  CDG_TRY(check_coefs(k));
  return pointwise_assembly(ctx, p, L, k, coef_host);
}

int level_errors(cdg_context* ctx, cdg_problem* p, DevLevel& L, const cdg_assembly_params& a,
                 double* errors) {
  AsmCoefs k = make_coefs(a, L.shape, L.order);
  if (k.nqp > 128) { set_error("quadrature rule too large"); return CDG_ERR_ARG; }
  CDG_TRY(check_multilinear(L, k));
  RhsTables tb;
  CDG_TRY(get_rhs_tables(ctx, L.shape, L.order, k.nqp1, &tb));
  double* acc = nullptr;
  CDG_TRY(dalloc(&acc, 5));
  CDG_CUDA(cudaMemsetAsync(acc, 0, 5 * sizeof(double), ctx->stream));
  unsigned long long* lm = (unsigned long long*)(acc + 4);
  if (L.dim == 2)
    CDG_LAUNCH(ctx, k_errors<2>, grid_for<int>(L.ncells, 8), 256, 0, k, L.ncells, L.verts,
               L.gdof, L.sol, tb, L.multilinear, acc, lm);
  else
    CDG_LAUNCH(ctx, k_errors<3>, grid_for<int>(L.ncells, 8), 256, 0, k, L.ncells, L.verts,
               L.gdof, L.sol, tb, L.multilinear, acc, lm);
  double h[5];
  CDG_CUDA(cudaMemcpyAsync(h, acc, 5 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  cudaFree(acc);
  errors[0] = sqrt(h[0]);
  errors[1] = sqrt(h[1]);
  errors[2] = sqrt(h[2]);
  errors[3] = sqrt(fabs(h[3]));
  errors[4] = h[4];
  (void)p;
  return CDG_OK;
}

// ---------------------------------------------------------------------------
// time-dependent CD host pieces
// ---------------------------------------------------------------------------
static int ensure_tcd(DevLevel& L) {
  if (L.tcd_A) return CDG_OK;
  CDG_TRY(dalloc(&L.tcd_A, (size_t)L.nnz));
  CDG_TRY(dalloc(&L.tcd_M, (size_t)L.nnz));
  CDG_TRY(dalloc(&L.tcd_f, (size_t)L.ndof));
  CDG_TRY(dalloc(&L.tcd_fold, (size_t)L.ndof));
  CDG_CUDA(cudaMemset(L.tcd_fold, 0, (size_t)L.ndof * sizeof(double)));
  return CDG_OK;
}

int tcd_interpolate(cdg_context* ctx, cdg_problem* p, const cdg_assembly_params& a) {
  DevLevel& L = p->lev[0];
  AsmCoefs k = make_coefs(a, L.shape, L.order);
  long n = (long)L.ncells * L.nloc;
  int g = (int)std::min<long>((n + 255) / 256, (long)ctx->num_sms * 16);
  CDG_LAUNCH(ctx, k_interpolate, g, 256, 0, k, L.ncells, L.verts, L.gdof, L.sol);
  return CDG_OK;
}

// TimeConvectionDiffusion::call_assembling_routine with assemble_dirichlet_rows
// (TimeConvectionDiffusion.C:987-1052): stiffness (and mass) with full
// Dirichlet rows, rhs f at time a.t
// With SUPG (TCDStiffSUPG, TCDMassSUPG, TCDRhsSUPG) the stabilisation
// parameter depends on theta1 * tau, and the mass matrix carries a SUPG term,
// so it is reassembled with every step (TimeConvectionDiffusion.C:315-346).
int tcd_assemble_level(cdg_context* ctx, cdg_problem* p, DevLevel& L,
                       const cdg_assembly_params& a, bool with_mass, double theta1,
                       double tau) {
  if (L.multilinear) {
    set_error("the time-dependent problem takes affine cells (parallelograms, "
              "parallelepipeds, tetrahedra)");
    return CDG_ERR_ARG;
  }
  CDG_TRY(ensure_tables(ctx, p));
  CDG_TRY(ensure_tcd(L));
  L.mf_valid = 0;   // the FP32 operator becomes the time-dependent system
  L.fp64_stale = 0;
  AsmCoefs k = make_coefs(a, L.shape, L.order);
  k.tcd = 1;
  k.theta1 = theta1;
  k.tau = tau;
  k.ttau = theta1 * tau;
  CDG_TRY(check_coefs(k));
  if (k.supg && !(k.ttau > 0)) {
    set_error("SUPG for the time-dependent problem needs the time step");
    return CDG_ERR_ARG;
  }
  cudaStream_t st = ctx->stream;
  CDG_CUDA(cudaMemsetAsync(L.tcd_A, 0, (size_t)L.nnz * sizeof(double), st));
  CDG_TRY(contract(ctx, k, L, p->d_tables, stiffness_set(k), true, L.tcd_A));
  if (with_mass || k.supg) {
    CDG_CUDA(cudaMemsetAsync(L.tcd_M, 0, (size_t)L.nnz * sizeof(double), st));
    CDG_TRY(contract(ctx, k, L, p->d_tables, k.supg ? TermSet::MassSupg : TermSet::Mass, true,
                     L.tcd_M));
  }
  CDG_CUDA(cudaMemsetAsync(L.tcd_f, 0, (size_t)L.ndof * sizeof(double), st));
  return launch_rhs(ctx, k, L, L.tcd_f);
}

// rhs of the step into L.rhs from L.sol (u_old), tcd_u2 (BDF2), tcd_f (new)
// and tcd_fold; then tcd_fold <- tcd_f and tcd_u2 <- u_old (solution_m2 =
// solution_m1, TimeConvectionDiffusion::solve)
int tcd_rhs(cdg_context* ctx, DevLevel& L, TimeScheme ts, double tau) {
  const int tpr = 4;
  const int grid = (int)(((long)L.ndof * tpr + 255) / 256);
  const double c_new = ts.kind == CDG_TIME_BDF_TWO ? (2. / 3.) * tau : ts.theta1 * tau;
  if (ts.kind == CDG_TIME_CRANK_NICOLSON)
    CDG_LAUNCH(ctx, (k_tcd_rhs<4, CDG_TIME_CRANK_NICOLSON>), grid, 256, 0, L.ndof, L.nactive,
               L.row_ptr, L.col, L.tcd_A, L.tcd_M, L.sol, nullptr, L.tcd_f, L.tcd_fold, c_new,
               L.rhs);
  else if (ts.kind == CDG_TIME_BACKWARD_EULER)
    CDG_LAUNCH(ctx, (k_tcd_rhs<4, CDG_TIME_BACKWARD_EULER>), grid, 256, 0, L.ndof, L.nactive,
               L.row_ptr, L.col, nullptr, L.tcd_M, L.sol, nullptr, L.tcd_f, nullptr, c_new,
               L.rhs);
  else
    CDG_LAUNCH(ctx, (k_tcd_rhs<4, CDG_TIME_BDF_TWO>), grid, 256, 0, L.ndof, L.nactive,
               L.row_ptr, L.col, nullptr, L.tcd_M, L.sol, L.tcd_u2, L.tcd_f, nullptr, c_new,
               L.rhs);
  CDG_CUDA(cudaMemcpyAsync(L.tcd_fold, L.tcd_f, (size_t)L.ndof * sizeof(double),
                           cudaMemcpyDeviceToDevice, ctx->stream));
  CDG_CUDA(cudaMemcpyAsync(L.tcd_u2, L.sol, (size_t)L.ndof * sizeof(double),
                           cudaMemcpyDeviceToDevice, ctx->stream));
  return CDG_OK;
}

int tcd_start_history(cdg_context* ctx, DevLevel& L) {
  if (!L.tcd_u2) CDG_TRY(dalloc(&L.tcd_u2, (size_t)L.ndof));
  CDG_CUDA(cudaMemcpyAsync(L.tcd_u2, L.sol, (size_t)L.ndof * sizeof(double),
                           cudaMemcpyDeviceToDevice, ctx->stream));
  return CDG_OK;
}

// system matrix into val64 (+ FP32 copy and inverse diagonals); the factor is
// TimeDiscretization::get_scale_factor: tau, tau/2, 2/3 tau
int tcd_system(cdg_context* ctx, cdg_problem* p, DevLevel& L, TimeScheme ts, double tau) {
  const int nae = L.pattern.row_ptr[L.nactive];
  const double factor = ts.kind == CDG_TIME_BDF_TWO ? tau * (2. / 3.) : ts.theta1 * tau;
  int g = (int)std::min<long>(((long)L.nnz + 255) / 256, (long)ctx->num_sms * 16);
  CDG_LAUNCH(ctx, k_tcd_system, g, 256, 0, nae, L.nnz, L.tcd_A, L.tcd_M, factor, L.val64);
  return finish_matrix(ctx, p, L);
}

}  // namespace cdg

namespace cdg {

// ---------------------------------------------------------------------------
// Error norms without any allocation.
//
// cdg_problem_errors allocates a small accumulator on every call and keeps
// reference tables it allocates on first use.  Some callers cannot allocate
// device memory at that point: an application that hands the GPU's memory to
// its own pool or budget and forbids allocations outside it, or a serving
// loop that must not call cudaMalloc/cudaFree because those calls can
// synchronise the whole device and stall work other streams have in flight.
// cdg_problem_errors_noalloc computes the same norms with its scratch in the
// fixed device array below, which every GPU that loads this library keeps
// until the process exits.
// ---------------------------------------------------------------------------
constexpr int kNoAllocCellsPerBlock = 8;          // one warp per cell
constexpr int kNoAllocMaxBlocks = 16384;          // -> at most 131,072 cells
constexpr int kNoAllocMaxCells = kNoAllocCellsPerBlock * kNoAllocMaxBlocks;
// layout: [block partials: kNoAllocMaxBlocks x 5][5 results][pad][counter]
constexpr int kNoAllocSlots = kNoAllocMaxBlocks * 5 + 8;
static __device__ __align__(256) double g_errors_noalloc_scratch[kNoAllocSlots];

struct LineRule {
  int n;
  double x[kMaxQp1], w[kMaxQp1];
};

__device__ void line_basis_deriv(int p, double t, double* v, double* d) {
  line_basis_d(p, t, v);
  if (p == 1) {
    d[0] = -0.5;
    d[1] = 0.5;
  } else {
    d[0] = t - 0.5;
    d[1] = -2.0 * t;
    d[2] = t + 0.5;
  }
}

// same norms as k_errors; basis values at the Gauss points are evaluated in
// place from the 1D rule, and block partials go to the fixed scratch array;
// the last block to finish sums them in block order
template <int DIM>
__global__ void __launch_bounds__(256)
k_errors_noalloc(AsmCoefs k, LineRule rule, int ncells, const double* __restrict__ verts,
                 const int* __restrict__ gdof, const double* __restrict__ sol,
                 double* __restrict__ scratch) {
  constexpr int NV = DIM == 2 ? 4 : 8;
  __shared__ double wsum[kNoAllocCellsPerBlock][5];
  __shared__ bool last;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cell = blockIdx.x * kNoAllocCellsPerBlock + warp;
  double e[4] = {0, 0, 0, 0}, emax = 0.0;
  if (cell < ncells) {
    const double* cv = verts + (size_t)cell * NV * DIM;
    Affine A;
    cell_affine(DIM, cv, A);
    const double adet = fabs(A.det);
    const double hK = cell_hK(DIM, cv, k.cell_measure, A.det);
    const int nl = k.nloc, n1 = k.order + 1;
    const double fv = lane < nl ? sol[gdof[(size_t)cell * nl + lane]] : 0.0;
    const int ki[3] = {lane % n1, (lane / n1) % n1, lane / (n1 * n1)};
    const int nq = DIM == 2 ? rule.n * rule.n : rule.n * rule.n * rule.n;
    for (int q = 0; q < nq; ++q) {
      const int qi[3] = {q % rule.n, (q / rule.n) % rule.n, q / (rule.n * rule.n)};
      double xi[3] = {rule.x[qi[0]], rule.x[qi[1]], DIM == 3 ? rule.x[qi[2]] : 0.0};
      const double wq = rule.w[qi[0]] * rule.w[qi[1]] * (DIM == 3 ? rule.w[qi[2]] : 1.0);
      double uh = 0.0, gr[3] = {0, 0, 0};
      if (lane < nl) {
        double v[3][3], d[3][3];
        for (int a = 0; a < DIM; ++a) line_basis_deriv(k.order, xi[a], v[a], d[a]);
        double val = v[0][ki[0]] * v[1][ki[1]] * (DIM == 3 ? v[2][ki[2]] : 1.0);
        uh = fv * val;
        gr[0] = fv * d[0][ki[0]] * v[1][ki[1]] * (DIM == 3 ? v[2][ki[2]] : 1.0);
        gr[1] = fv * v[0][ki[0]] * d[1][ki[1]] * (DIM == 3 ? v[2][ki[2]] : 1.0);
        if (DIM == 3) gr[2] = fv * v[0][ki[0]] * v[1][ki[1]] * d[2][ki[2]];
      }
      for (int o = 16; o > 0; o >>= 1) {
        uh += __shfl_xor_sync(0xffffffffu, uh, o);
        for (int a = 0; a < DIM; ++a) gr[a] += __shfl_xor_sync(0xffffffffu, gr[a], o);
      }
      if (lane == 0) {
        double g[3] = {0, 0, 0};
        for (int r = 0; r < DIM; ++r)
          for (int a = 0; a < DIM; ++a) g[r] += A.Ji[a][r] * gr[a];
        double x[3], u[6], bx[3];
        for (int r = 0; r < DIM; ++r) {
          double s = A.x0[r];
          for (int a = 0; a < DIM; ++a) s += A.J[r][a] * xi[a];
          x[r] = s;
        }
        ex_exact(k, x, u);
        // convection (and with it delta) at the point: b may be linear in x
        b_at(k, x, bx);
        double linfb = fmax(fabs(bx[0]), fabs(bx[1]));
        if (DIM == 3) linfb = fmax(linfb, fabs(bx[2]));
        const double delta = sdfem_delta(k, cv, hK, k.eps, bx, k.c, linfb);
        const double w = wq * adet;
        const double e0 = uh - u[0];
        emax = fmax(emax, fabs(e0));
        const double e1 = g[0] - u[1], e2 = g[1] - u[2], e3 = DIM == 2 ? 0.0 : g[2] - u[3];
        e[0] += w * e0 * e0;
        e[1] += w * (e1 * e1 + e2 * e2 + e3 * e3);
        const double e4 = bx[0] * e1 + bx[1] * e2 + (DIM == 3 ? bx[2] * e3 : 0.0);
        e[2] += w * (k.eps * (e1 * e1 + e2 * e2 + e3 * e3) + k.c * e0 * e0 + delta * e4 * e4);
        e[3] += w * (k.eps * (e1 * e1 + e2 * e2 + e3 * e3) + (e4 + k.c * e0) * e0);
      }
    }
  }
  if (lane == 0) {
    for (int i = 0; i < 4; ++i) wsum[warp][i] = e[i];
    wsum[warp][4] = emax;
  }
  __syncthreads();
  unsigned* counter = reinterpret_cast<unsigned*>(scratch + kNoAllocSlots - 1);
  if (threadIdx.x == 0) {
    double b[5] = {0, 0, 0, 0, 0};
    for (int w = 0; w < kNoAllocCellsPerBlock; ++w) {
      for (int i = 0; i < 4; ++i) b[i] += wsum[w][i];
      b[4] = fmax(b[4], wsum[w][4]);
    }
    for (int i = 0; i < 5; ++i) scratch[(size_t)blockIdx.x * 5 + i] = b[i];
    __threadfence();
    last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  double r[5] = {0, 0, 0, 0, 0};
  for (int bl = 0; bl < (int)gridDim.x; ++bl) {
    const volatile double* pb = scratch + (size_t)bl * 5;
    for (int i = 0; i < 4; ++i) r[i] += pb[i];
    r[4] = fmax(r[4], pb[4]);
  }
  for (int i = 0; i < 5; ++i) scratch[(size_t)kNoAllocMaxBlocks * 5 + i] = r[i];
}

}  // namespace cdg

// per-device address of the scratch array, looked up once per device with the
// device current (the symbol's host-side name is not a device address)
static double* g_errors_noalloc_ptr[64];
static std::once_flag g_errors_noalloc_once[64];
static cudaError_t g_errors_noalloc_status[64];

extern "C" int cdg_problem_errors_noalloc(cdg_problem* p, const cdg_assembly_params* a,
                                          double* errors) {
  using namespace cdg;
  // the same argument checks as cdg_problem_errors
  CDG_TRY(check_assembly_params(p, a));
  if (!errors) {
    set_error("null output");
    return CDG_ERR_ARG;
  }
  cdg_context* ctx = p->ctx;
  DevLevel& L = p->lev[0];
  if (L.multilinear) {
    set_error("cdg_problem_errors_noalloc maps cells affinely; use cdg_problem_errors on "
              "meshes with multilinear cells");
    return CDG_ERR_ARG;
  }
  if (L.shape == kTetra) {
    set_error("cdg_problem_errors_noalloc evaluates tensor-product bases only "
              "(quadrilaterals, hexahedra); use cdg_problem_errors");
    return CDG_ERR_ARG;
  }
  if (L.ncells > kNoAllocMaxCells) {
    set_error("cdg_problem_errors_noalloc handles at most %d cells (its fixed scratch holds "
              "%d block partials); this level has %d cells, use cdg_problem_errors",
              kNoAllocMaxCells, kNoAllocMaxBlocks, L.ncells);
    return CDG_ERR_LIMIT;
  }
  if (ctx->device < 0 || ctx->device >= 64) {
    set_error("device index %d out of range", ctx->device);
    return CDG_ERR_ARG;
  }
  CDG_CUDA(cudaSetDevice(ctx->device));
  std::call_once(g_errors_noalloc_once[ctx->device], [&]() {
    g_errors_noalloc_status[ctx->device] = cudaGetSymbolAddress(
        (void**)&g_errors_noalloc_ptr[ctx->device], g_errors_noalloc_scratch);
  });
  if (g_errors_noalloc_status[ctx->device] != cudaSuccess) {
    set_error("cudaGetSymbolAddress of the error-norm scratch failed: %s",
              cudaGetErrorString(g_errors_noalloc_status[ctx->device]));
    return CDG_ERR_CUDA;
  }
  double* scratch = g_errors_noalloc_ptr[ctx->device];
  AsmCoefs k = make_coefs(*a, L.shape, L.order);
  LineRule rule;
  rule.n = k.nqp1;
  gauss_legendre(rule.n, rule.x, rule.w);
  // the last-block counter must start at zero on every call
  CDG_CUDA(cudaMemsetAsync(scratch + kNoAllocSlots - 1, 0, sizeof(double), ctx->stream));
  const int grid = (L.ncells + kNoAllocCellsPerBlock - 1) / kNoAllocCellsPerBlock;
  if (L.dim == 2)
    CDG_LAUNCH(ctx, k_errors_noalloc<2>, grid, 256, 0, k, rule, L.ncells, L.verts, L.gdof,
               L.sol, scratch);
  else
    CDG_LAUNCH(ctx, k_errors_noalloc<3>, grid, 256, 0, k, rule, L.ncells, L.verts, L.gdof,
               L.sol, scratch);
  double h[5];
  CDG_CUDA(cudaMemcpyAsync(h, scratch + (size_t)kNoAllocMaxBlocks * 5, 5 * sizeof(double),
                           cudaMemcpyDeviceToHost, ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  errors[0] = sqrt(h[0]);
  errors[1] = sqrt(h[1]);
  errors[2] = sqrt(h[2]);
  errors[3] = sqrt(fabs(h[3]));
  errors[4] = h[4];
  return CDG_OK;
}
