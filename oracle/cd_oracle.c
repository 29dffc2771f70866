/*
 * cd_oracle.c -- CPU restatement of ParMooN's scalar convection-diffusion
 * path.  TEST INFRASTRUCTURE ONLY (the checker for the CUDA path); see
 * cd_oracle.h.  Plain C99, single thread, FP64 everywhere, per quadrature
 * point exactly like the reference cell loop.
 *
 * Reference files restated (paths inside the ParMooN2022 tree):
 *   mesh refinement   src/Refinement/RefQuadRegDesc.C:21-29,
 *                     src/Refinement/RefHexaRegDesc.C:17-21,211-275,
 *                     src/Geometry/It_Finest.C (depth-first cell order),
 *                     src/Geometry/Tests.C:473-517 (UnitSquare root cell)
 *   DOF numbering     src/FE/FESpace2D.C:58-312, src/FE/FESpace3D.C:186-,
 *                     src/FE/FEMapper.C:385-610, src/FE/FESpace.C:1863-2099
 *   sparsity pattern  src/Matrix/Structure.C:226-618 (full rows, sorted cols)
 *   quadrature        src/QuadFormulas/QuadratureFormulaDatabase.C:22-151,
 *                     src/FE/FEDatabase.C:1553-1556 (degree = N_terms*p)
 *   basis             include/FE2D/BF_C_Q_Q1_2D.h, BF_C_Q_Q2_2D.h,
 *                     include/FE3D/BF_C_H_Q1_3D.h, BF_C_H_Q2_3D.h
 *   reference maps    src/FE/QuadAffin.C:175-, src/FE/HexaAffin.C:221-252
 *   local forms       src/AssembleRoutines/ConvDiff.C:1776-1999 (Galerkin,
 *                     SUPG), :269-495 (Compute_SDFEM_delta),
 *                     src/AssembleRoutines/LocalAssembling.C:734-970
 *   scatter           src/AssembleRoutines/Assemble3D.C:236-292,
 *                     src/AssembleRoutines/Assemble2D.C:3024-3046,
 *                     Dirichlet/Neumann data Assemble2D.C:3140-3260
 *   cell measure      src/Geometry/BaseCell.C:102-131, Rectangle.C:12-33,
 *                     Hexahedron.C:70-121
 *   solver            src/Solver/Iteration_gmres.C:430-620,
 *                     src/Solver/Utilities_gmres.C:60-108,
 *                     include/Solver/IterativeMethod.h:83-163,
 *                     src/Solver/Iteration_jacobi.C:14-39,168-182
 *   multigrid         src/Multigrid/Multigrid.C:157-410, CycleControl.C:15-111,
 *                     MultigridLevel.C:118-151, JacobiSmoother.C:21-29,
 *                     GridTransfer.C:29-410
 *   BlockFEMatrix     src/Matrix/BlockFEMatrix.C:969-1095 (identity on
 *                     non-active rows)
 *   error norms       src/FE/FEFunction2D.C:291-470,
 *                     src/AssembleRoutines/ConvDiff.C:2124-2183
 */
#include "cd_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MAXLOC 27
#define MAXQP 125
#define MAXV 8

static char g_err[256];
const char *orc_last_error(void) { return g_err; }
#define FAIL(...)                                                              \
  do {                                                                         \
    snprintf(g_err, sizeof g_err, __VA_ARGS__);                                \
    return -1;                                                                 \
  } while (0)

/* ------------------------------------------------------------------------ */
/* quadrature: Gauss-Legendre rules, tensorised                              */
/* ------------------------------------------------------------------------ */
static void gauss_legendre(int n, double *x, double *w) {
  /* Newton iteration on P_n in long double, nodes in ascending order */
  for (int i = 0; i < n; ++i) {
    long double z = cosl(3.14159265358979323846264338327950288L *
                         (i + 0.75L) / (n + 0.5L));
    long double pp = 0;
    for (int it = 0; it < 100; ++it) {
      long double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; ++j) {
        long double p3 = p2;
        p2 = p1;
        p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1);
      long double z1 = z;
      z = z1 - p1 / pp;
      if (fabsl(z - z1) < 1e-30L) break;
    }
    x[n - 1 - i] = (double)z;
    w[n - 1 - i] = (double)(2 / ((1 - z * z) * pp * pp));
  }
}

/* number of 1D Gauss points for a quad/hexa rule of the given accuracy
 * (QuadratureFormulaDatabase.C:41-81: 0-2 -> Gauss2, 3-5 -> Gauss3,
 * 6-7 -> Gauss4, 8-9 -> Gauss5, ...) */
static int gauss_points_for_degree(int deg) {
  if (deg > 17) deg = 17;
  if (deg <= 2) return 2;
  if (deg <= 5) return 3;
  return deg / 2 + 1;
}
/* line rules (QuadratureFormulaDatabase.C:108-133) */
static int line_points_for_degree(int deg) { return deg / 2 + 1; }

typedef struct {
  int nqp;
  double xi[MAXQP][3];
  double w[MAXQP];
} quad_rule;

static void make_rule(int dim, int n1, quad_rule *q) {
  double x[10], w[10];
  gauss_legendre(n1, x, w);
  q->nqp = 0;
  if (dim == 2) {
    for (int j = 0; j < n1; ++j)
      for (int i = 0; i < n1; ++i) {
        q->xi[q->nqp][0] = x[i];
        q->xi[q->nqp][1] = x[j];
        q->xi[q->nqp][2] = 0;
        q->w[q->nqp++] = w[i] * w[j];
      }
  } else {
    for (int k = 0; k < n1; ++k)
      for (int j = 0; j < n1; ++j)
        for (int i = 0; i < n1; ++i) {
          q->xi[q->nqp][0] = x[i];
          q->xi[q->nqp][1] = x[j];
          q->xi[q->nqp][2] = x[k];
          q->w[q->nqp++] = w[i] * w[j] * w[k];
        }
  }
}

/* collapsed Gauss rule on the unit tetrahedron, n points per direction:
 * xi = u, eta = v (1-u), zeta = w (1-u)(1-v), weight (1-u)^2 (1-v) / 8 */
static void make_tet_rule(int n, quad_rule *q) {
  double x[10], w[10];
  gauss_legendre(n, x, w);
  q->nqp = 0;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double u = 0.5 * (x[i] + 1), v = 0.5 * (x[j] + 1), t = 0.5 * (x[k] + 1);
        q->xi[q->nqp][0] = u;
        q->xi[q->nqp][1] = v * (1 - u);
        q->xi[q->nqp][2] = t * (1 - u) * (1 - v);
        q->w[q->nqp++] = 0.125 * w[i] * w[j] * w[k] * (1 - u) * (1 - u) * (1 - v);
      }
}
/* QuadratureFormulaDatabase.C:30-37: degree <= 2 P2Tetra, 3-4 P4Tetra, 5-6
 * P5Tetra; the rules of QuadFormula.C (P4Tetra :1693, P5Tetra :1739) are
 * Keast's symmetric rules (Comput. Methods Appl. Mech. Engrg. 55 (1986)
 * 339-348), written here as orbits in barycentric coordinates: kind 1 the
 * centroid, 4 the permutations of (a,b,b,b), 6 those of (a,a,b,b); w per
 * point.  Degrees above 6 fall back to the collapsed Gauss rule. */
typedef struct { int kind; double a, b, w; } tet_orbit;

static void tet_orbit_add(const tet_orbit *o, quad_rule *q) {
  double l[4];
  if (o->kind == 1) {
    for (int i = 0; i < 4; ++i) l[i] = 0.25;
    q->xi[q->nqp][0] = l[1]; q->xi[q->nqp][1] = l[2]; q->xi[q->nqp][2] = l[3];
    q->w[q->nqp++] = o->w;
    return;
  }
  for (int i = 0; i < 4; ++i)
    for (int j = (o->kind == 4 ? i : i + 1); j < (o->kind == 4 ? i + 1 : 4); ++j) {
      for (int m = 0; m < 4; ++m) l[m] = o->b;
      l[i] = o->a;
      l[j] = o->a;
      q->xi[q->nqp][0] = l[1]; q->xi[q->nqp][1] = l[2]; q->xi[q->nqp][2] = l[3];
      q->w[q->nqp++] = o->w;
    }
}

static int tet_points_for_degree(int deg) {
  if (deg <= 2) return 102;
  if (deg <= 4) return 104;
  if (deg <= 6) return 105;
  return (deg + 4) / 2;
}

static void make_tet_rule_by_code(int code, quad_rule *q) {
  if (code < 100) {
    make_tet_rule(code, q);
    return;
  }
  q->nqp = 0;
  if (code == 102) {
    const tet_orbit o = {4, 0.585410196624968454461376050311,
                         0.138196601125010515179541316563, 1.0 / 24.0};
    tet_orbit_add(&o, q);
  } else if (code == 104) {
    const tet_orbit o[3] = {
        {1, 0.25, 0.25, -74.0 / 5625.0},
        {4, 11.0 / 14.0, 1.0 / 14.0, 343.0 / 45000.0},
        {6, 0.399403576166799204996102147462, 0.100596423833200795003897852538,
         56.0 / 2250.0}};
    for (int i = 0; i < 3; ++i) tet_orbit_add(&o[i], q);
  } else {
    const tet_orbit o[4] = {
        {4, 0.0, 1.0 / 3.0, 0.602678571428571428571428571428571e-2},
        {1, 0.25, 0.25, 0.302836780970891758063769725577305e-1},
        {4, 8.0 / 11.0, 1.0 / 11.0, 0.116452490860289694108936091443380e-1},
        {6, 0.665501535736642982398804642263025e-1, 0.433449846426335701760119535773697,
         0.109491415613864593456430191124068e-1}};
    for (int i = 0; i < 4; ++i) tet_orbit_add(&o[i], q);
  }
}

/* ------------------------------------------------------------------------ */
/* Lagrange tensor basis Q1/Q2, derivatives up to order 2                    */
/* ------------------------------------------------------------------------ */
static void lag1d(int p, double t, double *v, double *d, double *dd) {
  if (p == 1) {
    v[0] = 0.5 * (1 - t); v[1] = 0.5 * (1 + t);
    d[0] = -0.5; d[1] = 0.5;
    dd[0] = 0; dd[1] = 0;
  } else {
    v[0] = 0.5 * t * (t - 1); v[1] = 1 - t * t; v[2] = 0.5 * t * (t + 1);
    d[0] = t - 0.5; d[1] = -2 * t; d[2] = t + 0.5;
    dd[0] = 1; dd[1] = -2; dd[2] = 1;
  }
}

/* values: [0]=phi, [1..d]=grad, then hessian entries (xx,xy,yy) in 2D,
 * (xx,xy,xz,yy,yz,zz) in 3D.  Local DOF k = k0 + (p+1)(k1 + (p+1)k2). */
#define NDER 10
static void ref_basis(int dim, int p, const double *xi, double out[][NDER]) {
  double v[3][3], d[3][3], dd[3][3];
  for (int a = 0; a < dim; ++a) lag1d(p, xi[a], v[a], d[a], dd[a]);
  int n1 = p + 1;
  if (dim == 2) {
    for (int k1 = 0; k1 < n1; ++k1)
      for (int k0 = 0; k0 < n1; ++k0) {
        int k = k0 + n1 * k1;
        out[k][0] = v[0][k0] * v[1][k1];
        out[k][1] = d[0][k0] * v[1][k1];
        out[k][2] = v[0][k0] * d[1][k1];
        out[k][3] = dd[0][k0] * v[1][k1];
        out[k][4] = d[0][k0] * d[1][k1];
        out[k][5] = v[0][k0] * dd[1][k1];
      }
  } else {
    for (int k2 = 0; k2 < n1; ++k2)
      for (int k1 = 0; k1 < n1; ++k1)
        for (int k0 = 0; k0 < n1; ++k0) {
          int k = k0 + n1 * (k1 + n1 * k2);
          double a = v[0][k0], b = v[1][k1], c = v[2][k2];
          out[k][0] = a * b * c;
          out[k][1] = d[0][k0] * b * c;
          out[k][2] = a * d[1][k1] * c;
          out[k][3] = a * b * d[2][k2];
          out[k][4] = dd[0][k0] * b * c;
          out[k][5] = d[0][k0] * d[1][k1] * c;
          out[k][6] = d[0][k0] * b * d[2][k2];
          out[k][7] = a * dd[1][k1] * c;
          out[k][8] = a * d[1][k1] * d[2][k2];
          out[k][9] = a * b * dd[2][k2];
        }
  }
}

/* P1/P2 on the unit tetrahedron, local DOF order of
 * include/FE3D/BF_C_T_P2_3D.h: vertices 0,2,5,9, edge midpoints 1 (v0v1),
 * 3 (v0v2), 4 (v1v2), 6 (v0v3), 7 (v1v3), 8 (v2v3); values laid out like
 * ref_basis: [0] phi, [1..3] grad, [4..9] Hessian (xx,xy,xz,yy,yz,zz) */
static const double TET_P2_NODES[10][3] = {{0, 0, 0}, {.5, 0, 0}, {1, 0, 0}, {0, .5, 0},
                                           {.5, .5, 0}, {0, 1, 0}, {0, 0, .5}, {.5, 0, .5},
                                           {0, .5, .5}, {0, 0, 1}};
static const double TET_P1_NODES[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
static void tet_basis(int p, const double *xi, double out[][NDER]) {
  double l[4] = {1 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]};
  double dl[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  static const int hp[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
  if (p == 1) {
    for (int k = 0; k < 4; ++k) {
      out[k][0] = l[k];
      for (int a = 0; a < 3; ++a) out[k][1 + a] = dl[k][a];
      for (int s2 = 0; s2 < 6; ++s2) out[k][4 + s2] = 0;
    }
    return;
  }
  static const int va[10] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3};
  static const int vb[10] = {0, 1, 1, 2, 2, 2, 3, 3, 3, 3};
  for (int k = 0; k < 10; ++k) {
    int a0 = va[k], b0 = vb[k];
    if (a0 == b0) {
      out[k][0] = l[a0] * (2 * l[a0] - 1);
      for (int a = 0; a < 3; ++a) out[k][1 + a] = (4 * l[a0] - 1) * dl[a0][a];
      for (int s2 = 0; s2 < 6; ++s2) out[k][4 + s2] = 4 * dl[a0][hp[s2][0]] * dl[a0][hp[s2][1]];
    } else {
      out[k][0] = 4 * l[a0] * l[b0];
      for (int a = 0; a < 3; ++a) out[k][1 + a] = 4 * (dl[a0][a] * l[b0] + l[a0] * dl[b0][a]);
      for (int s2 = 0; s2 < 6; ++s2)
        out[k][4 + s2] = 4 * (dl[a0][hp[s2][0]] * dl[b0][hp[s2][1]] +
                              dl[a0][hp[s2][1]] * dl[b0][hp[s2][0]]);
    }
  }
}

static void local_dof_ref(int dim, int p, int k, double *r) {
  int n1 = p + 1;
  int i0 = k % n1, i1 = (k / n1) % n1, i2 = k / (n1 * n1);
  double step = 2.0 / p;
  r[0] = -1 + step * i0;
  r[1] = -1 + step * i1;
  r[2] = dim == 3 ? -1 + step * i2 : 0;
}

/* ------------------------------------------------------------------------ */
/* mesh: unit square / cube root cell, regular refinement, depth-first order */
/* ------------------------------------------------------------------------ */
/* new-vertex definitions: each new vertex is the mean of a set of old ones */
static const int QUAD_NEWV[9][4] = {{0}, {1}, {2}, {3}, {0, 1}, {1, 2},
                                    {2, 3}, {3, 0}, {0, 1, 2, 3}};
static const int QUAD_NEWV_N[9] = {1, 1, 1, 1, 2, 2, 2, 2, 4};
static const int QUAD_CHILD[4][4] = {
    {0, 4, 8, 7}, {1, 5, 8, 4}, {2, 6, 8, 5}, {3, 7, 8, 6}};

static const int HEX_NEWV[27][8] = {
    {0}, {1}, {2}, {3}, {4}, {5}, {6}, {7},
    {0, 1},              /* 8  */
    {1, 2},              /* 9  */
    {2, 3},              /* 10 */
    {3, 0},              /* 11 */
    {0, 1, 2, 3},        /* 12 */
    {1, 5},              /* 13 */
    {4, 5},              /* 14 */
    {0, 4},              /* 15 */
    {0, 4, 5, 1},        /* 16 */
    {2, 6},              /* 17 */
    {5, 6},              /* 18 */
    {1, 5, 6, 2},        /* 19 */
    {3, 7},              /* 20 */
    {6, 7},              /* 21 */
    {2, 6, 7, 3},        /* 22 */
    {7, 4},              /* 23 */
    {0, 3, 7, 4},        /* 24 */
    {4, 7, 6, 5},        /* 25 */
    {0, 1, 2, 3, 4, 5, 6, 7}};
static const int HEX_NEWV_N[27] = {1, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 4, 2,
                                   2, 2, 4, 2, 2, 4, 2, 2, 4, 2, 4, 4, 8};
static const int HEX_CHILD[8][8] = {
    {0, 8, 12, 11, 15, 16, 26, 24}, {1, 9, 12, 8, 13, 19, 26, 16},
    {2, 10, 12, 9, 17, 22, 26, 19}, {3, 11, 12, 10, 20, 24, 26, 22},
    {4, 23, 25, 14, 15, 24, 26, 16}, {5, 14, 25, 18, 13, 16, 26, 19},
    {6, 18, 25, 21, 17, 19, 26, 22}, {7, 21, 25, 23, 20, 22, 26, 24}};

/* joints: 2D edges (j, j+1), 3D faces (Hexahedron shape descriptor) */
static const int HEX_FACE[6][4] = {{0, 1, 2, 3}, {0, 4, 5, 1}, {1, 5, 6, 2},
                                   {2, 6, 7, 3}, {0, 3, 7, 4}, {4, 7, 6, 5}};

typedef struct {
  int ncells, nloc, ndof, nactive, nnz, nv;
  double *verts;    /* ncells*nv*dim */
  int *gdof;        /* ncells*nloc */
  int *row_ptr, *col;
  double *val, *rhs, *sol, *diag;
  /* multigrid work vectors */
  double *mg_rhs, *mg_sol, *mg_def;
  double *lu;       /* dense LU of the coarse matrix (coarsest level only) */
  int *piv;
  int lu_gen;       /* assembly generation the LU belongs to */
  /* time-dependent problem: stiffness, mass, rhs of this and the last step */
  double *tA, *tM, *tf, *tfold;
  double *tu2;      /* BDF2: solution of the step before the last (finest level) */
} level_t;

struct orc_problem {
  orc_config cfg;
  int shape;        /* 0 quadrilateral, 1 hexahedron, 2 tetrahedron */
  int from_arrays;  /* levels supplied by the caller */
  int nlev;
  level_t *lev;
  quad_rule qr;
  int nqp1;
  int asm_gen;      /* incremented by every orc_assemble */
  int tcd;          /* assembling for the time-dependent problem */
  double ttau;      /* THETA1 * CURRENTTIMESTEPLENGTH (Crank-Nicolson: tau/2) */
  double tau, theta1; /* CURRENTTIMESTEPLENGTH and THETA1 (SDFEM types 9-11) */
  int tcd_step;     /* TimeDiscretization::current_step_ */
  /* coefficients supplied per (cell, quadrature point) by the caller, the
   * reference's CoeffFct contract; NULL: the example's coefficients */
  const double *coef_in;
};

static int nverts(int dim) { return dim == 2 ? 4 : 8; }

static double *refine_mesh(int dim, int nref, int *ncells_out) {
  int nv = nverts(dim);
  int nc = 1;
  double *v = (double *)malloc(sizeof(double) * nv * dim);
  if (dim == 2) {
    const double sq[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
    memcpy(v, sq, sizeof sq);
  } else {
    const double cu[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                             {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    memcpy(v, cu, sizeof cu);
  }
  for (int r = 0; r < nref; ++r) {
    int nch = dim == 2 ? 4 : 8;
    double *nvv = (double *)malloc(sizeof(double) * nc * nch * nv * dim);
    for (int c = 0; c < nc; ++c) {
      const double *pv = v + (size_t)c * nv * dim;
      double newv[27][3];
      int nnew = dim == 2 ? 9 : 27;
      for (int k = 0; k < nnew; ++k) {
        int n = dim == 2 ? QUAD_NEWV_N[k] : HEX_NEWV_N[k];
        for (int a = 0; a < dim; ++a) {
          double s = 0;
          for (int m = 0; m < n; ++m)
            s += pv[(dim == 2 ? QUAD_NEWV[k][m] : HEX_NEWV[k][m]) * dim + a];
          newv[k][a] = s / n;
        }
      }
      for (int ch = 0; ch < nch; ++ch) {
        double *cv = nvv + ((size_t)c * nch + ch) * nv * dim;
        for (int m = 0; m < nv; ++m) {
          int id = dim == 2 ? QUAD_CHILD[ch][m] : HEX_CHILD[ch][m];
          for (int a = 0; a < dim; ++a) cv[m * dim + a] = newv[id][a];
        }
      }
    }
    free(v);
    v = nvv;
    nc *= nch;
  }
  *ncells_out = nc;
  return v;
}

/* affine reference map of a cell: x = x0 + J xi (QuadAffin / HexaAffin) */
typedef struct {
  double x0[3], J[3][3], Jinv[3][3], det;
} affine_t;

static void cell_affine(int dim, const double *cv, affine_t *A) {
  /* xi along v0->v1, eta along v0->v3, zeta along v0->v4 */
  const int e[3] = {1, 3, 4};
  for (int r = 0; r < dim; ++r) {
    for (int a = 0; a < dim; ++a)
      A->J[r][a] = (cv[e[a] * dim + r] - cv[0 * dim + r]) * 0.5;
  }
  for (int r = 0; r < dim; ++r) {
    double s = cv[r];
    for (int a = 0; a < dim; ++a) s += A->J[r][a];
    A->x0[r] = s;
  }
  if (dim == 2) {
    double a = A->J[0][0], b = A->J[0][1], c = A->J[1][0], d = A->J[1][1];
    A->det = a * d - b * c;
    A->Jinv[0][0] = d / A->det; A->Jinv[0][1] = -b / A->det;
    A->Jinv[1][0] = -c / A->det; A->Jinv[1][1] = a / A->det;
  } else {
    double(*J)[3] = A->J;
    double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                 J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                 J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    A->det = det;
    A->Jinv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
    A->Jinv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    A->Jinv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    A->Jinv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
    A->Jinv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    A->Jinv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    A->Jinv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
    A->Jinv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    A->Jinv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  }
}

static void affine_map(int dim, const affine_t *A, const double *xi,
                       double *x) {
  for (int r = 0; r < dim; ++r) {
    double s = A->x0[r];
    for (int a = 0; a < dim; ++a) s += A->J[r][a] * xi[a];
    x[r] = s;
  }
}

/* cell measure hK (BaseCell.C:102-131) */
static double cell_hK(int dim, const double *cv, int measure) {
  if (dim == 2) {
    if (measure == 2) {
      double dx1 = cv[0] - cv[2], dy1 = cv[1] - cv[3];
      double dx2 = cv[2] - cv[4], dy2 = cv[3] - cv[5];
      double l1 = dx1 * dx1 + dy1 * dy1, l2 = dx2 * dx2 + dy2 * dy2;
      return l1 < l2 ? sqrt(l1) : sqrt(l2);
    }
    if (measure == 1 || measure == 3) {
      affine_t A;
      cell_affine(2, cv, &A);
      return sqrt(fabs(4 * A.det));
    }
    double dx = cv[0] - cv[4], dy = cv[1] - cv[5];
    return sqrt(dx * dx + dy * dy);
  }
  if (measure == 2) {
    const int pr[3][2] = {{0, 4}, {0, 1}, {0, 3}};
    double m = 1e10;
    for (int k = 0; k < 3; ++k) {
      double s = 0;
      for (int a = 0; a < 3; ++a) {
        double dd = cv[pr[k][0] * 3 + a] - cv[pr[k][1] * 3 + a];
        s += dd * dd;
      }
      if (s < m) m = s;
    }
    return sqrt(m);
  }
  if (measure == 1 || measure == 3) {
    affine_t A;
    cell_affine(3, cv, &A);
    return sqrt(fabs(8 * A.det));
  }
  const int pr[4][2] = {{0, 6}, {1, 7}, {2, 4}, {3, 5}};
  double m = 0;
  for (int k = 0; k < 4; ++k) {
    double s = 0;
    for (int a = 0; a < 3; ++a) {
      double dd = cv[pr[k][0] * 3 + a] - cv[pr[k][1] * 3 + a];
      s += dd * dd;
    }
    if (s > m) m = s;
  }
  return sqrt(m);
}

/* ------------------------------------------------------------------------ */
/* examples: coefficients, exact solution, boundary data                      */
/* ------------------------------------------------------------------------ */
/* exact solution: u[0]=value, u[1..dim]=gradient, u[dim+1]=laplacian,
 * u[dim+2]=time derivative */
static void exact_sol(const orc_config *c, const double *x, double *u) {
  int d = c->dim;
  for (int k = 0; k < 6; ++k) u[k] = 0;
  switch (c->example) {
  case ORC_EX_SINE_LAPLACE:
  case ORC_EX_SINE: {
    double k = c->example == ORC_EX_SINE_LAPLACE ? M_PI : c->freq * M_PI;
    double s[3], co[3];
    for (int a = 0; a < d; ++a) {
      s[a] = sin(k * x[a]);
      co[a] = cos(k * x[a]);
    }
    if (d == 2) {
      u[0] = s[0] * s[1];
      u[1] = k * co[0] * s[1];
      u[2] = k * s[0] * co[1];
      u[3] = -2 * k * k * s[0] * s[1];
    } else {
      u[0] = s[0] * s[1] * s[2];
      u[1] = k * co[0] * s[1] * s[2];
      u[2] = k * s[0] * co[1] * s[2];
      u[3] = k * s[0] * s[1] * co[2];
      u[4] = -3 * k * k * s[0] * s[1] * s[2];
    }
    break;
  }
  case ORC_EX_POLYEXP: {
    /* u = p(x) q(y) q(z), p = x(1-x)e^x, q = y(1-y) */
    double ex = exp(x[0]);
    double p = x[0] * (1 - x[0]) * ex;
    double p1 = ex * (1 - x[0] - x[0] * x[0]);
    double p2 = -ex * x[0] * (3 + x[0]);
    double qy = x[1] * (1 - x[1]), qz = x[2] * (1 - x[2]);
    double qy1 = 1 - 2 * x[1], qz1 = 1 - 2 * x[2];
    u[0] = p * qy * qz;
    u[1] = p1 * qy * qz;
    u[2] = p * qy1 * qz;
    u[3] = p * qy * qz1;
    u[4] = p2 * qy * qz - 2 * p * qz - 2 * p * qy;
    break;
  }
  case ORC_EX_EXP_SIN: {
    /* u = e^{sin 2 pi t} prod sin(2 pi x_a): include/Examples/TCD_2D/exp.h
       (exp_sin_cos, src/Examples/Example_TimeCD2D.C:12-15) */
    double w = 2 * M_PI, e = exp(sin(w * c->t)), s[3] = {0, 0, 0}, co[3] = {0, 0, 0};
    for (int a = 0; a < d; ++a) {
      s[a] = sin(w * x[a]);
      co[a] = cos(w * x[a]);
    }
    double p = d == 2 ? s[0] * s[1] : s[0] * s[1] * s[2];
    u[0] = e * p;
    u[1] = e * w * co[0] * s[1] * (d == 3 ? s[2] : 1.0);
    u[2] = e * w * s[0] * co[1] * (d == 3 ? s[2] : 1.0);
    if (d == 3) u[3] = e * w * s[0] * s[1] * co[2];
    u[d + 1] = -d * w * w * e * p;
    u[d + 2] = w * cos(w * c->t) * e * p;
    break;
  }
  case ORC_EX_LINEAR_ST: {
    /* include/Examples/TCD_3D/linear_space_time.h (TCD_2D: z = 0) */
    double z = d == 3 ? x[2] : 0.0;
    u[0] = 1 + 2 * x[0] + 3 * c->t * x[1] + 4 * c->t * z;
    u[1] = 2;
    u[2] = 3 * c->t;
    if (d == 3) u[3] = 4 * c->t;
    u[d + 2] = 3 * x[1] + 4 * z;
    break;
  }
  case ORC_EX_QUAD_ST: {
    /* include/Examples/TCD_3D/quadratic_space_time.h */
    double z = d == 3 ? x[2] : 0.0, t2 = c->t * c->t, q = x[0] * x[0] + x[1] * z;
    u[0] = t2 * q;
    u[1] = 2 * x[0] * t2;
    u[2] = z * t2;
    if (d == 3) u[3] = x[1] * t2;
    u[d + 1] = 2 * t2;
    u[d + 2] = 2 * c->t * q;
    break;
  }
  case ORC_EX_POLY1:
  case ORC_EX_POLY1_T: {
    double sc = c->example == ORC_EX_POLY1_T ? 1 + c->t : 1.0;
    double q = 1 + x[0] + 2 * x[1] + (d == 3 ? 3 * x[2] : 0);
    u[0] = sc * q;
    u[1] = sc;
    u[2] = 2 * sc;
    if (d == 3) u[3] = 3 * sc;
    if (c->example == ORC_EX_POLY1_T) u[d + 2] = q;
    break;
  }
  default:
    break;
  }
}

/* convection at x: constant part plus the gradient times x */
static void b_at(const orc_config *c, const double *x, double *bx) {
  for (int i = 0; i < 3; ++i) {
    double s = i < c->dim ? c->b[i] : 0.0;
    for (int j = 0; j < c->dim; ++j) s += c->b_grad[3 * i + j] * x[j];
    bx[i] = i < c->dim ? s : 0.0;
  }
}

/* coefficients at a point: co[0]=eps, co[1..d]=b, co[d+1]=c, co[d+2]=f,
 * co[d+3] = |b|_inf (ConvDiff.C:1858-1863, 1970-1976 coefficient layout) */
static void coeffs_at(const orc_config *c, const double *x, double *co) {
  int d = c->dim;
  double bx[3];
  b_at(c, x, bx);
  co[0] = c->eps;
  double binf = 0;
  for (int a = 0; a < d; ++a) {
    co[1 + a] = bx[a];
    if (fabs(bx[a]) > binf) binf = fabs(bx[a]);
  }
  co[d + 1] = c->c;
  if (c->example == ORC_EX_CONST_F) {
    co[d + 2] = 1.0;
  } else if (c->example == ORC_EX_BUMP) {
    co[d + 2] = 0.0;
  } else {
    double u[6];
    exact_sol(c, x, u);
    /* f = u_t - eps lap u + b.grad u + c u, with the reference's summation
     * order (SineLaplace.h BilinearCoeffs) */
    double f = -c->eps * u[d + 1];
    for (int a = 0; a < d; ++a) f += bx[a] * u[1 + a];
    f += c->c * u[0];
    f += u[d + 2];
    co[d + 2] = f;
  }
  co[d + 3] = binf;
}

static double initial_value(const orc_config *c, const double *x) {
  if (c->example == ORC_EX_BUMP) {
    double r2 = 0;
    for (int a = 0; a < c->dim; ++a) r2 += (x[a] - c->ic[a]) * (x[a] - c->ic[a]);
    return exp(-r2 / (2 * c->ic[3] * c->ic[3]));
  }
  double u[6];
  exact_sol(c, x, u);
  return u[0];
}

/* boundary component of a boundary joint centre (2D: SineLaplace transform,
 * comps 0:y=0, 1:x=1, 2:y=1, 3:x=0; 3D: 0:z=0 1:y=0 2:x=1 3:y=1 4:x=0 5:z=1) */
static int boundary_comp(int dim, const double *x) {
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
static int bc_type(const orc_config *c, int comp) {
  return (c->neumann_mask >> comp) & 1; /* 0 DIRICHLET, 1 NEUMANN */
}

/* ------------------------------------------------------------------------ */
/* FE space: DOF numbering by the reference's marker algorithm               */
/* ------------------------------------------------------------------------ */
#define FIRSTMARK (-10)
#define N_BC_TYPES 7

static int find_root(const int *gn, int w) {
  int v;
  while ((v = gn[w]) > -1) w = v;
  return w;
}

/* FEMapper::map_single_dof (FEMapper.C:456-545) */
static int map_single_dof(int *gn, int dof0, int dof1, int *counter) {
  int w0 = find_root(gn, dof0), w1 = find_root(gn, dof1);
  if (gn[dof0] == -1 && gn[dof1] == -1) {
    (*counter)--;
    if (dof0 < dof1) {
      gn[dof0] = *counter;
      gn[dof1] = dof0;
    } else {
      gn[dof1] = *counter;
      gn[dof0] = dof1;
    }
  } else if (gn[dof0] == -1) {
    if (w1 > dof0) {
      gn[dof0] = gn[w1];
      gn[dof1] = dof0;
      gn[w1] = dof0;
    } else {
      gn[dof0] = w1;
    }
  } else if (gn[dof1] == -1) {
    if (w0 > dof1) {
      gn[dof1] = gn[w0];
      gn[dof0] = dof1;
      gn[w0] = dof1;
    } else {
      gn[dof1] = w0;
    }
  } else if (gn[w0] != gn[w1]) {
    int e = gn[w0] > gn[w1] ? gn[w0] : gn[w1];
    int w = w0 < w1 ? w0 : w1;
    gn[w0] = w;
    gn[w1] = w;
    gn[w] = e;
  } else if (w0 != w1) {
    FAIL("map_single_dof: inconsistent identification");
  }
  if (gn[dof0] >= dof0 || gn[w0] >= w0 || gn[dof1] >= dof1 || gn[w1] >= w1)
    FAIL("map_single_dof: link to a later entry");
  return 0;
}

/* FEMapper::map_single_boundary_dof (FEMapper.C:555-600), no hanging nodes */
static void map_single_boundary_dof(int *gn, int dof, int *bcounter) {
  int w = find_root(gn, dof);
  if (gn[w] == -1) {
    (*bcounter)--;
    gn[dof] = *bcounter;
  } else if (gn[w] < *bcounter) {
    (*bcounter)--;
    gn[w] = *bcounter;
    if (dof != w) gn[dof] = w;
  }
}

/* local DOFs of a cell lying on joint j, in joint order */
static int joint_dofs(int dim, int p, int j, int *idx) {
  int nloc = dim == 2 ? (p + 1) * (p + 1) : (p + 1) * (p + 1) * (p + 1);
  /* fixed ref coordinate of joint j */
  int axis, side;
  if (dim == 2) {
    static const int ax[4] = {1, 0, 1, 0}, sd[4] = {-1, 1, 1, -1};
    axis = ax[j];
    side = sd[j];
  } else {
    static const int ax[6] = {2, 1, 0, 1, 0, 2}, sd[6] = {-1, -1, 1, 1, -1, 1};
    axis = ax[j];
    side = sd[j];
  }
  int n = 0;
  for (int k = 0; k < nloc; ++k) {
    double r[3];
    local_dof_ref(dim, p, k, r);
    if (r[axis] == side) idx[n++] = k;
  }
  return n;
}

static long lattice_key(int dim, const double *x, double scale, long n1) {
  long k = 0;
  for (int a = dim - 1; a >= 0; --a) k = k * n1 + lround(x[a] * scale);
  return k;
}

static void dof_position(int dim, int p, const double *cv, int k, double *x) {
  affine_t A;
  cell_affine(dim, cv, &A);
  double r[3];
  local_dof_ref(dim, p, k, r);
  affine_map(dim, &A, r, x);
}

/* shape-aware cell helpers (shape 2: tetrahedron; TetraAffin.C:235-265:
 * x = v0 + (v1-v0) xi + (v2-v0) eta + (v3-v0) zeta) */
static void cell_affine_s(int shape, int dim, const double *cv, affine_t *A) {
  if (shape != 2) {
    cell_affine(dim, cv, A);
    return;
  }
  for (int r = 0; r < 3; ++r) {
    A->x0[r] = cv[r];
    for (int a = 0; a < 3; ++a) A->J[r][a] = cv[(a + 1) * 3 + r] - cv[r];
  }
  double(*J)[3] = A->J;
  double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
               J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
               J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  A->det = det;
  A->Jinv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
  A->Jinv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
  A->Jinv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
  A->Jinv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
  A->Jinv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
  A->Jinv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
  A->Jinv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
  A->Jinv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
  A->Jinv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
}

/* TQuadrangle::CheckQuad (Quadrangle.C:119-128) and THexahedron::CheckHexa
 * (Hexahedron.C:196-235): 1 when a quadrilateral is not a parallelogram (a
 * hexahedron not a parallelepiped, "Brick"); the reference maps those cells
 * by TQuadBilinear / THexaTrilinear (FESpace.C:83-84 picks the _M elements
 * for them) and the others affinely */
static int cell_is_multilinear(int shape, int dim, const double *cv) {
  if (shape == 2) return 0;
  if (dim == 2) {
    double t1 = cv[0] - cv[2] + cv[4] - cv[6];
    double t2 = cv[1] - cv[3] + cv[5] - cv[7];
    return fabs(t1) > 1e-8 || fabs(t2) > 1e-8;
  }
  for (int a = 0; a < 3; ++a) {
#define X(i) cv[3 * (i) + a]
    double t1 = fabs(X(0) - X(1) - X(3) + X(2) + X(4) - X(5) - X(7) + X(6));
    double t2 = fabs(X(0) - X(1) + X(3) - X(2) - X(4) + X(5) - X(7) + X(6));
    double t3 = fabs(X(0) + X(1) - X(3) - X(2) - X(4) - X(5) + X(7) + X(6));
    double t4 = fabs(-X(0) + X(1) + X(3) - X(2) + X(4) - X(5) - X(7) + X(6));
#undef X
    if (t1 + t2 + t3 + t4 >= 1e-8) return 1;
  }
  return 0;
}

/* the bilinear / trilinear map at a reference point (TQuadBilinear::SetCell,
 * QuadBilinear.C:243-263, GetOrigValues :87-129; THexaTrilinear::SetCell,
 * HexaTrilinear.C:225-270, GetOrigValues): x(xi), J = dx/dxi, its inverse
 * and determinant in the affine_t layout; c[r][k] the map's coefficients */
static void multilinear_coeffs(int dim, const double *cv, double c[3][8]) {
  for (int r = 0; r < dim; ++r) {
    if (dim == 2) {
      double v0 = cv[r], v1 = cv[2 + r], v2 = cv[4 + r], v3 = cv[6 + r];
      c[r][0] = (v0 + v1 + v2 + v3) * 0.25;
      c[r][1] = (-v0 + v1 + v2 - v3) * 0.25;
      c[r][2] = (-v0 - v1 + v2 + v3) * 0.25;
      c[r][3] = (v0 - v1 + v2 - v3) * 0.25;
    } else {
      double v[8];
      for (int i = 0; i < 8; ++i) v[i] = cv[3 * i + r];
      c[r][0] = (v[0] + v[1] + v[3] + v[2] + v[4] + v[5] + v[7] + v[6]) * 0.125;
      c[r][1] = (-v[0] + v[1] - v[3] + v[2] - v[4] + v[5] - v[7] + v[6]) * 0.125;
      c[r][2] = (-v[0] - v[1] + v[3] + v[2] - v[4] - v[5] + v[7] + v[6]) * 0.125;
      c[r][3] = (-v[0] - v[1] - v[3] - v[2] + v[4] + v[5] + v[7] + v[6]) * 0.125;
      c[r][4] = (v[0] - v[1] - v[3] + v[2] + v[4] - v[5] - v[7] + v[6]) * 0.125;
      c[r][5] = (v[0] - v[1] + v[3] - v[2] - v[4] + v[5] - v[7] + v[6]) * 0.125;
      c[r][6] = (v[0] + v[1] - v[3] - v[2] - v[4] - v[5] + v[7] + v[6]) * 0.125;
      c[r][7] = (-v[0] + v[1] + v[3] - v[2] + v[4] - v[5] - v[7] + v[6]) * 0.125;
    }
  }
}

static void multilinear_at(int dim, const double *cv, const double *xi, affine_t *P) {
  double c[3][8];
  multilinear_coeffs(dim, cv, c);
  double (*J)[3] = P->J;
  if (dim == 2) {
    double s = xi[0], t = xi[1];
    for (int r = 0; r < 2; ++r) {
      P->x0[r] = c[r][0] + c[r][1] * s + c[r][2] * t + c[r][3] * s * t;
      J[r][0] = c[r][1] + c[r][3] * t;
      J[r][1] = c[r][2] + c[r][3] * s;
    }
    P->det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    P->Jinv[0][0] = J[1][1] / P->det; P->Jinv[0][1] = -J[0][1] / P->det;
    P->Jinv[1][0] = -J[1][0] / P->det; P->Jinv[1][1] = J[0][0] / P->det;
    return;
  }
  double s = xi[0], t = xi[1], u = xi[2];
  for (int r = 0; r < 3; ++r) {
    P->x0[r] = c[r][0] + c[r][1] * s + c[r][2] * t + c[r][3] * u + c[r][4] * s * t +
               c[r][5] * s * u + c[r][6] * t * u + c[r][7] * s * t * u;
    J[r][0] = c[r][1] + c[r][4] * t + c[r][5] * u + c[r][7] * t * u;
    J[r][1] = c[r][2] + c[r][4] * s + c[r][6] * u + c[r][7] * s * u;
    J[r][2] = c[r][3] + c[r][5] * s + c[r][6] * t + c[r][7] * s * t;
  }
  double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
               J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
               J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  P->det = det;
  P->Jinv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
  P->Jinv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
  P->Jinv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
  P->Jinv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
  P->Jinv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
  P->Jinv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
  P->Jinv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
  P->Jinv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
  P->Jinv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
}

/* second derivatives through the bilinear map
 * (TQuadBilinear::GetOrigAllDerivatives, QuadBilinear.C:131-205): the 5 x 5
 * matrix G taking (u_x, u_y, u_xx, u_xy, u_yy) to (u_xi, u_eta, u_xixi,
 * u_xieta, u_etaeta) is inverted by Gaussian elimination with partial pivoting
 * (SolveMultipleSystemsNew solves G X = I the same way); lw = rows 2 + 4 of
 * G^-1: the Laplacian of a function from its reference derivatives */
static void bilinear_lap_weights(const double *cv, const double *xi, double *lw) {
  double c[3][8];
  multilinear_coeffs(2, cv, c);
  double s = xi[0], t = xi[1];
  double xx = c[0][1] + c[0][3] * t, yx = c[1][1] + c[1][3] * t;
  double xe = c[0][2] + c[0][3] * s, ye = c[1][2] + c[1][3] * s;
  double G[5][10] = {{xx, yx, 0, 0, 0}, {xe, ye, 0, 0, 0},
                     {0, 0, xx * xx, 2 * xx * yx, yx * yx},
                     {c[0][3], c[1][3], xx * xe, yx * xe + xx * ye, yx * ye},
                     {0, 0, xe * xe, 2 * xe * ye, ye * ye}};
  for (int i = 0; i < 5; ++i) G[i][5 + i] = 1.0;
  for (int col = 0; col < 5; ++col) {
    int pr = col;
    for (int i = col + 1; i < 5; ++i)
      if (fabs(G[i][col]) > fabs(G[pr][col])) pr = i;
    if (pr != col)
      for (int j = 0; j < 10; ++j) {
        double tmp = G[col][j];
        G[col][j] = G[pr][j];
        G[pr][j] = tmp;
      }
    double inv = 1.0 / G[col][col];
    for (int j = 0; j < 10; ++j) G[col][j] *= inv;
    for (int i = 0; i < 5; ++i) {
      if (i == col) continue;
      double f = G[i][col];
      if (f != 0.0)
        for (int j = 0; j < 10; ++j) G[i][j] -= f * G[col][j];
    }
  }
  for (int k = 0; k < 5; ++k) lw[k] = G[2][5 + k] + G[4][5 + k];
}

/* TQuadrangle::GetMeasure (Quadrangle.C:102-117): two triangles */
static double quad_measure(const double *cv) {
  double x1 = cv[0], y1 = cv[1], x2 = cv[2], y2 = cv[3], x3 = cv[4], y3 = cv[5], x4 = cv[6],
         y4 = cv[7];
  return 0.5 * fabs(x2 * y3 - x3 * y2 - x1 * y3 + x3 * y1 + x1 * y2 - x2 * y1) +
         0.5 * fabs(x4 * y3 - x3 * y4 - x1 * y3 + x3 * y1 + x1 * y4 - x4 * y1);
}

/* Tetrahedron.C:64-113 (diameter = longest edge, shortest edge) */
static double cell_hK_s(int shape, int dim, const double *cv, int measure) {
  if (shape != 2 && dim == 2 && (measure == 1 || measure == 3) &&
      cell_is_multilinear(shape, dim, cv))
    return sqrt(quad_measure(cv));
  if (shape != 2) return cell_hK(dim, cv, measure);
  if (measure == 1 || measure == 3) {
    affine_t A;
    cell_affine_s(2, 3, cv, &A);
    return sqrt(fabs(A.det) / 6.0);
  }
  double m = measure == 2 ? 1e10 : 0.0;
  for (int i = 0; i < 4; ++i)
    for (int j = i + 1; j < 4; ++j) {
      double s2 = 0;
      for (int a = 0; a < 3; ++a) {
        double dd = cv[i * 3 + a] - cv[j * 3 + a];
        s2 += dd * dd;
      }
      if (measure == 2 ? s2 < m : s2 > m) m = s2;
    }
  return sqrt(m);
}

static void basis_s(int shape, int dim, int p, const double *xi, double out[][NDER]) {
  if (shape == 2)
    tet_basis(p, xi, out);
  else
    ref_basis(dim, p, xi, out);
}

static void local_dof_ref_s(int shape, int dim, int p, int k, double *r) {
  if (shape == 2) {
    const double *q = p == 1 ? TET_P1_NODES[k] : TET_P2_NODES[k];
    r[0] = q[0];
    r[1] = q[1];
    r[2] = q[2];
    return;
  }
  local_dof_ref(dim, p, k, r);
}

static void dof_position_s(int shape, int dim, int p, const double *cv, int k, double *x) {
  affine_t A;
  cell_affine_s(shape, dim, cv, &A);
  double r[3];
  local_dof_ref_s(shape, dim, p, k, r);
  affine_map(dim, &A, r, x);
}

static int nloc_of(int shape, int dim, int p) {
  if (shape == 2) return p == 1 ? 4 : 10;
  return dim == 2 ? (p + 1) * (p + 1) : (p + 1) * (p + 1) * (p + 1);
}

/* compute_various_numbers (FESpace.C:1863-2099), no hanging nodes: the
 * marks left by the cell loop become the global numbers (inner classes,
 * then each boundary-condition type, then Dirichlet, each in the order of
 * its first local DOF); gn is taken over by L */
static int number_classes(int *gn, int sumlocdof, const int *bub, level_t *L) {
  int total_bub = 0;
  for (int i = 0; i < N_BC_TYPES; ++i) total_bub += bub[i];
  int boundmark[N_BC_TYPES];
  int l = FIRSTMARK;
  for (int i = 0; i < N_BC_TYPES; ++i) {
    l -= bub[i];
    boundmark[i] = l;
  }
  int innermark = l;
  int slavemark = l - sumlocdof;
  int dirichlet_counter = 0;
  int boundcounter[N_BC_TYPES];
  l = 0;
  for (int i = 0; i < N_BC_TYPES; ++i) {
    l += bub[i];
    boundcounter[i] = l;
  }
  int count = l;
  int n_dirichlet = 0, n_inner = 0, n_bound[N_BC_TYPES] = {0};
  for (int i = 0; i < sumlocdof; ++i) {
    int v = gn[i];
    if (v < -1) {
      if (v <= slavemark) FAIL("hanging node in a conforming mesh");
      if (v <= innermark) {
        gn[i] = count++;
        n_inner++;
        continue;
      }
      int m = N_BC_TYPES - 1;
      for (; m >= 0; m--) {
        if (v <= boundmark[m]) {
          gn[i] = boundcounter[m]++;
          n_bound[m]++;
          m = -2;
          break;
        }
      }
      if (m != -2 && v <= FIRSTMARK) {
        gn[i] = dirichlet_counter++;
        n_dirichlet++;
      }
    } else if (v >= 0) {
      gn[i] = gn[v];
    } else {
      FAIL("unhandled local dof");
    }
  }
  int nb = 0;
  for (int i = 0; i < N_BC_TYPES; ++i) nb += n_bound[i];
  int dirichlet_offset = n_inner + nb;
  int inner_offset = -total_bub;
  int boundoffset[N_BC_TYPES];
  l = n_inner;
  for (int i = 0, m = 0; i < N_BC_TYPES; ++i) {
    m += bub[i];
    boundoffset[i] = l - m;
    l += n_bound[i];
  }
  int dirichletmark = bub[0];
  l = bub[0];
  for (int i = 0; i < N_BC_TYPES - 1; ++i) {
    l += bub[i + 1];
    boundmark[i] = l;
  }
  boundmark[N_BC_TYPES - 1] = l;
  for (int i = 0; i < sumlocdof; ++i) {
    int v = gn[i];
    if (v < dirichletmark) {
      gn[i] += dirichlet_offset;
    } else if (v < boundmark[N_BC_TYPES - 1]) {
      for (int m = 0; m < N_BC_TYPES; ++m)
        if (v < boundmark[m]) {
          gn[i] += boundoffset[m];
          break;
        }
    } else {
      gn[i] += inner_offset;
    }
  }
  L->gdof = gn;
  L->nactive = n_inner + nb;
  L->ndof = n_inner + nb + n_dirichlet;
  return 0;
}

static int build_space(const orc_config *cfg, level_t *L, int nref) {
  int dim = cfg->dim, p = cfg->order, nv = L->nv;
  int nj = dim == 2 ? 4 : 6;
  int nc = L->ncells, nloc = L->nloc;
  long N = 1L << nref;
  /* joint centre lattice (resolution 2N) -> (cell, joint) of first owner */
  long jn1 = 2 * N + 1;
  long jsize = dim == 2 ? jn1 * jn1 : jn1 * jn1 * jn1;
  int *jowner = (int *)malloc(sizeof(int) * jsize);
  for (long i = 0; i < jsize; ++i) jowner[i] = -1;
  int *neigh = (int *)malloc(sizeof(int) * nc * nj);   /* neighbour cell */
  int *bcomp = (int *)malloc(sizeof(int) * nc * nj);   /* boundary comp */
  for (int c = 0; c < nc; ++c) {
    const double *cv = L->verts + (size_t)c * nv * dim;
    for (int j = 0; j < nj; ++j) {
      double ctr[3] = {0, 0, 0};
      int nvj = dim == 2 ? 2 : 4;
      for (int m = 0; m < nvj; ++m) {
        int vid = dim == 2 ? (m == 0 ? j : (j + 1) % 4) : HEX_FACE[j][m];
        for (int a = 0; a < dim; ++a) ctr[a] += cv[vid * dim + a] / nvj;
      }
      bcomp[c * nj + j] = boundary_comp(dim, ctr);
      long key = lattice_key(dim, ctr, 2.0 * N, jn1);
      neigh[c * nj + j] = -1;
      if (bcomp[c * nj + j] < 0) {
        if (jowner[key] < 0) {
          jowner[key] = c * nj + j;
        } else {
          int o = jowner[key];
          neigh[c * nj + j] = o / nj;
          neigh[o] = c;
        }
      }
    }
  }
  free(jowner);

  /* find_boundary_upper_bounds (FESpace2D.C:58-81) */
  int jd[MAXLOC];
  int njd = joint_dofs(dim, p, 0, jd);
  int bub[N_BC_TYPES] = {0};
  for (int c = 0; c < nc; ++c)
    for (int j = 0; j < nj; ++j)
      if (bcomp[c * nj + j] >= 0) bub[bc_type(cfg, bcomp[c * nj + j])] += njd;

  int counters[N_BC_TYPES + 1];
  counters[0] = FIRSTMARK + 1;
  for (int i = 0; i < N_BC_TYPES; ++i) counters[i + 1] = counters[i] - bub[i];
  int *counter = &counters[N_BC_TYPES];

  int *gn = (int *)malloc(sizeof(int) * nc * nloc);
  for (int i = 0; i < nc * nloc; ++i) gn[i] = -1;

  /* ConstructSpace cell loop (FESpace2D.C:118-309) */
  for (int c = 0; c < nc; ++c) {
    const double *cv = L->verts + (size_t)c * nv * dim;
    int I0 = c * nloc;
    for (int j = 0; j < nj; ++j) {
      int idx0[MAXLOC];
      int n0 = joint_dofs(dim, p, j, idx0);
      if (bcomp[c * nj + j] >= 0) {
        int t = bc_type(cfg, bcomp[c * nj + j]);
        for (int m = 0; m < n0; ++m)
          map_single_boundary_dof(gn, I0 + idx0[m], &counters[t]);
      } else {
        int n = neigh[c * nj + j];
        if (n > c) {
          const double *nvv = L->verts + (size_t)n * nv * dim;
          int I1 = n * nloc;
          /* joint of the neighbour: the one whose DOFs coincide */
          for (int m = 0; m < n0; ++m) {
            double x0[3], x1[3];
            dof_position(dim, p, cv, idx0[m], x0);
            int found = -1;
            for (int k = 0; k < nloc && found < 0; ++k) {
              dof_position(dim, p, nvv, k, x1);
              double dd = 0;
              for (int a = 0; a < dim; ++a) dd += fabs(x0[a] - x1[a]);
              if (dd < 1e-12) found = k;
            }
            if (found < 0) FAIL("neighbour DOF not found");
            if (map_single_dof(gn, I0 + idx0[m], I1 + found, counter))
              return -1;
          }
        }
      }
    }
    /* cell-inner DOFs (all ref coords strictly inside) */
    for (int k = 0; k < nloc; ++k) {
      double r[3];
      local_dof_ref(dim, p, k, r);
      int inner = 1;
      for (int a = 0; a < dim; ++a)
        if (r[a] == -1 || r[a] == 1) inner = 0;
      if (inner) {
        (*counter)--;
        gn[I0 + k] = *counter;
      }
    }
  }
  free(neigh);
  free(bcomp);

  return number_classes(gn, nc * nloc, bub, L);
}

/* Tetrahedra: the face-by-face identification of TFESpace3D::ConstructSpace
 * (FESpace3D.C:186-420) on the caller's mesh.  Two cells share a face when
 * the face's three vertex positions coincide (found through a hash of the
 * sorted positions); a face without a neighbour is a boundary face of the
 * unit cube, its component from its centroid; the DOFs of face j are the
 * local DOFs whose barycentric coordinate j vanishes (the JointDOF lists of
 * C_T_P1_3D / C_T_P2_3D, FE_C_T_P2_3D.h); a neighbour's DOF is identified by
 * position.  P1 and P2 tetrahedra have no cell-inner DOFs.  The order in
 * which a face's DOFs are identified does not change the result: the
 * numbers go to the classes in the order of their first local DOF, and a
 * boundary DOF keeps the lowest boundary-condition type it meets. */
static const int TET_FACE_OPP[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};

static void tet_face_key(const double *cv, int j, double *key) {
  double v[3][3];
  for (int m = 0; m < 3; ++m)
    for (int a = 0; a < 3; ++a) v[m][a] = cv[TET_FACE_OPP[j][m] * 3 + a];
  for (int i = 0; i < 2; ++i)
    for (int k = 0; k < 2 - i; ++k) {
      int gt = 0;
      for (int a = 0; a < 3; ++a)
        if (v[k][a] != v[k + 1][a]) {
          gt = v[k][a] > v[k + 1][a];
          break;
        }
      if (gt)
        for (int a = 0; a < 3; ++a) {
          double t = v[k][a];
          v[k][a] = v[k + 1][a];
          v[k + 1][a] = t;
        }
    }
  memcpy(key, v, 9 * sizeof(double));
}

static unsigned long long hash_bytes(const void *p, size_t n) {
  const unsigned char *b = (const unsigned char *)p;
  unsigned long long h = 1469598103934665603ULL;
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 1099511628211ULL;
  }
  return h;
}

static int build_space_tet(const orc_config *cfg, level_t *L) {
  const int p = cfg->order, nc = L->ncells, nloc = L->nloc;
  int fd[4][MAXLOC], nfd = 0;
  for (int j = 0; j < 4; ++j) {
    int cnt = 0;
    for (int k = 0; k < nloc; ++k) {
      double r[3];
      local_dof_ref_s(2, 3, p, k, r);
      const double lam[4] = {1.0 - r[0] - r[1] - r[2], r[0], r[1], r[2]};
      if (fabs(lam[j]) < 1e-14) fd[j][cnt++] = k;
    }
    nfd = cnt;
  }
  const size_t nf = (size_t)nc * 4;
  size_t cap = 1;
  while (cap < 2 * nf) cap <<= 1;
  int *tab = (int *)malloc(sizeof(int) * cap);
  int *neigh = (int *)malloc(sizeof(int) * nf);
  int *bcomp = (int *)malloc(sizeof(int) * nf);
  for (size_t i = 0; i < cap; ++i) tab[i] = -1;
  double key[9], key2[9];
  for (int c = 0; c < nc; ++c)
    for (int j = 0; j < 4; ++j) {
      const int f = c * 4 + j;
      neigh[f] = -1;
      bcomp[f] = -1;
      tet_face_key(L->verts + (size_t)c * 12, j, key);
      size_t h = (size_t)(hash_bytes(key, sizeof key) & (cap - 1));
      while (tab[h] >= 0) {
        const int g = tab[h];
        tet_face_key(L->verts + (size_t)(g / 4) * 12, g % 4, key2);
        if (memcmp(key, key2, sizeof key) == 0) break;
        h = (h + 1) & (cap - 1);
      }
      if (tab[h] < 0) {
        tab[h] = f;
      } else {
        const int g = tab[h];
        if (neigh[g] >= 0) FAIL("a face shared by three cells");
        neigh[g] = c;
        neigh[f] = g / 4;
      }
    }
  free(tab);
  int bub[N_BC_TYPES] = {0};
  for (size_t f = 0; f < nf; ++f) {
    if (neigh[f] >= 0) continue;
    const double *cv = L->verts + (f / 4) * 12;
    double ctr[3] = {0, 0, 0};
    for (int m = 0; m < 3; ++m)
      for (int a = 0; a < 3; ++a) ctr[a] += cv[TET_FACE_OPP[f % 4][m] * 3 + a] / 3.0;
    bcomp[f] = boundary_comp(3, ctr);
    if (bcomp[f] < 0) FAIL("a face without a neighbour inside the cube");
    bub[bc_type(cfg, bcomp[f])] += nfd;
  }
  int counters[N_BC_TYPES + 1];
  counters[0] = FIRSTMARK + 1;
  for (int i = 0; i < N_BC_TYPES; ++i) counters[i + 1] = counters[i] - bub[i];
  int *counter = &counters[N_BC_TYPES];
  int *gn = (int *)malloc(sizeof(int) * nc * nloc);
  for (int i = 0; i < nc * nloc; ++i) gn[i] = -1;
  for (int c = 0; c < nc; ++c) {
    const double *cv = L->verts + (size_t)c * 12;
    const int I0 = c * nloc;
    for (int j = 0; j < 4; ++j) {
      const int f = c * 4 + j;
      if (neigh[f] < 0) {
        const int t = bc_type(cfg, bcomp[f]);
        for (int m = 0; m < nfd; ++m) map_single_boundary_dof(gn, I0 + fd[j][m], &counters[t]);
      } else if (neigh[f] > c) {
        const int n = neigh[f];
        const double *nvv = L->verts + (size_t)n * 12;
        const int I1 = n * nloc;
        for (int m = 0; m < nfd; ++m) {
          double x0[3], x1[3];
          dof_position_s(2, 3, p, cv, fd[j][m], x0);
          int found = -1;
          for (int k = 0; k < nloc && found < 0; ++k) {
            dof_position_s(2, 3, p, nvv, k, x1);
            if (fabs(x0[0] - x1[0]) + fabs(x0[1] - x1[1]) + fabs(x0[2] - x1[2]) < 1e-12)
              found = k;
          }
          if (found < 0) FAIL("neighbour DOF not found");
          if (map_single_dof(gn, I0 + fd[j][m], I1 + found, counter)) return -1;
        }
      }
    }
  }
  free(neigh);
  free(bcomp);
  return number_classes(gn, nc * nloc, bub, L);
}

int orc_marker_numbering(const orc_config *cfg, int ncells, const double *verts, int *gdof,
                         int *ndof, int *nactive) {
  if (!cfg->tetra || cfg->dim != 3 || (cfg->order != 1 && cfg->order != 2) || ncells < 1 ||
      !verts || !gdof || !ndof || !nactive) {
    snprintf(g_err, sizeof g_err,
             "tetrahedral P1/P2 meshes only (orc_create numbers its own hexahedra)");
    return -1;
  }
  level_t L;
  memset(&L, 0, sizeof L);
  L.nv = 4;
  L.nloc = nloc_of(2, 3, cfg->order);
  L.ncells = ncells;
  L.verts = (double *)verts;   /* read only */
  if (build_space_tet(cfg, &L)) return -1;
  memcpy(gdof, L.gdof, sizeof(int) * (size_t)ncells * L.nloc);
  *ndof = L.ndof;
  *nactive = L.nactive;
  free(L.gdof);
  return 0;
}

/* TStructure: union of cell couplings, full rows, sorted columns */
static int cmp_int(const void *a, const void *b) {
  int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}
static int build_structure(level_t *L) {
  int n = L->ndof, nloc = L->nloc;
  int *ub = (int *)calloc(n + 1, sizeof(int));
  for (int c = 0; c < L->ncells; ++c)
    for (int m = 0; m < nloc; ++m) ub[L->gdof[c * nloc + m] + 1] += nloc;
  for (int i = 0; i < n; ++i) ub[i + 1] += ub[i];
  int *tmp = (int *)malloc(sizeof(int) * ub[n]);
  int *fill = (int *)calloc(n, sizeof(int));
  for (int c = 0; c < L->ncells; ++c)
    for (int m = 0; m < nloc; ++m) {
      int r = L->gdof[c * nloc + m];
      for (int k = 0; k < nloc; ++k)
        tmp[ub[r] + fill[r]++] = L->gdof[c * nloc + k];
    }
  L->row_ptr = (int *)malloc(sizeof(int) * (n + 1));
  L->row_ptr[0] = 0;
  int nnz = 0;
  for (int r = 0; r < n; ++r) {
    int *seg = tmp + ub[r];
    qsort(seg, fill[r], sizeof(int), cmp_int);
    int u = 0;
    for (int k = 0; k < fill[r]; ++k)
      if (k == 0 || seg[k] != seg[k - 1]) seg[u++] = seg[k];
    fill[r] = u;
    nnz += u;
    L->row_ptr[r + 1] = nnz;
  }
  L->col = (int *)malloc(sizeof(int) * nnz);
  for (int r = 0; r < n; ++r)
    memcpy(L->col + L->row_ptr[r], tmp + ub[r], sizeof(int) * fill[r]);
  L->nnz = nnz;
  free(tmp);
  free(fill);
  free(ub);
  return 0;
}

orc_problem *orc_create(const orc_config *cfg, int n_levels) {
  if (cfg->dim != 2 && cfg->dim != 3) {
    snprintf(g_err, sizeof g_err, "dim must be 2 or 3");
    return NULL;
  }
  if (cfg->order != 1 && cfg->order != 2) {
    snprintf(g_err, sizeof g_err, "order must be 1 or 2");
    return NULL;
  }
  if (n_levels < 1 || n_levels > cfg->nref + 1) {
    snprintf(g_err, sizeof g_err, "bad number of levels");
    return NULL;
  }
  if (cfg->tetra) {
    snprintf(g_err, sizeof g_err, "tetrahedral levels come from orc_create_from_arrays");
    return NULL;
  }
  orc_problem *p = (orc_problem *)calloc(1, sizeof(orc_problem));
  p->cfg = *cfg;
  p->shape = cfg->dim == 2 ? 0 : 1;
  if (p->cfg.poly_degree <= 0) p->cfg.poly_degree = cfg->order;
  p->nlev = n_levels;
  p->lev = (level_t *)calloc(n_levels, sizeof(level_t));
  int dim = cfg->dim;
  for (int k = 0; k < n_levels; ++k) {
    level_t *L = &p->lev[k];
    L->nv = nverts(dim);
    L->nloc = dim == 2 ? (cfg->order + 1) * (cfg->order + 1)
                       : (cfg->order + 1) * (cfg->order + 1) * (cfg->order + 1);
    L->verts = refine_mesh(dim, cfg->nref - k, &L->ncells);
    if (build_space(&p->cfg, L, cfg->nref - k)) {
      orc_destroy(p);
      return NULL;
    }
    build_structure(L);
    L->val = (double *)calloc(L->nnz, sizeof(double));
    L->rhs = (double *)calloc(L->ndof, sizeof(double));
    L->sol = (double *)calloc(L->ndof, sizeof(double));
    L->diag = (double *)calloc(L->ndof, sizeof(double));
    L->mg_rhs = (double *)calloc(L->ndof, sizeof(double));
    L->mg_sol = (double *)calloc(L->ndof, sizeof(double));
    L->mg_def = (double *)calloc(L->ndof, sizeof(double));
  }
  /* quadrature rule: degree N_terms * p (FEDatabase.C:1553-1556) */
  int nterms = cfg->problem_linear ? 2 : 3;
  p->nqp1 = gauss_points_for_degree(nterms * cfg->order);
  make_rule(dim, p->nqp1, &p->qr);
  return p;
}

void orc_destroy(orc_problem *p) {
  if (!p) return;
  for (int k = 0; k < p->nlev; ++k) {
    level_t *L = &p->lev[k];
    free(L->verts); free(L->gdof); free(L->row_ptr); free(L->col);
    free(L->val); free(L->rhs); free(L->sol); free(L->diag);
    free(L->mg_rhs); free(L->mg_sol); free(L->mg_def);
    free(L->lu); free(L->piv);
    free(L->tA); free(L->tM); free(L->tf); free(L->tfold); free(L->tu2);
  }
  free(p->lev);
  free(p);
}

/* ConvectionDiffusion<d> on the caller's levels: the FE spaces, DOF maps and
 * TStructure patterns are taken as given (FESpace GlobalNumbers,
 * TStructure row_ptr/columns), the cell type from cfg->tetra / cfg->dim */
orc_problem *orc_create_from_arrays(const orc_config *cfg, int n_levels,
                                    const int *ncells, const double *const *verts,
                                    const int *const *gdof, const int *ndof,
                                    const int *nactive, const int *const *row_ptr,
                                    const int *const *col) {
  if (cfg->dim != 2 && cfg->dim != 3) {
    snprintf(g_err, sizeof g_err, "dim must be 2 or 3");
    return NULL;
  }
  if ((cfg->order != 1 && cfg->order != 2) || (cfg->tetra && cfg->dim != 3) ||
      n_levels < 1) {
    snprintf(g_err, sizeof g_err, "bad order, cell type or number of levels");
    return NULL;
  }
  orc_problem *p = (orc_problem *)calloc(1, sizeof(orc_problem));
  p->cfg = *cfg;
  p->shape = cfg->tetra ? 2 : (cfg->dim == 2 ? 0 : 1);
  p->from_arrays = 1;
  if (p->cfg.poly_degree <= 0) p->cfg.poly_degree = cfg->order;
  p->nlev = n_levels;
  p->lev = (level_t *)calloc(n_levels, sizeof(level_t));
  int dim = cfg->dim;
  for (int k = 0; k < n_levels; ++k) {
    level_t *L = &p->lev[k];
    L->nv = p->shape == 2 ? 4 : nverts(dim);
    L->nloc = nloc_of(p->shape, dim, cfg->order);
    L->ncells = ncells[k];
    L->ndof = ndof[k];
    L->nactive = nactive[k];
    L->nnz = row_ptr[k][ndof[k]];
    size_t nvd = (size_t)L->ncells * L->nv * dim, ng = (size_t)L->ncells * L->nloc;
    L->verts = (double *)malloc(sizeof(double) * nvd);
    memcpy(L->verts, verts[k], sizeof(double) * nvd);
    L->gdof = (int *)malloc(sizeof(int) * ng);
    memcpy(L->gdof, gdof[k], sizeof(int) * ng);
    L->row_ptr = (int *)malloc(sizeof(int) * (L->ndof + 1));
    memcpy(L->row_ptr, row_ptr[k], sizeof(int) * (L->ndof + 1));
    L->col = (int *)malloc(sizeof(int) * (L->nnz ? L->nnz : 1));
    memcpy(L->col, col[k], sizeof(int) * L->nnz);
    L->val = (double *)calloc(L->nnz, sizeof(double));
    L->rhs = (double *)calloc(L->ndof, sizeof(double));
    L->sol = (double *)calloc(L->ndof, sizeof(double));
    L->diag = (double *)calloc(L->ndof, sizeof(double));
    L->mg_rhs = (double *)calloc(L->ndof, sizeof(double));
    L->mg_sol = (double *)calloc(L->ndof, sizeof(double));
    L->mg_def = (double *)calloc(L->ndof, sizeof(double));
  }
  int nterms = cfg->problem_linear ? 2 : 3;
  if (p->shape == 2) {
    p->nqp1 = tet_points_for_degree(nterms * cfg->order);
    make_tet_rule_by_code(p->nqp1, &p->qr);
  } else {
    p->nqp1 = gauss_points_for_degree(nterms * cfg->order);
    make_rule(dim, p->nqp1, &p->qr);
  }
  return p;
}

int orc_level_info(const orc_problem *p, int level, int *info) {
  if (level < 0 || level >= p->nlev) FAIL("bad level");
  const level_t *L = &p->lev[level];
  info[0] = L->ncells; info[1] = L->nloc; info[2] = L->ndof;
  info[3] = L->nactive; info[4] = L->nnz; info[5] = L->nv;
  return 0;
}
int orc_get_mesh(const orc_problem *p, int level, double *v) {
  const level_t *L = &p->lev[level];
  memcpy(v, L->verts, sizeof(double) * L->ncells * L->nv * p->cfg.dim);
  return 0;
}
int orc_get_gdof(const orc_problem *p, int level, int *g) {
  const level_t *L = &p->lev[level];
  memcpy(g, L->gdof, sizeof(int) * L->ncells * L->nloc);
  return 0;
}
int orc_get_structure(const orc_problem *p, int level, int *rp, int *col) {
  const level_t *L = &p->lev[level];
  memcpy(rp, L->row_ptr, sizeof(int) * (L->ndof + 1));
  memcpy(col, L->col, sizeof(int) * L->nnz);
  return 0;
}
int orc_get_matrix(const orc_problem *p, int level, double *v) {
  const level_t *L = &p->lev[level];
  memcpy(v, L->val, sizeof(double) * L->nnz);
  return 0;
}
int orc_get_rhs(const orc_problem *p, int level, double *v) {
  const level_t *L = &p->lev[level];
  memcpy(v, L->rhs, sizeof(double) * L->ndof);
  return 0;
}
int orc_get_solution(const orc_problem *p, double *v) {
  memcpy(v, p->lev[0].sol, sizeof(double) * p->lev[0].ndof);
  return 0;
}
int orc_set_solution(orc_problem *p, const double *v) {
  memcpy(p->lev[0].sol, v, sizeof(double) * p->lev[0].ndof);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* local assembly                                                            */
/* ------------------------------------------------------------------------ */
/* Mesh_size_in_convection_direction (ConvDiff.C:26-254), CELL_MEASURE 4:
 * the vertex functions of the cell fitted in physical coordinates --
 * (1,x,y,xy) on quadrilaterals, (1,x,y,z) on tetrahedra,
 * (1,x,y,z,xy,xz,yz,xyz) on hexahedra -- and h = 2|b| / sum_i |b . grad
 * phi_i(barycentre)|, hK when the sum vanishes.  The inverse of the vertex
 * system by Gauss-Jordan elimination with partial pivoting. */
static double conv_hK(int shape, int dim, const double *cv, const double *b, double hK) {
  int n = shape == 1 ? 8 : 4;   /* shape: 0 quadrilateral, 1 hexahedron, 2 tetrahedron */
  double a[8][8], x[8][8], sc[3] = {0, 0, 0}, den = 0, nb = 0;
  for (int i = 0; i < n; ++i) {
    const double *v = cv + i * dim;
    double px = v[0], py = v[1], pz = dim == 3 ? v[2] : 0.0;
    double r[8] = {1, px, py, shape == 0 ? px * py : pz, px * py, px * pz, py * pz, px * py * pz};
    sc[0] += px / n;
    sc[1] += py / n;
    sc[2] += pz / n;
    for (int j = 0; j < n; ++j) {
      a[i][j] = r[j];
      x[i][j] = i == j;
    }
  }
  for (int col = 0; col < n; ++col) {
    int pr = col;
    for (int r = col + 1; r < n; ++r)
      if (fabs(a[r][col]) > fabs(a[pr][col])) pr = r;
    if (a[pr][col] == 0.0) return hK;
    for (int j = 0; j < n; ++j) {
      double t = a[col][j]; a[col][j] = a[pr][j]; a[pr][j] = t;
      t = x[col][j]; x[col][j] = x[pr][j]; x[pr][j] = t;
    }
    double ip = 1.0 / a[col][col];
    for (int j = 0; j < n; ++j) {
      a[col][j] *= ip;
      x[col][j] *= ip;
    }
    for (int r = 0; r < n; ++r) {
      if (r == col || a[r][col] == 0.0) continue;
      double f = a[r][col];
      for (int j = 0; j < n; ++j) {
        a[r][j] -= f * a[col][j];
        x[r][j] -= f * x[col][j];
      }
    }
  }
  for (int a2 = 0; a2 < dim; ++a2) nb += b[a2] * b[a2];
  nb = sqrt(nb);
  for (int i = 0; i < n; ++i) {
    double g[3] = {0, 0, 0}, v = 0;
    if (shape == 0) {
      g[0] = x[1][i] + x[3][i] * sc[1];
      g[1] = x[2][i] + x[3][i] * sc[0];
    } else if (shape == 2) {
      g[0] = x[1][i];
      g[1] = x[2][i];
      g[2] = x[3][i];
    } else {
      g[0] = x[1][i] + x[4][i] * sc[1] + x[5][i] * sc[2] + x[7][i] * sc[1] * sc[2];
      g[1] = x[2][i] + x[4][i] * sc[0] + x[6][i] * sc[2] + x[7][i] * sc[0] * sc[2];
      g[2] = x[3][i] + x[5][i] * sc[0] + x[6][i] * sc[1] + x[7][i] * sc[0] * sc[1];
    }
    for (int a2 = 0; a2 < dim; ++a2) v += b[a2] * g[a2];
    den += fabs(v);
  }
  return den < 1e-10 ? hK : 2 * nb / den;
}

/* Compute_SDFEM_delta (ConvDiff.C:269-495); hK is the cell's Get_hK,
 * replaced by the size in convection direction for CELL_MEASURE 4 */
static double sdfem_delta(const orc_config *c, int shape, const double *cv, double tau,
                          double theta1, double hK, double eps, const double *b, double react,
                          double linfb) {
  int d = c->dim;
  double delta0 = c->delta0, delta1 = c->delta1, delta = 0, alpha;
  if (fabs(eps) < 1e-20) eps = 1e-20;
  double h = c->cell_measure == 4 ? conv_hK(shape, d, cv, b, hK) : hK;
  double nb = b[0] * b[0] + b[1] * b[1];
  if (d == 3) nb += b[2] * b[2];
  nb = sqrt(nb);
  double reaction = fabs(react);
  switch (c->sdfem_type) {
  case 0:
    if (eps < h * nb)
      delta = delta0 * h / nb;
    else
      delta = delta1 * h * h / eps;
    break;
  case 1:
  case 2: {
    double nu = 1.0 / c->poly_degree;
    if (nb > 0) {
      alpha = nu * nb * h / (2 * eps);
      delta = nu * h * (1 / tanh(alpha) - 1 / alpha) / (2 * nb);
    } else
      delta = 0;
    delta *= delta0;
    break;
  }
  case 4:
  case 5:
  case 8:
    delta = -1;
    if (c->sdfem_type == 4) {
      if (linfb > 0) delta = h / linfb;
    } else if (nb > 0)
      delta = h / (2 * nb);
    if (reaction > 0) {
      alpha = 1.0 / reaction;
      if (delta < 0 || alpha < delta) delta = alpha;
    }
    if (eps > 0) {
      alpha = h * h / eps;
      if (delta < 0 || alpha < delta) delta = alpha;
    }
    delta *= delta0;
    if (delta < 0) delta = 0;
    break;
  case 6: {
    /* Franca/Valentin (2000) */
    double r = reaction < 1e-20 ? 1e20 : reaction;
    double alpha2;
    alpha = 6 * eps / (h * h * r);
    if (alpha <= 1) alpha = 1;
    alpha2 = h * nb / (3 * eps);
    if (alpha2 <= 1) alpha2 = 1;
    delta = 1 / (r * h * h * alpha + 6 * eps * alpha2);
    delta *= delta0 * h * h;
    break;
  }
  case 7:
    delta = delta0 * h * h / (4 * eps + 2 * h * nb + h * h * reaction);
    break;
  /* the time-dependent estimates of John and Novo (tau = CURRENTTIMESTEPLENGTH,
   * theta1 = THETA1) */
  case 9:
    delta = delta0 * tau;
    break;
  case 10:
    eps /= (theta1 * tau);
    delta = eps <= h ? delta0 * h : delta0 * h * h / eps;
    break;
  case 11:
    nb /= tau;
    delta = nb > 0 ? delta0 * h * sqrt(tau) / nb : 0;
    break;
  case 12: {
    double c_inv = delta0;
    double m = sqrt(3.0) * h / (8 * eps * c_inv);
    m = m < 0.25 ? m : 0.25;
    m *= h / (2. * sqrt(3.0) * c_inv);
    delta = 100 * (m < 1. ? m : 1.);
    break;
  }
  default:
    delta = 0;
  }
  return delta;
}

/* Compute_SDFEM_delta throws for the types it does not have (3, above 12);
 * 9-11 take the time step: time-dependent problem only */
static int check_sdfem(const orc_config *c, int tcd) {
  if (!c->supg) return 0;
  int ty = c->sdfem_type;
  if (ty < 0 || ty == 3 || ty > 12) FAIL("SDFEM_TYPE not implemented");
  if (!tcd && ty >= 9 && ty <= 11) FAIL("SDFEM_TYPE depends on the time step");
  return 0;
}

/* the stabilisation parameter of TCDStiffSUPG, TCDMassSUPG and TCDRhsSUPG
 * (CD_local_assembling_routines.C:184-387): in 2D, except for SDFEM_TYPE 2
 * and 12, Compute_SDFEM_delta takes the coefficients scaled by theta1 * tau
 * (reaction 1 + theta1 tau c, type 8: theta1 tau c); the L_inf norm of b is
 * always the scaled one in 2D.  Then delta *= theta1 * tau except for the
 * types 2, 9, 10, 11, 12. */
static double tcd_delta(const orc_problem *p, const double *cv, double hK, double eps,
                        const double *b, double react, double linfb) {
  const orc_config *c = &p->cfg;
  const double tt = p->ttau;
  const int ty = c->sdfem_type;
  double delta;
  if (c->dim == 2) {
    double bs[3] = {tt * b[0], tt * b[1], 0};
    double bb = fabs(bs[0]) > fabs(bs[1]) ? fabs(bs[0]) : fabs(bs[1]);
    if (ty != 2 && ty != 12)
      delta = sdfem_delta(c, p->shape, cv, p->tau, p->theta1, hK, tt * eps, bs,
                          ty == 8 ? tt * react : 1.0 + tt * react, bb);
    else
      delta = sdfem_delta(c, p->shape, cv, p->tau, p->theta1, hK, eps, b, react, bb);
  } else {
    delta = sdfem_delta(c, p->shape, cv, p->tau, p->theta1, hK, eps, b, react, linfb);
  }
  if (ty != 2 && ty != 9 && ty != 10 && ty != 11 && ty != 12) delta *= tt;
  return delta;
}

int orc_local_system(orc_problem *p, int level, int cell, double *Aloc,
                     double *floc) {
  const orc_config *c = &p->cfg;
  level_t *L = &p->lev[level];
  int dim = c->dim, nl = L->nloc;
  const double *cv = L->verts + (size_t)cell * L->nv * dim;
  /* affine map per cell, or the bilinear / trilinear map at every point */
  const int multi = cell_is_multilinear(p->shape, dim, cv);
  if (multi && dim == 3 && (c->supg || p->tcd)) {
    /* THexaTrilinear::GetOrigAllDerivatives (HexaTrilinear.C:185-222) throws */
    FAIL("SUPG needs second derivatives on trilinear hexahedra");
  }
  if (multi && (p->tcd || c->neumann_mask || (dim == 3 && c->cell_measure != 0 &&
                                               c->cell_measure != 2)))
    FAIL("multilinear cells: stationary, Dirichlet, CELL_MEASURE 0/2 in 3D");
  affine_t A;
  cell_affine_s(p->shape, dim, cv, &A);
  double adet = fabs(A.det);
  double hK = cell_hK_s(p->shape, dim, cv, c->cell_measure);
  for (int i = 0; i < nl * nl; ++i) Aloc[i] = 0;
  for (int i = 0; i < nl; ++i) floc[i] = 0;
  double ref[MAXLOC][NDER];
  int nh = dim == 2 ? 3 : 6;
  for (int q = 0; q < p->qr.nqp; ++q) {
    double lw[5] = {0, 0, 0, 0, 0};
    if (multi) {
      multilinear_at(dim, cv, p->qr.xi[q], &A);
      adet = fabs(A.det);
      if (dim == 2) bilinear_lap_weights(cv, p->qr.xi[q], lw);
    }
    basis_s(p->shape, dim, c->order, p->qr.xi[q], ref);
    /* GetOrigValues: physical derivatives */
    double u[MAXLOC], g[MAXLOC][3], lap[MAXLOC];
    for (int k = 0; k < nl; ++k) {
      u[k] = ref[k][0];
      for (int r = 0; r < dim; ++r) {
        double s = 0;
        for (int a = 0; a < dim; ++a) s += A.Jinv[a][r] * ref[k][1 + a];
        g[k][r] = s;
      }
      /* Laplacian of the affine-transformed Hessian J^-T H J^-1 */
      double H[3][3];
      if (dim == 2) {
        H[0][0] = ref[k][3]; H[0][1] = H[1][0] = ref[k][4]; H[1][1] = ref[k][5];
      } else {
        H[0][0] = ref[k][4]; H[0][1] = H[1][0] = ref[k][5];
        H[0][2] = H[2][0] = ref[k][6]; H[1][1] = ref[k][7];
        H[1][2] = H[2][1] = ref[k][8]; H[2][2] = ref[k][9];
      }
      (void)nh;
      double l = 0;
      if (multi) {
        /* (u_xi, u_eta, u_xixi, u_xieta, u_etaeta) through G^-1; the
         * trilinear case takes no second derivatives (Galerkin only) */
        if (dim == 2)
          l = lw[0] * ref[k][1] + lw[1] * ref[k][2] + lw[2] * H[0][0] + lw[3] * H[0][1] +
              lw[4] * H[1][1];
      } else {
        for (int r = 0; r < dim; ++r)
          for (int a = 0; a < dim; ++a)
            for (int b2 = 0; b2 < dim; ++b2)
              l += A.Jinv[a][r] * A.Jinv[b2][r] * H[a][b2];
      }
      lap[k] = l;
    }
    double x[3];
    if (multi)
      for (int r = 0; r < dim; ++r) x[r] = A.x0[r];
    else
      affine_map(dim, &A, p->qr.xi[q], x);
    double co[8];
    if (p->coef_in) {
      /* CoeffFct values at this point: eps, b, c, f; the L_inf norm of b that
       * Compute_SDFEM_delta takes is formed here, as ConvDiff.C:1858-1863
       * lays out the coefficient vector */
      const double *ci = p->coef_in + ((size_t)cell * p->qr.nqp + q) * (dim + 3);
      double binf = 0;
      for (int k = 0; k < dim + 3; ++k) co[k] = ci[k];
      for (int a = 0; a < dim; ++a)
        if (fabs(ci[1 + a]) > binf) binf = fabs(ci[1 + a]);
      co[dim + 3] = binf;
    } else {
      coeffs_at(c, x, co);
    }
    double Mult = p->qr.w[q] * adet;
    double eps = co[0], b[3] = {co[1], co[2], dim == 3 ? co[3] : 0};
    double react = co[dim + 1], f = co[dim + 2];
    /* BilinearAssembleGalerkin<d> (ConvDiff.C:1776-1883) */
    for (int i = 0; i < nl; ++i) {
      floc[i] += Mult * u[i] * f;
      for (int j = 0; j < nl; ++j) {
        double val = 0;
        for (int r = 0; r < dim; ++r) val += g[i][r] * g[j][r];
        val *= eps;
        double bg = 0;
        for (int r = 0; r < dim; ++r) bg += b[r] * g[j][r];
        val += bg * u[i];
        val += react * u[j] * u[i];
        Aloc[i * nl + j] += val * Mult;
      }
    }
    if (c->supg) {
      /* BilinearAssemble_SD<d> (ConvDiff.C:1886-1999); the time-dependent
       * TCDStiffSUPG / TCDRhsSUPG have the same form with their own delta */
      double delta = p->tcd ? tcd_delta(p, cv, hK, eps, b, react, co[dim + 3])
                            : sdfem_delta(c, p->shape, cv, 0.0, 0.0, hK, eps, b, react,
                                          co[dim + 3]);
      for (int i = 0; i < nl; ++i) {
        double bgradv = 0;
        for (int r = 0; r < dim; ++r) bgradv += b[r] * g[i][r];
        floc[i] += Mult * (delta * bgradv) * f;
        for (int j = 0; j < nl; ++j) {
          double val = -eps * lap[j];
          for (int r = 0; r < dim; ++r) val += b[r] * g[j][r];
          val += react * u[j];
          Aloc[i * nl + j] += val * delta * bgradv * Mult;
        }
      }
    }
  }
  return 0;
}

/* Neumann boundary integral on a 2D boundary edge (Assemble2D.C:3210-3248):
 * g = eps * n.grad(u), line rule of degree 2p */
static void neumann_edge(orc_problem *p, level_t *L, int cell, int j,
                         double *rhs) {
  const orc_config *c = &p->cfg;
  const double *cv = L->verts + (size_t)cell * L->nv * 2;
  int nl = L->nloc;
  int np = line_points_for_degree(2 * c->order);
  double lx[10], lw[10];
  gauss_legendre(np, lx, lw);
  const double *a = cv + 2 * j, *bb = cv + 2 * ((j + 1) % 4);
  double hE = sqrt((bb[0] - a[0]) * (bb[0] - a[0]) +
                   (bb[1] - a[1]) * (bb[1] - a[1])) / 2;
  affine_t A;
  cell_affine(2, cv, &A);
  double ctr[2] = {0.5 * (a[0] + bb[0]), 0.5 * (a[1] + bb[1])};
  int comp = boundary_comp(2, ctr);
  const double nrm[4][2] = {{0, -1}, {1, 0}, {0, 1}, {-1, 0}};
  for (int l = 0; l < np; ++l) {
    double s = 0.5 * (lx[l] + 1);
    double x[2] = {a[0] + s * (bb[0] - a[0]), a[1] + s * (bb[1] - a[1])};
    double u[6];
    exact_sol(c, x, u);
    double g = c->eps * (nrm[comp][0] * u[1] + nrm[comp][1] * u[2]);
    /* reference coordinates of x */
    double xi[3] = {0, 0, 0};
    for (int aa = 0; aa < 2; ++aa) {
      double t = 0;
      for (int r = 0; r < 2; ++r) t += A.Jinv[aa][r] * (x[r] - A.x0[r]);
      xi[aa] = t;
    }
    double ref[MAXLOC][NDER];
    ref_basis(2, c->order, xi, ref);
    double sc = g * hE * lw[l];
    for (int k = 0; k < nl; ++k) {
      int d = L->gdof[cell * nl + k];
      if (d < L->nactive) rhs[d] += sc * ref[k][0];
    }
  }
}

/* Neumann boundary integral on a hexahedron face (Assemble3D.C:552-655,
 * quadrilateral faces): g = eps * n.grad(u) with the outward unit normal n of
 * the boundary component, tensor Gauss rule of degree 2p on [-1,1]^2 mapped
 * bilinearly through the face's vertices, weight times |dx/ds x dx/dt| */
static void neumann_face(orc_problem *p, level_t *L, int cell, int j, int comp,
                         double *rhs) {
  const orc_config *c = &p->cfg;
  const double *cv = L->verts + (size_t)cell * L->nv * 3;
  int nl = L->nloc;
  int np = line_points_for_degree(2 * c->order);
  double lx[10], lw[10];
  gauss_legendre(np, lx, lw);
  static const double nrm[6][3] = {{0, 0, -1}, {0, -1, 0}, {1, 0, 0},
                                   {0, 1, 0},  {-1, 0, 0}, {0, 0, 1}};
  double X[4][3];
  for (int m = 0; m < 4; ++m)
    for (int a = 0; a < 3; ++a) X[m][a] = cv[HEX_FACE[j][m] * 3 + a];
  double c1[3], c2[3], c3[3];
  for (int a = 0; a < 3; ++a) {
    c1[a] = (-X[0][a] + X[1][a] + X[2][a] - X[3][a]) * 0.25;
    c2[a] = (-X[0][a] - X[1][a] + X[2][a] + X[3][a]) * 0.25;
    c3[a] = (X[0][a] - X[1][a] + X[2][a] - X[3][a]) * 0.25;
  }
  affine_t A;
  cell_affine(3, cv, &A);
  for (int l1 = 0; l1 < np; ++l1)
    for (int l2 = 0; l2 < np; ++l2) {
      double ps = lx[l1], pt = lx[l2];
      double t0 = 0.5 * (ps + 1), t1 = 0.5 * (pt + 1);
      double lc[4] = {(1 - t0) * (1 - t1), t0 * (1 - t1), t0 * t1, (1 - t0) * t1};
      double x[3] = {0, 0, 0};
      for (int m = 0; m < 4; ++m)
        for (int a = 0; a < 3; ++a) x[a] += lc[m] * X[m][a];
      double u[6];
      exact_sol(c, x, u);
      double g = c->eps * (nrm[comp][0] * u[1] + nrm[comp][1] * u[2] + nrm[comp][2] * u[3]);
      double ta[3], tb[3];
      for (int a = 0; a < 3; ++a) {
        ta[a] = c1[a] + pt * c3[a];
        tb[a] = c2[a] + ps * c3[a];
      }
      double nx = ta[1] * tb[2] - ta[2] * tb[1];
      double ny = ta[2] * tb[0] - ta[0] * tb[2];
      double nz = ta[0] * tb[1] - ta[1] * tb[0];
      double sc = g * lw[l1] * lw[l2] * sqrt(nx * nx + ny * ny + nz * nz);
      double xi[3];
      for (int a = 0; a < 3; ++a) {
        double t = 0;
        for (int r = 0; r < 3; ++r) t += A.Jinv[a][r] * (x[r] - A.x0[r]);
        xi[a] = t;
      }
      double ref[MAXLOC][NDER];
      ref_basis(3, c->order, xi, ref);
      for (int k = 0; k < nl; ++k) {
        int d = L->gdof[cell * nl + k];
        if (d < L->nactive) rhs[d] += sc * ref[k][0];
      }
    }
}

/* Neumann boundary integral on a tetrahedron face (Assemble3D.C:552-655,
 * triangular faces, face j opposite vertex j): g = eps * n.grad(u) with the
 * outward unit normal n of the boundary component at x = X0 + s (X1-X0) +
 * t (X2-X0), weight times |(X1-X0) x (X2-X0)|.  The rule on the reference
 * triangle is Gauss-Legendre in (sigma, tau) with p+1 points each, collapsed
 * by s = sigma (1 - tau), t = tau with the factor (1 - tau): exact to degree
 * 2p, as the reference's triangle rule of degree 2p is. */
static void neumann_face_tet(orc_problem *p, level_t *L, int cell, int j, int comp,
                             double *rhs) {
  const orc_config *c = &p->cfg;
  static const int TET_FACE[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
  static const double nrm[6][3] = {{0, 0, -1}, {0, -1, 0}, {1, 0, 0},
                                   {0, 1, 0},  {-1, 0, 0}, {0, 0, 1}};
  const double *cv = L->verts + (size_t)cell * 4 * 3;
  int nl = L->nloc, np = c->order + 1;
  double lx[10], lw[10];
  gauss_legendre(np, lx, lw);
  double X[3][3], e1[3], e2[3];
  for (int m = 0; m < 3; ++m)
    for (int a = 0; a < 3; ++a) X[m][a] = cv[TET_FACE[j][m] * 3 + a];
  for (int a = 0; a < 3; ++a) {
    e1[a] = X[1][a] - X[0][a];
    e2[a] = X[2][a] - X[0][a];
  }
  double cx = e1[1] * e2[2] - e1[2] * e2[1];
  double cy = e1[2] * e2[0] - e1[0] * e2[2];
  double cz = e1[0] * e2[1] - e1[1] * e2[0];
  double area2 = sqrt(cx * cx + cy * cy + cz * cz);
  affine_t A;
  cell_affine_s(p->shape, 3, cv, &A);
  for (int l1 = 0; l1 < np; ++l1)
    for (int l2 = 0; l2 < np; ++l2) {
      double sg = 0.5 * (lx[l1] + 1), tau = 0.5 * (lx[l2] + 1);
      double fs = sg * (1 - tau), ft = tau;
      double w = 0.25 * lw[l1] * lw[l2] * (1 - tau);
      double x[3], u[6], xi[3];
      for (int a = 0; a < 3; ++a) x[a] = X[0][a] + fs * e1[a] + ft * e2[a];
      exact_sol(c, x, u);
      double g = c->eps * (nrm[comp][0] * u[1] + nrm[comp][1] * u[2] + nrm[comp][2] * u[3]);
      for (int a = 0; a < 3; ++a) {
        double t = 0;
        for (int r = 0; r < 3; ++r) t += A.Jinv[a][r] * (x[r] - A.x0[r]);
        xi[a] = t;
      }
      double ref[MAXLOC][NDER];
      tet_basis(c->order, xi, ref);
      for (int k = 0; k < nl; ++k) {
        int d = L->gdof[cell * nl + k];
        if (d < L->nactive) rhs[d] += g * w * area2 * ref[k][0];
      }
    }
}

/* local mass matrix, TCDMass (CD_local_assembling_routines.C:156-167):
 * M_ij = int phi_i phi_j; with SUPG plus TCDMassSUPG (:261-321):
 * int delta (b . grad phi_i) phi_j */
static void local_mass(orc_problem *p, level_t *L, int cell, double *Mloc) {
  const orc_config *c = &p->cfg;
  int dim = c->dim, nl = L->nloc;
  const double *cv = L->verts + (size_t)cell * L->nv * dim;
  affine_t A;
  cell_affine_s(p->shape, dim, cv, &A);
  double adet = fabs(A.det);
  double hK = cell_hK_s(p->shape, dim, cv, c->cell_measure);
  for (int i = 0; i < nl * nl; ++i) Mloc[i] = 0;
  double ref[MAXLOC][NDER];
  for (int q = 0; q < p->qr.nqp; ++q) {
    basis_s(p->shape, dim, c->order, p->qr.xi[q], ref);
    double Mult = p->qr.w[q] * adet;
    for (int i = 0; i < nl; ++i)
      for (int j = 0; j < nl; ++j) Mloc[i * nl + j] += Mult * ref[j][0] * ref[i][0];
    if (!c->supg) continue;
    double x[3], co[8];
    affine_map(dim, &A, p->qr.xi[q], x);
    coeffs_at(c, x, co);
    double b[3] = {co[1], co[2], dim == 3 ? co[3] : 0};
    double delta = tcd_delta(p, cv, hK, co[0], b, co[dim + 1], co[dim + 3]);
    for (int i = 0; i < nl; ++i) {
      double bgradv = 0;
      for (int r = 0; r < dim; ++r) {
        double gr = 0;
        for (int a = 0; a < dim; ++a) gr += A.Jinv[a][r] * ref[i][1 + a];
        bgradv += b[r] * gr;
      }
      bgradv *= delta;
      for (int j = 0; j < nl; ++j) Mloc[i * nl + j] += Mult * ref[j][0] * bgradv;
    }
  }
}

/* scatter of a local matrix by linear row search (Assemble3D.C:257-292) */
static int scatter_row(const level_t *L, int l, const int *dof, const double *row,
                       double *val) {
  for (int k = 0; k < L->nloc; ++k) {
    int found = 0;
    for (int n = L->row_ptr[l]; n < L->row_ptr[l + 1]; ++n)
      if (L->col[n] == dof[k]) {
        val[n] += row[k];
        found = 1;
        break;
      }
    if (!found) FAIL("entry not in pattern");
  }
  return 0;
}

/* Assemble2D/3D over one level into (val, rhs).  all_rows: Dirichlet rows
 * receive the full local rows (assemble_dirichlet_rows, as the time-dependent
 * problem does); otherwise they are identity rows (Matrix.C:225-233).
 * mval != NULL: the mass matrix is assembled alongside. */
static int assemble_into(orc_problem *p, int level, double *val, double *rhs,
                         int all_rows, double *mval) {
  const orc_config *c = &p->cfg;
  level_t *L = &p->lev[level];
  int dim = c->dim, nl = L->nloc;
  memset(val, 0, sizeof(double) * L->nnz);
  memset(rhs, 0, sizeof(double) * L->ndof);
  if (mval) memset(mval, 0, sizeof(double) * L->nnz);
  double Aloc[MAXLOC * MAXLOC], floc[MAXLOC], Mloc[MAXLOC * MAXLOC];
  for (int cell = 0; cell < L->ncells; ++cell) {
    if (orc_local_system(p, level, cell, Aloc, floc)) return -1;
    if (mval) local_mass(p, L, cell, Mloc);
    const int *dof = L->gdof + cell * nl;
    for (int m = 0; m < nl; ++m) {
      int l = dof[m];
      if (l < L->nactive || all_rows) {
        if (scatter_row(L, l, dof, Aloc + m * nl, val)) return -1;
        if (mval && scatter_row(L, l, dof, Mloc + m * nl, mval)) return -1;
        if (l < L->nactive) rhs[l] += floc[m];
      } else {
        for (int n = L->row_ptr[l]; n < L->row_ptr[l + 1]; ++n)
          if (L->col[n] == l) val[n] = 1.0;
      }
    }
  }
  if (p->shape == 2) {
    /* tetrahedra: every non-active DOF is a Dirichlet node; value = nodal
     * functional of P1/P2 = point value; Neumann integrals over the faces
     * that lie on a Neumann component */
    for (int cell = 0; cell < L->ncells; ++cell) {
      const double *cv = L->verts + (size_t)cell * L->nv * dim;
      for (int k = 0; k < nl; ++k) {
        int d = L->gdof[cell * nl + k];
        if (d < L->nactive) continue;
        double x[3], u[6];
        dof_position_s(2, 3, c->order, cv, k, x);
        exact_sol(c, x, u);
        rhs[d] = u[0];
      }
      if (!c->neumann_mask) continue;
      for (int j = 0; j < 4; ++j) {
        double ctr[3] = {0, 0, 0};
        for (int m = 0; m < 4; ++m)
          if (m != j)
            for (int a = 0; a < 3; ++a) ctr[a] += cv[m * 3 + a] / 3.0;
        int comp = boundary_comp(3, ctr);
        if (comp >= 0 && bc_type(c, comp) != 0) neumann_face_tet(p, L, cell, j, comp, rhs);
      }
    }
    return 0;
  }
  /* boundary data: Dirichlet values by point evaluation at the nodes (nodal
   * functionals of Q1/Q2), Neumann integrals over edges (2D) and faces (3D) */
  int nj = dim == 2 ? 4 : 6;
  for (int cell = 0; cell < L->ncells; ++cell) {
    const double *cv = L->verts + (size_t)cell * L->nv * dim;
    for (int j = 0; j < nj; ++j) {
      double ctr[3] = {0, 0, 0};
      int nvj = dim == 2 ? 2 : 4;
      for (int m = 0; m < nvj; ++m) {
        int vid = dim == 2 ? (m == 0 ? j : (j + 1) % 4) : HEX_FACE[j][m];
        for (int a = 0; a < dim; ++a) ctr[a] += cv[vid * dim + a] / nvj;
      }
      int comp = boundary_comp(dim, ctr);
      if (comp < 0) continue;
      if (bc_type(c, comp) == 0) {
        int idx[MAXLOC];
        int n = joint_dofs(dim, c->order, j, idx);
        const int multi = cell_is_multilinear(p->shape, dim, cv);
        for (int m = 0; m < n; ++m) {
          double x[3], u[6];
          if (multi) {
            /* the nodal functional's point on the bilinear / trilinear cell */
            double r[3];
            affine_t P;
            local_dof_ref(dim, c->order, idx[m], r);
            multilinear_at(dim, cv, r, &P);
            for (int a = 0; a < dim; ++a) x[a] = P.x0[a];
          } else {
            dof_position(dim, c->order, cv, idx[m], x);
          }
          exact_sol(c, x, u);
          rhs[L->gdof[cell * nl + idx[m]]] = u[0];
        }
      } else if (dim == 2) {
        neumann_edge(p, L, cell, j, rhs);
      } else {
        neumann_face(p, L, cell, j, comp, rhs);
      }
    }
  }
  return 0;
}

static int assemble_level(orc_problem *p, int level) {
  level_t *L = &p->lev[level];
  if (assemble_into(p, level, L->val, L->rhs, 0, NULL)) return -1;
  /* solution.copy_nonactive(rhs) (ConvectionDiffusion.C:445) */
  for (int i = L->nactive; i < L->ndof; ++i) L->sol[i] = L->rhs[i];
  /* diagonal for Jacobi (Iteration_jacobi.C:14-28) */
  for (int r = 0; r < L->ndof; ++r)
    for (int n = L->row_ptr[r]; n < L->row_ptr[r + 1]; ++n)
      if (L->col[n] == r) L->diag[r] = L->val[n];
  return 0;
}

/* physical coordinates of the quadrature points of every cell of a level,
 * x[(cell * nqp + q) * dim + r] (the points orc_local_system integrates at) */
int orc_quadrature_points(const orc_problem *p, int level, int *nqp, double *x) {
  if (level < 0 || level >= p->nlev) FAIL("level out of range");
  const level_t *L = &p->lev[level];
  const int dim = p->cfg.dim;
  *nqp = p->qr.nqp;
  if (!x) return 0;
  for (int cell = 0; cell < L->ncells; ++cell) {
    const double *cv = L->verts + (size_t)cell * L->nv * dim;
    affine_t A;
    cell_affine_s(p->shape, dim, cv, &A);
    const int multi = cell_is_multilinear(p->shape, dim, cv);
    for (int q = 0; q < p->qr.nqp; ++q) {
      double *xq = x + ((size_t)cell * p->qr.nqp + q) * dim;
      if (multi) {
        multilinear_at(dim, cv, p->qr.xi[q], &A);
        for (int r = 0; r < dim; ++r) xq[r] = A.x0[r];
      } else {
        affine_map(dim, &A, p->qr.xi[q], xq);
      }
    }
  }
  return 0;
}

/* ConvectionDiffusion::assemble of one level with the coefficients given per
 * (cell, quadrature point), co[(cell * nqp + q) * (dim + 3) + k]: k = 0 eps,
 * 1..dim b, dim+1 c, dim+2 f (the CoeffFct2D/3D output,
 * include/General/Constants.h:43-47); boundary values from the example */
int orc_assemble_coefficients(orc_problem *p, int level, const double *co) {
  if (level < 0 || level >= p->nlev) FAIL("level out of range");
  if (check_sdfem(&p->cfg, 0)) return -1;
  p->asm_gen++;
  p->coef_in = co;
  int rc = assemble_level(p, level);
  p->coef_in = NULL;
  return rc;
}

int orc_assemble(orc_problem *p) {
  if (check_sdfem(&p->cfg, 0)) return -1;
  p->asm_gen++;
  p->tcd = 0;
  for (int k = 0; k < p->nlev; ++k)
    if (assemble_level(p, k)) return -1;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* linear algebra                                                            */
/* ------------------------------------------------------------------------ */
/* y = a*A x + y on active rows; y += a*x on non-active rows */
static void apply_scaled_add(const level_t *L, const double *x, double *y,
                             double a) {
  for (int r = 0; r < L->nactive; ++r) {
    double s = 0;
    for (int n = L->row_ptr[r]; n < L->row_ptr[r + 1]; ++n)
      s += L->val[n] * x[L->col[n]];
    y[r] += a * s;
  }
  for (int r = L->nactive; r < L->ndof; ++r) y[r] += a * x[r];
}

int orc_apply(const orc_problem *p, int level, const double *x, double *y) {
  const level_t *L = &p->lev[level];
  memset(y, 0, sizeof(double) * L->ndof);
  apply_scaled_add(L, x, y, 1.0);
  return 0;
}

static double dot(int n, const double *a, const double *b) {
  double s = 0;
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

/* prolongation matrix of one child: QQ[k][l] = coarse basis l at fine local
 * dof k (nodal functionals of Lagrange elements are point values) */
static void child_prolongation(const orc_problem *p, const level_t *Lf,
                               const level_t *Lc, int fcell, double *QQ) {
  int dim = p->cfg.dim, nl = Lf->nloc;
  int nch = dim == 2 ? 4 : 8;   /* children per cell, also 8 for tetrahedra */
  int ccell = fcell / nch;
  const double *cvc = Lc->verts + (size_t)ccell * Lc->nv * dim;
  const double *cvf = Lf->verts + (size_t)fcell * Lf->nv * dim;
  affine_t Ac;
  cell_affine_s(p->shape, dim, cvc, &Ac);
  for (int k = 0; k < nl; ++k) {
    double x[3], xi[3] = {0, 0, 0};
    dof_position_s(p->shape, dim, p->cfg.order, cvf, k, x);
    for (int a = 0; a < dim; ++a) {
      double t = 0;
      for (int r = 0; r < dim; ++r) t += Ac.Jinv[a][r] * (x[r] - Ac.x0[r]);
      xi[a] = t;
    }
    double ref[MAXLOC][NDER];
    basis_s(p->shape, dim, p->cfg.order, xi, ref);
    for (int l = 0; l < nl; ++l) QQ[k * nl + l] = ref[l][0];
  }
}

/* GridTransfer::Prolongate (GridTransfer.C:29-218) */
int orc_prolongate(const orc_problem *p, int fine, const double *xc,
                   double *xf) {
  const level_t *Lf = &p->lev[fine], *Lc = &p->lev[fine + 1];
  int nl = Lf->nloc, nch = p->cfg.dim == 2 ? 4 : 8;
  double *aux = (double *)calloc(Lf->ndof, sizeof(double));
  memset(xf, 0, sizeof(double) * Lf->ndof);
  double QQ[MAXLOC * MAXLOC];
  for (int f = 0; f < Lf->ncells; ++f) {
    int cc = f / nch;
    child_prolongation(p, Lf, Lc, f, QQ);
    for (int k = 0; k < nl; ++k) {
      double s = 0;
      for (int l = 0; l < nl; ++l) s += QQ[k * nl + l] * xc[Lc->gdof[cc * nl + l]];
      int idx = Lf->gdof[f * nl + k];
      xf[idx] += s;
      aux[idx] += 1;
    }
  }
  for (int i = 0; i < Lf->ndof; ++i) xf[i] /= aux[i];
  free(aux);
  return 0;
}

/* GridTransfer::DefectRestriction (GridTransfer.C:222-410) */
int orc_restrict(const orc_problem *p, int fine, const double *df,
                 double *rc) {
  const level_t *Lf = &p->lev[fine], *Lc = &p->lev[fine + 1];
  int nl = Lf->nloc, nch = p->cfg.dim == 2 ? 4 : 8;
  double *aux = (double *)calloc(Lf->ndof, sizeof(double));
  double *cp = (double *)malloc(sizeof(double) * Lf->ndof);
  memset(rc, 0, sizeof(double) * Lc->ndof);
  for (int f = 0; f < Lf->ncells; ++f)
    for (int k = 0; k < nl; ++k) aux[Lf->gdof[f * nl + k]] += 1;
  for (int i = 0; i < Lf->ndof; ++i) cp[i] = df[i] / aux[i];
  double QQ[MAXLOC * MAXLOC];
  for (int f = 0; f < Lf->ncells; ++f) {
    int cc = f / nch;
    child_prolongation(p, Lf, Lc, f, QQ);
    for (int l = 0; l < nl; ++l) {
      double s = 0;
      for (int k = 0; k < nl; ++k) s += QQ[k * nl + l] * cp[Lf->gdof[f * nl + k]];
      rc[Lc->gdof[cc * nl + l]] += s;
    }
  }
  free(aux);
  free(cp);
  return 0;
}

/* dense LU with partial pivoting of the full coarse matrix */
static int coarse_factor(level_t *L) {
  int n = L->ndof;
  free(L->lu);
  free(L->piv);
  L->lu = (double *)calloc((size_t)n * n, sizeof(double));
  L->piv = (int *)malloc(sizeof(int) * n);
  for (int r = 0; r < L->nactive; ++r)
    for (int k = L->row_ptr[r]; k < L->row_ptr[r + 1]; ++k)
      L->lu[(size_t)r * n + L->col[k]] = L->val[k];
  for (int r = L->nactive; r < n; ++r) L->lu[(size_t)r * n + r] = 1.0;
  double *a = L->lu;
  for (int k = 0; k < n; ++k) {
    int pr = k;
    double mx = fabs(a[(size_t)k * n + k]);
    for (int i = k + 1; i < n; ++i)
      if (fabs(a[(size_t)i * n + k]) > mx) {
        mx = fabs(a[(size_t)i * n + k]);
        pr = i;
      }
    if (mx == 0) FAIL("singular coarse matrix");
    L->piv[k] = pr;
    if (pr != k)
      for (int j = 0; j < n; ++j) {
        double t = a[(size_t)k * n + j];
        a[(size_t)k * n + j] = a[(size_t)pr * n + j];
        a[(size_t)pr * n + j] = t;
      }
    double d = a[(size_t)k * n + k];
    for (int i = k + 1; i < n; ++i) {
      double m = a[(size_t)i * n + k] / d;
      a[(size_t)i * n + k] = m;
      if (m != 0)
        for (int j = k + 1; j < n; ++j) a[(size_t)i * n + j] -= m * a[(size_t)k * n + j];
    }
  }
  return 0;
}

static void coarse_solve(const level_t *L, const double *b, double *x) {
  int n = L->ndof;
  for (int i = 0; i < n; ++i) x[i] = b[i];
  for (int k = 0; k < n; ++k) {
    int pr = L->piv[k];
    if (pr != k) {
      double t = x[k];
      x[k] = x[pr];
      x[pr] = t;
    }
  }
  for (int i = 0; i < n; ++i) {
    double s = x[i];
    for (int j = 0; j < i; ++j) s -= L->lu[(size_t)i * n + j] * x[j];
    x[i] = s;
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = x[i];
    for (int j = i + 1; j < n; ++j) s -= L->lu[(size_t)i * n + j] * x[j];
    x[i] = s / L->lu[(size_t)i * n + i];
  }
}

/* JacobiSmoother::smooth (JacobiSmoother.C:21-29) */
static void jacobi_smooth(level_t *L, double damp) {
  int n = L->ndof;
  double *d = L->mg_def;
  memcpy(d, L->mg_rhs, sizeof(double) * n);
  apply_scaled_add(L, L->mg_sol, d, -1.0);
  for (int i = 0; i < n; ++i) d[i] /= L->diag[i];
  for (int i = 0; i < n; ++i) L->mg_sol[i] += damp * d[i];
}

static double calc_defect(level_t *L) {
  int n = L->ndof;
  memcpy(L->mg_def, L->mg_rhs, sizeof(double) * n);
  apply_scaled_add(L, L->mg_sol, L->mg_def, -1.0);
  return sqrt(dot(n, L->mg_def, L->mg_def));
}

/* CycleControl (CycleControl.C:15-111): direction sequence */
enum { DIR_DUMMY, DIR_DOWN, DIR_UP, DIR_END };
static void fill_cycle(int *seq, int *n, int *rec, int level, int nlev,
                       int cyc) {
  if (level == 0) {
    seq[(*n)++] = DIR_UP;
    return;
  }
  for (int j = 0; j < rec[level]; ++j) {
    seq[(*n)++] = DIR_DOWN;
    fill_cycle(seq, n, rec, level - 1, nlev, cyc);
  }
  if (cyc == 2) rec[level] = 1;
  seq[(*n)++] = level == nlev - 1 ? DIR_END : DIR_UP;
}

/* Multigrid::cycle (Multigrid.C:157-308); MG levels are indexed coarsest
 * first there, here lev[0] is the finest: mg level m <-> lev[nlev-1-m] */
int orc_mg_apply(orc_problem *p, const orc_solver_config *s, const double *v,
                 double *z) {
  int nl = s->mg_levels;
  if (nl < 1 || nl > p->nlev) FAIL("bad multigrid level count");
  level_t *fine = &p->lev[0];
  level_t *crs = &p->lev[nl - 1];
  if (s->coarse_direct && (crs->lu == NULL || crs->lu_gen != p->asm_gen)) {
    if (coarse_factor(crs)) return -1;
    crs->lu_gen = p->asm_gen;
  }
  memcpy(fine->mg_rhs, v, sizeof(double) * fine->ndof);
  /* finest start: 0, non-actives copied from rhs */
  memset(fine->mg_sol, 0, sizeof(double) * fine->ndof);
  for (int i = fine->nactive; i < fine->ndof; ++i) fine->mg_sol[i] = v[i];
  int rec[8];
  for (int i = 0; i < nl; ++i) rec[i] = s->mg_cycle == 0 ? 1 : 2;
  rec[nl - 1] = 1;
  static int seq[4096];
  int ns = 0;
  seq[ns++] = DIR_DUMMY;
  fill_cycle(seq, &ns, rec, nl - 1, nl, s->mg_cycle);
  int level = nl - 1; /* mg index */
  for (int step = 1; step < ns && level >= 0; ++step) {
    level_t *L = &p->lev[nl - 1 - level];
    if (level == 0) {
      double res = 1e10;
      calc_defect(L);
      for (int i = 0; i < s->coarse_maxit && res > s->coarse_eps; ++i) {
        if (s->coarse_direct)
          coarse_solve(L, L->mg_rhs, L->mg_sol);
        else
          jacobi_smooth(L, s->jacobi_damp);
        res = calc_defect(L);
      }
      if (nl == 1) break; /* the coarse solve is the whole cycle */
      /* update_solution_in_finer_grid */
      level_t *F = &p->lev[nl - 1 - (level + 1)];
      double *pr = (double *)malloc(sizeof(double) * F->ndof);
      orc_prolongate(p, nl - 1 - (level + 1), L->mg_sol, pr);
      for (int i = 0; i < F->nactive; ++i) F->mg_sol[i] += s->correction_damp * pr[i];
      free(pr);
      level = level + 1;
      continue;
    }
    int coming_from_below = seq[step - 1] == DIR_UP;
    int dir = seq[step];
    if (coming_from_below)
      for (int i = 0; i < s->n_post; ++i) jacobi_smooth(L, s->jacobi_damp);
    if (dir == DIR_DOWN) {
      for (int i = 0; i < s->n_pre; ++i) jacobi_smooth(L, s->jacobi_damp);
      calc_defect(L);
      level_t *C = &p->lev[nl - 1 - (level - 1)];
      memset(C->mg_sol, 0, sizeof(double) * C->ndof);
      orc_restrict(p, nl - 1 - level, L->mg_def, C->mg_rhs);
      for (int i = C->nactive; i < C->ndof; ++i) C->mg_rhs[i] = 0;
      level = level - 1;
    } else if (dir == DIR_UP) {
      level_t *F = &p->lev[nl - 1 - (level + 1)];
      double *pr = (double *)malloc(sizeof(double) * F->ndof);
      orc_prolongate(p, nl - 1 - (level + 1), L->mg_sol, pr);
      for (int i = 0; i < F->nactive; ++i) F->mg_sol[i] += s->correction_damp * pr[i];
      free(pr);
      level = level + 1;
    } else {
      break; /* END */
    }
  }
  memcpy(z, fine->mg_sol, sizeof(double) * fine->ndof);
  return 0;
}

/* GenerateGivensRotation / ApplyGivensRotation (Utilities_gmres.C:60-88) */
static void gen_givens(double dx, double dy, double *cs, double *sn) {
  if (dy == 0.0) {
    *cs = 1.0;
    *sn = 0.0;
  } else if (fabs(dy) > fabs(dx)) {
    double t = dx / dy;
    *sn = 1.0 / sqrt(1.0 + t * t);
    *cs = t * *sn;
  } else {
    double t = dy / dx;
    *cs = 1.0 / sqrt(1.0 + t * t);
    *sn = t * *cs;
  }
}
static void app_givens(double *dx, double *dy, double cs, double sn) {
  double t = cs * *dx + sn * *dy;
  *dy = -sn * *dx + cs * *dy;
  *dx = t;
}

typedef struct {
  double initial, previous;
} loop_info;

/* IterativeMethod::converged (IterativeMethod.h:83-163); returns 1 to stop,
 * 2 on divergence */
static int converged(const orc_solver_config *s, loop_info *li, double res,
                     int it) {
  if (it == 0) {
    li->initial = res;
    li->previous = res;
  }
  int small = res < s->tol_abs;
  int red = res < s->reduction * li->initial;
  int enough = it >= s->min_it;
  int stag = res > 1e10 * li->previous;
  int div = res > s->divergence * li->initial;
  int conv = (small || red || stag || div) && enough;
  if (it == s->max_it) conv = 1;
  li->previous = res;
  if (div) return 2;
  return conv;
}

static void precond(orc_problem *p, const orc_solver_config *s,
                    const double *v, double *z) {
  level_t *L = &p->lev[0];
  if (s->precond == 1) {
    for (int i = 0; i < L->ndof; ++i) z[i] = v[i] / L->diag[i];
  } else if (s->precond == 2) {
    orc_mg_apply(p, s, v, z);
  } else {
    memcpy(z, v, sizeof(double) * L->ndof);
  }
}

/* Iteration_gmres::flexible_gmres (Iteration_gmres.C:430-620) */
int orc_solve(orc_problem *p, const orc_solver_config *s, int *iters,
              double *residual, double *initial) {
  level_t *L = &p->lev[0];
  int n = L->ndof, m = s->restart;
  if (s->precond == 2) {
    if (s->mg_levels > p->nlev) FAIL("not enough levels for multigrid");
    for (int k = 0; k < s->mg_levels; ++k)
      for (int r = 0; r < p->lev[k].ndof; ++r)
        if (p->lev[k].diag[r] == 0) FAIL("zero diagonal entry");
    level_t *crs = &p->lev[s->mg_levels - 1];
    if (s->coarse_direct) {
      if (coarse_factor(crs)) return -1;
      crs->lu_gen = p->asm_gen;
    }
  } else if (s->precond == 1) {
    for (int r = 0; r < n; ++r)
      if (L->diag[r] == 0) FAIL("zero entry on the diagonal using Jacobi");
  }
  double *x = L->sol, *b = L->rhs;
  double *r = (double *)malloc(sizeof(double) * n);
  double **v = (double **)malloc(sizeof(double *) * (m + 1));
  double **z = (double **)malloc(sizeof(double *) * (m + 1));
  for (int i = 0; i <= m; ++i) {
    v[i] = (double *)malloc(sizeof(double) * n);
    z[i] = (double *)malloc(sizeof(double) * n);
  }
  double *H = (double *)calloc((size_t)(m + 1) * (m + 1), sizeof(double));
  double *sv = (double *)calloc(m + 1, sizeof(double));
  double *cs = (double *)calloc(m + 1, sizeof(double));
  double *sn = (double *)calloc(m + 1, sizeof(double));
  loop_info li = {0, 0};
#define HH(i, j) H[(size_t)(i) * (m + 1) + (j)]
  memcpy(r, b, sizeof(double) * n);
  apply_scaled_add(L, x, r, -1.0);
  double resid = sqrt(dot(n, r, r));
  double beta = resid;
  int rc = 0, done = 0, jj = 1;
  *initial = resid;
  if (converged(s, &li, resid, 0)) {
    *iters = 0;
    *residual = resid;
    done = 1;
  }
  while (!done && jj <= s->max_it) {
    for (int i = 0; i < n; ++i) v[0][i] = r[i] * (1.0 / beta);
    memset(sv, 0, sizeof(double) * (m + 1));
    sv[0] = beta;
    int i;
    for (i = 0; i < m && jj <= s->max_it; ++i, ++jj) {
      precond(p, s, v[i], z[i]);
      orc_apply(p, 0, z[i], r);
      if (s->classical_gs) {
        for (int k = 0; k <= i; ++k) HH(k, i) = dot(n, r, v[k]);
        for (int k = 0; k <= i; ++k) {
          double h = -HH(k, i);
          for (int t = 0; t < n; ++t) r[t] += h * v[k][t];
        }
      } else {
        for (int k = 0; k <= i; ++k) {
          HH(k, i) = dot(n, r, v[k]);
          double h = -HH(k, i);
          for (int t = 0; t < n; ++t) r[t] += h * v[k][t];
        }
      }
      HH(i + 1, i) = sqrt(dot(n, r, r));
      if (HH(i + 1, i) != 0.0) {
        double sc = 1.0 / HH(i + 1, i);
        for (int t = 0; t < n; ++t) v[i + 1][t] = r[t] * sc;
      } else {
        snprintf(g_err, sizeof g_err, "Unhappy breakdown in flexible gmres");
        rc = -1;
        done = 1;
        break;
      }
      for (int k = 0; k < i; ++k) app_givens(&HH(k, i), &HH(k + 1, i), cs[k], sn[k]);
      gen_givens(HH(i, i), HH(i + 1, i), &cs[i], &sn[i]);
      app_givens(&HH(i, i), &HH(i + 1, i), cs[i], sn[i]);
      app_givens(&sv[i], &sv[i + 1], cs[i], sn[i]);
      resid = fabs(sv[i + 1]);
      int cv = converged(s, &li, resid, jj);
      if (cv) {
        /* Update (Utilities_gmres.C:90-108) */
        double y[128];
        for (int k = 0; k <= i; ++k) y[k] = sv[k];
        for (int k = i; k >= 0; --k) {
          y[k] /= HH(k, k);
          for (int t = k - 1; t >= 0; --t) y[t] -= HH(t, k) * y[k];
        }
        for (int k = 0; k <= i; ++k)
          for (int t = 0; t < n; ++t) x[t] += y[k] * z[k][t];
        *iters = jj;
        *residual = resid;
        if (cv == 2) {
          snprintf(g_err, sizeof g_err, "solver divergence");
          rc = -2;
        }
        done = 1;
        break;
      }
    }
    if (done) break;
    {
      double y[128];
      int k0 = m - 1;
      for (int k = 0; k <= k0; ++k) y[k] = sv[k];
      for (int k = k0; k >= 0; --k) {
        y[k] /= HH(k, k);
        for (int t = k - 1; t >= 0; --t) y[t] -= HH(t, k) * y[k];
      }
      for (int k = 0; k <= k0; ++k)
        for (int t = 0; t < n; ++t) x[t] += y[k] * z[k][t];
    }
    memcpy(r, b, sizeof(double) * n);
    apply_scaled_add(L, x, r, -1.0);
    beta = sqrt(dot(n, r, r));
    int cv = converged(s, &li, resid, jj);
    if (cv) {
      *iters = jj;
      *residual = resid;
      if (cv == 2) rc = -2;
      done = 1;
    }
  }
  if (!done) {
    *iters = s->max_it;
    *residual = resid;
  }
#undef HH
  for (int i = 0; i <= m; ++i) {
    free(v[i]);
    free(z[i]);
  }
  free(v); free(z); free(r); free(H); free(sv); free(cs); free(sn);
  return rc;
}

/* errors: TFEFunction2D::GetErrors + conv_diff_l2_h1_linf_error */
int orc_errors(const orc_problem *p, double *errors) {
  const orc_config *c = &p->cfg;
  const level_t *L = &p->lev[0];
  int dim = c->dim, nl = L->nloc;
  double e[5] = {0, 0, 0, 0, 0};
  double maxe = 0;
  for (int cell = 0; cell < L->ncells; ++cell) {
    const double *cv = L->verts + (size_t)cell * L->nv * dim;
    affine_t A;
    cell_affine_s(p->shape, dim, cv, &A);
    const int multi = cell_is_multilinear(p->shape, dim, cv);
    double hK = cell_hK_s(p->shape, dim, cv, c->cell_measure);
    double fv[MAXLOC];
    for (int k = 0; k < nl; ++k) fv[k] = L->sol[L->gdof[cell * nl + k]];
    for (int q = 0; q < p->qr.nqp; ++q) {
      if (multi) multilinear_at(dim, cv, p->qr.xi[q], &A);
      double ref[MAXLOC][NDER];
      basis_s(p->shape, dim, c->order, p->qr.xi[q], ref);
      double der[4] = {0, 0, 0, 0};
      for (int k = 0; k < nl; ++k) {
        der[0] += fv[k] * ref[k][0];
      }
      for (int r = 0; r < dim; ++r) {
        double s = 0;
        for (int k = 0; k < nl; ++k) {
          double g = 0;
          for (int a = 0; a < dim; ++a) g += A.Jinv[a][r] * ref[k][1 + a];
          s += fv[k] * g;
        }
        der[1 + r] = s;
      }
      double x[3], u[6], co[8];
      if (multi)
        for (int r = 0; r < dim; ++r) x[r] = A.x0[r];
      else
        affine_map(dim, &A, p->qr.xi[q], x);
      exact_sol(c, x, u);
      coeffs_at(c, x, co);
      double le = fabs(u[0] - der[0]);
      if (le > maxe) maxe = le;
      double nu = co[0], bb[3] = {co[1], co[2], dim == 3 ? co[3] : 0};
      double react = co[dim + 1];
      double bn = fmax(fabs(bb[0]), fabs(bb[1]));
      if (dim == 3) bn = fmax(bn, fabs(bb[2]));
      double delta = sdfem_delta(c, p->shape, cv, 0.0, 0.0, hK, nu, bb, react, bn);
      double w = p->qr.w[q] * fabs(A.det);
      double e0 = der[0] - u[0];
      e[0] += w * e0 * e0;
      double e1 = der[1] - u[1], e2 = der[2] - u[2];
      double e3 = dim == 2 ? 0. : der[3] - u[3];
      e[1] += w * e1 * e1;
      e[1] += w * e2 * e2;
      e[1] += w * e3 * e3;
      double e4 = bb[0] * e1 + bb[1] * e2;
      if (dim == 3) e4 += bb[2] * e3;
      e[2] += w * (nu * (e1 * e1 + e2 * e2 + e3 * e3) + react * e0 * e0 +
                   delta * e4 * e4);
      e[3] += w * (nu * (e1 * e1 + e2 * e2 + e3 * e3) + (e4 + react * e0) * e0);
    }
  }
  errors[0] = sqrt(e[0]);
  errors[1] = sqrt(e[1]);
  errors[2] = sqrt(e[2]);
  errors[3] = sqrt(fabs(e[3]));
  errors[4] = maxe;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* TimeConvectionDiffusion, Crank-Nicolson                                    */
/* ------------------------------------------------------------------------ */
static void ensure_tcd(level_t *L) {
  if (L->tA) return;
  L->tA = (double *)calloc(L->nnz ? L->nnz : 1, sizeof(double));
  L->tM = (double *)calloc(L->nnz ? L->nnz : 1, sizeof(double));
  L->tf = (double *)calloc(L->ndof, sizeof(double));
  L->tfold = (double *)calloc(L->ndof, sizeof(double));
}

/* the scheme of step `step` (TimeDiscretization::set_time_disc_parameters,
 * TimeDiscretizations.C:422-475): BDF2 takes its first step (and the initial
 * assembly, step 0) by bdf_two_first_step; *theta1 = THETA1 */
static int step_scheme(const orc_config *c, int step, double *theta1) {
  int kind = c->time_disc;
  if (kind == ORC_TIME_BDF_TWO && step <= 1)
    kind = c->bdf_first == 1 ? ORC_TIME_CRANK_NICOLSON : ORC_TIME_BACKWARD_EULER;
  *theta1 = kind == ORC_TIME_CRANK_NICOLSON ? 0.5 : kind == ORC_TIME_BACKWARD_EULER ? 1.0 : 2. / 3.;
  return kind;
}

/* TimeConvectionDiffusion::assemble_initial_time (TimeConvectionDiffusion.C
 * call_assembling_routine with assemble_dirichlet_rows): stiffness, mass and
 * rhs at cfg.t on every level, old_rhs = rhs, then the initial condition
 * interpolated into the finest solution (every DOF); solution_m2 =
 * solution_m1 = solution (TimeConvectionDiffusion.C:306-310) */
int orc_tcd_initialize(orc_problem *p) {
  if (p->cfg.time_disc < 0 || p->cfg.time_disc > 2) FAIL("time discretization not supported");
  if (p->cfg.supg) {
    if (!(p->cfg.time_step > 0)) FAIL("SUPG for the time-dependent problem needs the time step");
  }
  double theta1;
  step_scheme(&p->cfg, 0, &theta1);
  p->tcd = 1;
  p->tcd_step = 0;
  if (check_sdfem(&p->cfg, 1)) return -1;
  p->ttau = theta1 * p->cfg.time_step;
  p->tau = p->cfg.time_step;
  p->theta1 = theta1;
  for (int k = 0; k < p->nlev; ++k) {
    level_t *L = &p->lev[k];
    ensure_tcd(L);
    if (assemble_into(p, k, L->tA, L->tf, 1, L->tM)) return -1;
    memcpy(L->tfold, L->tf, sizeof(double) * L->ndof);
  }
  level_t *F = &p->lev[0];
  int dim = p->cfg.dim, nl = F->nloc;
  for (int cell = 0; cell < F->ncells; ++cell) {
    const double *cv = F->verts + (size_t)cell * F->nv * dim;
    for (int k = 0; k < nl; ++k) {
      double x[3];
      dof_position_s(p->shape, dim, p->cfg.order, cv, k, x);
      F->sol[F->gdof[cell * nl + k]] = initial_value(&p->cfg, x);
    }
  }
  if (!F->tu2) F->tu2 = (double *)calloc(F->ndof, sizeof(double));
  memcpy(F->tu2, F->sol, sizeof(double) * F->ndof);
  return 0;
}

/* one step of the scheme (TimeDiscretizations.C:117-189 rhs, :195-251 system
 * matrix; TimeConvectionDiffusion::assemble / solve), on active rows
 *   Crank-Nicolson: rhs = tau/2 f_new + tau/2 f_old + M u1 - tau/2 A u1,
 *                   S = tau/2 A + M
 *   backward Euler: rhs = tau f_new + M u1, S = tau A + M
 *   BDF2:           rhs = (2/3 tau) f_new + 4/3 M u1 - 1/3 M u2,
 *                   S = (2/3 tau) A + M
 * (u1 the last solution, u2 the one before); non-active rows: rhs = f_new
 * (Dirichlet data at t_new), copied into u, and S keeps the rows of A.  The
 * SUPG parameter takes THETA1 * tau.  Then FGMRES on S from u1 */
int orc_tcd_step(orc_problem *p, double t_new, double tau, const orc_solver_config *s,
                 int *iterations, double *residual, double *initial_residual) {
  if (!p->lev[0].tA) FAIL("call orc_tcd_initialize first");
  if (!(tau > 0)) FAIL("time step must be positive");
  if (p->cfg.time_disc < 0 || p->cfg.time_disc > 2) FAIL("time discretization not supported");
  double theta1;
  const int kind = step_scheme(&p->cfg, ++p->tcd_step, &theta1);
  p->cfg.t = t_new;
  p->tcd = 1;
  p->ttau = theta1 * tau;
  p->tau = tau;
  p->theta1 = theta1;
  /* with SUPG the mass matrix is reassembled too (TimeConvectionDiffusion.C
   * assemble: TCDStiffMassRhs, assemble_both) */
  for (int k = 0; k < p->nlev; ++k) {
    level_t *L = &p->lev[k];
    if (assemble_into(p, k, L->tA, L->tf, 1, p->cfg.supg ? L->tM : NULL)) return -1;
  }
  level_t *F = &p->lev[0];
  const double c_new = kind == ORC_TIME_BDF_TWO ? (2. / 3.) * tau : theta1 * tau;
  for (int r = 0; r < F->ndof; ++r) {
    if (r < F->nactive) {
      double sa = 0, sm = 0, sm2 = 0;
      for (int n = F->row_ptr[r]; n < F->row_ptr[r + 1]; ++n) {
        sa += F->tA[n] * F->sol[F->col[n]];
        sm += F->tM[n] * F->sol[F->col[n]];
        sm2 += F->tM[n] * F->tu2[F->col[n]];
      }
      double v = c_new * F->tf[r];
      if (kind == ORC_TIME_CRANK_NICOLSON) {
        v += c_new * F->tfold[r];
        v += sm;
        v += -c_new * sa;
      } else if (kind == ORC_TIME_BDF_TWO) {
        v += (4. / 3.) * sm;
        v += (-1. / 3.) * sm2;
      } else {
        v += sm;
      }
      F->rhs[r] = v;
    } else {
      F->rhs[r] = F->tf[r];
    }
  }
  memcpy(F->tfold, F->tf, sizeof(double) * F->ndof);
  memcpy(F->tu2, F->sol, sizeof(double) * F->ndof);   /* solution_m2 = solution_m1 */
  for (int r = F->nactive; r < F->ndof; ++r) F->sol[r] = F->rhs[r];
  const double factor = kind == ORC_TIME_BDF_TWO ? tau * (2. / 3.) : theta1 * tau;
  for (int k = 0; k < p->nlev; ++k) {
    level_t *L = &p->lev[k];
    int nae = L->row_ptr[L->nactive];
    for (int n = 0; n < L->nnz; ++n)
      L->val[n] = n < nae ? L->tA[n] * factor + L->tM[n] : L->tA[n];
    for (int r = 0; r < L->ndof; ++r)
      for (int n = L->row_ptr[r]; n < L->row_ptr[r + 1]; ++n)
        if (L->col[n] == r) L->diag[r] = L->val[n];
  }
  p->asm_gen++;
  return orc_solve(p, s, iterations, residual, initial_residual);
}

int orc_get_tcd_matrix(const orc_problem *p, int level, int which, double *val) {
  if (level < 0 || level >= p->nlev || which < 0 || which > 2) FAIL("bad arguments");
  const level_t *L = &p->lev[level];
  if (!L->tA) FAIL("no time-dependent matrices");
  const double *src = which == 0 ? L->tA : which == 1 ? L->tM : L->val;
  memcpy(val, src, sizeof(double) * L->nnz);
  return 0;
}
