/*
 * cd_oracle.h -- CPU restatement of ParMooN's scalar convection-diffusion
 * hot path (assembly + FGMRES/Jacobi/multigrid solve + error norms).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it.  Nothing in parmoon2022_gb300/ links or calls it.
 *
 * Every routine names the reference file:line it restates (paths relative to
 * the ParMooN2022 source tree).  Parity of this restatement is pinned against
 * the reference's own golden values (test/cd2d_test.c++ error norms,
 * test/structure_test.c++ pattern counts) by tests/test_oracle_golden.py.
 */
#ifndef CD_ORACLE_H
#define CD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* example ids: problem data (coefficients, exact solution, boundary data) */
enum {
  ORC_EX_SINE_LAPLACE = 0, /* include/Examples/CD_2D/SineLaplace.h (ex. 0)   */
  ORC_EX_SINE = 1,         /* u = prod sin(k pi x_i), homogeneous Dirichlet    */
  ORC_EX_POLYEXP = 2,      /* u = x y z (1-x)(1-y)(1-z) exp(x) (3D)            */
  ORC_EX_CONST_F = 3,      /* f = 1, homogeneous Dirichlet, no exact solution  */
  ORC_EX_POLY1 = 4,        /* u = 1 + x + 2y (+3z): inside Q1, Dirichlet       */
  ORC_EX_BUMP = 5,         /* f = 0, u_D = 0, u0 = exp(-|x-c|^2/(2 s^2))       */
  ORC_EX_POLY1_T = 6,      /* u = (1+t)(1 + x + 2y (+3z))                      */
  ORC_EX_EXP_SIN = 7,      /* u = e^{sin 2 pi t} prod sin(2 pi x_i) (TCD2D example 0,
                              include/Examples/TCD_2D/exp.h)                   */
  ORC_EX_LINEAR_ST = 8,    /* u = 1 + 2x + 3ty (+4tz) (TCD example -2,
                              include/Examples/TCD_3D/linear_space_time.h)     */
  ORC_EX_QUAD_ST = 9       /* u = t^2 (x^2 + yz) (TCD3D example -1,
                              include/Examples/TCD_3D/quadratic_space_time.h)  */
};

/* TimeDiscretization schemes (src/TimeDiscRoutines/TimeDiscretizations.C) */
enum { ORC_TIME_CRANK_NICOLSON = 0, ORC_TIME_BACKWARD_EULER = 1, ORC_TIME_BDF_TWO = 2 };

typedef struct {
  int dim;             /* 2 or 3                                              */
  int order;           /* 1 (Q1) or 2 (Q2)                                    */
  int nref;            /* refinement steps of the unit square / cube         */
  int example;         /* ORC_EX_*                                            */
  double eps;          /* diffusion coefficient                               */
  double b[3];         /* convection                                          */
  double c;            /* reaction                                            */
  double freq;         /* k in sin(k pi x) for ORC_EX_SINE                    */
  int supg;            /* 0: galerkin, 1: supg                                */
  int sdfem_type;      /* TDatabase SDFEM_TYPE                                */
  double delta0, delta1;
  int cell_measure;    /* TDatabase CELL_MEASURE                              */
  int problem_linear;  /* TDatabase INTERNAL_PROBLEM_LINEAR (quad. degree)    */
  int neumann_mask;    /* bit k: boundary component k is Neumann              */
  int poly_degree;     /* TDatabase INTERNAL_POLYNOMIAL_DEGREE (SDFEM 1/2)    */
  int tetra;           /* cells are tetrahedra (P1/P2); arrays constructor    */
  double b_grad[9];    /* b_i(x) = b[i] + sum_j b_grad[3i+j] x_j              */
  double t;            /* time of f and the boundary data                     */
  double ic[4];        /* ORC_EX_BUMP centre and sigma                        */
  double time_step;    /* TIMESTEPLENGTH at orc_tcd_initialize (SUPG only)    */
  int time_disc;       /* ORC_TIME_*                                          */
  int bdf_first;       /* first BDF2 step: 0 backward Euler, 1 Crank-Nicolson */
} orc_config;

typedef struct {
  int precond;         /* 0 none, 1 jacobi, 2 multigrid                        */
  int max_it, min_it, restart;
  double tol_abs;      /* residual_tolerance (absolute)                       */
  double reduction;    /* residual_reduction                                  */
  double divergence;   /* divergence_factor                                   */
  int mg_levels;       /* multigrid_n_levels                                  */
  int mg_cycle;        /* 0 V, 1 W, 2 F                                       */
  int n_pre, n_post;
  double jacobi_damp;
  double correction_damp;
  int coarse_direct;   /* 1: direct_solve (dense LU), 0: jacobi iterations    */
  double coarse_eps;
  int coarse_maxit;
  int classical_gs;    /* 1: all inner products first (Iteration_gmres.C:515-527)
                          0: modified Gram-Schmidt (:528-534)                */
} orc_solver_config;

typedef struct orc_problem orc_problem;

/* n_levels grids: level 0 is the finest (nref refinements), level k has
 * nref-k refinements. */
orc_problem *orc_create(const orc_config *cfg, int n_levels);
void orc_destroy(orc_problem *p);
/* levels from the caller's arrays (finest first): cell vertices, DOF map,
 * numbers of DOFs / actives and CSR pattern per level; parents implied by
 * regular refinement (fine cell f has coarse parent f / 2^dim) */
orc_problem *orc_create_from_arrays(const orc_config *cfg, int n_levels,
                                    const int *ncells, const double *const *verts,
                                    const int *const *gdof, const int *ndof,
                                    const int *nactive, const int *const *row_ptr,
                                    const int *const *col);
/* TimeConvectionDiffusion with Crank-Nicolson: initialize (assemble stiffness,
 * mass and rhs at cfg.t on every level, interpolate the initial condition),
 * one step to time t_new with time step tau, matrices for parity checks */
int orc_tcd_initialize(orc_problem *p);
int orc_tcd_step(orc_problem *p, double t_new, double tau, const orc_solver_config *s,
                 int *iterations, double *residual, double *initial_residual);
/* which: 0 stiffness, 1 mass, 2 system */
int orc_get_tcd_matrix(const orc_problem *p, int level, int which, double *val);

/* info[0..5] = ncells, nloc, ndof, nactive, nnz, nverts_per_cell */
int orc_level_info(const orc_problem *p, int level, int *info);
int orc_get_mesh(const orc_problem *p, int level, double *verts);
int orc_get_gdof(const orc_problem *p, int level, int *gdof);
int orc_get_structure(const orc_problem *p, int level, int *row_ptr, int *col);
int orc_get_matrix(const orc_problem *p, int level, double *val);
int orc_get_rhs(const orc_problem *p, int level, double *rhs);
int orc_get_solution(const orc_problem *p, double *sol);
int orc_set_solution(orc_problem *p, const double *sol);

/* ConvectionDiffusion<d>::assemble over all levels */
int orc_assemble(orc_problem *p);
/* quadrature points of every cell of a level (physical coordinates,
 * x[(cell * nqp + q) * dim + r]); x == NULL returns *nqp only */
int orc_quadrature_points(const orc_problem *p, int level, int *nqp, double *x);
/* assemble one level with coefficients per (cell, quadrature point):
 * co[(cell * nqp + q) * (dim + 3) + k], k = 0 eps, 1..dim b, dim+1 c,
 * dim+2 f (CoeffFct2D/3D, include/General/Constants.h:43-47) */
int orc_assemble_coefficients(orc_problem *p, int level, const double *co);
/* local matrix and rhs of one cell of one level (before scatter) */
int orc_local_system(orc_problem *p, int level, int cell, double *A, double *f);
/* y = A x on active rows, identity on non-active rows (BlockFEMatrix::apply) */
int orc_apply(const orc_problem *p, int level, const double *x, double *y);
/* GridTransfer::Prolongate / DefectRestriction between level+1 (coarse) and
 * level (fine) */
int orc_prolongate(const orc_problem *p, int fine_level, const double *xc,
                   double *xf);
int orc_restrict(const orc_problem *p, int fine_level, const double *df,
                 double *rc);
/* one multigrid cycle as the FGMRES preconditioner: z = MG(v) */
int orc_mg_apply(orc_problem *p, const orc_solver_config *s, const double *v,
                 double *z);
/* Solver::solve on the finest level, starting from the current solution */
int orc_solve(orc_problem *p, const orc_solver_config *s, int *iterations,
              double *residual, double *initial_residual);
/* errors[0..4] = L2, H1-semi, SD, DG(volume), L_inf */
int orc_errors(const orc_problem *p, double *errors);
/* the reference's marker-algorithm DOF numbering (TFESpace3D::ConstructSpace,
 * FESpace3D.C:186-420; compute_various_numbers, FESpace.C:1863-2099) on the
 * caller's tetrahedral mesh: verts[(cell * 4 + v) * 3 + a]; cfg->order 1 or 2,
 * cfg->tetra set, cfg->neumann_mask the Neumann faces of the unit cube;
 * gdof[cell * nloc + k] receives the global numbers */
int orc_marker_numbering(const orc_config *cfg, int ncells, const double *verts, int *gdof,
                         int *ndof, int *nactive);
const char *orc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
