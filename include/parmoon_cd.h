/*
 * parmoon_cd.h -- C-ABI of the GB300 convection-diffusion hot path
 * (libparmoon_cd.so).  Plain C types only: pointers, sizes, int status codes.
 *
 * The library replaces, for scalar convection-diffusion, the following parts
 * of ParMooN2022 (paths inside the ParMooN2022 source tree):
 *   - Assemble2D / Assemble3D with a ConvDiff LocalAssembling object
 *       include/AssembleRoutines/Assemble2D.h:22-34, Assemble3D.h:26-32
 *       src/AssembleRoutines/LocalAssembling.C:211-249 (ConvDiff terms)
 *   - BlockFEMatrix::apply / apply_scaled_add (identity on non-active rows)
 *       src/Matrix/BlockFEMatrix.C:969-1095
 *   - Solver<BlockFEMatrix,BlockVector>::update_matrix + solve with
 *     iterative_solver_type fgmres and preconditioner jacobi | multigrid
 *       src/Solver/Solver.C:423-501,601-696, Iteration_gmres.C:430-620,
 *       src/Multigrid/Multigrid.C:106-410
 *   - ConvectionDiffusion<d>::assemble / solve / output (errors)
 *       include/System/ConvectionDiffusion.h:183-285
 *
 * Error convention: every entry point returns CDG_OK (0) or a negative
 * status; cdg_last_error() gives the message of the calling thread's last
 * failure (the reference throws std::runtime_error via ErrThrow,
 * include/General/MooNMD_Io.h:226-232; a host shim maps status -> ErrThrow).
 *
 * Threading: handles are not thread-safe; one handle is driven by one host
 * thread.  All device work of a context is ordered on the context's stream.
 */
#ifndef PARMOON_CD_H
#define PARMOON_CD_H

#ifdef __cplusplus
extern "C" {
#endif

#define CDG_OK 0
#define CDG_ERR_ARG (-1)          /* invalid argument                        */
#define CDG_ERR_CUDA (-2)         /* CUDA runtime error                      */
#define CDG_ERR_OOM (-3)          /* device allocation failed                */
#define CDG_ERR_DIVERGED (-4)     /* IterativeMethod::converged divergence   */
#define CDG_ERR_BREAKDOWN (-5)    /* FGMRES unhappy breakdown                */
#define CDG_ERR_ZERO_DIAG (-6)    /* zero diagonal entry (Jacobi)            */
#define CDG_ERR_PATTERN (-7)      /* local coupling missing in the pattern   */
#define CDG_ERR_SINGULAR (-8)     /* singular coarse matrix                  */
#define CDG_ERR_NO_DEVICE (-9)    /* no CUDA device                          */
#define CDG_ERR_LIMIT (-10)       /* size beyond a documented maximum        */
#define CDG_ERR_TIMEOUT (-11)     /* a bounded device-side wait ran out      */

/* example ids: coefficient function + exact solution + boundary data of the
 * problem (the reference's Example_CD2D/Example_CD3D callbacks) */
#define CDG_EX_SINE_LAPLACE 0     /* include/Examples/CD_2D/SineLaplace.h    */
#define CDG_EX_SINE 1             /* u = prod sin(freq pi x_i)               */
#define CDG_EX_POLYEXP 2          /* u = xyz(1-x)(1-y)(1-z)exp(x)            */
#define CDG_EX_CONST_F 3          /* f = 1, u = 0 on the boundary            */
#define CDG_EX_POLY1 4            /* u = 1 + x + 2y (+3z)                    */
#define CDG_EX_BUMP 5             /* f = 0, u = 0 on the boundary, initial
                                     condition exp(-|x-c|^2 / (2 sigma^2))    */
#define CDG_EX_POLY1_T 6          /* u = (1+t)(1 + x + 2y (+3z)), in time     */
#define CDG_EX_EXP_SIN 7          /* u = e^{sin 2 pi t} prod sin(2 pi x_i): the
                                     TCD2D example 0 of the reference's tests
                                     (include/Examples/TCD_2D/exp.h)          */
#define CDG_EX_LINEAR_ST 8        /* u = 1 + 2x + 3ty (+ 4tz): linear in space
                                     and time, example -2 of the TCD tests
                                     (include/Examples/TCD_3D/
                                     linear_space_time.h, TCD_2D/ the same
                                     at z = 0)                                */
#define CDG_EX_QUAD_ST 9          /* u = t^2 (x^2 + yz): quadratic space-time,
                                     example -1 of the TCD3D tests
                                     (include/Examples/TCD_3D/
                                     quadratic_space_time.h)                  */

/* time_discretization (TimeDiscretization, src/TimeDiscRoutines/
 * TimeDiscretizations.C:36-50,117-215,422-475); zero is Crank-Nicolson */
#define CDG_TIME_CRANK_NICOLSON 0
#define CDG_TIME_BACKWARD_EULER 1
#define CDG_TIME_BDF_TWO 2

/* local assembling + example: LocalAssembling<d>(db, ConvDiff, {}, coeffs,
 * disctype) with the TDatabase globals the CD routines read */
typedef struct {
  int example;          /* CDG_EX_*                                           */
  double eps;           /* diffusion coefficient                              */
  double b[3];          /* convection field (constant)                        */
  double c;             /* reaction                                           */
  double freq;          /* CDG_EX_SINE frequency                              */
  int supg;             /* space_discretization_type: 0 galerkin, 1 supg      */
  int sdfem_type;       /* SDFEM_TYPE: 0-2, 4-12 (9-11 time-dependent only);
                           others rejected with CDG_ERR_ARG                   */
  double delta0, delta1;/* DELTA0, DELTA1                                     */
  int cell_measure;     /* CELL_MEASURE: 0 diameter, 1/3 sqrt(measure), 2
                           shortest edge, 4 size in convection direction     */
  int problem_linear;   /* INTERNAL_PROBLEM_LINEAR (quadrature degree 2p)     */
  int neumann_mask;     /* bit k: boundary component k is Neumann             */
  int poly_degree;      /* INTERNAL_POLYNOMIAL_DEGREE (0: element order)      */
  double b_grad[9];     /* convection linear in x: b_i(x) = b[i] + sum_j
                           b_grad[3i+j] x_j (zero: constant field)           */
  double t;             /* time at which f and the boundary data are taken   */
  double ic[4];         /* CDG_EX_BUMP: centre x, y, z and sigma              */
  double time_step;     /* TIMESTEPLENGTH: the time step the SUPG parameter of
                           the time-dependent routines takes at
                           cdg_problem_tcd_initialize (each step uses its own
                           tau); ignored by the stationary problem          */
  int time_discretization; /* CDG_TIME_*: the scheme of cdg_problem_tcd_step  */
  int bdf_two_first_step;  /* bdf_two_first_step, the scheme of the first
                              CDG_TIME_BDF_TWO step: 0 backward Euler (the
                              reference's default), 1 Crank-Nicolson       */
} cdg_assembly_params;

/* Solver ParameterDatabase keys (src/Solver/Solver.C:26-209,
 * src/Multigrid/Multigrid.C:417-509) */
typedef struct {
  int preconditioner;          /* 0 no_preconditioner, 1 jacobi, 2 multigrid */
  int max_n_iterations;
  int min_n_iterations;
  int gmres_restart;
  double residual_tolerance;   /* absolute                                   */
  double residual_reduction;
  double divergence_factor;
  int multigrid_n_levels;
  int multigrid_cycle_type;    /* 0 V, 1 W, 2 F                              */
  int multigrid_n_pre_smooth;
  int multigrid_n_post_smooth;
  double jacobi_damp;
  double multigrid_correction_damp_factor;
  int multigrid_smoother_coarse; /* 0 direct_solve, 1 jacobi                 */
  double multigrid_coarse_residual;
  int multigrid_coarse_max_n_iterations;
  int precision;               /* 0: all FP64, 1: FP32 multigrid in FP64 FGMRES */
  int gram_schmidt;            /* Arnoldi orthogonalisation: 0 classical, all
                                  inner products first (Iteration_gmres.C:
                                  515-527), 1 modified (:528-534)            */
} cdg_solver_params;

typedef struct {
  int iterations;
  double residual;             /* final Givens residual estimate             */
  double initial_residual;
  double seconds;              /* wall time of the call                      */
} cdg_solve_stats;

#define CDG_CELL_QUAD 2
#define CDG_CELL_HEXA 3
#define CDG_CELL_TETRA 4

typedef struct cdg_context cdg_context;     /* device + stream + scratch       */
typedef struct cdg_hierarchy cdg_hierarchy; /* host mesh/space/pattern levels  */
typedef struct cdg_problem cdg_problem;     /* ConvectionDiffusion<d>          */

const char *cdg_last_error(void);
int cdg_version(void);

/* ---- context ------------------------------------------------------------ */
int cdg_context_create(int device, cdg_context **out);
/* destroy every problem of the context before the context itself */
int cdg_context_destroy(cdg_context *ctx);
int cdg_context_synchronize(cdg_context *ctx);
/* number of kernel launches the context issued since creation */
long long cdg_context_launch_count(const cdg_context *ctx);
/* the context's CUDA stream (a cudaStream_t), for callers that order their
 * own work or record timing events against the library's launches */
int cdg_context_stream(cdg_context *ctx, void **stream);

/* ---- host setup layer (no GPU) ------------------------------------------ */
/* TDomain(unit square/cube split into roots^dim cells) refined nref times,
 * TFESpace of Q_order, TStructure per level and the grid transfers; level 0
 * is the finest, level k has nref-k refinements (refine_and_get_hierarchy_
 * of_collections, src/Geometry/Domain.C:2796-2906; FESpace2D.C:83-312;
 * Structure.C:226-618; GridTransfer.C:29-410) */
int cdg_hierarchy_create(int dim, int order, int roots, int nref, int n_levels,
                         int neumann_mask, cdg_hierarchy **out);
/* move the finest level's interior vertices of a hierarchy by amplitude * h
 * in every coordinate (uniform, seeded; h = 1 / cells per direction), after
 * numbering: quadrilaterals and hexahedra become general (non-parallelogram,
 * non-parallelepiped) cells, mapped by the reference's bilinear / trilinear
 * maps (TQuadBilinear, THexaTrilinear); the coarser levels and the grid
 * transfers keep the nested positions.  amplitude in [0, 0.5). */
int cdg_hierarchy_perturb(cdg_hierarchy *h, double amplitude, unsigned long long seed);
/* unit cube split into roots^3 cubes of 6 Kuhn tetrahedra, P1 or P2 (order),
 * refined nref times (regular refinement, children of cell c are the eight
 * cells 8c..8c+7 of the next level); neumann_mask as above (bit k: boundary
 * face k of the cube is Neumann); perturb > 0 moves every interior vertex
 * of the finest level by perturb*h*U(-1,1) per coordinate (seeded), as the
 * perturbed-tetrahedra configuration of TCD3D asks */
int cdg_hierarchy_create_tetra(int order, int roots, int nref, int n_levels,
                               int neumann_mask, double perturb,
                               unsigned long long seed, cdg_hierarchy **out);
/* the same hierarchies with the FE space numbering and the TStructure of every
 * level built on the context's GPU (bit-exact with the host builders above) */
int cdg_hierarchy_create_device(cdg_context *ctx, int dim, int order, int roots,
                                int nref, int n_levels, int neumann_mask,
                                cdg_hierarchy **out);
int cdg_hierarchy_create_tetra_device(cdg_context *ctx, int order, int roots,
                                      int nref, int n_levels, int neumann_mask,
                                      double perturb, unsigned long long seed,
                                      cdg_hierarchy **out);
/* TFESpace numbering on the GPU (TFESpace3D::ConstructSpace,
 * src/FE/FESpace3D.C:186; TFESpace::compute_various_numbers,
 * src/FE/FESpace.C:1863-2099): inner DOFs, then non-Dirichlet boundary DOFs,
 * then Dirichlet DOFs, each class in order of first appearance over (cell,
 * local DOF).  Cells of a structured mesh of the unit square / cube (DOFs on
 * a lattice of the first cell's edge length / order); cell_type
 * CDG_CELL_QUAD, CDG_CELL_HEXA or CDG_CELL_TETRA, verts as in
 * cdg_problem_create_from_arrays; gdof receives n_cells * n_local_dofs */
int cdg_space_number_device(cdg_context *ctx, int cell_type, int order,
                            int neumann_mask, int n_cells, const double *verts,
                            int *gdof, int *ndof, int *nactive);
/* TStructure(space) on the GPU (src/Matrix/Structure.C:226-556): rows of
 * every DOF of every cell containing the row's DOF, columns sorted, full rows
 * for Dirichlet DOFs.  row_ptr receives ndof+1 offsets and *nnz the entry
 * count in every case; col receives the columns when col_capacity >= *nnz,
 * otherwise CDG_ERR_LIMIT (call again with a large enough buffer) */
int cdg_structure_build_device(cdg_context *ctx, int n_cells, int n_local_dofs,
                               int ndof, const int *gdof, int *row_ptr, int *col,
                               long long col_capacity, long long *nnz);
int cdg_hierarchy_destroy(cdg_hierarchy *h);
/* info[0..5] = n_cells, n_local_dofs, n_dofs, n_active, nnz, verts_per_cell */
int cdg_hierarchy_level_info(const cdg_hierarchy *h, int level, int *info);
int cdg_hierarchy_get_mesh(const cdg_hierarchy *h, int level, double *verts);
int cdg_hierarchy_get_dofs(const cdg_hierarchy *h, int level, int *global_numbers);
int cdg_hierarchy_get_pattern(const cdg_hierarchy *h, int level, int *row_ptr,
                              int *col);

/* ---- problem: ConvectionDiffusion<d> (src/System/ConvectionDiffusion.C) -- */
/* upload one hierarchy (all its levels) to the device */
int cdg_problem_create(cdg_context *ctx, const cdg_hierarchy *h,
                       cdg_problem **out);
/* drop-in form: the caller's own mesh, DOF map and pattern for n_levels
 * levels (finest first); cell_type CDG_CELL_QUAD (2), CDG_CELL_HEXA (3) or
 * CDG_CELL_TETRA (4): cell_vertices[l] has n_cells[l]*verts*dim doubles in
 * the cell's vertex order, global_numbers[l] n_cells[l]*n_local_dofs ints,
 * row_ptr[l]/col[l] the TStructure, parent[l] (l>=1) the coarse cell of each
 * cell of level l-1 (NULL: cell/2^dim, regular refinement) */
int cdg_problem_create_from_arrays(cdg_context *ctx, int cell_type, int order,
                                   int n_levels, const int *n_cells,
                                   const double *const *cell_vertices,
                                   const int *const *global_numbers,
                                   const int *n_dofs, const int *n_active,
                                   const int *const *row_ptr,
                                   const int *const *col,
                                   const int *const *parent,
                                   cdg_problem **out);
int cdg_problem_destroy(cdg_problem *p);
/* ConvectionDiffusion<d>::assemble: every level (Assemble2D/3D cell loop,
 * LocalAssembling ConvDiff, CSR scatter, Dirichlet rows and data) */
int cdg_problem_assemble(cdg_problem *p, const cdg_assembly_params *a);
/* Solver::solve(A, rhs, sol) on the finest level from the current solution */
int cdg_problem_solve(cdg_problem *p, const cdg_solver_params *s,
                      cdg_solve_stats *stats);
/* assemble + solve with host buffers in and out (the e2e call, the
 * reference's cd.assemble(); cd.solve() with the solution vector as start
 * iterate): solution_in is the start iterate, rhs_out and solution_out
 * receive the finest rhs and solution; all host, n_dofs of level 0, each may
 * be NULL */
int cdg_problem_assemble_solve(cdg_problem *p, const cdg_assembly_params *a,
                               const cdg_solver_params *s,
                               const double *solution_in, double *rhs_out,
                               double *solution_out, cdg_solve_stats *stats);

/* Many small solves in one launch (the served form's batch; no counterpart
 * in the reference, which solves one problem per ConvectionDiffusion::solve
 * call, src/Solver/Iteration_gmres.C:430-620 with Multigrid.C:157-410).  Each
 * problem (assembled, its solution holding the start iterate) is prepared on
 * its own context's stream (FP32 copies, coarse inverse, Krylov buffers);
 * then one kernel on ctx's stream runs one block per problem: FGMRES(m) in
 * FP64 with the FP32 multigrid V-cycle, every operation under block
 * barriers, and each block stops on its own convergence test.  Problems must
 * be distinct, on ctx's device, at most 20000 DOFs, and params[q] must ask
 * for precision 1 (mixed), multigrid (2 to 12 levels, V-cycle, at least one
 * pre-smoothing step, direct coarse solve with at most 2048 active coarse
 * DOFs), classical Gram-Schmidt and gmres_restart <= 64; otherwise
 * CDG_ERR_ARG and nothing runs.  status[q] receives CDG_OK,
 * CDG_ERR_DIVERGED or CDG_ERR_BREAKDOWN as cdg_problem_solve would return;
 * stats[q] the iterations and residuals (seconds: the whole call).  The
 * solutions stay on the device (cdg_problem_get_solution).  Results equal a
 * cdg_problem_solve of the same problem to round-off. */
int cdg_solve_batched(cdg_context *ctx, int count, cdg_problem *const *problems,
                      const cdg_solver_params *params, int *status,
                      cdg_solve_stats *stats);
/* ConvectionDiffusion<d>::output error norms against the example's exact
 * solution: errors[0..4] = L2, H1-semi, SD, DG(volume), L_inf */
int cdg_problem_errors(cdg_problem *p, const cdg_assembly_params *a,
                       double *errors);
/* The same error norms without allocating any device memory (this entry has
 * no counterpart in the reference).  For callers that cannot allocate at
 * this point: an application that hands the GPU's memory to its own pool or
 * budget, or a latency-sensitive loop that must not call cudaMalloc/cudaFree
 * because they can synchronise the device.  Its scratch is a fixed device
 * array of 16384 x 5 + 8 doubles (~640 KB) that every GPU loading the library
 * keeps until exit; it holds one partial sum row per 8 cells, so the finest
 * level may have at most 131,072 cells (larger: CDG_ERR_LIMIT, use
 * cdg_problem_errors).  It evaluates tensor-product bases only
 * (quadrilaterals and hexahedra; tetrahedral levels get CDG_ERR_ARG).
 * Otherwise it accepts what cdg_problem_errors accepts (every example, a
 * convection field linear in x, any time a->t) and returns the same status
 * for what that entry rejects.  The first call on a device looks up the
 * array's device address; make that first call before any stream capture.  All calls
 * share the array: calls that overlap on the GPU (other streams, other host
 * threads) race and must be serialised by the caller. */
int cdg_problem_errors_noalloc(cdg_problem *p, const cdg_assembly_params *a,
                               double *errors);

/* ---- time-dependent CD: TimeConvectionDiffusion<d> -------------------- */
/* assemble_initial_time (src/System/TimeConvectionDiffusion.C:260-311): on
 * every level stiffness, mass and rhs at time a->t (Dirichlet rows assembled
 * in full); the finest solution becomes the interpolant of the example's
 * initial condition.  With SUPG (TCDStiffSUPG, TCDMassSUPG, TCDRhsSUPG,
 * src/General/CD_local_assembling_routines.C:184-387) the stabilisation
 * parameter uses theta1 * a->time_step, which must then be positive; theta1
 * is that of the first step of a->time_discretization.  Resets the step
 * count (TimeDiscretization::current_step_ = 0). */
int cdg_problem_tcd_initialize(cdg_problem *p, const cdg_assembly_params *a);
/* one step to time a->t = t_old + tau of a->time_discretization
 * (TimeConvectionDiffusion.C:315-450, TimeDiscretizations.C:117-283,422-475):
 * reassemble stiffness and rhs on every level (with SUPG the mass matrix too,
 * with the parameter theta1 * tau), then on active rows
 *   Crank-Nicolson  rhs = tau/2 (f_new + f_old) + M u_old - tau/2 A u_old,
 *                   system M + tau/2 A          (theta1 = 1/2)
 *   backward Euler  rhs = tau f_new + M u_old, system M + tau A (theta1 = 1)
 *   BDF2            rhs = 2/3 tau f_new + 4/3 M u_old - 1/3 M u_older,
 *                   system M + 2/3 tau A        (theta1 = 2/3)
 * where the first step after cdg_problem_tcd_initialize of BDF2 is taken by
 * a->bdf_two_first_step; Dirichlet data at the new time, then Solver::solve
 * warm-started from u_old */
int cdg_problem_tcd_step(cdg_problem *p, const cdg_assembly_params *a, double tau,
                         const cdg_solver_params *s, cdg_solve_stats *stats);
/* which: 0 stiffness A, 1 mass M, 2 system matrix (after a step) */
int cdg_problem_get_tcd_matrix(cdg_problem *p, int level, int which,
                               double *values);

/* ---- checkpoints (src/FE/CheckpointIO.C, src/Matrix/BlockVector.C) ---- */
/* BlockVector::write_to_file (BlockVector.C:1064-1126): a text line with the
 * entry count, then the n entries as raw native doubles.  A file that cannot
 * be opened returns CDG_ERR_ARG (the reference prints a warning and returns) */
int cdg_vector_write_file(const char *filename, const double *v, long long n);
/* BlockVector::read_from_file (BlockVector.C:1075-1136): the first line must
 * hold only the entry count (else CDG_ERR_ARG, "formatting error");
 * n_expected > 0: the count must equal it (else CDG_ERR_ARG, "unexpected size
 * to be read"), 0: any count up to capacity (beyond: CDG_ERR_LIMIT).
 * *n_read receives the file's count whenever the first line parses */
int cdg_vector_read_file(const char *filename, double *v, long long capacity,
                         long long n_expected, long long *n_read);
/* CheckpointIO file name: base, or base + "." + std::to_string(time) unless
 * overwrite (CheckpointIO.C:68-93) */
int cdg_checkpoint_file_name(const char *base, double time, int overwrite,
                             char *out, long long capacity);
/* the finest-level solution to / from a file in that format
 * (ConvectionDiffusion: checkpoint_io.write / read, ConvectionDiffusion.C:162,307) */
int cdg_problem_write_solution(cdg_problem *p, const char *filename);
int cdg_problem_read_solution(cdg_problem *p, const char *filename);
/* CheckpointIO::write(data, time_stepping_scheme) (CheckpointIO.C:68-93):
 * writes the solution after every_n_steps completed steps, never at step 0,
 * into the CheckpointIO file name; *written = 1 when a file was written.
 * A restart is cdg_problem_tcd_initialize at the checkpoint's time followed
 * by cdg_problem_read_solution (the reference reads the checkpoint over the
 * interpolated initial condition, TimeConvectionDiffusion.C:112-149) */
int cdg_problem_checkpoint(cdg_problem *p, const char *base, int step, double time,
                           int every_n_steps, int overwrite, int *written);

/* ---- data access (host buffers) ----------------------------------------- */
int cdg_problem_level_info(const cdg_problem *p, int level, int *info);
/* storage and kernels of the level's operators on the device (no reference
 * counterpart: ParMooN keeps CSR only): *lanes = 0 for a CSR FP64 operator,
 * otherwise the sliced ELLPACK copy with *lanes lanes per row and *slots
 * stored entries (padding included); *smoother_chunk = 0 when the FP32
 * smoother streams CSR through registers, otherwise the entries per chunk it
 * stages through shared memory */
int cdg_problem_operator_layout(const cdg_problem *p, int level, int *lanes,
                                long long *slots, int *smoother_chunk);
/* The DOF lattice of a uniform Q2 hexahedral level (no counterpart in the
 * reference): dims[0..2] its extents in cell 0's axes (0 when the level is
 * not a full lattice with Dirichlet data on its whole boundary, or before
 * its first assembly); *transfer the grid transfer to the next coarser
 * level: -1 not decided yet (decided at the first multigrid solve or
 * transfer call after both levels are assembled, with CDG_LAT_TRANSFER=1 in
 * the environment; otherwise the CSR matrices are used), 0 the CSR
 * matrices, 1 the lattice kernels (tensor-product Q2 interpolation, every
 * row of P checked against it; slower than the CSR kernels on GB300). */
int cdg_problem_lattice(const cdg_problem *p, int level, int *dims, int *transfer);
int cdg_problem_get_matrix(cdg_problem *p, int level, double *values);
int cdg_problem_get_rhs(cdg_problem *p, int level, double *rhs);
int cdg_problem_get_solution(cdg_problem *p, double *sol);
/* sol == NULL sets the solution to zero on the device */
int cdg_problem_set_solution(cdg_problem *p, const double *sol);
/* CSR slot of every local coupling: slots[cell*nloc*nloc + i*nloc + j] */
int cdg_problem_get_slots(cdg_problem *p, int level, int *slots);

/* ---- operator pieces (host buffers) ------------------------------------- */
/* y = A x (BlockFEMatrix::apply) */
int cdg_problem_apply(cdg_problem *p, int level, const double *x, double *y);
/* GridTransfer::Prolongate (coarse level fine_level+1 -> fine_level) */
int cdg_problem_prolongate(cdg_problem *p, int fine_level, const double *xc,
                           double *xf);
/* GridTransfer::DefectRestriction (fine_level -> fine_level+1) */
int cdg_problem_restrict(cdg_problem *p, int fine_level, const double *df,
                         double *rc);
/* ---- coefficients from the caller (the reference's CoeffFct2D/3D) ------ */
/* An Example_CD2D/3D built from coefficient callbacks
 * (include/Examples/Example_CD2D.h:67-71) has
 *   CoeffFct2D/3D(n_points, x, y[, z], params, coeffs)
 * (include/General/Constants.h:43-47), called by LocalAssembling on the
 * quadrature points of every cell.  Here the caller asks for the points of a
 * level, evaluates its callback on them and hands the values back:
 *
 * cdg_problem_quadrature_points: *nqp = points per cell of the rule the
 * assembly uses for a (the rule by degree of the reference's
 * QuadratureFormulaDatabase, as for the built-in examples); x (may be NULL to
 * query *nqp) receives n_cells * nqp * dim physical coordinates,
 * x[(cell * nqp + q) * dim + r].
 *
 * cdg_problem_assemble_coefficients: assembles the matrix and rhs of one
 * level (Galerkin, or SUPG with delta per point from the point's
 * coefficients, Compute_SDFEM_delta) from coeffs[(cell * nqp + q) * (dim + 3)
 * + k], k = 0 eps, 1..dim b, dim+1 c, dim+2 f -- the reference's
 * coefficient vector layout (src/AssembleRoutines/ConvDiff.C:1858-1863).
 * Dirichlet values come from a->example's boundary data; Neumann parts are
 * rejected (CDG_ERR_ARG).  Call it once per multigrid level, as the
 * reference assembles every level; such levels keep the CSR multigrid
 * kernels. */
int cdg_problem_quadrature_points(cdg_problem *p, const cdg_assembly_params *a,
                                  int level, int *nqp, double *x);
int cdg_problem_assemble_coefficients(cdg_problem *p, const cdg_assembly_params *a,
                                      int level, const double *coeffs);
/* y = A x with the FP32 copy of a level's operator that the mixed-precision
 * multigrid smooths with (JacobiSmoother's BlockFEMatrix::apply, identity on
 * non-active rows), host float buffers of n_dofs entries.  variant 0: CSR
 * kernel; 1: matrix-free kernel (Q2 hexahedra after a stationary assembly,
 * the element matrices applied from per-cell factors or, on uniform levels,
 * from one shared element matrix in one launch per product); 2: the
 * matrix-free product as two launches (cell products, then the row sums),
 * which the one-launch form equals bit for bit; 3: the lattice stencil
 * sweep (uniform Q2 levels whose DOFs fill a lattice with Dirichlet data on
 * the whole boundary: each active row one of eight 125-point stencils summed
 * from the element matrix; CDG_ERR_ARG on other levels).  Parity access for
 * the multigrid kernels. */
int cdg_problem_apply32(cdg_problem *p, int level, int variant, const float *x,
                        float *y);
/* Operators used only in FP32 on tensor cores (no counterpart in the
 * reference, which assembles every level in double).  enable = 1: the next
 * assemblies form the matrices of the levels between the finest and the
 * coarsest -- which the mixed-precision multigrid uses only as FP32 copies
 * -- by a tcgen05 contraction of the cell factors with the reference
 * tensors, split TF32 with FP32 accumulation (FP32-level accuracy), instead
 * of the FP64 contraction.  Their FP64 values are formed when something
 * needs them (an FP64 multigrid solve, cdg_problem_get_matrix,
 * cdg_problem_apply), from the parameters of their last assembly.
 * Stationary assembly only (cdg_problem_assemble); SUPG with a convection
 * field linear in x keeps the FP64 path. */
int cdg_problem_set_fp32_tensor_levels(cdg_problem *p, int enable);
/* the FP32 values the multigrid smooths with (nnz floats, CSR order) */
int cdg_problem_get_matrix32(cdg_problem *p, int level, float *v);
/* the FP32 multigrid schedule chosen for a level (no counterpart in the
 * reference, which has one kernel).  At the first mixed-precision multigrid
 * solve every level above the coarsest is tuned once by timing one smoothing
 * step of each candidate (CUDA events): CSR lanes per row 2/4/8/16, and on Q2
 * hexahedra with a matrix-free operator its grid (one cell per warp, or 4 / 8
 * blocks per SM; uniform levels sweep in one launch of one block per 256
 * rows, or, on a lattice with Dirichlet data on the whole boundary, by the
 * stencil sweep with 4 or 8 lattice points per thread) and then CSR against
 * matrix-free.  *choice: -2 not tuned
 * yet, -1 CSR (no matrix-free operator), 0 CSR, 1 matrix-free; shape (may be
 * NULL): [0] FP32 CSR lanes per row, [1] matrix-free blocks per SM (0: one
 * cell per warp; -4, -5, -6: the one-launch sweep compiled for that many
 * resident blocks per SM; -104, -108: the stencil sweep with 4 or 8 points
 * per thread); ms (may be NULL): the best CSR and the best matrix-free
 * step in milliseconds (0 where not timed).  CDG_TUNE=0 in the environment
 * keeps the untuned defaults; CDG_MATFREE, CDG_TPR32, CDG_MF_CAP, CDG_MF_MINB
 * and CDG_MF_STENCIL (0: no stencil sweep, 4 or 8: that sweep; one value, or
 * one per level from the finest, comma-separated) fix choices. */
int cdg_problem_tuning(cdg_problem *p, int level, int *choice, int *shape, double *ms);
/* one preconditioner application z = M^-1 v (Iteration_multigrid::apply or
 * Iteration_jacobi::apply) */
int cdg_problem_precondition(cdg_problem *p, const cdg_solver_params *s,
                             const double *v, double *z);

/* ---- measurement -------------------------------------------------------- */
/* average device time (ms) of one launch of a hot kernel on `level`, from
 * CUDA events around `reps` back-to-back launches on the context stream.
 * kernel: 0 multigrid Jacobi smoothing step in FP32 (x' = x + w D^-1 (b-Ax)),
 *         1 FP64 operator SpMV (y = A x),
 *         2 element contraction + CSR scatter of the matrix (FP64),
 *         3 FP32 defect (d = b - A x).
 * Kernel 2 re-assembles the level afterwards (a is required for it). */
int cdg_problem_time_kernel(cdg_problem *p, const cdg_assembly_params *a,
                            int kernel, int level, int reps, double *ms);

/* ------------------------------------------------------------------------ */
/* Request server: stationary CD solves of differing meshes and coefficients,
 * served concurrently on one GPU.  Replaces a driver that constructs a
 * ConvectionDiffusion<d> per request and calls assemble() + solve()
 * (src/System/ConvectionDiffusion.C:112-281): here the meshes, CSR matrices,
 * multigrid hierarchies and Krylov state of each mesh class stay resident on
 * the device between requests.
 *
 * n_slots workers each own a stream; a request waits in the queue until a
 * slot is free and its problem instance fits the HBM budget (idle instances
 * are evicted least recently used first), then assemble + solve run on the
 * slot's stream, overlapping with the other slots' work on the device.  A
 * small request that cdg_solve_batched takes is assembled on its slot and
 * then solved by a batcher thread together with every other such request
 * handed over since the batcher's previous launch (one launch, one block per
 * request); its result's slot is then n_slots. */
typedef struct cdg_server cdg_server;

typedef struct {
  int dim;                 /* 2 or 3                                           */
  int order;               /* 1 (Q1) or 2 (Q2)                                 */
  int n;                   /* cells per direction: roots * 2^k, roots 1 or 3   */
  cdg_assembly_params a;   /* coefficients and discretisation                  */
  cdg_solver_params s;     /* solver; multigrid_n_levels <= 0: chosen so the
                              coarsest grid has 3 or 4 cells per direction     */
} cdg_request;

typedef struct {
  int status;              /* CDG_OK or an error code                          */
  cdg_solve_stats stats;
  double queue_seconds;    /* submit -> start on a slot                        */
  double latency_seconds;  /* submit -> solution copied out                     */
  int slot;                /* worker that ran it                               */
  int ndof;
} cdg_result;

/* n_slots concurrent workers (1..64); hbm_budget_bytes 0 = 80 % of free */
int cdg_server_create(int device, int n_slots, long long hbm_budget_bytes,
                      cdg_server **out);
int cdg_server_destroy(cdg_server *srv);
/* number of DOFs of a request's finest level (size of its solution) */
int cdg_request_ndof(const cdg_request *req, int *ndof);
/* queue a request; solution_out (ndof doubles, host) receives the solution;
 * the buffer must stay valid until the request is complete */
int cdg_server_submit(cdg_server *srv, const cdg_request *req, double *solution_out,
                      long long *ticket);
/* wait for a request (timeout_seconds < 0: no timeout); 1 = still pending
 * after the timeout, 0 = done and *res filled */
int cdg_server_wait(cdg_server *srv, long long ticket, double timeout_seconds,
                    cdg_result *res);
/* counters: [0] submitted, [1] completed, [2] failed, [3] queued now,
 * [4] running now, [5] instances resident, [6] bytes resident, [7] evictions,
 * [8] budget bytes, [9] peak concurrent running, [10] kernel launches of all
 * slots, [11] mesh classes seen */
int cdg_server_counters(cdg_server *srv, long long *c12);
/* per-launch batching of small requests (the batcher thread): [0] launches,
 * [1] requests solved in them, [2] 1 when batching is on (CDG_SERVER_BATCH
 * unset or not 0 at server creation) */
int cdg_server_batch_counters(cdg_server *srv, long long *c3);

#ifdef __cplusplus
}
#endif
#endif
