// common.cuh -- device-side helpers and the context / problem structures
// shared by the assembly, linear-algebra and solver translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "cdg_internal.h"
#include "parmoon_cd.h"

namespace cdg {

void set_error(const char* fmt, ...);

#define CDG_CUDA(expr)                                                        \
  do {                                                                         \
    cudaError_t e_ = (expr);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      cdg::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #expr,               \
                     cudaGetErrorString(e_));                                  \
      return e_ == cudaErrorMemoryAllocation ? CDG_ERR_OOM : CDG_ERR_CUDA;     \
    }                                                                          \
  } while (0)

#define CDG_TRY(expr)                                                          \
  do {                                                                         \
    int rc_ = (expr);                                                          \
    if (rc_ != CDG_OK) return rc_;                                             \
  } while (0)

// device-side error word bits (set by kernels, read by the host at syncs)
enum : int {
  kErrPattern = 1,     // a local coupling is not in the CSR pattern
  kErrZeroDiag = 2,    // zero diagonal entry
  kErrSingular = 4,    // zero pivot in the coarse Gauss-Jordan
  kErrBreakdown = 8,   // FGMRES H(i+1,i) == 0
  kErrLattice = 16,    // a DOF off the unit box lattice (device numbering)
  kErrTimeout = 32,    // a bounded wait on a shared-memory barrier ran out
};

constexpr int kMfFactors = 40;        // per-cell factors of the matrix-free Q2 operator
constexpr int kMfTileRows = 256;      // rows (threads) per tile of the one-launch sweep
constexpr int kMfCellStride = 28;     // floats per tile cell in shared memory (16-byte rows)
// batched solver (batch.cu): one block per request
constexpr int kBatchMaxLevels = 12;
constexpr int kBatchMaxRestart = 64;
constexpr int kBatchMaxDofs = 20000;    // larger requests keep the stream-level solver
constexpr int kBatchMaxCoarse = 2048;   // active DOFs of the coarsest level
constexpr int kBatchSmemCoarse = 96;    // coarse blocks inverted inside the batch (shared memory)
constexpr int kRedSlots = 32;         // partial-sum rows (one per inner product)
constexpr int kRedMaxBlocks = 1024;   // partial sums per reduction

}  // namespace cdg

struct cdg_context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  int* d_err = nullptr;           // device error word
  double* d_red = nullptr;        // kRedSlots * kRedMaxBlocks partial sums
  unsigned* d_cnt = nullptr;      // kRedSlots last-block counters
  double* h_pinned = nullptr;     // 64 doubles of pinned readback space
  long long launches = 0;
  // programmatic dependent launch of the solver kernels (CDG_PDL=1: on)
  int pdl = 0;
  // the runtime refused a cooperative launch inside the captured FGMRES loop
  int coop_graph_failed = 0;
  // request descriptors and results of the batched solver (pinned / device)
  void* batch_host = nullptr;
  void* batch_dev = nullptr;
  size_t batch_host_bytes = 0;
};

namespace cdg {

// one discretisation level on the device
struct DevLevel {
  int dim = 2, shape = kQuad, order = 1, nloc = 4, nv = 4;
  int ncells = 0, ndof = 0, nactive = 0, nnz = 0;
  // some cell is a quadrilateral that is not a parallelogram (hexahedron not
  // a parallelepiped): the level is assembled per point through the cells'
  // bilinear / trilinear maps (TQuadBilinear, THexaTrilinear)
  int multilinear = 0;
  // host copies of the inputs (info queries, transfers)
  Mesh mesh;
  Space space;
  Pattern pattern;
  // device arrays
  double* verts = nullptr;       // ncells*nv*dim
  int* gdof = nullptr;           // ncells*nloc
  int* row_ptr = nullptr;        // ndof+1
  int* col = nullptr;            // nnz
  int* slot = nullptr;           // ncells*nloc*nloc CSR slot of each coupling
  int* diag_slot = nullptr;      // ndof
  double* val64 = nullptr;       // nnz
  float* val32 = nullptr;        // nnz (FP32 copy for the multigrid)
  double* rhs = nullptr;         // ndof
  double* sol = nullptr;         // ndof
  double* invdiag64 = nullptr;   // ndof
  float* invdiag32 = nullptr;    // ndof
  int rows_per_warp_hint = 1;    // SpMV shape (avg row length)
  // FP32 smoothing / defect with the CSR stream staged through shared memory
  // (opt-in, measured slower than the register-streaming kernels on GB300):
  // active rows cut into chunks of at most kBulkChunk entries, chunk c =
  // rows [bulk_row[c], bulk_row[c+1]); col and val32 carry 4 entries of tail
  // padding so a chunk copy rounded out to 16 bytes stays inside them
  int bulk_nchunks = 0;
  int bulk_chunk = 0;            // entries per chunk at most
  int* bulk_row = nullptr;       // nchunks+1
  // sliced ELLPACK copy of the FP64 matrix (the FGMRES operator, the FP64
  // multigrid smoother and defect) on levels of at least kSellMinRows rows:
  // G = sell_lanes lanes per row, slices of 32/G rows (one warp),
  // rows sorted by length inside windows of 256 consecutive rows; entry k of
  // the slice's row i at sell_off[s] + 32 (k / G) + G i + k % G.  Non-active
  // rows are stored as identity rows; the padding is zero.
  int sell_nslices = 0;
  int sell_lanes = 0;
  long long sell_total = 0;      // stored entries (padding included)
  long long* sell_off = nullptr; // nslices+1
  int* sell_row = nullptr;       // nslices*32/G: row of each slice row (-1: none)
  int* sell_col = nullptr;       // sell_off[nslices]
  double* sell_val = nullptr;    // sell_off[nslices]
  int* sell_pos = nullptr;       // nnz: SELL position of each CSR entry (-1: non-active row)
  // rhs assembly: local entries per (cell, local DOF) and, per active DOF,
  // the list of its local entries (CSR over active rows)
  double* rhs_loc = nullptr;     // ncells*nloc
  int* dof_rp = nullptr;         // nactive+1
  int* dof_ent = nullptr;        // entries: cell*nloc + i
  // couplings of active rows to non-active columns: CSR over active rows,
  // column and CSR slot of each (first smoothing step from a zero start)
  int* dc_rp = nullptr;
  int* dc_col = nullptr;
  int* dc_pos = nullptr;
  double* dc_val64 = nullptr;    // their values (refreshed with the FP32 copy)
  float* dc_val32 = nullptr;
  int dc_n = 0;
  int* dc_rows = nullptr;        // the active rows with couplings, increasing
  int dc_nrows = 0;
  // multigrid work vectors (double or float, per precision)
  void* mg_rhs = nullptr;
  void* mg_sol = nullptr;
  void* mg_tmp = nullptr;
  void* mg_def = nullptr;
  int mg_elem = 0;               // sizeof element of mg vectors
  int realloc_count = 0;         // multigrid vector (re)allocations
  bool mg_visited = false;       // level already descended through this cycle
  // transfer to the next coarser level (this = fine)
  int* P_rp = nullptr; int* P_col = nullptr; double* P_val = nullptr; float* P_val32 = nullptr;
  int* R_rp = nullptr; int* R_col = nullptr; double* R_val = nullptr; float* R_val32 = nullptr;
  int P_nnz = 0, R_nnz = 0;
  // time-dependent CD: stiffness and mass values (the system M + theta1 tau A
  // lives in val64), rhs of the current and the previous step, and the
  // solution of the step before the last (finest level; BDF2 reads it)
  double* tcd_A = nullptr;
  double* tcd_M = nullptr;
  double* tcd_f = nullptr;
  double* tcd_fold = nullptr;
  double* tcd_u2 = nullptr;
  // matrix-free FP32 operator of Q2 hexahedral levels (matfree.cu): the
  // per-cell factors of A_cell = sum_t g_t R_t in FP32 (cells x kMfFactors)
  // and the local results of one application, DOF-major (the entries of
  // active row r at [dof_rp[r], dof_rp[r+1]), cells x 27 at most).  mf_valid:
  // the factors belong to the operator the FP32 multigrid uses (stationary
  // assembly); mf_mode: -1 not yet chosen, 0 CSR kernels, 1 matrix-free
  float* mf_fac = nullptr;
  float* mf_y = nullptr;
  int mf_valid = 0;
  int mf_lin = 0;                // factors of a convection field linear in x
  int mf_mode = -1;
  float* mf_ae = nullptr;        // 27 x 27 element matrix of a uniform level (transposed)
  int* mf_pos = nullptr;         // cells x 27: position of (cell, local DOF) in mf_y, -1 non-active
  int* mf_gdof = nullptr;        // cells x 27: DOFs in cell 0's local order
  int* mf_pos_c = nullptr;       // cells x 27: mf_pos in cell 0's local order
  int* mf_loc = nullptr;         // cells x 27: the cell's local index of cell 0's index i
  double* ue64 = nullptr;        // 27 x 27 FP64 element matrix of a uniform level
  int mf_geo = -1;               // every cell a translate of cell 0 (-1: not checked)
  int mf_geo_exact = 0;          // ... to 1e-13 (the FP64 matrix from one element matrix)
  int mf_uniform = 0;            // the last assembly has one element matrix for all cells
  int mf_blocks_per_sm = 0;      // grid cap of the cell kernel (0: one cell per warp)
  // one-launch sweep of a uniform level (k_mf_fused): rows cut into tiles of
  // kMfTileRows; tile t recomputes the cells mf_tile_rp[t] .. mf_tile_rp[t+1]
  // of the tile cell list, whose DOFs in cell 0's local order (kMfCellStride
  // per cell, the last one padding) are mf_tile_gdof[kMfCellStride * c ..];
  // entry e of the DOF-major order reads its local result at mf_ent_loc[e]
  // (tile cell * kMfCellStride + local DOF) of the tile's shared memory
  int mf_ntiles = 0;
  int mf_fused_minb = 4;         // resident blocks per SM the sweep is compiled for (4, 5, 6)
  int mf_tile_maxcells = 0;
  int* mf_tile_rp = nullptr;
  int* mf_tile_gdof = nullptr;
  int* mf_ent_loc = nullptr;
  // lattice stencil sweep of a uniform level (k_mf_stencil): the DOFs sit on
  // the points of an st_dims[0] x st_dims[1] x st_dims[2] lattice in cell 0's
  // axes (st_map: lattice point, x fastest -> DOF), every active DOF is an
  // interior point, so each active row is one of eight 125-point stencils
  // (by the parities of its point); st_coef holds them (kStCoef floats,
  // formed from the element matrix at each assembly); st_zt: the tuner's
  // choice (0: not used, 4 or 8 lattice points per thread along z)
  int st_dims[3] = {0, 0, 0};
  int* st_map = nullptr;
  float* st_coef = nullptr;
  int st_zt = 0;
  // lattice grid transfer to the next coarser level (both uniform lattices,
  // P checked against the tensor-product Q2 interpolation): -1 not checked,
  // 0 CSR transfers, 1 lattice kernels with lt_perm / lt_sign / lt_t2 (fine
  // axis d runs along coarse axis lt_perm[d]; coarse half-unit coordinate
  // lt_t2[k] + lt_sign[d] * p_d)
  int lt_state = -1;
  int lt_perm[3] = {0, 1, 2}, lt_sign[3] = {1, 1, 1}, lt_t2[3] = {0, 0, 0};
  int tpr32 = 0;                 // FP32 CSR lanes per row (0: rows_per_warp_hint)
  // FP32 values from the tensor-core contraction, FP64 values not formed
  // (assemble_level_tc); last_a assembles them on demand (ensure_fp64)
  int fp64_stale = 0;
  cdg_assembly_params last_a{};
  int tuned = 0;                 // the tuner has run on this level
  float tuned_ms[2] = {0.f, 0.f};   // tuner's smoothing-step times: CSR, matrix-free
  // dense inverse of the active block (coarsest multigrid level)
  double* coarse_inv = nullptr;  // na*na
  double* coarse_work = nullptr; // 2 na^2 (Gauss-Jordan ping-pong) + pivots + column map
  int coarse_na = 0;
};

// FGMRES device state
struct GmresState {
  int n = 0, m = 0;
  double* V = nullptr;       // (m+1)*n
  double* Z = nullptr;       // m*n
  double* w = nullptr;       // n
  double* H = nullptr;       // (m+1)*(m+1), column-major by Arnoldi column
  double* cs = nullptr;      // m+1
  double* sn = nullptr;      // m+1
  double* s = nullptr;       // m+1
  double* y = nullptr;       // m+1
  double* scal = nullptr;    // 8 scalars: [0] resid, [1] beta, [2] norm, [4..5] loop info
  // graph-captured iteration loop (a WHILE conditional node around one
  // FGMRES iteration); rebuilt when the solver parameters or buffers change
  int* dstate = nullptr;     // [0] i (column), [1] j (iteration), [2] flag
  double* zcur = nullptr;    // n: z_i for the operator application
  double* part = nullptr;    // block partial sums of the cooperative restart cycle
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  cdg_solver_params key{};   // parameters the graph was captured with
  unsigned long long key_gen = 0;
  int coop = -1;             // the graph's Gram-Schmidt: 1 the cooperative step, 0 three kernels
  long long body_launches = 0;   // kernels per iteration
};

}  // namespace cdg

struct cdg_problem {
  cdg_context* ctx = nullptr;
  unsigned long long alloc_gen = 1;   // bumped when device work buffers move
  int dim = 2, shape = cdg::kQuad, order = 1;
  std::vector<cdg::DevLevel> lev;
  cdg::GmresState gm;
  double* d_tables = nullptr;     // reference tensors (device)
  int* d_zero_diag = nullptr;     // set by the assembly when a diagonal is 0
  int nterms = 0;
  int rt_order = -1;
  int tcd_step = 0;               // TimeDiscretization::current_step_
  int tc_levels = 0;              // levels 1 .. n-2 assembled FP32-only on tensor cores
};

struct cdg_hierarchy {
  int dim = 2, shape = cdg::kQuad, order = 1;
  std::vector<cdg::Mesh> mesh;           // geometry (finest level perturbed)
  std::vector<cdg::Mesh> mesh_nested;    // unperturbed, locates fine nodes in parents
  std::vector<cdg::Space> space;
  std::vector<cdg::Pattern> pattern;
};

namespace cdg {

template <typename K>
inline int grid_for(long n, int block) {
  long g = (n + block - 1) / block;
  return (int)(g < 1 ? 1 : g);
}

// launch accounting: every kernel launch of the library goes through this
#define CDG_LAUNCH(ctx, kernel, grid, block, smem, ...)                        \
  do {                                                                         \
    kernel<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);           \
    (ctx)->launches++;                                                         \
    cudaError_t le_ = cudaGetLastError();                                      \
    if (le_ != cudaSuccess) {                                                  \
      cdg::set_error("launch %s: %s", #kernel, cudaGetErrorString(le_));       \
      return CDG_ERR_CUDA;                                                     \
    }                                                                          \
  } while (0)

// Programmatic dependent launch: a solver kernel launched with
// CDG_LAUNCH_PDL may be scheduled while its predecessor on the stream is
// still running, so its blocks are resident when the predecessor ends instead
// of being launched then.  Every such kernel starts with pdl_enter(): it waits
// until the predecessor grid has completed and its memory is visible (so
// nothing is read or written before then), and only then allows its own
// successor to be scheduled -- at most two grids are in flight, and the chain
// of waits keeps every earlier kernel complete.  Outside a programmatic
// launch both instructions do nothing.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

#define CDG_LAUNCH_PDL(ctx, kernel, grid, block, smem, ...)                    \
  do {                                                                         \
    cudaError_t le_;                                                           \
    if ((ctx)->pdl) {                                                          \
      cudaLaunchConfig_t cfg_ = {};                                            \
      cfg_.gridDim = dim3(grid);                                               \
      cfg_.blockDim = dim3(block);                                             \
      cfg_.dynamicSmemBytes = (smem);                                          \
      cfg_.stream = (ctx)->stream;                                             \
      cudaLaunchAttribute at_[1];                                              \
      at_[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;          \
      at_[0].val.programmaticStreamSerializationAllowed = 1;                   \
      cfg_.attrs = at_;                                                        \
      cfg_.numAttrs = 1;                                                       \
      le_ = cudaLaunchKernelEx(&cfg_, kernel, __VA_ARGS__);                    \
    } else {                                                                   \
      kernel<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);         \
      le_ = cudaGetLastError();                                                \
    }                                                                          \
    (ctx)->launches++;                                                         \
    if (le_ != cudaSuccess) {                                                  \
      cdg::set_error("launch %s: %s", #kernel, cudaGetErrorString(le_));       \
      return CDG_ERR_CUDA;                                                     \
    }                                                                          \
  } while (0)

// host launchers implemented in the .cu files
int upload_level(cdg_context* ctx, DevLevel& L);
// FE space numbering and CSR pattern built on the device (bit-exact with
// make_space / make_pattern); device_pattern takes gdof from the host or the
// device and can hand over its device row_ptr / col
int device_space(cdg_context* ctx, const Mesh& m, int order, int neumann_mask, Space* out);
int device_pattern(cdg_context* ctx, int ncells, int nloc, int ndof, const int* gdof_host,
                   const int* gdof_dev, std::vector<int>* row_ptr, std::vector<int>* col,
                   int** col_dev_out, int** rp_dev_out);
// sliced ELLPACK layout of L with G lanes per row built on the device (the
// layout of build_sell's host path); CDG_ERR_LIMIT: slots beyond 32-bit positions
int device_sell(cdg_context* ctx, DevLevel& L, int G);
// prolongation / restriction of the fine level F (the matrices of
// make_transfer) built on the device into F.P_* / F.R_*; fm, cm: the nested
// (unperturbed) meshes, parent: coarse cell of each fine cell (host)
int device_transfer(cdg_context* ctx, const Mesh& fm, const Space& fs, const Mesh& cm,
                    const Space& cs, const int* parent_host, const int* fgdof_dev,
                    const int* cgdof_dev, DevLevel& F);
constexpr int kSellWindow = 256;    // rows sorted by length inside windows of this many rows
constexpr int kBulkChunk = 0;       // CSR entries per staged chunk; 0: off unless
                                    // CDG_BULK_CHUNK (256, 512, 1024) asks for it
constexpr int kBulkMinRows = 65536; // smaller levels keep the register-streaming kernels
int build_bulk(cdg_context* ctx, DevLevel& L);
constexpr int kSellMinRows = 32768; // smaller levels keep the CSR kernels (latency bound)
constexpr int kSellMinWarps = 4096; // lanes per row doubled until a launch has this many warps
int build_sell(cdg_context* ctx, DevLevel& L);
int free_level(DevLevel& L);
int build_slots(cdg_context* ctx, DevLevel& L);
int assemble_level(cdg_context* ctx, cdg_problem* p, DevLevel& L,
                   const cdg_assembly_params& a);
int check_device_error(cdg_context* ctx);
// matrix-free FP32 operator of Q2 hexahedral levels (matfree.cu); mode as
// k_spmv: 0 y = Ax, 1 y = b - Ax, 2 Jacobi step, 3 Jacobi step + FP64 copy
bool mf_eligible(const DevLevel& L);
// a context's stream at the device's highest priority (api.cu)
int cdg_context_high_priority(cdg_context* c);
// batched solver (batch.cu): requests a launch can take (why: the reason
// when not), and one launch over prepared problems on ctx's stream
struct BatchResult {
  int status, iterations;
  double residual, initial;
};
bool batch_eligible(const cdg_problem* p, const cdg_solver_params& s, const char** why);
int batch_launch(cdg_context* ctx, cdg_problem* const* probs, const cdg_solver_params* params,
                 const int* inline_coarse, int count, BatchResult* results);
// the buffers and coarse inverse a batched solve reads (linalg.cu);
// *inline_coarse: the coarse block is inverted by the batch's coarse launch
int batch_prepare(cdg_context* ctx, cdg_problem* p, const cdg_solver_params& s,
                  int* inline_coarse);
// tiles of the one-launch sweep of a uniform level (once per level)
int mf_build_tiles(cdg_context* ctx, DevLevel& L);
// the DOF lattice of a uniform level for the stencil sweep (once per level;
// leaves st_dims zero where the level is not a full lattice with active
// DOFs exactly at its interior points), and the stencils of the element
// matrix in L.mf_ae (each assembly)
int mf_build_lattice(cdg_context* ctx, DevLevel& L);
int mf_stencil_coef(cdg_context* ctx, DevLevel& L);
// lattice grid transfers between F and C = the next coarser level (once per
// pair, after both are assembled; an option: CDG_LAT_TRANSFER=1)
int lattice_transfer_setup(cdg_context* ctx, DevLevel& F, const DevLevel& C);
int mf_ensure(DevLevel& L);
// the kernel form of a matrix-free application: as the tuner chose
// (stencil, one-launch tiles or two kernels), the two-kernel product, the
// one-launch tile sweep (two kernels where the level has no tiles), the
// lattice stencil sweep
enum { kMfAsTuned = 0, kMfTwoKernel = 1, kMfOneLaunch = 2, kMfStencil = 3 };
int mf_apply(cdg_context* ctx, const DevLevel& L, int mode, const float* x, const float* b,
             const float* invd, float w, float* y, double* z = nullptr, const int* di = nullptr,
             double* zcur = nullptr, int form = kMfAsTuned);
// y = A x with the FP32 multigrid operator of a level: 0 CSR, 1 matrix-free
// (one launch on uniform levels), 2 the two-kernel matrix-free product,
// 3 the lattice stencil sweep
int apply32(cdg_context* ctx, const DevLevel& L, int variant, const float* x, float* y);
// generic coefficients (CoeffFct): quadrature points of a level (host) and the
// assembly with eps, b, c, f per (cell, point)
int level_quadrature_points(const DevLevel& L, const cdg_assembly_params& a, int* nqp,
                            double* x);
int assemble_level_coefficients(cdg_context* ctx, cdg_problem* p, DevLevel& L,
                                const cdg_assembly_params& a, const double* coef_host);
// FP32-only level from the tensor-core contraction, and its FP64 values on demand
int assemble_level_tc(cdg_context* ctx, cdg_problem* p, DevLevel& L,
                      const cdg_assembly_params& a);
int ensure_fp64(cdg_context* ctx, cdg_problem* p, DevLevel& L);
// argument checks of every entry point that takes assembly parameters
int check_assembly_params(const cdg_problem* p, const cdg_assembly_params* a);
int level_errors(cdg_context* ctx, cdg_problem* p, DevLevel& L,
                 const cdg_assembly_params& a, double* errors);
// time-dependent CD (TimeConvectionDiffusion with the TimeDiscretization schemes)
int tcd_interpolate(cdg_context* ctx, cdg_problem* p, const cdg_assembly_params& a);
int tcd_assemble_level(cdg_context* ctx, cdg_problem* p, DevLevel& L,
                       const cdg_assembly_params& a, bool with_mass, double theta1,
                       double tau);
// The scheme one step takes (TimeDiscretization::set_time_disc_parameters,
// src/TimeDiscRoutines/TimeDiscretizations.C:422-475): step is the index of
// the step (TimeDiscretization::current_step_ after the increment; 0 for the
// initial assembly), and the first BDF2 step is taken by bdf_two_first_step.
struct TimeScheme {
  int kind;        // CDG_TIME_CRANK_NICOLSON, _BACKWARD_EULER or _BDF_TWO
  double theta1;   // THETA1: 1/2, 1, 2/3
};
inline TimeScheme time_scheme(const cdg_assembly_params& a, int step) {
  int kind = a.time_discretization;
  if (kind == CDG_TIME_BDF_TWO && step <= 1)
    kind = a.bdf_two_first_step == 1 ? CDG_TIME_CRANK_NICOLSON : CDG_TIME_BACKWARD_EULER;
  const double theta1 = kind == CDG_TIME_CRANK_NICOLSON ? 0.5
                        : kind == CDG_TIME_BACKWARD_EULER ? 1.0 : 2. / 3.;
  return TimeScheme{kind, theta1};
}
int tcd_rhs(cdg_context* ctx, DevLevel& L, TimeScheme ts, double tau);
// solution history: tcd_u2 (allocated on first use) <- the current solution
int tcd_start_history(cdg_context* ctx, DevLevel& L);
int tcd_system(cdg_context* ctx, cdg_problem* p, DevLevel& L, TimeScheme ts, double tau);

// linear algebra (linalg.cu)
int spmv_apply64(cdg_context* ctx, const DevLevel& L, const double* x, double* y);
int residual64(cdg_context* ctx, const DevLevel& L, const double* b, const double* x,
               double* r);
int dot64(cdg_context* ctx, int n, const double* a, const double* b, double* out,
          int slot);
int prolongate64(cdg_context* ctx, const DevLevel& F, const DevLevel& C, const double* xc,
                 double* xf, int add_actives_only, double damp);
int restrict64(cdg_context* ctx, const DevLevel& F, const DevLevel& C, const double* df,
               double* rc);
int precondition(cdg_context* ctx, cdg_problem* p, const cdg_solver_params& s,
                 const double* v, double* z, const int* di = nullptr, double* zcur = nullptr);
int prepare_solver(cdg_context* ctx, cdg_problem* p, const cdg_solver_params& s);
void free_gmres(GmresState& g);
int fgmres(cdg_context* ctx, cdg_problem* p, const cdg_solver_params& s,
           cdg_solve_stats* st);
// single hot-kernel launches for measurement
int smooth32_once(cdg_context* ctx, DevLevel& L, float damp);
int defect32_once(cdg_context* ctx, DevLevel& L);
int ensure_mg_vectors(cdg_context* ctx, DevLevel& L, int elem);
int contract_only(cdg_context* ctx, cdg_problem* p, DevLevel& L, const cdg_assembly_params& a);

}  // namespace cdg
