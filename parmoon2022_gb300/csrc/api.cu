// api.cu -- the extern "C" entry points of libparmoon_cd.so (declared in
// include/parmoon_cd.h): context, host setup hierarchy, the CD problem
// (ConvectionDiffusion<d> assemble / solve / output) and operator pieces.
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "common.cuh"

namespace cdg {
// the context's stream recreated at the device's highest priority (the
// request server's small requests and batched launches: their short,
// latency-bound kernels are scheduled ahead of large requests' blocks)
int cdg_context_high_priority(cdg_context* c) {
  if (!c) { set_error("null context"); return CDG_ERR_ARG; }
  int least = 0, greatest = 0;
  CDG_CUDA(cudaSetDevice(c->device));
  CDG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  CDG_CUDA(cudaStreamSynchronize(c->stream));
  cudaStream_t st = nullptr;
  CDG_CUDA(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, greatest));
  cudaStreamDestroy(c->stream);
  c->stream = st;
  return CDG_OK;
}

static thread_local char g_msg[512] = "";
void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_msg, sizeof g_msg, fmt, ap);
  va_end(ap);
}

int check_assembly_params(const cdg_problem* p, const cdg_assembly_params* a) {
  if (!p || !a) { set_error("null argument"); return CDG_ERR_ARG; }
  if (a->example < 0 || a->example > CDG_EX_QUAD_ST) { set_error("unknown example %d", a->example); return CDG_ERR_ARG; }
  if (a->time_discretization < CDG_TIME_CRANK_NICOLSON || a->time_discretization > CDG_TIME_BDF_TWO) {
    set_error("time discretization scheme %d is not supported", a->time_discretization);
    return CDG_ERR_ARG;
  }
  if (a->bdf_two_first_step < 0 || a->bdf_two_first_step > 1) {
    set_error("bdf_two_first_step %d: 0 backward Euler or 1 Crank-Nicolson", a->bdf_two_first_step);
    return CDG_ERR_ARG;
  }
  if (a->example == CDG_EX_POLYEXP && p->dim != 3) { set_error("example needs 3D"); return CDG_ERR_ARG; }
  return CDG_OK;
}
}  // namespace cdg

using namespace cdg;

#define API_GUARD(expr)                                                        \
  try {                                                                        \
    return (expr);                                                             \
  } catch (const std::bad_alloc&) {                                            \
    set_error("host allocation failed");                                       \
    return CDG_ERR_OOM;                                                        \
  } catch (const std::exception& e) {                                          \
    set_error("%s", e.what());                                                 \
    return CDG_ERR_ARG;                                                        \
  }

extern "C" {

const char* cdg_last_error(void) { return g_msg; }
int cdg_version(void) { return 1; }

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
int cdg_context_create(int device, cdg_context** out) {
  if (!out) { set_error("null output"); return CDG_ERR_ARG; }
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("no CUDA device");
    return CDG_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= ndev) { set_error("bad device %d", device); return CDG_ERR_ARG; }
  CDG_CUDA(cudaSetDevice(device));
  cdg_context* c = new cdg_context();
  c->device = device;
  CDG_CUDA(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
  CDG_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CDG_CUDA(cudaMalloc(&c->d_err, sizeof(int)));
  CDG_CUDA(cudaMemset(c->d_err, 0, sizeof(int)));
  CDG_CUDA(cudaMalloc(&c->d_red, (size_t)kRedSlots * kRedMaxBlocks * sizeof(double)));
  CDG_CUDA(cudaMalloc(&c->d_cnt, kRedSlots * sizeof(unsigned)));
  CDG_CUDA(cudaMemset(c->d_cnt, 0, kRedSlots * sizeof(unsigned)));
  CDG_CUDA(cudaMallocHost(&c->h_pinned, 64 * sizeof(double)));
  {
    // off by default: measured on GB300 (32^3 Q2 mixed step) the
    // graph-launched FGMRES iteration took 42.9 ms per solve with it and
    // 40.4 ms without, although single kernels repeated back to back gained
    // (matrix-free smoothing step 16.4 -> 11.7 us)
    const char* e = std::getenv("CDG_PDL");
    c->pdl = (e && e[0] == '1') ? 1 : 0;
  }
  *out = c;
  return CDG_OK;
}

int cdg_context_destroy(cdg_context* c) {
  if (!c) return CDG_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  cudaFree(c->d_err);
  cudaFree(c->d_red);
  cudaFree(c->d_cnt);
  cudaFreeHost(c->h_pinned);
  if (c->batch_host) cudaFreeHost(c->batch_host);
  if (c->batch_dev) cudaFree(c->batch_dev);
  cudaStreamDestroy(c->stream);
  delete c;
  return CDG_OK;
}

int cdg_context_synchronize(cdg_context* c) {
  if (!c) { set_error("null context"); return CDG_ERR_ARG; }
  CDG_CUDA(cudaStreamSynchronize(c->stream));
  return CDG_OK;
}

long long cdg_context_launch_count(const cdg_context* c) { return c ? c->launches : -1; }

int cdg_context_stream(cdg_context* c, void** stream) {
  if (!c || !stream) { set_error("null argument"); return CDG_ERR_ARG; }
  *stream = (void*)c->stream;
  return CDG_OK;
}

// ---------------------------------------------------------------------------
// host setup hierarchy
// ---------------------------------------------------------------------------
// numbering and pattern of one level: host (ctx == null) or device
static int level_space_pattern(cdg_context* ctx, const Mesh& m, int order, int nmask, Space* s,
                               Pattern* P) {
  if (!ctx) {
    *s = make_space(m, order, nmask);
    *P = make_pattern(*s);
    return CDG_OK;
  }
  CDG_CUDA(cudaSetDevice(ctx->device));
  CDG_TRY(device_space(ctx, m, order, nmask, s));
  P->nrows = s->ndof;
  return device_pattern(ctx, m.ncells, s->nloc, s->ndof, s->gdof.data(), nullptr, &P->row_ptr,
                        &P->col, nullptr, nullptr);
}

static int hierarchy_create(int dim, int order, int roots, int nref, int n_levels, int nmask,
                            cdg_hierarchy** out, cdg_context* ctx = nullptr) {
  if (!out || (dim != 2 && dim != 3) || (order != 1 && order != 2) || roots < 1 || nref < 0 ||
      n_levels < 1 || n_levels > nref + 1) {
    set_error("bad hierarchy arguments");
    return CDG_ERR_ARG;
  }
  cdg_hierarchy* h = new cdg_hierarchy();
  h->dim = dim;
  h->shape = dim == 2 ? kQuad : kHexa;
  h->order = order;
  for (int l = 0; l < n_levels; ++l) {
    h->mesh.push_back(make_refined_box(dim, roots, nref - l));
    h->space.emplace_back();
    h->pattern.emplace_back();
    const int rc = level_space_pattern(ctx, h->mesh.back(), order, nmask, &h->space.back(),
                                       &h->pattern.back());
    if (rc != CDG_OK) {
      delete h;
      return rc;
    }
  }
  h->mesh_nested = h->mesh;
  *out = h;
  return CDG_OK;
}

static int hierarchy_create_tetra(int order, int roots, int nref, int n_levels, int nmask,
                                  double perturb, unsigned long long seed, cdg_hierarchy** out,
                                  cdg_context* ctx = nullptr) {
  if (!out || (order != 1 && order != 2) || roots < 1 || nref < 0 || n_levels < 1 ||
      n_levels > nref + 1 || perturb < 0 || perturb >= 0.5 || nmask < 0 || nmask > 63) {
    set_error("bad tetrahedral hierarchy arguments");
    return CDG_ERR_ARG;
  }
  cdg_hierarchy* h = new cdg_hierarchy();
  h->dim = 3;
  h->shape = kTetra;
  h->order = order;
  for (int l = 0; l < n_levels; ++l) {
    h->mesh.push_back(make_kuhn_box(roots, nref - l));
    h->space.emplace_back();
    h->pattern.emplace_back();
    const int rc = level_space_pattern(ctx, h->mesh.back(), order, nmask, &h->space.back(),
                                       &h->pattern.back());
    if (rc != CDG_OK) {
      delete h;
      return rc;
    }
  }
  h->mesh_nested = h->mesh;
  if (perturb > 0) perturb_interior(h->mesh[0], 1.0 / (roots << nref), perturb, seed);
  *out = h;
  return CDG_OK;
}

int cdg_hierarchy_create(int dim, int order, int roots, int nref, int n_levels, int neumann_mask,
                         cdg_hierarchy** out) {
  API_GUARD(hierarchy_create(dim, order, roots, nref, n_levels, neumann_mask, out));
}

int cdg_hierarchy_perturb(cdg_hierarchy* h, double amplitude, unsigned long long seed) {
  if (!h || h->mesh.empty() || amplitude < 0 || amplitude >= 0.5) {
    set_error("bad arguments (amplitude in [0, 0.5))");
    return CDG_ERR_ARG;
  }
  Mesh& m = h->mesh[0];
  // cells per direction of the unit square / cube (6 tetrahedra per cube)
  const double cubes = (double)m.ncells / (m.shape == kTetra ? 6.0 : 1.0);
  const long n = std::lround(std::pow(cubes, 1.0 / m.dim));
  if (n < 1) {
    set_error("empty mesh");
    return CDG_ERR_ARG;
  }
  if (amplitude > 0) perturb_interior(m, 1.0 / (double)n, amplitude, seed);
  return CDG_OK;
}

int cdg_hierarchy_create_tetra(int order, int roots, int nref, int n_levels, int neumann_mask,
                               double perturb, unsigned long long seed, cdg_hierarchy** out) {
  API_GUARD(hierarchy_create_tetra(order, roots, nref, n_levels, neumann_mask, perturb, seed, out));
}

int cdg_hierarchy_create_device(cdg_context* ctx, int dim, int order, int roots, int nref,
                                int n_levels, int neumann_mask, cdg_hierarchy** out) {
  if (!ctx) { set_error("null context"); return CDG_ERR_ARG; }
  API_GUARD(hierarchy_create(dim, order, roots, nref, n_levels, neumann_mask, out, ctx));
}

int cdg_hierarchy_create_tetra_device(cdg_context* ctx, int order, int roots, int nref,
                                      int n_levels, int neumann_mask, double perturb,
                                      unsigned long long seed, cdg_hierarchy** out) {
  if (!ctx) { set_error("null context"); return CDG_ERR_ARG; }
  API_GUARD(hierarchy_create_tetra(order, roots, nref, n_levels, neumann_mask, perturb, seed,
                                   out, ctx));
}

static int space_number_device(cdg_context* ctx, int cell_type, int order, int neumann_mask,
                               int ncells, const double* verts, int* gdof, int* ndof,
                               int* nactive) {
  if (!ctx || !verts || !gdof || !ndof || !nactive || ncells < 1 || (order != 1 && order != 2) ||
      (cell_type != CDG_CELL_QUAD && cell_type != CDG_CELL_HEXA && cell_type != CDG_CELL_TETRA)) {
    set_error("bad arguments");
    return CDG_ERR_ARG;
  }
  CDG_CUDA(cudaSetDevice(ctx->device));
  Mesh m;
  m.shape = cell_type == CDG_CELL_QUAD ? kQuad : cell_type == CDG_CELL_HEXA ? kHexa : kTetra;
  m.dim = m.shape == kQuad ? 2 : 3;
  m.nv = n_vertices(m.shape);
  m.ncells = ncells;
  m.verts.assign(verts, verts + (size_t)ncells * m.nv * m.dim);
  Space s;
  CDG_TRY(device_space(ctx, m, order, neumann_mask, &s));
  std::memcpy(gdof, s.gdof.data(), s.gdof.size() * sizeof(int));
  *ndof = s.ndof;
  *nactive = s.nactive;
  return CDG_OK;
}

int cdg_space_number_device(cdg_context* ctx, int cell_type, int order, int neumann_mask,
                            int ncells, const double* verts, int* gdof, int* ndof, int* nactive) {
  API_GUARD(space_number_device(ctx, cell_type, order, neumann_mask, ncells, verts, gdof, ndof,
                                nactive));
}

static int structure_build_device(cdg_context* ctx, int ncells, int nloc, int ndof,
                                  const int* gdof, int* row_ptr, int* col, long long capacity,
                                  long long* nnz) {
  if (!ctx || !gdof || !row_ptr || !nnz || ncells < 1 || nloc < 1 || nloc > kMaxLoc || ndof < 1) {
    set_error("bad arguments");
    return CDG_ERR_ARG;
  }
  for (long i = 0; i < (long)ncells * nloc; ++i)
    if (gdof[i] < 0 || gdof[i] >= ndof) {
      set_error("global DOF %d out of range at %ld", gdof[i], i);
      return CDG_ERR_ARG;
    }
  CDG_CUDA(cudaSetDevice(ctx->device));
  std::vector<int> rp, cl;
  CDG_TRY(device_pattern(ctx, ncells, nloc, ndof, gdof, nullptr, &rp, &cl, nullptr, nullptr));
  std::memcpy(row_ptr, rp.data(), rp.size() * sizeof(int));
  *nnz = (long long)cl.size();
  if (!col || capacity < (long long)cl.size()) {
    set_error("column capacity %lld below nnz %lld", capacity, (long long)cl.size());
    return CDG_ERR_LIMIT;
  }
  std::memcpy(col, cl.data(), cl.size() * sizeof(int));
  return CDG_OK;
}

int cdg_structure_build_device(cdg_context* ctx, int ncells, int nloc, int ndof, const int* gdof,
                               int* row_ptr, int* col, long long col_capacity, long long* nnz) {
  API_GUARD(structure_build_device(ctx, ncells, nloc, ndof, gdof, row_ptr, col, col_capacity,
                                   nnz));
}

int cdg_hierarchy_destroy(cdg_hierarchy* h) {
  delete h;
  return CDG_OK;
}

int cdg_hierarchy_level_info(const cdg_hierarchy* h, int level, int* info) {
  if (!h || level < 0 || level >= (int)h->mesh.size() || !info) { set_error("bad level"); return CDG_ERR_ARG; }
  info[0] = h->mesh[level].ncells;
  info[1] = h->space[level].nloc;
  info[2] = h->space[level].ndof;
  info[3] = h->space[level].nactive;
  info[4] = (int)h->pattern[level].col.size();
  info[5] = h->mesh[level].nv;
  return CDG_OK;
}

int cdg_hierarchy_get_mesh(const cdg_hierarchy* h, int level, double* v) {
  if (!h || level < 0 || level >= (int)h->mesh.size() || !v) { set_error("bad level"); return CDG_ERR_ARG; }
  std::memcpy(v, h->mesh[level].verts.data(), h->mesh[level].verts.size() * sizeof(double));
  return CDG_OK;
}

int cdg_hierarchy_get_dofs(const cdg_hierarchy* h, int level, int* g) {
  if (!h || level < 0 || level >= (int)h->mesh.size() || !g) { set_error("bad level"); return CDG_ERR_ARG; }
  std::memcpy(g, h->space[level].gdof.data(), h->space[level].gdof.size() * sizeof(int));
  return CDG_OK;
}

int cdg_hierarchy_get_pattern(const cdg_hierarchy* h, int level, int* rp, int* col) {
  if (!h || level < 0 || level >= (int)h->mesh.size() || !rp || !col) { set_error("bad level"); return CDG_ERR_ARG; }
  const Pattern& P = h->pattern[level];
  std::memcpy(rp, P.row_ptr.data(), P.row_ptr.size() * sizeof(int));
  std::memcpy(col, P.col.data(), P.col.size() * sizeof(int));
  return CDG_OK;
}

// ---------------------------------------------------------------------------
// problem
// ---------------------------------------------------------------------------
}  // extern "C"
template <typename T>
static int up(T** d, const std::vector<T>& h, cudaStream_t st) {
  CDG_CUDA(cudaMalloc((void**)d, std::max<size_t>(h.size(), 1) * sizeof(T)));
  if (!h.empty())
    CDG_CUDA(cudaMemcpyAsync(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
  return CDG_OK;
}
extern "C" {

// CDG_SETUP_TIMING=1: print the seconds of each phase of problem creation
struct PhaseClock {
  bool on = getenv("CDG_SETUP_TIMING") != nullptr;
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  double acc[4] = {0, 0, 0, 0};
  void lap(int k, cudaStream_t st) {
    if (!on) return;
    cudaStreamSynchronize(st);
    const auto now = std::chrono::steady_clock::now();
    acc[k] += std::chrono::duration<double>(now - t).count();
    t = now;
  }
  ~PhaseClock() {
    if (on)
      fprintf(stderr, "problem setup: upload+slots %.3f s, sliced copy %.3f s, transfers %.3f s\n",
              acc[0], acc[1], acc[2]);
  }
};

// the first quadrilateral of the mesh that is not a parallelogram
// (hexahedron not a parallelepiped), -1 if all are, by the reference's shape
// tests (TQuadrangle::CheckQuad, Quadrangle.C:119-128: |x0 - x1 + x2 - x3| >
// 1e-8 in a coordinate; THexahedron::CheckHexa, Hexahedron.C:196-235: a
// Brick when the four bilinear-term combinations sum below 1e-8 in every
// coordinate).  The reference maps such cells with TQuadBilinear /
// THexaTrilinear; their levels are assembled per point here.
static long first_non_affine_cell(const Mesh& m) {
  if (m.shape == kTetra) return -1;
  const int dim = m.dim, nv = m.nv;
  for (long c = 0; c < m.ncells; ++c) {
    const double* v = &m.verts[(size_t)c * nv * dim];
    if (m.shape == kQuad) {
      for (int a = 0; a < 2; ++a)
        if (std::fabs(v[a] - v[2 + a] + v[4 + a] - v[6 + a]) > 1e-8) return c;
      continue;
    }
    for (int a = 0; a < 3; ++a) {
      auto x = [&](int i) { return v[3 * i + a]; };
      const double t1 = std::fabs(x(0) - x(1) - x(3) + x(2) + x(4) - x(5) - x(7) + x(6));
      const double t2 = std::fabs(x(0) - x(1) + x(3) - x(2) - x(4) + x(5) - x(7) + x(6));
      const double t3 = std::fabs(x(0) + x(1) - x(3) - x(2) - x(4) - x(5) + x(7) + x(6));
      const double t4 = std::fabs(-x(0) + x(1) + x(3) - x(2) + x(4) - x(5) - x(7) + x(6));
      if (t1 + t2 + t3 + t4 >= 1e-8) return c;
    }
  }
  return -1;
}

static int finish_problem(cdg_context* ctx, cdg_problem* p, const std::vector<std::vector<int>>& parents,
                          const std::vector<Mesh>* nested) {
  PhaseClock clk;
  CDG_CUDA(cudaMalloc(&p->d_zero_diag, sizeof(int)));
  CDG_CUDA(cudaMemsetAsync(p->d_zero_diag, 0, sizeof(int), ctx->stream));
  for (auto& L : p->lev) L.multilinear = first_non_affine_cell(L.mesh) >= 0 ? 1 : 0;
  for (auto& L : p->lev) {
    CDG_TRY(upload_level(ctx, L));
    clk.lap(0, ctx->stream);
    CDG_TRY(build_sell(ctx, L));
    CDG_TRY(build_bulk(ctx, L));
    clk.lap(1, ctx->stream);
  }
  for (size_t l = 0; l + 1 < p->lev.size(); ++l) {
    DevLevel& F = p->lev[l];
    DevLevel& C = p->lev[l + 1];
    const Mesh& fm = nested ? (*nested)[l] : F.mesh;
    const Mesh& cm = nested ? (*nested)[l + 1] : C.mesh;
    // on the device; the host builder stays for rows beyond the device sort
    const int drc = device_transfer(ctx, fm, F.space, cm, C.space, parents[l].data(), F.gdof,
                                    C.gdof, F);
    if (drc == CDG_OK) {
      clk.lap(2, ctx->stream);
      continue;
    }
    if (drc != CDG_ERR_LIMIT) return drc;
    HostCsr P, R;
    make_transfer(fm, F.space, cm, C.space, parents[l].data(), &P, &R);
    std::vector<float> pv(P.val.begin(), P.val.end()), rv(R.val.begin(), R.val.end());
    CDG_TRY(up(&F.P_rp, P.row_ptr, ctx->stream));
    CDG_TRY(up(&F.P_col, P.col, ctx->stream));
    CDG_TRY(up(&F.P_val, P.val, ctx->stream));
    CDG_TRY(up(&F.P_val32, pv, ctx->stream));
    CDG_TRY(up(&F.R_rp, R.row_ptr, ctx->stream));
    CDG_TRY(up(&F.R_col, R.col, ctx->stream));
    CDG_TRY(up(&F.R_val, R.val, ctx->stream));
    CDG_TRY(up(&F.R_val32, rv, ctx->stream));
    F.P_nnz = (int)P.col.size();
    F.R_nnz = (int)R.col.size();
    clk.lap(2, ctx->stream);
  }
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  return CDG_OK;
}

static void fill_level(DevLevel& L, int shape, int order) {
  L.shape = shape;
  L.dim = shape == kQuad ? 2 : 3;
  L.order = order;
  L.nv = n_vertices(shape);
  L.nloc = n_local_dofs(shape, order);
  L.ncells = L.mesh.ncells;
  L.ndof = L.space.ndof;
  L.nactive = L.space.nactive;
  L.nnz = (int)L.pattern.col.size();
}

static int problem_create(cdg_context* ctx, const cdg_hierarchy* h, cdg_problem** out) {
  if (!ctx || !h || !out) { set_error("null argument"); return CDG_ERR_ARG; }
  CDG_CUDA(cudaSetDevice(ctx->device));
  cdg_problem* p = new cdg_problem();
  p->ctx = ctx;
  p->dim = h->dim;
  p->shape = h->shape;
  p->order = h->order;
  p->lev.resize(h->mesh.size());
  std::vector<std::vector<int>> parents;
  for (size_t l = 0; l < h->mesh.size(); ++l) {
    DevLevel& L = p->lev[l];
    L.mesh = h->mesh[l];
    L.space = h->space[l];
    L.pattern = h->pattern[l];
    fill_level(L, h->shape, h->order);
    if (l + 1 < h->mesh.size()) {
      std::vector<int> par(L.ncells);
      int nch = h->dim == 2 ? 4 : 8;
      for (int f = 0; f < L.ncells; ++f) par[f] = f / nch;
      parents.push_back(par);
    }
  }
  int rc = finish_problem(ctx, p, parents, &h->mesh_nested);
  if (rc != CDG_OK) {
    cdg_problem_destroy(p);
    return rc;
  }
  *out = p;
  return CDG_OK;
}

int cdg_problem_create(cdg_context* ctx, const cdg_hierarchy* h, cdg_problem** out) {
  API_GUARD(problem_create(ctx, h, out));
}


static int problem_from_arrays(cdg_context* ctx, int cell_type, int order, int nl, const int* n_cells,
                               const double* const* verts, const int* const* gn,
                               const int* n_dofs, const int* n_active, const int* const* rp,
                               const int* const* col, const int* const* parent,
                               cdg_problem** out) {
  if (!ctx || !out || cell_type < CDG_CELL_QUAD || cell_type > CDG_CELL_TETRA ||
      (order != 1 && order != 2) || nl < 1 || !n_cells || !verts || !gn || !n_dofs ||
      !n_active || !rp || !col) {
    set_error("bad arguments");
    return CDG_ERR_ARG;
  }
  const int shape = cell_type == CDG_CELL_QUAD ? kQuad : cell_type == CDG_CELL_HEXA ? kHexa : kTetra;
  const int dim = shape == kQuad ? 2 : 3;
  CDG_CUDA(cudaSetDevice(ctx->device));
  cdg_problem* p = new cdg_problem();
  p->ctx = ctx;
  p->dim = dim;
  p->shape = shape;
  p->order = order;
  p->lev.resize(nl);
  int nv = n_vertices(shape);
  int nloc = n_local_dofs(shape, order);
  std::vector<std::vector<int>> parents;
  for (int l = 0; l < nl; ++l) {
    DevLevel& L = p->lev[l];
    if (n_cells[l] < 1 || n_dofs[l] < 1 || n_active[l] < 0 || n_active[l] > n_dofs[l]) {
      delete p;
      set_error("bad sizes on level %d", l);
      return CDG_ERR_ARG;
    }
    L.mesh.dim = dim;
    L.mesh.shape = shape;
    L.mesh.nv = nv;
    L.mesh.ncells = n_cells[l];
    L.mesh.verts.assign(verts[l], verts[l] + (size_t)n_cells[l] * nv * dim);
    L.space.dim = dim;
    L.space.shape = shape;
    L.space.order = order;
    L.space.nloc = nloc;
    L.space.ndof = n_dofs[l];
    L.space.nactive = n_active[l];
    L.space.gdof.assign(gn[l], gn[l] + (size_t)n_cells[l] * nloc);
    for (int v : L.space.gdof)
      if (v < 0 || v >= n_dofs[l]) {
        delete p;
        set_error("global number out of range on level %d", l);
        return CDG_ERR_ARG;
      }
    L.pattern.nrows = n_dofs[l];
    L.pattern.row_ptr.assign(rp[l], rp[l] + n_dofs[l] + 1);
    int nnz = rp[l][n_dofs[l]];
    L.pattern.col.assign(col[l], col[l] + nnz);
    for (int v : L.pattern.col)
      if (v < 0 || v >= n_dofs[l]) {
        delete p;
        set_error("column index out of range on level %d", l);
        return CDG_ERR_ARG;
      }
    fill_level(L, shape, order);
    if (l >= 1) {
      std::vector<int> par(n_cells[l - 1]);
      int nch = dim == 2 ? 4 : 8;
      for (int f = 0; f < n_cells[l - 1]; ++f) {
        par[f] = (parent && parent[l]) ? parent[l][f] : f / nch;
        if (par[f] < 0 || par[f] >= n_cells[l]) {
          delete p;
          set_error("parent index out of range on level %d", l);
          return CDG_ERR_ARG;
        }
      }
      parents.push_back(par);
    }
  }
  int rc = finish_problem(ctx, p, parents, nullptr);
  if (rc != CDG_OK) {
    cdg_problem_destroy(p);
    return rc;
  }
  *out = p;
  return CDG_OK;
}

int cdg_problem_create_from_arrays(cdg_context* ctx, int cell_type, int order, int n_levels,
                                   const int* n_cells, const double* const* cell_vertices,
                                   const int* const* global_numbers, const int* n_dofs,
                                   const int* n_active, const int* const* row_ptr,
                                   const int* const* col, const int* const* parent,
                                   cdg_problem** out) {
  API_GUARD(problem_from_arrays(ctx, cell_type, order, n_levels, n_cells, cell_vertices,
                                global_numbers, n_dofs, n_active, row_ptr, col, parent, out));
}

int cdg_problem_destroy(cdg_problem* p) {
  if (!p) return CDG_OK;
  cudaSetDevice(p->ctx->device);
  cudaStreamSynchronize(p->ctx->stream);
  for (auto& L : p->lev) free_level(L);
  free_gmres(p->gm);
  if (p->d_tables) cudaFree(p->d_tables);
  if (p->d_zero_diag) cudaFree(p->d_zero_diag);
  delete p;
  return CDG_OK;
}

static int assemble_all(cdg_problem* p, const cdg_assembly_params* a) {
  CDG_CUDA(cudaMemsetAsync(p->d_zero_diag, 0, sizeof(int), p->ctx->stream));
  const size_t nl = p->lev.size();
  for (size_t l = 0; l < nl; ++l) {
    // with the option, the levels between the finest and the coarsest (FP32
    // operators of the mixed-precision multigrid) come from the tensor cores
    if (p->tc_levels && l > 0 && l + 1 < nl && !p->lev[l].multilinear)
      CDG_TRY(assemble_level_tc(p->ctx, p, p->lev[l], *a));
    else
      CDG_TRY(assemble_level(p->ctx, p, p->lev[l], *a));
  }
  return CDG_OK;
}

int cdg_problem_assemble(cdg_problem* p, const cdg_assembly_params* a) {
  CDG_TRY(check_assembly_params(p, a));
  CDG_CUDA(cudaSetDevice(p->ctx->device));
  CDG_TRY(assemble_all(p, a));
  return check_device_error(p->ctx);
}

static int check_solver_params(const cdg_problem* p, const cdg_solver_params* s) {
  if (!p || !s) { set_error("null argument"); return CDG_ERR_ARG; }
  if (s->preconditioner < 0 || s->preconditioner > 2) { set_error("unknown preconditioner"); return CDG_ERR_ARG; }
  if (s->gmres_restart < 1 || s->gmres_restart > 120) { set_error("gmres_restart out of range [1,120]"); return CDG_ERR_ARG; }
  if (s->precision != 0 && s->precision != 1) { set_error("precision must be 0 or 1"); return CDG_ERR_ARG; }
  return CDG_OK;
}

int cdg_problem_solve(cdg_problem* p, const cdg_solver_params* s, cdg_solve_stats* st) {
  CDG_TRY(check_solver_params(p, s));
  CDG_CUDA(cudaSetDevice(p->ctx->device));
  auto t0 = std::chrono::steady_clock::now();
  cdg_solve_stats local{};
  CDG_TRY(prepare_solver(p->ctx, p, *s));
  int rc = fgmres(p->ctx, p, *s, &local);
  CDG_CUDA(cudaStreamSynchronize(p->ctx->stream));
  local.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (st) *st = local;
  return rc;
}

int cdg_solve_batched(cdg_context* ctx, int count, cdg_problem* const* probs,
                      const cdg_solver_params* params, int* status, cdg_solve_stats* stats) {
  if (!ctx || count < 0 || (count > 0 && (!probs || !params || !status || !stats))) {
    set_error("bad arguments");
    return CDG_ERR_ARG;
  }
  for (int q = 0; q < count; ++q) {
    cdg_problem* p = probs[q];
    if (!p || !p->ctx || p->ctx->device != ctx->device) {
      set_error("problem %d is null or on another device", q);
      return CDG_ERR_ARG;
    }
    CDG_TRY(check_solver_params(p, &params[q]));
    const char* why = nullptr;
    if (!batch_eligible(p, params[q], &why)) {
      set_error("problem %d: %s", q, why);
      return CDG_ERR_ARG;
    }
    for (int r = 0; r < q; ++r)
      if (probs[r] == p) {
        set_error("problem %d appears twice in the batch", q);
        return CDG_ERR_ARG;
      }
  }
  CDG_CUDA(cudaSetDevice(ctx->device));
  auto t0 = std::chrono::steady_clock::now();
  cudaEvent_t ev = nullptr;
  std::vector<int> inl((size_t)std::max(count, 1), 0);
  for (int q = 0; q < count; ++q) {
    cdg_problem* p = probs[q];
    CDG_TRY(batch_prepare(p->ctx, p, params[q], &inl[q]));
    if (p->ctx->stream != ctx->stream) {
      if (!ev) CDG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
      CDG_CUDA(cudaEventRecord(ev, p->ctx->stream));
      CDG_CUDA(cudaStreamWaitEvent(ctx->stream, ev, 0));
    }
  }
  std::vector<BatchResult> res((size_t)std::max(count, 1));
  int rc = batch_launch(ctx, probs, params, inl.data(), count, res.data());
  if (ev) cudaEventDestroy(ev);
  if (rc != CDG_OK) return rc;
  const double secs =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (int q = 0; q < count; ++q) {
    status[q] = res[q].status;
    stats[q].iterations = res[q].iterations;
    stats[q].residual = res[q].residual;
    stats[q].initial_residual = res[q].initial;
    stats[q].seconds = secs;
  }
  return CDG_OK;
}

int cdg_problem_assemble_solve(cdg_problem* p, const cdg_assembly_params* a,
                               const cdg_solver_params* s, const double* solution_in,
                               double* rhs_out, double* solution_out, cdg_solve_stats* st) {
  CDG_TRY(check_assembly_params(p, a));
  CDG_TRY(check_solver_params(p, s));
  CDG_CUDA(cudaSetDevice(p->ctx->device));
  auto t0 = std::chrono::steady_clock::now();
  DevLevel& F = p->lev[0];
  cudaStream_t stm = p->ctx->stream;
  if (solution_in)
    CDG_CUDA(cudaMemcpyAsync(F.sol, solution_in, (size_t)F.ndof * sizeof(double),
                             cudaMemcpyHostToDevice, stm));
  CDG_TRY(assemble_all(p, a));
  cdg_solve_stats local{};
  CDG_TRY(prepare_solver(p->ctx, p, *s));
  int rc = fgmres(p->ctx, p, *s, &local);
  if (rhs_out)
    CDG_CUDA(cudaMemcpyAsync(rhs_out, F.rhs, (size_t)F.ndof * sizeof(double),
                             cudaMemcpyDeviceToHost, stm));
  if (solution_out)
    CDG_CUDA(cudaMemcpyAsync(solution_out, F.sol, (size_t)F.ndof * sizeof(double),
                             cudaMemcpyDeviceToHost, stm));
  CDG_CUDA(cudaStreamSynchronize(stm));
  local.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (st) *st = local;
  return rc;
}

int cdg_problem_errors(cdg_problem* p, const cdg_assembly_params* a, double* errors) {
  CDG_TRY(check_assembly_params(p, a));
  if (!errors) { set_error("null output"); return CDG_ERR_ARG; }
  CDG_CUDA(cudaSetDevice(p->ctx->device));
  return level_errors(p->ctx, p, p->lev[0], *a, errors);
}

// ---------------------------------------------------------------------------
// time-dependent CD
// ---------------------------------------------------------------------------
int cdg_problem_tcd_initialize(cdg_problem* p, const cdg_assembly_params* a) {
  CDG_TRY(check_assembly_params(p, a));
  CDG_CUDA(cudaSetDevice(p->ctx->device));
  CDG_CUDA(cudaMemsetAsync(p->d_zero_diag, 0, sizeof(int), p->ctx->stream));
  p->tcd_step = 0;
  const TimeScheme ts = time_scheme(*a, 0);
  for (auto& L : p->lev) {
    CDG_TRY(tcd_assemble_level(p->ctx, p, L, *a, true, ts.theta1, a->time_step));
    // old_rhs = rhs
    CDG_CUDA(cudaMemcpyAsync(L.tcd_fold, L.tcd_f, (size_t)L.ndof * sizeof(double),
                             cudaMemcpyDeviceToDevice, p->ctx->stream));
  }
  CDG_TRY(tcd_interpolate(p->ctx, p, *a));
  DevLevel& F = p->lev[0];
  // solution_m2 = solution_m1 = the initial solution (TimeConvectionDiffusion.C:306-310)
  CDG_TRY(tcd_start_history(p->ctx, F));
  return check_device_error(p->ctx);
}

int cdg_problem_tcd_step(cdg_problem* p, const cdg_assembly_params* a, double tau,
                         const cdg_solver_params* s, cdg_solve_stats* st) {
  CDG_TRY(check_assembly_params(p, a));
  CDG_TRY(check_solver_params(p, s));
  if (!(tau > 0)) { set_error("time step must be positive"); return CDG_ERR_ARG; }
  if (!p->lev[0].tcd_A) { set_error("call cdg_problem_tcd_initialize first"); return CDG_ERR_ARG; }
  CDG_CUDA(cudaSetDevice(p->ctx->device));
  auto t0 = std::chrono::steady_clock::now();
  cudaStream_t stm = p->ctx->stream;
  CDG_CUDA(cudaMemsetAsync(p->d_zero_diag, 0, sizeof(int), stm));
  const TimeScheme ts = time_scheme(*a, ++p->tcd_step);
  DevLevel& F = p->lev[0];
  // reassemble stiffness and rhs on every level (the Galerkin mass is time
  // independent; the SUPG mass is reassembled with theta1 * tau)
  for (auto& L : p->lev)
    CDG_TRY(tcd_assemble_level(p->ctx, p, L, *a, false, ts.theta1, tau));
  CDG_TRY(tcd_rhs(p->ctx, F, ts, tau));
  // solution.copy_nonactive(rhs): Dirichlet data at the new time
  const int nd = F.ndof - F.nactive;
  if (nd > 0)
    CDG_CUDA(cudaMemcpyAsync(F.sol + F.nactive, F.rhs + F.nactive, (size_t)nd * sizeof(double),
                             cudaMemcpyDeviceToDevice, stm));
  for (auto& L : p->lev) CDG_TRY(tcd_system(p->ctx, p, L, ts, tau));
  cdg_solve_stats local{};
  CDG_TRY(prepare_solver(p->ctx, p, *s));
  int rc = fgmres(p->ctx, p, *s, &local);
  CDG_CUDA(cudaStreamSynchronize(stm));
  local.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (st) *st = local;
  return rc;
}

// ---------------------------------------------------------------------------
// data access
// ---------------------------------------------------------------------------
static DevLevel* get_level(cdg_problem* p, int level) {
  if (!p || level < 0 || level >= (int)p->lev.size()) {
    set_error("bad level %d", level);
    return nullptr;
  }
  cudaSetDevice(p->ctx->device);
  return &p->lev[level];
}

int cdg_problem_operator_layout(const cdg_problem* p, int level, int* lanes, long long* slots,
                                int* smoother_chunk) {
  if (!p || level < 0 || level >= (int)p->lev.size() || !lanes || !slots || !smoother_chunk) {
    set_error("bad arguments");
    return CDG_ERR_ARG;
  }
  const DevLevel& L = p->lev[level];
  *lanes = L.sell_nslices ? L.sell_lanes : 0;
  *slots = L.sell_nslices ? L.sell_total : 0;
  *smoother_chunk = L.bulk_nchunks ? L.bulk_chunk : 0;
  return CDG_OK;
}

int cdg_problem_lattice(const cdg_problem* p, int level, int* dims, int* transfer) {
  if (!p || level < 0 || level >= (int)p->lev.size() || !dims || !transfer) {
    set_error("bad arguments");
    return CDG_ERR_ARG;
  }
  const DevLevel& L = p->lev[level];
  for (int d = 0; d < 3; ++d) dims[d] = L.st_dims[d];
  *transfer = L.lt_state;
  return CDG_OK;
}

int cdg_problem_level_info(const cdg_problem* p, int level, int* info) {
  if (!p || level < 0 || level >= (int)p->lev.size() || !info) { set_error("bad level"); return CDG_ERR_ARG; }
  const DevLevel& L = p->lev[level];
  info[0] = L.ncells; info[1] = L.nloc; info[2] = L.ndof;
  info[3] = L.nactive; info[4] = L.nnz; info[5] = L.nv;
  return CDG_OK;
}

static int d2h(cdg_context* ctx, void* h, const void* d, size_t bytes) {
  CDG_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  return CDG_OK;
}

int cdg_problem_get_matrix(cdg_problem* p, int level, double* v) {
  DevLevel* L = get_level(p, level);
  if (!L || !v) return CDG_ERR_ARG;
  CDG_CUDA(cudaSetDevice(p->ctx->device));
  CDG_TRY(ensure_fp64(p->ctx, p, *L));
  return d2h(p->ctx, v, L->val64, (size_t)L->nnz * sizeof(double));
}
int cdg_problem_get_matrix32(cdg_problem* p, int level, float* v) {
  DevLevel* L = get_level(p, level);
  if (!L || !v) { set_error("bad arguments"); return CDG_ERR_ARG; }
  CDG_CUDA(cudaSetDevice(p->ctx->device));
  return d2h(p->ctx, v, L->val32, (size_t)L->nnz * sizeof(float));
}
int cdg_problem_set_fp32_tensor_levels(cdg_problem* p, int enable) {
  if (!p || enable < 0 || enable > 1) { set_error("bad arguments"); return CDG_ERR_ARG; }
  p->tc_levels = enable;
  return CDG_OK;
}
int cdg_problem_get_tcd_matrix(cdg_problem* p, int level, int which, double* v) {
  DevLevel* L = get_level(p, level);
  if (!L || !v || which < 0 || which > 2) { set_error("bad arguments"); return CDG_ERR_ARG; }
  if (!L->tcd_A) { set_error("no time-dependent matrices: call cdg_problem_tcd_initialize"); return CDG_ERR_ARG; }
  const double* src = which == 0 ? L->tcd_A : which == 1 ? L->tcd_M : L->val64;
  return d2h(p->ctx, v, src, (size_t)L->nnz * sizeof(double));
}

int cdg_problem_get_rhs(cdg_problem* p, int level, double* v) {
  DevLevel* L = get_level(p, level);
  if (!L || !v) return CDG_ERR_ARG;
  return d2h(p->ctx, v, L->rhs, (size_t)L->ndof * sizeof(double));
}
int cdg_problem_get_solution(cdg_problem* p, double* v) {
  DevLevel* L = get_level(p, 0);
  if (!L || !v) return CDG_ERR_ARG;
  return d2h(p->ctx, v, L->sol, (size_t)L->ndof * sizeof(double));
}
int cdg_problem_set_solution(cdg_problem* p, const double* v) {
  DevLevel* L = get_level(p, 0);
  if (!L) return CDG_ERR_ARG;
  if (!v)
    CDG_CUDA(cudaMemsetAsync(L->sol, 0, (size_t)L->ndof * sizeof(double), p->ctx->stream));
  else
    CDG_CUDA(cudaMemcpyAsync(L->sol, v, (size_t)L->ndof * sizeof(double), cudaMemcpyHostToDevice,
                             p->ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(p->ctx->stream));
  return CDG_OK;
}
int cdg_problem_get_slots(cdg_problem* p, int level, int* slots) {
  DevLevel* L = get_level(p, level);
  if (!L || !slots) return CDG_ERR_ARG;
  return d2h(p->ctx, slots, L->slot, (size_t)L->ncells * L->nloc * L->nloc * sizeof(int));
}

// ---------------------------------------------------------------------------
// operator pieces with host buffers
// ---------------------------------------------------------------------------
struct DevBuf {
  double* d = nullptr;
  ~DevBuf() { if (d) cudaFree(d); }
};

static int h2d_tmp(DevBuf& b, const double* h, size_t n, cudaStream_t st) {
  CDG_CUDA(cudaMalloc(&b.d, std::max<size_t>(n, 1) * sizeof(double)));
  if (h) CDG_CUDA(cudaMemcpyAsync(b.d, h, n * sizeof(double), cudaMemcpyHostToDevice, st));
  return CDG_OK;
}

int cdg_problem_apply(cdg_problem* p, int level, const double* x, double* y) {
  DevLevel* L = get_level(p, level);
  if (!L || !x || !y) return CDG_ERR_ARG;
  CDG_CUDA(cudaSetDevice(p->ctx->device));
  CDG_TRY(ensure_fp64(p->ctx, p, *L));
  DevBuf dx, dy;
  CDG_TRY(h2d_tmp(dx, x, L->ndof, p->ctx->stream));
  CDG_TRY(h2d_tmp(dy, nullptr, L->ndof, p->ctx->stream));
  CDG_TRY(spmv_apply64(p->ctx, *L, dx.d, dy.d));
  return d2h(p->ctx, y, dy.d, (size_t)L->ndof * sizeof(double));
}

int cdg_problem_quadrature_points(cdg_problem* p, const cdg_assembly_params* a, int level,
                                  int* nqp, double* x) {
  CDG_TRY(check_assembly_params(p, a));
  DevLevel* L = get_level(p, level);
  if (!L || !nqp) { set_error("bad arguments"); return CDG_ERR_ARG; }
  return level_quadrature_points(*L, *a, nqp, x);
}

int cdg_problem_assemble_coefficients(cdg_problem* p, const cdg_assembly_params* a, int level,
                                      const double* coeffs) {
  CDG_TRY(check_assembly_params(p, a));
  DevLevel* L = get_level(p, level);
  if (!L || !coeffs) { set_error("bad arguments"); return CDG_ERR_ARG; }
  CDG_CUDA(cudaSetDevice(p->ctx->device));
  CDG_CUDA(cudaMemsetAsync(p->d_zero_diag, 0, sizeof(int), p->ctx->stream));
  CDG_TRY(assemble_level_coefficients(p->ctx, p, *L, *a, coeffs));
  return check_device_error(p->ctx);
}

int cdg_problem_tuning(cdg_problem* p, int level, int* choice, int* shape, double* ms) {
  DevLevel* L = get_level(p, level);
  if (!L || !choice) { set_error("bad arguments"); return CDG_ERR_ARG; }
  *choice = L->tuned ? L->mf_mode : -2;
  if (shape) {
    shape[0] = L->tpr32 ? L->tpr32 : L->rows_per_warp_hint;
    shape[1] = L->mf_blocks_per_sm;
  }
  if (ms) {
    ms[0] = L->tuned_ms[0];
    ms[1] = L->tuned_ms[1];
  }
  return CDG_OK;
}

int cdg_problem_apply32(cdg_problem* p, int level, int variant, const float* x, float* y) {
  DevLevel* L = get_level(p, level);
  if (!L || !x || !y || variant < 0 || variant > 3) { set_error("bad arguments"); return CDG_ERR_ARG; }
  if (variant >= 1 && !L->mf_valid) {
    set_error("no matrix-free operator on level %d (Q2 hexahedra after a stationary assembly)",
              level);
    return CDG_ERR_ARG;
  }
  CDG_CUDA(cudaSetDevice(p->ctx->device));
  const size_t n = (size_t)std::max(L->ndof, 1);
  float *dx = nullptr, *dy = nullptr;
  CDG_CUDA(cudaMalloc(&dx, n * sizeof(float)));
  int rc = CDG_OK;
  if (cudaMalloc(&dy, n * sizeof(float)) != cudaSuccess) rc = CDG_ERR_OOM;
  if (rc == CDG_OK &&
      cudaMemcpyAsync(dx, x, (size_t)L->ndof * sizeof(float), cudaMemcpyHostToDevice,
                      p->ctx->stream) != cudaSuccess)
    rc = CDG_ERR_CUDA;
  if (rc == CDG_OK) rc = apply32(p->ctx, *L, variant, dx, dy);
  if (rc == CDG_OK) rc = d2h(p->ctx, y, dy, (size_t)L->ndof * sizeof(float));
  cudaFree(dx);
  if (dy) cudaFree(dy);
  if (rc == CDG_ERR_OOM) set_error("out of device memory");
  return rc;
}

int cdg_problem_prolongate(cdg_problem* p, int fine, const double* xc, double* xf) {
  DevLevel* F = get_level(p, fine);
  DevLevel* C = get_level(p, fine + 1);
  if (!F || !C || !xc || !xf) return CDG_ERR_ARG;
  DevBuf dc, df;
  CDG_TRY(h2d_tmp(dc, xc, C->ndof, p->ctx->stream));
  CDG_TRY(h2d_tmp(df, nullptr, F->ndof, p->ctx->stream));
  CDG_TRY(lattice_transfer_setup(p->ctx, *F, *C));
  CDG_TRY(prolongate64(p->ctx, *F, *C, dc.d, df.d, 0, 0.0));
  return d2h(p->ctx, xf, df.d, (size_t)F->ndof * sizeof(double));
}

int cdg_problem_restrict(cdg_problem* p, int fine, const double* dfine, double* rc) {
  DevLevel* F = get_level(p, fine);
  DevLevel* C = get_level(p, fine + 1);
  if (!F || !C || !dfine || !rc) return CDG_ERR_ARG;
  DevBuf df, dc;
  CDG_TRY(h2d_tmp(df, dfine, F->ndof, p->ctx->stream));
  CDG_TRY(h2d_tmp(dc, nullptr, C->ndof, p->ctx->stream));
  CDG_TRY(lattice_transfer_setup(p->ctx, *F, *C));
  CDG_TRY(restrict64(p->ctx, *F, *C, df.d, dc.d));
  return d2h(p->ctx, rc, dc.d, (size_t)C->ndof * sizeof(double));
}

int cdg_problem_precondition(cdg_problem* p, const cdg_solver_params* s, const double* v,
                             double* z) {
  CDG_TRY(check_solver_params(p, s));
  if (!v || !z) { set_error("null buffer"); return CDG_ERR_ARG; }
  CDG_CUDA(cudaSetDevice(p->ctx->device));
  CDG_TRY(prepare_solver(p->ctx, p, *s));
  DevLevel& F = p->lev[0];
  DevBuf dv, dz;
  CDG_TRY(h2d_tmp(dv, v, F.ndof, p->ctx->stream));
  CDG_TRY(h2d_tmp(dz, nullptr, F.ndof, p->ctx->stream));
  CDG_TRY(precondition(p->ctx, p, *s, dv.d, dz.d));
  CDG_TRY(d2h(p->ctx, z, dz.d, (size_t)F.ndof * sizeof(double)));
  return check_device_error(p->ctx);
}

// ---------------------------------------------------------------------------
// measurement
// ---------------------------------------------------------------------------
int cdg_problem_time_kernel(cdg_problem* p, const cdg_assembly_params* a, int kernel, int level,
                            int reps, double* ms) {
  DevLevel* L = get_level(p, level);
  if (!L || !ms || reps < 1 || kernel < 0 || kernel > 3 || (kernel == 2 && !a)) {
    set_error("bad arguments");
    return CDG_ERR_ARG;
  }
  cdg_context* ctx = p->ctx;
  if (kernel == 1 || kernel == 2) CDG_TRY(ensure_fp64(ctx, p, *L));
  cudaEvent_t e0, e1;
  CDG_CUDA(cudaEventCreate(&e0));
  CDG_CUDA(cudaEventCreate(&e1));
  auto once = [&]() -> int {
    switch (kernel) {
      case 0: return smooth32_once(ctx, *L, 0.8f);
      case 1: return spmv_apply64(ctx, *L, L->sol, L->invdiag64);
      case 2: return contract_only(ctx, p, *L, *a);
      default: return defect32_once(ctx, *L);
    }
  };
  // scratch target of the FP64 SpMV: invdiag64 is restored below
  int rc = once();  // warm-up (allocates multigrid vectors if needed)
  if (rc == CDG_OK) {
    CDG_CUDA(cudaEventRecord(e0, ctx->stream));
    for (int r = 0; r < reps && rc == CDG_OK; ++r) rc = once();
    CDG_CUDA(cudaEventRecord(e1, ctx->stream));
    CDG_CUDA(cudaEventSynchronize(e1));
    float t = 0;
    CDG_CUDA(cudaEventElapsedTime(&t, e0, e1));
    *ms = (double)t / reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != CDG_OK) return rc;
  if (kernel == 1 || kernel == 2) {
    // restore the level's matrix data (the timing loop overwrote them)
    if (!a) { set_error("assembly parameters needed to restore the level"); return CDG_ERR_ARG; }
    CDG_TRY(assemble_level(ctx, p, *L, *a));
    CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  return CDG_OK;
}

}  // extern "C"
