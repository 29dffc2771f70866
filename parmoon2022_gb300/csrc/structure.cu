// structure.cu -- FE space numbering and TStructure (CSR pattern) built on the
// device, bit-exact with the host setup layer (make_space / make_pattern).
//
// Numbering (TFESpace3D::ConstructSpace + TFESpace::compute_various_numbers,
// src/FE/FESpace3D.C:186, src/FE/FESpace.C:1863-2099): every (cell, local
// DOF) names a lattice point of the structured mesh; points are numbered per
// class (inner, non-Dirichlet boundary, Dirichlet last), each class in the
// order of the point's first appearance over (cell, local DOF).  On the
// device the first appearance of a point is an atomicMin over the flat index
// cell * nloc + k (a deterministic result), and the numbers are a three-class
// exclusive scan over the first appearances in flat order.
//
// Pattern (TStructure(space), src/Matrix/Structure.C:226-556, add_entry
// :122-140, Sort :607-618): row r holds every DOF of every cell containing r,
// columns sorted ascending, no duplicates, full rows for Dirichlet DOFs.  On
// the device every incidence appends its cell's DOFs to the row (atomic
// cursors, so the order is not fixed), then one CTA per row sorts its entries
// in shared memory (bitonic) and keeps the distinct ones, which fixes the
// result.  Row offsets are exclusive scans.
#include <algorithm>
#include <climits>
#include <cmath>

#include "common.cuh"

namespace cdg {

// ---------------------------------------------------------------------------
// exclusive scan with K counters per element (tiles of 2048 elements)
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanPer = 8;
constexpr int kScanTile = kScanThreads * kScanPer;

template <int K>
__device__ void block_exclusive_scan(long long (&v)[K], long long (&total)[K]) {
  __shared__ long long sh[kScanThreads / 32][K];
  const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    long long x = v[k];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (l >= o) x += y;
    }
    if (l == 31) sh[w][k] = x;
    v[k] = x - v[k];   // exclusive within the warp
  }
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      long long x = l < kScanThreads / 32 ? sh[l][k] : 0;
      const long long x0 = x;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (l >= o) x += y;
      }
      if (l < kScanThreads / 32) sh[l][k] = x - x0;
      if (l == kScanThreads / 32 - 1) total[k] = x;   // only lane 7 holds it
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] += sh[w][k];
  __syncthreads();
}

// per-tile sums of f over the tile's elements
template <int K, typename F>
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(long n, F f, long long* tile_sums) {
  const long base = (long)blockIdx.x * kScanTile + (long)threadIdx.x * kScanPer;
  long long s[K];
#pragma unroll
  for (int k = 0; k < K; ++k) s[k] = 0;
  for (int e = 0; e < kScanPer; ++e) {
    const long i = base + e;
    if (i < n) {
      long long v[K];
      f(i, v);
#pragma unroll
      for (int k = 0; k < K; ++k) s[k] += v[k];
    }
  }
  long long tot[K];
  block_exclusive_scan<K>(s, tot);
  __shared__ long long bt[K];
  // the totals are in lane kScanThreads/32-1 of warp 0
  if (threadIdx.x == kScanThreads / 32 - 1)
#pragma unroll
    for (int k = 0; k < K; ++k) bt[k] = tot[k];
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) tile_sums[(size_t)blockIdx.x * K + k] = bt[k];
}

// exclusive scan of the tile sums in place (one CTA); totals[k] = grand total
template <int K>
__global__ void __launch_bounds__(kScanThreads) k_scan_top(int ntiles, long long* tile_sums,
                                                           long long* totals) {
  const int per = (ntiles + kScanThreads - 1) / kScanThreads;
  const int b = threadIdx.x * per, e = min(ntiles, b + per);
  long long s[K];
#pragma unroll
  for (int k = 0; k < K; ++k) s[k] = 0;
  for (int t = b; t < e; ++t)
#pragma unroll
    for (int k = 0; k < K; ++k) s[k] += tile_sums[(size_t)t * K + k];
  long long tot[K];
  long long pre[K];
#pragma unroll
  for (int k = 0; k < K; ++k) pre[k] = s[k];
  block_exclusive_scan<K>(pre, tot);
  __shared__ long long bt[K];
  if (threadIdx.x == kScanThreads / 32 - 1)
#pragma unroll
    for (int k = 0; k < K; ++k) bt[k] = tot[k];
  for (int t = b; t < e; ++t)
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const long long v = tile_sums[(size_t)t * K + k];
      tile_sums[(size_t)t * K + k] = pre[k];
      pre[k] += v;
    }
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) totals[k] = bt[k];
}

// g(i, prefix) for every element, prefix = exclusive scan of f before i
template <int K, typename F, typename G>
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(long n, F f, G g,
                                                             const long long* tile_off) {
  const long base = (long)blockIdx.x * kScanTile + (long)threadIdx.x * kScanPer;
  long long v[kScanPer][K], s[K];
#pragma unroll
  for (int k = 0; k < K; ++k) s[k] = 0;
#pragma unroll
  for (int e = 0; e < kScanPer; ++e) {
    const long i = base + e;
    if (i < n) {
      f(i, v[e]);
    } else {
#pragma unroll
      for (int k = 0; k < K; ++k) v[e][k] = 0;
    }
#pragma unroll
    for (int k = 0; k < K; ++k) s[k] += v[e][k];
  }
  long long tot[K];
  block_exclusive_scan<K>(s, tot);
#pragma unroll
  for (int k = 0; k < K; ++k) s[k] += tile_off[(size_t)blockIdx.x * K + k];
#pragma unroll
  for (int e = 0; e < kScanPer; ++e) {
    const long i = base + e;
    if (i < n) g(i, s);
#pragma unroll
    for (int k = 0; k < K; ++k) s[k] += v[e][k];
  }
}

// scratch for the scans: tile sums + totals
struct ScanScratch {
  long long* tiles = nullptr;
  long long* totals = nullptr;
  int cap = 0;
  ~ScanScratch() {
    if (tiles) cudaFree(tiles);
    if (totals) cudaFree(totals);
  }
};

template <int K, typename F, typename G>
static int device_scan(cdg_context* ctx, ScanScratch& sc, long n, F f, G g, long long* host_totals) {
  const int ntiles = (int)std::max<long>(1, (n + kScanTile - 1) / kScanTile);
  if (sc.cap < ntiles * K) {
    if (sc.tiles) cudaFree(sc.tiles);
    CDG_CUDA(cudaMalloc(&sc.tiles, (size_t)ntiles * K * sizeof(long long)));
    sc.cap = ntiles * K;
  }
  if (!sc.totals) CDG_CUDA(cudaMalloc(&sc.totals, 8 * sizeof(long long)));
  CDG_LAUNCH(ctx, (k_scan_tiles<K, F>), ntiles, kScanThreads, 0, n, f, sc.tiles);
  CDG_LAUNCH(ctx, (k_scan_top<K>), 1, kScanThreads, 0, ntiles, sc.tiles, sc.totals);
  CDG_LAUNCH(ctx, (k_scan_apply<K, F, G>), ntiles, kScanThreads, 0, n, f, g, sc.tiles);
  if (host_totals) {
    CDG_CUDA(cudaMemcpyAsync(host_totals, sc.totals, K * sizeof(long long),
                             cudaMemcpyDeviceToHost, ctx->stream));
    CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  return CDG_OK;
}

// ---------------------------------------------------------------------------
// numbering
// ---------------------------------------------------------------------------
struct NumberingArgs {
  int shape, dim, nl, nres, n1l, neumann_mask;
  int comp[3][2];        // boundary component of the face x_a = side
  double ref[kMaxLoc][3];
};

// lattice point and class of every (cell, local DOF); first appearance of
// every point by atomicMin over the flat index
__global__ void k_dof_keys(long n, NumberingArgs a, const double* __restrict__ verts,
                           int* __restrict__ keys, signed char* __restrict__ cls,
                           int* __restrict__ first, int* err) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const long c = i / a.nl;
    const int k = (int)(i - c * a.nl);
    const int nv = a.shape == kHexa ? 8 : 4;
    const double* cv = verts + c * nv * a.dim;
    const double* r = a.ref[k];
    double x[3] = {0, 0, 0};
    if (a.shape == kTetra) {
      for (int d = 0; d < 3; ++d) {
        double s = cv[d];
        for (int q = 0; q < 3; ++q) s += r[q] * (cv[(q + 1) * 3 + d] - cv[d]);
        x[d] = s;
      }
    } else {
      const int e[3] = {1, 3, 4};
      for (int d = 0; d < a.dim; ++d) {
        double s = cv[d];
        for (int q = 0; q < a.dim; ++q) s += 0.5 * (r[q] + 1.0) * (cv[e[q] * a.dim + d] - cv[d]);
        x[d] = s;
      }
    }
    long key = 0;
    bool on = true;
    for (int d = a.dim - 1; d >= 0; --d) {
      const long li = lround(x[d] * a.nres);
      on = on && li >= 0 && li <= a.nres;
      key = key * a.n1l + li;
    }
    if (!on) {   // off the lattice: flag it, leave the point out
      atomicOr(err, kErrLattice);
      keys[i] = 0;
      cls[i] = 0;
      continue;
    }
    int cl = 0;
    for (int d = 0; d < a.dim; ++d)
      for (int side = 0; side < 2; ++side) {
        if (fabs(x[d] - side) >= 1e-12) continue;
        const int t = ((a.neumann_mask >> a.comp[d][side]) & 1) ? 1 : 2;
        cl = max(cl, t);
      }
    keys[i] = (int)key;
    cls[i] = (signed char)cl;
    atomicMin(first + key, (int)i);
  }
}

struct FirstClassCount {
  const int* keys;
  const signed char* cls;
  const int* first;
  __device__ void operator()(long i, long long (&v)[3]) const {
    const bool f = first[keys[i]] == (int)i;
    const int c = cls[i];
    v[0] = f && c == 0;
    v[1] = f && c == 1;
    v[2] = f && c == 2;
  }
};

struct FirstClassNumber {
  const int* keys;
  const signed char* cls;
  const int* first;
  int* num;
  signed char* clsk;
  __device__ void operator()(long i, const long long (&pre)[3]) const {
    const int key = keys[i];
    if (first[key] != (int)i) return;
    const int c = cls[i];
    num[key] = (int)pre[c];
    clsk[key] = (signed char)c;
  }
};

__global__ void k_gdof(long n, const int* __restrict__ keys, const int* __restrict__ num,
                       const signed char* __restrict__ clsk, int off1, int off2,
                       int* __restrict__ gdof) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const int key = keys[i];
    const int c = clsk[key];
    gdof[i] = (c == 0 ? 0 : c == 1 ? off1 : off2) + num[key];
  }
}

__global__ void k_fill_int(long n, int* p, int v) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x)
    p[i] = v;
}

// device buffers freed on scope exit
template <typename T>
struct DBuf {
  T* p = nullptr;
  ~DBuf() {
    if (p) cudaFree(p);
  }
  int alloc(size_t n) {
    CDG_CUDA(cudaMalloc((void**)&p, std::max<size_t>(n, 1) * sizeof(T)));
    return CDG_OK;
  }
};

template <typename T>
static int dalloc_raw(T** p, size_t n) {
  CDG_CUDA(cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T)));
  return CDG_OK;
}

static int fill_grid(cdg_context* ctx, long n) {
  return (int)std::max<long>(1, std::min<long>((n + 255) / 256, (long)ctx->num_sms * 16));
}

int device_space(cdg_context* ctx, const Mesh& m, int order, int neumann_mask, Space* out) {
  const int dim = m.dim, nl = n_local_dofs(m.shape, order);
  if (m.ncells < 1) { set_error("empty mesh"); return CDG_ERR_ARG; }
  double h = 0;
  for (int a = 0; a < dim; ++a) h += std::fabs(m.verts[dim + a] - m.verts[a]);
  if (!(h > 0) || order / h > 1e6) {
    set_error("first cell edge of length %g: no lattice", h);
    return CDG_ERR_ARG;
  }
  const long nres = std::lround(order / h);
  const long n1l = nres + 1;
  const double nk = dim == 2 ? (double)n1l * n1l : (double)n1l * n1l * n1l;
  const long n = (long)m.ncells * nl;
  if (nk >= 2147483647.0 || n >= 2147483647L) {
    set_error("mesh too large for 32-bit lattice keys");
    return CDG_ERR_LIMIT;
  }
  const long nkeys = (long)nk;
  NumberingArgs a{};
  a.shape = m.shape;
  a.dim = dim;
  a.nl = nl;
  a.nres = (int)nres;
  a.n1l = (int)n1l;
  a.neumann_mask = neumann_mask;
  for (int d = 0; d < dim; ++d)
    for (int side = 0; side < 2; ++side) {
      double probe[3] = {0.5, 0.5, 0.5};
      probe[d] = side;
      a.comp[d][side] = boundary_component(dim, probe);
    }
  for (int k = 0; k < nl; ++k) local_dof_ref_shape(m.shape, order, k, a.ref[k]);
  cudaStream_t st = ctx->stream;
  DBuf<double> verts;
  DBuf<int> keys, first, num, gdof;
  DBuf<signed char> cls, clsk;
  CDG_TRY(verts.alloc(m.verts.size()));
  CDG_TRY(keys.alloc(n));
  CDG_TRY(cls.alloc(n));
  CDG_TRY(first.alloc(nkeys));
  CDG_TRY(num.alloc(nkeys));
  CDG_TRY(clsk.alloc(nkeys));
  CDG_TRY(gdof.alloc(n));
  CDG_CUDA(cudaMemcpyAsync(verts.p, m.verts.data(), m.verts.size() * sizeof(double),
                           cudaMemcpyHostToDevice, st));
  CDG_LAUNCH(ctx, k_fill_int, fill_grid(ctx, nkeys), 256, 0, nkeys, first.p, INT_MAX);
  CDG_LAUNCH(ctx, k_dof_keys, fill_grid(ctx, n), 256, 0, n, a, verts.p, keys.p, cls.p, first.p,
             ctx->d_err);
  CDG_TRY(check_device_error(ctx));
  ScanScratch sc;
  long long tot[3];
  CDG_TRY((device_scan<3>(ctx, sc, n, FirstClassCount{keys.p, cls.p, first.p},
                          FirstClassNumber{keys.p, cls.p, first.p, num.p, clsk.p}, tot)));
  const int off1 = (int)tot[0], off2 = (int)(tot[0] + tot[1]);
  CDG_LAUNCH(ctx, k_gdof, fill_grid(ctx, n), 256, 0, n, keys.p, num.p, clsk.p, off1, off2, gdof.p);
  Space s;
  s.dim = dim;
  s.shape = m.shape;
  s.order = order;
  s.nloc = nl;
  s.nactive = off2;
  s.ndof = (int)(tot[0] + tot[1] + tot[2]);
  s.gdof.resize(n);
  CDG_CUDA(cudaMemcpyAsync(s.gdof.data(), gdof.p, n * sizeof(int), cudaMemcpyDeviceToHost, st));
  CDG_CUDA(cudaStreamSynchronize(st));
  CDG_TRY(check_device_error(ctx));
  *out = std::move(s);
  return CDG_OK;
}

// ---------------------------------------------------------------------------
// pattern
// ---------------------------------------------------------------------------
__global__ void k_row_count(long n, int nl, const int* __restrict__ gdof, int* __restrict__ cnt) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x)
    atomicAdd(cnt + gdof[i], nl);
}

__global__ void k_row_max(int nrows, const int* __restrict__ cnt, int* __restrict__ mx) {
  int m = 0;
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < nrows;
       r += (long)gridDim.x * blockDim.x)
    m = max(m, cnt[r]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(mx, m);
}

struct CountOf {
  const int* cnt;
  __device__ void operator()(long i, long long (&v)[1]) const { v[0] = cnt[i]; }
};
struct WriteOffset64 {
  long long* off;
  __device__ void operator()(long i, const long long (&pre)[1]) const { off[i] = pre[0]; }
};
struct WriteOffset32 {
  int* off;
  __device__ void operator()(long i, const long long (&pre)[1]) const { off[i] = (int)pre[0]; }
};

// every incidence (cell, m) appends the cell's DOFs to row gdof[cell, m]
__global__ void k_row_fill(long n, int nl, const int* __restrict__ gdof,
                           const long long* __restrict__ tp, int* __restrict__ cursor,
                           int* __restrict__ tmp) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const long c = i / nl;
    const int r = gdof[i];
    const long long at = tp[r] + atomicAdd(cursor + r, nl);
    for (int k = 0; k < nl; ++k) tmp[at + k] = gdof[c * nl + k];
  }
}

// one CTA per row: bitonic sort of the row's P (power of two) slots in
// shared memory, distinct values written back to the row's start in order
constexpr int kSortThreads = 128;
__global__ void __launch_bounds__(kSortThreads)
k_row_sort_unique(int nrows, int P, const long long* __restrict__ tp, const int* __restrict__ cnt,
                  int* __restrict__ tmp, int* __restrict__ ucnt) {
  extern __shared__ int s[];
  __shared__ int wsum[kSortThreads / 32];
  for (int r = blockIdx.x; r < nrows; r += gridDim.x) {
    const int len = cnt[r];
    int* row = tmp + tp[r];
    for (int t = threadIdx.x; t < P; t += kSortThreads) s[t] = t < len ? row[t] : INT_MAX;
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int t = threadIdx.x; t < P; t += kSortThreads) {
          const int u = t ^ j;
          if (u > t) {
            const int x = s[t], y = s[u];
            const bool up = (t & k) == 0;
            if ((x > y) == up) {
              s[t] = y;
              s[u] = x;
            }
          }
        }
        __syncthreads();
      }
    // distinct values: thread t owns slots [t*E, t*E+E)
    const int E = P / kSortThreads;
    const int b = threadIdx.x * E;
    int mine = 0;
    for (int q = b; q < b + E; ++q)
      if (q < len && (q == 0 || s[q] != s[q - 1])) ++mine;
    // block exclusive scan of `mine`
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (l >= o) x += y;
    }
    if (l == 31) wsum[w] = x;
    __syncthreads();
    int wo = 0, total = 0;
    for (int q = 0; q < kSortThreads / 32; ++q) {
      if (q < w) wo += wsum[q];
      total += wsum[q];
    }
    int at = wo + x - mine;
    for (int q = b; q < b + E; ++q)
      if (q < len && (q == 0 || s[q] != s[q - 1])) row[at++] = s[q];
    if (threadIdx.x == 0) ucnt[r] = total;
    __syncthreads();
  }
}

// one warp per row: the distinct entries to their final place
__global__ void k_row_copy(int nrows, const long long* __restrict__ tp, const int* __restrict__ tmp,
                           const int* __restrict__ rp, int* __restrict__ col) {
  const long wid = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  const int l = threadIdx.x & 31;
  for (long r = wid; r < nrows; r += ((long)gridDim.x * blockDim.x) >> 5) {
    const int b = rp[r], e = rp[r + 1];
    const int* src = tmp + tp[r];
    for (int q = b + l; q < e; q += 32) col[q] = src[q - b];
  }
}

int device_pattern(cdg_context* ctx, int ncells, int nloc, int ndof, const int* gdof_host,
                   const int* gdof_dev, std::vector<int>* row_ptr, std::vector<int>* col,
                   int** col_dev_out, int** rp_dev_out) {
  const long n = (long)ncells * nloc;
  cudaStream_t st = ctx->stream;
  DBuf<int> gd, cnt, cursor, tmp, ucnt, rp, cl, mx;
  DBuf<long long> tp;
  if (!gdof_dev) {
    CDG_TRY(gd.alloc(n));
    CDG_CUDA(cudaMemcpyAsync(gd.p, gdof_host, n * sizeof(int), cudaMemcpyHostToDevice, st));
    gdof_dev = gd.p;
  }
  CDG_TRY(cnt.alloc((size_t)ndof + 1));
  CDG_TRY(cursor.alloc((size_t)ndof + 1));
  CDG_TRY(ucnt.alloc((size_t)ndof + 1));
  CDG_TRY(tp.alloc((size_t)ndof + 1));
  CDG_TRY(rp.alloc((size_t)ndof + 1));
  CDG_TRY(mx.alloc(1));
  CDG_CUDA(cudaMemsetAsync(cnt.p, 0, ((size_t)ndof + 1) * sizeof(int), st));
  CDG_CUDA(cudaMemsetAsync(cursor.p, 0, ((size_t)ndof + 1) * sizeof(int), st));
  CDG_CUDA(cudaMemsetAsync(mx.p, 0, sizeof(int), st));
  CDG_LAUNCH(ctx, k_row_count, fill_grid(ctx, n), 256, 0, n, nloc, gdof_dev, cnt.p);
  CDG_LAUNCH(ctx, k_row_max, fill_grid(ctx, ndof), 256, 0, ndof, cnt.p, mx.p);
  ScanScratch sc;
  long long tot[1];
  CDG_TRY((device_scan<1>(ctx, sc, (long)ndof + 1, CountOf{cnt.p}, WriteOffset64{tp.p}, tot)));
  int maxlen = 0;
  CDG_CUDA(cudaMemcpyAsync(&maxlen, mx.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  CDG_CUDA(cudaStreamSynchronize(st));
  int P = kSortThreads;
  while (P < maxlen) P <<= 1;
  if (P > 16384) {
    set_error("row of %d entries before merging: beyond the shared-memory sort", maxlen);
    return CDG_ERR_LIMIT;
  }
  CDG_TRY(tmp.alloc((size_t)tot[0]));
  CDG_LAUNCH(ctx, k_row_fill, fill_grid(ctx, n), 256, 0, n, nloc, gdof_dev, tp.p, cursor.p, tmp.p);
  const int sgrid = (int)std::min<long>(ndof, (long)ctx->num_sms * 16);
  if (P * sizeof(int) > 48 * 1024)
    CDG_CUDA(cudaFuncSetAttribute(k_row_sort_unique, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(P * sizeof(int))));
  CDG_LAUNCH(ctx, k_row_sort_unique, std::max(1, sgrid), kSortThreads, P * sizeof(int), ndof, P,
             tp.p, cnt.p, tmp.p, ucnt.p);
  CDG_CUDA(cudaMemsetAsync(ucnt.p + ndof, 0, sizeof(int), st));
  long long nnz[1];
  CDG_TRY((device_scan<1>(ctx, sc, (long)ndof + 1, CountOf{ucnt.p}, WriteOffset32{rp.p}, nnz)));
  if (nnz[0] >= 2147483647LL) { set_error("pattern beyond 32-bit offsets"); return CDG_ERR_LIMIT; }
  CDG_TRY(cl.alloc((size_t)nnz[0]));
  CDG_LAUNCH(ctx, k_row_copy, fill_grid(ctx, (long)ndof * 32), 256, 0, ndof, tp.p, tmp.p, rp.p,
             cl.p);
  if (row_ptr) {
    row_ptr->resize((size_t)ndof + 1);
    CDG_CUDA(cudaMemcpyAsync(row_ptr->data(), rp.p, ((size_t)ndof + 1) * sizeof(int),
                             cudaMemcpyDeviceToHost, st));
  }
  if (col) {
    col->resize((size_t)nnz[0]);
    CDG_CUDA(cudaMemcpyAsync(col->data(), cl.p, (size_t)nnz[0] * sizeof(int),
                             cudaMemcpyDeviceToHost, st));
  }
  CDG_CUDA(cudaStreamSynchronize(st));
  CDG_TRY(check_device_error(ctx));
  if (col_dev_out) { *col_dev_out = cl.p; cl.p = nullptr; }
  if (rp_dev_out) { *rp_dev_out = rp.p; rp.p = nullptr; }
  return CDG_OK;
}


// ---------------------------------------------------------------------------
// grid transfer (GridTransfer::Prolongate / DefectRestriction with the child-
// local matrices of GetProlongationMatrix3D, src/Multigrid/GridTransfer.C,
// src/FE/FEDatabase.C:261-574) built on the device: the same matrices as
// make_transfer -- row i of P holds, for every coarse DOF j, the value of the
// parent's basis function j at fine node i, summed over the fine cells that
// contain node i in (cell, local DOF) order and divided by their number; R is
// the transpose with the fine indices of a row ascending
// ---------------------------------------------------------------------------
namespace {

struct TransferArgs {
  int shape, dim, p, nl, nv;
  double ref[kMaxLoc][3];
};

__device__ void parent_basis_values(const TransferArgs& a, const double* __restrict__ cvf,
                                    const double* __restrict__ cvc, int k, double* val) {
  const int dim = a.dim;
  double x0[3] = {0, 0, 0}, J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, Ji[3][3];
  for (int r = 0; r < dim; ++r) x0[r] = cvc[r];
  if (a.shape == kTetra) {
    for (int q = 0; q < 3; ++q)
      for (int r = 0; r < 3; ++r) J[r][q] = cvc[(q + 1) * 3 + r] - x0[r];
  } else {
    const int e[3] = {1, 3, 4};
    for (int q = 0; q < dim; ++q)
      for (int r = 0; r < dim; ++r) {
        const double xa = cvc[r] + 1.0 * (cvc[e[q] * dim + r] - cvc[r]);
        J[r][q] = (xa - x0[r]) / 2.0;
      }
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
  // the fine node (fine cell's affine map) in the parent's reference cell
  const double* r = a.ref[k];
  double x[3] = {0, 0, 0};
  if (a.shape == kTetra) {
    for (int d = 0; d < 3; ++d) {
      double s = cvf[d];
      for (int q = 0; q < 3; ++q) s += r[q] * (cvf[(q + 1) * 3 + d] - cvf[d]);
      x[d] = s;
    }
  } else {
    const int e[3] = {1, 3, 4};
    for (int d = 0; d < dim; ++d) {
      double s = cvf[d];
      for (int q = 0; q < dim; ++q) s += 0.5 * (r[q] + 1.0) * (cvf[e[q] * dim + d] - cvf[d]);
      x[d] = s;
    }
  }
  const double r0 = a.shape == kTetra ? 0.0 : -1.0;
  double xi[3] = {0, 0, 0};
  for (int q = 0; q < dim; ++q) {
    double t = 0;
    for (int rr = 0; rr < dim; ++rr) t += Ji[q][rr] * (x[rr] - x0[rr]);
    xi[q] = r0 + t;
  }
  if (a.shape == kTetra) {
    const double l[4] = {1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]};
    if (a.p == 1) {
      for (int q = 0; q < 4; ++q) val[q] = l[q];
    } else {
      const int va[10] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3};
      const int vb[10] = {0, 1, 1, 2, 2, 2, 3, 3, 3, 3};
      for (int q = 0; q < 10; ++q)
        val[q] = va[q] == vb[q] ? l[va[q]] * (2.0 * l[va[q]] - 1.0) : 4.0 * l[va[q]] * l[vb[q]];
    }
    return;
  }
  const int n1 = a.p + 1;
  double v[3][3];
  for (int q = 0; q < dim; ++q) {
    const double t = xi[q];
    if (a.p == 1) {
      v[q][0] = 0.5 * (1 - t); v[q][1] = 0.5 * (1 + t);
    } else {
      v[q][0] = 0.5 * t * (t - 1); v[q][1] = (1 - t) * (1 + t); v[q][2] = 0.5 * t * (t + 1);
    }
  }
  for (int q = 0; q < a.nl; ++q) {
    const int i0 = q % n1, i1 = (q / n1) % n1, i2 = q / (n1 * n1);
    val[q] = dim == 2 ? v[0][i0] * v[1][i1] : v[0][i0] * v[1][i1] * v[2][i2];
  }
}

constexpr double kTransferDrop = 1e-14;   // basis values below this are not entries

__global__ void k_tr_count(long n, TransferArgs a, const double* __restrict__ fverts,
                           const double* __restrict__ cverts, const int* __restrict__ parent,
                           const int* __restrict__ fgdof, int* __restrict__ cnt,
                           int* __restrict__ mult) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const long f = i / a.nl;
    const int k = (int)(i - f * a.nl);
    double val[kMaxLoc];
    parent_basis_values(a, fverts + f * a.nv * a.dim, cverts + (long)parent[f] * a.nv * a.dim, k,
                        val);
    int nz = 0;
    for (int q = 0; q < a.nl; ++q) nz += fabs(val[q]) >= kTransferDrop;
    const int fi = fgdof[i];
    atomicAdd(cnt + fi, nz);
    atomicAdd(mult + fi, 1);
  }
}

// entry key: coarse column in the high word, the flat source index (cell, local
// DOF) in the low word, so a row sorted by key sums its duplicates in cell order
__global__ void k_tr_fill(long n, TransferArgs a, const double* __restrict__ fverts,
                          const double* __restrict__ cverts, const int* __restrict__ parent,
                          const int* __restrict__ fgdof, const int* __restrict__ cgdof,
                          const long long* __restrict__ tp, int* __restrict__ cursor,
                          long long* __restrict__ key, double* __restrict__ tval) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const long f = i / a.nl;
    const int k = (int)(i - f * a.nl);
    const int c = parent[f];
    double val[kMaxLoc];
    parent_basis_values(a, fverts + f * a.nv * a.dim, cverts + (long)c * a.nv * a.dim, k, val);
    const int fi = fgdof[i];
    for (int q = 0; q < a.nl; ++q) {
      if (fabs(val[q]) < kTransferDrop) continue;
      const long long at = tp[fi] + atomicAdd(cursor + fi, 1);
      key[at] = ((long long)cgdof[(long)c * a.nl + q] << 32) | (long long)(unsigned)i;
      tval[at] = val[q];
    }
  }
}

// one CTA per segment: bitonic sort of the segment's (key, value) pairs
constexpr int kPairThreads = 128;
__global__ void __launch_bounds__(kPairThreads)
k_seg_sort_pairs(int nseg, int P, const long long* __restrict__ off, const int* __restrict__ len,
                 long long* __restrict__ key, double* __restrict__ val) {
  extern __shared__ __align__(16) unsigned char pair_smem[];
  long long* sk = reinterpret_cast<long long*>(pair_smem);
  double* sv = reinterpret_cast<double*>(pair_smem + (size_t)P * sizeof(long long));
  for (int s = blockIdx.x; s < nseg; s += gridDim.x) {
    const int n = len[s];
    long long* kk = key + off[s];
    double* vv = val + off[s];
    for (int t = threadIdx.x; t < P; t += kPairThreads) {
      sk[t] = t < n ? kk[t] : LLONG_MAX;
      sv[t] = t < n ? vv[t] : 0.0;
    }
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int t = threadIdx.x; t < P; t += kPairThreads) {
          const int u = t ^ j;
          if (u > t) {
            const long long x = sk[t], y = sk[u];
            const bool up = (t & k) == 0;
            if ((x > y) == up) {
              sk[t] = y; sk[u] = x;
              const double w = sv[t]; sv[t] = sv[u]; sv[u] = w;
            }
          }
        }
        __syncthreads();
      }
    for (int t = threadIdx.x; t < n; t += kPairThreads) {
      kk[t] = sk[t];
      vv[t] = sv[t];
    }
    __syncthreads();
  }
}

// one thread per fine row: sum the runs of equal columns in order, divide by
// the node's cell count, keep (column, value) compacted at the row's start
__global__ void k_tr_combine(int nrows, const long long* __restrict__ tp, const int* __restrict__ cnt,
                             const int* __restrict__ mult, long long* __restrict__ key,
                             double* __restrict__ val, int* __restrict__ ucnt) {
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < nrows;
       r += (long)gridDim.x * blockDim.x) {
    long long* kk = key + tp[r];
    double* vv = val + tp[r];
    const int n = cnt[r];
    const double m = (double)mult[r];
    int u = 0;
    for (int q = 0; q < n;) {
      const long long col = kk[q] >> 32;
      double s = 0.0;
      while (q < n && (kk[q] >> 32) == col) s += vv[q++];
      kk[u] = col;
      vv[u] = s / m;
      ++u;
    }
    ucnt[r] = u;
  }
}

__global__ void k_tr_copy_p(int nrows, const long long* __restrict__ tp, const long long* __restrict__ key,
                            const double* __restrict__ val, const int* __restrict__ rp,
                            int* __restrict__ col, double* __restrict__ pval,
                            float* __restrict__ pval32, int* __restrict__ rcnt) {
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < nrows;
       r += (long)gridDim.x * blockDim.x) {
    const long long* kk = key + tp[r];
    const double* vv = val + tp[r];
    const int b = rp[r], e = rp[r + 1];
    for (int q = b; q < e; ++q) {
      const int c = (int)kk[q - b];
      col[q] = c;
      pval[q] = vv[q - b];
      pval32[q] = (float)vv[q - b];
      atomicAdd(rcnt + c, 1);
    }
  }
}

__global__ void k_tr_fill_r(int nrows, const int* __restrict__ prp, const int* __restrict__ pcol,
                            const double* __restrict__ pval, const int* __restrict__ rrp,
                            int* __restrict__ rcur, long long* __restrict__ rkey,
                            double* __restrict__ rval) {
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < nrows;
       r += (long)gridDim.x * blockDim.x)
    for (int q = prp[r]; q < prp[r + 1]; ++q) {
      const int c = pcol[q];
      const int at = rrp[c] + atomicAdd(rcur + c, 1);
      rkey[at] = r;
      rval[at] = pval[q];
    }
}

__global__ void k_tr_copy_r(long n, const long long* __restrict__ rkey,
                            const double* __restrict__ rval, int* __restrict__ col,
                            double* __restrict__ val, float* __restrict__ val32) {
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n;
       q += (long)gridDim.x * blockDim.x) {
    col[q] = (int)rkey[q];
    val[q] = rval[q];
    val32[q] = (float)rval[q];
  }
}

__global__ void k_lengths(int n, const int* __restrict__ rp, int* __restrict__ len,
                          long long* __restrict__ off) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    len[i] = rp[i + 1] - rp[i];
    off[i] = rp[i];
  }
}

int seg_sort(cdg_context* ctx, int nseg, int maxlen, const long long* off, const int* len,
             long long* key, double* val) {
  int P = kPairThreads;
  while (P < maxlen) P <<= 1;
  if (P > 4096) {
    set_error("transfer row of %d entries beyond the shared-memory sort", maxlen);
    return CDG_ERR_LIMIT;
  }
  const size_t smem = (size_t)P * (sizeof(long long) + sizeof(double));
  if (smem > 48 * 1024)
    CDG_CUDA(cudaFuncSetAttribute(k_seg_sort_pairs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
  const int grid = (int)std::max<long>(1, std::min<long>(nseg, (long)ctx->num_sms * 16));
  CDG_LAUNCH(ctx, k_seg_sort_pairs, grid, kPairThreads, smem, nseg, P, off, len, key, val);
  return CDG_OK;
}

int max_of(cdg_context* ctx, int n, const int* v, int* mx_dev, int* out) {
  CDG_CUDA(cudaMemsetAsync(mx_dev, 0, sizeof(int), ctx->stream));
  CDG_LAUNCH(ctx, k_row_max, fill_grid(ctx, n), 256, 0, n, v, mx_dev);
  CDG_CUDA(cudaMemcpyAsync(out, mx_dev, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  return CDG_OK;
}

}  // namespace

int device_transfer(cdg_context* ctx, const Mesh& fm, const Space& fs, const Mesh& cm,
                    const Space& cs, const int* parent_host, const int* fgdof_dev,
                    const int* cgdof_dev, DevLevel& F) {
  const int nl = fs.nloc, nf = fs.ndof, nc = cs.ndof;
  const long n = (long)fm.ncells * nl;
  cudaStream_t st = ctx->stream;
  TransferArgs a{};
  a.shape = fm.shape;
  a.dim = fm.dim;
  a.p = fs.order;
  a.nl = nl;
  a.nv = fm.nv;
  for (int k = 0; k < nl; ++k) local_dof_ref_shape(fm.shape, fs.order, k, a.ref[k]);
  DBuf<double> fv, cv, tval, rval;
  DBuf<int> parent, cnt, mult, cursor, ucnt, mx, rcnt, rcur, rlen;
  DBuf<long long> tp, key, rkey, roff;
  CDG_TRY(fv.alloc(fm.verts.size()));
  CDG_TRY(cv.alloc(cm.verts.size()));
  CDG_TRY(parent.alloc(fm.ncells));
  CDG_TRY(cnt.alloc((size_t)nf + 1));
  CDG_TRY(mult.alloc((size_t)nf + 1));
  CDG_TRY(cursor.alloc((size_t)nf + 1));
  CDG_TRY(ucnt.alloc((size_t)nf + 1));
  CDG_TRY(tp.alloc((size_t)nf + 1));
  CDG_TRY(mx.alloc(1));
  CDG_CUDA(cudaMemcpyAsync(fv.p, fm.verts.data(), fm.verts.size() * sizeof(double),
                           cudaMemcpyHostToDevice, st));
  CDG_CUDA(cudaMemcpyAsync(cv.p, cm.verts.data(), cm.verts.size() * sizeof(double),
                           cudaMemcpyHostToDevice, st));
  CDG_CUDA(cudaMemcpyAsync(parent.p, parent_host, (size_t)fm.ncells * sizeof(int),
                           cudaMemcpyHostToDevice, st));
  CDG_CUDA(cudaMemsetAsync(cnt.p, 0, ((size_t)nf + 1) * sizeof(int), st));
  CDG_CUDA(cudaMemsetAsync(mult.p, 0, ((size_t)nf + 1) * sizeof(int), st));
  CDG_CUDA(cudaMemsetAsync(cursor.p, 0, ((size_t)nf + 1) * sizeof(int), st));
  CDG_CUDA(cudaMemsetAsync(ucnt.p, 0, ((size_t)nf + 1) * sizeof(int), st));
  CDG_LAUNCH(ctx, k_tr_count, fill_grid(ctx, n), 256, 0, n, a, fv.p, cv.p, parent.p, fgdof_dev,
             cnt.p, mult.p);
  ScanScratch sc;
  long long tot[1];
  CDG_TRY((device_scan<1>(ctx, sc, (long)nf + 1, CountOf{cnt.p}, WriteOffset64{tp.p}, tot)));
  CDG_TRY(key.alloc((size_t)tot[0]));
  CDG_TRY(tval.alloc((size_t)tot[0]));
  CDG_LAUNCH(ctx, k_tr_fill, fill_grid(ctx, n), 256, 0, n, a, fv.p, cv.p, parent.p, fgdof_dev,
             cgdof_dev, tp.p, cursor.p, key.p, tval.p);
  int maxlen = 0;
  CDG_TRY(max_of(ctx, nf, cnt.p, mx.p, &maxlen));
  CDG_TRY(seg_sort(ctx, nf, maxlen, tp.p, cnt.p, key.p, tval.p));
  CDG_LAUNCH(ctx, k_tr_combine, fill_grid(ctx, nf), 256, 0, nf, tp.p, cnt.p, mult.p, key.p,
             tval.p, ucnt.p);
  // P
  long long pnnz[1];
  int *prp = nullptr, *pcol = nullptr, *rrp = nullptr, *rcol = nullptr;
  double *pval = nullptr, *rv = nullptr;
  float *pval32 = nullptr, *rv32 = nullptr;
  auto release = [&]() {
    for (void* q : {(void*)prp, (void*)pcol, (void*)rrp, (void*)rcol, (void*)pval, (void*)rv,
                    (void*)pval32, (void*)rv32})
      if (q) cudaFree(q);
  };
  int rc = CDG_OK;
  do {
    if ((rc = dalloc_raw(&prp, (size_t)nf + 1)) != CDG_OK) break;
    rc = device_scan<1>(ctx, sc, (long)nf + 1, CountOf{ucnt.p}, WriteOffset32{prp}, pnnz);
    if (rc != CDG_OK) break;
    if ((rc = dalloc_raw(&pcol, (size_t)pnnz[0])) != CDG_OK) break;
    if ((rc = dalloc_raw(&pval, (size_t)pnnz[0])) != CDG_OK) break;
    if ((rc = dalloc_raw(&pval32, (size_t)pnnz[0])) != CDG_OK) break;
    if ((rc = rcnt.alloc((size_t)nc + 1)) != CDG_OK) break;
    if ((rc = rcur.alloc((size_t)nc + 1)) != CDG_OK) break;
    cudaMemsetAsync(rcnt.p, 0, ((size_t)nc + 1) * sizeof(int), st);
    cudaMemsetAsync(rcur.p, 0, ((size_t)nc + 1) * sizeof(int), st);
    CDG_LAUNCH(ctx, k_tr_copy_p, fill_grid(ctx, nf), 256, 0, nf, tp.p, key.p, tval.p, prp, pcol,
               pval, pval32, rcnt.p);
    // R = P^T, rows sorted by fine index
    if ((rc = dalloc_raw(&rrp, (size_t)nc + 1)) != CDG_OK) break;
    long long rnnz[1];
    rc = device_scan<1>(ctx, sc, (long)nc + 1, CountOf{rcnt.p}, WriteOffset32{rrp}, rnnz);
    if (rc != CDG_OK) break;
    if ((rc = rkey.alloc((size_t)rnnz[0])) != CDG_OK) break;
    if ((rc = rval.alloc((size_t)rnnz[0])) != CDG_OK) break;
    CDG_LAUNCH(ctx, k_tr_fill_r, fill_grid(ctx, nf), 256, 0, nf, prp, pcol, pval, rrp, rcur.p,
               rkey.p, rval.p);
    if ((rc = rlen.alloc((size_t)nc + 1)) != CDG_OK) break;
    if ((rc = roff.alloc((size_t)nc + 1)) != CDG_OK) break;
    CDG_LAUNCH(ctx, k_lengths, fill_grid(ctx, nc), 256, 0, nc, rrp, rlen.p, roff.p);
    int rmax = 0;
    if ((rc = max_of(ctx, nc, rlen.p, mx.p, &rmax)) != CDG_OK) break;
    if ((rc = seg_sort(ctx, nc, rmax, roff.p, rlen.p, rkey.p, rval.p)) != CDG_OK) break;
    if ((rc = dalloc_raw(&rcol, (size_t)rnnz[0])) != CDG_OK) break;
    if ((rc = dalloc_raw(&rv, (size_t)rnnz[0])) != CDG_OK) break;
    if ((rc = dalloc_raw(&rv32, (size_t)rnnz[0])) != CDG_OK) break;
    CDG_LAUNCH(ctx, k_tr_copy_r, fill_grid(ctx, rnnz[0]), 256, 0, rnnz[0], rkey.p, rval.p, rcol,
               rv, rv32);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      set_error("transfer build: %s", cudaGetErrorString(e));
      rc = CDG_ERR_CUDA;
      break;
    }
    if ((rc = check_device_error(ctx)) != CDG_OK) break;
    F.P_rp = prp; F.P_col = pcol; F.P_val = pval; F.P_val32 = pval32;
    F.R_rp = rrp; F.R_col = rcol; F.R_val = rv; F.R_val32 = rv32;
    F.P_nnz = (int)pnnz[0];
    F.R_nnz = (int)rnnz[0];
    return CDG_OK;
  } while (false);
  cudaStreamSynchronize(st);
  release();
  return rc;
}


// ---------------------------------------------------------------------------
// sliced ELLPACK layout of the FP64 operator, built on the device with the
// host builder's rules: rows stable-sorted by length (descending) inside
// windows of kSellWindow rows, slices of 32/G rows, entry k of slice row i at
// off[s] + 32 (k / G) + G i + k mod G, padding = own row with value 0,
// non-active rows = identity (1 at the first slot)
// ---------------------------------------------------------------------------
namespace {

__global__ void __launch_bounds__(kSellWindow)
k_sell_order(int n, int na, const int* __restrict__ rp, int* __restrict__ order) {
  __shared__ long long key[kSellWindow];
  const int w0 = blockIdx.x * kSellWindow, t = threadIdx.x, r = w0 + t;
  long long kv = LLONG_MAX;
  if (r < n) {
    const int len = r < na ? rp[r + 1] - rp[r] : 1;
    kv = ((long long)(INT_MAX - len) << 32) | (long long)(unsigned)t;   // ties: row order
  }
  key[t] = kv;
  __syncthreads();
  for (int k = 2; k <= kSellWindow; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      const int u = t ^ j;
      if (u > t) {
        const long long x = key[t], y = key[u];
        const bool up = (t & k) == 0;
        if ((x > y) == up) {
          key[t] = y;
          key[u] = x;
        }
      }
      __syncthreads();
    }
  if (w0 + t < n) order[w0 + t] = w0 + (int)(key[t] & 0xffffffffLL);
}

__global__ void k_sell_steps(int nslices, int R, int G, int n, int na, const int* __restrict__ rp,
                             const int* __restrict__ order, int* __restrict__ srow,
                             int* __restrict__ width) {
  for (long s = blockIdx.x * (long)blockDim.x + threadIdx.x; s < nslices;
       s += (long)gridDim.x * blockDim.x) {
    int steps = 0;
    for (int i = 0; i < R; ++i) {
      const long idx = s * R + i;
      int r = -1;
      if (idx < n) {
        r = order[idx];
        const int len = r < na ? rp[r + 1] - rp[r] : 1;
        steps = max(steps, (len + G - 1) / G);
      }
      srow[idx] = r;
    }
    width[s] = 32 * steps;
  }
}

__global__ void k_sell_fill(int nslices, int R, int G, int na, const int* __restrict__ rp,
                            const int* __restrict__ col, const long long* __restrict__ off,
                            const int* __restrict__ srow, int* __restrict__ scol,
                            int* __restrict__ pos, double* __restrict__ sval) {
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < (long)nslices * R;
       t += (long)gridDim.x * blockDim.x) {
    const long s = t / R;
    const int i = (int)(t - s * R);
    const int r = srow[t];
    if (r < 0) continue;                          // padding row: column 0, value 0
    const long long o = off[s];
    const int slots = (int)((off[s + 1] - o) / 32) * G;
    const int m = r < na ? rp[r + 1] - rp[r] : 0;
    const int b = r < na ? rp[r] : 0;
    for (int k = 0; k < slots; ++k) {
      const long long q = o + 32LL * (k / G) + G * i + k % G;
      if (k < m) {
        scol[q] = col[b + k];
        pos[b + k] = (int)q;
      } else {
        scol[q] = r;                              // padding: own row, value 0
      }
    }
    if (r >= na) sval[o + G * i] = 1.0;           // identity row
  }
}

struct SliceWidth {
  const int* w;
  __device__ void operator()(long i, long long (&v)[1]) const { v[0] = w[i]; }
};

}  // namespace

int device_sell(cdg_context* ctx, DevLevel& L, int G) {
  const int n = L.ndof, na = L.nactive;
  const int R = 32 / G;
  const int nslices = (n + R - 1) / R;
  cudaStream_t st = ctx->stream;
  DBuf<int> order, width;
  CDG_TRY(order.alloc(n));
  CDG_TRY(width.alloc((size_t)nslices + 1));
  int *srow = nullptr, *scol = nullptr, *pos = nullptr;
  long long* off = nullptr;
  double* sval = nullptr;
  auto release = [&]() {
    for (void* q : {(void*)srow, (void*)scol, (void*)pos, (void*)off, (void*)sval})
      if (q) cudaFree(q);
  };
  int rc = CDG_OK;
  do {
    if ((rc = dalloc_raw(&srow, (size_t)nslices * R)) != CDG_OK) break;
    if ((rc = dalloc_raw(&off, (size_t)nslices + 1)) != CDG_OK) break;
    CDG_LAUNCH(ctx, k_sell_order, (n + kSellWindow - 1) / kSellWindow, kSellWindow, 0, n, na,
               L.row_ptr, order.p);
    cudaMemsetAsync(width.p + nslices, 0, sizeof(int), st);
    CDG_LAUNCH(ctx, k_sell_steps, fill_grid(ctx, nslices), 256, 0, nslices, R, G, n, na,
               L.row_ptr, order.p, srow, width.p);
    ScanScratch sc;
    long long total[1];
    rc = device_scan<1>(ctx, sc, (long)nslices + 1, SliceWidth{width.p}, WriteOffset64{off}, total);
    if (rc != CDG_OK) break;
    if (total[0] >= (1LL << 31)) {
      set_error("sliced layout of %lld slots beyond 32-bit positions", total[0]);
      rc = CDG_ERR_LIMIT;
      break;
    }
    if ((rc = dalloc_raw(&scol, (size_t)total[0])) != CDG_OK) break;
    if ((rc = dalloc_raw(&sval, (size_t)total[0])) != CDG_OK) break;
    if ((rc = dalloc_raw(&pos, (size_t)L.nnz)) != CDG_OK) break;
    cudaMemsetAsync(scol, 0, (size_t)total[0] * sizeof(int), st);
    cudaMemsetAsync(sval, 0, (size_t)total[0] * sizeof(double), st);
    cudaMemsetAsync(pos, 0xff, (size_t)L.nnz * sizeof(int), st);   // -1: no slot
    CDG_LAUNCH(ctx, k_sell_fill, fill_grid(ctx, (long)nslices * R), 256, 0, nslices, R, G, na,
               L.row_ptr, L.col, off, srow, scol, pos, sval);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      set_error("sliced layout: %s", cudaGetErrorString(e));
      rc = CDG_ERR_CUDA;
      break;
    }
    L.sell_off = off;
    L.sell_row = srow;
    L.sell_col = scol;
    L.sell_val = sval;
    L.sell_pos = pos;
    L.sell_nslices = nslices;
    L.sell_lanes = G;
    L.sell_total = total[0];
    return CDG_OK;
  } while (false);
  cudaStreamSynchronize(st);
  release();
  return rc;
}

}  // namespace cdg
