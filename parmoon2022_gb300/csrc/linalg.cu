// linalg.cu -- GB300 kernels and host drivers of the CD solve: CSR SpMV with
// identity on non-active rows, damped-Jacobi smoothing, grid transfers,
// multigrid cycle, dense coarse inverse, Arnoldi reductions and the FGMRES
// loop with all Krylov scalars resident on the device.
//
// Reference path (ParMooN2022): Solver::solve (src/Solver/Solver.C:601-696)
// -> Iteration_gmres::flexible_gmres (src/Solver/Iteration_gmres.C:430-620,
// Utilities_gmres.C:60-108, IterativeMethod.h:83-163) with preconditioner
// Iteration_jacobi (src/Solver/Iteration_jacobi.C:168-182) or
// Iteration_multigrid -> Multigrid::cycle (src/Multigrid/Multigrid.C:157-410,
// CycleControl.C:15-111, MultigridLevel.C:118-151, JacobiSmoother.C:21-29,
// GridTransfer.C:29-410, DirectSmoother.C:25-42);
// BlockFEMatrix::apply_scaled_add (src/Matrix/BlockFEMatrix.C:969-1095).
#include <cooperative_groups.h>

#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "common.cuh"
#include "solver_dev.cuh"

namespace cgrp = cooperative_groups;

namespace cdg {

// ---------------------------------------------------------------------------
// CSR row reductions: TPR threads per row, each lane issues UNR independent
// (col, val) loads before the dependent x gathers, so a warp keeps
// TPR*UNR*(4+sizeof(T)) bytes of matrix data in flight per pass
// ---------------------------------------------------------------------------
template <typename T, int TPR, int UNR>
__device__ __forceinline__ T csr_row_partial(const int* __restrict__ rp, const int* __restrict__ col,
                                             const T* __restrict__ val, const T* __restrict__ x,
                                             int row, int sub) {
  T s = 0;
  const int b = __ldg(rp + row), e = __ldg(rp + row + 1);
  for (int k0 = b + sub; k0 < e; k0 += TPR * UNR) {
    int c[UNR];
    T v[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      const int k = k0 + u * TPR;
      c[u] = k < e ? __ldcs(col + k) : -1;
      v[u] = k < e ? __ldcs(val + k) : (T)0;
    }
    // padding slots issue neither a gather nor a multiply-add
#pragma unroll
    for (int u = 0; u < UNR; ++u)
      if (c[u] >= 0) s = fma(v[u], __ldg(x + c[u]), s);
  }
  return s;
}

// sum over the TPR lanes of a row group; every lane of the warp must call it
template <typename T, int TPR>
__device__ __forceinline__ T group_sum(T s) {
#pragma unroll
  for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, TPR);
  return s;
}

// SpMV family; non-active rows act as identity rows
//   MODE 0: y = A x
//   MODE 1: y = b - A x                         (calculate_defect)
//   MODE 2: y = x + w D^-1 (b - A x)            (JacobiSmoother::smooth)
//   MODE 3: MODE 2, and y also in FP64 into z (block z at vector *di when di
//           is given, and zcur): the last smoothing step of a mixed-precision
//           cycle hands its result to the FP64 Krylov method directly
template <typename T, int TPR, int UNR, int MODE>
__global__ void __launch_bounds__(256)
k_spmv(int n, int nactive, const int* __restrict__ rp, const int* __restrict__ col,
       const T* __restrict__ val, const T* __restrict__ x, const T* __restrict__ b,
       const T* __restrict__ invd, T w, T* __restrict__ y, double* __restrict__ z = nullptr,
       const int* di = nullptr, double* __restrict__ zcur = nullptr) {
  pdl_enter();
  const long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int row = (int)(gt / TPR);
  const int sub = threadIdx.x % TPR;
  T s = 0;
  if (row < nactive) s = csr_row_partial<T, TPR, UNR>(rp, col, val, x, row, sub);
  s = group_sum<T, TPR>(s);
  if (row >= n || sub != 0) return;
  const T xr = x[row];
  if (row >= nactive) s = xr;
  if (MODE == 0) y[row] = s;
  else if (MODE == 1) y[row] = b[row] - s;
  else {
    const T yr = xr + w * (invd[row] * (b[row] - s));
    y[row] = yr;
    if (MODE == 3) {
      const double zr = (double)yr;
      (di ? z + (size_t)(*di) * n : z)[row] = zr;
      if (zcur) zcur[row] = zr;
    }
  }
}

// ---------------------------------------------------------------------------
// FP32 smoothing / defect with the CSR stream staged through shared memory.
// Each warp owns a double buffer: lane 0 starts cp.async.bulk copies of the
// next chunk's (col, val) ranges into one buffer, completion counted on that
// buffer's mbarrier, while the warp reduces the current chunk's rows from the
// other buffer (TPR lanes per row, x gathered from L2/L1).  DRAM sees only
// bulk copies.  Opt-in (CDG_BULK_CHUNK): measured on GB300 at 59-105 us
// against 29.7 us for k_spmv on the 32^3 Q2 finest level, because each warp
// walks its chunks one after another and every chunk pays the row-pointer,
// gather and epilogue latencies in sequence, with 8-32 warps per SM where the
// register-streaming kernel keeps 64 independent warps.
// Copy ranges are rounded out to 16 bytes (4 entries): col and val32 carry 4
// entries of padding past nnz.  Every wait is bounded: on time-out the warp
// records kErrTimeout, waits (bounded) for its other copy, and stops.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes,
                                              unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
constexpr long kMbarSpin = 1L << 24;   // try_wait rounds before a wait counts as lost
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
  for (long i = 0; i < kMbarSpin; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

template <int WARPS, int TPR, int MODE>
__global__ void __launch_bounds__(WARPS * 32)
k_spmv_bulk(int n, int nactive, int nchunks, int stage, const int* __restrict__ crow,
            const int* __restrict__ rp, const int* __restrict__ col, const float* __restrict__ val,
            const float* __restrict__ x, const float* __restrict__ b,
            const float* __restrict__ invd, float w, float* __restrict__ y, int* err) {
  pdl_enter();
  extern __shared__ __align__(16) unsigned char bulk_smem[];
  __shared__ __align__(8) unsigned long long bars[WARPS][2];
  const int wp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane % TPR;
  // buffer st of this warp: columns at wbase + st * 8 * stage, values 4 * stage bytes later
  unsigned char* const wbase = bulk_smem + (size_t)wp * 16 * stage;
  auto scol = [&](int st) { return reinterpret_cast<int*>(wbase + (size_t)st * 8 * stage); };
  auto sval = [&](int st) {
    return reinterpret_cast<float*>(wbase + (size_t)st * 8 * stage + (size_t)stage * 4);
  };
  if (lane == 0) {
    mbar_init(&bars[wp][0], 1);
    mbar_init(&bars[wp][1], 1);
  }
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  __syncthreads();
  const int gw = blockIdx.x * WARPS + wp, nw = gridDim.x * WARPS;
  auto issue = [&](int c, int st) {
    const int e0 = __ldg(rp + __ldg(crow + c)), e1 = __ldg(rp + __ldg(crow + c + 1));
    const int a0 = e0 & ~3, a1 = (e1 + 3) & ~3;
    const unsigned bytes = (unsigned)(a1 - a0) * 4u;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&bars[wp][st], 2u * bytes);
    bulk_copy_g2s(scol(st), col + a0, bytes, &bars[wp][st]);
    bulk_copy_g2s(sval(st), val + a0, bytes, &bars[wp][st]);
  };
  unsigned phase0 = 0, phase1 = 0;
  int st = 0;
  if (gw < nchunks && lane == 0) issue(gw, 0);
  for (int c = gw; c < nchunks; c += nw, st ^= 1) {
    const bool next = c + nw < nchunks;
    if (next && lane == 0) issue(c + nw, st ^ 1);
    const unsigned ph = st ? phase1 : phase0;
    if (!mbar_wait_bounded(&bars[wp][st], ph)) {
      if (lane == 0) {
        atomicOr(err, kErrTimeout);
        if (next) mbar_wait_bounded(&bars[wp][st ^ 1], st ? phase0 : phase1);
      }
      return;
    }
    if (st) phase1 ^= 1; else phase0 ^= 1;
    const int r0 = __ldg(crow + c), r1 = __ldg(crow + c + 1);
    const int base = __ldg(rp + r0) & ~3;
    const int* sc = scol(st);
    const float* sv = sval(st);
    constexpr int RPP = 32 / TPR;   // rows per pass
    for (int q0 = r0; q0 < r1; q0 += RPP) {
      const int r = q0 + lane / TPR;
      float s = 0.f;
      if (r < r1) {
        const int kb = __ldg(rp + r) - base, ke = __ldg(rp + r + 1) - base;
        for (int k0 = kb + sub; k0 < ke; k0 += TPR * 8) {
          int cc[8];
          float vv[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int k = k0 + u * TPR;
            cc[u] = k < ke ? sc[k] : -1;
            vv[u] = k < ke ? sv[k] : 0.f;
          }
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (cc[u] >= 0) s = fmaf(vv[u], __ldg(x + cc[u]), s);
        }
      }
      s = group_sum<float, TPR>(s);
      if (r < r1 && sub == 0) {
        if (MODE == 1) y[r] = b[r] - s;
        else y[r] = x[r] + w * (invd[r] * (b[r] - s));
      }
    }
    __syncwarp();
  }
  // non-active rows act as identity rows
  for (long r = nactive + (long)gw * 32 + lane; r < n; r += (long)nw * 32) {
    const float xr = x[r];
    if (MODE == 1) y[r] = b[r] - xr;
    else y[r] = xr + w * (invd[r] * (b[r] - xr));
  }
}

template <int WARPS, int TPR, int MODE>
static int launch_bulk(cdg_context* ctx, const DevLevel& L, const float* val, const float* x,
                       const float* b, const float* invd, float w, float* y) {
  const int stage = L.bulk_chunk + 8;
  const size_t smem = (size_t)WARPS * 2 * 2 * stage * sizeof(float);
  static thread_local int configured_device = -1;
  if (configured_device != ctx->device) {
    CDG_CUDA(cudaFuncSetAttribute(k_spmv_bulk<WARPS, TPR, MODE>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured_device = ctx->device;
  }
  CDG_LAUNCH_PDL(ctx, (k_spmv_bulk<WARPS, TPR, MODE>), ctx->num_sms, WARPS * 32, smem, L.ndof,
             L.nactive, L.bulk_nchunks, stage, L.bulk_row, L.row_ptr, L.col, val, x, b, invd, w, y,
             ctx->d_err);
  return CDG_OK;
}

// warps per block so that the double buffers fill ~132 KB of shared memory
template <int TPR, int MODE>
static int spmv_bulk(cdg_context* ctx, const DevLevel& L, const float* val, const float* x,
                     const float* b, const float* invd, float w, float* y) {
  switch (L.bulk_chunk) {
    case 256: return launch_bulk<32, TPR, MODE>(ctx, L, val, x, b, invd, w, y);
    case 512: return launch_bulk<16, TPR, MODE>(ctx, L, val, x, b, invd, w, y);
    default: return launch_bulk<8, TPR, MODE>(ctx, L, val, x, b, invd, w, y);
  }
}

template <int MODE>
static int spmv_bulk_any(cdg_context* ctx, const DevLevel& L, const float* val, const float* x,
                         const float* b, const float* invd, float w, float* y) {
  switch (L.rows_per_warp_hint) {
    case 2: return spmv_bulk<2, MODE>(ctx, L, val, x, b, invd, w, y);
    case 4: return spmv_bulk<4, MODE>(ctx, L, val, x, b, invd, w, y);
    case 8: return spmv_bulk<8, MODE>(ctx, L, val, x, b, invd, w, y);
    default: return spmv_bulk<16, MODE>(ctx, L, val, x, b, invd, w, y);
  }
}

// lanes per row chosen from the average row length so that 8 * TPR covers a
// typical row in one pass (Q2 hexahedra: 62 entries -> 8 lanes, 4 rows/warp)
template <typename T, int MODE>
static int spmv_t(cdg_context* ctx, const DevLevel& L, const T* val, const T* x, const T* b,
                  const T* invd, T w, T* y) {
  const int tpr = std::is_same<T, float>::value && L.tpr32 ? L.tpr32 : L.rows_per_warp_hint;
  long threads = (long)L.ndof * tpr;
  int grid = (int)((threads + 255) / 256);
  switch (tpr) {
    case 2: CDG_LAUNCH_PDL(ctx, (k_spmv<T, 2, 8, MODE>), grid, 256, 0, L.ndof, L.nactive, L.row_ptr, L.col, val, x, b, invd, w, y,
                             (double*)nullptr, (const int*)nullptr, (double*)nullptr); break;
    case 4: CDG_LAUNCH_PDL(ctx, (k_spmv<T, 4, 8, MODE>), grid, 256, 0, L.ndof, L.nactive, L.row_ptr, L.col, val, x, b, invd, w, y,
                             (double*)nullptr, (const int*)nullptr, (double*)nullptr); break;
    case 8: CDG_LAUNCH_PDL(ctx, (k_spmv<T, 8, 8, MODE>), grid, 256, 0, L.ndof, L.nactive, L.row_ptr, L.col, val, x, b, invd, w, y,
                             (double*)nullptr, (const int*)nullptr, (double*)nullptr); break;
    default: CDG_LAUNCH_PDL(ctx, (k_spmv<T, 16, 8, MODE>), grid, 256, 0, L.ndof, L.nactive, L.row_ptr, L.col, val, x, b, invd, w, y,
                             (double*)nullptr, (const int*)nullptr, (double*)nullptr); break;
  }
  return CDG_OK;
}

// Sliced ELLPACK SpMV (same MODEs as k_spmv): one warp per slice of 32/G
// rows, G lanes per row; the slice's step count is warp-uniform, so every
// multiply-add issues for 32 useful lanes (padding: zero values) and every
// load of a step is one coalesced 32-wide access.  UNR steps are loaded
// before their gathers.  Non-active rows are identity rows of the layout.
template <typename T, int G, int UNR, int MODE>
__global__ void __launch_bounds__(256)
k_sell(int nslices, const long long* __restrict__ off, const int* __restrict__ srow,
       const int* __restrict__ scol, const T* __restrict__ sval, const T* __restrict__ x,
       const T* __restrict__ b, const T* __restrict__ invd, T w, T* __restrict__ y) {
  pdl_enter();
  const int slice = (int)((blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (slice >= nslices) return;              // warp-uniform
  const long long o = __ldg(off + slice);
  const int width = (int)((__ldg(off + slice + 1) - o) >> 5);
  const int* __restrict__ cp = scol + o + lane;
  const T* __restrict__ vp = sval + o + lane;
  T s = 0;
  for (int k0 = 0; k0 < width; k0 += UNR) {
    int c[UNR];
    T v[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      const bool in = k0 + u < width;       // warp-uniform
      c[u] = in ? __ldcs(cp + (long)(k0 + u) * 32) : 0;
      v[u] = in ? __ldcs(vp + (long)(k0 + u) * 32) : (T)0;
    }
#pragma unroll
    for (int u = 0; u < UNR; ++u)
      if (k0 + u < width) s = fma(v[u], __ldg(x + c[u]), s);
  }
  s = group_sum<T, G>(s);
  if (lane % G) return;
  const int row = __ldg(srow + (long)slice * (32 / G) + lane / G);
  if (row < 0) return;
  if (MODE == 0) y[row] = s;
  else if (MODE == 1) y[row] = b[row] - s;
  else y[row] = x[row] + w * (invd[row] * (b[row] - s));
}

// steps in flight per lane: 8 for long rows (Q2 hexahedra, ~31 steps of 2 lanes),
// 4 for short ones (P2 tetrahedra, ~14): measured 49.3 / 68.4 us against
// 50.7 / 74.9 us with the other depth
template <int G, int MODE>
static int sell64_g(cdg_context* ctx, const DevLevel& L, const double* x, const double* b,
                    double* y) {
  const int grid = (int)(((long)L.sell_nslices * 32 + 255) / 256);
  const double steps = (double)L.nnz / L.ndof / G;
  if (steps >= 24)
    CDG_LAUNCH_PDL(ctx, (k_sell<double, G, 8, MODE>), grid, 256, 0, L.sell_nslices, L.sell_off,
               L.sell_row, L.sell_col, L.sell_val, x, b, (const double*)nullptr, 0.0, y);
  else
    CDG_LAUNCH_PDL(ctx, (k_sell<double, G, 4, MODE>), grid, 256, 0, L.sell_nslices, L.sell_off,
               L.sell_row, L.sell_col, L.sell_val, x, b, (const double*)nullptr, 0.0, y);
  return CDG_OK;
}

template <int MODE>
static int sell64(cdg_context* ctx, const DevLevel& L, const double* x, const double* b,
                  double* y) {
  switch (L.sell_lanes) {
    case 1: return sell64_g<1, MODE>(ctx, L, x, b, y);
    case 2: return sell64_g<2, MODE>(ctx, L, x, b, y);
    case 4: return sell64_g<4, MODE>(ctx, L, x, b, y);
    case 8: return sell64_g<8, MODE>(ctx, L, x, b, y);
    default: return sell64_g<16, MODE>(ctx, L, x, b, y);
  }
}

// the FP64 operator: FP64 issue rate bounds it on GB300.  With the sliced
// ELLPACK copy every FP64 multiply-add is useful; otherwise CSR rows use 4
// lanes x 16-deep unrolling (2 reduction levels instead of 3)
int spmv_apply64(cdg_context* ctx, const DevLevel& L, const double* x, double* y) {
  if (L.sell_nslices) return sell64<0>(ctx, L, x, nullptr, y);
  if (L.rows_per_warp_hint == 8) {
    int grid = (int)(((long)L.ndof * 4 + 255) / 256);
    CDG_LAUNCH_PDL(ctx, (k_spmv<double, 4, 16, 0>), grid, 256, 0, L.ndof, L.nactive, L.row_ptr,
               L.col, L.val64, x, (const double*)nullptr, (const double*)nullptr, 0.0, y,
                   (double*)nullptr, (const int*)nullptr, (double*)nullptr);
    return CDG_OK;
  }
  return spmv_t<double, 0>(ctx, L, L.val64, x, nullptr, nullptr, 0.0, y);
}
int residual64(cdg_context* ctx, const DevLevel& L, const double* b, const double* x,
               double* r) {
  if (L.sell_nslices) return sell64<1>(ctx, L, x, b, r);
  return spmv_t<double, 1>(ctx, L, L.val64, x, b, nullptr, 0.0, r);
}

// ---------------------------------------------------------------------------
// deterministic reductions: per-block partial sums, the last block to finish
// sums the partials in block order and writes the result to device memory
// ---------------------------------------------------------------------------
template <int NT>
__device__ double block_sum(double v) {
  __shared__ double sh[NT / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = (l < NT / 32) ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
  }
  return r;  // valid in thread 0
}

// sum of p[start], p[start + stride], ... below n in that order, read from L2
// (the block partials other blocks published before their __threadfence and
// the counter update): the loads of eight terms are issued together, the
// additions stay in index order
__device__ __forceinline__ double sum_partials(const double* p, int start, int stride, int n) {
  double v = 0.0;
  int q = start;
  for (; q + 7 * stride < n; q += 8 * stride) {
    double t[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) t[u] = __ldcg(p + q + u * stride);
#pragma unroll
    for (int u = 0; u < 8; ++u) v += t[u];
  }
  for (; q < n; q += stride) v += __ldcg(p + q);
  return v;
}

template <int NT>
__device__ void finalize_sum(double blocksum, double* partials, unsigned* cnt, double* out,
                             bool take_sqrt) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = blocksum;
    __threadfence();
    unsigned t = atomicAdd(cnt, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double v = sum_partials(partials, threadIdx.x, NT, (int)gridDim.x);
  v = block_sum<NT>(v);
  if (threadIdx.x == 0) {
    *out = take_sqrt ? sqrt(v) : v;
    *cnt = 0u;
  }
}

// out = dot(a, b) (MODE 0) or ||a|| (MODE 1)
template <int MODE>
__global__ void __launch_bounds__(256)
k_dot(int n, const double* __restrict__ a, const double* __restrict__ b, double* partials,
      unsigned* cnt, double* out) {
  pdl_enter();
  double s = 0.0;
  for (long i = blockIdx.x * 256L + threadIdx.x; i < n; i += (long)gridDim.x * 256)
    s += MODE == 0 ? a[i] * b[i] : a[i] * a[i];
  s = block_sum<256>(s);
  finalize_sum<256>(s, partials, cnt, out, MODE == 1);
}

// modified Gram-Schmidt step k of the Arnoldi process, fused with the next
// inner product: w -= H(k,i) v_k; out = (w, v_{k+1}) or ||w|| (last step)
__global__ void __launch_bounds__(256)
k_mgs(int n, double* __restrict__ w, const double* __restrict__ vk, const double* hk,
      const double* __restrict__ vnext, double* partials, unsigned* cnt, double* out) {
  pdl_enter();
  const double h = -(*hk);
  double s = 0.0;
  for (long i = blockIdx.x * 256L + threadIdx.x; i < n; i += (long)gridDim.x * 256) {
    double wi = w[i] + h * vk[i];
    w[i] = wi;
    s += vnext ? wi * vnext[i] : wi * wi;
  }
  s = block_sum<256>(s);
  finalize_sum<256>(s, partials, cnt, out, vnext == nullptr);
}

// classical Gram-Schmidt (Iteration_gmres.C:515-527, the branch that queues
// all inner products before the updates): H(k0+j, i) = (w, v_{k0+j}) for
// j < cnt <= 32 in one pass over w and the basis
template <int NT>
__global__ void __launch_bounds__(NT)
k_multidot(int n, const double* __restrict__ w, const double* __restrict__ V, int k0, int cnt,
           double* partials, unsigned* counter, double* out, const int* di = nullptr,
           int hstride = 0) {
  pdl_enter();
  static_assert(NT == 256, "one reducing warp per inner product of a group of 8");
  if (di) {
    // graph-captured loop: inner products k0 .. min(k0 + 32, i + 1) of column i
    const int i = *di;
    cnt = min(32, i + 1 - k0);
    out += (size_t)i * hstride + k0;
    if (cnt <= 0) return;   // uniform over the grid
  }
  // FP64 issue is scarce on this GPU: per-thread partials are transposed
  // through shared memory so each inner product is reduced by one warp,
  // instead of every warp shuffling all eight
  __shared__ double tr[8][NT + 1];
  __shared__ double sh[32];
  __shared__ bool last;
  const int wp = threadIdx.x >> 5, l = threadIdx.x & 31;
  // eight inner products per pass (eight independent basis loads in flight);
  // the block's slice of w stays in L1 across passes
  for (int j0 = 0; j0 < cnt; j0 += 8) {
    double a[8];
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) a[jj] = 0.0;
    for (long t = blockIdx.x * (long)NT + threadIdx.x; t < n; t += (long)gridDim.x * NT) {
      const double wt = __ldg(w + t);
#pragma unroll
      for (int jj = 0; jj < 8; ++jj)
        if (j0 + jj < cnt) a[jj] = fma(wt, __ldcs(V + (size_t)(k0 + j0 + jj) * n + t), a[jj]);
    }
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) tr[jj][threadIdx.x] = a[jj];
    __syncthreads();
    if (j0 + wp < cnt) {
      double v = 0.0;
#pragma unroll
      for (int q = 0; q < NT / 32; ++q) v += tr[wp][q * 32 + l];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (l == 0) sh[j0 + wp] = v;
    }
    __syncthreads();
  }
  if (threadIdx.x < cnt) {
    partials[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = sh[threadIdx.x];
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  // one warp per inner product, lanes stride over the block partials
  for (int j = wp; j < cnt; j += NT / 32) {
    double v = sum_partials(partials + (size_t)j * gridDim.x, l, 32, (int)gridDim.x);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (l == 0) out[j] = v;
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// Givens rotations of Hessenberg column i (Utilities_gmres.C:60-88):
// givens_column_s in solver_dev.cuh, with s[i], s[i+1] in an array here
__device__ void givens_column(int i, double* col, double* cs, double* sn, double* s,
                              double* resid) {
  givens_column_s(i, col, cs, sn, s[i], s[i + 1], resid);
}

// w -= sum_k H(k,i) v_k (k in order), H(i+1,i) = ||w||, then the Givens
// step of column i in the block that finishes last
__global__ void __launch_bounds__(256)
k_cgs_update(int n, double* __restrict__ w, const double* __restrict__ V, int i,
             double* __restrict__ hcol, double* partials, unsigned* counter, double* cs,
             double* sn, double* gs, double* resid, double* norm_out, const int* di = nullptr,
             int hstride = 0) {
  pdl_enter();
  __shared__ double h[128];
  __shared__ bool last;
  if (di) {
    i = *di;
    hcol += (size_t)i * hstride;
  }
  for (int j = threadIdx.x; j <= i; j += 256) h[j] = -hcol[j];
  __syncthreads();
  double s = 0.0;
  for (long t = blockIdx.x * 256L + threadIdx.x; t < n; t += (long)gridDim.x * 256) {
    double wt = w[t];
    int j = 0;
    // eight independent basis loads in flight, additions kept in k order
    for (; j + 7 <= i; j += 8) {
      double a[8];
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) a[jj] = __ldcs(V + (size_t)(j + jj) * n + t);
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) wt = fma(h[j + jj], a[jj], wt);
    }
    for (; j <= i; ++j) wt = fma(h[j], __ldcs(V + (size_t)j * n + t), wt);
    w[t] = wt;
    s += wt * wt;
  }
  s = block_sum<256>(s);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = s;
    __threadfence();
    last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the rotation state in shared memory: the serial Givens chain then waits on
  // no global load (H(k,i) = -h[k] exactly)
  __shared__ double scs[128], ssn[128], ss[2];
  for (int j = threadIdx.x; j < i; j += 256) {
    scs[j] = cs[j];
    ssn[j] = sn[j];
  }
  if (threadIdx.x < 2) ss[threadIdx.x] = gs[i + threadIdx.x];
  for (int j = threadIdx.x; j <= i; j += 256) h[j] = -h[j];   // back to H(k,i)
  double v = sum_partials(partials, threadIdx.x, 256, (int)gridDim.x);
  v = block_sum<256>(v);   // synchronises the block
  if (threadIdx.x == 0) {
    const double nrm = sqrt(v);
    *norm_out = nrm;   // v_{i+1} = w / H(i+1,i) uses the value before rotation
    *counter = 0u;
    h[i + 1] = nrm;
    givens_column_s(i, h, scs, ssn, ss[0], ss[1], resid);   // on the staged copies
  }
  __syncthreads();
  for (int j = threadIdx.x; j <= i + 1; j += 256) hcol[j] = h[j];
  if (threadIdx.x == 0) {
    cs[i] = scs[i];
    sn[i] = ssn[i];
    gs[i] = ss[0];
    gs[i + 1] = ss[1];
  }
}

// One classical Gram-Schmidt step of FGMRES column i in one cooperative
// launch of one block per SM: the inner products (w, v_k), k <= i
// (Iteration_gmres.C:515-527), w -= sum_k H(k,i) v_k, H(i+1,i) = ||w||, the
// Givens step of column i and v_{i+1} = w / H(i+1,i) -- the work of
// k_multidot, k_cgs_update and k_scale_inv, with three grid-wide barriers in
// place of two launches and two single-block sums of every block's
// partials.  Inner product k is summed over the blocks' partials (in block
// order) by block k mod nb; the norm by every block, in block order, so all
// blocks hold the same value.  i from *di when di is given (graph-captured
// loop), else i_host.
__global__ void __launch_bounds__(256)
k_cgs_coop(int n, double* __restrict__ w, double* __restrict__ V, int i_host, const int* di,
           int hstride, double* __restrict__ H, double* __restrict__ part, int normoff,
           double* cs, double* sn, double* gs, double* resid, double* norm_out, int* err) {
  cgrp::grid_group grid = cgrp::this_grid();
  __shared__ double tr[8][257];
  __shared__ double h[128];
  __shared__ double scs[128], ssn[128], ss[2], nrm_s;
  const int i = di ? *di : i_host;
  const int nb = gridDim.x, wp = threadIdx.x >> 5, l = threadIdx.x & 31;
  const long stride = (long)nb * 256;
  double* hcol = H + (size_t)i * hstride;
  // (1) block partials of the inner products, eight per pass over w
  for (int j0 = 0; j0 <= i; j0 += 8) {
    double a[8];
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) a[jj] = 0.0;
    for (long t = blockIdx.x * 256L + threadIdx.x; t < n; t += stride) {
      const double wt = w[t];
#pragma unroll
      for (int jj = 0; jj < 8; ++jj)
        if (j0 + jj <= i) a[jj] = fma(wt, __ldcg(V + (size_t)(j0 + jj) * n + t), a[jj]);
    }
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) tr[jj][threadIdx.x] = a[jj];
    __syncthreads();
    if (j0 + wp <= i) {
      double v = 0.0;
#pragma unroll
      for (int q = 0; q < 8; ++q) v += tr[wp][q * 32 + l];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (l == 0) part[(size_t)(j0 + wp) * nb + blockIdx.x] = v;
    }
    __syncthreads();
  }
  grid.sync();
  // (2) H(k,i): inner product k over the blocks, by block k mod nb
  for (int k = blockIdx.x; k <= i; k += nb) {
    double v = 0.0;
    for (int b = threadIdx.x; b < nb; b += 256) v += __ldcg(part + (size_t)k * nb + b);
    v = block_sum<256>(v);
    if (threadIdx.x == 0) hcol[k] = v;
  }
  grid.sync();
  // (3) w -= sum_k H(k,i) v_k (k in order), block partial of ||w||^2
  for (int k = threadIdx.x; k <= i; k += 256) h[k] = -__ldcg(hcol + k);
  __syncthreads();
  double s = 0.0;
  for (long t = blockIdx.x * 256L + threadIdx.x; t < n; t += stride) {
    double wt = w[t];
    int j = 0;
    for (; j + 7 <= i; j += 8) {
      double a[8];
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) a[jj] = __ldcg(V + (size_t)(j + jj) * n + t);
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) wt = fma(h[j + jj], a[jj], wt);
    }
    for (; j <= i; ++j) wt = fma(h[j], __ldcg(V + (size_t)j * n + t), wt);
    w[t] = wt;
    s += wt * wt;
  }
  s = block_sum<256>(s);
  if (threadIdx.x == 0) part[normoff + blockIdx.x] = s;
  grid.sync();
  // (4) ||w|| (every block, block order), v_{i+1} = w / ||w||
  double v = 0.0;
  for (int b = threadIdx.x; b < nb; b += 256) v += __ldcg(part + normoff + b);
  v = block_sum<256>(v);
  if (threadIdx.x == 0) nrm_s = sqrt(v);
  __syncthreads();
  const double nrm = nrm_s;
  if (nrm == 0.0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, kErrBreakdown);
  } else {
    const double f = 1.0 / nrm;
    double* vn = V + (size_t)(i + 1) * n;
    for (long t = blockIdx.x * 256L + threadIdx.x; t < n; t += stride) vn[t] = w[t] * f;
  }
  if (blockIdx.x != 0) return;
  // the Givens step of column i (Utilities_gmres.C:60-88) on block 0's
  // copies of the rotations
  for (int j = threadIdx.x; j < i; j += 256) {
    scs[j] = cs[j];
    ssn[j] = sn[j];
  }
  if (threadIdx.x < 2) ss[threadIdx.x] = gs[i + threadIdx.x];
  for (int j = threadIdx.x; j <= i; j += 256) h[j] = -h[j];   // back to H(k,i)
  __syncthreads();
  if (threadIdx.x == 0) {
    *norm_out = nrm;
    h[i + 1] = nrm;
    givens_column_s(i, h, scs, ssn, ss[0], ss[1], resid);
  }
  __syncthreads();
  for (int j = threadIdx.x; j <= i + 1; j += 256) hcol[j] = h[j];
  if (threadIdx.x == 0) {
    cs[i] = scs[i];
    sn[i] = ssn[i];
    gs[i] = ss[0];
    gs[i + 1] = ss[1];
  }
}

static int red_grid(cdg_context* ctx, int n) {
  int g = (n + 255) / 256;
  int cap = ctx->num_sms * 4;
  if (g > cap) g = cap;
  if (g > kRedMaxBlocks) g = kRedMaxBlocks;
  return g < 1 ? 1 : g;
}

// the cooperative Gram-Schmidt step (k_cgs_coop), an option
// (CDG_CGS_COOP=1 in the environment) for large systems: cooperative
// launches supported, at least kCgsCoopRows rows (the served requests run on
// several streams at once), the partials fit the reduction buffer.  Off by
// default: measured on GB300 (32^3 Q2, 148 iterations per solve) the three
// grid-wide barriers cost more than the two launches and the two
// single-block sums they replace (mixed step 35.9 against 34.5 ms, FP64
// 72.9 against 70.9 ms).
constexpr int kCgsCoopRows = 100000;

static bool cgs_coop_on(cdg_context* ctx, int n, int m) {
  const char* e = std::getenv("CDG_CGS_COOP");
  if (!e || e[0] != '1') return false;
  int coop = 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device) != cudaSuccess)
    return false;
  return coop && n >= kCgsCoopRows &&
         (size_t)(m + 2) * ctx->num_sms <= (size_t)kRedSlots * kRedMaxBlocks;
}

static int cgs_coop(cdg_context* ctx, GmresState& g, int n, int m, int i_host, const int* di) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ctx->num_sms);
  cfg.blockDim = dim3(256);
  cfg.stream = ctx->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  const cudaError_t e =
      cudaLaunchKernelEx(&cfg, k_cgs_coop, n, g.w, g.V, i_host, di, m + 1, g.H, ctx->d_red,
                         (m + 1) * ctx->num_sms, g.cs, g.sn, g.s, g.scal + 0, g.scal + 2,
                         ctx->d_err);
  ctx->launches++;
  if (e != cudaSuccess) {
    set_error("launch k_cgs_coop: %s", cudaGetErrorString(e));
    return CDG_ERR_CUDA;
  }
  return CDG_OK;
}

int dot64(cdg_context* ctx, int n, const double* a, const double* b, double* out, int slot) {
  double* part = ctx->d_red + (size_t)slot * kRedMaxBlocks;
  unsigned* cnt = ctx->d_cnt + slot;
  if (b)
    CDG_LAUNCH_PDL(ctx, k_dot<0>, red_grid(ctx, n), 256, 0, n, a, b, part, cnt, out);
  else
    CDG_LAUNCH_PDL(ctx, k_dot<1>, red_grid(ctx, n), 256, 0, n, a, a, part, cnt, out);
  return CDG_OK;
}

// ---------------------------------------------------------------------------
// small vector kernels
// ---------------------------------------------------------------------------
// dst = src * (1 / *s); flags a zero scalar (FGMRES breakdown).  di != null:
// dst is the basis vector (*di + 1) of the block dst (graph-captured loop)
__global__ void k_scale_inv(int n, const double* __restrict__ src, const double* s,
                            double* __restrict__ dst, int* err, const int* di = nullptr) {
  pdl_enter();
  if (di) dst += (size_t)(*di + 1) * n;
  const double d = *s;
  if (d == 0.0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, kErrBreakdown);
    return;
  }
  const double f = 1.0 / d;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    dst[i] = src[i] * f;
}

// c = a .* b; di != null: a and c are vector *di of their blocks, c2 gets a copy
__global__ void k_mul(int n, const double* __restrict__ a, const double* __restrict__ b,
                      double* __restrict__ c, const int* di = nullptr, double* c2 = nullptr) {
  pdl_enter();
  if (di) {
    a += (size_t)(*di) * n;
    c += (size_t)(*di) * n;
  }
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double v = a[i] * b[i];
    c[i] = v;
    if (c2) c2[i] = v;
  }
}

// c = a (no preconditioner), same indexing as k_mul
__global__ void k_copy_idx(int n, const double* __restrict__ a, double* __restrict__ c,
                           const int* di, double* c2) {
  pdl_enter();
  if (di) {
    a += (size_t)(*di) * n;
    c += (size_t)(*di) * n;
  }
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    c[i] = a[i];
    if (c2) c2[i] = a[i];
  }
}

template <typename T>
__global__ void k_mg_init(int n, int nactive, const double* __restrict__ v, T* __restrict__ rhs,
                          T* __restrict__ sol, const int* di = nullptr) {
  pdl_enter();
  if (di) v += (size_t)(*di) * n;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    T r = (T)v[i];
    rhs[i] = r;
    sol[i] = i >= nactive ? r : (T)0;
  }
}

template <typename T>
__global__ void k_to_double(int n, const T* __restrict__ a, double* __restrict__ b,
                            const int* di = nullptr, double* b2 = nullptr) {
  pdl_enter();
  if (di) b += (size_t)(*di) * n;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double v = (double)a[i];
    b[i] = v;
    if (b2) b2[i] = v;
  }
}

// x_f[i] += damp * (P x_c)[i] for fine actives (update_solution_in_finer_grid)
// or x_f = P x_c for all rows (GridTransfer::Prolongate) when add == 0
template <typename T, int TPR>
__global__ void __launch_bounds__(256)
k_prolong(int nf, int nactive_f, const int* __restrict__ rp, const int* __restrict__ col,
          const T* __restrict__ val, const T* __restrict__ xc, T* __restrict__ xf, T damp,
          int add) {
  pdl_enter();
  const long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int i = (int)(gt / TPR), sub = threadIdx.x % TPR;
  T s = 0;
  if (i < nf) s = csr_row_partial<T, TPR, 4>(rp, col, val, xc, i, sub);
  s = group_sum<T, TPR>(s);
  if (i >= nf || sub != 0) return;
  if (!add) xf[i] = s;
  else if (i < nactive_f) xf[i] += damp * s;
}

// r_c = R d_f; coarse non-actives zeroed when mask (ResetNonActive)
template <typename T, int TPR>
__global__ void __launch_bounds__(256)
k_restrict(int nc, int nactive_c, const int* __restrict__ rp, const int* __restrict__ col,
           const T* __restrict__ val, const T* __restrict__ df, T* __restrict__ rc, int mask) {
  pdl_enter();
  const long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int j = (int)(gt / TPR), sub = threadIdx.x % TPR;
  T s = 0;
  if (j < nc && (!mask || j < nactive_c)) s = csr_row_partial<T, TPR, 8>(rp, col, val, df, j, sub);
  s = group_sum<T, TPR>(s);
  if (j >= nc || sub != 0) return;
  rc[j] = s;
}

// ---------------------------------------------------------------------------
// Grid transfers on nested uniform Q2 lattices.  The averaged child-local
// interpolation of GridTransfer::Prolongate (GridTransfer.C:29-410) on a
// refined uniform Q2 mesh is a tensor product of 1D interpolations: a fine
// point at coarse half-unit coordinate U takes coarse node U/2 (U even) or,
// inside coarse cell c = U div 4, the Q2 basis at the quarter points:
// (3/8, 3/4, -1/8) on nodes 2c, 2c+1, 2c+2 for U = 4c+1, reversed for 4c+3.
// The restriction is its transpose.  The kernels gather through the lattice
// maps instead of streaming P and R; lattice_transfer_setup checks every row
// of the level's P against these weights once.  An option (CDG_LAT_TRANSFER=1
// in the environment): measured on GB300 (32^3 Q2 mixed step, ncu launch
// list) the gathers and per-tap index arithmetic take 21.9 us per
// restriction and 16.1 us per prolongation against 6.2 and 7.8 us for the
// CSR kernels, which stream each row's few entries.
// ---------------------------------------------------------------------------
struct LatMap {
  int lf[3], lc[3];            // fine / coarse lattice extents (own axes)
  int perm[3], sign[3], t2[3];
  // per fine axis d: the coarse axis's half-unit offset and lattice stride
  int t2f[3], csf[3];
};

// the coarse taps of half-unit coordinate U along one axis
__device__ __forceinline__ int lat_taps(int U, int* q, double* w) {
  if ((U & 1) == 0) {
    q[0] = U >> 1;
    w[0] = 1.0;
    q[1] = q[2] = q[0];
    w[1] = w[2] = 0.0;
    return 1;
  }
  const int c2 = (U >> 2) * 2;
  q[0] = c2;
  q[1] = c2 + 1;
  q[2] = c2 + 2;
  const bool first = (U & 3) == 1;
  w[0] = first ? 0.375 : -0.125;
  w[1] = 0.75;
  w[2] = first ? -0.125 : 0.375;
  return 3;
}

// fine lattice point idx: per fine axis d its taps (count, coarse node,
// weight); the coarse lattice index of a tap is sum_d q_d * csf[d]
__device__ __forceinline__ void lat_fine_taps(const LatMap& M, long idx, int* nt, int (*q)[3],
                                              double (*w)[3]) {
  const int p[3] = {(int)(idx % M.lf[0]), (int)((idx / M.lf[0]) % M.lf[1]),
                    (int)(idx / ((long)M.lf[0] * M.lf[1]))};
#pragma unroll
  for (int d = 0; d < 3; ++d) nt[d] = lat_taps(M.t2f[d] + M.sign[d] * p[d], q[d], w[d]);
}

// tap j of one axis at half-unit coordinate U: coarse node and weight
// (prolongation: 1 tap at an even U, else the three quarter-point weights)
template <typename T>
__device__ __forceinline__ void lat_prolong_tap(int U, int j, int& q, T& w) {
  if ((U & 1) == 0) {
    q = U >> 1;
    w = (T)1;
    return;
  }
  q = (U >> 2) * 2 + j;
  const bool first = (U & 3) == 1;
  w = j == 1 ? (T)0.75 : ((j == 0) == first ? (T)0.375 : (T)-0.125);
}

// x_f[i] += damp * (P x_c)[i] on fine actives, or x_f = P x_c (add == 0);
// a thread per fine point, its 1 to 27 taps decoded from a flat index
template <typename T>
__global__ void __launch_bounds__(256)
k_lat_prolong(LatMap M, int nactive_f, const int* __restrict__ mapf, const int* __restrict__ mapc,
              const T* __restrict__ xc, T* __restrict__ xf, T damp, int add) {
  pdl_enter();
  const long nf = (long)M.lf[0] * M.lf[1] * M.lf[2];
  const long idx = blockIdx.x * 256L + threadIdx.x;
  if (idx >= nf) return;
  const int row = __ldg(mapf + idx);
  if (add && row >= nactive_f) return;
  const int p0 = (int)(idx % M.lf[0]), p1 = (int)((idx / M.lf[0]) % M.lf[1]),
            p2 = (int)(idx / ((long)M.lf[0] * M.lf[1]));
  const int U0 = M.t2f[0] + M.sign[0] * p0, U1 = M.t2f[1] + M.sign[1] * p1,
            U2 = M.t2f[2] + M.sign[2] * p2;
  const int n0 = (U0 & 1) ? 3 : 1, n1 = (U1 & 1) ? 3 : 1, n2 = (U2 & 1) ? 3 : 1;
  const int nt = n0 * n1 * n2;
  T s = 0;
#pragma unroll 3
  for (int t = 0; t < nt; ++t) {
    const int a = t % n0, r = t / n0, b = r % n1, c = r / n1;
    int qa, qb, qc;
    T wa, wb, wc;
    lat_prolong_tap<T>(U0, a, qa, wa);
    lat_prolong_tap<T>(U1, b, qb, wb);
    lat_prolong_tap<T>(U2, c, qc, wc);
    const long ci = (long)qa * M.csf[0] + (long)qb * M.csf[1] + (long)qc * M.csf[2];
    s += ((wc * wb) * wa) * xc[__ldg(mapc + ci)];
  }
  if (!add) xf[row] = s;
  else xf[row] += damp * s;
}

// r_c = P^T d_f on every coarse lattice point; coarse non-actives zeroed
// when mask.  Along its coarse axis a node q takes the fine points at
// half-unit offsets -3, -1, 0, 1, 3 (q even: weights -1/8, 3/8, 1, 3/8,
// -1/8) or -1, 0, 1 (q odd: 3/4, 1, 3/4); kLatLanes lanes per coarse point
// share its up to 125 taps and add their sums by shuffles
constexpr int kLatLanes = 8;

template <typename T>
__device__ __forceinline__ int lat_restrict_tap(int qk, int j, T& w) {
  if (qk & 1) {
    w = j == 1 ? (T)1 : (T)0.75;
    return j - 1;
  }
  const int off = j == 0 ? -3 : (j == 1 ? -1 : (j == 2 ? 0 : (j == 3 ? 1 : 3)));
  w = j == 2 ? (T)1 : ((j == 1 || j == 3) ? (T)0.375 : (T)-0.125);
  return off;
}

template <typename T>
__global__ void __launch_bounds__(256)
k_lat_restrict(LatMap M, int nactive_c, const int* __restrict__ mapf,
               const int* __restrict__ mapc, const T* __restrict__ df, T* __restrict__ rc,
               int mask) {
  pdl_enter();
  const long nc = (long)M.lc[0] * M.lc[1] * M.lc[2];
  const long gt = blockIdx.x * 256L + threadIdx.x;
  const long idx = gt / kLatLanes;
  const int lane = (int)(gt % kLatLanes);
  const bool live = idx < nc;
  int row = 0;
  bool act = false;
  int qd[3] = {0, 0, 0};
  if (live) {
    row = __ldg(mapc + idx);
    act = !(mask && row >= nactive_c);
    const int q[3] = {(int)(idx % M.lc[0]), (int)((idx / M.lc[0]) % M.lc[1]),
                      (int)(idx / ((long)M.lc[0] * M.lc[1]))};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int k = M.perm[d];
      qd[d] = k == 0 ? q[0] : (k == 1 ? q[1] : q[2]);
    }
  }
  T s = 0;
  if (live && act) {
    const int n0 = (qd[0] & 1) ? 3 : 5, n1 = (qd[1] & 1) ? 3 : 5, n2 = (qd[2] & 1) ? 3 : 5;
    const int nt = n0 * n1 * n2;
    for (int t = lane; t < nt; t += kLatLanes) {
      const int a = t % n0, r = t / n0, b = r % n1, c = r / n1;
      T wa, wb, wc;
      const int f0 = M.sign[0] * (2 * qd[0] + lat_restrict_tap<T>(qd[0], a, wa) - M.t2f[0]);
      const int f1 = M.sign[1] * (2 * qd[1] + lat_restrict_tap<T>(qd[1], b, wb) - M.t2f[1]);
      const int f2 = M.sign[2] * (2 * qd[2] + lat_restrict_tap<T>(qd[2], c, wc) - M.t2f[2]);
      if (f0 < 0 || f0 >= M.lf[0] || f1 < 0 || f1 >= M.lf[1] || f2 < 0 || f2 >= M.lf[2])
        continue;
      const long fi = ((long)f2 * M.lf[1] + f1) * M.lf[0] + f0;
      s += ((wc * wb) * wa) * df[__ldg(mapf + fi)];
    }
  }
#pragma unroll
  for (int o = kLatLanes / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, kLatLanes);
  if (live && lane == 0) rc[row] = act ? s : (T)0;
}

// every row of P against the lattice weights: the same coarse columns, the
// values to 1e-12 (P drops no lattice tap: none is below its 1e-14 cut)
__global__ void __launch_bounds__(256)
k_lat_check(LatMap M, const int* __restrict__ mapf, const int* __restrict__ mapc,
            const int* __restrict__ prp, const int* __restrict__ pcol,
            const double* __restrict__ pval, int* bad) {
  const long nf = (long)M.lf[0] * M.lf[1] * M.lf[2];
  const long idx = blockIdx.x * 256L + threadIdx.x;
  if (idx >= nf) return;
  const int row = mapf[idx];
  int nt[3], q[3][3];
  double w[3][3];
  lat_fine_taps(M, idx, nt, q, w);
  const int e0 = prp[row], e1 = prp[row + 1];
  if (e1 - e0 != nt[0] * nt[1] * nt[2]) {
    atomicOr(bad, 1);
    return;
  }
  for (int e = e0; e < e1; ++e) {
    bool found = false;
    for (int c = 0; c < nt[2] && !found; ++c)
      for (int b = 0; b < nt[1] && !found; ++b)
        for (int a = 0; a < nt[0] && !found; ++a) {
          const int g = mapc[(long)q[2][c] * M.csf[2] + (long)q[1][b] * M.csf[1] +
                             (long)q[0][a] * M.csf[0]];
          if (g != pcol[e]) continue;
          found = true;
          if (fabs(pval[e] - w[2][c] * w[1][b] * w[0][a]) > 1e-12) atomicOr(bad, 2);
        }
    if (!found) atomicOr(bad, 4);
  }
}

static LatMap lat_map(const DevLevel& F, const DevLevel& C) {
  LatMap M;
  for (int d = 0; d < 3; ++d) {
    M.lf[d] = F.st_dims[d];
    M.lc[d] = C.st_dims[d];
    M.perm[d] = F.lt_perm[d];
    M.sign[d] = F.lt_sign[d];
    M.t2[d] = F.lt_t2[d];
  }
  const int cst[3] = {1, C.st_dims[0], C.st_dims[0] * C.st_dims[1]};
  for (int d = 0; d < 3; ++d) {
    M.t2f[d] = F.lt_t2[F.lt_perm[d]];
    M.csf[d] = cst[F.lt_perm[d]];
  }
  return M;
}

// The fine points 0, 2 e_0, 2 e_1, 2 e_2 of F's lattice coincide with coarse
// nodes (their P rows hold one entry, 1): their coarse lattice coordinates
// give each fine axis's coarse axis, direction and offset; then every row of
// P is checked on the device.
int lattice_transfer_setup(cdg_context* ctx, DevLevel& F, const DevLevel& C) {
  if (F.lt_state >= 0) return CDG_OK;
  const char* e = std::getenv("CDG_LAT_TRANSFER");
  if (!e || e[0] != '1') return CDG_OK;
  if (F.mf_geo < 0 || C.mf_geo < 0) return CDG_OK;   // lattices not looked for yet
  F.lt_state = 0;
  if (!F.st_dims[0] || !C.st_dims[0] || !F.P_rp || !F.P_val) return CDG_OK;
  const int* lf = F.st_dims;
  const int* lc = C.st_dims;
  const long ncp = (long)lc[0] * lc[1] * lc[2];
  std::vector<int> cmap(ncp);
  CDG_CUDA(cudaMemcpyAsync(cmap.data(), C.st_map, ncp * sizeof(int), cudaMemcpyDeviceToHost,
                           ctx->stream));
  const long probe[4] = {0, 2, 2L * lf[0], 2L * lf[0] * lf[1]};
  int g[4], rp[8], col[4];
  double val[4];
  for (int k = 0; k < 4; ++k)
    CDG_CUDA(cudaMemcpyAsync(&g[k], F.st_map + probe[k], sizeof(int), cudaMemcpyDeviceToHost,
                             ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < 4; ++k) {
    CDG_CUDA(cudaMemcpyAsync(&rp[2 * k], F.P_rp + g[k], 2 * sizeof(int), cudaMemcpyDeviceToHost,
                             ctx->stream));
  }
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < 4; ++k) {
    if (rp[2 * k + 1] - rp[2 * k] != 1) return CDG_OK;
    CDG_CUDA(cudaMemcpyAsync(&col[k], F.P_col + rp[2 * k], sizeof(int), cudaMemcpyDeviceToHost,
                             ctx->stream));
    CDG_CUDA(cudaMemcpyAsync(&val[k], F.P_val + rp[2 * k], sizeof(double),
                             cudaMemcpyDeviceToHost, ctx->stream));
  }
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  int qc[4][3];
  for (int k = 0; k < 4; ++k) {
    if (std::fabs(val[k] - 1.0) > 1e-12) return CDG_OK;
    long at = -1;
    for (long i = 0; i < ncp && at < 0; ++i)
      if (cmap[i] == col[k]) at = i;
    if (at < 0) return CDG_OK;
    qc[k][0] = (int)(at % lc[0]);
    qc[k][1] = (int)((at / lc[0]) % lc[1]);
    qc[k][2] = (int)(at / ((long)lc[0] * lc[1]));
  }
  int used = 0;
  for (int d = 0; d < 3; ++d) {
    int axis = -1, sg = 0;
    for (int k = 0; k < 3; ++k) {
      const int dq = qc[d + 1][k] - qc[0][k];
      if (dq == 0) continue;
      if ((dq != 1 && dq != -1) || axis >= 0) return CDG_OK;
      axis = k;
      sg = dq;
    }
    if (axis < 0 || (used >> axis) & 1) return CDG_OK;
    used |= 1 << axis;
    if (lf[d] != 2 * lc[axis] - 1) return CDG_OK;
    F.lt_perm[d] = axis;
    F.lt_sign[d] = sg;
  }
  for (int k = 0; k < 3; ++k) F.lt_t2[k] = 2 * qc[0][k];
  int* bad = nullptr;
  CDG_CUDA(cudaMalloc(&bad, sizeof(int)));
  int hb = 1;
  cudaError_t err = cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream);
  const long nf = (long)lf[0] * lf[1] * lf[2];
  if (err == cudaSuccess) {
    k_lat_check<<<(unsigned)((nf + 255) / 256), 256, 0, ctx->stream>>>(
        lat_map(F, C), F.st_map, C.st_map, F.P_rp, F.P_col, F.P_val, bad);
    ++ctx->launches;
    err = cudaGetLastError();
  }
  if (err == cudaSuccess) err = cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost,
                                                ctx->stream);
  if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->stream);
  cudaFree(bad);
  CDG_CUDA(err);
  F.lt_state = hb == 0 ? 1 : 0;
  return CDG_OK;
}

template <typename T>
__global__ void k_coarse_init(int n, int na, const T* __restrict__ b, T* __restrict__ x) {
  pdl_enter();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    x[i] = i < na ? (T)0 : b[i];
}

// x_a += Inv d_a  (FP64 dense inverse of the coarsest active block), warp/row
template <typename T>
__global__ void k_coarse_apply(int na, const double* __restrict__ inv, const T* __restrict__ d,
                               T* __restrict__ x) {
  pdl_enter();
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, l = threadIdx.x & 31;
  if (row >= na) return;
  double s = 0.0;
  for (int j = l; j < na; j += 32) s += inv[(size_t)row * na + j] * (double)d[j];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (l == 0) x[row] = (T)((double)x[row] + s);
}

// ---------------------------------------------------------------------------
// coarsest level: in-place Gauss-Jordan inversion with partial pivoting of
// the active block (n x n, double-buffered between pivot steps).  Step k:
//   p = first row of maximal |a_ik|, i >= k; rows k and p exchange;
//   a_kj <- a_pj / a_pk (j != k),  a_kk <- 1 / a_pk;
//   a_ij <- a_rj - a_rk a_kj (j != k),  a_ik <- -a_rk / a_pk  (i != k, r =
//   the row that moves to i).
// After the last step the columns exchange in reverse pivot order, giving the
// inverse of the active block.  One reciprocal per step, one FMA per entry.
// ---------------------------------------------------------------------------
__global__ void k_extract_dense(int na, const int* __restrict__ rp, const int* __restrict__ col,
                                const double* __restrict__ val, double* __restrict__ M) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= na) return;
  for (int k = rp[i]; k < rp[i + 1]; ++k)
    if (col[k] < na) M[(size_t)i * na + col[k]] = val[k];
}

// pivot of step k (every block computes the same one)
__device__ __forceinline__ int gj_pivot(int na, int k, const double* __restrict__ Min,
                                        double* sv, int* si) {
  double best = -1.0;
  int bi = k;
  for (int i = k + threadIdx.x; i < na; i += 256) {
    double a = fabs(Min[(size_t)i * na + k]);
    if (a > best) { best = a; bi = i; }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double a = __shfl_xor_sync(0xffffffffu, best, o);
    int ai = __shfl_xor_sync(0xffffffffu, bi, o);
    if (a > best || (a == best && ai < bi)) { best = a; bi = ai; }
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { sv[w] = best; si[w] = bi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < 8; ++q)
      if (sv[q] > sv[0] || (sv[q] == sv[0] && si[q] < si[0])) { sv[0] = sv[q]; si[0] = si[q]; }
  }
  __syncthreads();
  const int p = si[0];
  __syncthreads();   // sv/si are reused by the next step
  return p;
}

// rows of step k handled by this block: i = blockIdx.x, + gridDim.x, ...
__device__ __forceinline__ bool gj_step(int na, int k, const double* __restrict__ Min,
                                        double* __restrict__ Mout, int* __restrict__ perm,
                                        int* err, double* sv, int* si) {
  const int p = gj_pivot(na, k, Min, sv, si);
  const double piv = Min[(size_t)p * na + k];
  if (piv == 0.0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, kErrSingular);
    return false;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) perm[k] = p;
  const double rpiv = 1.0 / piv;
  const double* prow = Min + (size_t)p * na;
  for (int i = blockIdx.x; i < na; i += gridDim.x) {
    double* out = Mout + (size_t)i * na;
    if (i == k) {
      for (int j = threadIdx.x; j < na; j += 256) out[j] = j == k ? rpiv : prow[j] * rpiv;
    } else {
      const double* src = Min + (size_t)(i == p ? k : i) * na;
      const double f = src[k];
      for (int j = threadIdx.x; j < na; j += 256)
        out[j] = j == k ? -f * rpiv : fma(-f, prow[j] * rpiv, src[j]);
    }
  }
  return true;
}

__global__ void __launch_bounds__(256)
k_gj_step(int na, int k, const double* __restrict__ Min, double* __restrict__ Mout,
          int* __restrict__ perm, int* err) {
  pdl_enter();
  __shared__ double sv[8];
  __shared__ int si[8];
  gj_step(na, k, Min, Mout, perm, err, sv, si);
}

// column exchanges in reverse pivot order: inv[:, j] = M[:, q[j]]
__global__ void k_gj_colmap(int na, const int* __restrict__ perm, int* __restrict__ q) {
  pdl_enter();
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int j = 0; j < na; ++j) q[j] = j;
  for (int k = na - 1; k >= 0; --k) {
    const int a = q[k];
    q[k] = q[perm[k]];
    q[perm[k]] = a;
  }
}

__global__ void k_gj_unpermute(int na, const double* __restrict__ M, const int* __restrict__ q,
                               double* __restrict__ inv) {
  pdl_enter();
  for (int i = blockIdx.x; i < na; i += gridDim.x)
    for (int j = threadIdx.x; j < na; j += blockDim.x)
      inv[(size_t)i * na + j] = M[(size_t)i * na + q[j]];
}

// all na pivot steps in one cooperative launch, grid-wide sync between steps;
// every block sees the same pivot, so all blocks leave together on a zero pivot
__global__ void __launch_bounds__(256)
k_gj_coop(int na, double* A, double* B, int* perm, int* q, double* inv, int* err) {
  pdl_enter();
  __shared__ double sv[8];
  __shared__ int si[8];
  cgrp::grid_group grid = cgrp::this_grid();
  double* Min = A;
  double* Mout = B;
  for (int k = 0; k < na; ++k) {
    if (!gj_step(na, k, Min, Mout, perm, err, sv, si)) return;
    grid.sync();
    double* t = Min;
    Min = Mout;
    Mout = t;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    for (int j = 0; j < na; ++j) q[j] = j;
    for (int k = na - 1; k >= 0; --k) {
      const int a = q[k];
      q[k] = q[perm[k]];
      q[perm[k]] = a;
    }
  }
  grid.sync();
  for (int i = blockIdx.x; i < na; i += gridDim.x)
    for (int j = threadIdx.x; j < na; j += 256) inv[(size_t)i * na + j] = Min[(size_t)i * na + q[j]];
}

// small active blocks (na <= 160): the whole matrix in one CTA's shared
// memory, in place; the pivot row (scaled) and column k are buffered first,
// then every row except k is eliminated (row p reads the old row k), then
// row k is replaced.  Same pivots and arithmetic as the cooperative kernel.
constexpr int kGjSmemThreads = 1024;

__global__ void __launch_bounds__(kGjSmemThreads)
k_gj_smem(int na, const double* __restrict__ Ain, double* __restrict__ inv, int* err) {
  pdl_enter();
  extern __shared__ double sm[];
  double* a = sm;                       // na * na
  double* prow = a + (size_t)na * na;   // na
  double* colk = prow + na;             // na
  int* perm = (int*)(colk + na);        // na
  int* q = perm + na;                   // na
  __shared__ double wv[32];
  __shared__ int wi[32];
  __shared__ int s_p;
  __shared__ double s_piv;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, w = tid >> 5;
  for (int t = tid; t < na * na; t += nt) a[t] = Ain[t];
  __syncthreads();
  for (int k = 0; k < na; ++k) {
    double best = -1.0;
    int bi = k;
    for (int i = k + tid; i < na; i += nt) {
      double v = fabs(a[(size_t)i * na + k]);
      if (v > best) { best = v; bi = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      double v = __shfl_xor_sync(0xffffffffu, best, o);
      int vi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (v > best || (v == best && vi < bi)) { best = v; bi = vi; }
    }
    if (lane == 0) { wv[w] = best; wi[w] = bi; }
    __syncthreads();
    if (tid == 0) {
      double b = wv[0];
      int p = wi[0];
      for (int u = 1; u < nt / 32; ++u)
        if (wv[u] > b || (wv[u] == b && wi[u] < p)) { b = wv[u]; p = wi[u]; }
      s_p = p;
      s_piv = a[(size_t)p * na + k];
      perm[k] = p;
    }
    __syncthreads();
    const int p = s_p;
    const double piv = s_piv;
    if (piv == 0.0) {
      if (tid == 0) atomicOr(err, kErrSingular);
      return;   // uniform: every thread read the same pivot
    }
    const double rpiv = 1.0 / piv;
    for (int j = tid; j < na; j += nt) prow[j] = j == k ? rpiv : a[(size_t)p * na + j] * rpiv;
    for (int i = tid; i < na; i += nt) colk[i] = a[(size_t)(i == p ? k : i) * na + k];
    __syncthreads();
    // rows i != k; row p takes the old row k (row k is not written in this
    // pass, row p is read by no other row)
    for (int t = tid; t < na * na; t += nt) {
      const int i = t / na, j = t - i * na;
      if (i == k) continue;
      const double f = colk[i];
      const double old = a[(size_t)(i == p ? k : i) * na + j];
      a[t] = j == k ? -f * rpiv : fma(-f, prow[j], old);
    }
    __syncthreads();
    for (int j = tid; j < na; j += nt) a[(size_t)k * na + j] = prow[j];
    __syncthreads();
  }
  if (tid == 0) {
    for (int j = 0; j < na; ++j) q[j] = j;
    for (int k = na - 1; k >= 0; --k) {
      const int t = q[k];
      q[k] = q[perm[k]];
      q[perm[k]] = t;
    }
  }
  __syncthreads();
  for (int t = tid; t < na * na; t += nt) {
    const int i = t / na, j = t - (t / na) * na;
    inv[t] = a[(size_t)i * na + q[j]];
  }
}

static size_t gj_smem_bytes(int na) {
  return (size_t)na * na * sizeof(double) + 2 * (size_t)na * sizeof(double) +
         2 * (size_t)na * sizeof(int);
}

static int coarse_inverse(cdg_context* ctx, DevLevel& C) {
  const int na = C.nactive;
  C.coarse_na = na;
  if (na == 0) return CDG_OK;
  if (na > 8192) { set_error("coarse level too large for the dense inverse (%d)", na); return CDG_ERR_LIMIT; }
  const size_t sz = (size_t)na * na;
  if (!C.coarse_work) {
    // two n x n buffers + pivot rows + column map
    CDG_CUDA(cudaMalloc(&C.coarse_work, (2 * sz + na) * sizeof(double)));
    CDG_CUDA(cudaMalloc(&C.coarse_inv, sz * sizeof(double)));
  }
  double* A = C.coarse_work;
  double* B = C.coarse_work + sz;
  int* perm = (int*)(C.coarse_work + 2 * sz);
  int* q = perm + na;
  CDG_CUDA(cudaMemsetAsync(A, 0, sz * sizeof(double), ctx->stream));
  CDG_LAUNCH_PDL(ctx, k_extract_dense, grid_for<int>(na, 128), 128, 0, na, C.row_ptr, C.col, C.val64, A);
  // the grid-wide kernel (a pivot step costs one grid sync); one CTA holding
  // the block in shared memory where cooperative launches are unavailable.
  // Measured on GB300: grid-wide 0.54 ms (125 rows) / 2.25 ms (343 rows), one
  // CTA 2.2 ms (125, one SM's FP64 pipe), a 16-CTA cluster with the rows in
  // distributed shared memory 0.71 / 3.56 ms (barriers per pivot step), a
  // blocked variant (panels of 4-32 pivot columns factored in one CTA, then a
  // rank-b update of the other columns by all SMs) 2.8-4.3 ms for 343 rows:
  // the panel steps run on one SM's FP64 pipe
  int coop = 0, per_sm = 0;
  CDG_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device));
  CDG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gj_coop, 256, 0));
  // one block per row up to one (or two) per SM: the elimination (na^2 FMA
  // per step) is bound by FP64 issue, so it wants every SM's pipe (32 blocks
  // measured 1.9x slower at 343 rows)
  int g = (int)std::min<long>((long)na, (long)ctx->num_sms * std::min(per_sm, na > 1024 ? 2 : 1));
  const size_t smem = gj_smem_bytes(na);
  if (!(coop && per_sm > 0) && smem <= 220 * 1024) {
    CDG_CUDA(cudaFuncSetAttribute(k_gj_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CDG_LAUNCH_PDL(ctx, k_gj_smem, 1, kGjSmemThreads, smem, na, A, C.coarse_inv, ctx->d_err);
    return CDG_OK;
  }
  if (coop && per_sm > 0 && g >= 1) {
    double* inv = C.coarse_inv;
    void* args[] = {(void*)&na, (void*)&A, (void*)&B, (void*)&perm, (void*)&q, (void*)&inv,
                    (void*)&ctx->d_err};
    CDG_CUDA(cudaLaunchCooperativeKernel((const void*)k_gj_coop, dim3(g), dim3(256), args, 0,
                                         ctx->stream));
    ctx->launches++;
    return CDG_OK;
  }
  for (int k = 0; k < na; ++k) {
    int gg = std::min(na, ctx->num_sms * 4);
    CDG_LAUNCH_PDL(ctx, k_gj_step, gg, 256, 0, na, k, A, B, perm, ctx->d_err);
    std::swap(A, B);
  }
  CDG_LAUNCH_PDL(ctx, k_gj_colmap, 1, 32, 0, na, perm, q);
  CDG_LAUNCH_PDL(ctx, k_gj_unpermute, std::min(na, ctx->num_sms * 4), 256, 0, na, A, q, C.coarse_inv);
  return CDG_OK;
}

// ---------------------------------------------------------------------------
// multigrid (Multigrid::cycle); levels: p->lev[0] finest ... lev[nl-1]
// ---------------------------------------------------------------------------
template <typename T> struct Prec;
template <> struct Prec<double> {
  static const double* val(const DevLevel& L) { return L.val64; }
  static const double* sell(const DevLevel& L) { return L.sell_val; }
  static bool has_sell(const DevLevel& L) { return L.sell_nslices > 0; }
  static const double* invd(const DevLevel& L) { return L.invdiag64; }
  static const double* dcv(const DevLevel& L) { return L.dc_val64; }
  static const double* P(const DevLevel& L) { return L.P_val; }
  static const double* R(const DevLevel& L) { return L.R_val; }
};
template <> struct Prec<float> {
  static const float* val(const DevLevel& L) { return L.val32; }
  static const float* sell(const DevLevel&) { return nullptr; }
  static bool has_sell(const DevLevel&) { return false; }   // CSR measured faster in FP32
  static const float* invd(const DevLevel& L) { return L.invdiag32; }
  static const float* dcv(const DevLevel& L) { return L.dc_val32; }
  static const float* P(const DevLevel& L) { return L.P_val32; }
  static const float* R(const DevLevel& L) { return L.R_val32; }
};

static int vec_grid(cdg_context* ctx, long n) {
  long g = (n + 255) / 256;
  long cap = (long)ctx->num_sms * 8;
  return (int)(g > cap ? cap : (g < 1 ? 1 : g));
}

// the FP32 multigrid applies a level's operator matrix-free where the level
// has valid cell factors and the tuner chose that kernel (matfree.cu)
template <typename T>
static bool mf_on(const DevLevel& L) {
  return std::is_same<T, float>::value && L.mf_valid && L.mf_mode == 1;
}

// last smoothing step of the finest level with the FP64 hand-over (MODE 3)
template <typename T>
static int smooth_out(cdg_context* ctx, const DevLevel& L, const T* val, const T* x, const T* b,
                      const T* invd, T w, T* y, double* z, const int* di, double* zcur) {
  if constexpr (std::is_same<T, float>::value)
    if (mf_on<T>(L)) return mf_apply(ctx, L, 3, x, b, invd, w, y, z, di, zcur);
  const int tpr = std::is_same<T, float>::value && L.tpr32 ? L.tpr32 : L.rows_per_warp_hint;
  const int grid = (int)(((long)L.ndof * tpr + 255) / 256);
  switch (tpr) {
    case 2: CDG_LAUNCH_PDL(ctx, (k_spmv<T, 2, 8, 3>), grid, 256, 0, L.ndof, L.nactive, L.row_ptr, L.col, val, x, b, invd, w, y, z, di, zcur); break;
    case 4: CDG_LAUNCH_PDL(ctx, (k_spmv<T, 4, 8, 3>), grid, 256, 0, L.ndof, L.nactive, L.row_ptr, L.col, val, x, b, invd, w, y, z, di, zcur); break;
    case 8: CDG_LAUNCH_PDL(ctx, (k_spmv<T, 8, 8, 3>), grid, 256, 0, L.ndof, L.nactive, L.row_ptr, L.col, val, x, b, invd, w, y, z, di, zcur); break;
    default: CDG_LAUNCH_PDL(ctx, (k_spmv<T, 16, 8, 3>), grid, 256, 0, L.ndof, L.nactive, L.row_ptr, L.col, val, x, b, invd, w, y, z, di, zcur); break;
  }
  return CDG_OK;
}

// sliced ELLPACK smoothing / defect on a multigrid level
template <typename T, int MODE>
static int sell_mg(cdg_context* ctx, const DevLevel& L, const T* val, const T* x, const T* b,
                   const T* invd, T w, T* y) {
  const int grid = (int)(((long)L.sell_nslices * 32 + 255) / 256);
  switch (L.sell_lanes) {
    case 1: CDG_LAUNCH_PDL(ctx, (k_sell<T, 1, 8, MODE>), grid, 256, 0, L.sell_nslices, L.sell_off, L.sell_row, L.sell_col, val, x, b, invd, w, y); break;
    case 2: CDG_LAUNCH_PDL(ctx, (k_sell<T, 2, 8, MODE>), grid, 256, 0, L.sell_nslices, L.sell_off, L.sell_row, L.sell_col, val, x, b, invd, w, y); break;
    case 4: CDG_LAUNCH_PDL(ctx, (k_sell<T, 4, 8, MODE>), grid, 256, 0, L.sell_nslices, L.sell_off, L.sell_row, L.sell_col, val, x, b, invd, w, y); break;
    case 8: CDG_LAUNCH_PDL(ctx, (k_sell<T, 8, 8, MODE>), grid, 256, 0, L.sell_nslices, L.sell_off, L.sell_row, L.sell_col, val, x, b, invd, w, y); break;
    default: CDG_LAUNCH_PDL(ctx, (k_sell<T, 16, 8, MODE>), grid, 256, 0, L.sell_nslices, L.sell_off, L.sell_row, L.sell_col, val, x, b, invd, w, y); break;
  }
  return CDG_OK;
}

// CSR smoothing / defect of a multigrid level: FP32 levels with staged chunks
// take the shared-memory streaming kernel
template <int MODE>
static int mg_spmv(cdg_context* ctx, const DevLevel& L, const float* val, const float* x,
                   const float* b, const float* invd, float w, float* y) {
  if (L.bulk_nchunks) return spmv_bulk_any<MODE>(ctx, L, val, x, b, invd, w, y);
  return spmv_t<float, MODE>(ctx, L, val, x, b, invd, w, y);
}
template <int MODE>
static int mg_spmv(cdg_context* ctx, const DevLevel& L, const double* val, const double* x,
                   const double* b, const double* invd, double w, double* y) {
  return spmv_t<double, MODE>(ctx, L, val, x, b, invd, w, y);
}

template <typename T>
static int smooth(cdg_context* ctx, DevLevel& L, T damp) {
  if constexpr (std::is_same<T, float>::value) {
    if (mf_on<T>(L)) {
      CDG_TRY(mf_apply(ctx, L, 2, (const float*)L.mg_sol, (const float*)L.mg_rhs, L.invdiag32,
                       damp, (float*)L.mg_tmp));
      std::swap(L.mg_sol, L.mg_tmp);
      return CDG_OK;
    }
  }
  if (Prec<T>::has_sell(L))
    CDG_TRY((sell_mg<T, 2>(ctx, L, Prec<T>::sell(L), (const T*)L.mg_sol, (const T*)L.mg_rhs,
                           Prec<T>::invd(L), damp, (T*)L.mg_tmp)));
  else
    CDG_TRY((mg_spmv<2>(ctx, L, Prec<T>::val(L), (const T*)L.mg_sol, (const T*)L.mg_rhs,
                        Prec<T>::invd(L), damp, (T*)L.mg_tmp)));
  std::swap(L.mg_sol, L.mg_tmp);
  return CDG_OK;
}

// sum_k dcv[k] * x[col[k]] over a row's couplings to non-active columns, in k
// order; the loads of eight terms are issued together (a boundary row has up
// to ~45 such couplings, and one thread walks them)
template <typename T, typename X>
__device__ __forceinline__ T dirichlet_coupling(int k, int ke, const int* __restrict__ col,
                                                const T* __restrict__ dcv,
                                                const X* __restrict__ x) {
  T s = 0;
  for (; k + 8 <= ke; k += 8) {
    T a[8];
    int c[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      a[u] = dcv[k + u];
      c[u] = col[k + u];
    }
    T xv[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) xv[u] = (T)x[c[u]];
#pragma unroll
    for (int u = 0; u < 8; ++u) s += a[u] * xv[u];
  }
  for (; k < ke; ++k) s += dcv[k] * (T)x[col[k]];
  return s;
}

// first smoothing step from x0 = 0 on active rows and x0 = b on non-active
// rows (zero there on coarse levels): A x0 on an active row only involves its
// non-active columns, so the step needs no full SpMV
template <typename T>
__global__ void __launch_bounds__(256)
k_first_smooth(int n, int nactive, int with_dirichlet, const int* __restrict__ dc_rp,
               const int* __restrict__ dc_col, const T* __restrict__ dcv,
               const T* __restrict__ b, const T* __restrict__ invd, T w, T* __restrict__ x1) {
  pdl_enter();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    if (i < nactive) {
      T s = 0;
      if (with_dirichlet) s = dirichlet_coupling(dc_rp[i], dc_rp[i + 1], dc_col, dcv, b);
      x1[i] = w * (invd[i] * (b[i] - s));
    } else {
      const T x0 = with_dirichlet ? b[i] : (T)0;
      x1[i] = x0 + w * (invd[i] * (b[i] - x0));
    }
  }
}

// the finest level's first smoothing step fused with the cycle's start
// (Iteration_multigrid::apply copies the Krylov vector into the multigrid
// rhs): rhs = v in T, and x1 as k_first_smooth computes it from that rhs,
// reading the Dirichlet neighbours' rhs straight from v.  Blocks below
// row_blocks take a row per thread (rows without couplings to non-active
// columns complete there); the others take the rows of dc_rows, 8 lanes per
// row over its couplings (up to ~45 on a Q2 boundary layer, which one thread
// walked in sequence while the rest of its warp waited)
constexpr int kDcLanes = 8;

template <typename T>
__global__ void __launch_bounds__(256)
k_first_smooth_init(int n, int nactive, int row_blocks, int ndc, const int* __restrict__ dc_rows,
                    const int* __restrict__ dc_rp, const int* __restrict__ dc_col,
                    const T* __restrict__ dcv, const double* __restrict__ v,
                    const T* __restrict__ invd, T w, T* __restrict__ rhs, T* __restrict__ x1,
                    const int* di) {
  pdl_enter();
  if (di) v += (size_t)(*di) * n;
  if ((int)blockIdx.x < row_blocks) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const T bi = (T)v[i];
    rhs[i] = bi;
    if (i < nactive) {
      if (dc_rp[i] == dc_rp[i + 1]) x1[i] = w * (invd[i] * (bi - (T)0));
    } else {
      x1[i] = bi + w * (invd[i] * (bi - bi));
    }
    return;
  }
  const int g = ((int)blockIdx.x - row_blocks) * (blockDim.x / kDcLanes) + threadIdx.x / kDcLanes;
  const int l = threadIdx.x % kDcLanes;
  T s = 0;
  int r = -1;
  if (g < ndc) {
    r = dc_rows[g];
    const int k1 = dc_rp[r + 1];
    for (int k = dc_rp[r] + l; k < k1; k += kDcLanes) s += dcv[k] * (T)v[dc_col[k]];
  }
#pragma unroll
  for (int o = kDcLanes / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (r >= 0 && l == 0) {
    const T bi = (T)v[r];
    x1[r] = w * (invd[r] * (bi - s));
  }
}

template <typename T>
static int first_smooth(cdg_context* ctx, DevLevel& L, T damp, bool finest) {
  CDG_LAUNCH_PDL(ctx, k_first_smooth<T>, vec_grid(ctx, L.ndof), 256, 0, L.ndof, L.nactive,
             finest ? 1 : 0, L.dc_rp, L.dc_col, Prec<T>::dcv(L), (const T*)L.mg_rhs,
             Prec<T>::invd(L), damp, (T*)L.mg_tmp);
  std::swap(L.mg_sol, L.mg_tmp);
  return CDG_OK;
}

template <typename T>
static int defect(cdg_context* ctx, DevLevel& L) {
  if constexpr (std::is_same<T, float>::value)
    if (mf_on<T>(L))
      return mf_apply(ctx, L, 1, (const float*)L.mg_sol, (const float*)L.mg_rhs, nullptr, 0.f,
                      (float*)L.mg_def);
  if (Prec<T>::has_sell(L))
    return sell_mg<T, 1>(ctx, L, Prec<T>::sell(L), (const T*)L.mg_sol, (const T*)L.mg_rhs,
                         nullptr, (T)0, (T*)L.mg_def);
  return mg_spmv<1>(ctx, L, Prec<T>::val(L), (const T*)L.mg_sol, (const T*)L.mg_rhs,
                    (const T*)nullptr, (T)0, (T*)L.mg_def);
}

// update_solution_in_finer_grid: fine.sol += damp * P coarse.sol on actives
template <typename T>
static int prolong_correct(cdg_context* ctx, DevLevel& F, DevLevel& C, T damp) {
  if (F.lt_state == 1) {
    const long nf = (long)F.st_dims[0] * F.st_dims[1] * F.st_dims[2];
    CDG_LAUNCH_PDL(ctx, k_lat_prolong<T>, (int)((nf + 255) / 256), 256, 0, lat_map(F, C),
                   F.nactive, F.st_map, C.st_map, (const T*)C.mg_sol, (T*)F.mg_sol, damp, 1);
    return CDG_OK;
  }
  // lanes per row (rows of 1 to 27 entries on Q2 hexahedra, mixed within a
  // warp): 4 in FP32 (32^3 Q2 mixed step 34.9 -> 34.2 ms with 16 lanes per
  // restriction row), 2 in FP64 (no gain measured)
  constexpr int kL = std::is_same<T, float>::value ? 4 : 2;
  CDG_LAUNCH_PDL(ctx, (k_prolong<T, kL>), grid_for<int>((long)F.ndof * kL, 256), 256, 0, F.ndof,
             F.nactive, F.P_rp, F.P_col, Prec<T>::P(F), (const T*)C.mg_sol, (T*)F.mg_sol, damp, 1);
  return CDG_OK;
}

// r_c = R d_f with coarse non-actives zeroed (the multigrid's restriction)
template <typename T>
static int restrict_defect(cdg_context* ctx, DevLevel& F, DevLevel& C) {
  if (F.lt_state == 1) {
    const long nc = (long)C.st_dims[0] * C.st_dims[1] * C.st_dims[2];
    CDG_LAUNCH_PDL(ctx, k_lat_restrict<T>, (int)((nc * kLatLanes + 255) / 256), 256, 0,
                   lat_map(F, C),
                   C.nactive, F.st_map, C.st_map, (const T*)F.mg_def, (T*)C.mg_rhs, 1);
    return CDG_OK;
  }
  // lanes per row (up to 125 entries on Q2 hexahedra): 16 in FP32, 8 in FP64
  constexpr int kL = std::is_same<T, float>::value ? 16 : 8;
  CDG_LAUNCH_PDL(ctx, (k_restrict<T, kL>), grid_for<int>((long)C.ndof * kL, 256), 256, 0,
             C.ndof, C.nactive, F.R_rp, F.R_col, Prec<T>::R(F), (const T*)F.mg_def,
             (T*)C.mg_rhs, 1);
  return CDG_OK;
}

template <typename T>
static int coarse_solve(cdg_context* ctx, DevLevel& C, const cdg_solver_params& s) {
  if (s.multigrid_smoother_coarse == 0) {
    // direct_solve: x = A^-1 rhs (idempotent, one application suffices)
    CDG_LAUNCH_PDL(ctx, k_coarse_init<T>, vec_grid(ctx, C.ndof), 256, 0, C.ndof, C.nactive,
               (const T*)C.mg_rhs, (T*)C.mg_sol);
    CDG_TRY(defect<T>(ctx, C));
    CDG_LAUNCH_PDL(ctx, k_coarse_apply<T>, grid_for<int>((long)C.nactive * 32, 256), 256, 0,
               C.nactive, C.coarse_inv, (const T*)C.mg_def, (T*)C.mg_sol);
    return CDG_OK;
  }
  // jacobi iterations until the coarse residual is small enough
  double res = 1e10;
  double* d_norm = ctx->d_red + (size_t)(kRedSlots - 1) * kRedMaxBlocks - 8;  // spare scalars
  (void)d_norm;
  for (int i = 0; i < s.multigrid_coarse_max_n_iterations && res > s.multigrid_coarse_residual; ++i) {
    CDG_TRY(smooth<T>(ctx, C, (T)s.jacobi_damp));
    CDG_TRY(defect<T>(ctx, C));
    // residual norm on the host (rarely used path)
    std::vector<T> h(C.ndof);
    CDG_CUDA(cudaMemcpyAsync(h.data(), C.mg_def, C.ndof * sizeof(T), cudaMemcpyDeviceToHost,
                             ctx->stream));
    CDG_CUDA(cudaStreamSynchronize(ctx->stream));
    double ss = 0;
    for (T v : h) ss += (double)v * (double)v;
    res = sqrt(ss);
  }
  return CDG_OK;
}

enum { kDummy, kDown, kUp, kEnd };
static void fill_cycle(std::vector<int>& seq, std::vector<int>& rec, int level, int nlev, int cyc) {
  if (level == 0) {
    seq.push_back(kUp);
    return;
  }
  for (int j = 0; j < rec[level]; ++j) {
    seq.push_back(kDown);
    fill_cycle(seq, rec, level - 1, nlev, cyc);
  }
  if (cyc == 2) rec[level] = 1;
  seq.push_back(level == nlev - 1 ? kEnd : kUp);
}

template <typename T>
static int mg_cycle(cdg_context* ctx, cdg_problem* p, const cdg_solver_params& s,
                    const double* v, double* z, const int* di = nullptr, double* zcur = nullptr) {
  const int nl = s.multigrid_n_levels;
  auto lv = [&](int m) -> DevLevel& { return p->lev[nl - 1 - m]; };
  DevLevel& F = p->lev[0];
  // with pre-smoothing on a finest level above the coarse solve, the first
  // smoothing step also does the start (rhs = v, x0 = Dirichlet values)
  const bool fused_start = nl > 1 && s.multigrid_n_pre_smooth > 0;
  if (fused_start) {
    const int rb = (F.ndof + 255) / 256;
    const int db = (F.dc_nrows + 256 / kDcLanes - 1) / (256 / kDcLanes);
    CDG_LAUNCH_PDL(ctx, k_first_smooth_init<T>, rb + db, 256, 0, F.ndof, F.nactive, rb,
               F.dc_nrows, F.dc_rows, F.dc_rp, F.dc_col, Prec<T>::dcv(F), v, Prec<T>::invd(F),
               (T)s.jacobi_damp, (T*)F.mg_rhs, (T*)F.mg_tmp, di);
    std::swap(F.mg_sol, F.mg_tmp);
  } else {
    CDG_LAUNCH_PDL(ctx, k_mg_init<T>, vec_grid(ctx, F.ndof), 256, 0, F.ndof, F.nactive, v,
               (T*)F.mg_rhs, (T*)F.mg_sol, di);
  }
  // the FP64 result of the last finest-level smoothing step goes to z directly
  // (CSR smoother; the FP64 sliced smoother keeps the separate conversion)
  bool z_written = false;
  std::vector<int> rec(nl, s.multigrid_cycle_type == 0 ? 1 : 2), seq;
  rec[nl - 1] = 1;
  seq.push_back(kDummy);
  fill_cycle(seq, rec, nl - 1, nl, s.multigrid_cycle_type);
  const T damp = (T)s.jacobi_damp;
  const T cdamp = (T)s.multigrid_correction_damp_factor;
  for (int m = 0; m < nl; ++m) lv(m).mg_visited = false;
  int level = nl - 1;
  if (nl == 1) {
    CDG_TRY(coarse_solve<T>(ctx, F, s));
  } else {
    for (size_t step = 1; step < seq.size() && level >= 0; ++step) {
      DevLevel& L = lv(level);
      if (level == 0) {
        CDG_TRY(coarse_solve<T>(ctx, L, s));
        CDG_TRY(prolong_correct<T>(ctx, lv(level + 1), L, cdamp));
        level += 1;
        continue;
      }
      const bool from_below = seq[step - 1] == kUp;
      const int dir = seq[step];
      if (from_below) {
        const bool hand_over = level == nl - 1 && dir == kEnd && !Prec<T>::has_sell(L) &&
                               s.multigrid_n_post_smooth > 0;
        for (int i = 0; i < s.multigrid_n_post_smooth; ++i) {
          if (hand_over && i + 1 == s.multigrid_n_post_smooth) {
            CDG_TRY(smooth_out<T>(ctx, L, Prec<T>::val(L), (const T*)L.mg_sol,
                                  (const T*)L.mg_rhs, Prec<T>::invd(L), damp, (T*)L.mg_tmp, z,
                                  di, zcur));
            std::swap(L.mg_sol, L.mg_tmp);
            z_written = true;
          } else {
            CDG_TRY(smooth<T>(ctx, L, damp));
          }
        }
      }
      if (dir == kDown) {
        for (int i = 0; i < s.multigrid_n_pre_smooth; ++i) {
          // the start iterate is zero (finest: Dirichlet values) unless the
          // level was smoothed since its solution was last reset (W, F cycles)
          if (i == 0 && level == nl - 1 && fused_start && !L.mg_visited)
            continue;   // done by k_first_smooth_init
          if (i == 0 && !L.mg_visited)
            CDG_TRY(first_smooth<T>(ctx, L, damp, level == nl - 1));
          else
            CDG_TRY(smooth<T>(ctx, L, damp));
        }
        L.mg_visited = true;
        CDG_TRY(defect<T>(ctx, L));
        DevLevel& C = lv(level - 1);
        // the coarse solution starts from zero; a first smoothing step or the
        // direct coarse solve overwrites it without reading it
        const bool coarsest = level - 1 == 0;
        const bool read_start = coarsest ? s.multigrid_smoother_coarse != 0
                                         : s.multigrid_n_pre_smooth == 0;
        if (read_start)
          CDG_CUDA(cudaMemsetAsync(C.mg_sol, 0, (size_t)C.ndof * sizeof(T), ctx->stream));
        C.mg_visited = false;   // zero start iterate again: shortcut valid
        CDG_TRY(restrict_defect<T>(ctx, L, C));
        level -= 1;
      } else if (dir == kUp) {
        CDG_TRY(prolong_correct<T>(ctx, lv(level + 1), L, cdamp));
        level += 1;
      } else {
        break;
      }
    }
  }
  if (!z_written)
    CDG_LAUNCH_PDL(ctx, k_to_double<T>, vec_grid(ctx, F.ndof), 256, 0, F.ndof, (const T*)F.mg_sol, z,
               di, zcur);
  return CDG_OK;
}

int ensure_mg_vectors(cdg_context* ctx, DevLevel& L, int elem) {
  if (L.mg_elem == elem) return CDG_OK;
  L.realloc_count++;
  void** bufs[4] = {&L.mg_rhs, &L.mg_sol, &L.mg_tmp, &L.mg_def};
  for (void** b : bufs) {
    if (*b) cudaFree(*b);
    *b = nullptr;
    CDG_CUDA(cudaMalloc(b, (size_t)std::max(L.ndof, 1) * elem));
    CDG_CUDA(cudaMemsetAsync(*b, 0, (size_t)std::max(L.ndof, 1) * elem, ctx->stream));
  }
  L.mg_elem = elem;
  return CDG_OK;
}

// y = A x with the FP32 multigrid operator of a level (identity on
// non-active rows): variant 0 the CSR kernel, 1 the matrix-free kernel
int apply32(cdg_context* ctx, const DevLevel& L, int variant, const float* x, float* y) {
  if (variant >= 1)
    return mf_apply(ctx, L, 0, x, nullptr, nullptr, 0.f, y, nullptr, nullptr, nullptr,
                    variant == 3 ? kMfStencil : (variant == 2 ? kMfTwoKernel : kMfOneLaunch));
  return spmv_t<float, 0>(ctx, L, L.val32, x, (const float*)nullptr, (const float*)nullptr, 0.f,
                          y);
}

int smooth32_once(cdg_context* ctx, DevLevel& L, float damp) {
  CDG_TRY(ensure_mg_vectors(ctx, L, (int)sizeof(float)));
  return smooth<float>(ctx, L, damp);
}

int defect32_once(cdg_context* ctx, DevLevel& L) {
  CDG_TRY(ensure_mg_vectors(ctx, L, (int)sizeof(float)));
  return defect<float>(ctx, L);
}

// per-level value of an environment override: one value for every level, or
// one per level from the finest ("8,4,4"; digits without commas for 0/1
// switches, "100"); -1 when unset
static int env_level(const char* name, int level) {
  const char* e = getenv(name);
  if (!e || !*e) return -1;
  if (!strchr(e, ',')) {
    const size_t len = strlen(e);
    if (len > 1 && (e[0] == '0' || e[0] == '1') && strspn(e, "01") == len)
      return level < (int)len ? e[level] - '0' : 0;
    return atoi(e);
  }
  const char* q = e;
  for (int l = 0; l < level && q; ++l) {
    q = strchr(q, ',');
    if (q) ++q;
  }
  return q && *q ? atoi(q) : -1;
}

// Per-level kernel schedule of the FP32 multigrid, chosen once per level by
// timing one smoothing step of each candidate (CUDA events on the context
// stream, the level's own vectors, 3 warm-up + 10 timed steps):
//   * CSR: lanes per row 2 / 4 / 8 / 16 (those with 8 * lanes >= a quarter of
//     the mean row length);
//   * matrix-free (Q2 hexahedra): grid of one cell per warp, or 4 / 8 blocks
//     per SM walking the cells;
//   * on a uniform lattice with Dirichlet data on the whole boundary, the
//     stencil sweep with 8 or 4 lattice points per thread against the best
//     of the above;
// and the faster of the best CSR and the best matrix-free step.  The grid
// size and, for a given lane count, the loop unrolling do not change any
// result; the lane count and the kernel kind change FP32 rounding only.
// Environment overrides (a profiler's per-launch overhead distorts timing):
// CDG_MATFREE (0/1), CDG_TPR32 (lanes), CDG_MF_CAP (blocks per SM),
// CDG_MF_MINB (4/5/6), CDG_MF_STENCIL (0, or 4/8 points per thread).
static int tune_level(cdg_context* ctx, cdg_problem* p, DevLevel& L, int level) {
  if (L.tuned) return CDG_OK;
  L.tuned = 1;
  p->alloc_gen++;   // the captured iteration graph holds the kernels of the old choice
  const char* off = getenv("CDG_TUNE");
  if (off && off[0] == '0') {   // untuned defaults: CSR, lanes by mean row length
    L.mf_mode = 0;
    return CDG_OK;
  }
  cudaEvent_t e0, e1;
  CDG_CUDA(cudaEventCreate(&e0));
  CDG_CUDA(cudaEventCreate(&e1));
  int rc = CDG_OK;
  auto time_step = [&](float* ms) {
    for (int r = 0; r < 3 && rc == CDG_OK; ++r) rc = smooth<float>(ctx, L, 0.8f);
    if (rc != CDG_OK) return;
    cudaEventRecord(e0, ctx->stream);
    for (int r = 0; r < 10 && rc == CDG_OK; ++r) rc = smooth<float>(ctx, L, 0.8f);
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms, e0, e1);
    *ms /= 10;
  };
  const int mf_env = env_level("CDG_MATFREE", level);
  const int tpr_env = env_level("CDG_TPR32", level);
  const int cap_env = env_level("CDG_MF_CAP", level);
  // CSR lanes per row (not for the opt-in staged kernel, which has its own)
  L.mf_mode = 0;
  if (tpr_env == 2 || tpr_env == 4 || tpr_env == 8 || tpr_env == 16) {
    L.tpr32 = tpr_env;
  } else if (mf_env != 1 && !L.bulk_nchunks) {
    const double avg = L.ndof ? (double)L.nnz / L.ndof : 1.0;
    float best = 1e30f;
    int bt = L.rows_per_warp_hint;
    for (int t : {2, 4, 8, 16}) {
      if (8.0 * t < avg / 4 || (t == 2 && avg > 32)) continue;
      L.tpr32 = t;
      float ms = 0.f;
      time_step(&ms);
      if (rc != CDG_OK) break;
      if (ms < best) {
        best = ms;
        bt = t;
      }
    }
    L.tpr32 = bt;
    L.tuned_ms[0] = best;
  }
  // matrix-free grid, then the faster kind
  L.st_zt = 0;
  const int st_env = env_level("CDG_MF_STENCIL", level);
  const bool lattice = L.mf_uniform && L.st_dims[0] > 0;
  if (rc == CDG_OK && L.mf_valid && mf_env != 0) {
    L.mf_mode = 1;
    if (lattice && (st_env == 4 || st_env == 8)) {
      L.st_zt = st_env;
      L.mf_blocks_per_sm = -100 - st_env;
      time_step(&L.tuned_ms[1]);
    } else if (L.mf_uniform && L.mf_ntiles > 0) {
      // the one-launch sweep has one block per row tile; its register budget
      // (4, 5 or 6 resident blocks per SM) is timed, reported as -blocks
      const int mb_env = env_level("CDG_MF_MINB", level);
      if (mb_env >= 4 && mb_env <= 6) {
        L.mf_fused_minb = mb_env;
        time_step(&L.tuned_ms[1]);
      } else {
        float best = 1e30f;
        int bm = 4;
        for (int mb : {4, 5, 6}) {
          L.mf_fused_minb = mb;
          float ms = 0.f;
          time_step(&ms);
          if (rc != CDG_OK) break;
          if (ms < best) {
            best = ms;
            bm = mb;
          }
        }
        L.mf_fused_minb = bm;
        L.tuned_ms[1] = best;
      }
      L.mf_blocks_per_sm = -L.mf_fused_minb;
    } else if (cap_env >= 0) {
      L.mf_blocks_per_sm = cap_env;
      time_step(&L.tuned_ms[1]);
    } else {
      float best = 1e30f;
      int bc = 0;
      for (int cap : {0, 4, 8}) {
        L.mf_blocks_per_sm = cap;
        float ms = 0.f;
        time_step(&ms);
        if (rc != CDG_OK) break;
        if (ms < best) {
          best = ms;
          bc = cap;
        }
      }
      L.mf_blocks_per_sm = bc;
      L.tuned_ms[1] = best;
    }
    // the stencil sweep (4 or 8 lattice points per thread along z) against
    // the best tile or cell sweep
    if (rc == CDG_OK && lattice && st_env != 0 && L.st_zt == 0) {
      float best = 1e30f;
      int bz = 0;
      for (int zt : {8, 4}) {
        L.st_zt = zt;
        float ms = 0.f;
        time_step(&ms);
        if (rc != CDG_OK) break;
        if (ms < best) {
          best = ms;
          bz = zt;
        }
      }
      L.st_zt = 0;
      if (rc == CDG_OK && best < L.tuned_ms[1]) {
        L.st_zt = bz;
        L.tuned_ms[1] = best;
        L.mf_blocks_per_sm = -100 - bz;
      }
    }
    if (mf_env != 1 && !(L.tuned_ms[1] < L.tuned_ms[0])) {
      L.mf_mode = 0;
      L.mf_blocks_per_sm = 0;   // unused by the CSR kernel
      L.st_zt = 0;
    }
  }
  if (!L.mf_valid) L.mf_mode = -1;   // no matrix-free operator on this level
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

int prepare_solver(cdg_context* ctx, cdg_problem* p, const cdg_solver_params& s) {
  CDG_TRY(check_device_error(ctx));
  if (s.preconditioner != 0) {
    // extract_diagonal_entries (Iteration_jacobi.C:14-28) rejects zero
    // diagonals; the assembly recorded them per problem
    int zd = 0;
    CDG_CUDA(cudaMemcpyAsync(&zd, p->d_zero_diag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CDG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (zd) {
      set_error("zero entry on the diagonal using Jacobi solver/preconditioner");
      return CDG_ERR_ZERO_DIAG;
    }
  }
  if (s.preconditioner != 2) return CDG_OK;
  const int nl = s.multigrid_n_levels;
  if (nl < 1 || nl > (int)p->lev.size()) {
    set_error("multigrid_n_levels=%d but the problem has %d levels", nl, (int)p->lev.size());
    return CDG_ERR_ARG;
  }
  for (int k = 0; k + 1 < nl; ++k)
    CDG_TRY(lattice_transfer_setup(ctx, p->lev[k], p->lev[k + 1]));
  const int elem = s.precision == 1 ? (int)sizeof(float) : (int)sizeof(double);
  // FP64 values of FP32-only levels where this solve needs them: every level
  // of an FP64 multigrid, the coarse inverse's level otherwise
  for (int k = 0; k < nl; ++k)
    if (s.precision == 0 || k == nl - 1) CDG_TRY(ensure_fp64(ctx, p, p->lev[k]));
  for (int k = 0; k < nl; ++k) CDG_TRY(ensure_mg_vectors(ctx, p->lev[k], elem));
  if (s.precision == 1)
    for (int k = 0; k + 1 < nl; ++k) CDG_TRY(tune_level(ctx, p, p->lev[k], k));

  if (s.multigrid_smoother_coarse == 0) {
    CDG_TRY(coarse_inverse(ctx, p->lev[nl - 1]));
    CDG_TRY(check_device_error(ctx));
  }
  return CDG_OK;
}

// z = B v (Iteration_jacobi / Iteration_multigrid apply, or a copy).  di !=
// null: v and z are the blocks V and Z, the vector index *di is read on the
// device (graph-captured FGMRES loop) and zcur receives a copy of z_i
int precondition(cdg_context* ctx, cdg_problem* p, const cdg_solver_params& s, const double* v,
                 double* z, const int* di, double* zcur) {
  DevLevel& F = p->lev[0];
  if (s.preconditioner == 1) {
    CDG_LAUNCH_PDL(ctx, k_mul, vec_grid(ctx, F.ndof), 256, 0, F.ndof, v, F.invdiag64, z, di, zcur);
    return CDG_OK;
  }
  if (s.preconditioner == 2) {
    if (s.precision == 1) return mg_cycle<float>(ctx, p, s, v, z, di, zcur);
    return mg_cycle<double>(ctx, p, s, v, z, di, zcur);
  }
  if (di) {
    CDG_LAUNCH_PDL(ctx, k_copy_idx, vec_grid(ctx, F.ndof), 256, 0, F.ndof, v, z, di, zcur);
    return CDG_OK;
  }
  CDG_CUDA(cudaMemcpyAsync(z, v, (size_t)F.ndof * sizeof(double), cudaMemcpyDeviceToDevice,
                           ctx->stream));
  return CDG_OK;
}

int prolongate64(cdg_context* ctx, const DevLevel& F, const DevLevel& C, const double* xc,
                 double* xf, int add_actives_only, double damp) {
  if (F.lt_state == 1) {
    const long nf = (long)F.st_dims[0] * F.st_dims[1] * F.st_dims[2];
    CDG_LAUNCH_PDL(ctx, k_lat_prolong<double>, (int)((nf + 255) / 256), 256, 0, lat_map(F, C),
                   F.nactive, F.st_map, C.st_map, xc, xf, damp, add_actives_only);
    return CDG_OK;
  }
  CDG_LAUNCH_PDL(ctx, (k_prolong<double, 2>), grid_for<int>((long)F.ndof * 2, 256), 256, 0, F.ndof,
             F.nactive, F.P_rp, F.P_col, F.P_val, xc, xf, damp, add_actives_only);
  return CDG_OK;
}

int restrict64(cdg_context* ctx, const DevLevel& F, const DevLevel& C, const double* df,
               double* rc) {
  if (F.lt_state == 1) {
    const long nc = (long)C.st_dims[0] * C.st_dims[1] * C.st_dims[2];
    CDG_LAUNCH_PDL(ctx, k_lat_restrict<double>, (int)((nc * kLatLanes + 255) / 256), 256, 0,
                   lat_map(F, C),
                   C.nactive, F.st_map, C.st_map, df, rc, 0);
    return CDG_OK;
  }
  CDG_LAUNCH_PDL(ctx, (k_restrict<double, 8>), grid_for<int>((long)C.ndof * 8, 256), 256, 0,
             C.ndof, C.nactive, F.R_rp, F.R_col, F.R_val, df, rc, 0);
  return CDG_OK;
}

// ---------------------------------------------------------------------------
// FGMRES(m): Hessenberg column i stored at H[i*(m+1) + k] = H(k, i)
// ---------------------------------------------------------------------------
__global__ void k_givens(int i, int m, double* H, double* cs, double* sn, double* s,
                         double* resid) {
  pdl_enter();
  givens_column(i, H + (size_t)i * (m + 1), cs, sn, s, resid);
}

// s = (beta, 0, ..., 0)
__global__ void k_init_s(int m, const double* beta, double* s) {
  pdl_enter();
  for (int i = threadIdx.x; i <= m; i += blockDim.x) s[i] = i == 0 ? *beta : 0.0;
}

// Hessenberg back substitution (Utilities_gmres.C:90-108)
// y = R^{-1} s for the rotated Hessenberg columns 0..k (Utilities_gmres.C
// Update): one block, columns and s staged in shared memory by one coalesced
// pass, then the column sweep -- y_i /= R(i,i), y_j -= R(j,i) y_i for j < i in
// parallel -- in the serial order of every y_j
constexpr int kBacksolveThreads = 128;
__global__ void __launch_bounds__(kBacksolveThreads)
k_backsolve(int k, int m, const double* __restrict__ H, const double* __restrict__ s,
            double* __restrict__ y) {
  pdl_enter();
  extern __shared__ double bs[];
  double* ys = bs;               // k + 1
  double* hs = bs + (k + 1);     // column i at hs[i * (k + 1)], rows 0..i
  const int n1 = k + 1;
  for (int t = threadIdx.x; t < n1 * n1; t += blockDim.x) {
    const int i = t / n1, j = t - i * n1;
    if (j <= i) hs[t] = H[(size_t)i * (m + 1) + j];
  }
  for (int j = threadIdx.x; j < n1; j += blockDim.x) ys[j] = s[j];
  __syncthreads();
  for (int i = k; i >= 0; --i) {
    if (threadIdx.x == 0) ys[i] /= hs[i * n1 + i];
    __syncthreads();
    const double yi = ys[i];
    for (int j = threadIdx.x; j < i; j += blockDim.x) ys[j] -= hs[i * n1 + j] * yi;
    __syncthreads();
  }
  for (int j = threadIdx.x; j < n1; j += blockDim.x) y[j] = ys[j];
}

static int launch_backsolve(cdg_context* ctx, int k, int m, const double* H, const double* s,
                            double* y) {
  const size_t smem = (size_t)(k + 1) * (k + 2) * sizeof(double);
  // restarts up to 120: at most 120 * 121 doubles (the attribute is per device)
  CDG_CUDA(cudaFuncSetAttribute(k_backsolve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(120 * 121 * sizeof(double))));
  CDG_LAUNCH_PDL(ctx, k_backsolve, 1, kBacksolveThreads, smem, k, m, H, s, y);
  return CDG_OK;
}

// x += sum_j y_j z_j (accumulated from zero in order j = 0..k, then added)
__global__ void k_update(int n, int k, const double* __restrict__ Z, const double* __restrict__ y,
                         double* __restrict__ x) {
  pdl_enter();
  __shared__ double ys[128];
  for (int j = threadIdx.x; j <= k; j += blockDim.x) ys[j] = y[j];
  __syncthreads();
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j <= k; ++j) acc += ys[j] * Z[(size_t)j * n + t];
    x[t] += acc;
  }
}

void free_gmres(GmresState& g) {
  double* ptrs[] = {g.V, g.Z, g.w, g.H, g.cs, g.sn, g.s, g.y, g.scal, g.zcur, g.part};
  for (double* q : ptrs)
    if (q) cudaFree(q);
  if (g.dstate) cudaFree(g.dstate);
  if (g.exec) cudaGraphExecDestroy(g.exec);
  if (g.graph) cudaGraphDestroy(g.graph);
  g = GmresState();
}

static int ensure_gmres(cdg_problem* p, int n, int m) {
  GmresState& g = p->gm;
  if (g.n == n && g.m == m && g.V) return CDG_OK;
  free_gmres(g);
  p->alloc_gen++;
  g.n = n;
  g.m = m;
  CDG_CUDA(cudaMalloc(&g.zcur, (size_t)n * sizeof(double)));
  CDG_CUDA(cudaMalloc(&g.dstate, 4 * sizeof(int)));
  CDG_CUDA(cudaMalloc(&g.V, (size_t)(m + 1) * n * sizeof(double)));
  CDG_CUDA(cudaMalloc(&g.Z, (size_t)m * n * sizeof(double)));
  CDG_CUDA(cudaMalloc(&g.w, (size_t)n * sizeof(double)));
  CDG_CUDA(cudaMalloc(&g.H, (size_t)(m + 1) * (m + 1) * sizeof(double)));
  CDG_CUDA(cudaMalloc(&g.cs, (size_t)(m + 1) * sizeof(double)));
  CDG_CUDA(cudaMalloc(&g.sn, (size_t)(m + 1) * sizeof(double)));
  CDG_CUDA(cudaMalloc(&g.s, (size_t)(m + 1) * sizeof(double)));
  CDG_CUDA(cudaMalloc(&g.y, (size_t)(m + 1) * sizeof(double)));
  CDG_CUDA(cudaMalloc(&g.scal, 8 * sizeof(double)));
  CDG_CUDA(cudaMemset(g.H, 0, (size_t)(m + 1) * (m + 1) * sizeof(double)));
  return CDG_OK;
}

// what the batched solver needs of a problem, without synchronising: FP64
// values of the levels it reads in FP64 (finest, coarsest), FP32 multigrid
// vectors, Krylov buffers, and the coarse inverse -- formed here only for a
// coarse block above kBatchSmemCoarse rows (*inline_coarse = 0); smaller
// ones are inverted by the batch's own coarse launch (the zero-diagonal test
// then runs in the solve kernel, on the problem's flag)
int batch_prepare(cdg_context* ctx, cdg_problem* p, const cdg_solver_params& s,
                  int* inline_coarse) {
  const int nl = s.multigrid_n_levels;
  if (nl < 2 || nl > (int)p->lev.size()) {
    set_error("multigrid_n_levels=%d but the problem has %d levels", nl, (int)p->lev.size());
    return CDG_ERR_ARG;
  }
  CDG_TRY(ensure_fp64(ctx, p, p->lev[0]));
  CDG_TRY(ensure_fp64(ctx, p, p->lev[nl - 1]));
  for (int k = 0; k < nl; ++k) CDG_TRY(ensure_mg_vectors(ctx, p->lev[k], (int)sizeof(float)));
  CDG_TRY(ensure_gmres(p, p->lev[0].ndof, s.gmres_restart));
  DevLevel& C = p->lev[nl - 1];
  const int na = C.nactive;
  C.coarse_na = na;
  if (na <= kBatchSmemCoarse) {
    if (!C.coarse_inv && na > 0)
      CDG_CUDA(cudaMalloc(&C.coarse_inv, (size_t)na * na * sizeof(double)));
    *inline_coarse = 1;
    return CDG_OK;
  }
  *inline_coarse = 0;
  CDG_TRY(coarse_inverse(ctx, C));
  return check_device_error(ctx);
}

struct LoopInfo {
  double initial = 0, previous = 0;
};

// IterativeMethod::converged: 0 continue, 1 stop, 2 diverged
static int converged(const cdg_solver_params& s, LoopInfo& li, double res, int it) {
  if (it == 0) {
    li.initial = res;
    li.previous = res;
  }
  bool small = res < s.residual_tolerance;
  bool red = res < s.residual_reduction * li.initial;
  bool enough = it >= s.min_n_iterations;
  bool stag = res > 1e10 * li.previous;
  bool div = res > s.divergence_factor * li.initial;
  bool conv = (small || red || stag || div) && enough;
  if (it == s.max_n_iterations) conv = true;
  li.previous = res;
  if (div) return 2;
  return conv ? 1 : 0;
}

static int read_scalar(cdg_context* ctx, const double* d, double* h) {
  CDG_CUDA(cudaMemcpyAsync(ctx->h_pinned, d, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  *h = ctx->h_pinned[0];
  return CDG_OK;
}

// ---------------------------------------------------------------------------
// device-resident FGMRES: one iteration is captured once as the body of a
// WHILE conditional graph node; the convergence test (IterativeMethod::
// converged) runs on the device and ends the loop, so the host waits once
// per restart cycle instead of once per iteration
// ---------------------------------------------------------------------------
// st: [0] column i, [1] iteration j, [2] flag (0 run, 1 converged,
// 2 diverged, 3 end of the restart cycle)
__global__ void k_fgmres_start(ConvParams c, int* st, const double* beta, double* li) {
  pdl_enter();
  st[0] = 0;
  st[1] = 1;
  st[2] = conv_test(c, li, *beta, 0);
}

__global__ void k_fgmres_iter_check(ConvParams c, int* st, const double* resid, double* li,
                                    cudaGraphConditionalHandle h) {
  pdl_enter();
  const int i = st[0], j = st[1];
  const int cv = conv_test(c, li, *resid, j);
  unsigned cont = 0;
  if (cv == 2) {
    st[2] = 2;
  } else if (cv == 1) {
    st[2] = 1;
  } else if (i + 1 == c.m) {
    st[2] = 3;
    st[1] = j + 1;
  } else {
    st[0] = i + 1;
    st[1] = j + 1;
    cont = 1;
  }
  cudaGraphSetConditional(h, cont);
}

// after a full cycle: the test with the last estimate at iteration j
__global__ void k_fgmres_restart_check(ConvParams c, int* st, const double* resid, double* li) {
  pdl_enter();
  st[2] = conv_test(c, li, *resid, st[1]);
  st[0] = 0;
}

static ConvParams conv_params(const cdg_solver_params& s) {
  return ConvParams{s.residual_tolerance, s.residual_reduction, s.divergence_factor,
                    s.min_n_iterations, s.max_n_iterations, s.gmres_restart};
}

// one FGMRES iteration (classical Gram-Schmidt), column index on the device
static int iteration_body(cdg_context* ctx, cdg_problem* p, const cdg_solver_params& s,
                          cudaGraphConditionalHandle h) {
  DevLevel& L = p->lev[0];
  GmresState& g = p->gm;
  const int n = L.ndof, m = s.gmres_restart;
  int* di = g.dstate;
  CDG_TRY(precondition(ctx, p, s, g.V, g.Z, di, g.zcur));
  CDG_TRY(spmv_apply64(ctx, L, g.zcur, g.w));
  if (g.coop) {
    CDG_TRY(cgs_coop(ctx, g, n, m, 0, di));
  } else {
    const int mg = std::min(red_grid(ctx, n), ctx->num_sms * 2);
    for (int k0 = 0; k0 < m; k0 += 32)
      CDG_LAUNCH_PDL(ctx, k_multidot<256>, mg, 256, 0, n, g.w, g.V, k0, 0, ctx->d_red,
                 ctx->d_cnt + 1, g.H, di, m + 1);
    CDG_LAUNCH_PDL(ctx, k_cgs_update, red_grid(ctx, n), 256, 0, n, g.w, g.V, 0, g.H, ctx->d_red,
               ctx->d_cnt, g.cs, g.sn, g.s, g.scal + 0, g.scal + 2, di, m + 1);
    CDG_LAUNCH_PDL(ctx, k_scale_inv, vec_grid(ctx, n), 256, 0, n, g.w, g.scal + 2, g.V,
                   ctx->d_err, di);
  }
  CDG_LAUNCH_PDL(ctx, k_fgmres_iter_check, 1, 1, 0, conv_params(s), g.dstate, g.scal + 0,
             g.scal + 4, h);
  return CDG_OK;
}

static unsigned long long graph_generation(const cdg_problem* p) {
  // the captured kernels use the context's stream and scratch: a problem
  // moved to another context is recaptured
  unsigned long long gen = p->alloc_gen * 1000003ull + (unsigned long long)(uintptr_t)p->ctx;
  for (const DevLevel& L : p->lev)
    gen = gen * 1000003ull + (unsigned long long)L.realloc_count * 7919ull +
          (unsigned long long)(uintptr_t)L.coarse_inv +
          (unsigned long long)(L.mf_valid * 4 + L.mf_uniform * 2 + (L.mf_mode == 1 ? 1 : 0)) *
              104729ull;
  return gen;
}

static int capture_iteration_graph(cdg_context* ctx, cdg_problem* p, const cdg_solver_params& s,
                                   unsigned long long gen, int coop);

// the captured loop with the cooperative Gram-Schmidt step where it applies;
// a runtime that cannot capture or instantiate a cooperative launch inside
// the conditional node gets the three kernels (remembered per context)
static int ensure_iteration_graph(cdg_context* ctx, cdg_problem* p, const cdg_solver_params& s) {
  GmresState& g = p->gm;
  const unsigned long long gen = graph_generation(p);
  const int coop =
      !ctx->coop_graph_failed && cgs_coop_on(ctx, p->lev[0].ndof, s.gmres_restart) ? 1 : 0;
  if (g.exec && g.key_gen == gen && g.coop == coop && std::memcmp(&g.key, &s, sizeof(s)) == 0)
    return CDG_OK;
  const int rc = capture_iteration_graph(ctx, p, s, gen, coop);
  if (rc == CDG_OK || !coop) return rc;
  cudaGetLastError();
  ctx->coop_graph_failed = 1;
  return capture_iteration_graph(ctx, p, s, gen, 0);
}

static int capture_iteration_graph(cdg_context* ctx, cdg_problem* p, const cdg_solver_params& s,
                                   unsigned long long gen, int coop) {
  GmresState& g = p->gm;
  g.coop = coop;
  if (g.exec) cudaGraphExecDestroy(g.exec);
  if (g.graph) cudaGraphDestroy(g.graph);
  g.exec = nullptr;
  g.graph = nullptr;
  cudaGraph_t graph = nullptr;
  CDG_CUDA(cudaGraphCreate(&graph, 0));
  cudaGraphConditionalHandle h;
  cudaGraphNodeParams np = {};
  cudaGraphNode_t node;
  cudaError_t e = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault);
  if (e == cudaSuccess) {
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np);
  }
  if (e == cudaSuccess)
    e = cudaStreamBeginCaptureToGraph(ctx->stream, np.conditional.phGraph_out[0], nullptr,
                                      nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    set_error("graph setup: %s", cudaGetErrorString(e));
    return CDG_ERR_CUDA;
  }
  const long long l0 = ctx->launches;
  int rc = iteration_body(ctx, p, s, h);
  cudaGraph_t body = nullptr;
  e = cudaStreamEndCapture(ctx->stream, &body);
  g.body_launches = ctx->launches - l0;
  ctx->launches = l0;   // captured, not launched
  if (rc != CDG_OK || e != cudaSuccess) {
    cudaGetLastError();
    cudaGraphDestroy(graph);
    if (rc == CDG_OK) set_error("graph capture: %s", cudaGetErrorString(e));
    return rc != CDG_OK ? rc : CDG_ERR_CUDA;
  }
  e = cudaGraphInstantiate(&g.exec, graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    g.exec = nullptr;
    set_error("graph instantiate: %s", cudaGetErrorString(e));
    return CDG_ERR_CUDA;
  }
  g.graph = graph;
  g.key = s;
  g.key_gen = gen;
  return CDG_OK;
}

static int read_state(cdg_context* ctx, const GmresState& g, int* st4, double* resid) {
  CDG_CUDA(cudaMemcpyAsync(st4, g.dstate, 4 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CDG_CUDA(cudaMemcpyAsync(ctx->h_pinned, g.scal, sizeof(double), cudaMemcpyDeviceToHost,
                           ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  *resid = ctx->h_pinned[0];
  return CDG_OK;
}

// ---------------------------------------------------------------------------
// One FGMRES restart cycle with the Jacobi preconditioner as a single
// cooperative kernel, for small systems: the iteration of iteration_body
// (z_i = D^-1 v_i, w = A z_i, classical Gram-Schmidt, norm, Givens, test,
// v_{i+1} = w / h_{i+1,i}) with three grid-wide barriers where the graph runs
// seven dependent kernels.  A thread owns up to kCycleRows rows and keeps
// their w in registers from the operator to the normalisation (one row per
// thread measured best on GB300: 64^2 Q1, 387 iterations, 84.9 solves/s
// against 68.8 with two rows, 57.2 with four and 58.9 for the graph; 64-thread
// blocks over 67 SMs instead of 17 gave 69.3 against 91.9: the barriers, not
// the FP64 work, bound an iteration of this size).  The inner
// products of a block are reduced through shared memory (one warp per
// product); every block sums the blocks' partials in block order, so all
// blocks hold the same values, run the Givens step and the convergence test
// on their own copy of the rotations and take the same branch without a
// further barrier.  Block 0 writes the shared state (H, rotations, s, the
// residual and the loop state) for the back substitution on the host side.
// ---------------------------------------------------------------------------
constexpr int kCycleThreads = 256, kCycleRows = 1, kCycleMaxM = 64;
constexpr int kCycleMaxRows = 65536;   // larger systems keep the graph-captured kernels

__global__ void __launch_bounds__(kCycleThreads)
k_fgmres_cycle_jacobi(int n, int nactive, int m, ConvParams cp, const int* __restrict__ rp,
                      const int* __restrict__ col, const double* __restrict__ val,
                      const double* __restrict__ invd, double* __restrict__ V,
                      double* __restrict__ Z, double* __restrict__ H, double* __restrict__ cs,
                      double* __restrict__ sn, double* __restrict__ s, double* __restrict__ scal,
                      int* __restrict__ st, double* __restrict__ part, int* err) {
  pdl_enter();
  cgrp::grid_group grid = cgrp::this_grid();
  __shared__ double tr[8][kCycleThreads + 1];
  __shared__ double hc[kCycleMaxM + 2];
  __shared__ double lcs[kCycleMaxM + 1], lsn[kCycleMaxM + 1], ls[kCycleMaxM + 2];
  __shared__ double lli[2], red[kCycleThreads / 32], nrm_s;
  __shared__ int dec[4];   // next i, next j, flag, continue
  const int nb = gridDim.x, wp = threadIdx.x >> 5, l = threadIdx.x & 31;
  const long nthr = (long)nb * kCycleThreads;
  const long tid = blockIdx.x * (long)kCycleThreads + threadIdx.x;
  double* part2 = part + (size_t)nb * (m + 1);   // norm partials
  for (int k = threadIdx.x; k <= m; k += kCycleThreads) {
    ls[k] = s[k];
    lcs[k] = cs[k];
    lsn[k] = sn[k];
  }
  if (threadIdx.x == 0) {
    lli[0] = scal[4];
    lli[1] = scal[5];
  }
  int i = st[0], j = st[1];
  __syncthreads();
  for (;;) {
    // z_i = D^-1 v_i on the own rows (Iteration_jacobi::apply)
#pragma unroll
    for (int q = 0; q < kCycleRows; ++q) {
      const long r = tid + q * nthr;
      if (r < n) Z[(size_t)i * n + r] = V[(size_t)i * n + r] * invd[r];
    }
    grid.sync();
    // w = A z_i (non-active rows: identity)
    double wv[kCycleRows];
#pragma unroll
    for (int q = 0; q < kCycleRows; ++q) {
      const long r = tid + q * nthr;
      double a = 0.0;
      if (r < nactive) {
        for (int k = rp[r]; k < rp[r + 1]; ++k) a = fma(val[k], Z[(size_t)i * n + col[k]], a);
      } else if (r < n) {
        a = Z[(size_t)i * n + r];
      }
      wv[q] = a;
    }
    // block partials of (w, v_k), k <= i, eight products per pass
    for (int k0 = 0; k0 <= i; k0 += 8) {
      double a[8];
#pragma unroll
      for (int kk = 0; kk < 8; ++kk) a[kk] = 0.0;
#pragma unroll
      for (int q = 0; q < kCycleRows; ++q) {
        const long r = tid + q * nthr;
        if (r < n)
#pragma unroll
          for (int kk = 0; kk < 8; ++kk)
            if (k0 + kk <= i) a[kk] = fma(wv[q], V[(size_t)(k0 + kk) * n + r], a[kk]);
      }
#pragma unroll
      for (int kk = 0; kk < 8; ++kk) tr[kk][threadIdx.x] = a[kk];
      __syncthreads();
      if (k0 + wp <= i) {
        double v = 0.0;
#pragma unroll
        for (int q = 0; q < kCycleThreads / 32; ++q) v += tr[wp][q * 32 + l];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (l == 0) part[(size_t)blockIdx.x * (m + 1) + k0 + wp] = v;
      }
      __syncthreads();
    }
    grid.sync();
    // every block: h_k = sum of the block partials in block order
    for (int k = threadIdx.x; k <= i; k += kCycleThreads) {
      double v = 0.0;
      for (int b = 0; b < nb; ++b) v += part[(size_t)b * (m + 1) + k];
      hc[k] = v;
    }
    __syncthreads();
    // w -= sum_k h_k v_k (k in order), norm partial
    double nn = 0.0;
#pragma unroll
    for (int q = 0; q < kCycleRows; ++q) {
      const long r = tid + q * nthr;
      if (r < n) {
        double w = wv[q];
        for (int k = 0; k <= i; ++k) w = fma(-hc[k], V[(size_t)k * n + r], w);
        wv[q] = w;
        nn = fma(w, w, nn);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nn += __shfl_xor_sync(0xffffffffu, nn, o);
    if (l == 0) red[wp] = nn;
    __syncthreads();
    if (threadIdx.x == 0) {
      double v = 0.0;
      for (int q = 0; q < kCycleThreads / 32; ++q) v += red[q];
      part2[blockIdx.x] = v;
    }
    grid.sync();
    // every block: the norm, Givens, the test (k_fgmres_iter_check)
    if (threadIdx.x == 0) {
      double v = 0.0;
      for (int b = 0; b < nb; ++b) v += part2[b];
      const double nrm = sqrt(v);
      nrm_s = nrm;
      hc[i + 1] = nrm;
      double resid = 0.0;
      givens_column(i, hc, lcs, lsn, ls, &resid);
      const int cv = conv_test(cp, lli, resid, j);
      int flag = 0, ni = i, nj = j, cont = 0;
      if (cv == 2) flag = 2;
      else if (cv == 1) flag = 1;
      else if (i + 1 == m) { flag = 3; nj = j + 1; }
      else { ni = i + 1; nj = j + 1; cont = 1; }
      if (nrm == 0.0) {   // H(i+1,i) == 0: unhappy breakdown (k_scale_inv)
        cont = 0;
        if (blockIdx.x == 0) atomicOr(err, kErrBreakdown);
      }
      dec[0] = ni; dec[1] = nj; dec[2] = flag; dec[3] = cont;
      if (blockIdx.x == 0) {
        for (int k = 0; k <= i + 1; ++k) H[(size_t)i * (m + 1) + k] = hc[k];
        cs[i] = lcs[i];
        sn[i] = lsn[i];
        s[i] = ls[i];
        s[i + 1] = ls[i + 1];
        scal[0] = resid;
        scal[2] = nrm;
        scal[4] = lli[0];
        scal[5] = lli[1];
        st[0] = ni;
        st[1] = nj;
        st[2] = flag;
      }
    }
    __syncthreads();
    const double nrm = nrm_s;
    if (nrm != 0.0) {
      const double f = 1.0 / nrm;
#pragma unroll
      for (int q = 0; q < kCycleRows; ++q) {
        const long r = tid + q * nthr;
        if (r < n) V[(size_t)(i + 1) * n + r] = wv[q] * f;
      }
    }
    if (!dec[3]) break;
    i = dec[0];
    j = dec[1];
    __syncthreads();
  }
}

constexpr int kGraphUnavailable = 1;   // internal: use the host loop

static int fgmres_graph(cdg_context* ctx, cdg_problem* p, const cdg_solver_params& s,
                        cdg_solve_stats* st) {
  DevLevel& L = p->lev[0];
  const int n = L.ndof, m = s.gmres_restart;
  GmresState& g = p->gm;
  double* x = L.sol;
  const double* b = L.rhs;
  double* beta_d = g.scal + 1;
  const int vg = vec_grid(ctx, n);
  const ConvParams cp = conv_params(s);
  // small Jacobi-preconditioned systems: one cooperative kernel per restart
  // cycle (CDG_FGMRES_CYCLE=0 keeps the graph)
  int cycle_blocks = 0;
  {
    const char* ce = std::getenv("CDG_FGMRES_CYCLE");
    const bool cycle_off = ce && ce[0] == '0';
    int coop = 0, per_sm = 0;
    if (!cycle_off && s.preconditioner == 1 && n <= kCycleMaxRows && m <= kCycleMaxM &&
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device) == cudaSuccess &&
        coop &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fgmres_cycle_jacobi,
                                                      kCycleThreads, 0) == cudaSuccess &&
        per_sm > 0) {
      const long per_block = (long)kCycleThreads * kCycleRows;
      const long need = (n + per_block - 1) / per_block;
      if (need <= (long)ctx->num_sms * per_sm) cycle_blocks = (int)std::max<long>(1, need);
    }
  }
  // a graph that cannot be built (capture rejected) falls back to the host
  // loop; one whose programmatic launch edges are rejected is built without
  if (!cycle_blocks) {
    int rc = ensure_iteration_graph(ctx, p, s);
    if (rc != CDG_OK && ctx->pdl) {
      cudaGetLastError();
      ctx->pdl = 0;
      rc = ensure_iteration_graph(ctx, p, s);
      ctx->pdl = 1;
    }
    if (rc != CDG_OK) {
      cudaGetLastError();
      return kGraphUnavailable;
    }
  }
  if (cycle_blocks && g.part == nullptr)
    CDG_CUDA(cudaMalloc(&g.part, ((size_t)ctx->num_sms * 8 * (kCycleMaxM + 2)) * sizeof(double)));
  // r = b - A x; beta = ||r||; the test at iteration 0
  CDG_TRY(residual64(ctx, L, b, x, g.w));
  CDG_TRY(dot64(ctx, n, g.w, nullptr, beta_d, 0));
  CDG_LAUNCH_PDL(ctx, k_fgmres_start, 1, 1, 0, cp, g.dstate, beta_d, g.scal + 4);
  int sv[4];
  double beta = 0;
  CDG_CUDA(cudaMemcpyAsync(sv, g.dstate, 4 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CDG_TRY(read_scalar(ctx, beta_d, &beta));
  st->initial_residual = beta;
  st->iterations = 0;
  st->residual = beta;
  if (sv[2] != 0) return CDG_OK;
  double resid = beta;
  for (;;) {
    CDG_LAUNCH_PDL(ctx, k_scale_inv, vg, 256, 0, n, g.w, beta_d, g.V, ctx->d_err,
                   (const int*)nullptr);
    CDG_LAUNCH_PDL(ctx, k_init_s, 1, 128, 0, m, beta_d, g.s);
    if (cycle_blocks) {
      const int* rp = L.row_ptr;
      const int* cl = L.col;
      const double* vl = L.val64;
      const double* di = L.invdiag64;
      int na = L.nactive, nn = n, mm = m;
      ConvParams cpp = cp;
      void* args[] = {(void*)&nn,   (void*)&na,   (void*)&mm,    (void*)&cpp,  (void*)&rp,
                      (void*)&cl,   (void*)&vl,   (void*)&di,    (void*)&g.V,  (void*)&g.Z,
                      (void*)&g.H,  (void*)&g.cs, (void*)&g.sn,  (void*)&g.s,  (void*)&g.scal,
                      (void*)&g.dstate, (void*)&g.part, (void*)&ctx->d_err};
      CDG_CUDA(cudaLaunchCooperativeKernel((const void*)k_fgmres_cycle_jacobi, dim3(cycle_blocks),
                                           dim3(kCycleThreads), args, 0, ctx->stream));
      ctx->launches++;
    } else {
      CDG_CUDA(cudaGraphLaunch(g.exec, ctx->stream));
    }
    CDG_TRY(read_state(ctx, g, sv, &resid));
    const int i = sv[0], j = sv[1], flag = sv[2];
    if (!cycle_blocks) ctx->launches += g.body_launches * (long long)(flag == 3 ? m : i + 1);
    CDG_TRY(check_device_error(ctx));
    if (flag == 2) {
      set_error("Execution of the code stopped because of solver divergence.");
      st->iterations = j;
      st->residual = resid;
      return CDG_ERR_DIVERGED;
    }
    if (flag == 1) {
      CDG_TRY(launch_backsolve(ctx, i, m, g.H, g.s, g.y));
      CDG_LAUNCH_PDL(ctx, k_update, vg, 256, 0, n, i, g.Z, g.y, x);
      st->iterations = j;
      st->residual = resid;
      return CDG_OK;
    }
    // end of the restart cycle: update x, new residual, test
    CDG_TRY(launch_backsolve(ctx, m - 1, m, g.H, g.s, g.y));
    CDG_LAUNCH_PDL(ctx, k_update, vg, 256, 0, n, m - 1, g.Z, g.y, x);
    CDG_TRY(residual64(ctx, L, b, x, g.w));
    CDG_TRY(dot64(ctx, n, g.w, nullptr, beta_d, 0));
    CDG_LAUNCH_PDL(ctx, k_fgmres_restart_check, 1, 1, 0, cp, g.dstate, g.scal + 0, g.scal + 4);
    CDG_TRY(read_state(ctx, g, sv, &resid));
    if (sv[2] == 2) {
      set_error("Execution of the code stopped because of solver divergence.");
      return CDG_ERR_DIVERGED;
    }
    if (sv[2] == 1 || sv[1] > s.max_n_iterations) {
      st->iterations = std::min(sv[1], s.max_n_iterations);
      st->residual = resid;
      return CDG_OK;
    }
  }
}

// Iteration_gmres::flexible_gmres on the finest level: x = lev[0].sol,
// b = lev[0].rhs
int fgmres(cdg_context* ctx, cdg_problem* p, const cdg_solver_params& s, cdg_solve_stats* st) {
  DevLevel& L = p->lev[0];
  const int n = L.ndof, m = s.gmres_restart;
  if (m < 1 || m > 120) { set_error("gmres_restart must be in [1, 120]"); return CDG_ERR_ARG; }
  CDG_TRY(ensure_gmres(p, n, m));
  // classical Gram-Schmidt with a preconditioner free of host reads: the
  // graph-captured loop (same kernels, same order).  CDG_FGMRES_GRAPH=0 in
  // the environment selects the host loop, whose kernels profilers list one
  // by one (kernels inside conditional graph nodes are not listed)
  static const bool graph_off = [] {
    const char* e = std::getenv("CDG_FGMRES_GRAPH");
    return e && e[0] == '0';
  }();
  if (!graph_off && s.gram_schmidt == 0 &&
      !(s.preconditioner == 2 && s.multigrid_smoother_coarse != 0)) {
    const int rc = fgmres_graph(ctx, p, s, st);
    if (rc != kGraphUnavailable) return rc;
  }
  GmresState& g = p->gm;
  double* x = L.sol;
  const double* b = L.rhs;
  double* beta_d = g.scal + 1;
  double* resid_d = g.scal + 0;
  LoopInfo li;
  // r = b - A x; beta = ||r||
  CDG_TRY(residual64(ctx, L, b, x, g.w));
  CDG_TRY(dot64(ctx, n, g.w, nullptr, beta_d, 0));
  double beta = 0;
  CDG_TRY(read_scalar(ctx, beta_d, &beta));
  double resid = beta;
  st->initial_residual = beta;
  st->iterations = 0;
  st->residual = beta;
  if (converged(s, li, resid, 0)) return CDG_OK;
  int j = 1;
  const int vg = vec_grid(ctx, n);
  const bool coop = s.gram_schmidt == 0 && cgs_coop_on(ctx, n, m);
  while (j <= s.max_n_iterations) {
    CDG_LAUNCH_PDL(ctx, k_scale_inv, vg, 256, 0, n, g.w, beta_d, g.V, ctx->d_err,
                   (const int*)nullptr);
    CDG_LAUNCH_PDL(ctx, k_init_s, 1, 128, 0, m, beta_d, g.s);
    int i;
    for (i = 0; i < m && j <= s.max_n_iterations; ++i, ++j) {
      double* vi = g.V + (size_t)i * n;
      double* zi = g.Z + (size_t)i * n;
      double* col = g.H + (size_t)i * (m + 1);
      CDG_TRY(precondition(ctx, p, s, vi, zi));
      CDG_TRY(spmv_apply64(ctx, L, zi, g.w));
      if (s.gram_schmidt == 0 && coop) {
        // classical, the inner products, updates, norm, Givens step and
        // normalisation in one cooperative launch
        CDG_TRY(cgs_coop(ctx, g, n, m, i, (const int*)nullptr));
      } else if (s.gram_schmidt == 0) {
        // classical: all inner products, then all updates and the norm
        for (int k0 = 0; k0 <= i; k0 += 32) {
          int cnt = std::min(32, i + 1 - k0);
          // two blocks per SM: several elements per thread, fewer FP64 reductions
          CDG_LAUNCH_PDL(ctx, k_multidot<256>, std::min(red_grid(ctx, n), ctx->num_sms * 2), 256, 0,
                     n, g.w, g.V, k0, cnt, ctx->d_red, ctx->d_cnt + 1, col + k0,
                     (const int*)nullptr, 0);
        }
        CDG_LAUNCH_PDL(ctx, k_cgs_update, red_grid(ctx, n), 256, 0, n, g.w, g.V, i, col,
                   ctx->d_red, ctx->d_cnt, g.cs, g.sn, g.s, resid_d, g.scal + 2,
                   (const int*)nullptr, 0);
        CDG_LAUNCH_PDL(ctx, k_scale_inv, vg, 256, 0, n, g.w, g.scal + 2,
                   g.V + (size_t)(i + 1) * n, ctx->d_err, (const int*)nullptr);
      } else {
        // modified: dot and update interleaved (sequential build)
        CDG_TRY(dot64(ctx, n, g.w, g.V, col + 0, 0));
        for (int k = 0; k <= i; ++k) {
          const double* vk = g.V + (size_t)k * n;
          const double* vn = (k < i) ? g.V + (size_t)(k + 1) * n : nullptr;
          CDG_LAUNCH_PDL(ctx, k_mgs, red_grid(ctx, n), 256, 0, n, g.w, vk, col + k, vn,
                     ctx->d_red, ctx->d_cnt, col + k + 1);
        }
      }
      if (s.gram_schmidt != 0) {
        CDG_LAUNCH_PDL(ctx, k_scale_inv, vg, 256, 0, n, g.w, col + i + 1,
                   g.V + (size_t)(i + 1) * n, ctx->d_err, (const int*)nullptr);
        CDG_LAUNCH_PDL(ctx, k_givens, 1, 1, 0, i, m, g.H, g.cs, g.sn, g.s, resid_d);
      }
      CDG_TRY(read_scalar(ctx, resid_d, &resid));
      CDG_TRY(check_device_error(ctx));
      int cv = converged(s, li, resid, j);
      if (cv == 2) {
        set_error("Execution of the code stopped because of solver divergence.");
        st->iterations = j;
        st->residual = resid;
        return CDG_ERR_DIVERGED;
      }
      if (cv) {
        CDG_TRY(launch_backsolve(ctx, i, m, g.H, g.s, g.y));
        CDG_LAUNCH_PDL(ctx, k_update, vg, 256, 0, n, i, g.Z, g.y, x);
        st->iterations = j;
        st->residual = resid;
        return CDG_OK;
      }
    }
    CDG_TRY(launch_backsolve(ctx, m - 1, m, g.H, g.s, g.y));
    CDG_LAUNCH_PDL(ctx, k_update, vg, 256, 0, n, m - 1, g.Z, g.y, x);
    CDG_TRY(residual64(ctx, L, b, x, g.w));
    CDG_TRY(dot64(ctx, n, g.w, nullptr, beta_d, 0));
    CDG_TRY(read_scalar(ctx, beta_d, &beta));
    int cv = converged(s, li, resid, j);
    if (cv == 2) {
      set_error("Execution of the code stopped because of solver divergence.");
      return CDG_ERR_DIVERGED;
    }
    if (cv) {
      st->iterations = j;
      st->residual = resid;
      return CDG_OK;
    }
  }
  st->iterations = s.max_n_iterations;
  st->residual = resid;
  return CDG_OK;
}

}  // namespace cdg
