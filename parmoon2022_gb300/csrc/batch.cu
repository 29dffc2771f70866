// batch.cu -- many small stationary solves in one launch, one block per
// request: FGMRES(m) in FP64 preconditioned by the FP32 multigrid V-cycle
// (Iteration_gmres.C:430-620 around Multigrid.C:157-410, the mixed-precision
// form of the graph-captured solver in linalg.cu), with every vector
// operation, smoothing step, transfer and the coarse direct solve done by the
// block under block barriers.
//
// A small request (a few thousand DOFs) spends its stream-level solve waiting
// on ~30 dependent kernel launches per FGMRES iteration (~85 us); here a block
// runs the whole iteration in a few tens of microseconds and the GPU holds
// hundreds of requests at once.  Instances are segmented: each block reads
// its request's CSR levels, transfer matrices, coarse inverse and Krylov
// buffers through its descriptor (the per-request pointers into that
// request's own device-resident problem instance), and stops on its own
// convergence test (per-instance mask: a converged request's block exits
// while the others iterate).
//
// Arithmetic follows the stream path operation by operation (the same
// updates, the same convergence test and Givens steps, FP32 multigrid
// vectors, FP64 Krylov vectors), with row sums in CSR order and block
// reductions in a fixed order: results agree with a stream-path solve of the
// same request to round-off (deterministic run to run, not bit-equal to the
// stream kernels' lane-split sums).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "solver_dev.cuh"

namespace cdg {

namespace {

constexpr int kBatchThreads = 512;
constexpr int kBatchWarps = kBatchThreads / 32;

struct BLevel {
  int n, na;
  int tpr;           // lanes per CSR row of the operator (4 or 8)
  const int* rp;
  const int* col;
  const float* val;
  const float* invd;
  const int* R_rp;   // restriction of this level's defect to the next coarser level
  const int* R_col;
  const float* R_val;
  const int* P_rp;   // prolongation from the next coarser level
  const int* P_col;
  const float* P_val;
  float* rhs;
  float* sol;
  float* tmp;
  float* def;
};

struct BJob {
  int nl, m, npre, npost;
  ConvParams cp;
  float damp, cdamp;
  BLevel L[kBatchMaxLevels];
  const int* dc_rp;   // finest level: couplings of active rows to non-active columns
  const int* dc_col;
  const float* dcv;
  const int* rp64;    // finest level FP64 operator
  const int* col64;
  const double* val64;
  const double* b;
  double* x;
  double* V;
  double* Z;
  double* w;
  double* H;
  double* cinv;         // coarsest level: dense inverse of the active block
  const int* zero_diag; // the problem's zero-diagonal flag (set by its assembly)
  // coarse block inverted by k_batch_coarse (cinline), from the coarsest
  // level's FP64 CSR rows
  int cinline, cna;
  const int* c_rp;
  const int* c_col;
  const double* c_val;
};

// deterministic block sum (warp trees, then the warps' sums in order); every
// thread returns the total
__device__ double bsum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();   // red free again
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
#pragma unroll
  for (int q = 0; q < kBatchWarps; ++q) t += red[q];
  return t;
}

// sum of the TPR lanes of a row group (fixed tree: the same order every run)
template <int TPR, typename T>
__device__ __forceinline__ T group_total(T v) {
#pragma unroll
  for (int o = TPR / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// FP32 CSR row operations on a level (non-active rows are identity rows), TPR
// lanes per row: MODE 1 y = b - A x, 2 y = x + w D^-1 (b - A x), 3 mode 2 and
// z = y in FP64
template <int MODE, int TPR>
__device__ void b_csr_t(const BLevel& L, const float* x, const float* b, float w, float* y,
                        double* z) {
  const int sub = threadIdx.x % TPR;
  for (int r0 = 0; r0 < L.n; r0 += kBatchThreads / TPR) {
    const int r = r0 + threadIdx.x / TPR;
    float s = 0.f;
    if (r < L.na) {
      const int k1 = L.rp[r + 1];
      for (int k = L.rp[r] + sub; k < k1; k += TPR) s += L.val[k] * x[L.col[k]];
    }
    s = group_total<TPR>(s);
    if (r >= L.n || sub != 0) continue;
    const float xr = x[r];
    if (r >= L.na) s = xr;
    if (MODE == 1) {
      y[r] = b[r] - s;
    } else {
      const float yr = xr + w * (L.invd[r] * (b[r] - s));
      y[r] = yr;
      if (MODE == 3) z[r] = (double)yr;
    }
  }
}

template <int MODE>
__device__ void b_csr(const BLevel& L, const float* x, const float* b, float w, float* y,
                      double* z) {
  if (L.tpr == 8)
    b_csr_t<MODE, 8>(L, x, b, w, y, z);
  else
    b_csr_t<MODE, 4>(L, x, b, w, y, z);
}

// FP64 finest operator, TPR lanes per row: MODE 0 y = A x, 1 y = b - A x
template <int MODE, int TPR>
__device__ void b_csr64_t(const BJob& J, const double* x, double* y) {
  const BLevel& F = J.L[0];
  const int sub = threadIdx.x % TPR;
  for (int r0 = 0; r0 < F.n; r0 += kBatchThreads / TPR) {
    const int r = r0 + threadIdx.x / TPR;
    double s = 0.0;
    if (r < F.na) {
      const int k1 = J.rp64[r + 1];
      for (int k = J.rp64[r] + sub; k < k1; k += TPR) s += J.val64[k] * x[J.col64[k]];
    }
    s = group_total<TPR>(s);
    if (r >= F.n || sub != 0) continue;
    if (r >= F.na) s = x[r];
    y[r] = MODE == 0 ? s : J.b[r] - s;
  }
}

template <int MODE>
__device__ void b_csr64(const BJob& J, const double* x, double* y) {
  if (J.L[0].tpr == 8)
    b_csr64_t<MODE, 8>(J, x, y);
  else
    b_csr64_t<MODE, 4>(J, x, y);
}

// restriction of level l's defect to level l + 1 (coarse non-active rows
// zero) and the prolongation correction of level l, eight and four lanes per
// row
__device__ void b_restrict(const BLevel& L, const BLevel& C) {
  constexpr int TPR = 8;
  const int sub = threadIdx.x % TPR;
  for (int j0 = 0; j0 < C.n; j0 += kBatchThreads / TPR) {
    const int j = j0 + threadIdx.x / TPR;
    float s = 0.f;
    if (j < C.na) {
      const int k1 = L.R_rp[j + 1];
      for (int k = L.R_rp[j] + sub; k < k1; k += TPR) s += L.R_val[k] * L.def[L.R_col[k]];
    }
    s = group_total<TPR>(s);
    if (j < C.n && sub == 0) C.rhs[j] = s;
  }
}

__device__ void b_prolong(const BLevel& L, const float* xc, float* xf, float cdamp) {
  constexpr int TPR = 4;
  const int sub = threadIdx.x % TPR;
  for (int i0 = 0; i0 < L.n; i0 += kBatchThreads / TPR) {
    const int i = i0 + threadIdx.x / TPR;
    float s = 0.f;
    if (i < L.n) {
      const int k1 = L.P_rp[i + 1];
      for (int k = L.P_rp[i] + sub; k < k1; k += TPR) s += L.P_val[k] * xc[L.P_col[k]];
    }
    s = group_total<TPR>(s);
    if (i < L.na && sub == 0) xf[i] += cdamp * s;
  }
}

// z = B v: one V-cycle (pre- and post-smoothing by damped Jacobi, direct
// coarse solve), the finest level's first step fused with the start
// (rhs = v in FP32, x0 = the Dirichlet values) and the last post-smoothing
// step writing z in FP64, as mg_cycle<float> does
__device__ void b_vcycle(const BJob& J, const double* v, double* z, float** sol, float** tmp) {
  const int nl = J.nl;
  const float w = J.damp;
  // down
  for (int l = 0; l + 1 < nl; ++l) {
    const BLevel& L = J.L[l];
    for (int it = 0; it < J.npre; ++it) {
      if (it == 0 && l == 0) {
        for (int r = threadIdx.x; r < L.n; r += kBatchThreads) {
          const float bi = (float)v[r];
          L.rhs[r] = bi;
          if (r < L.na) {
            float s = 0.f;
            const int k1 = J.dc_rp[r + 1];
            for (int k = J.dc_rp[r]; k < k1; ++k) s += J.dcv[k] * (float)v[J.dc_col[k]];
            tmp[l][r] = w * (L.invd[r] * (bi - s));
          } else {
            tmp[l][r] = bi + w * (L.invd[r] * (bi - bi));
          }
        }
      } else if (it == 0) {
        // zero start iterate on a coarser level
        for (int r = threadIdx.x; r < L.n; r += kBatchThreads)
          tmp[l][r] = w * (L.invd[r] * L.rhs[r]);
      } else {
        b_csr<2>(L, sol[l], L.rhs, w, tmp[l], nullptr);
      }
      float* t = sol[l];
      sol[l] = tmp[l];
      tmp[l] = t;
      __syncthreads();
    }
    b_csr<1>(L, sol[l], L.rhs, 0.f, L.def, nullptr);
    __syncthreads();
    b_restrict(L, J.L[l + 1]);
    __syncthreads();
  }
  // coarsest level: x = (0 on active rows, b elsewhere), d = b - A x,
  // x_a += Inv d_a (a warp per row)
  {
    const int c = nl - 1;
    const BLevel& C = J.L[c];
    for (int r = threadIdx.x; r < C.n; r += kBatchThreads) sol[c][r] = r < C.na ? 0.f : C.rhs[r];
    __syncthreads();
    b_csr<1>(C, sol[c], C.rhs, 0.f, C.def, nullptr);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (int row = threadIdx.x >> 5; row < C.na; row += kBatchWarps) {
      double s = 0.0;
      for (int j = lane; j < C.na; j += 32) s += J.cinv[(size_t)row * C.na + j] * (double)C.def[j];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) sol[c][row] = (float)((double)sol[c][row] + s);
    }
    __syncthreads();
  }
  // up
  for (int l = nl - 2; l >= 0; --l) {
    const BLevel& L = J.L[l];
    b_prolong(L, sol[l + 1], sol[l], J.cdamp);
    __syncthreads();
    for (int it = 0; it < J.npost; ++it) {
      if (l == 0 && it + 1 == J.npost)
        b_csr<3>(L, sol[l], L.rhs, w, tmp[l], z);
      else
        b_csr<2>(L, sol[l], L.rhs, w, tmp[l], nullptr);
      float* t = sol[l];
      sol[l] = tmp[l];
      tmp[l] = t;
      __syncthreads();
    }
  }
  if (J.npost == 0) {
    for (int r = threadIdx.x; r < J.L[0].n; r += kBatchThreads) z[r] = (double)sol[0][r];
    __syncthreads();
  }
}

// The coarse direct solve's inverse of every small coarse block of the batch
// (DirectSmoother, DirectSmoother.C:25-42; the dense block inverted as
// k_gj_smem does: Gauss-Jordan with partial pivoting, the first row of
// maximal |a_ik| as pivot, in shared memory, then the column exchanges in
// reverse pivot order), one block per request; cstat[q] = kErrSingular on a
// zero pivot
constexpr int kCoarseThreads = 256;

__global__ void __launch_bounds__(kCoarseThreads)
k_batch_coarse(const BJob* __restrict__ jobs, int* __restrict__ cstat) {
  const BJob& J = jobs[blockIdx.x];
  const int na = J.cna, tid = threadIdx.x, nt = kCoarseThreads;
  if (tid == 0) cstat[blockIdx.x] = 0;
  if (!J.cinline || na == 0) return;
  extern __shared__ double s_gj[];
  double* a = s_gj;                     // na * na
  double* prow = a + (size_t)na * na;   // na
  double* colk = prow + na;             // na
  int* perm = (int*)(colk + na);        // na
  int* q = perm + na;                   // na
  __shared__ double wv[kCoarseThreads / 32];
  __shared__ int wi[kCoarseThreads / 32];
  __shared__ int s_p;
  __shared__ double s_piv;
  const int lane = tid & 31, w = tid >> 5;
  for (int t = tid; t < na * na; t += nt) a[t] = 0.0;
  __syncthreads();
  for (int i = tid; i < na; i += nt)
    for (int k = J.c_rp[i]; k < J.c_rp[i + 1]; ++k)
      if (J.c_col[k] < na) a[(size_t)i * na + J.c_col[k]] = J.c_val[k];
  __syncthreads();
  for (int k = 0; k < na; ++k) {
    double best = -1.0;
    int bi = k;
    for (int i = k + tid; i < na; i += nt) {
      const double v = fabs(a[(size_t)i * na + k]);
      if (v > best) { best = v; bi = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double v = __shfl_xor_sync(0xffffffffu, best, o);
      const int vi = __shfl_xor_sync(0xffffffffu, bi, o);
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
      if (tid == 0) cstat[blockIdx.x] = kErrSingular;
      return;   // uniform: every thread read the same pivot
    }
    const double rpiv = 1.0 / piv;
    for (int j = tid; j < na; j += nt) prow[j] = j == k ? rpiv : a[(size_t)p * na + j] * rpiv;
    for (int i = tid; i < na; i += nt) colk[i] = a[(size_t)(i == p ? k : i) * na + k];
    __syncthreads();
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
    J.cinv[t] = a[(size_t)i * na + q[j]];
  }
}

__global__ void __launch_bounds__(kBatchThreads)
k_batch_solve(const BJob* __restrict__ jobs, const int* __restrict__ cstat,
              BatchResult* __restrict__ out) {
  const BJob& J = jobs[blockIdx.x];
  // a zero diagonal found by the assembly (Iteration_jacobi.C:14-28 throws)
  // or a singular coarse block: nothing to iterate
  if (*J.zero_diag || cstat[blockIdx.x]) {
    if (threadIdx.x == 0)
      out[blockIdx.x] = BatchResult{*J.zero_diag ? CDG_ERR_ZERO_DIAG : CDG_ERR_SINGULAR, 0,
                                    0.0, 0.0};
    return;
  }
  __shared__ double red[kBatchWarps];
  __shared__ double part[kBatchWarps][kBatchMaxRestart + 1];
  __shared__ double hcol[kBatchMaxRestart + 2], cs[kBatchMaxRestart + 1],
      sn[kBatchMaxRestart + 1], gs[kBatchMaxRestart + 2], ys[kBatchMaxRestart + 1];
  __shared__ double li[2], s_resid, s_beta;
  __shared__ int s_flag, s_j;
  __shared__ float* s_ptr[2][kBatchMaxLevels];
  const int n = J.L[0].n, m = J.m, tid = threadIdx.x;
  if (tid < J.nl) {
    s_ptr[0][tid] = J.L[tid].sol;
    s_ptr[1][tid] = J.L[tid].tmp;
  }
  // the level buffers swap roles uniformly across the block: every thread
  // keeps its own copy of the pointers
  float* sol[kBatchMaxLevels];
  float* tmp[kBatchMaxLevels];
  __syncthreads();
  for (int l = 0; l < J.nl; ++l) {
    sol[l] = s_ptr[0][l];
    tmp[l] = s_ptr[1][l];
  }
  double* w = J.w;
  int status = CDG_OK;
  // r = b - A x; beta = ||r||; the test at iteration 0
  b_csr64<1>(J, J.x, w);
  __syncthreads();
  double ss = 0.0;
  for (int t = tid; t < n; t += kBatchThreads) ss += w[t] * w[t];
  double beta = sqrt(bsum(ss, red));
  if (tid == 0) {
    s_flag = conv_test(J.cp, li, beta, 0);
    s_j = 1;
    s_resid = beta;
  }
  __syncthreads();
  const double initial = beta;
  int iterations = 0;
  double resid = beta;
  if (s_flag != 0) {
    if (tid == 0) out[blockIdx.x] = BatchResult{CDG_OK, 0, beta, initial};
    return;
  }
  // restart cycles; the iteration count j rises by one per inner step and
  // the convergence test stops at max_n_iterations
  for (int cycle = 0; cycle <= J.cp.max_it; ++cycle) {
    if (beta == 0.0) {
      status = CDG_ERR_BREAKDOWN;
      break;
    }
    {
      const double f = 1.0 / beta;
      for (int t = tid; t < n; t += kBatchThreads) J.V[t] = w[t] * f;
    }
    if (tid == 0) {
      gs[0] = beta;
      for (int k = 1; k <= m; ++k) gs[k] = 0.0;
    }
    __syncthreads();
    int flag = 0, iend = m - 1;
    for (int i = 0; i < m; ++i) {
      const double* vi = J.V + (size_t)i * n;
      double* zi = J.Z + (size_t)i * n;
      b_vcycle(J, vi, zi, sol, tmp);
      b_csr64<0>(J, zi, w);
      __syncthreads();
      // classical Gram-Schmidt: all inner products, then the update
      for (int k = 0; k <= i; ++k) {
        const double* vk = J.V + (size_t)k * n;
        double p = 0.0;
        for (int t = tid; t < n; t += kBatchThreads) p = fma(w[t], vk[t], p);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
        if ((tid & 31) == 0) part[tid >> 5][k] = p;
      }
      __syncthreads();
      if (tid <= i) {
        double h = 0.0;
#pragma unroll
        for (int q = 0; q < kBatchWarps; ++q) h += part[q][tid];
        hcol[tid] = h;
      }
      __syncthreads();
      ss = 0.0;
      for (int t = tid; t < n; t += kBatchThreads) {
        double wt = w[t];
        for (int k = 0; k <= i; ++k) wt = fma(-hcol[k], J.V[(size_t)k * n + t], wt);
        w[t] = wt;
        ss += wt * wt;
      }
      const double nrm = sqrt(bsum(ss, red));
      if (tid == 0) {
        hcol[i + 1] = nrm;
        double r;
        givens_column_s(i, hcol, cs, sn, gs[i], gs[i + 1], &r);
        for (int k = 0; k <= i + 1; ++k) J.H[(size_t)i * (m + 1) + k] = hcol[k];
        s_resid = r;
        s_beta = nrm;
        const int j = s_j;
        const int cv = conv_test(J.cp, li, r, j);
        if (cv == 2) {
          s_flag = 2;
        } else if (cv == 1) {
          s_flag = 1;
        } else if (i + 1 == m) {
          s_flag = 3;
          s_j = j + 1;
        } else {
          s_flag = 0;
          s_j = j + 1;
        }
      }
      __syncthreads();
      flag = s_flag;
      resid = s_resid;
      if (flag != 0) {
        iend = i;
        break;
      }
      // v_{i+1} = w / H(i+1,i)
      if (s_beta == 0.0) {
        flag = -1;
        break;
      }
      const double f = 1.0 / s_beta;
      double* vn = J.V + (size_t)(i + 1) * n;
      for (int t = tid; t < n; t += kBatchThreads) vn[t] = w[t] * f;
      __syncthreads();
    }
    if (flag == -1) {
      status = CDG_ERR_BREAKDOWN;
      iterations = s_j;
      break;
    }
    if (flag == 2) {
      status = CDG_ERR_DIVERGED;
      iterations = s_j;
      break;
    }
    // y = R^{-1} s on columns 0..iend (Utilities_gmres.C:90-108), x += Z y
    if (tid == 0) {
      for (int k = 0; k <= iend; ++k) ys[k] = gs[k];
      for (int c = iend; c >= 0; --c) {
        ys[c] /= J.H[(size_t)c * (m + 1) + c];
        const double yc = ys[c];
        for (int k = 0; k < c; ++k) ys[k] -= J.H[(size_t)c * (m + 1) + k] * yc;
      }
    }
    __syncthreads();
    for (int t = tid; t < n; t += kBatchThreads) {
      double acc = 0.0;
      for (int k = 0; k <= iend; ++k) acc += ys[k] * J.Z[(size_t)k * n + t];
      J.x[t] += acc;
    }
    __syncthreads();
    if (flag == 1) {
      iterations = s_j;
      break;
    }
    // end of a restart cycle: the true residual starts the next one; the
    // test takes the last estimate at iteration j
    b_csr64<1>(J, J.x, w);
    __syncthreads();
    ss = 0.0;
    for (int t = tid; t < n; t += kBatchThreads) ss += w[t] * w[t];
    beta = sqrt(bsum(ss, red));
    if (tid == 0) s_flag = conv_test(J.cp, li, resid, s_j);
    __syncthreads();
    const int cv = s_flag, j = s_j;
    if (cv == 2) {
      status = CDG_ERR_DIVERGED;
      iterations = j;
      break;
    }
    if (cv == 1 || j > J.cp.max_it) {
      iterations = min(j, J.cp.max_it);
      break;
    }
  }
  if (tid == 0) out[blockIdx.x] = BatchResult{status, iterations, resid, initial};
}

}  // namespace

bool batch_eligible(const cdg_problem* p, const cdg_solver_params& s, const char** why) {
  const char* r = nullptr;
  if (s.preconditioner != 2) r = "the batched solver runs multigrid-preconditioned FGMRES";
  else if (s.precision != 1) r = "the batched solver runs the mixed-precision multigrid";
  else if (s.multigrid_cycle_type != 0) r = "the batched solver runs V-cycles";
  else if (s.multigrid_smoother_coarse != 0) r = "the batched solver needs the direct coarse solve";
  else if (s.gram_schmidt != 0) r = "the batched solver uses classical Gram-Schmidt";
  else if (s.multigrid_n_levels < 2 || s.multigrid_n_levels > kBatchMaxLevels)
    r = "the batched solver needs 2 to kBatchMaxLevels multigrid levels";
  else if (s.multigrid_n_pre_smooth < 1) r = "the batched solver needs pre-smoothing";
  else if (s.gmres_restart < 1 || s.gmres_restart > kBatchMaxRestart)
    r = "the batched solver takes gmres_restart up to kBatchMaxRestart";
  else if (p->lev.empty() || p->lev[0].ndof > kBatchMaxDofs)
    r = "request larger than kBatchMaxDofs";
  else if (p->lev[s.multigrid_n_levels - 1].nactive > kBatchMaxCoarse)
    r = "coarsest level larger than kBatchMaxCoarse";
  if (why) *why = r;
  return r == nullptr;
}

int batch_launch(cdg_context* ctx, cdg_problem* const* probs, const cdg_solver_params* params,
                 const int* inline_coarse, int count, BatchResult* results) {
  if (count <= 0) return CDG_OK;
  std::vector<BJob> jobs(count);
  int max_cna = 0;
  for (int q = 0; q < count; ++q) {
    cdg_problem* p = probs[q];
    const cdg_solver_params& s = params[q];
    BJob& J = jobs[q];
    std::memset(&J, 0, sizeof(J));
    J.nl = s.multigrid_n_levels;
    J.m = s.gmres_restart;
    J.npre = s.multigrid_n_pre_smooth;
    J.npost = s.multigrid_n_post_smooth;
    J.cp = ConvParams{s.residual_tolerance, s.residual_reduction, s.divergence_factor,
                      s.min_n_iterations, s.max_n_iterations, s.gmres_restart};
    J.damp = (float)s.jacobi_damp;
    J.cdamp = (float)s.multigrid_correction_damp_factor;
    for (int l = 0; l < J.nl; ++l) {
      const DevLevel& L = p->lev[l];
      BLevel& B = J.L[l];
      B.n = L.ndof;
      B.na = L.nactive;
      B.tpr = L.nnz > 12LL * std::max(L.ndof, 1) ? 8 : 4;
      B.rp = L.row_ptr;
      B.col = L.col;
      B.val = L.val32;
      B.invd = L.invdiag32;
      B.R_rp = L.R_rp;
      B.R_col = L.R_col;
      B.R_val = L.R_val32;
      B.P_rp = L.P_rp;
      B.P_col = L.P_col;
      B.P_val = L.P_val32;
      B.rhs = (float*)L.mg_rhs;
      B.sol = (float*)L.mg_sol;
      B.tmp = (float*)L.mg_tmp;
      B.def = (float*)L.mg_def;
    }
    const DevLevel& F = p->lev[0];
    J.dc_rp = F.dc_rp;
    J.dc_col = F.dc_col;
    J.dcv = F.dc_val32;
    J.rp64 = F.row_ptr;
    J.col64 = F.col;
    J.val64 = F.val64;
    J.b = F.rhs;
    J.x = F.sol;
    J.V = p->gm.V;
    J.Z = p->gm.Z;
    J.w = p->gm.w;
    J.H = p->gm.H;
    const DevLevel& Cl = p->lev[J.nl - 1];
    J.cinv = Cl.coarse_inv;
    J.zero_diag = p->d_zero_diag;
    J.cinline = inline_coarse[q];
    J.cna = Cl.nactive;
    J.c_rp = Cl.row_ptr;
    J.c_col = Cl.col;
    J.c_val = Cl.val64;
    if (J.cinline) max_cna = std::max(max_cna, Cl.nactive);
  }
  // descriptors, results, coarse status (16-byte aligned pieces)
  const size_t jb = (size_t)count * sizeof(BJob), rb = (size_t)count * sizeof(BatchResult);
  const size_t cb = ((size_t)count * sizeof(int) + 15) / 16 * 16;
  if (ctx->batch_host_bytes < jb + rb + cb) {
    if (ctx->batch_host) cudaFreeHost(ctx->batch_host);
    if (ctx->batch_dev) cudaFree(ctx->batch_dev);
    ctx->batch_host = nullptr;
    ctx->batch_dev = nullptr;
    ctx->batch_host_bytes = 0;
    CDG_CUDA(cudaMallocHost(&ctx->batch_host, jb + rb + cb));
    CDG_CUDA(cudaMalloc(&ctx->batch_dev, jb + rb + cb));
    ctx->batch_host_bytes = jb + rb + cb;
  }
  char* hb = (char*)ctx->batch_host;
  char* db = (char*)ctx->batch_dev;
  std::memcpy(hb, jobs.data(), jb);
  CDG_CUDA(cudaMemcpyAsync(db, hb, jb, cudaMemcpyHostToDevice, ctx->stream));
  int* cstat = (int*)(db + jb + rb);
  const size_t csm = (size_t)max_cna * max_cna * sizeof(double) +
                     2 * (size_t)max_cna * sizeof(double) + 2 * (size_t)max_cna * sizeof(int);
  static const bool attr_set = [] {
    return cudaFuncSetAttribute(k_batch_coarse, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)((size_t)kBatchSmemCoarse * kBatchSmemCoarse * 8 +
                                      4 * kBatchSmemCoarse * 8)) == cudaSuccess;
  }();
  if (!attr_set) {
    set_error("shared memory of the batched coarse inverse");
    return CDG_ERR_CUDA;
  }
  CDG_LAUNCH(ctx, k_batch_coarse, count, kCoarseThreads, csm, (const BJob*)db, cstat);
  CDG_LAUNCH(ctx, k_batch_solve, count, kBatchThreads, 0, (const BJob*)db, (const int*)cstat,
             (BatchResult*)(db + jb));
  CDG_CUDA(cudaMemcpyAsync(hb + jb, db + jb, rb, cudaMemcpyDeviceToHost, ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::memcpy(results, hb + jb, rb);
  return CDG_OK;
}

}  // namespace cdg
