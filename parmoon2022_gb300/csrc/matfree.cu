// matfree.cu -- matrix-free FP32 operator of the multigrid levels on Q2
// hexahedra (JacobiSmoother::smooth / calculate_defect without the CSR
// matrix, src/Multigrid/JacobiSmoother.C:21-29).
//
// The assembled element matrix of an affine hexahedron with cell-constant
// coefficients is A_cell = sum_t g_t R_t (the contraction in assemble.cu):
// 40 per-cell factors g_t (diffusion + SUPG gradient pairs, convection,
// reaction, convection linear in x, SUPG reaction, SUPG diffusion-Hessian)
// times exact reference integrals R_t.  Two kernels apply it:
//
// k_mf_uniform: where every cell is a translate of cell 0 and the
// coefficients are constant (uniform meshes and their affine images), the
// cells' DOFs are listed in cell 0's local frame once per level, and all
// cells share cell 0's 27 x 27 element matrix, kept in registers (one row per
// lane): 27 multiply-adds per lane and cell.
//
// k_mf_cell: any affine hexahedra.  Every integrand of a Q2 cell is a
// polynomial of degree <= 5 per direction, so the 3-point Gauss rule per
// direction reproduces R_t exactly, and A_cell u is applied by sum
// factorisation: values, gradients and Hessians of u at the 27 Gauss points
// by 1D passes (B, B', B'' along each direction), four test fields per point
// from the factors, and three transposed 1D passes back to the 27 local DOFs
// -- about 3.3k FP32 multiply-adds per cell.  One warp per cell, lane = Gauss
// point / local DOF (27 of 32 lanes); the 1D passes exchange values through
// per-warp shared memory (only __syncwarp, no block barrier).
//
// Both write each local result to its position in a DOF-major array (the
// entries of active row r contiguous, in the fixed (cell, local DOF) order of
// the rhs gather); k_mf_gather sums a row's range (deterministic, no atomics)
// and applies the smoothing / defect update.  Non-active rows act as identity
// rows, as in the CSR kernels.
#include <algorithm>
#include <cstdlib>
#include <vector>

#include "common.cuh"

namespace cdg {

namespace {

constexpr int kMfWarps = 8;            // cells in flight per block
constexpr int kMfBuf = 10;             // per-warp 32-float exchange buffers
constexpr float kGs = 0.7745966692414834f;   // sqrt(3/5), 3-point Gauss point
constexpr int kMfGather = 12;          // cell values per thread and batch (one-launch sweep)
constexpr int kMfRowRegs = 8;          // entries of a row held in registers (a Q2 vertex: 8 cells)

// 1D Q2 Lagrange basis on [-1, 1] (nodes -1, 0, 1; local index i):
// phi_0 = (t^2 - t)/2, phi_1 = 1 - t^2, phi_2 = (t^2 + t)/2,
// phi'_i = (t - 1/2, -2t, t + 1/2), phi''_i = (1, -2, 1),
// at the Gauss points t_q = (-sqrt(3/5), 0, sqrt(3/5))
__device__ __forceinline__ float gpt(int q) { return (float)(q - 1) * kGs; }
__device__ __forceinline__ float phi(int i, float t) {
  const float t2 = t * t;
  return i == 0 ? 0.5f * (t2 - t) : (i == 1 ? 1.0f - t2 : 0.5f * (t2 + t));
}
__device__ __forceinline__ float dphi(int i, float t) {
  return i == 0 ? t - 0.5f : (i == 1 ? -2.0f * t : t + 0.5f);
}
__device__ __forceinline__ float gw(int q) { return q == 1 ? 8.0f / 9.0f : 5.0f / 9.0f; }

// row q of B / B' (values at point q) and column i (basis i at all points)
struct Line {
  float br[3], dr[3];   // B[q][.], B'[q][.] for this lane's q
  float bc[3], dc[3];   // B[.][i], B'[.][i] for this lane's i
};
__device__ __forceinline__ Line make_line(int l) {
  Line L;
  const float t = gpt(l);
  for (int i = 0; i < 3; ++i) {
    L.br[i] = phi(i, t);
    L.dr[i] = dphi(i, t);
    L.bc[i] = phi(l, gpt(i));
    L.dc[i] = dphi(l, gpt(i));
  }
  return L;
}

__device__ __forceinline__ float dot3(const float* a, float x0, float x1, float x2) {
  return fmaf(a[2], x2, fmaf(a[1], x1, a[0] * x0));
}

// factor offsets (the Terms<3> order of assemble.cu)
constexpr int kS = 0, kC = 6, kM = 9, kL = 10, kD = 19, kT = 22;

template <bool LIN>
__global__ void __launch_bounds__(kMfWarps * 32)
k_mf_cell(int ncells, const int* __restrict__ gdof, const int* __restrict__ pos,
          const float* __restrict__ fac, const float* __restrict__ x,
          float* __restrict__ ycell) {
  pdl_enter();
  __shared__ float sb[kMfWarps][kMfBuf][32];
  __shared__ float sf[kMfWarps][kMfFactors];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool act = lane < 27;
  const int l0 = lane % 3, l1 = (lane / 3) % 3, l2 = act ? lane / 9 : 0;
  const Line X0 = make_line(l0), X1 = make_line(l1), X2 = make_line(l2);
  const float wq = gw(l0) * gw(l1) * gw(l2);
  float (*B)[32] = sb[warp];
  float* F = sf[warp];
  for (int cell = blockIdx.x * kMfWarps + warp; cell < ncells; cell += gridDim.x * kMfWarps) {
    // factors and local values (lane = local DOF)
    const float* fc = fac + (size_t)cell * kMfFactors;
    F[lane] = __ldg(fc + lane);
    if (lane < kMfFactors - 32) F[32 + lane] = __ldg(fc + 32 + lane);
    if (act) B[0][lane] = __ldg(x + __ldg(gdof + (size_t)cell * 27 + lane));
    __syncwarp();
    // direction 0: lane (q0, i1, i2)
    if (act) {
      const float* u = &B[0][3 * l1 + 9 * l2];
      const float u0 = u[0], u1 = u[1], u2 = u[2];
      B[1][lane] = dot3(X0.br, u0, u1, u2);
      B[2][lane] = dot3(X0.dr, u0, u1, u2);
      B[3][lane] = u0 - 2.0f * u1 + u2;
    }
    __syncwarp();
    // direction 1: lane (q0, q1, i2)
    if (act) {
      const int o = l0 + 9 * l2;
      const float a0 = B[1][o], a1 = B[1][o + 3], a2 = B[1][o + 6];
      const float d0 = B[2][o], d1 = B[2][o + 3], d2 = B[2][o + 6];
      const float h0 = B[3][o], h1 = B[3][o + 3], h2 = B[3][o + 6];
      B[4][lane] = dot3(X1.br, a0, a1, a2);   // B B
      B[5][lane] = dot3(X1.br, d0, d1, d2);   // B' B
      B[6][lane] = dot3(X1.dr, a0, a1, a2);   // B B'
      B[7][lane] = dot3(X1.br, h0, h1, h2);   // B'' B
      B[8][lane] = a0 - 2.0f * a1 + a2;       // B B''
      B[9][lane] = dot3(X1.dr, d0, d1, d2);   // B' B'
    }
    __syncwarp();
    // direction 2 and the point values: lane (q0, q1, q2)
    if (act) {
      const int o = l0 + 3 * l1;
      float c[6][3];
#pragma unroll
      for (int k = 0; k < 6; ++k)
#pragma unroll
        for (int j = 0; j < 3; ++j) c[k][j] = B[4 + k][o + 9 * j];
      const float u = dot3(X2.br, c[0][0], c[0][1], c[0][2]);
      const float u_2 = dot3(X2.dr, c[0][0], c[0][1], c[0][2]);
      const float u_22 = c[0][0] - 2.0f * c[0][1] + c[0][2];
      const float u_0 = dot3(X2.br, c[1][0], c[1][1], c[1][2]);
      const float u_02 = dot3(X2.dr, c[1][0], c[1][1], c[1][2]);
      const float u_1 = dot3(X2.br, c[2][0], c[2][1], c[2][2]);
      const float u_12 = dot3(X2.dr, c[2][0], c[2][1], c[2][2]);
      const float u_00 = dot3(X2.br, c[3][0], c[3][1], c[3][2]);
      const float u_11 = dot3(X2.br, c[4][0], c[4][1], c[4][2]);
      const float u_01 = dot3(X2.br, c[5][0], c[5][1], c[5][2]);
      const float g[3] = {u_0, u_1, u_2};
      const float h[6] = {u_00, u_01, u_02, u_11, u_12, u_22};   // pair order (00,01,02,11,12,22)
      float f0 = F[kM] * u;
#pragma unroll
      for (int a = 0; a < 3; ++a) f0 = fmaf(F[kC + a], g[a], f0);
      if (LIN) {
        const float xi[3] = {gpt(l0), gpt(l1), gpt(l2)};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const float s = fmaf(F[kL + 3 * a + 2], xi[2],
                               fmaf(F[kL + 3 * a + 1], xi[1], F[kL + 3 * a] * xi[0]));
          f0 = fmaf(s, g[a], f0);
        }
      }
      // symmetric K from the six pair factors
      const float K00 = F[kS], K01 = F[kS + 1], K02 = F[kS + 2], K11 = F[kS + 3],
                  K12 = F[kS + 4], K22 = F[kS + 5];
      float f1 = fmaf(K02, u_2, fmaf(K01, u_1, K00 * u_0));
      float f2 = fmaf(K12, u_2, fmaf(K11, u_1, K01 * u_0));
      float f3 = fmaf(K22, u_2, fmaf(K12, u_1, K02 * u_0));
      f1 = fmaf(F[kD], u, f1);
      f2 = fmaf(F[kD + 1], u, f2);
      f3 = fmaf(F[kD + 2], u, f3);
#pragma unroll
      for (int s = 0; s < 6; ++s) {
        f1 = fmaf(F[kT + 3 * s], h[s], f1);
        f2 = fmaf(F[kT + 3 * s + 1], h[s], f2);
        f3 = fmaf(F[kT + 3 * s + 2], h[s], f3);
      }
      // buffers 0..3 are free: this phase reads 4..9 only
      B[0][lane] = wq * f0;
      B[1][lane] = wq * f1;
      B[2][lane] = wq * f2;
      B[3][lane] = wq * f3;
    }
    __syncwarp();
    // transposed direction 2: lane (q0, q1, i2)
    if (act) {
      const int o = l0 + 3 * l1;
      float g[4][3];
#pragma unroll
      for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int j = 0; j < 3; ++j) g[k][j] = B[k][o + 9 * j];
      B[4][lane] = dot3(X2.bc, g[0][0], g[0][1], g[0][2]);   // value path
      B[5][lane] = dot3(X2.bc, g[1][0], g[1][1], g[1][2]);   // d/dxi_0 path
      B[6][lane] = dot3(X2.bc, g[2][0], g[2][1], g[2][2]);   // d/dxi_1 path
      B[7][lane] = dot3(X2.dc, g[3][0], g[3][1], g[3][2]);   // d/dxi_2 path
    }
    __syncwarp();
    // transposed direction 1: lane (q0, i1, i2)
    if (act) {
      const int o = l0 + 9 * l2;
      const float p00 = B[4][o], p01 = B[4][o + 3], p02 = B[4][o + 6];
      const float p10 = B[5][o], p11 = B[5][o + 3], p12 = B[5][o + 6];
      const float p20 = B[6][o], p21 = B[6][o + 3], p22 = B[6][o + 6];
      const float p30 = B[7][o], p31 = B[7][o + 3], p32 = B[7][o + 6];
      B[0][lane] = dot3(X1.bc, p00 + p30, p01 + p31, p02 + p32) + dot3(X1.dc, p20, p21, p22);
      B[1][lane] = dot3(X1.bc, p10, p11, p12);
    }
    __syncwarp();
    // transposed direction 0: lane (i0, i1, i2) = local DOF
    if (act) {
      const int o = 3 * l1 + 9 * l2;
      const float y = dot3(X0.bc, B[0][o], B[0][o + 1], B[0][o + 2]) +
                      dot3(X0.dc, B[1][o], B[1][o + 1], B[1][o + 2]);
      const int ps = __ldg(pos + (size_t)cell * 27 + lane);
      if (ps >= 0) ycell[ps] = y;
    }
    __syncwarp();   // buffers 0, 1 and the factors are rewritten for the next cell
  }
}

// A uniform level (every cell a translate of cell 0, constant coefficients):
// with each cell's DOFs in cell 0's local order (gdof_c, pos_c), all cells
// share cell 0's element matrix.  Lane m keeps row m of the 27 x 27 FP32
// matrix in registers for the whole launch; per cell it gathers one local
// value, broadcasts the 27 values by shuffles and forms its row's product
// -- 27 multiply-adds per lane in place of the sum-factorised ~124 and the
// shared-memory passes -- and stores it at its gather position
__global__ void __launch_bounds__(256)
k_mf_uniform(int ncells, const int* __restrict__ gdof_c, const int* __restrict__ pos_c,
             const float* __restrict__ AeT, const float* __restrict__ x,
             float* __restrict__ ycell) {
  pdl_enter();
  const int lane = threadIdx.x & 31;
  const int il = lane < 27 ? lane : 26;
  float a[27];
#pragma unroll
  for (int j = 0; j < 27; ++j) a[j] = __ldg(AeT + j * 27 + il);
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int cell = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); cell < ncells;
       cell += nw) {
    const size_t o = (size_t)cell * 27;
    float xv = 0.f;
    int ps = -1;
    if (lane < 27) {
      xv = __ldg(x + __ldg(gdof_c + o + lane));
      ps = __ldg(pos_c + o + lane);
    }
    float y = 0.f;
#pragma unroll
    for (int j = 0; j < 27; ++j) y = fmaf(a[j], __shfl_sync(0xffffffffu, xv, j), y);
    if (ps >= 0) ycell[ps] = y;
  }
}

// per-row update from the local results (a contiguous range per active
// row), in the modes of k_spmv:
//   0: y = A x, 1: y = b - A x, 2: y = x + w D^-1 (b - A x),
//   3: mode 2, and y also in FP64 into z (block *di when given) and zcur
template <int MODE>
__global__ void __launch_bounds__(256)
k_mf_gather(int n, int nactive, const int* __restrict__ dof_rp,
            const float* __restrict__ ycell, const float* __restrict__ x,
            const float* __restrict__ b, const float* __restrict__ invd, float w,
            float* __restrict__ y, double* __restrict__ z, const int* di,
            double* __restrict__ zcur) {
  pdl_enter();
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  const float xr = x[row];
  float s;
  if (row < nactive) {
    s = 0.f;
    const int e1 = dof_rp[row + 1];
    for (int e = dof_rp[row]; e < e1; ++e) s += ycell[e];
  } else {
    s = xr;
  }
  if (MODE == 0) {
    y[row] = s;
  } else if (MODE == 1) {
    y[row] = b[row] - s;
  } else {
    const float yr = xr + w * (invd[row] * (b[row] - s));
    y[row] = yr;
    if (MODE == 3) {
      const double zr = (double)yr;
      (di ? z + (size_t)(*di) * n : z)[row] = zr;
      if (zcur) zcur[row] = zr;
    }
  }
}

// One launch per sweep on a uniform level: the product and the row update of
// k_mf_uniform + k_mf_gather with the local results kept in shared memory.
// Block t owns rows [256 t, 256 t + 256) and recomputes every cell that
// touches them (the cells of neighbouring tiles are computed again, about 2.5
// times the cells on a 32^3 Q2 level): (1) the cells' x values, cell-major,
// 28 floats per cell, from the tile's DOF list; (2) a warp per cell, lane m
// forms row m of the element product from the 27 values (seven broadcast
// 16-byte loads) and writes it over the cell's x values; (3) a thread per row
// sums its entries in the DOF-major order.  The same multiply-adds in the
// same order as the two-kernel path: the results agree bit for bit.
// (Measured on GB300, 32^3 Q2 finest level: 14.4 us per Jacobi step against
// 16.4 us for the two kernels; forming only the (cell, row) products the
// tile's rows need, grouped by row, cut the instructions by a quarter but
// took 16.4 us: its 16-byte loads of different cells conflict in shared
// memory where the warp-per-cell loads broadcast.)
template <int MODE, int MINB>
__global__ void __launch_bounds__(kMfTileRows, MINB)
k_mf_fused(int n, int nactive, const int* __restrict__ tile_rp,
           const int* __restrict__ tile_gdof, const float* __restrict__ AeT,
           const int* __restrict__ dof_rp, const int* __restrict__ ent_loc,
           const float* __restrict__ x, const float* __restrict__ b,
           const float* __restrict__ invd, float w, float* __restrict__ y,
           double* __restrict__ z, const int* di, double* __restrict__ zcur) {
  pdl_enter();
  extern __shared__ float4 s_cell4[];
  float* s_cell = reinterpret_cast<float*>(s_cell4);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int c0 = tile_rp[blockIdx.x], nc = tile_rp[blockIdx.x + 1] - c0;
  const int row = blockIdx.x * kMfTileRows + tid;
  // the row's entries (up to kMfRowRegs slots in registers) are fetched
  // while the cell values arrive
  int e0 = 0, e1 = 0;
  if (row < nactive) {
    e0 = __ldg(dof_rp + row);
    e1 = __ldg(dof_rp + row + 1);
  }
  // (1) the tile's DOF list, coalesced, in batches of kMfGather entries per
  // thread: every load of a batch is issued before the first one is used
  const int* tg = tile_gdof + (size_t)c0 * kMfCellStride;
  const int ne = nc * kMfCellStride;
  for (int base = 0; base < ne; base += kMfGather * kMfTileRows) {
    int g[kMfGather];
#pragma unroll
    for (int k = 0; k < kMfGather; ++k) {
      const int q = base + k * kMfTileRows + tid;
      g[k] = q < ne ? __ldg(tg + q) : -1;
    }
#pragma unroll
    for (int k = 0; k < kMfGather; ++k) {
      const int q = base + k * kMfTileRows + tid;
      if (q < ne) s_cell[q] = __ldg(x + g[k]);
    }
  }
  int slot[kMfRowRegs];
#pragma unroll
  for (int k = 0; k < kMfRowRegs; ++k) slot[k] = e0 + k < e1 ? __ldg(ent_loc + e0 + k) : 0;
  float xr = 0.f, br = 0.f, dr = 0.f;
  if (row < n) {
    xr = x[row];
    if (MODE >= 1) br = b[row];
    if (MODE >= 2) dr = invd[row];
  }
  const int il = lane < 27 ? lane : 26;
  float a[27];
#pragma unroll
  for (int j = 0; j < 27; ++j) a[j] = __ldg(AeT + j * 27 + il);
  __syncthreads();
  // (2) element products, a warp per cell, lane m = row m of the element matrix
  for (int cl = warp; cl < nc; cl += kMfTileRows / 32) {
    const float4* xc = s_cell4 + cl * (kMfCellStride / 4);
    float acc = 0.f;
#pragma unroll
    for (int jj = 0; jj < 7; ++jj) {
      const float4 v = xc[jj];
      acc = fmaf(a[4 * jj], v.x, acc);
      acc = fmaf(a[4 * jj + 1], v.y, acc);
      acc = fmaf(a[4 * jj + 2], v.z, acc);
      if (jj < 6) acc = fmaf(a[4 * jj + 3], v.w, acc);
    }
    __syncwarp();
    if (lane < 27) s_cell[cl * kMfCellStride + lane] = acc;
  }
  __syncthreads();
  // (3) the row sums and the update
  if (row >= n) return;
  float s;
  if (row < nactive) {
    s = 0.f;
#pragma unroll
    for (int k = 0; k < kMfRowRegs; ++k)
      if (e0 + k < e1) s += s_cell[slot[k]];
    for (int e = e0 + kMfRowRegs; e < e1; ++e) s += s_cell[__ldg(ent_loc + e)];
  } else {
    s = xr;
  }
  if (MODE == 0) {
    y[row] = s;
  } else if (MODE == 1) {
    y[row] = br - s;
  } else {
    const float yr = xr + w * (dr * (br - s));
    y[row] = yr;
    if (MODE == 3) {
      const double zr = (double)yr;
      (di ? z + (size_t)(*di) * n : z)[row] = zr;
      if (zcur) zcur[row] = zr;
    }
  }
}

// ---------------------------------------------------------------------------
// Lattice stencil sweep of a uniform level.  The DOFs of a uniform Q2 mesh
// sit on a lattice of half-cell spacing; a point with odd coordinate d lies
// inside one cell along d, one with even coordinate on the face between two,
// so an active row (an interior point) couples to the points within 1 (odd)
// or 2 (even) along each direction, with the sum over the cells around the
// point of the element matrix entries: one of eight 125-point stencils,
// chosen by the parities of the point (zeros outside the couplings).
//
// Block: 32 (x) x kStTY (y) lattice columns of ZT points along z, starting
// at odd z; the x values of the block's points and a halo of two are staged
// in shared memory through the lattice map (z innermost, a 12-float column
// per (x, y): three conflict-free 16-byte loads), a staged column per
// thread.  Five threads share a column, one per stencil plane dy: per dx
// each loads its column and the eight z coefficients of its (x, y) parity
// (odd z points couple to dz = -1..1, even ones to -2..2) and adds to its ZT
// partial sums (32 multiply-adds per 5 shared loads); the planes' partials
// meet in shared memory and are summed in plane order.  The b and D^-1 of
// the rows a thread finishes are loaded before the products.  Rows of
// non-active DOFs (identity) are taken by the blocks past the lattice tiles.
// ---------------------------------------------------------------------------
constexpr int kStTX = 32, kStTY = 4, kStDY = 5;
constexpr int kStThreads = kStTX * kStTY * kStDY;   // 640
constexpr int kStXS = kStTX + 4, kStYS = kStTY + 4, kStZS = 12;
constexpr int kStCoef = 4 * 25 * 8;   // (x, y parity) x (dy, dx) x 8 z slots

// the row update of the k_spmv modes from the row sum s, with the row's b
// and D^-1 already loaded
template <int MODE>
__device__ __forceinline__ void st_finish(int row, int n, float xr, float s, float br, float dr,
                                          float w, float* __restrict__ y,
                                          double* __restrict__ z, const int* di,
                                          double* __restrict__ zcur) {
  if (MODE == 0) {
    y[row] = s;
  } else if (MODE == 1) {
    y[row] = br - s;
  } else {
    const float yr = xr + w * (dr * (br - s));
    y[row] = yr;
    if (MODE == 3) {
      const double zr = (double)yr;
      (di ? z + (size_t)(*di) * n : z)[row] = zr;
      if (zcur) zcur[row] = zr;
    }
  }
}

// the eight stencils from the element matrix (A(row, col) = AeT[col * 27 +
// row], local index ix + 3 iy + 9 iz in cell 0's frame).  Entry t: slot
// s = t % 8 (0..2: odd z, dz = -1..1; 3..7: even z, dz = -2..2), offsets
// dx, dy = (t / 8) % 25 as (dx + 2) + 5 (dy + 2), parities cls = t / 200 as
// (x odd) + 2 (y odd).  Summed in FP64 over the cells around the point in a
// fixed order, rounded once.
__global__ void k_st_coef(const float* __restrict__ AeT, float* __restrict__ coef) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= kStCoef) return;
  const int s = t % 8, pair = t / 8, dxy = pair % 25, cls = pair / 25;
  const int par[3] = {cls & 1, cls >> 1, s < 3 ? 1 : 0};
  const int off[3] = {dxy % 5 - 2, dxy / 5 - 2, s < 3 ? s - 1 : s - 5};
  double a = 0.0;
  for (int c = 0; c < 8; ++c) {
    int r[3], q[3];
    bool ok = true;
    for (int d = 0; d < 3; ++d) {
      const int side = (c >> d) & 1;
      if (par[d]) {
        if (side) ok = false;   // one cell along d
        r[d] = 1;
      } else {
        r[d] = side ? 2 : 0;    // the cell below (local 2) or above (local 0)
      }
      q[d] = r[d] + off[d];
      if (q[d] < 0 || q[d] > 2) ok = false;
    }
    if (!ok) continue;
    const int row = r[0] + 3 * r[1] + 9 * r[2], col = q[0] + 3 * q[1] + 9 * q[2];
    a += (double)AeT[col * 27 + row];
  }
  coef[t] = (float)a;
}

template <int MODE, int ZT>
__global__ void __launch_bounds__(kStThreads, 2)
k_mf_stencil(int n, int nactive, int lx, int ly, int lz, int bx, int by, int nst,
             const int* __restrict__ lmap, const float* __restrict__ coef,
             const float* __restrict__ x, const float* __restrict__ b,
             const float* __restrict__ invd, float w, float* __restrict__ y,
             double* __restrict__ z, const int* di, double* __restrict__ zcur) {
  static_assert(ZT % 4 == 0 && ZT + 4 <= kStZS, "z column of ZT points and a halo of two");
  constexpr int NO = ZT * kStTY * kStTX;   // points of the block
  static_assert(NO <= 2 * kStThreads, "two finished points per thread at most");
  pdl_enter();
  __shared__ __align__(16) float s_x[kStYS * kStXS * kStZS];
  __shared__ __align__(16) float s_c[kStCoef];
  __shared__ float s_p[kStDY * NO];
  __shared__ int s_g[NO];
  const int tid = threadIdx.x;
  if ((int)blockIdx.x >= nst) {
    const int row = nactive + ((int)blockIdx.x - nst) * kStThreads + tid;
    if (row < n) {
      const float xr = x[row];
      st_finish<MODE>(row, n, xr, xr, MODE >= 1 ? b[row] : 0.f, MODE >= 2 ? invd[row] : 0.f, w,
                      y, z, di, zcur);
    }
    return;
  }
  const int bxi = (int)blockIdx.x % bx, rest = (int)blockIdx.x / bx;
  const int X0 = 1 + bxi * kStTX, Y0 = 1 + (rest % by) * kStTY, Z0 = 1 + (rest / by) * ZT;
  for (int i = tid; i < kStCoef; i += kStThreads) s_c[i] = __ldg(coef + i);
  // stage the tile: a thread per (x, y) column of the tile and its halo
  // loads the column's ZT + 4 lattice map entries, then their x values, and
  // stores the column as 16-byte words (conflict-free, as the loads below)
  constexpr int NCOL = kStXS * kStYS;
  static_assert(NCOL <= kStThreads, "one staged column per thread");
  if (tid < NCOL) {
    const int qx = tid % kStXS, qy = tid / kStXS;
    const int ax = X0 - 2 + qx, ay = Y0 - 2 + qy;
    const bool in = ax >= 0 && ax < lx && ay >= 0 && ay < ly;
    const int* mp = lmap + (in ? (size_t)ay * lx + ax : 0);
    const size_t plane = (size_t)lx * ly;
    int g[ZT + 4];
#pragma unroll
    for (int qz = 0; qz < ZT + 4; ++qz) {
      const int az = Z0 - 2 + qz;
      g[qz] = in && az >= 0 && az < lz ? __ldg(mp + (size_t)az * plane) : -1;
    }
    float v[ZT + 4];
#pragma unroll
    for (int qz = 0; qz < ZT + 4; ++qz) v[qz] = g[qz] >= 0 ? __ldg(x + g[qz]) : 0.f;
    float4* dst = reinterpret_cast<float4*>(s_x + (qy * kStXS + qx) * kStZS);
#pragma unroll
    for (int j = 0; j < (ZT + 4) / 4; ++j)
      dst[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
    if (qx >= 2 && qx < 2 + kStTX && qy >= 2 && qy < 2 + kStTY) {
#pragma unroll
      for (int k = 0; k < ZT; ++k) s_g[(k * kStTY + qy - 2) * kStTX + qx - 2] = g[k + 2];
    }
  }
  __syncthreads();
  // the points this thread finishes (o = tid, tid + kStThreads): their rows'
  // b and D^-1 are in flight during the products
  int orow[2] = {-1, -1};
  float ob[2] = {0.f, 0.f}, od[2] = {0.f, 0.f};
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int o = tid + u * kStThreads;
    if (o < NO) {
      const int k = o / (kStTY * kStTX), ty = (o / kStTX) % kStTY, tx = o % kStTX;
      if (X0 + tx <= lx - 2 && Y0 + ty <= ly - 2 && Z0 + k <= lz - 2) {
        orow[u] = s_g[o];
        if (MODE >= 1) ob[u] = __ldg(b + orow[u]);
        if (MODE >= 2) od[u] = __ldg(invd + orow[u]);
      }
    }
  }
  const int tx = tid % kStTX, ty = (tid / kStTX) % kStTY, dy = tid / (kStTX * kStTY);
  const int ax = X0 + tx, ay = Y0 + ty;
  const float* cb = s_c + ((ax & 1) | ((ay & 1) << 1)) * 200 + dy * 40;
  float acc[ZT];
#pragma unroll
  for (int k = 0; k < ZT; ++k) acc[k] = 0.f;
  // a point at odd y couples to dy = -1..1 only: the planes dy = +-2 of such
  // rows (whole warps: a warp is one (y, dy)) have zero coefficients
  const bool plane = !((ay & 1) && (dy == 0 || dy == 4));
#pragma unroll
  for (int dx = 0; dx < 5; ++dx) {
    if (!plane) break;
    const float4* cp = reinterpret_cast<const float4*>(s_x + ((ty + dy) * kStXS + tx + dx) * kStZS);
    float col[ZT + 4];
#pragma unroll
    for (int j = 0; j < (ZT + 4) / 4; ++j) {
      const float4 v = cp[j];
      col[4 * j] = v.x;
      col[4 * j + 1] = v.y;
      col[4 * j + 2] = v.z;
      col[4 * j + 3] = v.w;
    }
    const float4 c0 = *reinterpret_cast<const float4*>(cb + dx * 8);
    const float4 c1 = *reinterpret_cast<const float4*>(cb + dx * 8 + 4);
#pragma unroll
    for (int k = 0; k < ZT; k += 2) {
      // lattice z = Z0 + k is odd: dz = -1, 0, 1 at col[k + 2 + dz]
      acc[k] = fmaf(c0.x, col[k + 1], acc[k]);
      acc[k] = fmaf(c0.y, col[k + 2], acc[k]);
      acc[k] = fmaf(c0.z, col[k + 3], acc[k]);
      // z = Z0 + k + 1 is even: dz = -2 .. 2 at col[k + 3 + dz]
      acc[k + 1] = fmaf(c0.w, col[k + 1], acc[k + 1]);
      acc[k + 1] = fmaf(c1.x, col[k + 2], acc[k + 1]);
      acc[k + 1] = fmaf(c1.y, col[k + 3], acc[k + 1]);
      acc[k + 1] = fmaf(c1.z, col[k + 4], acc[k + 1]);
      acc[k + 1] = fmaf(c1.w, col[k + 5], acc[k + 1]);
    }
  }
#pragma unroll
  for (int k = 0; k < ZT; ++k) s_p[dy * NO + (k * kStTY + ty) * kStTX + tx] = acc[k];
  __syncthreads();
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    if (orow[u] < 0) continue;
    const int o = tid + u * kStThreads;
    const int k = o / (kStTY * kStTX), oy = (o / kStTX) % kStTY, ox = o % kStTX;
    float sum = s_p[o];
#pragma unroll
    for (int d = 1; d < kStDY; ++d) sum += s_p[d * NO + o];
    const float xr = s_x[((oy + 2) * kStXS + ox + 2) * kStZS + k + 2];
    st_finish<MODE>(orow[u], n, xr, sum, ob[u], od[u], w, y, z, di, zcur);
  }
}

}  // namespace

// the sweep's register budget: 4, 5 or 6 resident blocks per SM (64, 48 or
// 40 registers; the tuner times them, L.mf_fused_minb)
template <int MINB>
static int fused_smem_attr(int smem) {
  CDG_CUDA(cudaFuncSetAttribute(k_mf_fused<0, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  CDG_CUDA(cudaFuncSetAttribute(k_mf_fused<1, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  CDG_CUDA(cudaFuncSetAttribute(k_mf_fused<2, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  CDG_CUDA(cudaFuncSetAttribute(k_mf_fused<3, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  return CDG_OK;
}

template <int MODE>
static int fused_launch(cdg_context* ctx, const DevLevel& L, int g, size_t sm, const float* x,
                        const float* b, const float* invd, float w, float* y, double* z,
                        const int* di, double* zcur) {
  switch (L.mf_fused_minb) {
    case 5:
      CDG_LAUNCH_PDL(ctx, (k_mf_fused<MODE, 5>), g, kMfTileRows, sm, L.ndof, L.nactive, L.mf_tile_rp, L.mf_tile_gdof, L.mf_ae, L.dof_rp, L.mf_ent_loc, x, b, invd, w, y, z, di, zcur);
      break;
    case 6:
      CDG_LAUNCH_PDL(ctx, (k_mf_fused<MODE, 6>), g, kMfTileRows, sm, L.ndof, L.nactive, L.mf_tile_rp, L.mf_tile_gdof, L.mf_ae, L.dof_rp, L.mf_ent_loc, x, b, invd, w, y, z, di, zcur);
      break;
    default:
      CDG_LAUNCH_PDL(ctx, (k_mf_fused<MODE, 4>), g, kMfTileRows, sm, L.ndof, L.nactive, L.mf_tile_rp, L.mf_tile_gdof, L.mf_ae, L.dof_rp, L.mf_ent_loc, x, b, invd, w, y, z, di, zcur);
      break;
  }
  return CDG_OK;
}

// Tiles of the one-launch sweep, from the DOF-major positions of the cells'
// local DOFs in cell 0's frame (mf_pos_c): tile t lists the cells that own an
// entry of its active rows in first-use order (their DOFs padded to
// kMfCellStride), and every entry gets the shared-memory slot of its (tile
// cell, local DOF).  Levels whose largest tile does not fit one block's
// shared memory keep the two-kernel sweep, as do all levels when
// CDG_MF_FUSED=0 is set at the first assembly.
int mf_build_tiles(cdg_context* ctx, DevLevel& L) {
  L.mf_ntiles = 0;
  const int n = L.ndof, na = L.nactive, nc = L.ncells;
  const char* off = std::getenv("CDG_MF_FUSED");   // 0: keep the two-kernel sweep
  if (na == 0 || nc == 0 || (off && off[0] == '0')) return CDG_OK;
  std::vector<int> rp(na + 1), posc((size_t)nc * 27), gdc((size_t)nc * 27);
  CDG_CUDA(cudaMemcpyAsync(rp.data(), L.dof_rp, rp.size() * sizeof(int), cudaMemcpyDeviceToHost,
                           ctx->stream));
  CDG_CUDA(cudaMemcpyAsync(posc.data(), L.mf_pos_c, posc.size() * sizeof(int),
                           cudaMemcpyDeviceToHost, ctx->stream));
  CDG_CUDA(cudaMemcpyAsync(gdc.data(), L.mf_gdof, gdc.size() * sizeof(int),
                           cudaMemcpyDeviceToHost, ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  const int nent = rp[na];
  std::vector<int> ent_cell(nent, -1), ent_i(nent, 0);
  for (int c = 0; c < nc; ++c)
    for (int i = 0; i < 27; ++i) {
      const int e = posc[(size_t)c * 27 + i];
      if (e < 0) continue;
      if (e >= nent || ent_cell[e] >= 0) {
        set_error("matrix-free positions are not a permutation of the DOF-major entries");
        return CDG_ERR_ARG;
      }
      ent_cell[e] = c;
      ent_i[e] = i;
    }
  const int ntiles = (n + kMfTileRows - 1) / kMfTileRows;
  std::vector<int> trp(ntiles + 1, 0), tcells, loc(nent), mark(nc, -1), local(nc, 0);
  tcells.reserve((size_t)nc * 3);
  int maxc = 0;
  for (int t = 0; t < ntiles; ++t) {
    const int ra = std::min(t * kMfTileRows, na), rb = std::min((t + 1) * kMfTileRows, na);
    const int start = (int)tcells.size();
    for (int e = rp[ra]; e < rp[rb]; ++e) {
      const int c = ent_cell[e];
      if (c < 0) {
        set_error("matrix-free positions leave a DOF-major entry unset");
        return CDG_ERR_ARG;
      }
      if (mark[c] != t) {
        mark[c] = t;
        local[c] = (int)tcells.size() - start;
        tcells.push_back(c);
      }
      loc[e] = local[c] * kMfCellStride + ent_i[e];
    }
    trp[t + 1] = (int)tcells.size();
    maxc = std::max(maxc, trp[t + 1] - start);
  }
  const size_t smem = (size_t)maxc * kMfCellStride * sizeof(float);
  if (smem > 200 * 1024) return CDG_OK;
  // the tile cells' DOFs in cell 0's order, padded with the cell's first DOF
  std::vector<int> tg(tcells.size() * kMfCellStride);
  for (size_t c = 0; c < tcells.size(); ++c)
    for (int i = 0; i < kMfCellStride; ++i)
      tg[c * kMfCellStride + i] = gdc[(size_t)tcells[c] * 27 + (i < 27 ? i : 0)];
  if (!L.mf_tile_rp) {
    CDG_CUDA(cudaMalloc(&L.mf_tile_rp, trp.size() * sizeof(int)));
    CDG_CUDA(cudaMalloc(&L.mf_tile_gdof, std::max<size_t>(1, tg.size()) * sizeof(int)));
    CDG_CUDA(cudaMalloc(&L.mf_ent_loc, std::max(1, nent) * sizeof(int)));
  }
  CDG_CUDA(cudaMemcpyAsync(L.mf_tile_rp, trp.data(), trp.size() * sizeof(int),
                           cudaMemcpyHostToDevice, ctx->stream));
  if (!tg.empty())
    CDG_CUDA(cudaMemcpyAsync(L.mf_tile_gdof, tg.data(), tg.size() * sizeof(int),
                             cudaMemcpyHostToDevice, ctx->stream));
  if (nent > 0)
    CDG_CUDA(cudaMemcpyAsync(L.mf_ent_loc, loc.data(), (size_t)nent * sizeof(int),
                             cudaMemcpyHostToDevice, ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));   // host vectors go out of scope
  if (smem > 48 * 1024) {
    CDG_TRY(fused_smem_attr<4>((int)smem));
    CDG_TRY(fused_smem_attr<5>((int)smem));
    CDG_TRY(fused_smem_attr<6>((int)smem));
  }
  L.mf_tile_maxcells = maxc;
  L.mf_ntiles = ntiles;
  return CDG_OK;
}

// The DOF lattice of a uniform level, from the cells' DOFs in cell 0's frame
// (mf_gdof): cells sharing a face-centre DOF are neighbours along that
// face's axis, so a walk from cell 0 places every cell at integer offsets;
// local DOF (ix, iy, iz) of the cell at offset o sits at lattice point
// 2 o + (ix, iy, iz).  The stencil sweep needs a full box of cells, one DOF
// per lattice point and the active DOFs exactly at the interior points
// (Dirichlet data on the whole boundary); any level that is not such a
// lattice keeps st_dims zero.
int mf_build_lattice(cdg_context* ctx, DevLevel& L) {
  L.st_dims[0] = L.st_dims[1] = L.st_dims[2] = 0;
  const int nc = L.ncells, n = L.ndof, na = L.nactive;
  if (nc == 0 || na == 0 || L.mf_geo != 1) return CDG_OK;
  std::vector<int> gdc((size_t)nc * 27);
  CDG_CUDA(cudaMemcpyAsync(gdc.data(), L.mf_gdof, gdc.size() * sizeof(int),
                           cudaMemcpyDeviceToHost, ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));
  // face-centre local DOFs: -x, +x, -y, +y, -z, +z
  static const int kFace[6] = {12, 14, 10, 16, 4, 22};
  std::vector<int> fa(n, -1), fb(n, -1);   // the (cell, face) holders of a DOF
  for (int c = 0; c < nc; ++c)
    for (int f = 0; f < 6; ++f) {
      const int g = gdc[(size_t)c * 27 + kFace[f]];
      if (g < 0 || g >= n) return CDG_OK;
      if (fa[g] < 0) fa[g] = c * 6 + f;
      else if (fb[g] < 0) fb[g] = c * 6 + f;
      else return CDG_OK;   // a face-centre DOF in three cells
    }
  std::vector<int> off((size_t)nc * 3, 0), seen(nc, 0), queue;
  queue.reserve(nc);
  queue.push_back(0);
  seen[0] = 1;
  for (size_t h = 0; h < queue.size(); ++h) {
    const int c = queue[h];
    for (int f = 0; f < 6; ++f) {
      const int g = gdc[(size_t)c * 27 + kFace[f]];
      const int other = fa[g] == c * 6 + f ? fb[g] : fa[g];
      if (other < 0) continue;   // boundary face
      const int c2 = other / 6, f2 = other % 6;
      if (f2 != (f ^ 1)) return CDG_OK;   // not a translate across the face
      int o[3] = {off[(size_t)c * 3], off[(size_t)c * 3 + 1], off[(size_t)c * 3 + 2]};
      o[f / 2] += (f & 1) ? 1 : -1;
      if (seen[c2]) {
        for (int d = 0; d < 3; ++d)
          if (off[(size_t)c2 * 3 + d] != o[d]) return CDG_OK;
        continue;
      }
      seen[c2] = 1;
      for (int d = 0; d < 3; ++d) off[(size_t)c2 * 3 + d] = o[d];
      queue.push_back(c2);
    }
  }
  if ((int)queue.size() != nc) return CDG_OK;   // not connected through faces
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int c = 0; c < nc; ++c)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], off[(size_t)c * 3 + d]);
      hi[d] = std::max(hi[d], off[(size_t)c * 3 + d]);
    }
  long ld[3], npts = 1, ncb = 1;
  for (int d = 0; d < 3; ++d) {
    ld[d] = 2L * (hi[d] - lo[d] + 1) + 1;
    npts *= ld[d];
    ncb *= hi[d] - lo[d] + 1;
  }
  if (ncb != nc || npts != n) return CDG_OK;   // not a full box, or not one DOF per point
  std::vector<int> map((size_t)npts, -1), inv(n, -1);
  for (int c = 0; c < nc; ++c)
    for (int m = 0; m < 27; ++m) {
      const long px = 2L * (off[(size_t)c * 3] - lo[0]) + m % 3;
      const long py = 2L * (off[(size_t)c * 3 + 1] - lo[1]) + (m / 3) % 3;
      const long pz = 2L * (off[(size_t)c * 3 + 2] - lo[2]) + m / 9;
      const long idx = (pz * ld[1] + py) * ld[0] + px;
      const int g = gdc[(size_t)c * 27 + m];
      if (g < 0 || g >= n) return CDG_OK;
      if (map[idx] >= 0 && map[idx] != g) return CDG_OK;
      if (inv[g] >= 0 && inv[g] != idx) return CDG_OK;
      map[idx] = g;
      inv[g] = (int)idx;
    }
  for (long idx = 0; idx < npts; ++idx) {
    if (map[idx] < 0) return CDG_OK;
    const long px = idx % ld[0], py = (idx / ld[0]) % ld[1], pz = idx / (ld[0] * ld[1]);
    const bool interior = px > 0 && px < ld[0] - 1 && py > 0 && py < ld[1] - 1 && pz > 0 &&
                          pz < ld[2] - 1;
    if (interior != (map[idx] < na)) return CDG_OK;
  }
  if (L.st_map) cudaFree(L.st_map);
  L.st_map = nullptr;
  CDG_CUDA(cudaMalloc(&L.st_map, (size_t)npts * sizeof(int)));
  if (!L.st_coef) CDG_CUDA(cudaMalloc(&L.st_coef, kStCoef * sizeof(float)));
  CDG_CUDA(cudaMemcpyAsync(L.st_map, map.data(), (size_t)npts * sizeof(int),
                           cudaMemcpyHostToDevice, ctx->stream));
  CDG_CUDA(cudaStreamSynchronize(ctx->stream));   // the host map goes out of scope
  for (int d = 0; d < 3; ++d) L.st_dims[d] = (int)ld[d];
  return CDG_OK;
}

int mf_stencil_coef(cdg_context* ctx, DevLevel& L) {
  if (L.st_dims[0] == 0) return CDG_OK;
  CDG_LAUNCH(ctx, k_st_coef, (kStCoef + 255) / 256, 256, 0, L.mf_ae, L.st_coef);
  return CDG_OK;
}

template <int MODE, int ZT>
static int stencil_launch(cdg_context* ctx, const DevLevel& L, const float* x, const float* b,
                          const float* invd, float w, float* y, double* z, const int* di,
                          double* zcur) {
  const int lx = L.st_dims[0], ly = L.st_dims[1], lz = L.st_dims[2];
  const int bx = (lx - 2 + kStTX - 1) / kStTX, by = (ly - 2 + kStTY - 1) / kStTY;
  const int bz = (lz - 2 + ZT - 1) / ZT;
  const int nst = bx * by * bz;
  const int nb = nst + (L.ndof - L.nactive + kStThreads - 1) / kStThreads;
  CDG_LAUNCH_PDL(ctx, (k_mf_stencil<MODE, ZT>), nb, kStThreads, 0, L.ndof, L.nactive, lx, ly,
                 lz, bx, by, nst, L.st_map, L.st_coef, x, b, invd, w, y, z, di, zcur);
  return CDG_OK;
}

template <int ZT>
static int stencil_mode(cdg_context* ctx, const DevLevel& L, int mode, const float* x,
                        const float* b, const float* invd, float w, float* y, double* z,
                        const int* di, double* zcur) {
  switch (mode) {
    case 0: return stencil_launch<0, ZT>(ctx, L, x, b, invd, w, y, z, di, zcur);
    case 1: return stencil_launch<1, ZT>(ctx, L, x, b, invd, w, y, z, di, zcur);
    case 2: return stencil_launch<2, ZT>(ctx, L, x, b, invd, w, y, z, di, zcur);
    default: return stencil_launch<3, ZT>(ctx, L, x, b, invd, w, y, z, di, zcur);
  }
}

bool mf_eligible(const DevLevel& L) {
  return L.shape == kHexa && L.order == 2 && !L.multilinear;
}

int mf_ensure(DevLevel& L) {
  if (L.mf_fac) return CDG_OK;
  CDG_CUDA(cudaMalloc(&L.mf_fac, (size_t)L.ncells * kMfFactors * sizeof(float)));
  CDG_CUDA(cudaMalloc(&L.mf_y, (size_t)L.ncells * 27 * sizeof(float)));
  CDG_CUDA(cudaMalloc(&L.mf_ae, 27 * 27 * sizeof(float)));
  CDG_CUDA(cudaMalloc(&L.mf_pos, (size_t)L.ncells * 27 * sizeof(int)));
  CDG_CUDA(cudaMalloc(&L.mf_gdof, (size_t)L.ncells * 27 * sizeof(int)));
  CDG_CUDA(cudaMalloc(&L.mf_pos_c, (size_t)L.ncells * 27 * sizeof(int)));
  CDG_CUDA(cudaMalloc(&L.mf_loc, (size_t)L.ncells * 27 * sizeof(int)));
  CDG_CUDA(cudaMalloc(&L.ue64, 27 * 27 * sizeof(double)));
  return CDG_OK;
}

int mf_apply(cdg_context* ctx, const DevLevel& L, int mode, const float* x, const float* b,
             const float* invd, float w, float* y, double* z, const int* di, double* zcur,
             int form) {
  if (!L.mf_valid) {
    set_error("matrix-free operator used without valid cell factors");
    return CDG_ERR_ARG;
  }
  const bool lattice = L.mf_uniform && L.st_dims[0] > 0;
  if (form == kMfStencil && !lattice) {
    set_error("the level is not a uniform lattice with Dirichlet data on its whole boundary");
    return CDG_ERR_ARG;
  }
  if (lattice && (form == kMfStencil || (form == kMfAsTuned && L.st_zt > 0))) {
    if (L.st_zt == 4) return stencil_mode<4>(ctx, L, mode, x, b, invd, w, y, z, di, zcur);
    return stencil_mode<8>(ctx, L, mode, x, b, invd, w, y, z, di, zcur);
  }
  if (L.mf_uniform && L.mf_ntiles > 0 && form != kMfTwoKernel) {
    const int g = L.mf_ntiles;
    const size_t sm = (size_t)L.mf_tile_maxcells * kMfCellStride * sizeof(float);
    switch (mode) {
      case 0: return fused_launch<0>(ctx, L, g, sm, x, b, invd, w, y, z, di, zcur);
      case 1: return fused_launch<1>(ctx, L, g, sm, x, b, invd, w, y, z, di, zcur);
      case 2: return fused_launch<2>(ctx, L, g, sm, x, b, invd, w, y, z, di, zcur);
      default: return fused_launch<3>(ctx, L, g, sm, x, b, invd, w, y, z, di, zcur);
    }
  }
  const int cblocks = (L.ncells + kMfWarps - 1) / kMfWarps;
  const int cap = ctx->num_sms * L.mf_blocks_per_sm;
  const int grid = cap > 0 && cblocks > cap ? cap : cblocks;
  if (L.mf_uniform)
    CDG_LAUNCH_PDL(ctx, k_mf_uniform, grid, kMfWarps * 32, 0, L.ncells, L.mf_gdof, L.mf_pos_c,
               L.mf_ae, x, L.mf_y);
  else if (L.mf_lin)
    CDG_LAUNCH_PDL(ctx, k_mf_cell<true>, grid, kMfWarps * 32, 0, L.ncells, L.gdof, L.mf_pos,
               L.mf_fac, x, L.mf_y);
  else
    CDG_LAUNCH_PDL(ctx, k_mf_cell<false>, grid, kMfWarps * 32, 0, L.ncells, L.gdof, L.mf_pos,
               L.mf_fac, x, L.mf_y);
  const int g2 = (L.ndof + 255) / 256;
  switch (mode) {
    case 0: CDG_LAUNCH_PDL(ctx, k_mf_gather<0>, g2, 256, 0, L.ndof, L.nactive, L.dof_rp, L.mf_y, x, b, invd, w, y, z, di, zcur); break;
    case 1: CDG_LAUNCH_PDL(ctx, k_mf_gather<1>, g2, 256, 0, L.ndof, L.nactive, L.dof_rp, L.mf_y, x, b, invd, w, y, z, di, zcur); break;
    case 2: CDG_LAUNCH_PDL(ctx, k_mf_gather<2>, g2, 256, 0, L.ndof, L.nactive, L.dof_rp, L.mf_y, x, b, invd, w, y, z, di, zcur); break;
    default: CDG_LAUNCH_PDL(ctx, k_mf_gather<3>, g2, 256, 0, L.ndof, L.nactive, L.dof_rp, L.mf_y, x, b, invd, w, y, z, di, zcur); break;
  }
  return CDG_OK;
}

}  // namespace cdg
