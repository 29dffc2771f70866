// solver_dev.cuh -- device pieces of FGMRES shared by the graph-captured
// solver (linalg.cu) and the batched one-block-per-request solver (batch.cu).
#pragma once

#include <cuda_runtime.h>

namespace cdg {

struct ConvParams {
  double tol, red, div;
  int min_it, max_it, m;
};

// IterativeMethod::converged (IterativeMethod.h:83-163): 0 continue, 1 stop,
// 2 diverged; li[0] initial, li[1] previous residual
__device__ __forceinline__ int conv_test(const ConvParams& c, double* li, double res, int it) {
  if (it == 0) {
    li[0] = res;
    li[1] = res;
  }
  const bool small = res < c.tol;
  const bool red = res < c.red * li[0];
  const bool enough = it >= c.min_it;
  const bool stag = res > 1e10 * li[1];
  const bool div = res > c.div * li[0];
  bool conv = (small || red || stag || div) && enough;
  if (it == c.max_it) conv = true;
  li[1] = res;
  if (div) return 2;
  return conv ? 1 : 0;
}

// Givens rotations of Hessenberg column i (Utilities_gmres.C:60-88): apply
// the previous rotations, generate and apply rotation i, rotate (si, si1),
// write |s_{i+1}| to *resid
__device__ __forceinline__ void givens_column_s(int i, double* col, double* cs, double* sn,
                                                double& si, double& si1, double* resid) {
  for (int k = 0; k < i; ++k) {
    double dx = col[k], dy = col[k + 1];
    col[k] = cs[k] * dx + sn[k] * dy;
    col[k + 1] = -sn[k] * dx + cs[k] * dy;
  }
  double dx = col[i], dy = col[i + 1], c, sg;
  if (dy == 0.0) {
    c = 1.0;
    sg = 0.0;
  } else if (fabs(dy) > fabs(dx)) {
    double t = dx / dy;
    sg = 1.0 / sqrt(1.0 + t * t);
    c = t * sg;
  } else {
    double t = dy / dx;
    c = 1.0 / sqrt(1.0 + t * t);
    sg = t * c;
  }
  cs[i] = c;
  sn[i] = sg;
  col[i] = c * dx + sg * dy;
  col[i + 1] = -sg * dx + c * dy;
  double a = si, b = si1;
  si = c * a + sg * b;
  si1 = -sg * a + c * b;
  *resid = fabs(si1);
}

}  // namespace cdg
