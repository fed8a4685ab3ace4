// Batched Jacobi-PCG (see k_pcg.cu).
#pragma once
#include "ncgm_internal.cuh"

#include <cuda_runtime.h>

#include <cstddef>
#include <functional>

namespace ncgm {

struct PcgCol {
  double absNew, absOld, beta, thr, rhsNorm2;
  double alphaR, alphaI; // step of the current iteration (dot kernel)
  int iters, done, zero, pad;
};

// Buffers are device pointers to complex numbers of type T (interleaved),
// N rows per column, ncols columns, column stride N except X (ldx).
template <class T> struct PcgPlan {
  size_t N = 0;
  int ncols = 0;
  const void *X = nullptr; // initial guess and right-hand-side direction
  size_t ldx = 0;
  void *W = nullptr, *R = nullptr, *Z = nullptr, *P = nullptr, *AP = nullptr;
  const double *lamShift = nullptr; // lambda_k + shift per column (device)
  const double *coef = nullptr;     // Jacobi diagonal c0 per point (n^3)
  // FP32 plans: 1 / (c0 + shift) per point in FP32 (n^3), for the step's
  // preconditioner (null: FP64 division from coef)
  const float *invd = nullptr;
  double shift = 0, tol = 0;
  int maxSteps = 0;
  PcgCol *st = nullptr;
  double *partials = nullptr, *partials2 = nullptr; // ncols*128*3, ncols*128*2
  int *live = nullptr; // count of column-iterations (stats)
  int *ndone = nullptr; // device counter of finished columns: early exit
  // per-column arrival counters of the fused reductions (2 x ncols, zeroed
  // by pcgRun)
  unsigned *arrive = nullptr;
  // correction form: when AX64 is set the plan solves for d = w - x from the
  // FP64 residual x lam - A x; X64 = x, W64 receives w = x + d (FP64)
  const double2 *X64 = nullptr, *AX64 = nullptr;
  double2 *W64 = nullptr;
  // correction form only: initial correction d0 (precision T, N x ncols);
  // the PCG starts from alpha d0 with the energy-minimising alpha, or from 0
  // when alpha <= 0 (useNet[col] records the choice, device, may be null)
  const void *D0 = nullptr;
  int *useNet = nullptr;
  // correction form: W64 receives d instead of x + d (span(x, x + d) =
  // span(x, d); used when the search space is orthonormalised from a Gram
  // product with FP32-level resolution of near-dependent columns)
  bool onlyCorrection = false;
  // Y = (A + shift) X on device buffers (ld of X given, Y stride N)
  std::function<void(const void *, size_t, void *, int, double, cudaStream_t)>
      apply;
};

int pcgBlocks(size_t N);
// The Jacobi diagonal c0 = U + UC + 7.5 f / h^2 of a species' current
// coefficient table, one double per lattice point, in a context buffer.
double *jacobiDiagonal(ncgm_ctx *ctx, int species, cudaStream_t s);
// inv[p] = 1 / (c0[p] + shift) in FP32 (1 where the sum is 0)
void inverseDiagonal32(const double *c0, double shift, size_t ns, float *inv,
                       cudaStream_t s);
template <class T> void pcgRun(const PcgPlan<T> &plan, cudaStream_t s);

} // namespace ncgm
