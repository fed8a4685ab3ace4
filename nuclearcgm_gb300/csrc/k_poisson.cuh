// Coulomb Poisson solve (see k_poisson.cu).
#pragma once
#include "../../include/ncgm.h"

#include <cuda_runtime.h>

#include <cstddef>

namespace ncgm {

constexpr double kE2Poisson = 1.43996446;

struct PoissonArgs {
  int n;
  double a, h;
  double Z;
  const double *rhoP; // n^3
  double *U;          // in: warm start (if warm), out: direct potential
  double *UC;         // out: direct + Slater exchange (the Coulomb field)
  int warm;
  double tol;         // relative residual target
  double *work;       // poissonWorkDoubles(n) doubles
};

int poissonSolve(const PoissonArgs &args, cudaStream_t s, int *iterations);
size_t poissonWorkDoubles(int n);

} // namespace ncgm
