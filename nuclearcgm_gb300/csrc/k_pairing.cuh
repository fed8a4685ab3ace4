// Pairing and guess kernels (see k_pairing.cu).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>

namespace ncgm {

// Y = T X (time reverse); oddOnly: numericalTR pairing of columns.
void timeReverse(const double2 *X, double2 *Y, size_t ns, int ncols, size_t ld,
                 bool oddOnly, cudaStream_t s);
// G (np x np, col-major) = V0 int rho_{cols[p]} rho_{cols[q]}
void densityGram(const double2 *X, size_t ld, const int *cols, int np, int n,
                 double h, double V0, double *G, cudaStream_t s);
// solveBCS on pairs; scal[0] = lambda, scal[1] = Epair; work >= 3 np
void bcsSolve(const double *eps, const double *Gp, int np, int A,
              double window, int windowBoth, const double *oldDelta,
              bool useOld, double oldLambda, double *u2, double *v2,
              double *Delta, double *scal, double *work, cudaStream_t s);
// kappa(r) from K_ab f_a f_b (Kff, nS x nS col-major) over states start..
void kappaField(const double2 *Phi, size_t ld, int start, int nS,
                const double *Kff, size_t ns, double *kappa, cudaStream_t s);
// Delta (nS x nS col-major, antisymmetric)
void deltaMatrix(const double2 *Phi, size_t ld, int start, int nS,
                 const double *ff, const double *kappa, int n, double h,
                 double V0, double *Delta, cudaStream_t s);
// HO guess: orbs (nr, l, j2, mj2) per column; columns normalised to 1
void hoGuess(const int4 *orbs, int nev, int n, double a, double h, double b,
             double2 *X, size_t ld, double *work, cudaStream_t s);
// Euclidean column normalisation (Eigen normalize(); zero columns kept)
void normalizeEuclid(double2 *X, size_t ld, size_t N, int ncols, double *work,
                     cudaStream_t s);

} // namespace ncgm
