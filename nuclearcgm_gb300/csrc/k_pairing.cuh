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
// Dense-product back ends of the two HFB pairing-field routines: the
// exact-digit tensor-core kernels when exactScratch is set (gemmVCExact and
// gramTCExact scratch sized for nS columns), otherwise the FP64 kernels with
// `partials` (>= maxChunks nS^2 double2) for the Gram.
struct PairingGemm {
  void *exactScratch = nullptr;
  double2 *partials = nullptr;
  int maxChunks = 1;
};
// kappa(r) from Kff (K_ab f_a f_b, nS x nS col-major) over the nS columns of
// Phi (ld): Q = Phi Kff^T (one N x nS by nS x nS product), then one pass over
// the points. Q: N x nS scratch, C: nS x nS complex scratch.
void kappaFieldGemm(const double2 *Phi, size_t ld, int nS, const double *Kff,
                    size_t ns, double *kappa, double2 *Q, double2 *C,
                    const PairingGemm &g, cudaStream_t s);
// Delta (nS x nS col-major, antisymmetric) = 0.5 V0 f_a f_b Re(G - G^T) with
// G = phi(r,0)^T diag(h^3 w kappa) phi(r,1), one weighted Gram over the
// points. work: >= 2 ns nS double2; G: nS x nS complex.
void deltaMatrixGemm(const double2 *Phi, size_t ld, int nS, const double *ff,
                     const double *kappa, int n, double h, double V0,
                     double *Delta, double2 *work, double2 *G,
                     const PairingGemm &g, cudaStream_t s);
// HFB quasiparticle step (iteration_data.cpp:605-850), all on the device;
// state matrices M x M, window matrices nS x nS, col-major.
// Kff(a, b) = kappa(start + a, start + b) f_a f_b
void hfbKff(const double *kappa, int M, int start, int nS, const double *ff,
            double *Kff, cudaStream_t s);
// out[0] = sum of squares of an nS x nS matrix
void hfbNorm2(const double *D, int nS, double *out, cudaStream_t s);
// the 2nS x 2nS quasiparticle matrix at Fermi level lambda
void hfbMatrix(const double *e, const double *Delta, int nS, double lambda,
               double2 *H, cudaStream_t s);
// U, V of the positive-energy half of Ev; num[0] = sum V^2 (NaN when
// *status != 0)
void hfbExtract(const double2 *Ev, int nS, const int *status, double *Uw,
                double *Vw, double *num, cudaStream_t s);
// U, V padded to the basis and kappa = U V^T
void hfbAmplitudes(const double *Uw, const double *Vw, int nS, int start,
                   int M, double *U, double *V, double *kappa, cudaStream_t s);
// pe[0] = 0.5 sum_ij Delta(i, j) kappa(start + j, start + i)
void hfbPairEnergy(const double *Delta, const double *kappa, int M, int start,
                   int nS, double *pe, cudaStream_t s);
// the unpaired amplitudes: V = 1 on the first target states, U = kappa = 0
void hfbNull(int M, int target, double *U, double *V, double *kappa,
             cudaStream_t s);
// rho = V V^T (complex storage) and T = W diag(sqrt(w)) (w < 1e-12 -> 0)
void hfbDensityMatrix(const double *V, int M, double2 *rho, cudaStream_t s);
void hfbNatural(const double2 *W, const double *w, int M, double2 *T,
                cudaStream_t s);
// HO guess: orbs (nr, l, j2, mj2) per column; columns normalised to 1
void hoGuess(const int4 *orbs, int nev, int n, double a, double h, double b,
             double2 *X, size_t ld, double *work, cudaStream_t s);
// Euclidean column normalisation (Eigen normalize(); zero columns kept)
void normalizeEuclid(double2 *X, size_t ld, size_t N, int ncols, double *work,
                     cudaStream_t s);

} // namespace ncgm
