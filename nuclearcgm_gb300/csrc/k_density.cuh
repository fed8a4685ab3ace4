// Lattice density / mean-field / energy kernels (see k_density.cu).
#pragma once
#include "../../include/ncgm.h"

#include <cuda_runtime.h>

#include <cstddef>

namespace ncgm {

constexpr double kE2 = 1.43996446;       // e^2 [MeV fm]
constexpr double kHbarC = 197.327053;    // hbar c [MeV fm]
constexpr double kNucleonMass = 938.91869;

struct FieldsIn {
  size_t ns;
  ncgm_edf edf;
  double hbar2m; // hbar^2 / (2 m_corr)
  int spinOrbit, useJ;
  const double *rhoN, *rhoP, *tauN, *tauP, *lapN, *lapP, *divJN, *divJP;
  const double *gN, *gP;   // grad rho_q, n^3 x 3
  const double *JN, *JP;   // J_{mu nu}, n^3 x 9
};
struct FieldsOut {
  double *fN, *fP, *gfN, *gfP, *UN, *UP, *WN, *WP;
};

// energy densities integrated with trapezoid weights, in this order:
// 0 C0rho 1 C1rho 2 C0lap 3 C1lap 4 C0tau 5 C1tau 6 C0J2 7 C1J2 8 C0divJ
// 9 C1divJ 10 rho_p U_dir 11 Slater 12 kinetic 13 rearrangement
constexpr int kEnergyTerms = 14;
struct EnergyIn {
  size_t ns;
  int n;
  double h;
  ncgm_edf edf;
  double hbar2, massCorr;
  const double *rhoN, *rhoP, *tauN, *tauP, *lapN, *lapP, *divJN, *divJP;
  const double *JN, *JP;
  const double *UCDir; // may be null
};

void densities(const double2 *Phi, size_t ld, int M, int n, double h,
               double *rho, double *tau, double *J9, double *divJ,
               cudaStream_t s);
void gradLap(const double *v, int n, double h, double *g3, double *lap,
             cudaStream_t s);
void mix(double *old, const double *nw, double mu, size_t count, bool first,
         cudaStream_t s);
void meanFields(const FieldsIn &in, const FieldsOut &out, cudaStream_t s);
void energyIntegrals(const EnergyIn &in, double *partials, double *out,
                     cudaStream_t s);
// out[0] = int f g (g may be null) with trapezoid weights
void integral(const double *f, const double *g, int n, double h,
              double *partials, double *out, cudaStream_t s);
// Wavefunction::normalize: each column scaled to unit trapezoid norm
void normalizeColumns(double2 *X, size_t ld, int ncols, int n, double h,
                      double *work, cudaStream_t s);

// Lagrange-mesh recompute of the output step (k_lagrange.cu): tau and J9
// of the orbitals Phi (both or neither), the Laplacian of rho and its
// gradient (n^3 x 3; lap and grad3 may be null), with the Lagrange-mesh
// derivative matrices. scratch holds lagrangeScratchBytes(n) device bytes.
// Synchronises s.
size_t lagrangeScratchBytes(int n);
int lagrangeDensities(const double2 *Phi, size_t ld, int M, int n, double h,
                      const double *rho, double *tau, double *J9, double *lap,
                      double *grad3, void *scratch, cudaStream_t s);
// Shell observables of ncols spinor columns (k_shells.cu): per column
// [int psi conj(L^2 psi), int psi conj(J^2 psi), int psi conj(Jz Jz psi),
// Re sum psi(-r)^* psi(r), int psi conj(L.S psi)] (real parts).
// scratch holds shellScratchBytes(n) device bytes. Synchronises s.
size_t shellScratchBytes(int n);
int shellObservables(const double2 *Psi, size_t ld, int ncols, int n,
                     double a, void *scratch, double *obs, cudaStream_t s);

} // namespace ncgm
