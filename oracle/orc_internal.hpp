// Test infrastructure (oracle): internal declarations of the FP64 CPU
// restatement. See ncgm_oracle.h for the role of the oracle.
#pragma once
#include "../include/ncgm.h"
#include "orc_linalg.hpp"

#include <vector>

namespace orc {

// nuclearConstants (include/constants.hpp:11-25)
constexpr double kHbar = 197.327053;
constexpr double kMass = 938.91869;
constexpr double kE2 = 1.43996446;

// Grid (include/grid.hpp:87-92, src/grid/grid.cpp:7-41)
struct Grid {
  int n;
  double a, h;
  std::vector<double> xs;
  Grid(int n_, double a_) : n(n_), a(a_), h(2.0 * a_ / (n_ - 1)) {
    xs.resize(n);
    for (int i = 0; i < n; ++i) xs[i] = -a + static_cast<double>(i) * h;
  }
  std::size_t ns() const { return (std::size_t)n * n * n; }
  std::size_t N() const { return 2 * ns(); }
  std::size_t idxNS(int i, int j, int k) const {
    return (std::size_t)i + (std::size_t)n * (j + (std::size_t)n * k);
  }
  std::size_t idx(int i, int j, int k, int s) const {
    return (std::size_t)s + 2 * idxNS(i, j, k);
  }
};

struct Csr {
  long long N = 0;
  std::vector<long long> rowptr, diagpos;
  std::vector<int> col;
  std::vector<cd> val;
};

struct WSParams {
  int A, Z;
  double V0, r0, diff, kappa, beta, beta3, soV0;
  bool so;
};

struct GcgOut {
  CMat X;
  std::vector<double> lambda;
  int iterations = 0, converged = 0, pcgSteps = 0, basisCols = 0;
};

// lattice operators
void gradSpinor(const Grid &g, const cd *psi, std::vector<cd> out[3]);
std::vector<double> gradNoSpin(const Grid &g, const std::vector<double> &v);
std::vector<double> lapNoSpin(const Grid &g, const std::vector<double> &v);
double integral(const Grid &g, const double *v);
std::vector<double> density(const Grid &g, const CMat &psi);
std::vector<double> kineticDensity(const Grid &g, const CMat &psi);
std::vector<double> soDensity(const Grid &g, const CMat &psi);
std::vector<double> divJ(const Grid &g, const CMat &psi);
// Lagrange-mesh forms of the output step
std::vector<double> lagrangeD1(int n, double h);
void gradLagrangeSpinor(const Grid &g, const cd *psi, std::vector<cd> out[3]);
std::vector<double> kineticDensityLagrange(const Grid &g, const CMat &psi);
std::vector<double> soDensityLagrange(const Grid &g, const CMat &psi);
std::vector<double> lapLagrangeNoSpin(const Grid &g,
                                      const std::vector<double> &v);
std::vector<double> gradLagrangeNoSpin(const Grid &g,
                                       const std::vector<double> &v);
// Shell::l/j/mj/P quantities and <L.S> of one spinor
void shellObservables(const Grid &g, const cd *psi, double obs[5]);
void normalize(const Grid &g, CMat &psi);
CMat timeReverse(const Grid &g, const CMat &psi);
CMat TROrder(const Grid &g, const CMat &psi);

// Hamiltonian and solver
Csr buildSkyrme(const Grid &g, const double *f, const double *gradf,
                const double *U, const double *W, const double *UC);
Csr buildWS(const Grid &g, const WSParams &P);
double wsValue(const WSParams &P, double x, double y, double z);
void wsSOFactor(const WSParams &P, double x, double y, double z,
                double out[3]);
double wsSOls();
void spmm(const Csr &H, const cd *X, cd *Y, int ncols, double shift);
void mgs(CMat &V);
int pcgColumn(const Csr &H, double shift, const cd *b, const cd *x0, cd *x,
              int max_steps, double tol);
GcgOut gcgLock(const Csr &A, const CMat &X_initial, const CMat &ConjDir,
               int nev, double shift, int max_iter, double tolerance,
               int cg_steps, double cg_tol, int ordering);

// physics
int poisson(const Grid &g, const std::vector<double> &rhoP, int Z,
            const std::vector<double> *Uguess, std::vector<double> &Uout);
CMat hoGuess(const Grid &g, int nev, double b, double beta);

} // namespace orc

namespace orc {
int hfRun(const ncgm_hf_config &cfg, ncgm_hf_result &res, double *spe_n,
          double *spe_p, double *rho_n, double *rho_p, double *energies,
          int verbose, ncgm_hf_outputs *out = nullptr);
int stateRun(const ncgm_hf_config &cfg, const double *Xn, const double *en,
             int cn, const double *Xp, const double *ep, int cp, int calls,
             int flags, const double *en2, const double *ep2, double *out,
             double *E);
}
