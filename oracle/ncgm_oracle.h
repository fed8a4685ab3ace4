/*
 * Test infrastructure: the FP64 CPU oracle of the nuclearcgm lattice hot path.
 *
 * A plain C++17/OpenMP restatement of the reference algorithm (no Eigen), used
 * ONLY by tests/, the smoke check and bench.py's CPU-baseline leg as the
 * checker. The product library (nuclearcgm_gb300/csrc) never links it.
 *
 * Parity status: the reference ships no tests, golden vectors or fixtures for
 * this path and cannot be compiled here (Eigen is absent), so this oracle is
 * "parity unpinned" against the reference binary. It is pinned instead by
 * known-answer tests (harmonic-oscillator levels, free Laplacian spectrum,
 * analytic derivatives) and by numpy cross-checks in tests/.
 *
 * Layouts are those of include/ncgm.h.
 */
#ifndef NCGM_ORACLE_H
#define NCGM_ORACLE_H
#include "../include/ncgm.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Assembled CSR Hamiltonian (Hamiltonian::buildMatrix, term list of
 * Utilities::skyrmeHamiltonian). W / UC may be NULL. */
void *orc_h_build_skyrme(int n, double a, const double *f, const double *gradf,
                         const double *U, const double *W, const double *UC);
/* Woods-Saxon guess Hamiltonian (Hamiltonian::build_matrix5p). */
void *orc_h_build_ws(int n, double a, int A, int Z, double V0, double r0,
                     double diff, double kappa, double beta, double beta3,
                     double so_V0, int spin_orbit);
long long orc_h_nnz(void *h);
void orc_h_export(void *h, long long *rowptr, int *col, double *val);
/* Y = (H + shift I) X; X, Y: N x ncols interleaved complex. */
void orc_h_apply(void *h, const double *X, double *Y, int ncols, double shift);
/* diag(H), N complex. */
void orc_h_diag(void *h, double *d);
void orc_h_free(void *h);

/* gcgm_complex_no_B_lock on an oracle Hamiltonian. Returns kept columns. */
int orc_gcg(void *h, const double *X_init, int xcols, const double *ConjDir,
            int pcols, int nev, double shift, int max_iter, double tol,
            int cg_steps, double cg_tol, int ordering, double *X_out,
            double *lambda_out, int *pcg_steps_total);

/* One Jacobi-PCG solve per column (Eigen ConjugateGradient + diagonal
 * preconditioner restated): (H + shift I) W = B, initial guess X0. */
void orc_pcg(void *h, const double *B, const double *X0, double *W, int ncols,
             double shift, int max_steps, double tol, int *steps_out);

/* Modified Gram-Schmidt (b_modified_gram_schmidt_complex_no_B), in place. */
void orc_mgs(double *V, long long N, int ncols);

/* Hermitian eigensolver (lower triangle of an m x m complex matrix). */
int orc_heig(const double *A, int m, double *w, double *V);

/* Lattice operators. psi: N x ncols complex; outputs n^3 (x9 / x3). */
void orc_density(int n, double a, const double *psi, int ncols, double *rho);
void orc_kinetic_density(int n, double a, const double *psi, int ncols,
                         double *tau);
void orc_so_density(int n, double a, const double *psi, int ncols,
                    double *J9);
void orc_divj(int n, double a, const double *psi, int ncols, double *divj);
void orc_grad_nospin(int n, double a, const double *v, double *g3);
void orc_lap_nospin(int n, double a, const double *v, double *lap);
void orc_grad_spinor(int n, double a, const double *psi, double *g3);
/* Lagrange-mesh gradient (g3: 3 x N complex) and the output step's
 * recomputed tau, J9 and Laplacian of rho (rho and lap may be NULL) */
void orc_grad_lagrange(int n, double a, const double *psi, double *g3);
void orc_lagrange_densities(int n, double a, const double *psi, int ncols,
                            const double *rho, double *tau, double *J9,
                            double *lap);
double orc_integral(int n, double a, const double *v);

/* Coulomb direct potential by the Poisson solve (coulombFieldPoisson).
 * U_guess may be NULL. Returns CG iterations. */
int orc_poisson(int n, double a, const double *rhoP, int Z,
                const double *U_guess, double *U_out);

/* Initial guess (harmonic_oscillator_guess, spin-orbit branch). */
void orc_ho_guess(int n, double a, int nev, double b, double beta,
                  double *out);

/* Whole self-consistent run (main.cpp loop). Same outputs as ncgm_hf_run.
 * verbose: print one line per iteration. */
int orc_hf_run(const ncgm_hf_config *cfg, ncgm_hf_result *res, double *spe_n,
               double *spe_p, double *rho_n, double *rho_p, double *energies,
               int verbose);
int orc_hf_run_ex(const ncgm_hf_config *cfg, ncgm_hf_result *res,
                  double *spe_n, double *spe_p, double *rho_n, double *rho_p,
                  double *energies, ncgm_hf_outputs *out, int verbose);
/* The state-update counterpart of ncgm_state_*: `calls` updates from the
 * same eigenpairs (iterations 0 .. calls-1), then the energies E[0..1] with
 * the levels en2, ep2; out: per species f, grad f, U, W, UC, rho, tau
 * (11 n^3). flags: 1 normalise, 2 TROrder (with pairing). */
int orc_state_run(const ncgm_hf_config *cfg, const double *Xn,
                  const double *en, int cn, const double *Xp,
                  const double *ep, int cp, int calls, int flags,
                  const double *en2, const double *ep2, double *out,
                  double *E);
/* obs: ncols x 5 as ncgm_shell_observables */
void orc_shell_observables(int n, double a, const double *psi, int ncols,
                           double *obs);

#ifdef __cplusplus
}
#endif
#endif
