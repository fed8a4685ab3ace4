/*
 * ncgm.h — C ABI of the GB300 (sm_103a) build of the nuclearcgm self-consistent
 * lattice hot path: the finite-difference single-particle Hamiltonian apply,
 * the block GCG eigensolver, density/field accumulation, the Coulomb Poisson
 * solve, BCS/HFB pairing and the Hartree-Fock iteration that sequences them.
 *
 * Every entry point returns an int status (NCGM_OK == 0) and never throws.
 * Matrices use the reference's Eigen layout: column-major, complex numbers as
 * interleaved (re, im) doubles, spinor rows ordered s + 2*(i + n*(j + n*k)).
 * Scalar lattice fields are n^3 doubles in i-fastest order; vector fields are
 * n^3 x 3 column-major (x block, y block, z block), like Eigen::MatrixX3d.
 *
 * Pointers passed to ncgm_apply_h / ncgm_gcg may be host or device memory:
 * the library asks the CUDA runtime which and copies when needed.
 *
 * Reference interfaces each entry point replaces are cited beside it as
 * path:line inside the nuclearcgm source tree.
 */
#ifndef NCGM_H
#define NCGM_H

#ifdef __cplusplus
extern "C" {
#endif

#define NCGM_OK 0
#define NCGM_ERR_ARG 1      /* bad argument (sizes, null pointers, species) */
#define NCGM_ERR_CUDA 2     /* CUDA runtime error or no CUDA device */
#define NCGM_ERR_NAN 3      /* NaN / Inf detected in a result */
#define NCGM_ERR_RANK 4     /* orthonormalisation found no independent columns */
#define NCGM_ERR_TIMEOUT 5  /* a bounded device wait gave up */
#define NCGM_ERR_EIG 6      /* projected eigensolver did not converge */
#define NCGM_ERR_NOMEM 7    /* device allocation failed */

#define NCGM_FP64 0         /* Hamiltonian apply in FP64 */
#define NCGM_FP32 1         /* Hamiltonian apply in FP32 (inputs rounded) */
#define NCGM_FP32_TC 2      /* GCG: FP32 corrections and tensor-core Gram
                               products split into exact BF16 digits
                               (~1e-13 relative) */

#define NCGM_NEUTRON 0
#define NCGM_PROTON 1

#define NCGM_ORDER_MATCH_PREVIOUS 0 /* EigenpairsOrdering::MATCH_PREVIOUS */
#define NCGM_ORDER_ASCENDING 1      /* EigenpairsOrdering::ASCENDING_ENERGIES */

typedef struct ncgm_ctx ncgm_ctx;
typedef struct ncgm_lp ncgm_lp; /* learned preconditioner (network + data) */

#define NCGM_PRECOND_JACOBI 0  /* reference: Jacobi PCG from d = 0 */
#define NCGM_PRECOND_LEARNED 1 /* Jacobi PCG from the network's d0 */

/* Skyrme EDF coupling constants, in the order of FunctionalParameters
 * (include/EDF.hpp:20-23). */
typedef struct ncgm_edf {
  double C0rr, C1rr, C0Drr, C1Drr, C0rt, C1rt, C0J2, C1J2, C0rdr, C1rdr, C0nJ,
      C1nJ, sigma;
} ncgm_edf;

/* Skyrme interaction parameters (include/EDF.hpp:4-18). */
typedef struct ncgm_skyrme {
  double W0, W0_pr, t0, t1, t2, t3, x0, x1, x2, x3, sigma, te, to;
} ncgm_skyrme;

/* Replaces EDF::setFromInteraction (src/skyrme/EDF.cpp:61-103). */
int ncgm_edf_from_skyrme(const ncgm_skyrme *in, ncgm_edf *out);

/* GCG parameters: GCGParameters (include/input_parser.hpp:29-35). */
typedef struct ncgm_gcg_params {
  int max_iter;    /* outer GCG iterations */
  double tol;      /* absolute residual-norm lock tolerance */
  int cg_steps;    /* max Jacobi-PCG steps per column */
  double cg_tol;   /* relative PCG tolerance */
  double shift;    /* initial shift (reference passes 0) */
  int ordering;    /* NCGM_ORDER_* */
  int precision;   /* NCGM_FP64; NCGM_FP32: FP32 PCG corrections; NCGM_FP32_TC:
                      also the search-space Gram products on the tensor
                      cores (exact-digit form, ~1e-13 relative) */
  int precond;     /* NCGM_PRECOND_*: 1 needs a network (ncgm_set_lp) */
} ncgm_gcg_params;

typedef struct ncgm_gcg_stats {
  int iterations;       /* outer iterations run */
  int converged;        /* locked columns at exit */
  int pcg_steps_max;    /* max PCG steps over columns, last outer iteration */
  int pcg_steps_total;  /* sum of PCG steps over columns and iterations */
  int basis_cols;       /* columns kept by the last orthonormalisation */
  double max_residual;  /* max residual norm of the returned pairs */
  double ms_total;      /* device wall time of the call */
  double ms_pcg;        /* part spent in the PCG correction */
  int lp_columns;       /* PCG columns started from the learned correction */
} ncgm_gcg_stats;

/* ---- context: grid and device state ------------------------------------ */

/* Replaces Grid(n, a) (src/grid/grid.cpp:7-21): x_i = -a + i*h, h = 2a/(n-1).
 * max_cols bounds the spinor columns any later call may pass. */
int ncgm_create(ncgm_ctx **out, int n, double a, int max_cols, int flags);
int ncgm_destroy(ncgm_ctx *ctx);
/* Text of the last error on this thread. */
const char *ncgm_last_error(void);
/* Device sync; returns the first pending error. */
int ncgm_sync(ncgm_ctx *ctx);

/* ---- Hamiltonian -------------------------------------------------------- */

/* Replaces Hamiltonian(grid, terms).buildMatrix() (src/hamiltonian/
 * hamiltonian.cpp:303-372) with the term list of Utilities::skyrmeHamiltonian
 * (src/util/utilities.cpp:56-70): SkyrmeU (src/skyrme/skyrme_u.cpp:15-24),
 * NonLocalKineticPotential (src/potentials/non_local_kinetic_potential.cpp:
 * 23-71), LocalKineticPotential (src/potentials/local_kinetic_potential.cpp:
 * 22-46), SkyrmeSO (src/skyrme/skyrme_so.cpp:12-58) and LocalCoulombPotential
 * (src/skyrme/local_coulomb_potential.cpp:12-41). No matrix is assembled: the
 * fields are uploaded and H is applied as a stencil.
 *   f      : hbar^2/2m*(r), n^3            (EffectiveMass::vector)
 *   gradf  : grad f, n^3 x 3              (EffectiveMass::gradient)
 *   U      : central field incl. constraint field, n^3 (IterationData::UN/UP)
 *   W      : spin-orbit field, n^3 x 3, or NULL for no spin-orbit term (BN/BP)
 *   UC     : Coulomb field, n^3, or NULL (IterationData::UCoul)           */
int ncgm_set_fields(ncgm_ctx *ctx, int species, const double *f,
                    const double *gradf, const double *U, const double *W,
                    const double *UC);

/* Replaces the Woods-Saxon guess Hamiltonian Hamiltonian::build_matrix5p()
 * (src/hamiltonian/hamiltonian.cpp:207-302) with DeformedWoodsSaxonPotential
 * (src/potentials/deformed_woods_saxon.cpp:12-17) and
 * DeformedSpinOrbitPotential (src/potentials/deformed_spin_orbit.cpp:69-114),
 * as assembled by main() (src/main.cpp:72-86). The fields are computed on the
 * device from the parameters. */
int ncgm_set_woods_saxon(ncgm_ctx *ctx, int species, int A, int Z, double V0,
                         double r0, double diff, double kappa, double beta,
                         double beta3, double so_V0, int spin_orbit);

/* Y = H X for ncols spinor columns (replaces ComplexSparseMatrix * MatrixXcd,
 * e.g. src/solver/solver.cpp:766). X, Y: N x ncols complex, N = 2 n^3. */
int ncgm_apply_h(ncgm_ctx *ctx, int species, const double *X, double *Y,
                 int ncols, int precision);

/* Device-resident form of ncgm_apply_h: Y = (H + shift I) X enqueued on the
 * context's stream without synchronising. X, Y are device buffers of complex
 * numbers in the precision's type (complex<double> for NCGM_FP64,
 * complex<float> for NCGM_FP32), N x ncols column-major. */
int ncgm_apply_h_device(ncgm_ctx *ctx, int species, const void *X, void *Y,
                        int ncols, int precision, double shift);

/* Makes the context enqueue its work on `stream` (a cudaStream_t; NULL for
 * the context's own stream). */
int ncgm_set_stream(ncgm_ctx *ctx, void *stream);

/* ---- eigensolver -------------------------------------------------------- */

/* Replaces gcgm_complex_no_B_lock (src/solver/solver.cpp:642-959, declared in
 * include/solver.hpp:43-47) as called by Utilities::solve (src/util/
 * utilities.cpp:20-36) on the Hamiltonian set for `species`.
 *   X_init : N x xcols (the first nev columns are used), ConjDir: N x pcols
 *   X_out  : N x nev (may alias X_init), lambda_out: nev.                 */
int ncgm_gcg(ncgm_ctx *ctx, int species, const double *X_init, int xcols,
             const double *ConjDir, int pcols, int nev,
             const ncgm_gcg_params *params, double *X_out, double *lambda_out,
             ncgm_gcg_stats *stats);

/* ---- lattice densities and Coulomb field -------------------------------- */

/* Densities of a block of (occupation-weighted) spinor columns Phi (N x
 * ncols): rho, tau (n^3), J_{mu nu} (n^3 x 9, column mu*3+nu) and div J (n^3).
 * Replaces Wavefunction::density / kineticDensity / soDensity / divJ
 * (src/util/wavefunction.cpp:21-44, 348-360, 421-464, 466-517). */
int ncgm_densities(ncgm_ctx *ctx, const double *Phi, int ncols, double *rho,
                   double *tau, double *J9, double *divJ);

/* The output step's Lagrange-mesh densities of the same columns: tau and
 * J_{mu nu} with the Lagrange-mesh first derivative (Operators::gradLagrange)
 * and, when rho and lap are both given, the Lagrange-mesh Laplacian of rho.
 * Replaces Wavefunction::kineticDensityLagrange / soDensityLagrange
 * (src/util/wavefunction.cpp:334-414) and Operators::lapLagrangeNoSpin
 * (src/operators/differential_operators.cpp:196-235), the parts of
 * IterationData::recomputeLagrange (src/util/iteration_data.cpp:346-382)
 * that enter the recomputed energy. */
int ncgm_lagrange_densities(ncgm_ctx *ctx, const double *Phi, int ncols,
                            const double *rho, double *tau, double *J9,
                            double *lap);

/* Coulomb direct potential of a proton density by the Poisson equation with
 * the multipole boundary halo, and UC = direct + Slater exchange. U_guess may
 * be NULL (cold start). Replaces Wavefunction::coulombFieldPoisson and
 * exchangeCoulombField (src/util/wavefunction.cpp:45-229). */
int ncgm_poisson(ncgm_ctx *ctx, const double *rhoP, int Z,
                 const double *U_guess, double *U_out, double *UC_out,
                 int *iterations);

/* Allocation-free form of ncgm_poisson, for callers that cannot allocate
 * device memory: hosts that hand the whole GPU to their own memory pool up
 * front, and loops that must not stall on cudaMalloc/cudaFree, which
 * synchronise the device. It has no counterpart in the reference. It needs
 * no context and allocates nothing: rhoP, U_guess (may be NULL for a cold
 * start), U_out and UC_out (may be NULL) must be device buffers of n^3
 * doubles, a is the box half-width and stream a cudaStream_t (NULL: the
 * default stream). The solver's scratch (4 n^3 + 560 doubles) is a static
 * device array sized for n <= NCGM_POISSON_NOALLOC_MAX_N (about 3.5 MB, held
 * by every GPU that loads the library until the process exits); larger n is
 * rejected with NCGM_ERR_ARG. The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture. All calls on a device share
 * the array: calls that overlap on the GPU race. Nothing in the scratch needs
 * to start at zero (every word is written before it is read). */
#define NCGM_POISSON_NOALLOC_MAX_N 48
int ncgm_poisson_noalloc(int n, double a, const double *rhoP, int Z,
                         const double *U_guess, double *U_out, double *UC_out,
                         void *stream, int *iterations);

/* ---- self-consistent iteration ----------------------------------------- */

/* Run configuration: the fields of InputParser (src/system/input_parser.cpp:
 * 50-261) that the HF/HFB loop of main() (src/main.cpp:38-369) reads. */
typedef struct ncgm_pairing {
  double V0;          /* pairing strength (positive, reference convention) */
  double window;      /* Fermi-window half width [MeV] */
  int basis_size;     /* HFbasisSize: columns carried for this species */
  int window_both;    /* two-sided smooth window */
  int active;         /* pairing on for this species */
} ncgm_pairing;

#define NCGM_PAIRING_NONE 0
#define NCGM_PAIRING_HFB 1
#define NCGM_PAIRING_BCS 2

#define NCGM_MAX_MULTIPOLE 8

typedef struct ncgm_hf_config {
  int n;               /* axisMeshPoints */
  double box_size;     /* boxSize (a = box_size / 2) */
  int A, Z;
  ncgm_edf edf;
  int spin_orbit, use_j, com_corr, use_coulomb;
  double density_mix;  /* densityMix */
  int max_iterations;  /* maxIterations */
  double energy_tol;   /* energyTol */
  double initial_beta, beta3;
  /* Woods-Saxon guess (parameters/woods_saxon.json) */
  double ws_V0, ws_r0, ws_diff, ws_kappa, wsso_V0;
  ncgm_gcg_params ws_gcg; /* initial GCG (maxIter 10, tol 1e-2, 40, 1e-4) */
  ncgm_gcg_params hf_gcg; /* per-iteration GCG (1, 1e-6, 80, 1e-5) */
  /* pairing */
  int pairing_type;    /* NCGM_PAIRING_* */
  ncgm_pairing pair_n, pair_p;
  int start_hfb_iter;
  double pairing_threshold;
  /* constraints */
  int constrain_com;   /* constrainCOM */
  int curve_mode;      /* deformation-curve constraint set at target mu20 */
  double mu20;         /* quadrupole target when curve_mode */
  double constraints_tol;
  /* stop rule extensions (0 = reference rule only) */
  double spe_tol;      /* also require max |dSPE| < spe_tol when > 0 */
  /* learned preconditioner (no reference counterpart; NULL / 0 = off) */
  ncgm_lp *lp;          /* network used when hf_gcg.precond = LEARNED */
  int lp_collect_every; /* > 0: log training pairs every k-th HF iteration */
  /* general multipole constraints, the input's "constraints" list of
   * {l, m, target} (input_parser.cpp:189-196): MultipoleConstraint on
   * X_lm r^l (src/skyrme/multipole_constraint.cpp:7-56), added from HF
   * iteration 1 (main.cpp:201-207) */
  int n_multipole;
  int mp_l[NCGM_MAX_MULTIPOLE], mp_m[NCGM_MAX_MULTIPOLE];
  double mp_target[NCGM_MAX_MULTIPOLE];
} ncgm_hf_config;

typedef struct ncgm_hf_result {
  int iterations;      /* HF iterations run */
  int converged;
  double E_int;        /* integrated EDF energy + kinetic (main.cpp:300-301) */
  double E_HF;         /* HFEnergy (iteration_data.cpp:212-224) */
  double E_pair_n, E_pair_p;
  double lambda_n, lambda_p; /* Fermi energies when pairing */
  double beta, gamma;  /* quadrupole deformation (output only) */
  double wall_s;       /* wall time of the run */
  double last_dE;      /* |Delta E_int| of the final iteration */
  double t_gcg_s, t_fields_s, t_poisson_s, t_pairing_s; /* phase times */
  /* E_INT recomputed with Lagrange-mesh derivatives for tau, J and the
   * Laplacian of rho from the final orbitals ("EintLag",
   * src/system/output.cpp:252-256, iteration_data.cpp:346-382) */
  double E_int_lagrange;
} ncgm_hf_result;

/* Runs the WS guess and the HF(B) loop of main() (src/main.cpp:59-342) on the
 * GPU. Optional outputs (may be NULL): spe_n/spe_p (orbitals per species),
 * rho_n/rho_p (n^3), energies (max_iterations x 2: E_int, E_HF per iter). */
int ncgm_hf_run(const ncgm_hf_config *cfg, ncgm_hf_result *res, double *spe_n,
                double *spe_p, double *rho_n, double *rho_p, double *energies);

/* ---- self-consistent state (IterationData) ------------------------------ */

/* The state of one self-consistent run: densities and their mixing history,
 * mean fields, Coulomb field, constraints and pairing (BCS / HFB) state, for
 * callers that drive their own HF loop around ncgm_gcg as main() does. */
typedef struct ncgm_state ncgm_state;

/* Replaces IterationData(input) (include/util/iteration_data.hpp:81-88,
 * src/util/iteration_data.cpp:9-151) with the constraint set main() builds
 * (src/main.cpp:164-185) from cfg: lattice, EDF, options, pairing, COM /
 * curve / multipole constraints. The guess and loop fields of cfg are not
 * used. */
int ncgm_state_create(ncgm_state **out, const ncgm_hf_config *cfg);
int ncgm_state_destroy(ncgm_state *st);

#define NCGM_UPDATE_NORMALIZE 1 /* Wavefunction::normalize first (main.cpp:254) */
#define NCGM_UPDATE_TRORDER 2   /* Wavefunction::TROrder first when pairing
                                   (main.cpp:256-263) */
/* Replaces IterationData::updateQuantities(neutronsPair, protonsPair, iter,
 * constraints) (include/util/iteration_data.hpp:89-92,
 * src/util/iteration_data.cpp:852-1125): pairing (BCS, or HFB from
 * startHFBIter), occupations, densities rho, tau, J, div J with mixing,
 * grad / Laplacian of rho, mean fields f, grad f, U (+ constraint field), W,
 * and the Coulomb field of the protons. X*: 2 n^3 x ncols complex, e*: the
 * eigenvalues (host or device X, host e); ncols must be the configured
 * orbital counts. iter: the HF iteration (constraints join at 1). flags:
 * NCGM_UPDATE_* steps of main() applied to the eigenvectors first. */
int ncgm_state_update(ncgm_state *st, const double *Xn, const double *en,
                      int ncols_n, const double *Xp, const double *ep,
                      int ncols_p, int iter, int flags);
/* The mean fields of a species after the last update, in the layout of
 * ncgm_set_fields (host or device outputs; any may be NULL): f, grad f
 * (n^3 x 3), U with the constraint field, W (n^3 x 3), UC (the Coulomb field
 * for protons, zeros otherwise). */
int ncgm_state_fields(ncgm_state *st, int species, double *f, double *gradf,
                      double *U, double *W, double *UC);
/* rho and tau of a species (n^3 each, either may be NULL) */
int ncgm_state_densities(ncgm_state *st, int species, double *rho,
                         double *tau);
/* E_int = kinetic + totalEnergyIntegral and E_HF = HFEnergy
 * (iteration_data.cpp:153-271, main.cpp:300-305) of the current densities
 * with the new single-particle energies en, ep (host); also records
 * |Delta E_HF| as IterationData::energyDiff for the constraints. */
int ncgm_state_energy(ncgm_state *st, const double *en, const double *ep,
                      double *E_int, double *E_HF);

/* What the reference's output step (Output::shellsToFile,
 * src/system/output.cpp:97-408) reads from the final state. Array pointers
 * may be NULL (not wanted) and may be host or device memory. */
#define NCGM_ENERGY_TABLE 16
typedef struct ncgm_hf_outputs {
  /* final single-particle states, 2 n^3 x orbitals complex (Eigen layout) */
  double *orbitals_n, *orbitals_p;
  /* kinetic densities after the Lagrange-mesh recompute (n^3) */
  double *tau_n, *tau_p;
  /* Lagrange-mesh gradients of rho_n / rho_p (n^3 x 3, column-major),
   * Operators::gradLagrangeNoSpin (differential_operators.cpp:156-194) */
  double *grad_rho_n, *grad_rho_p;
  /* mean fields U_n / U_p (n^3) */
  double *U_n, *U_p;
  /* filled always: the "Density Functional contributions" table
   * (output.cpp:205-236) in its order: E_kin, C0 rho0, C1 rho1,
   * C0 nabla2rho0, C1 nabla2rho1, C0 tau0, C1 tau1, C0 div J, C1 div J,
   * C0 J2, C1 J2, E coulomb direct, E pairing n, E pairing p,
   * E coulomb exchange, E rearrangement (Erear) */
  double terms[NCGM_ENERGY_TABLE];
  /* filled always: sum of the constraints' evaluate() on the final
   * densities (output.cpp:357-360) */
  double constraints_energy;
} ncgm_hf_outputs;

/* ncgm_hf_run plus the output step's arrays and energy table. */
int ncgm_hf_run_ex(const ncgm_hf_config *cfg, ncgm_hf_result *res,
                   double *spe_n, double *spe_p, double *rho_n, double *rho_p,
                   double *energies, ncgm_hf_outputs *out);

/* Shell observables of ncols spinor columns Psi (N x ncols, Eigen layout),
 * obs (ncols x 5, one row per column): the real parts of
 * int psi conj(L^2 psi), int psi conj(J^2 psi), int psi conj(Jz Jz psi)
 * (trapezoid integrals with hbar = 197.327053 MeV fm),
 * sum_r psi(-r)^* psi(r), and int psi conj(L.S psi). These are the
 * quantities of Shell::l / j / mj / P (src/util/shell.cpp:22-51) and of the
 * spin-orbit correction of IterationData::chargeRadius
 * (src/util/iteration_data.cpp:121-151), with the operators of
 * src/operators/angular_momentum.cpp. */
int ncgm_shell_observables(ncgm_ctx *ctx, const double *Psi, int ncols,
                           double *obs);

/* C (p x q) = A^H B for complex column blocks of ctx->N rows (A: N x p,
 * B: N x q, Eigen layout; host or device buffers): the Gram / projection
 * products of the GCG (src/solver/solver.cpp:750-777, V.adjoint() * W).
 * precision NCGM_FP64: FP64 CUDA cores, deterministic reduction;
 * NCGM_FP32: tensor cores (tcgen05 kind::tf32 with split TF32 operands,
 * FP32 accumulation over row chunks, FP64 chunk sums; ~2e-6 relative);
 * NCGM_FP32_TC: tensor cores (tcgen05 kind::f16, values split into six
 * 7-bit integer digits held exactly in BF16 and written once per operand,
 * exact FP32 sums per digit level, exact 64-bit combination, FP64 chunk
 * sums; ~1e-13 relative). With A == B (the same buffer) and p == q the
 * block is staged and split once. */
int ncgm_gram(ncgm_ctx *ctx, const double *A, int p, const double *B, int q,
              double *C, int precision);

/* Y = V C for a block V (N x m, N = 2 n^3, column-major complex<double>)
 * and a small matrix C (m x k, column-major): the subspace rotation of the
 * GCG's orthonormalisation and Rayleigh-Ritz steps (the reference forms it
 * with Eigen products, src/solver/solver.cpp:418-463, 669-677). Host or
 * device pointers. precision NCGM_FP64: FP64 CUDA cores; NCGM_FP32_TC:
 * tensor cores with the exact digit products of ncgm_gram (~1e-12 relative
 * of the column maxima). */
int ncgm_vc(ncgm_ctx *ctx, const double *V, int m, const double *C, int k,
            double *Y, int precision);

/* Eigenpairs of a Hermitian m x m matrix A (column-major complex<double>,
 * lower triangle read; m <= 1024): w ascending, V the eigenvectors in the
 * same order. This is the projected eigenproblem of the GCG's Rayleigh-Ritz
 * step (the reference's SelfAdjointEigenSolver on the lower triangle,
 * src/solver/solver.cpp:766-777) and of the HFB step. m <= 80: one-CTA
 * Jacobi in shared memory (NCGM_FP64: FP64 rotations; NCGM_FP32 and
 * NCGM_FP32_TC: double-float rotations); m > 80: Householder
 * tridiagonalisation, bisection and inverse iteration over the whole GPU.
 * Host or device pointers. */
int ncgm_heig(ncgm_ctx *ctx, const double *A, int m, double *w, double *V,
              int precision);

/* Batch of independent HF runs on one GPU (the reference runs the points of
 * a deformation curve one after another, src/main.cpp:176-185 with
 * Utilities::curve, src/util/utilities.cpp:71-73). Every configuration runs
 * on its own host thread, context and stream, at most max_concurrent at a
 * time (0: all), so the latency-bound launches of the runs overlap. Each
 * result equals ncgm_hf_run's for that configuration. status (count ints)
 * and rho_n / rho_p (count pointers to n^3 host doubles) may be NULL. */
int ncgm_hf_run_batch(const ncgm_hf_config *cfgs, int count,
                      int max_concurrent, ncgm_hf_result *res, int *status,
                      double *const *rho_n, double *const *rho_p);

/* ---- learned preconditioner (no reference counterpart) ----------------
 * The reference's GCG correction is Jacobi PCG from d = 0 on
 * (A + shift) d = x lambda - A x (src/solver/solver.cpp:723-745). With
 * precond = NCGM_PRECOND_LEARNED the PCG starts from d0 = N(r), a 3-D
 * convolutional network (4-level U-Net, 47,489 BF16 weights, FP32
 * accumulation) of the residual component and the local fields, scaled by
 * the step that minimises the CG energy along it (a column where that step
 * is not positive starts from 0 as before); the Jacobi PCG then runs to the
 * usual tolerance and the GCG locks on the FP64 residual. The
 * network is trained on the device on pairs (r, exact d) that the solver
 * itself produces. */
int ncgm_lp_num_params(void);
int ncgm_lp_create(ncgm_lp **lp, unsigned long long seed); /* He-normal init */
int ncgm_lp_destroy(ncgm_lp *lp);
/* FP32 master weights, ncgm_lp_num_params() floats (host or device) */
int ncgm_lp_get_params(ncgm_lp *lp, float *theta);
int ncgm_lp_set_params(ncgm_lp *lp, const float *theta);
/* y [batch][n^3] = N(x [batch][3][n^3]) (host or device buffers) */
int ncgm_lp_forward(ncgm_lp *lp, int n, int batch, const float *x, float *y);
/* loss (mean relative squared error against t [batch][n^3]) and its
 * gradient with respect to the FP32 master weights */
int ncgm_lp_gradient(ncgm_lp *lp, int n, int batch, const float *x,
                     const float *t, float *loss, float *grad);
/* Adds 4 training pairs per column: r = X lambda - H X (X: N x ncols, host
 * or device; lambda: host) and the exact correction d of (H + shift) d = r
 * from FP64 Jacobi PCG (cg_steps, relative cg_tol) on ctx's fields. Columns
 * whose solve does not reach cg_tol (H + shift indefinite) are skipped;
 * ncgm_lp_dataset_size reports what was kept. */
int ncgm_lp_collect(ncgm_lp *lp, ncgm_ctx *ctx, int species, const double *X,
                    int ncols, const double *lambda, double shift,
                    int cg_steps, double cg_tol);
int ncgm_lp_dataset_size(ncgm_lp *lp, int n);
/* Adam on random minibatches of the collected pairs; loss_curve (host,
 * steps floats, may be NULL) receives the minibatch losses. */
int ncgm_lp_train(ncgm_lp *lp, int steps, int batch, double lr,
                  unsigned long long seed, float *loss_curve);
/* mean per-pair loss over the pairs of lattice n */
int ncgm_lp_eval(ncgm_lp *lp, int n, double *mean_loss);
/* network used by ncgm_gcg with precond = NCGM_PRECOND_LEARNED */
int ncgm_set_lp(ncgm_ctx *ctx, ncgm_lp *lp);

/* ---- measurement ------------------------------------------------------- */

/* FP64 FMA throughput of the current device in GFLOP/s (2 flops per FMA),
 * timed with CUDA events over one launch of independent FMA chains: the
 * compute ceiling the FP64 stencil is reported against. A measurement helper
 * with no counterpart in the reference. */
int ncgm_measure_fp64_gflops(double *gflops);

#ifdef __cplusplus
}
#endif
#endif /* NCGM_H */
