// Test infrastructure (oracle): extern "C" entry points of the FP64 CPU
// restatement, loaded by tests/ and bench.py through ctypes (checker only).
#include "ncgm_oracle.h"
#include "orc_internal.hpp"

#include <cstring>

using namespace orc;

namespace {
struct OrcH {
  Grid g;
  Csr H;
  OrcH(int n, double a) : g(n, a) {}
};
const cd *asC(const double *p) { return reinterpret_cast<const cd *>(p); }
cd *asC(double *p) { return reinterpret_cast<cd *>(p); }
} // namespace

extern "C" {

void *orc_h_build_skyrme(int n, double a, const double *f, const double *gradf,
                         const double *U, const double *W, const double *UC) {
  auto *h = new OrcH(n, a);
  h->H = buildSkyrme(h->g, f, gradf, U, W, UC);
  return h;
}

void *orc_h_build_ws(int n, double a, int A, int Z, double V0, double r0,
                     double diff, double kappa, double beta, double beta3,
                     double so_V0, int spin_orbit) {
  auto *h = new OrcH(n, a);
  WSParams P{A, Z, V0, r0, diff, kappa, beta, beta3, so_V0, spin_orbit != 0};
  h->H = buildWS(h->g, P);
  return h;
}

long long orc_h_nnz(void *h) {
  return static_cast<OrcH *>(h)->H.rowptr.back();
}

void orc_h_export(void *hp, long long *rowptr, int *col, double *val) {
  auto *h = static_cast<OrcH *>(hp);
  std::memcpy(rowptr, h->H.rowptr.data(), sizeof(long long) * (h->H.N + 1));
  std::memcpy(col, h->H.col.data(), sizeof(int) * h->H.col.size());
  std::memcpy(val, h->H.val.data(), sizeof(cd) * h->H.val.size());
}

void orc_h_apply(void *hp, const double *X, double *Y, int ncols,
                 double shift) {
  auto *h = static_cast<OrcH *>(hp);
  spmm(h->H, asC(X), asC(Y), ncols, shift);
}

void orc_h_diag(void *hp, double *d) {
  auto *h = static_cast<OrcH *>(hp);
  for (long long r = 0; r < h->H.N; ++r) {
    cd v = h->H.diagpos[r] >= 0 ? h->H.val[h->H.diagpos[r]] : cd(0, 0);
    d[2 * r] = v.real();
    d[2 * r + 1] = v.imag();
  }
}

void orc_h_free(void *h) { delete static_cast<OrcH *>(h); }

int orc_gcg(void *hp, const double *X_init, int xcols, const double *ConjDir,
            int pcols, int nev, double shift, int max_iter, double tol,
            int cg_steps, double cg_tol, int ordering, double *X_out,
            double *lambda_out, int *pcg_steps_total) {
  auto *h = static_cast<OrcH *>(hp);
  const std::size_t N = h->H.N;
  CMat X0(N, xcols), P(N, pcols);
  std::memcpy(X0.d.data(), X_init, sizeof(cd) * N * xcols);
  if (pcols > 0) std::memcpy(P.d.data(), ConjDir, sizeof(cd) * N * pcols);
  GcgOut o = gcgLock(h->H, X0, P, nev, shift, max_iter, tol, cg_steps, cg_tol,
                     ordering);
  std::memcpy(X_out, o.X.d.data(), sizeof(cd) * N * nev);
  std::memcpy(lambda_out, o.lambda.data(), sizeof(double) * nev);
  if (pcg_steps_total) *pcg_steps_total = o.pcgSteps;
  return o.basisCols;
}

void orc_pcg(void *hp, const double *B, const double *X0, double *W, int ncols,
             double shift, int max_steps, double tol, int *steps_out) {
  auto *h = static_cast<OrcH *>(hp);
  const std::size_t N = h->H.N;
#pragma omp parallel for schedule(dynamic)
  for (int c = 0; c < ncols; ++c) {
    int s = pcgColumn(h->H, shift, asC(B) + c * N, asC(X0) + c * N,
                      asC(W) + c * N, max_steps, tol);
    if (steps_out) steps_out[c] = s;
  }
}

void orc_mgs(double *V, long long N, int ncols) {
  CMat M(N, ncols);
  std::memcpy(M.d.data(), V, sizeof(cd) * N * ncols);
  mgs(M);
  std::memcpy(V, M.d.data(), sizeof(cd) * N * ncols);
}

int orc_heig(const double *A, int m, double *w, double *V) {
  CMat M(m, m);
  std::memcpy(M.d.data(), A, sizeof(cd) * m * m);
  std::vector<double> ev;
  CMat Vm;
  bool ok = hermitianEig(M, ev, Vm);
  std::memcpy(w, ev.data(), sizeof(double) * m);
  std::memcpy(V, Vm.d.data(), sizeof(cd) * m * m);
  return ok ? 0 : 1;
}

static CMat wrap(const Grid &g, const double *psi, int ncols) {
  CMat M(g.N(), ncols);
  std::memcpy(M.d.data(), psi, sizeof(cd) * g.N() * ncols);
  return M;
}

void orc_density(int n, double a, const double *psi, int ncols, double *rho) {
  Grid g(n, a);
  auto r = density(g, wrap(g, psi, ncols));
  std::memcpy(rho, r.data(), sizeof(double) * r.size());
}
void orc_kinetic_density(int n, double a, const double *psi, int ncols,
                         double *tau) {
  Grid g(n, a);
  auto r = kineticDensity(g, wrap(g, psi, ncols));
  std::memcpy(tau, r.data(), sizeof(double) * r.size());
}
void orc_so_density(int n, double a, const double *psi, int ncols,
                    double *J9) {
  Grid g(n, a);
  auto r = soDensity(g, wrap(g, psi, ncols));
  std::memcpy(J9, r.data(), sizeof(double) * r.size());
}
void orc_divj(int n, double a, const double *psi, int ncols, double *divj) {
  Grid g(n, a);
  auto r = divJ(g, wrap(g, psi, ncols));
  std::memcpy(divj, r.data(), sizeof(double) * r.size());
}
void orc_grad_nospin(int n, double a, const double *v, double *g3) {
  Grid g(n, a);
  std::vector<double> in(v, v + g.ns());
  auto r = gradNoSpin(g, in);
  std::memcpy(g3, r.data(), sizeof(double) * r.size());
}
void orc_lap_nospin(int n, double a, const double *v, double *lap) {
  Grid g(n, a);
  std::vector<double> in(v, v + g.ns());
  auto r = lapNoSpin(g, in);
  std::memcpy(lap, r.data(), sizeof(double) * r.size());
}
void orc_grad_spinor(int n, double a, const double *psi, double *g3) {
  Grid g(n, a);
  std::vector<cd> out[3];
  gradSpinor(g, asC(psi), out);
  for (int ax = 0; ax < 3; ++ax)
    std::memcpy(g3 + 2 * ax * g.N(), out[ax].data(), sizeof(cd) * g.N());
}
void orc_grad_lagrange(int n, double a, const double *psi, double *g3) {
  Grid g(n, a);
  std::vector<cd> out[3];
  gradLagrangeSpinor(g, asC(psi), out);
  for (int ax = 0; ax < 3; ++ax)
    std::memcpy(g3 + 2 * ax * g.N(), out[ax].data(), sizeof(cd) * g.N());
}
void orc_lagrange_densities(int n, double a, const double *psi, int ncols,
                            const double *rho, double *tau, double *J9,
                            double *lap) {
  Grid g(n, a);
  const CMat P = wrap(g, psi, ncols);
  auto t = kineticDensityLagrange(g, P);
  auto J = soDensityLagrange(g, P);
  std::memcpy(tau, t.data(), sizeof(double) * t.size());
  std::memcpy(J9, J.data(), sizeof(double) * J.size());
  if (rho && lap) {
    std::vector<double> in(rho, rho + g.ns());
    auto l = lapLagrangeNoSpin(g, in);
    std::memcpy(lap, l.data(), sizeof(double) * l.size());
  }
}
double orc_integral(int n, double a, const double *v) {
  Grid g(n, a);
  return integral(g, v);
}
int orc_poisson(int n, double a, const double *rhoP, int Z,
                const double *U_guess, double *U_out) {
  Grid g(n, a);
  std::vector<double> r(rhoP, rhoP + g.ns()), U, G;
  if (U_guess) G.assign(U_guess, U_guess + g.ns());
  int it = poisson(g, r, Z, U_guess ? &G : nullptr, U);
  std::memcpy(U_out, U.data(), sizeof(double) * g.ns());
  return it;
}
void orc_ho_guess(int n, double a, int nev, double b, double beta,
                  double *out) {
  Grid g(n, a);
  CMat M = hoGuess(g, nev, b, beta);
  std::memcpy(out, M.d.data(), sizeof(cd) * M.d.size());
}

int orc_hf_run(const ncgm_hf_config *cfg, ncgm_hf_result *res, double *spe_n,
               double *spe_p, double *rho_n, double *rho_p, double *energies,
               int verbose) {
  std::memset(res, 0, sizeof(*res));
  return hfRun(*cfg, *res, spe_n, spe_p, rho_n, rho_p, energies, verbose);
}

int orc_hf_run_ex(const ncgm_hf_config *cfg, ncgm_hf_result *res,
                  double *spe_n, double *spe_p, double *rho_n, double *rho_p,
                  double *energies, ncgm_hf_outputs *out, int verbose) {
  std::memset(res, 0, sizeof(*res));
  std::memset(out->terms, 0, sizeof(out->terms));
  return hfRun(*cfg, *res, spe_n, spe_p, rho_n, rho_p, energies, verbose, out);
}
int orc_state_run(const ncgm_hf_config *cfg, const double *Xn,
                  const double *en, int cn, const double *Xp,
                  const double *ep, int cp, int calls, int flags,
                  const double *en2, const double *ep2, double *out,
                  double *E) {
  return stateRun(*cfg, Xn, en, cn, Xp, ep, cp, calls, flags, en2, ep2, out,
                  E);
}
void orc_shell_observables(int n, double a, const double *psi, int ncols,
                           double *obs) {
  Grid g(n, a);
  for (int c = 0; c < ncols; ++c)
    shellObservables(g, asC(psi) + (std::size_t)c * g.N(), obs + 5 * c);
}

} // extern "C"
