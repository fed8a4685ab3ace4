// Test infrastructure (oracle): mean fields, Coulomb Poisson solve, pairing,
// constraints, energies, initial guess and the self-consistent driver of the
// nuclearcgm hot path, restated in plain FP64 C++. Checker only: used by
// tests/, the smoke check and bench.py's CPU-baseline leg.
#include "orc_internal.hpp"

#include <chrono>
#include <cstdio>
#include <cstring>
#include <memory>
#include <tuple>

namespace orc {

using Vec = std::vector<double>;

// ---------------------------------------------------------------------------
// Coulomb: Wavefunction::coulombFieldPoisson (src/util/wavefunction.cpp:
// 55-229) and exchangeCoulombField (45-53).
// The boundary potential lives on an (n+4)^3 halo indexed i*dim*dim + j*dim + k
// (i slowest), while the right-hand side is indexed with the same lambda, so
// the x and z roles of the halo are swapped relative to the lattice; this is
// reproduced. The reference solves with Eigen's BiCGSTAB at machine-epsilon
// tolerance; the operator is the symmetric 5-point Laplacian, so the oracle
// solves it with conjugate gradients (Hestenes-Stiefel) to a relative residual
// of 1e-14, which reaches the same solution to rounding.
// ---------------------------------------------------------------------------
static double Y20xyz(double x, double y, double z) {
  double theta = std::acos(z / std::sqrt(x * x + y * y + z * z));
  return std::sqrt(5.0 / (16.0 * M_PI)) *
         (3.0 * std::cos(theta) * std::cos(theta) - 1.0);
}
static double Y22xyz(double x, double y, double z) {
  double theta = std::acos(z / std::sqrt(x * x + y * y + z * z));
  double phi = std::atan2(y, x);
  return std::sqrt(15.0 / (32.0 * M_PI)) * std::cos(2 * phi) *
         std::sin(theta) * std::sin(theta);
}

// Laplacian (LaplacianPotential, src/coulomb/laplacianp_potential.cpp:18-73)
// applied matrix-free with Dirichlet truncation: out = L v.
static void lap5(const Grid &g, const double *v, double *out) {
  const int n = g.n;
  const double hh = g.h * g.h;
  const double c0 = -(90.0 / 12.0) / hh, c1 = (16.0 / 12.0) / hh,
               c2 = -(1.0 / 12.0) / hh;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        // ascending column order: k-2, k-1, j-2, j-1, i-2, i-1, c, i+1, ...
        double s = 0.0;
        auto at = [&](int a, int b, int c) { return v[g.idxNS(a, b, c)]; };
        if (k >= 2) s += c2 * at(i, j, k - 2);
        if (k >= 1) s += c1 * at(i, j, k - 1);
        if (j >= 2) s += c2 * at(i, j - 2, k);
        if (j >= 1) s += c1 * at(i, j - 1, k);
        if (i >= 2) s += c2 * at(i - 2, j, k);
        if (i >= 1) s += c1 * at(i - 1, j, k);
        s += c0 * at(i, j, k);
        if (i + 1 < n) s += c1 * at(i + 1, j, k);
        if (i + 2 < n) s += c2 * at(i + 2, j, k);
        if (j + 1 < n) s += c1 * at(i, j + 1, k);
        if (j + 2 < n) s += c2 * at(i, j + 2, k);
        if (k + 1 < n) s += c1 * at(i, j, k + 1);
        if (k + 2 < n) s += c2 * at(i, j, k + 2);
        out[g.idxNS(i, j, k)] = s;
      }
}

void poissonRhs(const Grid &g, const Vec &rhoP, int Z, Vec &rhs) {
  const int n = g.n;
  const double a = g.a, h = g.h, hh = h * h;
  const std::size_t ns = g.ns();
  const double eps0inv = kE2 * 4 * M_PI;
  Vec Q20int(ns), Q22int(ns);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      for (int k = 0; k < n; k++) {
        std::size_t id = g.idxNS(i, j, k);
        double x = g.xs[i], y = g.xs[j], z = g.xs[k];
        Q20int[id] = rhoP[id] * (2.0 * z * z - x * x - y * y);
        Q22int[id] = rhoP[id] * (x * x - y * y);
      }
  for (auto &q : Q20int) q *= std::sqrt(5.0 / (16.0 * M_PI));
  for (auto &q : Q22int) q *= std::sqrt(15.0 / (32.0 * M_PI));
  double Q20 = integral(g, Q20int.data());
  double Q22 = integral(g, Q22int.data());
  const int nnew = n + 4;
  auto L = [](int i, int j, int k, int dim) {
    return (std::size_t)i * dim * dim + (std::size_t)j * dim + k;
  };
  Vec Uq((std::size_t)nnew * nnew * nnew);
  for (int k = 0; k < nnew; k++)
    for (int j = 0; j < nnew; j++)
      for (int i = 0; i < nnew; i++) {
        double x = -a - 2 * h + i * h, y = -a - 2 * h + j * h,
               z = -a - 2 * h + k * h;
        double r = std::sqrt(x * x + y * y + z * z);
        if (r < 1e-9) r = 1e-9;
        double v = (kE2 * Z) / r;
        v += kE2 * (Y20xyz(x, y, z) * Q20 + 2.0 * Y22xyz(x, y, z) * Q22) / r;
        Uq[L(i, j, k, nnew)] = v;
      }
  rhs.resize(ns);
  for (std::size_t p = 0; p < ns; ++p) rhs[p] = -eps0inv * rhoP[p];
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j) {
      rhs[L(0, j, k, n)] -= (16.0 / 12.0) * Uq[L(1, j + 2, k + 2, nnew)] / hh;
      rhs[L(0, j, k, n)] += (1.0 / 12.0) * Uq[L(0, j + 2, k + 2, nnew)] / hh;
      rhs[L(1, j, k, n)] += (1.0 / 12.0) * Uq[L(1, j + 2, k + 2, nnew)] / hh;
    }
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j) {
      rhs[L(n - 1, j, k, n)] -=
          (16.0 / 12.0) * Uq[L(n + 2, j + 2, k + 2, nnew)] / hh;
      rhs[L(n - 1, j, k, n)] +=
          (1.0 / 12.0) * Uq[L(n + 3, j + 2, k + 2, nnew)] / hh;
      rhs[L(n - 2, j, k, n)] +=
          (1.0 / 12.0) * Uq[L(n + 2, j + 2, k + 2, nnew)] / hh;
    }
  for (int k = 0; k < n; ++k)
    for (int i = 0; i < n; ++i) {
      rhs[L(i, 0, k, n)] -= (16.0 / 12.0) * Uq[L(i + 2, 1, k + 2, nnew)] / hh;
      rhs[L(i, 0, k, n)] += (1.0 / 12.0) * Uq[L(i + 2, 0, k + 2, nnew)] / hh;
      rhs[L(i, 1, k, n)] += (1.0 / 12.0) * Uq[L(i + 2, 1, k + 2, nnew)] / hh;
    }
  for (int k = 0; k < n; ++k)
    for (int i = 0; i < n; ++i) {
      rhs[L(i, n - 1, k, n)] -=
          (16.0 / 12.0) * Uq[L(i + 2, n + 2, k + 2, nnew)] / hh;
      rhs[L(i, n - 1, k, n)] +=
          (1.0 / 12.0) * Uq[L(i + 2, n + 3, k + 2, nnew)] / hh;
      rhs[L(i, n - 2, k, n)] +=
          (1.0 / 12.0) * Uq[L(i + 2, n + 2, k + 2, nnew)] / hh;
    }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      rhs[L(i, j, 0, n)] -= (16.0 / 12.0) * Uq[L(i + 2, j + 2, 1, nnew)] / hh;
      rhs[L(i, j, 0, n)] += (1.0 / 12.0) * Uq[L(i + 2, j + 2, 0, nnew)] / hh;
      rhs[L(i, j, 1, n)] += (1.0 / 12.0) * Uq[L(i + 2, j + 2, 1, nnew)] / hh;
    }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      rhs[L(i, j, n - 1, n)] -=
          (16.0 / 12.0) * Uq[L(i + 2, j + 2, n + 2, nnew)] / hh;
      rhs[L(i, j, n - 1, n)] +=
          (1.0 / 12.0) * Uq[L(i + 2, j + 2, n + 3, nnew)] / hh;
      rhs[L(i, j, n - 2, n)] +=
          (1.0 / 12.0) * Uq[L(i + 2, j + 2, n + 2, nnew)] / hh;
    }
}

int poisson(const Grid &g, const Vec &rhoP, int Z, const Vec *Uguess,
            Vec &U) {
  Vec rhs;
  poissonRhs(g, rhoP, Z, rhs);
  const std::size_t ns = g.ns();
  // CG on (-L) U = -rhs
  U = Uguess ? *Uguess : Vec(ns, 0.0);
  Vec r(ns), p(ns), Ap(ns);
  lap5(g, U.data(), Ap.data());
  double bn = 0, rr = 0;
  for (std::size_t i = 0; i < ns; ++i) {
    r[i] = -rhs[i] + Ap[i]; // b - A x with A = -L, b = -rhs
    bn += rhs[i] * rhs[i];
    rr += r[i] * r[i];
  }
  if (bn == 0) {
    U.assign(ns, 0.0);
    return 0;
  }
  const double tol2 = 1e-28 * bn;
  p = r;
  int it = 0;
  const int maxit = 4 * (int)ns;
  while (rr > tol2 && it < maxit) {
    lap5(g, p.data(), Ap.data());
    double pAp = 0;
    for (std::size_t i = 0; i < ns; ++i) pAp += -p[i] * Ap[i];
    double alpha = rr / pAp;
    double rrn = 0;
    for (std::size_t i = 0; i < ns; ++i) {
      U[i] += alpha * p[i];
      r[i] -= alpha * (-Ap[i]);
      rrn += r[i] * r[i];
    }
    double beta = rrn / rr;
    rr = rrn;
    for (std::size_t i = 0; i < ns; ++i) p[i] = r[i] + beta * p[i];
    ++it;
  }
  return it;
}

static Vec exchangeCoulomb(const Vec &rhoP) {
  Vec res(rhoP.size(), 0.0);
  for (std::size_t i = 0; i < rhoP.size(); ++i)
    res[i] -= kE2 * std::pow(3.0 / M_PI, 1.0 / 3.0) * std::pow(rhoP[i], 1.0 / 3.0);
  return res;
}

// Wavefunction::field (wavefunction.cpp:264-310)
static Vec skyrmeField(const ncgm_edf &P, const Vec &rho, const Vec &rhoQ,
                       const Vec &tau, const Vec &tauQ, const Vec &n2rho,
                       const Vec &n2rhoQ, const Vec &divJ, const Vec &divJQ) {
  const std::size_t ns = rho.size();
  Vec field(ns, 0.0);
  double t3 = 48 * P.C0Drr / 3;
  double x3 = -0.5 - 24 * P.C1Drr / t3;
  double sigma = P.sigma;
  for (std::size_t i = 0; i < ns; ++i) {
    double f = 0.0;
    f += (2 * P.C0rr - 2 * P.C1rr) * rho[i] + 4 * P.C1rr * rhoQ[i];
    f += (P.C0rt - P.C1rt) * tau[i] + 2 * P.C1rt * tauQ[i];
    f += (2 * P.C0rdr - 2 * P.C1rdr) * n2rho[i] + 4 * P.C1rdr * n2rhoQ[i];
    f += (P.C0nJ - P.C1nJ) * divJ[i] + 2 * P.C1nJ * divJQ[i];
    double rm = rho[i] - rhoQ[i];
    f += (t3 / 12.0) * std::pow(rho[i], sigma - 1.0) *
         ((1.0 + 0.5 * x3) * (sigma + 2.0) * std::pow(rho[i], 2.0) -
          (x3 + 0.5) * (sigma * (rhoQ[i] * rhoQ[i] + rm * rm) +
                        2.0 * rho[i] * rhoQ[i]));
    field[i] = f;
  }
  return field;
}

// ---------------------------------------------------------------------------
// Pairing: BCS (src/util/bcs.cpp:10-321, iteration_data.cpp:384-465)
// ---------------------------------------------------------------------------
struct BCSResult {
  Vec u2, v2, Delta, qp;
  double lambda = 0, Epair = 0;
};

static std::vector<int> matchTimeReversal(const RMat &O, double thr = 1e-6) {
  int M = (int)O.rows;
  std::vector<std::tuple<double, int, int>> list;
  for (int k = 0; k < M; ++k)
    for (int j = 0; j < M; ++j) {
      double v = std::abs(O(k, j));
      if (v > thr) list.emplace_back(v, k, j);
    }
  std::stable_sort(list.begin(), list.end(), [](const auto &a, const auto &b) {
    return std::get<0>(a) > std::get<0>(b);
  });
  std::vector<int> partner(M, -1);
  std::vector<char> used(M, 0);
  for (auto &e : list) {
    int k = std::get<1>(e), j = std::get<2>(e);
    if (used[k] || used[j]) continue;
    if (k == j) continue;
    partner[k] = j;
    partner[j] = k;
    used[k] = used[j] = 1;
  }
  return partner;
}

static BCSResult solveBCS(const Vec &eps, const RMat &Gp, int A,
                          const ncgm_pairing &params, const Vec &oldDelta,
                          double oldLambda) {
  const double initDelta = 1.0, tol = 1e-10, PairingPrec = 1e-10;
  const int maxIter = 2000;
  const double EPS_SMALL = 1e-12;
  const int np = (int)eps.size();
  BCSResult res;
  if (np == 0) return res;
  RMat G(np, np);
  for (int i = 0; i < np * np; ++i) G.d[i] = 0.5 * Gp.d[i];
  Vec Delta(np, initDelta);
  if ((int)oldDelta.size() == np &&
      *std::max_element(oldDelta.begin(), oldDelta.end()) > 1e-3)
    Delta = oldDelta;
  const double ws = params.window / 10.0;
  double lambda = oldLambda;
  if (!std::isfinite(lambda)) {
    int mid = std::clamp((A / 2) - 1, 0, np - 1);
    lambda = eps[mid];
  }
  const double mixDelta = 0.9, mixLambda = 0.9;
  Vec ww(np), Eqp(np, 0.0);
  for (int iter = 0; iter < maxIter; ++iter) {
    double prevLambda = lambda;
    for (int p = 0; p < np; ++p) {
      ww[p] = 1.0 / (1.0 + std::exp((eps[p] - lambda - params.window) / ws));
      if (params.window_both)
        ww[p] *= 1.0 / (1.0 + std::exp(-(eps[p] - lambda + params.window) / ws));
    }
    for (int p = 0; p < np; ++p) {
      double xi = eps[p] - lambda;
      Eqp[p] = std::sqrt(xi * xi + Delta[p] * Delta[p] * ww[p]);
    }
    double sum1 = 0.0, sumInv = 0.0;
    for (int p = 0; p < np; ++p) {
      sum1 += (1.0 - eps[p] / Eqp[p]);
      sumInv += 1.0 / Eqp[p];
    }
    double raw = (sumInv < EPS_SMALL) ? prevLambda
                                      : (static_cast<double>(A) - sum1) / sumInv;
    lambda = mixLambda * raw + (1.0 - mixLambda) * lambda;
    Vec DeltaNew(np, 0.0);
    for (int p = 0; p < np; ++p) {
      double s = 0.0;
      for (int q = 0; q < np; ++q)
        if (ww[q] > EPS_SMALL) s += G(p, q) * ww[q] * Delta[q] / Eqp[q];
      DeltaNew[p] = s;
    }
    double dn2 = 0;
    Vec mixed(np);
    for (int p = 0; p < np; ++p) {
      mixed[p] = (1.0 - mixDelta) * Delta[p] + mixDelta * DeltaNew[p];
      dn2 += (mixed[p] - Delta[p]) * (mixed[p] - Delta[p]);
    }
    double ldiff = std::abs(raw - prevLambda);
    Delta = mixed;
    if (ldiff < PairingPrec && std::sqrt(dn2) < tol) break;
  }
  res.v2.resize(np);
  res.u2.resize(np);
  for (int i = 0; i < np; ++i) {
    ww[i] = 1.0 / (1.0 + std::exp((eps[i] - lambda - params.window) / ws));
    if (params.window_both)
      ww[i] *= 1.0 / (1.0 + std::exp(-(eps[i] - lambda + params.window) / ws));
    double xi = eps[i] - lambda;
    Eqp[i] = std::sqrt(xi * xi + Delta[i] * Delta[i] * ww[i]);
    double v2 = std::clamp(0.5 * (1 - xi / Eqp[i]), 0.0, 1.0);
    res.v2[i] = v2;
    res.u2[i] = 1 - v2;
  }
  double Ep = 0.0;
  for (int p = 0; p < np; ++p)
    for (int q = 0; q < np; ++q)
      if (ww[q] > EPS_SMALL)
        Ep += -0.5 * ww[q] * ww[p] * Delta[p] * Delta[q] * G(p, q) / Eqp[p] /
              Eqp[q];
  res.Delta = Delta;
  res.qp.resize(np);
  for (int i = 0; i < np; ++i) res.qp[i] = eps[i] * res.v2[i];
  res.lambda = lambda;
  res.Epair = Ep;
  return res;
}

// BCS::BCSiter (bcs.cpp:256-321)
static BCSResult bcsIter(const Grid &g, const CMat &phi, const Vec &eps, int A,
                         const ncgm_pairing &params, const Vec &oldDelta,
                         double oldLambda) {
  const int M = (int)phi.cols;
  CMat ov = adjointTimes(phi, timeReverse(g, phi));
  RMat O(M, M);
  for (int j = 0; j < M; ++j)
    for (int i = 0; i < M; ++i) O(i, j) = std::norm(ov(i, j));
  auto partners = matchTimeReversal(O);
  std::vector<int> unique;
  std::vector<int> s2p(M, 0);
  std::vector<bool> visited(M, false);
  for (int i = 0; i < M; ++i)
    if (!visited[i]) {
      int pt = partners[i];
      if (pt != i && pt != -1) {
        int pi = (int)unique.size();
        unique.push_back(i);
        s2p[i] = pi;
        s2p[pt] = pi;
        visited[i] = visited[pt] = true;
      }
    }
  const int np = (int)unique.size();
  Vec epsP(np);
  for (int p = 0; p < np; ++p) epsP[p] = eps[unique[p]];
  Vec oldU;
  if ((int)oldDelta.size() == np * 2) {
    oldU.resize(std::min(M / 2, np));
    for (int i = 0; i < (int)oldU.size(); ++i) oldU[i] = oldDelta[unique[i]];
  } else {
    oldU = oldDelta;
  }
  // compute_G_pairing (bcs.cpp:10-63): G_pq = V0 * int rho_p rho_q
  std::vector<Vec> dens(np);
  for (int p = 0; p < np; ++p) {
    dens[p].resize(g.ns());
    const cd *c = phi.col(unique[p]);
    for (std::size_t l = 0; l < g.ns(); ++l)
      dens[p][l] = std::norm(c[2 * l]) + std::norm(c[2 * l + 1]);
  }
  RMat Gp(np, np);
  Vec prod(g.ns());
  for (int p = 0; p < np; ++p)
    for (int q = 0; q < np; ++q) {
      for (std::size_t l = 0; l < g.ns(); ++l) prod[l] = dens[p][l] * dens[q][l];
      Gp(p, q) = params.V0 * integral(g, prod.data());
    }
  RMat Gs(np, np);
  for (int p = 0; p < np; ++p)
    for (int q = 0; q < np; ++q) Gs(p, q) = 0.5 * (Gp(p, q) + Gp(q, p));
  BCSResult pr = solveBCS(epsP, Gs, A, params, oldU, oldLambda);
  BCSResult fr;
  fr.u2.assign(M, 0.0);
  fr.v2.assign(M, 0.0);
  fr.Delta.assign(M, 0.0);
  for (int i = 0; i < M; ++i)
    if (visited[i]) {
      int pi = s2p[i];
      fr.u2[i] = pr.u2[pi];
      fr.v2[i] = pr.v2[pi];
      fr.Delta[i] = pr.Delta[pi];
    }
  fr.qp.resize(M);
  for (int i = 0; i < M; ++i) fr.qp[i] = eps[i] * fr.v2[i];
  fr.lambda = pr.lambda;
  fr.Epair = pr.Epair;
  return fr;
}

// ---------------------------------------------------------------------------
// HFB (iteration_data.cpp:467-850)
// ---------------------------------------------------------------------------
struct UV {
  RMat U, V, kappa;
  Vec pairingField;
  double lambda = 0, energy = 0;
};

static CMat numericalTR(const Grid &g, const CMat &phi) {
  CMat out(phi.rows, phi.cols);
  CMat tr = timeReverse(g, phi);
  for (std::size_t c = 0; c < phi.cols; ++c) {
    if (c % 2 == 1)
      std::copy(tr.col(c - 1), tr.col(c - 1) + phi.rows, out.col(c));
    else
      std::copy(phi.col(c), phi.col(c) + phi.rows, out.col(c));
  }
  return out;
}

static UV nullHFB(int target, const Vec &e) {
  UV h;
  int M = (int)e.size();
  h.lambda = e[target - 1];
  h.V = RMat(M, M);
  h.U = RMat(M, M);
  h.pairingField.assign(M, 0.0);
  h.energy = 0.0;
  for (int i = 0; i < target; ++i) h.V(i, i) = 1.0;
  return h;
}

static UV hfbSpecies(const Grid &g, const CMat &phi, const Vec &e,
                     const UV &prev, int target, const ncgm_pairing &params,
                     double pairingThreshold) {
  const double window = params.window, smooth = params.window / 10.0;
  auto ff = [&](double en, double lam) {
    double v = 1.0 / (1.0 + std::exp((en - lam - window) / smooth));
    v *= 1.0 / (1.0 + std::exp(-(en - lam + window) / smooth));
    return std::sqrt(v);
  };
  double lambda = prev.lambda;
  const int M = (int)e.size();
  Vec fac(M);
  for (int i = 0; i < M; ++i) fac[i] = ff(e[i], lambda);
  int start = 0, end = M - 1;
  for (int i = 0; i < M; i += 2)
    if (fac[i] > pairingThreshold) {
      start = i;
      break;
    }
  for (int i = start; i < M; i += 2)
    if (fac[i] < pairingThreshold) {
      end = i;
      break;
    }
  const int nS = end - start + 1;
  CMat pr = numericalTR(g, phi);
  const std::size_t ns = g.ns();
  // kappa_field (iteration_data.cpp:467-501)
  Vec kappa_r(ns, 0.0);
  {
    std::vector<cd> acc(ns, cd(0, 0));
    for (int a = start; a < end + 1; ++a)
      for (int b = start; b < end + 1; ++b) {
        double kab = prev.kappa(a, b);
        for (std::size_t l = 0; l < ns; ++l)
          for (int s = 0; s < 2; ++s) {
            double sg = s == 0 ? 1.0 : -1.0;
            acc[l] += -(sg * pr(2 * l + (1 - s), b) * pr(2 * l + s, a) * fac[a] *
                        fac[b]) *
                      kab;
          }
      }
    for (std::size_t l = 0; l < ns; ++l) kappa_r[l] = acc[l].real();
  }
  // delta_matrix (iteration_data.cpp:503-538)
  RMat Delta(nS, nS);
  {
    std::vector<cd> tmp(ns);
    const double hhh = g.h * g.h * g.h;
    for (int a = start; a < end + 1; ++a)
      for (int b = start; b < end + 1; ++b) {
        if (b < a) continue;
        std::fill(tmp.begin(), tmp.end(), cd(0, 0));
        for (std::size_t l = 0; l < ns; ++l)
          for (int s = 0; s < 2; ++s) {
            double sg = s == 0 ? 1.0 : -1.0;
            tmp[l] += sg * (pr(2 * l + s, a) * pr(2 * l + (1 - s), b)) * fac[a] *
                      fac[b];
          }
        cd val(0, 0);
        for (int k = 0; k < g.n; ++k)
          for (int j = 0; j < g.n; ++j)
            for (int i = 0; i < g.n; ++i) {
              std::size_t l = g.idxNS(i, j, k);
              double w = 1.0;
              if (i == 0 || i == g.n - 1) w *= 0.5;
              if (j == 0 || j == g.n - 1) w *= 0.5;
              if (k == 0 || k == g.n - 1) w *= 0.5;
              val += (std::conj(tmp[l]) * kappa_r[l]) * hhh * w;
            }
        Delta(a - start, b - start) = 0.5 * params.V0 * val.real();
        Delta(b - start, a - start) = -0.5 * params.V0 * val.real();
      }
  }
  double dn = 0;
  for (double x : Delta.d) dn += x * x;
  if (std::sqrt(dn) < 1e-3) return nullHFB(target, e);

  double bmin = lambda - 1.7, bmax = lambda + 1.7;
  double cur = lambda;
  RMat U(nS, nS), V(nS, nS);
  RMat H(2 * nS, 2 * nS);
  for (int bIter = 0; bIter < 100; ++bIter) {
    for (auto &x : H.d) x = 0.0;
    for (int i = 0; i < nS; ++i) {
      H(i, i) = e[start + i] - cur;
      H(nS + i, nS + i) = -(e[start + i] - cur);
    }
    for (int j = 0; j < nS; ++j)
      for (int i = 0; i < nS; ++i) {
        H(i, nS + j) = Delta(i, j);
        H(nS + i, j) = -Delta(i, j);
      }
    std::vector<double> w;
    RMat Ev;
    symmetricEig(H, w, Ev);
    double num = 0.0;
    for (int k = 0; k < nS; ++k) {
      int q = k + nS;
      for (int i = 0; i < nS; ++i) {
        U(i, k) = Ev(i, q);
        V(i, k) = Ev(nS + i, q);
        num += V(i, k) * V(i, k);
      }
    }
    num += start;
    double diff = num - target;
    if (std::abs(diff) < 1e-12) break;
    if (diff > 0) bmax = cur;
    else bmin = cur;
    cur = (bmax + bmin) / 2.0;
  }
  lambda = cur;
  // kappaNew = V U^T, pairingEnergy = 0.5 tr(Delta kappaNew^T)
  double pe = 0.0;
  for (int i = 0; i < nS; ++i)
    for (int j = 0; j < nS; ++j) {
      double kij = 0; // kappaNew(i, j) = (V U^T)(i, j)
      for (int k = 0; k < nS; ++k) kij += V(i, k) * U(j, k);
      pe += Delta(i, j) * kij; // tr(Delta kappa^T) = sum_ij Delta_ij kappa_ij
    }
  pe *= 0.5;
  UV out;
  out.U = RMat(M, M);
  out.V = RMat(M, M);
  for (int j = 0; j < nS; ++j)
    for (int i = 0; i < nS; ++i) {
      out.V(start + i, start + j) = V(i, j);
      out.U(start + i, start + j) = U(i, j);
    }
  for (int i = 0; i < start; ++i) out.V(i, i) = 1.0;
  for (int i = end + 1; i < M; ++i) out.U(i, i) = 1.0;
  out.kappa = RMat(M, M);
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < M; ++j) {
      double s = 0;
      for (int k = 0; k < M; ++k) s += out.U(i, k) * out.V(j, k);
      out.kappa(i, j) = s;
    }
  out.pairingField = kappa_r;
  out.lambda = lambda;
  out.energy = pe;
  return out;
}

// ---------------------------------------------------------------------------
// Constraints (src/skyrme/*_constraint.cpp): augmented-Lagrangian penalty.
// ---------------------------------------------------------------------------
struct Constraint {
  int kind; // 0 xcm 1 ycm 2 zcm 3 x2-y2 4 xy 5 Q30 6 Q20
  double target, C, lambda = 0, value = 0, gamma;
  bool firstIter = true;
  Vec O;
  // error() (src/skyrme/constraint.cpp:3-10); COM constraints report 0
  // (xcm_constraint.cpp:13). x2-y2 / xy / Q30 compare against the base-class
  // target, which those classes never set; it is taken as 0.
  double error() const {
    if (kind <= 2) return 0.0;
    double t = (kind == 6 || kind >= 1000) ? target : 0.0;
    if (std::abs(t) <= 1e-12) return std::abs(value);
    return std::abs(value / t - 1.0);
  }
};

static Vec constraintOperator(const Grid &g, int kind) {
  Vec O(g.ns());
  for (int k = 0; k < g.n; ++k)
    for (int j = 0; j < g.n; ++j)
      for (int i = 0; i < g.n; ++i) {
        double x = g.xs[i], y = g.xs[j], z = g.xs[k];
        double v = 0;
        switch (kind) {
        case 0: v = x; break;
        case 1: v = y; break;
        case 2: v = z; break;
        case 3: v = std::pow(x, 2) - std::pow(y, 2); break;
        case 4: v = 2.0 * x * y; break;
        case 5: {
          double r = std::sqrt(x * x + y * y + z * z);
          double ct = std::cos(std::acos(z / r));
          double Y30 = std::sqrt(7.0 / (4.0 * M_PI)) * 0.5 *
                       (5.0 * ct * ct * ct - 3.0 * ct);
          v = std::pow(std::abs(r), 3) * Y30;
          break;
        }
        case 6:
          v = 0.25 * std::sqrt(5 / (M_PI)) *
              (2.0 * std::pow(z, 2) - std::pow(y, 2) - std::pow(x, 2));
          break;
        }
        O[g.idxNS(i, j, k)] = v;
      }
  return O;
}

static Constraint makeConstraint(const Grid &g, int kind, double target) {
  Constraint c;
  c.kind = kind;
  c.target = target;
  c.C = (kind <= 2) ? 0.05 : (kind == 5 ? 0.001 : 0.005);
  c.gamma = (kind <= 2) ? 0.2 : 0.3;
  c.O = constraintOperator(g, kind);
  return c;
}

static double qValue(const Grid &g, const Constraint &c, const Vec &rho) {
  Vec f(rho.size());
  for (std::size_t i = 0; i < rho.size(); ++i) f[i] = c.O[i] * rho[i];
  return integral(g, f.data());
}

static double constraintEvaluate(const Grid &g, const Constraint &c,
                                 const Vec &rho) {
  double Q = qValue(g, c, rho);
  return c.C * std::pow(Q - c.target, 2) + c.lambda * (Q - c.target);
}

// getField of each constraint class; energyDiff / constraintTol gate the COM
// multiplier update (xcm_constraint.cpp:50-53).
static Vec constraintField(const Grid &g, Constraint &c, const Vec &rho,
                           double energyDiff) {
  double Q = qValue(g, c, rho);
  double mu;
  if (c.kind >= 1000) {
    // MultipoleConstraint::getField (multipole_constraint.cpp:18-40)
    c.lambda += c.gamma * 2.0 * c.C * (Q - c.target);
    mu = c.target - c.lambda / (2.0 * c.C);
    c.value = Q;
  } else if (c.firstIter) {
    c.firstIter = false;
    mu = (c.kind == 6) ? c.target - c.lambda / (2.0 * c.C) : c.target;
  } else {
    if (c.kind > 2 || energyDiff < 5e-3)
      c.lambda += c.gamma * 2.0 * c.C * (Q - c.target);
    mu = c.target - c.lambda / (2.0 * c.C);
    c.value = Q;
  }
  Vec out(rho.size());
  for (std::size_t i = 0; i < rho.size(); ++i)
    out[i] = 2.0 * c.C * (Q - mu) * c.O[i];
  return out;
}

// ---------------------------------------------------------------------------
// Harmonic-oscillator spinor guess (src/solver/guess.cpp:10-248, spin-orbit
// branch) with SphericalHarmonics::Y (spherical_harmonics.cpp:10-99).
// ---------------------------------------------------------------------------
static double factorial(int n) {
  double r = 1.0;
  for (int i = 2; i <= n; i++) r *= i;
  return r;
}
static double assocLegendre(int l, int m, double x) {
  double pmm = 1.0;
  if (m > 0) {
    double fact = 1.0;
    for (int i = 1; i <= 2 * m - 1; i += 2) fact *= i;
    pmm = fact * std::pow(1.0 - x * x, m / 2.0);
  }
  if (l == m) return pmm;
  double pmmp1 = x * (2 * m + 1) * pmm;
  if (l == m + 1) return pmmp1;
  double pll = 0.0, p1 = pmmp1, p2 = pmm;
  for (int ll = m + 2; ll <= l; ++ll) {
    pll = ((2 * ll - 1) * x * p1 - (ll + m - 1) * p2) / (ll - m);
    p2 = p1;
    p1 = pll;
  }
  return pll;
}
static cd Ylm(int l, int m, double theta, double phi) {
  int mm = std::abs(m);
  double norm = std::sqrt(((2.0 * l + 1.0) / (4.0 * M_PI)) *
                          (factorial(l - mm) / factorial(l + mm)));
  double leg = assocLegendre(l, mm, std::cos(theta));
  cd phase = std::polar(1.0, mm * phi);
  cd res = std::pow(-1.0, mm) * norm * leg * phase;
  if (m < 0) return std::pow(-1.0, mm) * std::conj(res);
  return res;
}

// MultipoleConstraint's operator X_lm r^l (multipole_constraint.cpp:24-27)
// with SphericalHarmonics::X (spherical_harmonics.cpp:45-58)
static Vec multipoleOperator(const Grid &g, int l, int m) {
  Vec O(g.ns());
  for (int k = 0; k < g.n; ++k)
    for (int j = 0; j < g.n; ++j)
      for (int i = 0; i < g.n; ++i) {
        const double x = g.xs[i], y = g.xs[j], z = g.xs[k];
        const double r = std::sqrt(x * x + y * y + z * z);
        const double th = std::acos(z / r), ph = std::atan2(y, x);
        double X;
        if (m > 0) {
          const cd Y = Ylm(l, -m, th, ph);
          X = (Y + std::conj(Y)).real() / std::sqrt(2.0);
        } else if (m < 0) {
          const cd Y = Ylm(l, m, th, ph);
          X = (cd(0, -1) * (Y - std::conj(Y))).real() / std::sqrt(2.0);
        } else {
          X = Ylm(l, 0, th, ph).real();
        }
        O[g.idxNS(i, j, k)] = X * std::pow(std::abs(r), (double)l);
      }
  return O;
}

CMat hoGuess(const Grid &g, int nev, double omega, double /*beta*/) {
  CMat guess(g.N(), nev);
  auto laguerre = [](int n, double alpha, double x) {
    if (n == 0) return 1.0;
    if (n == 1) return 1.0 + alpha - x;
    double Lnm2 = 1.0, Lnm1 = 1.0 + alpha - x, Ln = 0.0;
    for (int k = 2; k <= n; ++k) {
      Ln = ((2.0 * k - 1.0 + alpha - x) * Lnm1 - (k - 1.0 + alpha) * Lnm2) / k;
      Lnm2 = Lnm1;
      Lnm1 = Ln;
    }
    return Ln;
  };
  auto radial = [&](int nr, int l, double r) {
    double rho = r / omega;
    double norm = std::sqrt(2.0 * std::tgamma(nr + 1.0) /
                            (omega * omega * omega * std::tgamma(nr + l + 1.5)));
    return norm * std::pow(rho, l) * laguerre(nr, l + 0.5, rho * rho) *
           std::exp(-0.5 * rho * rho);
  };
  std::vector<std::tuple<int, int, int, int>> orbs;
  for (int N = 0; (int)orbs.size() < nev; ++N)
    for (int nr = 0; nr <= N / 2 && (int)orbs.size() < nev; ++nr) {
      int l = N - 2 * nr;
      int jp = 2 * l + 1;
      for (int m = 1; m <= jp && (int)orbs.size() < nev; m += 2) {
        orbs.emplace_back(nr, l, jp, m);
        if ((int)orbs.size() < nev) orbs.emplace_back(nr, l, jp, -m);
      }
      if (l > 0) {
        int jm = 2 * l - 1;
        for (int m = 1; m <= jm && (int)orbs.size() < nev; m += 2) {
          orbs.emplace_back(nr, l, jm, m);
          if ((int)orbs.size() < nev) orbs.emplace_back(nr, l, jm, -m);
        }
      }
    }
  for (int si = 0; si < (int)orbs.size() && si < nev; ++si) {
    int nr, l, j2, mj2;
    std::tie(nr, l, j2, mj2) = orbs[si];
    double mj = mj2 * 0.5;
    double denom = 2.0 * l + 1.0;
    double Cu, Cd;
    if (j2 == 2 * l + 1) {
      Cu = std::sqrt((l + mj + 0.5) / denom);
      Cd = std::sqrt((l - mj + 0.5) / denom);
    } else {
      Cu = std::sqrt((l - mj + 0.5) / denom);
      Cd = -std::sqrt((l + mj - 0.5) / denom);
    }
    int mlu = (mj2 - 1) / 2, mld = (mj2 + 1) / 2;
    bool hu = std::abs(mlu) <= l, hd = std::abs(mld) <= l;
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 0; i < g.n; ++i)
      for (int jg = 0; jg < g.n; ++jg)
        for (int k = 0; k < g.n; ++k) {
          double x = g.xs[i], y = g.xs[jg], z = g.xs[k];
          double r = std::sqrt(x * x + y * y + z * z);
          double theta = (r > 1e-12) ? std::acos(z / r) : 0.0;
          double phi = std::atan2(y, x);
          double R = radial(nr, l, r);
          cd up(0, 0), dn(0, 0);
          if (hu) up = (Cu * R) * Ylm(l, mlu, theta, phi);
          if (hd) dn = (Cd * R) * Ylm(l, mld, theta, phi);
          guess(g.idx(i, jg, k, 0), si) = up;
          guess(g.idx(i, jg, k, 1), si) = dn;
        }
    double s = std::sqrt(colNorm2(guess.col(si), g.N()));
    for (std::size_t r = 0; r < g.N(); ++r) guess(r, si) /= s;
  }
  return guess;
}

// ---------------------------------------------------------------------------
// Self-consistent state and driver (IterationData, src/util/
// iteration_data.cpp:852-1125; main(), src/main.cpp:38-369).
// ---------------------------------------------------------------------------
struct State {
  bool have = false;
  Vec rhoN, rhoP, tauN, tauP, divJN, divJP, n2N, n2P, gN, gP; // g*: n^3 x 3
  Vec JN, JP, JvN, JvP;                                        // 9 / 3 comps
  Vec fN, fP, gfN, gfP, UN, UP, UConstr, UCoul, UCDir, BN, BP;
  bool haveCoul = false;
  BCSResult bcsN, bcsP;
  UV hfbN, hfbP;
  double energyDiff = 1.0, massCorr = kMass;
  ncgm_pairing pN, pP;
};

static Vec leviCivita(const Vec &J, std::size_t ns) {
  Vec r(3 * ns);
  for (std::size_t i = 0; i < ns; ++i) {
    r[i] = J[(3 * 1 + 2) * ns + i] - J[(2 * 3 + 1) * ns + i];
    r[ns + i] = J[(3 * 2 + 0) * ns + i] - J[(3 * 0 + 2) * ns + i];
    r[2 * ns + i] = J[(3 * 0 + 1) * ns + i] - J[(3 * 1 + 0) * ns + i];
  }
  return r;
}

static void mix(Vec &old, const Vec &nw, double mu, bool have) {
  if (!have) {
    old = nw;
    return;
  }
  for (std::size_t i = 0; i < old.size(); ++i)
    old[i] = old[i] * (1.0 - mu) + nw[i] * mu;
}

struct Pair {
  CMat X;
  Vec e;
};

static CMat occupied(const Grid &g, const CMat &phi, const ncgm_hf_config &cfg,
                     const State &st, bool neutron, bool useBCS) {
  const ncgm_pairing &p = neutron ? st.pN : st.pP;
  if (useBCS) {
    const Vec &v2 = neutron ? st.bcsN.v2 : st.bcsP.v2;
    CMat out(phi.rows, phi.cols);
    for (std::size_t c = 0; c < phi.cols; ++c) {
      double s = std::sqrt(v2[c]);
      for (std::size_t r = 0; r < phi.rows; ++r) out(r, c) = phi(r, c) * s;
    }
    return out;
  }
  if (!p.active || cfg.pairing_type == NCGM_PAIRING_NONE) {
    // phi * nullOcc(particles).asDiagonal() (iteration_data.cpp:290-294,
    // 319-323). When pairing was switched off during the run the basis is
    // larger than the particle number; the reference's release build
    // (-DNDEBUG, no size check) then keeps the first `particles` columns
    const int particles = neutron ? cfg.A - cfg.Z : cfg.Z;
    if ((int)phi.cols <= particles) return phi;
    CMat out(phi.rows, particles);
    for (int c = 0; c < particles; ++c)
      for (std::size_t r = 0; r < phi.rows; ++r) out(r, c) = phi(r, c);
    return out;
  }
  if (cfg.pairing_type == NCGM_PAIRING_HFB) {
    const UV &h = neutron ? st.hfbN : st.hfbP;
    const int M = (int)h.V.rows;
    CMat rho(M, M);
    for (int i = 0; i < M; ++i)
      for (int j = 0; j < M; ++j) {
        double s = 0;
        for (int k = 0; k < M; ++k) s += h.V(i, k) * h.V(j, k);
        rho(i, j) = s;
      }
    std::vector<double> w;
    CMat Wm;
    hermitianEig(rho, w, Wm);
    for (auto &x : w)
      if (x < 1e-12) x = 0.0;
    CMat T(M, M);
    for (int j = 0; j < M; ++j)
      for (int i = 0; i < M; ++i) T(i, j) = Wm(i, j) * std::sqrt(w[j]);
    return times(phi, T);
  }
  // BCS
  const Vec &v2 = neutron ? st.bcsN.v2 : st.bcsP.v2;
  CMat out(phi.rows, phi.cols);
  for (std::size_t c = 0; c < phi.cols; ++c) {
    double s = std::sqrt(v2[c]);
    for (std::size_t r = 0; r < phi.rows; ++r) out(r, c) = phi(r, c) * s;
  }
  return out;
}

static void solvePairingBCS(const Grid &g, const ncgm_hf_config &cfg,
                            State &st, const Pair &n, const Pair &p) {
  int A = cfg.A, Z = cfg.Z, N = A - Z;
  auto nul = [&](const Pair &pr, int num) {
    BCSResult b;
    int M = (int)pr.e.size();
    b.u2.assign(M, 1.0);
    b.v2.assign(M, 0.0);
    for (int i = 0; i < num; ++i) {
      b.u2[i] = 0.0;
      b.v2[i] = 1.0;
    }
    b.Delta.assign(num, 0.0);
    b.qp.resize(M);
    for (int i = 0; i < M; ++i) b.qp[i] = b.v2[i] * pr.e[i];
    return b;
  };
  BCSResult nN = nul(n, N), nP = nul(p, Z);
  if (cfg.pairing_type == NCGM_PAIRING_NONE) {
    st.bcsN = nN;
    st.bcsP = nP;
  } else if (!st.have) {
    Vec tmp(1, 0.0);
    st.bcsN = st.pN.active ? bcsIter(g, n.X, n.e, N, st.pN, tmp,
                                     0.5 * (n.e[N - 1] + n.e[N]))
                           : nN;
    st.bcsP = st.pP.active ? bcsIter(g, p.X, p.e, Z, st.pP, tmp,
                                     0.5 * (p.e[Z - 1] + p.e[Z]))
                           : nP;
  } else {
    st.bcsN = st.pN.active ? bcsIter(g, n.X, n.e, N, st.pN, st.bcsN.Delta,
                                     st.bcsN.lambda)
                           : nN;
    st.bcsP = st.pP.active ? bcsIter(g, p.X, p.e, Z, st.pP, st.bcsP.Delta,
                                     st.bcsP.lambda)
                           : nP;
  }
  double sN = 0, sP = 0;
  for (double v : st.bcsN.v2) sN += v;
  for (double v : st.bcsP.v2) sP += v;
  if (std::isnan(sN) || std::isnan(sP)) {
    st.bcsN = nN;
    st.bcsP = nP;
  }
}

struct PhaseTimes {
  double gcg = 0, fields = 0, poisson = 0, pairing = 0;
};
static double now() {
  return std::chrono::duration<double>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

static void updateQuantities(const Grid &g, const ncgm_hf_config &cfg,
                             State &st, const Pair &n, const Pair &p, int iter,
                             std::vector<Constraint> &cons, PhaseTimes &pt) {
  const std::size_t ns = g.ns();
  const int Z = cfg.Z;
  double mu = cfg.density_mix;
  double t0 = now();
  bool bcsOcc = false;
  if (cfg.pairing_type == NCGM_PAIRING_HFB) {
    if (iter < cfg.start_hfb_iter) {
      solvePairingBCS(g, cfg, st, n, p);
      bcsOcc = true;
    } else {
      if (iter == cfg.start_hfb_iter) {
        auto seed = [&](UV &h, const BCSResult &b, int M) {
          h.pairingField.clear();
          h.kappa = RMat(M, M);
          h.V = RMat(M, M);
          h.lambda = b.lambda;
          for (int i = 0; i < M - 1; ++i) {
            int j = i + 1;
            if (i % 2 == 0) {
              double uv = std::sqrt(b.u2[i] * b.v2[i]);
              h.kappa(i, j) = uv;
              h.kappa(j, i) = -1.0 * uv;
            }
          }
        };
        seed(st.hfbN, st.bcsN, (int)n.e.size());
        seed(st.hfbP, st.bcsP, (int)p.e.size());
      }
      auto run = [&](UV &h, const Pair &pr, int target, ncgm_pairing &pp) {
        if (!pp.active) return;
        UV nw = hfbSpecies(g, pr.X, pr.e, h, target, pp, cfg.pairing_threshold);
        if (std::isnan(nw.energy)) {
        } else if (std::abs(nw.energy) < 1e-12) {
          pp.active = 0;
        } else {
          h = nw;
        }
      };
      run(st.hfbN, n, cfg.A - cfg.Z, st.pN);
      run(st.hfbP, p, cfg.Z, st.pP);
    }
  } else {
    solvePairingBCS(g, cfg, st, n, p);
  }
  pt.pairing += now() - t0;
  t0 = now();
  CMat neu = occupied(g, n.X, cfg, st, true, bcsOcc);
  CMat pro = occupied(g, p.X, cfg, st, false, bcsOcc);
  bool have = st.have;
  mix(st.rhoN, density(g, neu), mu, have);
  mix(st.rhoP, density(g, pro), mu, have);
  Vec rho(ns);
  for (std::size_t i = 0; i < ns; ++i) rho[i] = st.rhoN[i] + st.rhoP[i];
  st.gN = gradNoSpin(g, st.rhoN);
  st.gP = gradNoSpin(g, st.rhoP);
  Vec gr(3 * ns);
  for (std::size_t i = 0; i < 3 * ns; ++i) gr[i] = st.gN[i] + st.gP[i];
  mix(st.tauN, kineticDensity(g, neu), mu, have);
  mix(st.tauP, kineticDensity(g, pro), mu, have);
  st.n2N = lapNoSpin(g, st.rhoN);
  st.n2P = lapNoSpin(g, st.rhoP);
  mix(st.JN, soDensity(g, neu), mu, have);
  mix(st.JP, soDensity(g, pro), mu, have);
  st.JvN = leviCivita(st.JN, ns);
  st.JvP = leviCivita(st.JP, ns);
  mix(st.divJN, divJ(g, neu), mu, have);
  mix(st.divJP, divJ(g, pro), mu, have);
  Vec dJN(ns, 0.0), dJP(ns, 0.0);
  if (cfg.spin_orbit) {
    dJN = st.divJN;
    dJP = st.divJP;
  }
  Vec dJ(ns), tau(ns), n2(ns);
  for (std::size_t i = 0; i < ns; ++i) {
    dJ[i] = dJN[i] + dJP[i];
    tau[i] = st.tauN[i] + st.tauP[i];
    n2[i] = st.n2N[i] + st.n2P[i];
  }
  const ncgm_edf &P = cfg.edf;
  // EffectiveMass (src/util/effective_mass.cpp:7-34)
  auto mass = [&](const Vec &rq, const Vec &grq, Vec &f, Vec &gf) {
    f.assign(ns, 0.0);
    gf.assign(3 * ns, 0.0);
    for (std::size_t i = 0; i < ns; ++i) {
      f[i] += 1.0 * kHbar * kHbar / (2 * st.massCorr);
      f[i] += (P.C0rt - P.C1rt) * rho[i] + 2 * P.C1rt * rq[i];
    }
    for (std::size_t i = 0; i < 3 * ns; ++i)
      gf[i] += (P.C0rt - P.C1rt) * gr[i] + 2 * P.C1rt * grq[i];
  };
  mass(st.rhoN, st.gN, st.fN, st.gfN);
  mass(st.rhoP, st.gP, st.fP, st.gfP);
  Vec UNn = skyrmeField(P, rho, st.rhoN, tau, st.tauN, n2, st.n2N, dJ, dJN);
  Vec UPn = skyrmeField(P, rho, st.rhoP, tau, st.tauP, n2, st.n2P, dJ, dJP);
  Vec cf(ns, 0.0);
  if (iter > 0)
    for (auto &c : cons) {
      Vec f = constraintField(g, c, rho, st.energyDiff);
      for (std::size_t i = 0; i < ns; ++i) cf[i] += f[i];
    }
  pt.fields += now() - t0;
  Vec coul(ns, 0.0);
  if (cfg.use_coulomb) {
    double tp = now();
    Vec U;
    poisson(g, st.rhoP, Z, st.haveCoul ? &st.UCDir : nullptr, U);
    st.UCDir = U;
    Vec ex = exchangeCoulomb(st.rhoP);
    for (std::size_t i = 0; i < ns; ++i) coul[i] = U[i] + ex[i];
    pt.poisson += now() - tp;
  }
  t0 = now();
  st.UN = UNn;
  st.UP = UPn;
  st.UConstr = cf;
  for (std::size_t i = 0; i < ns; ++i) {
    st.UN[i] += st.UConstr[i];
    st.UP[i] += st.UConstr[i];
  }
  st.UCoul = coul;
  st.haveCoul = cfg.use_coulomb;
  st.BN.assign(3 * ns, 0.0);
  st.BP.assign(3 * ns, 0.0);
  if (cfg.spin_orbit)
    for (std::size_t i = 0; i < 3 * ns; ++i) {
      double s = st.gN[i] + st.gP[i];
      st.BN[i] += -(P.C0nJ - P.C1nJ) * s;
      st.BN[i] += -2 * P.C1nJ * st.gN[i];
      st.BP[i] += -(P.C0nJ - P.C1nJ) * s;
      st.BP[i] += -2 * P.C1nJ * st.gP[i];
    }
  if (cfg.use_j)
    for (std::size_t i = 0; i < 3 * ns; ++i) {
      double s = st.JvN[i] + st.JvP[i];
      st.BN[i] += 2 * (P.C0J2 - P.C1J2) * s;
      st.BN[i] += 4 * P.C1J2 * st.JvN[i];
      st.BP[i] += 2 * (P.C0J2 - P.C1J2) * s;
      st.BP[i] += 4 * P.C1J2 * st.JvP[i];
    }
  st.have = true;
  pt.fields += now() - t0;
}

// Energies (iteration_data.cpp:153-271, iteration_data_integrals.cpp:95-262)
struct Energies {
  double Eint, kin, Epn, Epp;
};
static double epair(const ncgm_hf_config &cfg, const State &st, bool neutron) {
  if (cfg.pairing_type == NCGM_PAIRING_NONE) return 0.0;
  const ncgm_pairing &p = neutron ? st.pN : st.pP;
  if (!p.active) return 0.0;
  if (cfg.pairing_type == NCGM_PAIRING_HFB)
    return neutron ? st.hfbN.energy : st.hfbP.energy;
  return neutron ? st.bcsN.Epair : st.bcsP.Epair;
}
static double totalEnergyIntegral(const Grid &g, const ncgm_hf_config &cfg,
                                  const State &st) {
  const std::size_t ns = g.ns();
  const ncgm_edf &P = cfg.edf;
  Vec f0(ns), f1(ns), fr0(ns), fr1(ns), ft0(ns), ft1(ns), fj0(ns), fj1(ns),
      fd0(ns), fd1(ns), fc(ns), fs(ns);
  for (std::size_t i = 0; i < ns; ++i) {
    double r0 = st.rhoN[i] + st.rhoP[i], r1 = st.rhoN[i] - st.rhoP[i];
    double t0 = st.tauN[i] + st.tauP[i], t1 = st.tauN[i] - st.tauP[i];
    double l0 = st.n2N[i] + st.n2P[i], l1 = st.n2N[i] - st.n2P[i];
    double rs = std::pow(r0, P.sigma);
    f0[i] = (P.C0rr * 1.0 + P.C0Drr * rs) * (r0 * r0);
    f1[i] = (P.C1rr * 1.0 + P.C1Drr * rs) * (r1 * r1);
    fr0[i] = P.C0rdr * (r0 * l0);
    fr1[i] = P.C1rdr * (l1 * r1);
    ft0[i] = P.C0rt * (t0 * r0);
    ft1[i] = P.C1rt * (t1 * r1);
    double j0 = 0, j1 = 0;
    for (int a = 0; a < 3; ++a) {
      double s0 = st.JvN[a * ns + i] + st.JvP[a * ns + i];
      double s1 = st.JvN[a * ns + i] - st.JvP[a * ns + i];
      j0 += s0 * s0;
      j1 += s1 * s1;
    }
    fj0[i] = P.C0J2 * j0;
    fj1[i] = P.C1J2 * j1;
    fd0[i] = P.C0nJ * ((st.divJN[i] + st.divJP[i]) * r0);
    fd1[i] = P.C1nJ * ((st.divJN[i] - st.divJP[i]) * r1);
    fc[i] = cfg.use_coulomb ? st.rhoP[i] * st.UCDir[i] : 0.0;
    fs[i] = std::pow(st.rhoP[i], 4.0 / 3.0) * (-3.0 * kE2 / 4.0) *
            std::pow(3.0 / M_PI, 1.0 / 3.0);
  }
  double eC0 = integral(g, f0.data()), eC1 = integral(g, f1.data());
  double eN0 = integral(g, fr0.data()), eN1 = integral(g, fr1.data());
  double eT0 = integral(g, ft0.data()), eT1 = integral(g, ft1.data());
  double eJ0 = integral(g, fj0.data()), eJ1 = integral(g, fj1.data());
  double eD0 = integral(g, fd0.data()), eD1 = integral(g, fd1.data());
  double eCd = cfg.use_coulomb ? 0.5 * integral(g, fc.data()) : 0.0;
  double eSl = cfg.use_coulomb ? integral(g, fs.data()) : 0.0;
  return eC0 + eC1 + eN0 + eN1 + eT0 + eT1 + eCd + epair(cfg, st, true) +
         epair(cfg, st, false) + eSl + eJ0 + eJ1 + eD0 + eD1;
}
static double kineticEnergy(const Grid &g, const State &st) {
  const std::size_t ns = g.ns();
  Vec t(ns);
  for (std::size_t i = 0; i < ns; ++i)
    t[i] = 0.5 * kHbar * kHbar * st.tauN[i] / st.massCorr +
           0.5 * kHbar * kHbar * st.tauP[i] / st.massCorr;
  return integral(g, t.data());
}
static double HFEnergy(const Grid &g, const ncgm_hf_config &cfg,
                       const State &st, std::vector<Constraint> &cons) {
  const std::size_t ns = g.ns();
  Vec rho(ns);
  for (std::size_t i = 0; i < ns; ++i) rho[i] = st.rhoN[i] + st.rhoP[i];
  double ce = 0;
  for (auto &c : cons) ce += constraintEvaluate(g, c, rho);
  double qN = 0, qP = 0;
  for (double v : st.bcsN.qp) qN += v;
  for (double v : st.bcsP.qp) qP += v;
  const ncgm_edf &P = cfg.edf;
  Vec fr(ns), fs(ns);
  for (std::size_t i = 0; i < ns; ++i) {
    double r0 = rho[i], r1 = st.rhoN[i] - st.rhoP[i];
    fr[i] = -0.5 * P.sigma *
            (P.C0Drr * std::pow(r0, P.sigma + 2) +
             P.C1Drr * std::pow(r0, P.sigma) * (r1 * r1));
    fs[i] = std::pow(st.rhoP[i], 4.0 / 3.0) * (-3.0 * kE2 / 4.0) *
            std::pow(3.0 / M_PI, 1.0 / 3.0);
  }
  double erear = integral(g, fr.data());
  double slater = cfg.use_coulomb ? integral(g, fs.data()) : 0.0;
  return ce + 0.5 * (qN + qP + kineticEnergy(g, st)) + erear + slater / 3.0 +
         epair(cfg, st, true) + epair(cfg, st, false);
}

static void quadDef(const Grid &g, const State &st, int A, double &beta,
                    double &gamma) {
  const std::size_t ns = g.ns();
  Vec f20(ns), f22(ns);
  for (int k = 0; k < g.n; ++k)
    for (int j = 0; j < g.n; ++j)
      for (int i = 0; i < g.n; ++i) {
        std::size_t l = g.idxNS(i, j, k);
        double x = g.xs[i], y = g.xs[j], z = g.xs[k];
        double r0 = st.rhoN[l] + st.rhoP[l];
        f20[l] = std::sqrt(5.0 / (16.0 * M_PI)) * (2 * z * z - x * x - y * y) * r0;
        f22[l] = std::sqrt(15.0 / (32.0 * M_PI)) * (x * x - y * y) * r0;
      }
  double a20 = integral(g, f20.data()), a22 = integral(g, f22.data());
  double R = 1.2 * std::pow(A, 1.0 / 3.0);
  gamma = std::atan2(std::sqrt(2) * a22, a20);
  beta = 4 * M_PI * a20 / (3 * A * R * R);
}

// the "Density Functional contributions" table of Output::shellsToFile
// (output.cpp:205-236), in the order of ncgm_hf_outputs.terms
static void energyTable(const Grid &g, const ncgm_hf_config &cfg,
                        const State &st, double *t) {
  const std::size_t ns = g.ns();
  const ncgm_edf &P = cfg.edf;
  Vec f[14];
  for (auto &v : f) v.assign(ns, 0.0);
  for (std::size_t i = 0; i < ns; ++i) {
    const double r0 = st.rhoN[i] + st.rhoP[i], r1 = st.rhoN[i] - st.rhoP[i];
    const double t0 = st.tauN[i] + st.tauP[i], t1 = st.tauN[i] - st.tauP[i];
    const double l0 = st.n2N[i] + st.n2P[i], l1 = st.n2N[i] - st.n2P[i];
    const double rs = std::pow(r0, P.sigma);
    double j0 = 0, j1 = 0;
    for (int a = 0; a < 3; ++a) {
      const double s0 = st.JvN[a * ns + i] + st.JvP[a * ns + i];
      const double s1 = st.JvN[a * ns + i] - st.JvP[a * ns + i];
      j0 += s0 * s0;
      j1 += s1 * s1;
    }
    f[0][i] = 0.5 * kHbar * kHbar * st.tauN[i] / st.massCorr +
              0.5 * kHbar * kHbar * st.tauP[i] / st.massCorr;
    f[1][i] = (P.C0rr * 1.0 + P.C0Drr * rs) * (r0 * r0);
    f[2][i] = (P.C1rr * 1.0 + P.C1Drr * rs) * (r1 * r1);
    f[3][i] = P.C0rdr * (r0 * l0);
    f[4][i] = P.C1rdr * (l1 * r1);
    f[5][i] = P.C0rt * (t0 * r0);
    f[6][i] = P.C1rt * (t1 * r1);
    f[7][i] = P.C0nJ * ((st.divJN[i] + st.divJP[i]) * r0);
    f[8][i] = P.C1nJ * ((st.divJN[i] - st.divJP[i]) * r1);
    f[9][i] = P.C0J2 * j0;
    f[10][i] = P.C1J2 * j1;
    f[11][i] = cfg.use_coulomb ? st.rhoP[i] * st.UCDir[i] : 0.0;
    f[12][i] = std::pow(st.rhoP[i], 4.0 / 3.0) * (-3.0 * kE2 / 4.0) *
               std::pow(3.0 / M_PI, 1.0 / 3.0);
    f[13][i] = -0.5 * P.sigma *
               (P.C0Drr * std::pow(r0, P.sigma + 2) +
                P.C1Drr * std::pow(r0, P.sigma) * (r1 * r1));
  }
  for (int q = 0; q < 11; ++q) t[q] = integral(g, f[q].data());
  t[11] = cfg.use_coulomb ? 0.5 * integral(g, f[11].data()) : 0.0;
  t[12] = epair(cfg, st, true);
  t[13] = epair(cfg, st, false);
  t[14] = cfg.use_coulomb ? integral(g, f[12].data()) : 0.0;
  t[15] = integral(g, f[13].data());
}

int hfRun(const ncgm_hf_config &cfg, ncgm_hf_result &res, double *spe_n,
          double *spe_p, double *rho_n, double *rho_p, double *energies,
          int verbose, ncgm_hf_outputs *out) {
  double tStart = now();
  Grid g(cfg.n, cfg.box_size / 2.0);
  const int A = cfg.A, Z = cfg.Z, N = A - Z;
  const bool pairing = cfg.pairing_type != NCGM_PAIRING_NONE;
  int orbN = pairing && cfg.pair_n.active ? cfg.pair_n.basis_size : N;
  int orbP = pairing && cfg.pair_p.active ? cfg.pair_p.basis_size : Z;
  PhaseTimes pt;
  WSParams W{A,          Z,           cfg.ws_V0,       cfg.ws_r0,
             cfg.ws_diff, cfg.ws_kappa, cfg.initial_beta, cfg.beta3,
             cfg.wsso_V0, cfg.spin_orbit != 0};
  Csr Hws = buildWS(g, W);
  double nucR = std::pow(A, 0.3333333) * 1.20;
  int mx = std::max(orbN, orbP);
  CMat guess = hoGuess(g, mx, nucR, cfg.initial_beta);
  double tg = now();
  GcgOut first = gcgLock(Hws, guess, CMat(g.N(), 0), (int)guess.cols, 0.0,
                         cfg.ws_gcg.max_iter, cfg.ws_gcg.tol,
                         cfg.ws_gcg.cg_steps, cfg.ws_gcg.cg_tol,
                         NCGM_ORDER_ASCENDING);
  pt.gcg += now() - tg;
  Pair n, p;
  n.X = first.X.leftCols(N >= Z ? first.X.cols : orbN);
  n.e.assign(first.lambda.begin(), first.lambda.begin() + n.X.cols);
  p.X = first.X.leftCols(N >= Z ? orbP : first.X.cols);
  p.e.assign(first.lambda.begin(), first.lambda.begin() + p.X.cols);
  normalize(g, n.X);
  normalize(g, p.X);

  State st;
  st.massCorr = cfg.com_corr ? kMass * ((double)A) / ((double)(A - 1)) : kMass;
  st.pN = cfg.pair_n;
  st.pP = cfg.pair_p;
  if (!pairing) {
    st.pN.active = 0;
    st.pP.active = 0;
  }
  std::vector<Constraint> cons;
  if (cfg.constrain_com)
    for (int k = 0; k < 3; ++k) cons.push_back(makeConstraint(g, k, 0.0));
  if (cfg.curve_mode) {
    for (int k = 0; k < 3; ++k) cons.push_back(makeConstraint(g, k, 0.0));
    cons.push_back(makeConstraint(g, 3, 0.0));
    cons.push_back(makeConstraint(g, 4, 0.0));
    cons.push_back(makeConstraint(g, 5, 0.0));
    cons.push_back(makeConstraint(g, 6, cfg.mu20));
  }
  CMat CDN(g.N(), 0), CDP(g.N(), 0);
  double Eint = 0.0, EHF = 0.0;
  int it = 0;
  bool conv = false;
  double lastdE = 0;
  for (it = 0; it < cfg.max_iterations; ++it) {
    if (it == 1) {
      // main.cpp:201-207: the input's multipole constraints join at HF
      // iteration 1; C = 0.01 / (Q - target)^2 on the current densities
      // (MultipoleConstraint constructor, multipole_constraint.cpp:7-16)
      Vec rho(g.ns());
      for (std::size_t i = 0; i < g.ns(); ++i) rho[i] = st.rhoN[i] + st.rhoP[i];
      for (int q = 0; q < cfg.n_multipole && q < NCGM_MAX_MULTIPOLE; ++q) {
        Constraint c;
        c.kind = 1000 + 100 * cfg.mp_l[q] + (cfg.mp_m[q] + 50);
        c.target = cfg.mp_target[q];
        c.gamma = 0.3;
        c.firstIter = false;
        c.O = multipoleOperator(g, cfg.mp_l[q], cfg.mp_m[q]);
        c.C = 1.0;
        const double Q = qValue(g, c, rho);
        c.C = 0.01 / (c.C * std::pow(Q - c.target, 2));
        cons.push_back(c);
      }
    }
    updateQuantities(g, cfg, st, n, p, it, cons, pt);
    double t0 = now();
    Csr hN = buildSkyrme(g, st.fN.data(), st.gfN.data(), st.UN.data(),
                         cfg.spin_orbit ? st.BN.data() : nullptr, nullptr);
    GcgOut nn = gcgLock(hN, n.X, CDN, orbN, 0.0, cfg.hf_gcg.max_iter,
                        cfg.hf_gcg.tol, cfg.hf_gcg.cg_steps, cfg.hf_gcg.cg_tol,
                        NCGM_ORDER_ASCENDING);
    GcgOut np;
    if (cfg.use_coulomb || N != Z) {
      Csr hP = buildSkyrme(g, st.fP.data(), st.gfP.data(), st.UP.data(),
                           cfg.spin_orbit ? st.BP.data() : nullptr,
                           cfg.use_coulomb ? st.UCoul.data() : nullptr);
      np = gcgLock(hP, p.X, CDP, orbP, 0.0, cfg.hf_gcg.max_iter, cfg.hf_gcg.tol,
                   cfg.hf_gcg.cg_steps, cfg.hf_gcg.cg_tol, NCGM_ORDER_ASCENDING);
    } else {
      np.X = nn.X.leftCols(orbP);
      np.lambda.assign(nn.lambda.begin(), nn.lambda.begin() + orbP);
    }
    pt.gcg += now() - t0;
    double maxdSPE = 0;
    for (int i = 0; i < orbN; ++i)
      maxdSPE = std::max(maxdSPE, std::abs(nn.lambda[i] - n.e[i]));
    for (int i = 0; i < orbP; ++i)
      maxdSPE = std::max(maxdSPE, std::abs(np.lambda[i] - p.e[i]));
    normalize(g, nn.X);
    normalize(g, np.X);
    if (pairing) {
      nn.X = TROrder(g, nn.X);
      np.X = TROrder(g, np.X);
    }
    if (it > 0) {
      auto cd_ = [&](const CMat &old, const CMat &nw) {
        CMat tmp = adjointTimes(old, nw);
        CMat prod = times(old, tmp);
        CMat out(nw.rows, nw.cols);
        for (std::size_t i = 0; i < nw.d.size(); ++i) out.d[i] = nw.d[i] - prod.d[i];
        for (std::size_t c = 0; c < out.cols; ++c) {
          double s = colNorm2(out.col(c), out.rows);
          if (s > 0) {
            s = std::sqrt(s);
            for (std::size_t r = 0; r < out.rows; ++r) out(r, c) /= s;
          }
        }
        return out;
      };
      CDN = cd_(n.X, nn.X);
      CDP = cd_(p.X, np.X);
    }
    n.X = nn.X;
    n.e = nn.lambda;
    p.X = np.X;
    p.e = np.lambda;
    double nE = totalEnergyIntegral(g, cfg, st) + kineticEnergy(g, st);
    double nH = HFEnergy(g, cfg, st, cons);
    bool cconv = true;
    for (auto &c : cons)
      if (c.error() != 0.0) cconv = cconv && (c.error() < cfg.constraints_tol);
    if (energies) {
      energies[2 * it] = nE;
      energies[2 * it + 1] = nH;
    }
    lastdE = std::abs(nE - Eint);
    if (verbose)
      std::printf("[oracle] it %d Eint %.9f EHF %.9f dE %.3e dSPE %.3e\n", it,
                  nE, nH, lastdE, maxdSPE);
    bool speOk = cfg.spe_tol <= 0 || maxdSPE < cfg.spe_tol;
    if (std::abs(nE - Eint) < cfg.energy_tol &&
        std::abs(nH - EHF) < cfg.energy_tol && cconv && speOk) {
      Eint = nE;
      EHF = nH;
      conv = true;
      ++it;
      break;
    }
    st.energyDiff = std::abs(nH - EHF);
    Eint = nE;
    EHF = nH;
  }
  if (out) {
    energyTable(g, cfg, st, out->terms);
    {
      Vec rho(g.ns());
      for (std::size_t i = 0; i < g.ns(); ++i) rho[i] = st.rhoN[i] + st.rhoP[i];
      double ce = 0;
      for (auto &c : cons) ce += constraintEvaluate(g, c, rho);
      out->constraints_energy = ce;
    }
    if (out->orbitals_n)
      std::memcpy(out->orbitals_n, n.X.d.data(), sizeof(cd) * n.X.d.size());
    if (out->orbitals_p)
      std::memcpy(out->orbitals_p, p.X.d.data(), sizeof(cd) * p.X.d.size());
    if (out->U_n) std::copy(st.UN.begin(), st.UN.end(), out->U_n);
    if (out->U_p) std::copy(st.UP.begin(), st.UP.end(), out->U_p);
  }
  // Output::shellsToFile: tau, J and the Laplacian of rho recomputed with
  // the Lagrange-mesh derivatives from the final orbitals, then E_INT again
  // ("EintLag", src/system/output.cpp:252-256; iteration_data.cpp:346-382).
  // rho and div J keep their values from the loop.
  {
    State L = st;
    const CMat on = occupied(g, n.X, cfg, st, true, false);
    const CMat op = occupied(g, p.X, cfg, st, false, false);
    L.tauN = kineticDensityLagrange(g, on);
    L.tauP = kineticDensityLagrange(g, op);
    L.JN = soDensityLagrange(g, on);
    L.JP = soDensityLagrange(g, op);
    L.JvN = leviCivita(L.JN, g.ns());
    L.JvP = leviCivita(L.JP, g.ns());
    L.n2N = lapLagrangeNoSpin(g, st.rhoN);
    L.n2P = lapLagrangeNoSpin(g, st.rhoP);
    res.E_int_lagrange = kineticEnergy(g, L) + totalEnergyIntegral(g, cfg, L);
    if (out) {
      if (out->tau_n) std::copy(L.tauN.begin(), L.tauN.end(), out->tau_n);
      if (out->tau_p) std::copy(L.tauP.begin(), L.tauP.end(), out->tau_p);
      if (out->grad_rho_n) {
        const Vec gN = gradLagrangeNoSpin(g, st.rhoN);
        std::copy(gN.begin(), gN.end(), out->grad_rho_n);
      }
      if (out->grad_rho_p) {
        const Vec gP = gradLagrangeNoSpin(g, st.rhoP);
        std::copy(gP.begin(), gP.end(), out->grad_rho_p);
      }
    }
  }
  res.iterations = it;
  res.converged = conv;
  res.E_int = Eint;
  res.E_HF = EHF;
  res.E_pair_n = epair(cfg, st, true);
  res.E_pair_p = epair(cfg, st, false);
  res.lambda_n = cfg.pairing_type == NCGM_PAIRING_HFB ? st.hfbN.lambda
                                                       : st.bcsN.lambda;
  res.lambda_p = cfg.pairing_type == NCGM_PAIRING_HFB ? st.hfbP.lambda
                                                       : st.bcsP.lambda;
  quadDef(g, st, A, res.beta, res.gamma);
  res.last_dE = lastdE;
  res.t_gcg_s = pt.gcg;
  res.t_fields_s = pt.fields;
  res.t_poisson_s = pt.poisson;
  res.t_pairing_s = pt.pairing;
  if (spe_n) std::copy(n.e.begin(), n.e.end(), spe_n);
  if (spe_p) std::copy(p.e.begin(), p.e.end(), spe_p);
  if (rho_n) std::copy(st.rhoN.begin(), st.rhoN.end(), rho_n);
  if (rho_p) std::copy(st.rhoP.begin(), st.rhoP.end(), rho_p);
  res.wall_s = now() - tStart;
  return NCGM_OK;
}


// IterationData held by a caller that drives its own loop (the device state
// handle's counterpart; test infrastructure): `calls` updates of the state
// from the same eigenpairs (HF iterations 0 .. calls-1, so the first sets
// the densities and later ones mix; iteration_data.cpp:852-1125), then the
// energies with the new levels en2, ep2 as main() evaluates them
// (main.cpp:300-305). out, per species (neutrons then protons): f, grad f
// (3), U, W (3), UC, rho, tau, 11 n^3 values. E: E_int, E_HF.
int stateRun(const ncgm_hf_config &cfg, const double *Xn, const double *en,
             int cn, const double *Xp, const double *ep, int cp, int calls,
             int flags, const double *en2, const double *ep2, double *out,
             double *E) {
  Grid g(cfg.n, cfg.box_size / 2.0);
  const std::size_t ns = g.ns();
  const bool pairing = cfg.pairing_type != NCGM_PAIRING_NONE;
  State st;
  st.massCorr = cfg.com_corr ? kMass * ((double)cfg.A) / ((double)(cfg.A - 1))
                             : kMass;
  st.pN = cfg.pair_n;
  st.pP = cfg.pair_p;
  if (!pairing) {
    st.pN.active = 0;
    st.pP.active = 0;
  }
  std::vector<Constraint> cons;
  if (cfg.constrain_com)
    for (int k = 0; k < 3; ++k) cons.push_back(makeConstraint(g, k, 0.0));
  if (cfg.curve_mode) {
    for (int k = 0; k < 3; ++k) cons.push_back(makeConstraint(g, k, 0.0));
    cons.push_back(makeConstraint(g, 3, 0.0));
    cons.push_back(makeConstraint(g, 4, 0.0));
    cons.push_back(makeConstraint(g, 5, 0.0));
    cons.push_back(makeConstraint(g, 6, cfg.mu20));
  }
  Pair n, p;
  n.X = CMat(g.N(), cn);
  p.X = CMat(g.N(), cp);
  std::memcpy(n.X.d.data(), Xn, sizeof(cd) * n.X.d.size());
  std::memcpy(p.X.d.data(), Xp, sizeof(cd) * p.X.d.size());
  n.e.assign(en, en + cn);
  p.e.assign(ep, ep + cp);
  PhaseTimes pt;
  for (int it = 0; it < calls; ++it) {
    if (flags & 1) {
      normalize(g, n.X);
      normalize(g, p.X);
    }
    if ((flags & 2) && pairing) {
      n.X = TROrder(g, n.X);
      p.X = TROrder(g, p.X);
    }
    updateQuantities(g, cfg, st, n, p, it, cons, pt);
  }
  n.e.assign(en2, en2 + cn);
  p.e.assign(ep2, ep2 + cp);
  E[0] = totalEnergyIntegral(g, cfg, st) + kineticEnergy(g, st);
  E[1] = HFEnergy(g, cfg, st, cons);
  const Vec zero(ns, 0.0);
  const Vec *parts[2][7] = {
      {&st.fN, &st.gfN, &st.UN, &st.BN, &zero, &st.rhoN, &st.tauN},
      {&st.fP, &st.gfP, &st.UP, &st.BP,
       (cfg.use_coulomb && st.haveCoul) ? &st.UCoul : &zero, &st.rhoP,
       &st.tauP}};
  double *o = out;
  for (int q = 0; q < 2; ++q)
    for (int k = 0; k < 7; ++k) {
      const std::size_t len = (k == 1 || k == 3) ? 3 * ns : ns;
      const Vec &v = *parts[q][k];
      if (v.size() >= len)
        std::copy(v.begin(), v.begin() + len, o);
      else
        std::fill(o, o + len, 0.0);
      o += len;
    }
  return NCGM_OK;
}

} // namespace orc
