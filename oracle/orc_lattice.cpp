// Test infrastructure (oracle): lattice operators, Hamiltonian assembly and
// the block GCG eigensolver of the nuclearcgm hot path, restated in plain
// FP64 C++ (no Eigen). Used only as the checker by tests/, the smoke check and
// the CPU-baseline leg of bench.py; never linked into the product library.
#include "orc_internal.hpp"

#include <cstdio>
#include <cstring>
#include <omp.h>

namespace orc {

// ---------------------------------------------------------------------------
// Finite differences: Operators::derivative / derivativeNoSpin
// (src/operators/differential_operators.cpp:356-543) and derivative2 /
// derivative2NoSpin (545-678). The stencil order drops towards the box edge;
// at pos 0 and n-1 the second derivative uses a first-derivative formula.
// ---------------------------------------------------------------------------
template <class T, class Get>
static inline T d1(const Get &g, int pos, int n, double h) {
  if (pos == 0) {
    T f0 = g(pos), f1 = g(pos + 1);
    return (f1 - f0) / h;
  } else if (pos == 1 || pos == n - 2) {
    T f_1 = g(pos - 1), f1 = g(pos + 1);
    return (f1 - f_1) / (2.0 * h);
  } else if (pos == n - 1) {
    T f0 = g(pos), f_1 = g(pos - 1);
    return (f0 - f_1) / h;
  } else if (pos == 2 || pos == n - 3) {
    T f_2 = g(pos - 2), f_1 = g(pos - 1), f1 = g(pos + 1), f2 = g(pos + 2);
    return (-f2 + 8.0 * f1 - 8.0 * f_1 + f_2) / (12.0 * h);
  } else if (pos == 3 || pos == n - 4) {
    T f_3 = g(pos - 3), f_2 = g(pos - 2), f_1 = g(pos - 1);
    T f1 = g(pos + 1), f2 = g(pos + 2), f3 = g(pos + 3);
    return (-f_3 + 9.0 * f_2 - 45.0 * f_1 + 45.0 * f1 - 9.0 * f2 + f3) /
           (60.0 * h);
  } else {
    T f_4 = g(pos - 4), f_3 = g(pos - 3), f_2 = g(pos - 2), f_1 = g(pos - 1);
    T f1 = g(pos + 1), f2 = g(pos + 2), f3 = g(pos + 3), f4 = g(pos + 4);
    return (3.0 * f_4 - 32.0 * f_3 + 168.0 * f_2 - 672.0 * f_1 + 672.0 * f1 -
            168.0 * f2 + 32.0 * f3 - 3.0 * f4) /
           (840.0 * h);
  }
}

template <class T, class Get>
static inline T d2(const Get &g, int pos, int n, double h) {
  if (pos == 0) {
    T f0 = g(pos), f1 = g(pos + 1);
    return (f1 - f0) / (h);
  } else if (pos == 1 || pos == n - 2) {
    T f_1 = g(pos - 1), f0 = g(pos), f1 = g(pos + 1);
    return (f_1 - 2.0 * f0 + f1) / (h * h);
  } else if (pos == n - 1) {
    T f0 = g(pos), f_1 = g(pos - 1);
    return (f0 - f_1) / (h);
  } else if (pos == 2 || pos == n - 3) {
    T f_2 = g(pos - 2), f_1 = g(pos - 1), f0 = g(pos), f1 = g(pos + 1),
      f2 = g(pos + 2);
    return (-f2 + 16.0 * f1 - 30.0 * f0 + 16.0 * f_1 - f_2) / (12.0 * h * h);
  } else if (pos == 3 || pos == n - 4) {
    T f_3 = g(pos - 3), f_2 = g(pos - 2), f_1 = g(pos - 1), f0 = g(pos);
    T f1 = g(pos + 1), f2 = g(pos + 2), f3 = g(pos + 3);
    return (2.0 * f3 - 27.0 * f2 + 270.0 * f1 + -490.0 * f0 + 270.0 * f_1 -
            27.0 * f_2 + 2.0 * f_3) /
           (180.0 * h * h);
  } else {
    T f_4 = g(pos - 4), f_3 = g(pos - 3), f_2 = g(pos - 2), f_1 = g(pos - 1),
      f0 = g(pos);
    T f1 = g(pos + 1), f2 = g(pos + 2), f3 = g(pos + 3), f4 = g(pos + 4);
    return (-9.0 * f_4 + 128.0 * f_3 - 1008.0 * f_2 + 8064.0 * f_1 -
            14350.0 * f0 + 8064.0 * f1 - 1008.0 * f2 + 128.0 * f3 - 9.0 * f4) /
           (5040.0 * h * h);
  }
}

// Gradient of one spinor column (Operators::grad, differential_operators.cpp:
// 280-292): out[axis][row], rows = 2 n^3. NaNs are scrubbed to 0 like dv().
void gradSpinor(const Grid &g, const cd *psi, std::vector<cd> out[3]) {
  const int n = g.n;
  const double h = g.h;
  for (int ax = 0; ax < 3; ++ax) out[ax].assign(g.N(), cd(0, 0));
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        for (int s = 0; s < 2; ++s) {
          std::size_t r = g.idx(i, j, k, s);
          cd vx = d1<cd>([&](int p) { return psi[g.idx(p, j, k, s)]; }, i, n, h);
          cd vy = d1<cd>([&](int p) { return psi[g.idx(i, p, k, s)]; }, j, n, h);
          cd vz = d1<cd>([&](int p) { return psi[g.idx(i, j, p, s)]; }, k, n, h);
          auto scrub = [](cd v) {
            return (std::isnan(v.real()) || std::isnan(v.imag())) ? cd(0, 0) : v;
          };
          out[0][r] = scrub(vx);
          out[1][r] = scrub(vy);
          out[2][r] = scrub(vz);
        }
}

// Operators::gradNoSpin (differential_operators.cpp:295-306), n^3 x 3.
std::vector<double> gradNoSpin(const Grid &g, const std::vector<double> &v) {
  const int n = g.n;
  const double h = g.h;
  const std::size_t ns = g.ns();
  std::vector<double> out(3 * ns);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        std::size_t r = g.idxNS(i, j, k);
        double vals[3] = {
            d1<double>([&](int p) { return v[g.idxNS(p, j, k)]; }, i, n, h),
            d1<double>([&](int p) { return v[g.idxNS(i, p, k)]; }, j, n, h),
            d1<double>([&](int p) { return v[g.idxNS(i, j, p)]; }, k, n, h)};
        for (int ax = 0; ax < 3; ++ax)
          out[ax * ns + r] = std::isnan(vals[ax]) ? 0.0 : vals[ax];
      }
  return out;
}

// Operators::lapNoSpin (differential_operators.cpp:308-316): sum of the three
// derivative2NoSpin passes (no NaN scrub in dv2NoSpin).
std::vector<double> lapNoSpin(const Grid &g, const std::vector<double> &v) {
  const int n = g.n;
  const double h = g.h;
  std::vector<double> out(g.ns(), 0.0);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        std::size_t r = g.idxNS(i, j, k);
        double acc = 0.0;
        acc += d2<double>([&](int p) { return v[g.idxNS(p, j, k)]; }, i, n, h);
        acc += d2<double>([&](int p) { return v[g.idxNS(i, p, k)]; }, j, n, h);
        acc += d2<double>([&](int p) { return v[g.idxNS(i, j, p)]; }, k, n, h);
        out[r] = acc;
      }
  return out;
}

// Operators::integral (src/operators/integral_operators.cpp:62-87):
// trapezoid weights, half weight on each boundary face index.
double integral(const Grid &g, const double *v) {
  const int n = g.n;
  const double hhh = g.h * g.h * g.h;
  double res = 0.0;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double w = 1.0;
        if (i == 0 || i == n - 1) w *= 0.5;
        if (j == 0 || j == n - 1) w *= 0.5;
        if (k == 0 || k == n - 1) w *= 0.5;
        res += v[g.idxNS(i, j, k)] * hhh * w;
      }
  return res;
}

// ---------------------------------------------------------------------------
// Densities (src/util/wavefunction.cpp)
// ---------------------------------------------------------------------------

// Wavefunction::density (wavefunction.cpp:21-44)
std::vector<double> density(const Grid &g, const CMat &psi) {
  std::vector<double> rho(g.ns(), 0.0);
#pragma omp parallel for schedule(static)
  for (long long p = 0; p < (long long)g.ns(); ++p) {
    double acc = 0.0;
    for (std::size_t c = 0; c < psi.cols; ++c) {
      acc += std::norm(psi(2 * p, c));
      acc += std::norm(psi(2 * p + 1, c));
    }
    rho[p] = acc;
  }
  return rho;
}

// Wavefunction::kineticDensity (wavefunction.cpp:348-360)
std::vector<double> kineticDensity(const Grid &g, const CMat &psi) {
  std::vector<double> tau(g.ns(), 0.0);
  std::vector<cd> gr[3];
  for (std::size_t c = 0; c < psi.cols; ++c) {
    gradSpinor(g, psi.col(c), gr);
#pragma omp parallel for schedule(static)
    for (long long l = 0; l < (long long)g.ns(); ++l) {
      double m0 = 0.0, m1 = 0.0;
      for (int ax = 0; ax < 3; ++ax) {
        m0 += std::norm(gr[ax][2 * l]);
        m1 += std::norm(gr[ax][2 * l + 1]);
      }
      tau[l] += m0 + m1;
    }
  }
  return tau;
}

// sigma_nu * (a, b) for the Pauli matrices of nuclearConstants::getPauli
// (src/common/constants.cpp:4-23): x, y, z.
static inline void pauliApply(int nu, cd a, cd b, cd &o0, cd &o1) {
  const cd I(0, 1);
  if (nu == 0) {
    o0 = b;
    o1 = a;
  } else if (nu == 1) {
    o0 = -I * b;
    o1 = I * a;
  } else {
    o0 = a;
    o1 = -b;
  }
}

// Wavefunction::soDensity (wavefunction.cpp:421-464): J_{mu nu} =
// sum Im(psi^* sigma_nu d_mu psi), stored n^3 x 9 column-major, col mu*3+nu.
std::vector<double> soDensity(const Grid &g, const CMat &psi) {
  const std::size_t ns = g.ns();
  std::vector<double> J(9 * ns, 0.0);
  std::vector<cd> gr[3];
  for (std::size_t c = 0; c < psi.cols; ++c) {
    gradSpinor(g, psi.col(c), gr);
    const cd *ps = psi.col(c);
#pragma omp parallel for schedule(static)
    for (long long l = 0; l < (long long)ns; ++l) {
      cd p0 = ps[2 * l], p1 = ps[2 * l + 1];
      for (int mu = 0; mu < 3; ++mu)
        for (int nu = 0; nu < 3; ++nu) {
          cd q0, q1;
          pauliApply(nu, gr[mu][2 * l], gr[mu][2 * l + 1], q0, q1);
          J[(mu * 3 + nu) * ns + l] += p0.real() * q0.imag() -
                                       p0.imag() * q0.real() +
                                       p1.real() * q1.imag() -
                                       p1.imag() * q1.real();
        }
    }
  }
  return J;
}

// Wavefunction::divJ (wavefunction.cpp:466-517)
std::vector<double> divJ(const Grid &g, const CMat &psi) {
  const std::size_t ns = g.ns();
  std::vector<double> W(ns, 0.0);
  std::vector<cd> gr[3];
  for (std::size_t c = 0; c < psi.cols; ++c) {
    gradSpinor(g, psi.col(c), gr);
#pragma omp parallel for schedule(static)
    for (long long l = 0; l < (long long)ns; ++l) {
      cd sum(0, 0);
      for (int mu = 0; mu < 3; ++mu)
        for (int nu = 0; nu < 3; ++nu)
          for (int la = 0; la < 3; ++la) {
            double eps = 0;
            if ((mu == 0 && nu == 1 && la == 2) ||
                (mu == 1 && nu == 2 && la == 0) ||
                (mu == 2 && nu == 0 && la == 1))
              eps = +1.0;
            else if ((mu == 2 && nu == 1 && la == 0) ||
                     (mu == 0 && nu == 2 && la == 1) ||
                     (mu == 1 && nu == 0 && la == 2))
              eps = -1.0;
            if (eps == 0.0) continue;
            cd q0, q1;
            pauliApply(la, gr[mu][2 * l], gr[mu][2 * l + 1], q0, q1);
            cd term = std::conj(gr[nu][2 * l]) * q0 +
                      std::conj(gr[nu][2 * l + 1]) * q1;
            sum += eps * term;
          }
      W[l] += sum.imag();
    }
  }
  for (auto &x : W) x = -x;
  return W;
}

// ---------------------------------------------------------------------------
// Lagrange-mesh derivatives of the output step (IterationData::
// recomputeLagrange, src/util/iteration_data.cpp:346-382)
// ---------------------------------------------------------------------------

// lagrangeFirstDerivative (differential_operators.cpp:108-129), row-major:
// D(s, t) = (-1)^(t-s) pi / (n h) / sin(pi (t - s) / n), zero diagonal
std::vector<double> lagrangeD1(int n, double h) {
  std::vector<double> D((std::size_t)n * n, 0.0);
  for (int s = 0; s < n; ++s)
    for (int t = 0; t < n; ++t) {
      if (s == t) continue;
      const double diff = static_cast<double>(t - s);
      D[(std::size_t)s * n + t] = std::pow(-1.0, diff) * (M_PI / (n * h)) *
                                  (1.0 / std::sin(M_PI * diff / n));
    }
  return D;
}

// Operators::gradLagrange (differential_operators.cpp:237-278): D's second
// index contracted with each axis, negated: g_a = -D psi, both spins
void gradLagrangeSpinor(const Grid &g, const cd *psi, std::vector<cd> out[3]) {
  const int n = g.n;
  const std::vector<double> D = lagrangeD1(n, g.h);
  for (int ax = 0; ax < 3; ++ax) out[ax].assign(g.N(), cd(0, 0));
#pragma omp parallel for schedule(static)
  for (long long p = 0; p < (long long)g.ns(); ++p) {
    const int i = (int)(p % n), j = (int)((p / n) % n), k = (int)(p / ((long long)n * n));
    for (int s2 = 0; s2 < 2; ++s2) {
      cd ax(0, 0), ay(0, 0), az(0, 0);
      for (int t = 0; t < n; ++t) {
        ax += D[(std::size_t)i * n + t] * psi[g.idx(t, j, k, s2)];
        ay += D[(std::size_t)j * n + t] * psi[g.idx(i, t, k, s2)];
        az += D[(std::size_t)k * n + t] * psi[g.idx(i, j, t, s2)];
      }
      out[0][2 * p + s2] = -ax;
      out[1][2 * p + s2] = -ay;
      out[2][2 * p + s2] = -az;
    }
  }
}

// kineticDensityLagrange (wavefunction.cpp:334-346)
std::vector<double> kineticDensityLagrange(const Grid &g, const CMat &psi) {
  std::vector<double> tau(g.ns(), 0.0);
  std::vector<cd> gr[3];
  for (std::size_t c = 0; c < psi.cols; ++c) {
    gradLagrangeSpinor(g, psi.col(c), gr);
    for (std::size_t l = 0; l < g.ns(); ++l) {
      double m0 = 0.0, m1 = 0.0;
      for (int ax = 0; ax < 3; ++ax) {
        m0 += std::norm(gr[ax][2 * l]);
        m1 += std::norm(gr[ax][2 * l + 1]);
      }
      tau[l] += m0 + m1;
    }
  }
  return tau;
}

// soDensityLagrange (wavefunction.cpp:372-414): as soDensity with the
// Lagrange gradient, n^3 x 9 column-major, col mu*3+nu
std::vector<double> soDensityLagrange(const Grid &g, const CMat &psi) {
  const std::size_t ns = g.ns();
  std::vector<double> J(9 * ns, 0.0);
  std::vector<cd> gr[3];
  for (std::size_t c = 0; c < psi.cols; ++c) {
    gradLagrangeSpinor(g, psi.col(c), gr);
    const cd *ps = psi.col(c);
    for (std::size_t l = 0; l < ns; ++l) {
      const cd p0 = ps[2 * l], p1 = ps[2 * l + 1];
      for (int mu = 0; mu < 3; ++mu)
        for (int nu = 0; nu < 3; ++nu) {
          cd q0, q1;
          pauliApply(nu, gr[mu][2 * l], gr[mu][2 * l + 1], q0, q1);
          J[(mu * 3 + nu) * ns + l] += p0.real() * q0.imag() -
                                       p0.imag() * q0.real() +
                                       p1.real() * q1.imag() -
                                       p1.imag() * q1.real();
        }
    }
  }
  return J;
}

// Operators::lapLagrangeNoSpin (differential_operators.cpp:196-235): the
// first index of D D contracted with each axis, x + y + z
std::vector<double> lapLagrangeNoSpin(const Grid &g,
                                      const std::vector<double> &v) {
  const int n = g.n;
  const std::vector<double> D = lagrangeD1(n, g.h);
  std::vector<double> D2((std::size_t)n * n, 0.0); // D2(a, b) row-major
  for (int a = 0; a < n; ++a)
    for (int b = 0; b < n; ++b) {
      double acc = 0.0;
      for (int u = 0; u < n; ++u)
        acc += D[(std::size_t)a * n + u] * D[(std::size_t)u * n + b];
      D2[(std::size_t)a * n + b] = acc;
    }
  std::vector<double> out(g.ns(), 0.0);
#pragma omp parallel for schedule(static)
  for (long long p = 0; p < (long long)g.ns(); ++p) {
    const int i = (int)(p % n), j = (int)((p / n) % n), k = (int)(p / ((long long)n * n));
    double ax = 0, ay = 0, az = 0;
    for (int s = 0; s < n; ++s) {
      ax += D2[(std::size_t)s * n + i] * v[g.idxNS(s, j, k)];
      ay += D2[(std::size_t)s * n + j] * v[g.idxNS(i, s, k)];
      az += D2[(std::size_t)s * n + k] * v[g.idxNS(i, j, s)];
    }
    out[p] = ax + ay + az;
  }
  return out;
}

// Operators::gradLagrangeNoSpin (differential_operators.cpp:156-194): D's
// first index contracted with each axis, no sign change; n^3 x 3
// column-major
std::vector<double> gradLagrangeNoSpin(const Grid &g,
                                       const std::vector<double> &v) {
  const int n = g.n;
  const std::vector<double> D = lagrangeD1(n, g.h);
  const std::size_t ns = g.ns();
  std::vector<double> out(3 * ns, 0.0);
  for (std::size_t p = 0; p < ns; ++p) {
    const int i = (int)(p % n), j = (int)((p / n) % n), k = (int)(p / ((std::size_t)n * n));
    double gx = 0, gy = 0, gz = 0;
    for (int s = 0; s < n; ++s) {
      gx += D[(std::size_t)s * n + i] * v[g.idxNS(s, j, k)];
      gy += D[(std::size_t)s * n + j] * v[g.idxNS(i, s, k)];
      gz += D[(std::size_t)s * n + k] * v[g.idxNS(i, j, s)];
    }
    out[p] = gx;
    out[ns + p] = gy;
    out[2 * ns + p] = gz;
  }
  return out;
}

// ---------------------------------------------------------------------------
// Shell observables (src/util/shell.cpp:22-51, angular_momentum.cpp)
// ---------------------------------------------------------------------------

// L_a psi = -i hbar (r x grad)_a psi for a = x, y, z (:206-267)
static void angularL(const Grid &g, const cd *psi, std::vector<cd> L[3]) {
  std::vector<cd> gr[3];
  gradSpinor(g, psi, gr);
  const cd mih(0.0, -kHbar);
  for (int a = 0; a < 3; ++a) L[a].assign(g.N(), cd(0, 0));
  for (int k = 0; k < g.n; ++k)
    for (int j = 0; j < g.n; ++j)
      for (int i = 0; i < g.n; ++i)
        for (int s = 0; s < 2; ++s) {
          const std::size_t r = g.idx(i, j, k, s);
          const double x = g.xs[i], y = g.xs[j], z = g.xs[k];
          L[0][r] = mih * (y * gr[2][r] - z * gr[1][r]);
          L[1][r] = mih * (z * gr[0][r] - x * gr[2][r]);
          L[2][r] = mih * (x * gr[1][r] - y * gr[0][r]);
        }
}

// Operators::integral of a spinor-length complex vector (trapezoid weights
// on both components, integral_operators.cpp:4-32)
static cd integralSpinor(const Grid &g, const std::vector<cd> &f) {
  const double hhh = g.h * g.h * g.h;
  cd acc(0, 0);
  for (int k = 0; k < g.n; ++k)
    for (int j = 0; j < g.n; ++j)
      for (int i = 0; i < g.n; ++i)
        for (int s = 0; s < 2; ++s) {
          double w = 1.0;
          if (i == 0 || i == g.n - 1) w *= 0.5;
          if (j == 0 || j == g.n - 1) w *= 0.5;
          if (k == 0 || k == g.n - 1) w *= 0.5;
          acc += f[g.idx(i, j, k, s)] * hhh * w;
        }
  return acc;
}

// obs = [Re int psi conj(L^2 psi), Re int psi conj(J^2 psi),
//        Re int psi conj(Jz Jz psi), Re psi(-r)^* . psi, Re int psi conj(LS psi)]
void shellObservables(const Grid &g, const cd *psi, double obs[5]) {
  const std::size_t N = g.N();
  std::vector<cd> L[3], LL[3];
  angularL(g, psi, L);
  std::vector<cd> L2(N, cd(0, 0));
  for (int a = 0; a < 3; ++a) {
    angularL(g, L[a].data(), LL);
    for (std::size_t r = 0; r < N; ++r) L2[r] += LL[a][r];
  }
  // S_z = hbar/2 sigma_z; J_z = L_z + S_z (:185-205, 269-272)
  std::vector<cd> Jz(N), JJ(N);
  for (std::size_t r = 0; r < N; ++r)
    Jz[r] = L[2][r] + ((r % 2 == 0) ? 0.5 : -0.5) * kHbar * psi[r];
  angularL(g, Jz.data(), LL);
  for (std::size_t r = 0; r < N; ++r)
    JJ[r] = LL[2][r] + ((r % 2 == 0) ? 0.5 : -0.5) * kHbar * Jz[r];
  // L.S psi (:118-183): prefactor -i hbar^2 / 2 on (r x grad) without -i hbar
  std::vector<cd> LS(N);
  {
    const cd I(0, 1), pref = -I * kHbar * kHbar * 0.5, mih(0.0, -kHbar);
    for (std::size_t q = 0; q < g.ns(); ++q) {
      // L[a] = -i hbar L'_a, so L'_a = L[a] / (-i hbar)
      const cd lx0 = L[0][2 * q] / mih, ly0 = L[1][2 * q] / mih,
               lz0 = L[2][2 * q] / mih;
      const cd lx1 = L[0][2 * q + 1] / mih, ly1 = L[1][2 * q + 1] / mih,
               lz1 = L[2][2 * q + 1] / mih;
      LS[2 * q] = pref * (lz0 + (lx1 - I * ly1));
      LS[2 * q + 1] = pref * ((lx0 + I * ly0) - lz1);
    }
  }
  std::vector<cd> f(N);
  auto expect = [&](const std::vector<cd> &Op) {
    for (std::size_t r = 0; r < N; ++r) f[r] = psi[r] * std::conj(Op[r]);
    return integralSpinor(g, f).real();
  };
  double nrm = 0;
  {
    for (std::size_t r = 0; r < N; ++r) f[r] = psi[r] * std::conj(psi[r]);
    nrm = integralSpinor(g, f).real();
  }
  const double l2 = expect(L2), jj = expect(JJ);
  double ls = 0;
  for (std::size_t r = 0; r < N; ++r) f[r] = LS[r] * std::conj(psi[r]);
  ls = integralSpinor(g, f).real();
  // P psi(r) = psi(-r) (common_operators.cpp:4-22); par.dot(psi)
  cd par(0, 0);
  for (int k = 0; k < g.n; ++k)
    for (int j = 0; j < g.n; ++j)
      for (int i = 0; i < g.n; ++i)
        for (int s = 0; s < 2; ++s)
          par += std::conj(psi[g.idx(g.n - 1 - i, g.n - 1 - j, g.n - 1 - k, s)]) *
                 psi[g.idx(i, j, k, s)];
  obs[0] = l2;
  obs[1] = l2 + 0.75 * kHbar * kHbar * nrm + 2.0 * ls;
  obs[2] = jj;
  obs[3] = par.real();
  obs[4] = ls;
}

// Wavefunction::normalize (wavefunction.cpp:362-370)
void normalize(const Grid &g, CMat &psi) {
  std::vector<double> rho(g.ns());
  for (std::size_t c = 0; c < psi.cols; ++c) {
    cd *p = psi.col(c);
    for (std::size_t l = 0; l < g.ns(); ++l)
      rho[l] = std::norm(p[2 * l]) + std::norm(p[2 * l + 1]);
    double I = integral(g, rho.data());
    double s = std::sqrt(I);
    for (std::size_t r = 0; r < g.N(); ++r) p[r] /= s;
  }
}

// Wavefunction::timeReverse (wavefunction.cpp:554-580): T psi = i sigma_y psi*
CMat timeReverse(const Grid &g, const CMat &psi) {
  CMat res(psi.rows, psi.cols);
  const cd I(0, 1);
  for (std::size_t c = 0; c < psi.cols; ++c)
    for (std::size_t l = 0; l < g.ns(); ++l) {
      cd a = std::conj(psi(2 * l, c)), b = std::conj(psi(2 * l + 1, c));
      cd o0, o1;
      pauliApply(1, a, b, o0, o1);
      res(2 * l, c) = I * o0;
      res(2 * l + 1, c) = I * o1;
    }
  return res;
}

// Wavefunction::TROrder (wavefunction.cpp:581-635)
CMat TROrder(const Grid &g, const CMat &psi) {
  const int nStates = (int)psi.cols;
  CMat ord = adjointTimes(psi, timeReverse(g, psi));
  CMat sorted(psi.rows, psi.cols);
  std::vector<bool> used(nStates, false);
  int currentSlot = 0;
  for (int i = 0; i < nStates; ++i) {
    if (used[i]) continue;
    std::copy(psi.col(i), psi.col(i) + psi.rows, sorted.col(currentSlot));
    used[i] = true;
    int best_j = -1;
    double max_overlap = -1.0;
    for (int j = 0; j < nStates; ++j) {
      if (used[j]) continue;
      double overlap = std::abs(ord(i, j));
      if (overlap > max_overlap) {
        max_overlap = overlap;
        best_j = j;
      }
    }
    if (best_j != -1) {
      std::copy(psi.col(best_j), psi.col(best_j) + psi.rows,
                sorted.col(currentSlot + 1));
      used[best_j] = true;
    } else {
      return psi;
    }
    currentSlot += 2;
    if (currentSlot >= nStates) break;
  }
  return sorted;
}

// ---------------------------------------------------------------------------
// Hamiltonian assembly (src/hamiltonian/hamiltonian.cpp:207-372). Entries are
// generated per row in ascending column order, so the row sums of the SpMV
// follow the same order as Eigen's column-major sparse x dense product.
// ---------------------------------------------------------------------------

static inline void pauliMat(int a, cd m[2][2]) {
  const cd I(0, 1);
  if (a == 0) {
    m[0][0] = 0; m[0][1] = 1; m[1][0] = 1; m[1][1] = 0;
  } else if (a == 1) {
    m[0][0] = 0; m[0][1] = -I; m[1][0] = I; m[1][1] = 0;
  } else {
    m[0][0] = 1; m[0][1] = 0; m[1][0] = 0; m[1][1] = -1;
  }
}

// SkyrmeSO::getElement5p (src/skyrme/skyrme_so.cpp:12-58) and
// DeformedSpinOrbitPotential::getElement5p (src/potentials/
// deformed_spin_orbit.cpp:69-114): both are combinations of Pauli matrices
// weighted by a field vector; `sign` selects the term's own arrangement.
static cd soElement(int ax, int d, int s, int s1, const double Wv[3],
                    double h, bool wsForm, double ls) {
  cd px[2][2], py[2][2], pz[2][2];
  pauliMat(0, px);
  pauliMat(1, py);
  pauliMat(2, pz);
  cd M[2][2];
  for (int r = 0; r < 2; ++r)
    for (int c = 0; c < 2; ++c) {
      if (!wsForm) {
        if (ax == 0) M[r][c] = py[r][c] * Wv[2] - pz[r][c] * Wv[1];
        else if (ax == 1) M[r][c] = -px[r][c] * Wv[2] + pz[r][c] * Wv[0];
        else M[r][c] = px[r][c] * Wv[1] - py[r][c] * Wv[0];
      } else {
        if (ax == 0) M[r][c] = pz[r][c] * Wv[1] - py[r][c] * Wv[2];
        else if (ax == 1) M[r][c] = -pz[r][c] * Wv[0] + px[r][c] * Wv[2];
        else M[r][c] = py[r][c] * Wv[0] - px[r][c] * Wv[1];
      }
    }
  double coef;
  if (std::abs(d) == 1) coef = (2.0 / 3.0) * d;
  else coef = -d * (1.0 / 24.0);
  cd v = coef * M[s][s1];
  const cd img(0, 1);
  if (!wsForm) return -img * v / h;
  return (1.0 / h) * img * ls * v;
}

struct FieldsView {
  const double *f, *gradf, *U, *W, *UC;
  std::size_t ns;
};

// Sum of the Skyrme term list for one matrix entry, in the order of
// Utilities::skyrmeHamiltonian: SkyrmeU, NonLocalKinetic, LocalKinetic,
// SkyrmeSO, LocalCoulomb.
static cd skyrmeEntry(const Grid &g, const FieldsView &F, int i, int j, int k,
                      int s, int ax, int d, int s1) {
  const std::size_t p = g.idxNS(i, j, k);
  const double h = g.h, hh = h * h;
  cd val(0, 0);
  const bool same = (d == 0);
  // SkyrmeU (skyrme_u.cpp:15-24)
  if (same && s == s1) val += cd(F.U[p], 0.0);
  // NonLocalKineticPotential (non_local_kinetic_potential.cpp:23-71)
  if (!same && s == s1) {
    double C = -F.gradf[ax * F.ns + p];
    double v = 0.0;
    if (std::abs(d) == 1) v += d * 8.0 * C;
    else v += -d * C / 2.0;
    val += cd(v / (12.0 * h), 0.0);
  }
  // LocalKineticPotential (local_kinetic_potential.cpp:22-46)
  {
    double C = -F.f[p];
    double v = 0.0;
    if (same && s == s1) v = -C * (90.0 / 12.0) / hh;
    else if (!same && s == s1 && std::abs(d) == 1) v = C * (16.0 / 12.0) / hh;
    else if (!same && s == s1 && std::abs(d) == 2) v = -C * (1.0 / 12.0) / hh;
    val += cd(v, 0.0);
  }
  // SkyrmeSO (skyrme_so.cpp:12-58)
  if (F.W && !same) {
    double Wv[3] = {F.W[p], F.W[F.ns + p], F.W[2 * F.ns + p]};
    val += soElement(ax, d, s, s1, Wv, h, false, 0.0);
  }
  // LocalCoulombPotential (local_coulomb_potential.cpp:12-41)
  if (F.UC && same && s == s1) val += cd(F.UC[p], 0.0);
  return val;
}


// Radius::getRadius / getGradient (src/common/radius.cpp:7-17) with
// SphericalHarmonics::Y20 / Y20Grad (src/common/spherical_harmonics.cpp:
// 155-188). Y20Grad starts from setIdentity() on a 3-vector, i.e. (1,0,0),
// so only its x component survives; this is kept.
static double y20theta(double theta) {
  return std::sqrt(5.0 / (16.0 * M_PI)) *
         (3.0 * std::cos(theta) * std::cos(theta) - 1.0);
}
static double radiusAt(const WSParams &P, double x, double y, double z) {
  double R = P.r0 * std::pow(P.A, 1.0 / 3.0);
  double theta = std::acos(z / std::sqrt(x * x + y * y + z * z));
  return R * (1 + P.beta * y20theta(theta));
}
static void radiusGrad(const WSParams &P, double x, double y, double z,
                       double out[3]) {
  double R = P.r0 * std::pow(P.A, 1.0 / 3.0);
  double r2 = x * x + y * y + z * z;
  double r = std::sqrt(r2);
  double theta = std::acos(z / r);
  double g[3] = {1.0, 0.0, 0.0};
  for (int a = 0; a < 3; ++a) g[a] = g[a] * 1.0 / (r2 * std::sin(theta));
  for (int a = 0; a < 3; ++a)
    g[a] = g[a] * std::sqrt(5.0 / (16.0 * M_PI)) *
           (-6.0 * std::sin(theta) * std::cos(theta));
  g[0] = -g[0] * x * z;
  g[1] = -g[1] * y * z;
  g[2] = g[2] * (+x * x + y * y);
  for (int a = 0; a < 3; ++a) out[a] = R * P.beta * g[a];
}
double wsValue(const WSParams &P, double x, double y, double z) {
  double locR = radiusAt(P, x, y, z);
  double r = std::sqrt(x * x + y * y + z * z);
  double beta3def = 0.0;
  if (P.beta3 != 0.0) {
    // SphericalHarmonics::Y(3,0,x,y,z).real()
    double ct = z / r;
    double Y30 = std::sqrt(7.0 / (4.0 * M_PI)) * 0.5 * (5 * ct * ct * ct - 3 * ct);
    beta3def = P.beta3 * P.r0 * std::pow(P.A, 1.0 / 3.0) * Y30;
  }
  return -P.V0 * (1 + P.kappa * (P.A - 2 * P.Z) / ((double)P.A)) /
         (1 + std::exp((r - (locR + beta3def)) / P.diff));
}
// DeformedSpinOrbitPotential::getFactor (deformed_spin_orbit.cpp:12-27)
void wsSOFactor(const WSParams &P, double x, double y, double z,
                double out[3]) {
  double r2 = x * x + y * y + z * z;
  double r = std::sqrt(r2);
  double gr[3] = {x / r, y / r, z / r};
  out[0] = out[1] = out[2] = 0.0;
  if (r > 1e-12) {
    double t = (r - radiusAt(P, x, y, z)) / P.diff;
    double expt = std::exp(t);
    double rg[3];
    radiusGrad(P, x, y, z, rg);
    double sc = (P.soV0 / P.diff) * std::pow(1 + expt, -2) * expt;
    for (int a = 0; a < 3; ++a) out[a] = sc * (gr[a] - rg[a]);
  }
}
double wsSOls() { return -35.0 * std::pow(kHbar * 0.5 / kMass, 2); }

static cd wsEntry(const Grid &g, const WSParams &P, int i, int j, int k, int s,
                  int ax, int d, int s1) {
  const double h = g.h;
  const double C_const = -2 * kMass / (kHbar * kHbar);
  const double Chh = C_const * h * h;
  const cd diag_kin = -(90.0 / 12.0) / Chh;
  const cd off1 = (16.0 / 12.0) / Chh;
  const cd off2 = -(1.0 / 12.0) / Chh;
  const bool same = (d == 0);
  cd val(0, 0);
  if (same && s == s1) val = diag_kin;
  else if (!same && s == s1 && std::abs(d) == 1) val = off1;
  else if (!same && s == s1 && std::abs(d) == 2) val = off2;
  double x = g.xs[i], y = g.xs[j], z = g.xs[k];
  if (same && s == s1) val += cd(wsValue(P, x, y, z), 0.0);
  if (P.so && !same) {
    double gv[3];
    wsSOFactor(P, x, y, z, gv);
    val += soElement(ax, d, s, s1, gv, h, true, wsSOls());
  }
  return val;
}

// Builds CSR with columns ascending per row.
template <class Entry>
static Csr buildCsr(const Grid &g, Entry entry) {
  Csr H;
  const int n = g.n;
  H.N = (long long)g.N();
  H.rowptr.assign(H.N + 1, 0);
  std::vector<std::vector<std::pair<int, cd>>> rows(H.N);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        for (int s = 0; s < 2; ++s) {
          auto &R = rows[g.idx(i, j, k, s)];
          R.reserve(26);
          // candidate columns in ascending order: k1, j1, i1, s1
          for (int dk = -2; dk <= 2; ++dk) {
            int k1 = k + dk;
            if (k1 < 0 || k1 >= n) continue;
            for (int dj = -2; dj <= 2; ++dj) {
              int j1 = j + dj;
              if (j1 < 0 || j1 >= n) continue;
              for (int di = -2; di <= 2; ++di) {
                int i1 = i + di;
                if (i1 < 0 || i1 >= n) continue;
                int nz = (di != 0) + (dj != 0) + (dk != 0);
                if (nz > 1) continue;
                int ax = di != 0 ? 0 : (dj != 0 ? 1 : (dk != 0 ? 2 : 0));
                int d = di + dj + dk;
                for (int s1 = 0; s1 < 2; ++s1) {
                  cd v = entry(i, j, k, s, ax, d, s1);
                  if (v != cd(0.0, 0.0))
                    R.emplace_back((int)g.idx(i1, j1, k1, s1), v);
                }
              }
            }
          }
        }
  for (long long r = 0; r < H.N; ++r)
    H.rowptr[r + 1] = H.rowptr[r] + (long long)rows[r].size();
  H.col.resize(H.rowptr[H.N]);
  H.val.resize(H.rowptr[H.N]);
  H.diagpos.assign(H.N, -1);
#pragma omp parallel for schedule(static)
  for (long long r = 0; r < H.N; ++r) {
    long long o = H.rowptr[r];
    for (std::size_t q = 0; q < rows[r].size(); ++q) {
      H.col[o + q] = rows[r][q].first;
      H.val[o + q] = rows[r][q].second;
      if (rows[r][q].first == r) H.diagpos[r] = o + (long long)q;
    }
  }
  return H;
}

Csr buildSkyrme(const Grid &g, const double *f, const double *gradf,
                const double *U, const double *W, const double *UC) {
  FieldsView F{f, gradf, U, W, UC, g.ns()};
  return buildCsr(g, [&](int i, int j, int k, int s, int ax, int d, int s1) {
    return skyrmeEntry(g, F, i, j, k, s, ax, d, s1);
  });
}

Csr buildWS(const Grid &g, const WSParams &P) {
  return buildCsr(g, [&](int i, int j, int k, int s, int ax, int d, int s1) {
    return wsEntry(g, P, i, j, k, s, ax, d, s1);
  });
}

// Y = (H + shift I) X, the shift added to the stored diagonal entry as in
// A + shift*Id (src/solver/solver.cpp:720).
void spmm(const Csr &H, const cd *X, cd *Y, int ncols, double shift) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int c = 0; c < ncols; ++c)
    for (long long r = 0; r < H.N; ++r) {
      const cd *x = X + (std::size_t)c * H.N;
      cd s(0, 0);
      for (long long q = H.rowptr[r]; q < H.rowptr[r + 1]; ++q) {
        cd v = H.val[q];
        if (q == H.diagpos[r]) v += cd(shift, 0.0);
        s += v * x[H.col[q]];
      }
      Y[(std::size_t)c * H.N + r] = s;
    }
}

// ---------------------------------------------------------------------------
// Eigensolver pieces (src/solver/solver.cpp)
// ---------------------------------------------------------------------------

// b_modified_gram_schmidt_complex_no_B (solver.cpp:389-416)
void mgs(CMat &V) {
  const std::size_t N = V.rows;
  for (std::size_t j = 0; j < V.cols; ++j) {
    cd *vj = V.col(j);
    cd nb(0, 0);
    for (std::size_t r = 0; r < N; ++r) nb += std::conj(vj[r]) * vj[r];
    double norm_b_sq = nb.real();
    double norm_b = (norm_b_sq > 1e-24) ? std::sqrt(norm_b_sq) : 0.0;
    if (norm_b < 1e-12) {
      std::fill(vj, vj + N, cd(0, 0));
      continue;
    }
    for (std::size_t r = 0; r < N; ++r) vj[r] /= norm_b;
#pragma omp parallel for schedule(static)
    for (long long k = (long long)j + 1; k < (long long)V.cols; ++k) {
      cd *vk = V.col(k);
      cd proj(0, 0);
      for (std::size_t r = 0; r < N; ++r) proj += std::conj(vj[r]) * vk[r];
      for (std::size_t r = 0; r < N; ++r) vk[r] -= proj * vj[r];
    }
  }
}

// Eigen::ConjugateGradient with DiagonalPreconditioner, restated from the
// textbook Jacobi-PCG (Saad, "Iterative Methods for Sparse Linear Systems",
// Alg. 9.1) with Eigen's stopping rule: |r|^2 < max(tol^2 |b|^2, DBL_MIN),
// at most max_steps iterations, initial guess x0 (solver.cpp:733-743).
int pcgColumn(const Csr &H, double shift, const cd *b, const cd *x0, cd *x,
              int max_steps, double tol) {
  const long long N = H.N;
  std::vector<cd> r(N), z(N), p(N), tmp(N);
  std::vector<double> invdiag(N);
  for (long long i = 0; i < N; ++i) {
    cd d = H.diagpos[i] >= 0 ? H.val[H.diagpos[i]] + cd(shift, 0) : cd(shift, 0);
    invdiag[i] = (d.real() != 0.0) ? 1.0 / d.real() : 1.0;
  }
  std::copy(x0, x0 + N, x);
  auto apply = [&](const cd *in, cd *out) {
    for (long long row = 0; row < N; ++row) {
      cd s(0, 0);
      for (long long q = H.rowptr[row]; q < H.rowptr[row + 1]; ++q) {
        cd v = H.val[q];
        if (q == H.diagpos[row]) v += cd(shift, 0.0);
        s += v * in[H.col[q]];
      }
      out[row] = s;
    }
  };
  apply(x, tmp.data());
  double rhsNorm2 = 0;
  for (long long i = 0; i < N; ++i) {
    r[i] = b[i] - tmp[i];
    rhsNorm2 += std::norm(b[i]);
  }
  if (rhsNorm2 == 0) {
    std::fill(x, x + N, cd(0, 0));
    return 0;
  }
  const double considerAsZero = 2.2250738585072014e-308;
  double threshold = std::max(tol * tol * rhsNorm2, considerAsZero);
  double residualNorm2 = 0;
  for (long long i = 0; i < N; ++i) residualNorm2 += std::norm(r[i]);
  if (residualNorm2 < threshold) return 0;
  for (long long i = 0; i < N; ++i) p[i] = invdiag[i] * r[i];
  double absNew = 0;
  for (long long i = 0; i < N; ++i) absNew += (std::conj(r[i]) * p[i]).real();
  int it = 0;
  while (it < max_steps) {
    apply(p.data(), tmp.data());
    cd pAp(0, 0);
    for (long long i = 0; i < N; ++i) pAp += std::conj(p[i]) * tmp[i];
    cd alpha = absNew / pAp;
    for (long long i = 0; i < N; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * tmp[i];
    }
    residualNorm2 = 0;
    for (long long i = 0; i < N; ++i) residualNorm2 += std::norm(r[i]);
    if (residualNorm2 < threshold) break;
    for (long long i = 0; i < N; ++i) z[i] = invdiag[i] * r[i];
    double absOld = absNew;
    absNew = 0;
    for (long long i = 0; i < N; ++i) absNew += (std::conj(r[i]) * z[i]).real();
    double beta = absNew / absOld;
    for (long long i = 0; i < N; ++i) p[i] = z[i] + beta * p[i];
    ++it;
  }
  return it;
}

// gcgm_complex_no_B_lock (solver.cpp:642-959)
GcgOut gcgLock(const Csr &A, const CMat &X_initial, const CMat &ConjDir,
               int nev, double shift, int max_iter, double tolerance,
               int cg_steps, double cg_tol, int ordering) {
  GcgOut out;
  const std::size_t n = A.N;
  double current_shift = shift;
  CMat X0(n, 0);
  CMat X = X_initial.leftCols(nev);
  CMat P(n, 0);
  if (ConjDir.cols > 0) P = ConjDir;

  mgs(X);
  // initial Rayleigh-Ritz (rayleighRitz_complex_no_B, solver.cpp:418-463)
  std::vector<double> Lambda;
  {
    CMat AX(n, X.cols);
    spmm(A, X.d.data(), AX.d.data(), (int)X.cols, current_shift);
    CMat Ap = adjointTimes(X, AX);
    std::vector<double> w;
    CMat C;
    hermitianEig(Ap, w, C);
    X = times(X, C);
    Lambda.resize(w.size());
    for (std::size_t i = 0; i < w.size(); ++i) Lambda[i] = w[i] - current_shift;
  }

  bool earlyConverged = false;
  for (int iter = 0; iter < max_iter; ++iter) {
    int num_converged = (int)X0.cols;
    int num_active = (int)X.cols;
    if (num_converged == nev) {
      earlyConverged = true; // solver.cpp:697-716 returns sorted ascending
      break;
    }
    if (Lambda.size() > 1)
      current_shift = (Lambda[Lambda.size() - 1] - 100.0 * Lambda[0]) / 99.0;
    CMat W(n, num_active);
    if (num_active > 0) {
      CMat BX(n, num_active);
      for (int k = 0; k < num_active; ++k)
        for (std::size_t r = 0; r < n; ++r)
          BX(r, k) = X(r, k) * (Lambda[k] + current_shift);
      int tot = 0;
#pragma omp parallel for schedule(dynamic) reduction(+ : tot)
      for (int k = 0; k < num_active; ++k)
        tot += pcgColumn(A, current_shift, BX.col(k), X.col(k), W.col(k),
                         cg_steps, cg_tol);
      out.pcgSteps += tot;
    }
    int p_cols = (int)P.cols;
    CMat V(n, num_converged + num_active + p_cols + num_active);
    std::size_t o = 0;
    auto put = [&](const CMat &M) {
      std::copy(M.d.begin(), M.d.end(), V.d.begin() + o * n);
      o += M.cols;
    };
    put(X0);
    put(X);
    if (p_cols > 0) put(P);
    if (num_active > 0) put(W);
    mgs(V);
    std::vector<std::size_t> keep;
    for (std::size_t k = 0; k < V.cols; ++k)
      if (colNorm2(V.col(k), n) > 1e-20) keep.push_back(k);
    CMat Veff(n, keep.size());
    for (std::size_t i = 0; i < keep.size(); ++i)
      std::copy(V.col(keep[i]), V.col(keep[i]) + n, Veff.col(i));
    out.basisCols = (int)keep.size();
    CMat AV(n, Veff.cols);
    spmm(A, Veff.d.data(), AV.d.data(), (int)Veff.cols, current_shift);
    CMat Ap = adjointTimes(Veff, AV);
    std::vector<double> w;
    CMat Cfull;
    hermitianEig(Ap, w, Cfull);
    int rr_nev = std::min(nev, (int)Veff.cols);
    CMat C = Cfull.leftCols(rr_nev);
    CMat Xnew = times(Veff, C);
    if (iter == max_iter - 1) {
      // ConjDir update inside the solver is discarded (P is local); kept for
      // structural fidelity only.
    }
    P = CMat(n, 0);
    std::vector<double> Lnew(rr_nev);
    for (int i = 0; i < rr_nev; ++i) Lnew[i] = w[i] - current_shift;
    CMat AXn(n, rr_nev);
    spmm(A, Xnew.d.data(), AXn.d.data(), rr_nev, 0.0);
    std::vector<double> resn(rr_nev);
    for (int i = 0; i < rr_nev; ++i) {
      double s = 0;
      for (std::size_t r = 0; r < n; ++r)
        s += std::norm(AXn(r, i) - Xnew(r, i) * Lnew[i]);
      resn[i] = std::sqrt(s);
    }
    // locking
    CMat newX0(n, 0);
    std::vector<int> newly, next_active;
    for (int i = num_converged; i < rr_nev; ++i) {
      if (resn[i] < tolerance &&
          (num_converged + (int)newly.size() < nev))
        newly.push_back(i);
      else
        next_active.push_back(i);
    }
    CMat X0n(n, num_converged + newly.size());
    for (int i = 0; i < num_converged; ++i)
      std::copy(Xnew.col(i), Xnew.col(i) + n, X0n.col(i));
    for (std::size_t i = 0; i < newly.size(); ++i)
      std::copy(Xnew.col(newly[i]), Xnew.col(newly[i]) + n,
                X0n.col(num_converged + i));
    X0 = X0n;
    CMat Xa(n, next_active.size());
    std::vector<double> La(next_active.size());
    for (std::size_t i = 0; i < next_active.size(); ++i) {
      std::copy(Xnew.col(next_active[i]), Xnew.col(next_active[i]) + n,
                Xa.col(i));
      La[i] = Lnew[next_active[i]];
    }
    X = Xa;
    Lambda = La;
    out.iterations = iter + 1;
  }
  int ncf = (int)X0.cols;
  int need = nev - ncf;
  int take = std::min((int)X.cols, need);
  CMat finalX(n, nev);
  std::vector<double> finalL(nev, 0.0);
  for (int i = 0; i < ncf; ++i)
    std::copy(X0.col(i), X0.col(i) + n, finalX.col(i));
  for (int i = 0; i < take; ++i)
    std::copy(X.col(i), X.col(i) + n, finalX.col(ncf + i));
  if (ncf > 0) {
    CMat AX0(n, ncf);
    spmm(A, X0.d.data(), AX0.d.data(), ncf, 0.0);
    for (int i = 0; i < ncf; ++i) {
      cd s(0, 0);
      for (std::size_t r = 0; r < n; ++r) s += std::conj(X0(r, i)) * AX0(r, i);
      finalL[i] = s.real();
    }
  }
  for (int i = 0; i < take; ++i) finalL[ncf + i] = Lambda[i];
  out.converged = ncf;
  std::vector<int> idx(nev);
  std::iota(idx.begin(), idx.end(), 0);
  if (ordering == NCGM_ORDER_ASCENDING || earlyConverged) {
    std::stable_sort(idx.begin(), idx.end(),
                     [&](int a, int b) { return finalL[a] < finalL[b]; });
    out.X = CMat(n, nev);
    out.lambda.resize(nev);
    for (int k = 0; k < nev; ++k) {
      out.lambda[k] = finalL[idx[k]];
      std::copy(finalX.col(idx[k]), finalX.col(idx[k]) + n, out.X.col(k));
    }
  } else {
    // MATCH_PREVIOUS (solver.cpp:877-935): greedy overlap matching.
    CMat ov = adjointTimes(X_initial.leftCols(nev), finalX);
    std::vector<bool> at(nev, false), as(nev, false);
    out.X = CMat(n, nev);
    out.lambda.assign(nev, 0.0);
    for (int count = 0; count < nev; ++count) {
      double mx = -1;
      int bt = -1, bs = -1;
      for (int i = 0; i < nev; ++i) {
        if (at[i]) continue;
        for (int k = 0; k < nev; ++k) {
          if (as[k]) continue;
          if (std::abs(ov(i, k)) > mx) {
            mx = std::abs(ov(i, k));
            bt = i;
            bs = k;
          }
        }
      }
      if (bt < 0) break;
      cd o = ov(bt, bs);
      cd ph = std::abs(o) > 1e-12 ? o / std::abs(o) : cd(1, 0);
      for (std::size_t r = 0; r < n; ++r) out.X(r, bt) = finalX(r, bs) * ph;
      out.lambda[bt] = finalL[bs];
      at[bt] = as[bs] = true;
    }
  }
  return out;
}

} // namespace orc
