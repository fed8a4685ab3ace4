// Test infrastructure (oracle): dense FP64 helpers used by the CPU restatement
// of the nuclearcgm hot path. Nothing here is part of the product library; only
// tests, the smoke check and the CPU baseline leg of bench.py use it.
//
// Column-major complex matrices (the reference uses Eigen::MatrixXcd with the
// same layout) and Jacobi eigensolvers. The reference calls
// Eigen::SelfAdjointEigenSolver (src/solver/solver.cpp:768,
// src/util/iteration_data.cpp:301,329,732); Eigen's source is not available
// here, so the projected eigenproblems are solved with the cyclic Jacobi
// method (Golub & Van Loan, "Matrix Computations", sec. 8.5). Eigenvalues agree
// to rounding; eigenvectors agree up to a phase per column (and up to a
// unitary mix inside degenerate subspaces), which no phase-invariant quantity
// (densities, energies, projectors) sees.
#pragma once
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstddef>
#include <numeric>
#include <vector>

namespace orc {

using cd = std::complex<double>;

struct CMat {
  std::size_t rows = 0, cols = 0;
  std::vector<cd> d;
  CMat() = default;
  CMat(std::size_t r, std::size_t c) : rows(r), cols(c), d(r * c, cd(0, 0)) {}
  cd *col(std::size_t j) { return d.data() + j * rows; }
  const cd *col(std::size_t j) const { return d.data() + j * rows; }
  cd &operator()(std::size_t i, std::size_t j) { return d[j * rows + i]; }
  const cd &operator()(std::size_t i, std::size_t j) const {
    return d[j * rows + i];
  }
  CMat leftCols(std::size_t c) const {
    CMat r(rows, c);
    std::copy(d.begin(), d.begin() + rows * c, r.d.begin());
    return r;
  }
};

struct RMat {
  std::size_t rows = 0, cols = 0;
  std::vector<double> d;
  RMat() = default;
  RMat(std::size_t r, std::size_t c) : rows(r), cols(c), d(r * c, 0.0) {}
  double &operator()(std::size_t i, std::size_t j) { return d[j * rows + i]; }
  const double &operator()(std::size_t i, std::size_t j) const {
    return d[j * rows + i];
  }
};

// C = A^H B  (A: N x p, B: N x q) -> p x q
inline CMat adjointTimes(const CMat &A, const CMat &B) {
  CMat C(A.cols, B.cols);
  const std::size_t N = A.rows;
#pragma omp parallel for collapse(2) schedule(static)
  for (long long j = 0; j < (long long)B.cols; ++j)
    for (long long i = 0; i < (long long)A.cols; ++i) {
      const cd *a = A.col(i);
      const cd *b = B.col(j);
      cd s(0, 0);
      for (std::size_t r = 0; r < N; ++r) s += std::conj(a[r]) * b[r];
      C(i, j) = s;
    }
  return C;
}

// C = A B  (A: N x p, B: p x q) -> N x q
inline CMat times(const CMat &A, const CMat &B) {
  CMat C(A.rows, B.cols);
  const std::size_t N = A.rows;
#pragma omp parallel for schedule(static)
  for (long long r = 0; r < (long long)N; ++r)
    for (std::size_t j = 0; j < B.cols; ++j) {
      cd s(0, 0);
      for (std::size_t k = 0; k < A.cols; ++k) s += A(r, k) * B(k, j);
      C(r, j) = s;
    }
  return C;
}

inline double colNorm2(const cd *v, std::size_t N) {
  double s = 0;
  for (std::size_t i = 0; i < N; ++i) s += std::norm(v[i]);
  return s;
}

// Hermitian eigensolver by cyclic Jacobi rotations. Reads only the lower
// triangle of A (like Eigen::SelfAdjointEigenSolver). Returns ascending
// eigenvalues; V holds the eigenvectors column by column.
inline bool hermitianEig(const CMat &Ain, std::vector<double> &w, CMat &V) {
  const std::size_t n = Ain.rows;
  CMat A(n, n);
  for (std::size_t j = 0; j < n; ++j)
    for (std::size_t i = j; i < n; ++i) {
      if (i == j) {
        A(i, i) = cd(Ain(i, i).real(), 0.0);
      } else {
        A(i, j) = Ain(i, j);
        A(j, i) = std::conj(Ain(i, j));
      }
    }
  V = CMat(n, n);
  for (std::size_t i = 0; i < n; ++i) V(i, i) = 1.0;
  double fro = 0;
  for (auto &z : A.d) fro += std::norm(z);
  bool ok = false;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (std::size_t j = 0; j < n; ++j)
      for (std::size_t i = j + 1; i < n; ++i) off += std::norm(A(i, j));
    if (off <= 1e-32 * fro || off == 0.0) {
      ok = true;
      break;
    }
    for (std::size_t p = 0; p + 1 < n; ++p)
      for (std::size_t q = p + 1; q < n; ++q) {
        cd apq = A(p, q);
        double mag = std::abs(apq);
        if (mag == 0.0) continue;
        double app = A(p, p).real(), aqq = A(q, q).real();
        if (sweep > 3 &&
            mag < 1e-18 * std::sqrt(std::fabs(app * aqq)) + 1e-300) {
          A(p, q) = 0;
          A(q, p) = 0;
          continue;
        }
        cd ph = apq / mag; // e^{i phi}
        double tau = (aqq - app) / (2.0 * mag);
        double t = (tau >= 0 ? 1.0 : -1.0) /
                   (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        double c = 1.0 / std::sqrt(1.0 + t * t);
        double s = t * c;
        cd phc = std::conj(ph);
        // A <- A U, U = D R with columns u_p = c e_p - s e^{-i phi} e_q,
        // u_q = s e_p + c e^{-i phi} e_q
        for (std::size_t r = 0; r < n; ++r) {
          cd arp = A(r, p), arq = A(r, q);
          A(r, p) = c * arp - s * phc * arq;
          A(r, q) = s * arp + c * phc * arq;
        }
        for (std::size_t r = 0; r < n; ++r) {
          cd apr = A(p, r), aqr = A(q, r);
          A(p, r) = c * apr - s * ph * aqr;
          A(q, r) = s * apr + c * ph * aqr;
        }
        A(p, q) = 0;
        A(q, p) = 0;
        A(p, p) = cd(A(p, p).real(), 0);
        A(q, q) = cd(A(q, q).real(), 0);
        for (std::size_t r = 0; r < n; ++r) {
          cd vrp = V(r, p), vrq = V(r, q);
          V(r, p) = c * vrp - s * phc * vrq;
          V(r, q) = s * vrp + c * phc * vrq;
        }
      }
  }
  std::vector<std::size_t> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::vector<double> ev(n);
  for (std::size_t i = 0; i < n; ++i) ev[i] = A(i, i).real();
  std::stable_sort(idx.begin(), idx.end(),
                   [&](std::size_t a, std::size_t b) { return ev[a] < ev[b]; });
  w.resize(n);
  CMat Vs(n, n);
  for (std::size_t k = 0; k < n; ++k) {
    w[k] = ev[idx[k]];
    std::copy(V.col(idx[k]), V.col(idx[k]) + n, Vs.col(k));
  }
  V = Vs;
  return ok;
}

// Real symmetric eigensolver (lower triangle), ascending.
inline bool symmetricEig(const RMat &Ain, std::vector<double> &w, RMat &V) {
  const std::size_t n = Ain.rows;
  CMat A(n, n);
  for (std::size_t j = 0; j < n; ++j)
    for (std::size_t i = 0; i < n; ++i) A(i, j) = Ain(i, j);
  CMat Vc;
  bool ok = hermitianEig(A, w, Vc);
  V = RMat(n, n);
  for (std::size_t j = 0; j < n; ++j)
    for (std::size_t i = 0; i < n; ++i) V(i, j) = Vc(i, j).real();
  return ok;
}

} // namespace orc
