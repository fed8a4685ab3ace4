// ncgm_reference.hpp — header-only C++ shim that re-exposes the nuclearcgm
// interfaces of the lattice hot path on top of the C ABI in ncgm.h, so the
// reference's JSON-driven run loop can call the GB300 library with the same
// names and argument meaning:
//
//   Grid                          (include/grid.hpp:12-92)
//   Hamiltonian / buildMatrix     (include/hamiltonian.hpp:16-46)
//   gcgm_complex_no_B_lock        (include/solver.hpp:43-47)
//   Utilities::solve              (include/util/utilities.hpp:19-24)
//   EDF, setFromInteraction       (include/EDF.hpp:4-31)
//
// Matrices are raw column-major complex<double> buffers in the Eigen layout
// (rows s + 2(i + n(j + n k))). Define NCGM_WITH_EIGEN before including this
// header to get overloads that take Eigen::MatrixXcd / Eigen::VectorXd
// directly. Errors are thrown as std::runtime_error on the C++ side only; the
// C ABI itself never throws.
#pragma once
#include "ncgm.h"

#include <complex>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#ifdef NCGM_WITH_EIGEN
#include <Eigen/Dense>
#endif

namespace ncgm_ref {

inline void check(int status, const char *what) {
  if (status != NCGM_OK)
    throw std::runtime_error(std::string(what) + ": " + ncgm_last_error());
}

// Grid(n, a): x_i = -a + i h, h = 2a/(n-1). Owns the device context.
class Grid {
public:
  Grid(int n, double a, int max_cols = 256) : n_(n), a_(a) {
    if (n < 2) throw std::invalid_argument("Grid error: n must be >= 2");
    ncgm_ctx *c = nullptr;
    check(ncgm_create(&c, n, a, max_cols, 0), "ncgm_create");
    ctx_.reset(c, [](ncgm_ctx *p) { ncgm_destroy(p); });
  }
  int get_n() const noexcept { return n_; }
  double get_a() const noexcept { return a_; }
  double get_h() const noexcept { return 2.0 * a_ / (n_ - 1); }
  double dV() const noexcept { return get_h() * get_h() * get_h(); }
  size_t get_total_spatial_points() const noexcept {
    return (size_t)n_ * n_ * n_;
  }
  size_t get_total_points() const noexcept { return 2 * get_total_spatial_points(); }
  size_t idx(size_t i, size_t j, size_t k, size_t s) const noexcept {
    return s + 2 * (i + n_ * (j + n_ * k));
  }
  size_t idxNoSpin(size_t i, size_t j, size_t k) const noexcept {
    return i + n_ * (j + n_ * k);
  }
  ncgm_ctx *ctx() const { return ctx_.get(); }

private:
  int n_;
  double a_;
  std::shared_ptr<ncgm_ctx> ctx_;
};

// The Skyrme mean fields of one species: what SkyrmeU, NonLocalKinetic,
// LocalKinetic, SkyrmeSO and LocalCoulomb read from IterationData.
struct SkyrmeFields {
  const double *f = nullptr;     // hbar^2/2m*, n^3
  const double *gradf = nullptr; // n^3 x 3
  const double *U = nullptr;     // central + constraint field, n^3
  const double *W = nullptr;     // spin-orbit field n^3 x 3, or null
  const double *UC = nullptr;    // Coulomb field n^3 (protons), or null
};

// Hamiltonian(grid, terms).buildMatrix() becomes a field upload; the
// returned handle applies H matrix-free on the device.
class Hamiltonian {
public:
  Hamiltonian(std::shared_ptr<Grid> grid, int species, const SkyrmeFields &F)
      : grid_(std::move(grid)), species_(species) {
    if (!grid_) throw std::invalid_argument("Hamiltonian error: Grid pointer cannot be null.");
    check(ncgm_set_fields(grid_->ctx(), species, F.f, F.gradf, F.U, F.W, F.UC),
          "ncgm_set_fields");
  }
  // build_matrix5p() with the deformed Woods-Saxon + spin-orbit terms
  static Hamiltonian woodsSaxon(std::shared_ptr<Grid> grid, int species, int A,
                                int Z, double V0, double r0, double diff,
                                double kappa, double beta, double beta3,
                                double soV0, bool spinOrbit) {
    Hamiltonian h(std::move(grid), species);
    check(ncgm_set_woods_saxon(h.grid_->ctx(), species, A, Z, V0, r0, diff,
                               kappa, beta, beta3, soV0, spinOrbit ? 1 : 0),
          "ncgm_set_woods_saxon");
    return h;
  }
  // Y = H X (X, Y: N x ncols column-major complex<double>)
  void apply(const std::complex<double> *X, std::complex<double> *Y,
             int ncols, int precision = NCGM_FP64) const {
    check(ncgm_apply_h(grid_->ctx(), species_,
                       reinterpret_cast<const double *>(X),
                       reinterpret_cast<double *>(Y), ncols, precision),
          "ncgm_apply_h");
  }
  std::shared_ptr<Grid> grid() const { return grid_; }
  int species() const { return species_; }

private:
  Hamiltonian(std::shared_ptr<Grid> g, int s) : grid_(std::move(g)), species_(s) {}
  std::shared_ptr<Grid> grid_;
  int species_;
};

enum EigenpairsOrdering { MATCH_PREVIOUS = NCGM_ORDER_MATCH_PREVIOUS,
                          ASCENDING_ENERGIES = NCGM_ORDER_ASCENDING };

struct Eigenpairs {
  std::vector<std::complex<double>> X; // N x nev column-major
  std::vector<double> lambda;          // nev
};

// gcgm_complex_no_B_lock(A, X_initial, ConjDir, nev, shift, max_iter, tol,
// cg_steps, cg_tol, benchmark, ordering) on a device Hamiltonian.
inline Eigenpairs gcgm_complex_no_B_lock(
    const Hamiltonian &A, const std::complex<double> *X_initial, int xcols,
    const std::complex<double> *ConjDir, int pcols, int nev, double shift,
    int max_iter, double tolerance, int cg_steps, double cg_tol,
    bool /*benchmark*/, EigenpairsOrdering ordering,
    int precision = NCGM_FP64) {
  const size_t N = A.grid()->get_total_points();
  Eigenpairs out;
  out.X.resize(N * nev);
  out.lambda.resize(nev);
  ncgm_gcg_params p{max_iter, tolerance, cg_steps, cg_tol, shift,
                    (int)ordering, precision, 0};
  check(ncgm_gcg(A.grid()->ctx(), A.species(),
                 reinterpret_cast<const double *>(X_initial), xcols,
                 reinterpret_cast<const double *>(ConjDir), pcols, nev, &p,
                 reinterpret_cast<double *>(out.X.data()), out.lambda.data(),
                 nullptr),
        "ncgm_gcg");
  return out;
}

// GCGParameters (include/input_parser.hpp:29-35)
struct GCGParameters {
  int nev;
  double tol;
  int maxIter;
  int steps;
  double cgTol;
};

// Utilities::solve: shift 0, ascending order, nev = guess columns by default
inline Eigenpairs solve(const Hamiltonian &H, const std::complex<double> *ConjDir,
                        int pcols, const GCGParameters &calc,
                        const std::complex<double> *guess, int guessCols,
                        int nev = -1, int precision = NCGM_FP64) {
  return gcgm_complex_no_B_lock(H, guess, guessCols, ConjDir, pcols,
                                nev < 0 ? guessCols : nev, 0.0, calc.maxIter,
                                calc.tol, calc.steps, calc.cgTol, false,
                                ASCENDING_ENERGIES, precision);
}

// EDF::setFromInteraction
inline ncgm_edf edfFromSkyrme(const ncgm_skyrme &s) {
  ncgm_edf e;
  check(ncgm_edf_from_skyrme(&s, &e), "ncgm_edf_from_skyrme");
  return e;
}

// SkyrmeParameters / FunctionalParameters (include/EDF.hpp:4-23): the same
// fields in the same order as the C structs
using SkyrmeParameters = ncgm_skyrme;
using FunctionalParameters = ncgm_edf;

// EDF (include/EDF.hpp:25-31, src/skyrme/EDF.cpp:4-59), built from one
// functional-file object. `Json` is anything with contains(key) and
// operator[](key) whose values have get<double>(): nlohmann::json itself, so
// EDF(functional) reads the reference's functionals/<name>.json objects
// unchanged. An interaction (a "t0" key) is converted with
// setFromInteraction (W0_pr defaults to W0; te/to from "te"/"to", else from
// "aT"/"bT", else zero); otherwise the coupling constants are read directly.
class EDF {
public:
  FunctionalParameters params{};

  template <class Json> explicit EDF(const Json &functional) {
    auto num = [&](const char *key) {
      return functional[key].template get<double>();
    };
    if (functional.contains("t0")) {
      SkyrmeParameters p{};
      p.W0 = num("W0");
      p.W0_pr = functional.contains("W0_pr") ? num("W0_pr") : p.W0;
      p.te = p.to = 0.0;
      if (functional.contains("te")) {
        p.te = num("te");
        p.to = num("to");
      } else if (functional.contains("aT")) {
        p.to = 4 * num("aT") / 5;
        p.te = 8 * num("bT") / 5 - p.to;
      }
      p.t0 = num("t0");
      p.t1 = num("t1");
      p.t2 = num("t2");
      p.t3 = num("t3");
      p.x0 = num("x0");
      p.x1 = num("x1");
      p.x2 = num("x2");
      p.x3 = num("x3");
      p.sigma = num("sigma");
      setFromInteraction(p);
    } else {
      params = FunctionalParameters{
          num("C0rr"),  num("C1rr"),  num("C0Drr"), num("C1Drr"),
          num("C0rt"),  num("C1rt"),  num("C0J2"),  num("C1J2"),
          num("C0rdr"), num("C1rdr"), num("C0nJ"),  num("C1nJ"),
          num("sigma")};
    }
  }
  void setFromInteraction(const SkyrmeParameters &p) {
    check(ncgm_edf_from_skyrme(&p, &params), "ncgm_edf_from_skyrme");
  }
};

#ifdef NCGM_WITH_EIGEN
inline Eigen::MatrixXcd apply(const Hamiltonian &H, const Eigen::MatrixXcd &X,
                              int precision = NCGM_FP64) {
  Eigen::MatrixXcd Y(X.rows(), X.cols());
  H.apply(X.data(), Y.data(), (int)X.cols(), precision);
  return Y;
}
inline std::pair<Eigen::MatrixXcd, Eigen::VectorXd>
solve(const Hamiltonian &H, const Eigen::MatrixXcd &ConjDir,
      const GCGParameters &calc, const Eigen::MatrixXcd &guess, int nev = -1) {
  Eigenpairs e = solve(H, ConjDir.cols() ? ConjDir.data() : nullptr,
                       (int)ConjDir.cols(), calc, guess.data(),
                       (int)guess.cols(), nev);
  const int k = (int)e.lambda.size();
  Eigen::MatrixXcd X = Eigen::Map<Eigen::MatrixXcd>(e.X.data(), guess.rows(), k);
  Eigen::VectorXd l = Eigen::Map<Eigen::VectorXd>(e.lambda.data(), k);
  return {X, l};
}
#endif

} // namespace ncgm_ref
