// The NCGM_WITH_EIGEN overloads of ncgm_reference.hpp (MatrixXcd in and out,
// as the reference's run loop passes them) and EDF(functional) on a
// functional-file object, built against a declaration-level Eigen stand-in.
// Line 1: "edf C0rr C1rr C0nJ C1nJ" of SLy4 read as an interaction.
// Line 2: "no-device" without a CUDA device, else
// "solved <columns> <eigenvalues> <lowest eigenvalue>" of a harmonic
// oscillator solved through the Eigen overloads.
#define NCGM_WITH_EIGEN
#include "ncgm_reference.hpp"

#include <cmath>
#include <cstdio>
#include <map>
#include <memory>
#include <string>

// the part of nlohmann::json's interface that EDF(functional) uses
struct Num {
  double v;
  template <class T> T get() const { return (T)v; }
};
struct Obj {
  std::map<std::string, double> m;
  bool contains(const std::string &k) const { return m.count(k) != 0; }
  Num operator[](const std::string &k) const { return Num{m.at(k)}; }
};

int main() {
  // functionals/SLy4.json as an interaction
  Obj sly4{{{"t0", -2488.91}, {"t1", 486.82}, {"t2", -546.39},
            {"t3", 13777.0}, {"W0", 123.0}, {"x0", 0.834}, {"x1", -0.344},
            {"x2", -1.0}, {"x3", 1.354}, {"sigma", 0.16666666}}};
  ncgm_ref::EDF edf(sly4);
  std::printf("edf %.9f %.9f %.9f %.9f\n", edf.params.C0rr, edf.params.C1rr,
              edf.params.C0nJ, edf.params.C1nJ);
  // the coupling-constant form reads the same numbers back
  Obj direct;
  const char *keys[] = {"C0rr", "C1rr",  "C0Drr", "C1Drr", "C0rt",
                        "C1rt", "C0J2",  "C1J2",  "C0rdr", "C1rdr",
                        "C0nJ", "C1nJ",  "sigma"};
  const double *vals = &edf.params.C0rr;
  for (int i = 0; i < 13; ++i) direct.m[keys[i]] = vals[i];
  ncgm_ref::EDF back(direct);
  if (back.params.C1nJ != edf.params.C1nJ ||
      back.params.sigma != edf.params.sigma) {
    std::printf("mismatch\n");
    return 1;
  }

  const int n = 16;
  const double a = 8.0;
  std::shared_ptr<ncgm_ref::Grid> grid;
  try {
    grid = std::make_shared<ncgm_ref::Grid>(n, a, 16);
  } catch (const std::exception &e) {
    std::printf("no-device\n");
    return 0;
  }
  const size_t ns = grid->get_total_spatial_points();
  const double hbar = 197.327053, m = 938.91869, hw = 10.0;
  std::vector<double> f(ns, hbar * hbar / (2 * m)), gradf(3 * ns, 0.0),
      U(ns);
  const double h = grid->get_h();
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double x = -a + i * h, y = -a + j * h, z = -a + k * h;
        U[grid->idxNoSpin(i, j, k)] =
            0.5 * m * (hw / hbar) * (hw / hbar) * (x * x + y * y + z * z);
      }
  ncgm_ref::SkyrmeFields F;
  F.f = f.data();
  F.gradf = gradf.data();
  F.U = U.data();
  ncgm_ref::Hamiltonian H(grid, NCGM_NEUTRON, F);
  const int nev = 8;
  Eigen::MatrixXcd guess((std::ptrdiff_t)grid->get_total_points(), nev);
  for (std::ptrdiff_t r = 0; r < guess.size(); ++r)
    guess.data()[r] =
        std::complex<double>(std::sin(0.37 * r + 1.0), std::cos(0.11 * r));
  Eigen::MatrixXcd none;
  ncgm_ref::GCGParameters calc{nev, 1e-8, 60, 40, 1e-8};
  auto res = ncgm_ref::solve(H, none, calc, guess);
  Eigen::MatrixXcd HX = ncgm_ref::apply(H, res.first);
  std::printf("solved %ld %ld %.6f %ld\n", (long)res.first.cols(),
              (long)res.second.size(), res.second(0), (long)HX.cols());
  return 0;
}
