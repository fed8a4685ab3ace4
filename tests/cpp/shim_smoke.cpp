// Builds against include/ncgm_reference.hpp the way the reference's run loop
// would: Grid -> Hamiltonian (fields) -> solve (GCG) -> eigenvalues.
// Exit 0 and print "no-device" when no CUDA device is visible; on a GPU
// print the lowest eigenvalues of a harmonic-oscillator Hamiltonian.
#include "ncgm_reference.hpp"

#include <cmath>
#include <cstdio>
#include <memory>

int main() {
  const int n = 16;
  const double a = 8.0;
  std::shared_ptr<ncgm_ref::Grid> grid;
  try {
    grid = std::make_shared<ncgm_ref::Grid>(n, a, 16);
  } catch (const std::exception &e) {
    std::printf("no-device: %s\n", e.what());
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
  std::vector<std::complex<double>> guess(grid->get_total_points() * nev);
  for (size_t r = 0; r < guess.size(); ++r)
    guess[r] = std::complex<double>(std::sin(0.37 * r + 1.0), std::cos(0.11 * r));
  ncgm_ref::GCGParameters calc{nev, 1e-8, 60, 40, 1e-8};
  auto e = ncgm_ref::solve(H, nullptr, 0, calc, guess.data(), nev);
  for (double l : e.lambda) std::printf("%.6f\n", l);
  return 0;
}
