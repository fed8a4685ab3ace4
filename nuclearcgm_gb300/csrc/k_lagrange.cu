// Lagrange-mesh recompute of the output step. After the HF loop the
// reference's Output::shellsToFile (src/system/output.cpp:252-256) calls
// IterationData::recomputeLagrange (src/util/iteration_data.cpp:346-382):
// tau and J_{mu nu} are rebuilt from the final occupied orbitals with the
// Lagrange-mesh first derivative instead of the 5-point stencil, the
// Laplacian of rho with the square of that matrix, and the integrated energy
// kinetic + totalEnergyIntegral is evaluated again ("EintLag").
//
// The derivative matrix is lagrangeFirstDerivative
// (src/operators/differential_operators.cpp:108-129):
//   D(s, t) = (-1)^(t-s) pi / (n h) / sin(pi (t - s) / n),  D(s, s) = 0,
// antisymmetric. Operators::gradLagrange (differential_operators.cpp:237-278)
// contracts D's second index with the axis and negates: g_a = -D psi along
// axis a, for both spin components. lapLagrangeNoSpin (:196-235) contracts
// the first index of D D with each axis and sums x + y + z.
//
// One thread per lattice point loops over the orbitals, as the density
// kernel does, so tau and J are sums in a fixed order (no atomics). The
// derivative matrices sit in shared memory. Per point and orbital: 3 axes x
// 2 spins x n complex multiply-adds in FP64; this runs once per HF run.
#include "k_density.cuh"
#include "ncgm_internal.cuh"

#include <cmath>
#include <vector>

namespace ncgm {

namespace {

struct Cz {
  double x, y;
};

__device__ __forceinline__ void pauliLg(int nu, Cz a, Cz b, Cz &o0, Cz &o1) {
  // sigma_x, sigma_y, sigma_z of nuclearConstants::getPauli
  // (src/common/constants.cpp:4-23) applied to the spinor (a, b)
  if (nu == 0) {
    o0 = b;
    o1 = a;
  } else if (nu == 1) {
    o0 = {b.y, -b.x}; // -i b
    o1 = {-a.y, a.x}; //  i a
  } else {
    o0 = a;
    o1 = {-b.x, -b.y};
  }
}

// Ds[r * n + c] = D(r, c) (row-major); tau and J9 (9 x ns, column mu*3+nu)
// of the M orbitals Phi (N x M, Eigen layout: spin fastest)
__global__ void lagrangeTauJKernel(const double2 *__restrict__ Phi, size_t ld,
                                   int M, int n, const double *__restrict__ D,
                                   double *tau, double *J9) {
  extern __shared__ double Ds[];
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) Ds[e] = D[e];
  __syncthreads();
  const size_t ns = (size_t)n * n * n;
  const size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (p >= ns) return;
  const int i = (int)(p % n), j = (int)((p / n) % n),
            k = (int)(p / ((size_t)n * n));
  const size_t sy = n, sz = (size_t)n * n;
  const size_t bx = p - i, by = p - (size_t)j * sy, bz = p - (size_t)k * sz;
  const double *Dx = Ds + (size_t)i * n, *Dy = Ds + (size_t)j * n,
               *Dz = Ds + (size_t)k * n;
  double t = 0.0, J[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) J[q] = 0.0;
  for (int c = 0; c < M; ++c) {
    const double2 *ps = Phi + (size_t)c * ld;
    Cz g[3][2];
#pragma unroll
    for (int s2 = 0; s2 < 2; ++s2) {
      double xr = 0, xi = 0, yr = 0, yi = 0, zr = 0, zi = 0;
      for (int s = 0; s < n; ++s) {
        const double2 vx = ps[2 * (bx + s) + s2];
        const double2 vy = ps[2 * (by + s * sy) + s2];
        const double2 vz = ps[2 * (bz + s * sz) + s2];
        xr += Dx[s] * vx.x;
        xi += Dx[s] * vx.y;
        yr += Dy[s] * vy.x;
        yi += Dy[s] * vy.y;
        zr += Dz[s] * vz.x;
        zi += Dz[s] * vz.y;
      }
      g[0][s2] = {-xr, -xi};
      g[1][s2] = {-yr, -yi};
      g[2][s2] = {-zr, -zi};
    }
    const double2 a0 = ps[2 * p], a1 = ps[2 * p + 1];
    const Cz psi0 = {a0.x, a0.y}, psi1 = {a1.x, a1.y};
    // kinetic density (wavefunction.cpp:334-346): sum over axes and spins
    double m0 = 0, m1 = 0;
#pragma unroll
    for (int mu = 0; mu < 3; ++mu) {
      m0 += g[mu][0].x * g[mu][0].x + g[mu][0].y * g[mu][0].y;
      m1 += g[mu][1].x * g[mu][1].x + g[mu][1].y * g[mu][1].y;
    }
    t += m0 + m1;
    // soDensityLagrange (wavefunction.cpp:372-414): Im(psi^* sigma_nu g_mu)
#pragma unroll
    for (int mu = 0; mu < 3; ++mu)
#pragma unroll
      for (int nu = 0; nu < 3; ++nu) {
        Cz q0, q1;
        pauliLg(nu, g[mu][0], g[mu][1], q0, q1);
        J[mu * 3 + nu] += psi0.x * q0.y - psi0.y * q0.x + psi1.x * q1.y -
                          psi1.y * q1.x;
      }
  }
  tau[p] = t;
#pragma unroll
  for (int q = 0; q < 9; ++q) J9[(size_t)q * ns + p] = J[q];
}

// lap(p) = sum over axes of sum_s D2(s, t_a) v(s along a), D2 = D D;
// D2t[r * n + c] = D2(c, r) so a thread reads its own row. With g3 also
// gradLagrangeNoSpin (differential_operators.cpp:156-194): g_a(t) =
// sum_s D(s, t) v(s along a) from Dt[r * n + c] = D(c, r), n^3 x 3
// column-major.
__global__ void lagrangeLapKernel(const double *__restrict__ v, int n,
                                  const double *__restrict__ D2t,
                                  const double *__restrict__ Dt, double *lap,
                                  double *g3) {
  extern __shared__ double Ds[];
  double *Dg = Ds + (size_t)n * n;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    Ds[e] = D2t[e];
    if (g3) Dg[e] = Dt[e];
  }
  __syncthreads();
  const size_t ns = (size_t)n * n * n;
  const size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (p >= ns) return;
  const int i = (int)(p % n), j = (int)((p / n) % n),
            k = (int)(p / ((size_t)n * n));
  const size_t sy = n, sz = (size_t)n * n;
  const size_t bx = p - i, by = p - (size_t)j * sy, bz = p - (size_t)k * sz;
  double ax = 0, ay = 0, az = 0;
  for (int s = 0; s < n; ++s) {
    ax += Ds[(size_t)i * n + s] * v[bx + s];
    ay += Ds[(size_t)j * n + s] * v[by + s * sy];
    az += Ds[(size_t)k * n + s] * v[bz + s * sz];
  }
  if (lap) lap[p] = ax + ay + az;
  if (g3) {
    double gx = 0, gy = 0, gz = 0;
    for (int s = 0; s < n; ++s) {
      gx += Dg[(size_t)i * n + s] * v[bx + s];
      gy += Dg[(size_t)j * n + s] * v[by + s * sy];
      gz += Dg[(size_t)k * n + s] * v[bz + s * sz];
    }
    g3[p] = gx;
    g3[ns + p] = gy;
    g3[2 * ns + p] = gz;
  }
}

// lagrangeFirstDerivative (differential_operators.cpp:108-129), row-major
std::vector<double> firstDerivative(int n, double h) {
  std::vector<double> D((size_t)n * n, 0.0);
  for (int s = 0; s < n; ++s)
    for (int t = 0; t < n; ++t) {
      if (s == t) continue;
      const double diff = (double)(t - s);
      D[(size_t)s * n + t] = std::pow(-1.0, diff) * (M_PI / (n * h)) *
                             (1.0 / std::sin(M_PI * diff / n));
    }
  return D;
}

} // namespace

size_t lagrangeScratchBytes(int n) { return 3 * (size_t)n * n * sizeof(double); }

int lagrangeDensities(const double2 *Phi, size_t ld, int M, int n, double h,
                      const double *rho, double *tau, double *J9, double *lap,
                      double *grad3, void *scratch, cudaStream_t s) {
  const size_t smem = (size_t)n * n * sizeof(double);
  if (2 * smem > 200 * 1024) {
    setError("Lagrange recompute: lattice above 113 points per axis");
    return NCGM_ERR_ARG;
  }
  static const bool attr = [] {
    cudaFuncSetAttribute(lagrangeTauJKernel,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         200 * 1024);
    cudaFuncSetAttribute(lagrangeLapKernel,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         200 * 1024);
    return true;
  }();
  (void)attr;
  const std::vector<double> D = firstDerivative(n, h);
  // D2 = D D (Eigen's product in lapLagrangeNoSpin), stored transposed
  std::vector<double> D2t((size_t)n * n, 0.0);
  for (int a = 0; a < n; ++a)
    for (int b = 0; b < n; ++b) {
      double acc = 0.0;
      for (int u = 0; u < n; ++u) acc += D[(size_t)a * n + u] * D[(size_t)u * n + b];
      D2t[(size_t)b * n + a] = acc;
    }
  std::vector<double> Dt((size_t)n * n);
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) Dt[(size_t)r * n + c] = D[(size_t)c * n + r];
  double *dD = static_cast<double *>(scratch);
  double *dD2 = dD + (size_t)n * n, *dDt = dD2 + (size_t)n * n;
  NCGM_CUDA(cudaMemcpyAsync(dD, D.data(), smem, cudaMemcpyHostToDevice, s));
  NCGM_CUDA(cudaMemcpyAsync(dD2, D2t.data(), smem, cudaMemcpyHostToDevice, s));
  NCGM_CUDA(cudaMemcpyAsync(dDt, Dt.data(), smem, cudaMemcpyHostToDevice, s));
  const size_t ns = (size_t)n * n * n;
  const unsigned blocks = (unsigned)((ns + 127) / 128);
  if (tau && J9) {
    if (Phi && M > 0) {
      lagrangeTauJKernel<<<blocks, 128, smem, s>>>(Phi, ld, M, n, dD, tau,
                                                   J9);
    } else {
      NCGM_CUDA(cudaMemsetAsync(tau, 0, ns * sizeof(double), s));
      NCGM_CUDA(cudaMemsetAsync(J9, 0, 9 * ns * sizeof(double), s));
    }
  }
  if (rho && (lap || grad3))
    lagrangeLapKernel<<<blocks, 128, 2 * smem, s>>>(rho, n, dD2, dDt, lap,
                                                     grad3);
  NCGM_CUDA(cudaGetLastError());
  // the host vectors must outlive the copies
  NCGM_CUDA(cudaStreamSynchronize(s));
  return NCGM_OK;
}

} // namespace ncgm
