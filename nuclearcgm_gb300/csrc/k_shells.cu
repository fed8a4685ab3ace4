// Single-particle shell observables of the output step: the expectation
// values behind Shell::l / j / mj / P (src/util/shell.cpp:22-51) and the
// <L.S> sums of IterationData::chargeRadius (src/util/iteration_data.cpp:
// 121-151), with the operators of src/operators/angular_momentum.cpp:
//   L_x = -i hbar (y d_z - z d_y), L_y = -i hbar (z d_x - x d_z),
//   L_z = -i hbar (x d_y - y d_x)                          (:206-267)
//   S_z = hbar/2 sigma_z, S^2 = 3/4 hbar^2                  (:54-57,185-205)
//   L^2 = L_x L_x + L_y L_y + L_z L_z, each L_a applied twice (:59-62)
//   L.S psi = -i hbar^2 / 2 [L'_z psi_up + (L'_x - i L'_y) psi_dn,
//                            (L'_x + i L'_y) psi_up - L'_z psi_dn]   (:118-183)
//   J^2 = L^2 + S^2 + 2 L.S, J_z = L_z + S_z                 (:50-53,269-272)
//   P psi(r) = psi(-r)                          (common_operators.cpp:4-22)
// with d_a the order-dropping first derivative of Operators::derivative.
// Per column, pass 1 writes L_x psi, L_y psi, L_z psi and J_z psi and sums
// int psi conj(L.S psi), int |psi|^2 and psi(-r)^* psi(r); pass 2 applies
// L_a to L_a psi and J_z to J_z psi and sums int psi conj(L^2 psi) and
// int psi conj(J_z J_z psi). The integrals carry the trapezoid weights of
// Operators::integral (integral_operators.cpp:4-32). Block partial sums are
// added in a fixed order on the host.
#include "fd_deriv.cuh"
#include "ncgm_internal.cuh"

#include <vector>

namespace ncgm {

namespace {

constexpr double kHbarSh = 197.327053; // nuclearConstants::h_bar
constexpr int kShT = 128;

struct Cs {
  double x, y;
  __device__ Cs operator+(Cs o) const { return {x + o.x, y + o.y}; }
  __device__ Cs operator-(Cs o) const { return {x - o.x, y - o.y}; }
  __device__ Cs operator-() const { return {-x, -y}; }
  __device__ Cs operator/(double d) const { return {x / d, y / d}; }
  __device__ friend Cs operator*(double a, Cs c) { return {a * c.x, a * c.y}; }
};
// -i hbar u
__device__ __forceinline__ Cs mihb(Cs u, double hb) { return {hb * u.y, -hb * u.x}; }
// Re(a conj(b))
__device__ __forceinline__ double reAcB(Cs a, Cs b) { return a.x * b.x + a.y * b.y; }

__device__ __forceinline__ double trapWeight(int i, int j, int k, int n) {
  double w = 1.0;
  if (i == 0 || i == n - 1) w *= 0.5;
  if (j == 0 || j == n - 1) w *= 0.5;
  if (k == 0 || k == n - 1) w *= 0.5;
  return w;
}

__device__ double blockSumSh(double v, double *sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// d/dx_a of component s of the spinor field F at point (i, j, k)
struct Deriv {
  const double2 *F;
  int n;
  double h;
  __device__ Cs at(size_t q, int s) const {
    const double2 v = F[2 * q + s];
    return {v.x, v.y};
  }
  __device__ Cs d(int axis, int i, int j, int k, int s) const {
    const size_t p = (size_t)i + (size_t)n * (j + (size_t)n * k);
    if (axis == 0)
      return fd::d1<Cs>([&](int q) { return at(p - i + q, s); }, i, n, h);
    if (axis == 1)
      return fd::d1<Cs>(
          [&](int q) { return at(p + ((long long)q - j) * n, s); }, j, n, h);
    return fd::d1<Cs>(
        [&](int q) { return at(p + ((long long)q - k) * n * n, s); }, k, n, h);
  }
};

// T: 4 x N complex (L_x psi, L_y psi, L_z psi, J_z psi); part: 3 x gridDim
__global__ void shellPass1(const double2 *__restrict__ psi, int n, double a,
                           double h, double2 *T, double *part) {
  __shared__ double sh[kShT];
  const size_t ns = (size_t)n * n * n, N = 2 * ns;
  const size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  double ls = 0, nrm = 0, par = 0;
  if (p < ns) {
    const int i = (int)(p % n), j = (int)((p / n) % n),
              k = (int)(p / ((size_t)n * n));
    const double x = -a + i * h, y = -a + j * h, z = -a + k * h;
    const Deriv D{psi, n, h};
    Cs lp[3][2]; // (r x grad)_a psi_s without -i hbar
    Cs ps[2];
    for (int s = 0; s < 2; ++s) {
      const Cs dx = D.d(0, i, j, k, s), dy = D.d(1, i, j, k, s),
               dz = D.d(2, i, j, k, s);
      lp[0][s] = y * dz - z * dy;
      lp[1][s] = z * dx - x * dz;
      lp[2][s] = x * dy - y * dx;
      ps[s] = D.at(p, s);
    }
    for (int s = 0; s < 2; ++s) {
      const Cs lx = mihb(lp[0][s], kHbarSh), ly = mihb(lp[1][s], kHbarSh),
               lz = mihb(lp[2][s], kHbarSh);
      const double sz = s == 0 ? 0.5 * kHbarSh : -0.5 * kHbarSh;
      const Cs jz = lz + sz * ps[s];
      T[2 * p + s] = make_double2(lx.x, lx.y);
      T[N + 2 * p + s] = make_double2(ly.x, ly.y);
      T[2 * N + 2 * p + s] = make_double2(lz.x, lz.y);
      T[3 * N + 2 * p + s] = make_double2(jz.x, jz.y);
    }
    // L.S psi with prefactor -i hbar^2 / 2
    const double hb2 = 0.5 * kHbarSh * kHbarSh;
    const Cs iLy1 = {-lp[1][1].y, lp[1][1].x}, iLy0 = {-lp[1][0].y, lp[1][0].x};
    const Cs up = mihb(lp[2][0] + (lp[0][1] - iLy1), hb2);
    const Cs dn = mihb((lp[0][0] + iLy0) - lp[2][1], hb2);
    const double w = trapWeight(i, j, k, n) * h * h * h;
    ls = w * (reAcB(up, ps[0]) + reAcB(dn, ps[1]));
    nrm = w * (ps[0].x * ps[0].x + ps[0].y * ps[0].y + ps[1].x * ps[1].x +
               ps[1].y * ps[1].y);
    const size_t q = (size_t)(n - 1 - i) +
                     (size_t)n * ((n - 1 - j) + (size_t)n * (n - 1 - k));
    par = reAcB(ps[0], D.at(q, 0)) + reAcB(ps[1], D.at(q, 1));
  }
  ls = blockSumSh(ls, sh);
  nrm = blockSumSh(nrm, sh);
  par = blockSumSh(par, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = ls;
    part[gridDim.x + blockIdx.x] = nrm;
    part[2 * gridDim.x + blockIdx.x] = par;
  }
}

// part: 2 x gridDim (int psi conj(L^2 psi), int psi conj(J_z J_z psi))
__global__ void shellPass2(const double2 *__restrict__ psi,
                           const double2 *__restrict__ T, int n, double a,
                           double h, double *part) {
  __shared__ double sh[kShT];
  const size_t ns = (size_t)n * n * n, N = 2 * ns;
  const size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  double l2 = 0, jj = 0;
  if (p < ns) {
    const int i = (int)(p % n), j = (int)((p / n) % n),
              k = (int)(p / ((size_t)n * n));
    const double x = -a + i * h, y = -a + j * h, z = -a + k * h;
    const Deriv Dx{T, n, h}, Dy{T + N, n, h}, Dz{T + 2 * N, n, h},
        Dj{T + 3 * N, n, h}, P{psi, n, h};
    const double w = trapWeight(i, j, k, n) * h * h * h;
    for (int s = 0; s < 2; ++s) {
      // L_x (L_x psi) + L_y (L_y psi) + L_z (L_z psi)
      const Cs a1 = mihb(y * Dx.d(2, i, j, k, s) - z * Dx.d(1, i, j, k, s),
                         kHbarSh);
      const Cs a2 = mihb(z * Dy.d(0, i, j, k, s) - x * Dy.d(2, i, j, k, s),
                         kHbarSh);
      const Cs a3 = mihb(x * Dz.d(1, i, j, k, s) - y * Dz.d(0, i, j, k, s),
                         kHbarSh);
      const Cs L2 = a1 + a2 + a3;
      // J_z (J_z psi) = L_z (J_z psi) + S_z (J_z psi)
      const double sz = s == 0 ? 0.5 * kHbarSh : -0.5 * kHbarSh;
      const Cs JJ = mihb(x * Dj.d(1, i, j, k, s) - y * Dj.d(0, i, j, k, s),
                         kHbarSh) +
                    sz * Dj.at(p, s);
      const Cs ps = P.at(p, s);
      l2 += w * reAcB(ps, L2);
      jj += w * reAcB(ps, JJ);
    }
  }
  l2 = blockSumSh(l2, sh);
  jj = blockSumSh(jj, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = l2;
    part[gridDim.x + blockIdx.x] = jj;
  }
}

} // namespace

size_t shellScratchBytes(int n) {
  const size_t ns = (size_t)n * n * n;
  const size_t blocks = (ns + kShT - 1) / kShT;
  return 4 * 2 * ns * sizeof(double2) + 5 * blocks * sizeof(double) + 256;
}

// obs: per column [L2, J2, JzJz, parity, LS] (see the file comment)
int shellObservables(const double2 *Psi, size_t ld, int ncols, int n,
                     double a, void *scratch, double *obs, cudaStream_t s) {
  const size_t ns = (size_t)n * n * n, N = 2 * ns;
  const unsigned blocks = (unsigned)((ns + kShT - 1) / kShT);
  double2 *T = static_cast<double2 *>(scratch);
  double *part = reinterpret_cast<double *>(T + 4 * N);
  const double h = 2.0 * a / (n - 1);
  std::vector<double> hp(5 * (size_t)blocks);
  for (int c = 0; c < ncols; ++c) {
    const double2 *psi = Psi + (size_t)c * ld;
    shellPass1<<<blocks, kShT, 0, s>>>(psi, n, a, h, T, part);
    shellPass2<<<blocks, kShT, 0, s>>>(psi, T, n, a, h, part + 3 * blocks);
    NCGM_CUDA(cudaGetLastError());
    NCGM_CUDA(cudaMemcpyAsync(hp.data(), part, hp.size() * sizeof(double),
                              cudaMemcpyDeviceToHost, s));
    NCGM_CUDA(cudaStreamSynchronize(s));
    double sums[5] = {0, 0, 0, 0, 0}; // ls, norm, parity, l2, jzjz
    for (int t = 0; t < 5; ++t)
      for (unsigned b = 0; b < blocks; ++b) sums[t] += hp[(size_t)t * blocks + b];
    const double hb2 = kHbarSh * kHbarSh;
    double *o = obs + 5 * (size_t)c;
    o[0] = sums[3];
    o[1] = sums[3] + 0.75 * hb2 * sums[1] + 2.0 * sums[0];
    o[2] = sums[4];
    o[3] = sums[2];
    o[4] = sums[0];
  }
  return NCGM_OK;
}

} // namespace ncgm
