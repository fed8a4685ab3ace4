// Matrix-free single-particle Hamiltonian H.X on blocks of complex 2-spinors.
//
// Replaces the assembled sparse H of Hamiltonian::buildMatrix
// (src/hamiltonian/hamiltonian.cpp:303-372) built from the term list of
// Utilities::skyrmeHamiltonian (src/util/utilities.cpp:56-70). Row point
// fields, 5-point (4th-order) stencils truncated at the box edge:
//   (H psi)(r) = [U + UC + 7.5 f/h^2] psi
//              - f/h^2 sum_a [4/3 (psi_{+a} + psi_{-a}) - 1/12 (psi_{+2a} + psi_{-2a})]
//              + sum_a (-d_a f - i (sigma x W)_a) D_a psi,
//   D_a psi = [8 (psi_{+a} - psi_{-a}) - (psi_{+2a} - psi_{-2a})] / (12 h),
// which is LocalKineticPotential (local_kinetic_potential.cpp:22-46),
// NonLocalKineticPotential (non_local_kinetic_potential.cpp:23-71), SkyrmeU
// (skyrme_u.cpp:15-24), SkyrmeSO (skyrme_so.cpp:12-58) and
// LocalCoulombPotential (local_coulomb_potential.cpp:12-41) summed.
//
// This file holds the FP64 kernel stencilPoint (one thread per (point,
// column), neighbours through the L1/L2 caches; GB300's FP64 pipe, not HBM,
// bounds it), the per-point coefficient builders and the Woods-Saxon guess
// fields. The HBM-bound FP32 kernel is in k_stencil32.cu.
#include "ncgm_internal.cuh"
#include "stencil_core.cuh"

#include <algorithm>
#include <vector>
#include <cmath>
#include <cstdio>

namespace ncgm {

namespace {

constexpr double kHbar = 197.327053;
constexpr double kMass = 938.91869;

template <class T> struct V4;
template <> struct V4<double> { using type = double4_32a; };
template <> struct V4<float> { using type = float4; };

template <class T>
__device__ __forceinline__ Spinor<T> ldSpinor(const typename V4<T>::type *p) {
  typename V4<T>::type v = *p;
  return {v.x, v.y, v.z, v.w};
}

// ---- simple kernel: one thread per (point, column) ----------------------
template <class T>
__global__ void __launch_bounds__(256)
    stencilPoint(const typename V4<T>::type *__restrict__ X,
                 typename V4<T>::type *__restrict__ Y,
                 const typename V4<T>::type *__restrict__ coef, int n,
                 size_t ns, T shift) {
  using Vt = typename V4<T>::type;
  const size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (p >= ns) return;
  const int col = blockIdx.y;
  const Vt *x = X + (size_t)col * ns;
  const int i = (int)(p % n), j = (int)((p / n) % n), k = (int)(p / ((size_t)n * n));
  const size_t sy = n, sz = (size_t)n * n;
  auto at = [&](int di, int dj, int dk) -> Spinor<T> {
    int ii = i + di, jj = j + dj, kk = k + dk;
    if (ii < 0 || ii >= n || jj < 0 || jj >= n || kk < 0 || kk >= n)
      return {T(0), T(0), T(0), T(0)};
    const long long q = (long long)p + di + dj * (long long)sy + dk * (long long)sz;
    return ldSpinor<T>(x + q);
  };
  Vt c0 = coef[2 * p], c1 = coef[2 * p + 1];
  T c[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
  Spinor<T> o = pointH<T>(c, shift, at(0, 0, 0), at(1, 0, 0), at(-1, 0, 0),
                          at(2, 0, 0), at(-2, 0, 0), at(0, 1, 0), at(0, -1, 0),
                          at(0, 2, 0), at(0, -2, 0), at(0, 0, 1), at(0, 0, -1),
                          at(0, 0, 2), at(0, 0, -2));
  Y[(size_t)col * ns + p] = Vt{o.r0, o.i0, o.r1, o.i1};
}

// ---- coefficient builders -------------------------------------------------
__global__ void buildCoefKernel(const double *f, const double *gf,
                                const double *U, const double *W,
                                const double *UC, size_t ns, double h,
                                double *c64, float *c32, float *c32s) {
  size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (p >= ns) return;
  const double hh = h * h, i12h = 1.0 / (12.0 * h);
  double c[8];
  double u = U[p] + (UC ? UC[p] : 0.0);
  c[0] = u + (90.0 / 12.0) * f[p] / hh;
  c[1] = f[p] / hh;
  for (int a = 0; a < 3; ++a) c[2 + a] = -gf[a * ns + p] * i12h;
  for (int a = 0; a < 3; ++a) c[5 + a] = W ? W[a * ns + p] * i12h : 0.0;
  for (int q = 0; q < 8; ++q) {
    c64[8 * p + q] = c[q];
    c32[8 * p + q] = (float)c[q];
    c32s[(q < 4 ? 4 * p : 4 * (ns + p) - 4) + q] = (float)c[q];
  }
}

// Deformed Woods-Saxon guess fields (deformed_woods_saxon.cpp:12-17,
// deformed_spin_orbit.cpp:12-27,55-58, radius.cpp:7-17): f = hbar^2/2m,
// grad f = 0, U = V_WS, W = ls * grad V_SO, ls = -35 (hbar/2m)^2. The radius
// gradient keeps the reference's Y20Grad, whose only non-zero component is x.
__global__ void wsFieldKernel(int n, double a, double h, int A, int Z,
                              double V0, double r0, double diff, double kappa,
                              double beta, double beta3, double soV0, int so,
                              double *f, double *gf, double *U, double *W) {
  size_t ns = (size_t)n * n * n;
  size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (p >= ns) return;
  int i = (int)(p % n), j = (int)((p / n) % n), k = (int)(p / ((size_t)n * n));
  double x = -a + i * h, y = -a + j * h, z = -a + k * h;
  double r = sqrt(x * x + y * y + z * z);
  double R = r0 * pow((double)A, 1.0 / 3.0);
  double theta = acos(z / r);
  double y20 = sqrt(5.0 / (16.0 * M_PI)) * (3.0 * cos(theta) * cos(theta) - 1.0);
  double locR = R * (1 + beta * y20);
  double b3 = 0.0;
  if (beta3 != 0.0) {
    double ct = z / r;
    b3 = beta3 * r0 * pow((double)A, 1.0 / 3.0) * sqrt(7.0 / (4.0 * M_PI)) *
         0.5 * (5 * ct * ct * ct - 3 * ct);
  }
  U[p] = -V0 * (1 + kappa * (A - 2 * Z) / ((double)A)) /
         (1 + exp((r - (locR + b3)) / diff));
  f[p] = kHbar * kHbar / (2.0 * kMass);
  gf[p] = gf[ns + p] = gf[2 * ns + p] = 0.0;
  double w[3] = {0, 0, 0};
  if (so && r > 1e-12) {
    double r2 = r * r;
    double t = (r - locR) / diff;
    double et = exp(t);
    double g0 = 1.0 / (r2 * sin(theta));
    g0 = g0 * sqrt(5.0 / (16.0 * M_PI)) * (-6.0 * sin(theta) * cos(theta));
    g0 = -g0 * x * z;
    double rg[3] = {R * beta * g0, 0.0, 0.0};
    double sc = (soV0 / diff) * pow(1 + et, -2) * et;
    double ls = -35.0 * pow(kHbar * 0.5 / kMass, 2);
    double gr[3] = {x / r, y / r, z / r};
    for (int q = 0; q < 3; ++q) w[q] = ls * sc * (gr[q] - rg[q]);
  }
  for (int q = 0; q < 3; ++q) W[q * ns + p] = w[q];
}

__global__ void cvt64to32(const double2 *in, float2 *out, size_t count) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < count) out[i] = make_float2((float)in[i].x, (float)in[i].y);
}
__global__ void cvt32to64(const float2 *in, double2 *out, size_t count) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i < count) out[i] = make_double2(in[i].x, in[i].y);
}

int *errWordImpl() {
  // thread-safe one-time allocation (concurrent contexts on host threads)
  static int *d = [] {
    int *p = nullptr;
    if (cudaMalloc(&p, sizeof(int)) == cudaSuccess)
      cudaMemset(p, 0, sizeof(int));
    return p;
  }();
  return d;
}

} // namespace

int *stencilErrWord() { return errWordImpl(); }

void convert64to32(const double2 *in, float2 *out, size_t count,
                   cudaStream_t s) {
  cvt64to32<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(in, out, count);
}
void convert32to64(const float2 *in, double2 *out, size_t count,
                   cudaStream_t s) {
  cvt32to64<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(in, out, count);
}

int buildCoefficients(ncgm_ctx *ctx, int species, const double *f,
                      const double *gradf, const double *U, const double *W,
                      const double *UC) {
  SpeciesFields &F = ctx->sp[species];
  if (!F.coef64) {
    NCGM_CUDA(cudaMalloc(&F.coef64, ctx->ns * 8 * sizeof(double)));
    NCGM_CUDA(cudaMalloc(&F.coef32, ctx->ns * 8 * sizeof(float)));
    NCGM_CUDA(cudaMalloc(&F.coef32s, ctx->ns * 8 * sizeof(float)));
  }
  buildCoefKernel<<<(unsigned)((ctx->ns + 255) / 256), 256, 0, ctx->stream>>>(
      f, gradf, U, W, UC, ctx->ns, ctx->h, F.coef64, F.coef32, F.coef32s);
  NCGM_CUDA(cudaGetLastError());
  F.ready = true;
  return NCGM_OK;
}

int buildWoodsSaxon(ncgm_ctx *ctx, int species, int A, int Z, double V0,
                    double r0, double diff, double kappa, double beta,
                    double beta3, double so_V0, int spin_orbit) {
  const size_t ns = ctx->ns;
  double *buf = static_cast<double *>(ctx->buf(0, ns * 8 * sizeof(double)));
  if (!buf) return NCGM_ERR_NOMEM;
  double *f = buf, *gf = buf + ns, *U = buf + 4 * ns, *W = buf + 5 * ns;
  wsFieldKernel<<<(unsigned)((ns + 127) / 128), 128, 0, ctx->stream>>>(
      ctx->n, ctx->a, ctx->h, A, Z, V0, r0, diff, kappa, beta, beta3, so_V0,
      spin_orbit, f, gf, U, W);
  NCGM_CUDA(cudaGetLastError());
  return buildCoefficients(ctx, species, f, gf, U, W, nullptr);
}

void applyH64(ncgm_ctx *ctx, int species, const double2 *X, double2 *Y,
              int ncols, double shift, cudaStream_t s) {
  dim3 grid((unsigned)((ctx->ns + 255) / 256), ncols);
  stencilPoint<double><<<grid, 256, 0, s>>>(
      reinterpret_cast<const double4_32a *>(X), reinterpret_cast<double4_32a *>(Y),
      reinterpret_cast<const double4_32a *>(ctx->sp[species].coef64), ctx->n,
      ctx->ns, shift);
}

int stencilErrorFlag() {
  int h = 0;
  cudaMemcpy(&h, errWordImpl(), sizeof(int), cudaMemcpyDeviceToHost);
  return h;
}

} // namespace ncgm
