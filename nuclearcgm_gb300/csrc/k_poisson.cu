// Coulomb direct potential by the Poisson equation, the device form of
// Wavefunction::coulombFieldPoisson (src/util/wavefunction.cpp:55-229):
//   L U = -4 pi e^2 rho_p - (boundary terms),
// L the 5-point (4th-order) Laplacian truncated at the box edge
// (LaplacianPotential, src/coulomb/laplacianp_potential.cpp:18-73), with a
// Dirichlet halo potential e^2 Z / r + e^2 (Y20 Q20 + 2 Y22 Q22) / r two
// layers deep. The halo is indexed i*dim*dim + j*dim + k while the
// right-hand side uses the same index expression, so the halo's x and z roles
// are swapped relative to the lattice; that is kept. The reference solves with
// BiCGSTAB to machine epsilon; L is symmetric negative definite, so the device
// uses conjugate gradients on -L to a relative residual of 1e-13 (warm start
// from the previous potential), which reaches the same solution to rounding.
#include "k_poisson.cuh"
#include "k_dense.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>

namespace ncgm {

namespace {

__device__ __forceinline__ double trapW(size_t p, int n) {
  const int i = (int)(p % n), j = (int)((p / n) % n), k = (int)(p / ((size_t)n * n));
  double w = 1.0;
  if (i == 0 || i == n - 1) w *= 0.5;
  if (j == 0 || j == n - 1) w *= 0.5;
  if (k == 0 || k == n - 1) w *= 0.5;
  return w;
}

__device__ double blockReduce(double v, double *sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  double r = sh[0];
  __syncthreads();
  return r;
}

// Q20 / Q22 integrals of rho_p (wavefunction.cpp:74-92), partials per block
__global__ void quadKernel(const double *rho, int n, double a, double h,
                           double *partials) {
  __shared__ double sh[256];
  const size_t ns = (size_t)n * n * n;
  const double hhh = h * h * h;
  double q20 = 0, q22 = 0;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < ns;
       p += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(p % n), j = (int)((p / n) % n), k = (int)(p / ((size_t)n * n));
    const double x = -a + i * h, y = -a + j * h, z = -a + k * h;
    const double w = trapW(p, n) * hhh;
    q20 += (rho[p] * (2.0 * z * z - x * x - y * y)) * sqrt(5.0 / (16.0 * M_PI)) * w;
    q22 += (rho[p] * (x * x - y * y)) * sqrt(15.0 / (32.0 * M_PI)) * w;
  }
  double s0 = blockReduce(q20, sh), s1 = blockReduce(q22, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = s0;
    partials[gridDim.x + blockIdx.x] = s1;
  }
}

// halo potential at halo index (a, b, c) of the (n+4)^3 box
__device__ __forceinline__ double haloV(int ia, int ib, int ic, double A,
                                        double h, double Z, double Q20,
                                        double Q22) {
  const double x = -A - 2 * h + ia * h, y = -A - 2 * h + ib * h,
               z = -A - 2 * h + ic * h;
  double r = sqrt(x * x + y * y + z * z);
  const double rr = r;
  if (r < 1e-9) r = 1e-9;
  const double theta = acos(z / rr);
  const double phi = atan2(y, x);
  const double y20 = sqrt(5.0 / (16.0 * M_PI)) * (3.0 * cos(theta) * cos(theta) - 1.0);
  const double y22 = sqrt(15.0 / (32.0 * M_PI)) * cos(2 * phi) * sin(theta) * sin(theta);
  double v = (kE2Poisson * Z) / r;
  v += kE2Poisson * (y20 * Q20 + 2.0 * y22 * Q22) / r;
  return v;
}

__global__ void rhsKernel(const double *rho, int n, double A, double h,
                          double Z, const double *q, double *rhs) {
  const size_t ns = (size_t)n * n * n;
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= ns) return;
  const double Q20 = q[0], Q22 = q[1];
  const double hh = h * h;
  const double eps0inv = kE2Poisson * 4 * M_PI;
  double v = -eps0inv * rho[e];
  // rhs index e = a n^2 + b n + c (the reference's face lambda)
  const int a = (int)(e / ((size_t)n * n)), b = (int)((e / n) % n),
            c = (int)(e % n);
  auto H = [&](int ia, int ib, int ic) {
    return haloV(ia, ib, ic, A, h, Z, Q20, Q22);
  };
  // faces in the reference's order: first, second, third lambda index
  if (a == 0) {
    v -= (16.0 / 12.0) * H(1, b + 2, c + 2) / hh;
    v += (1.0 / 12.0) * H(0, b + 2, c + 2) / hh;
  }
  if (a == 1) v += (1.0 / 12.0) * H(1, b + 2, c + 2) / hh;
  if (a == n - 1) {
    v -= (16.0 / 12.0) * H(n + 2, b + 2, c + 2) / hh;
    v += (1.0 / 12.0) * H(n + 3, b + 2, c + 2) / hh;
  }
  if (a == n - 2) v += (1.0 / 12.0) * H(n + 2, b + 2, c + 2) / hh;
  if (b == 0) {
    v -= (16.0 / 12.0) * H(a + 2, 1, c + 2) / hh;
    v += (1.0 / 12.0) * H(a + 2, 0, c + 2) / hh;
  }
  if (b == 1) v += (1.0 / 12.0) * H(a + 2, 1, c + 2) / hh;
  if (b == n - 1) {
    v -= (16.0 / 12.0) * H(a + 2, n + 2, c + 2) / hh;
    v += (1.0 / 12.0) * H(a + 2, n + 3, c + 2) / hh;
  }
  if (b == n - 2) v += (1.0 / 12.0) * H(a + 2, n + 2, c + 2) / hh;
  if (c == 0) {
    v -= (16.0 / 12.0) * H(a + 2, b + 2, 1) / hh;
    v += (1.0 / 12.0) * H(a + 2, b + 2, 0) / hh;
  }
  if (c == 1) v += (1.0 / 12.0) * H(a + 2, b + 2, 1) / hh;
  if (c == n - 1) {
    v -= (16.0 / 12.0) * H(a + 2, b + 2, n + 2) / hh;
    v += (1.0 / 12.0) * H(a + 2, b + 2, n + 3) / hh;
  }
  if (c == n - 2) v += (1.0 / 12.0) * H(a + 2, b + 2, n + 2) / hh;
  rhs[e] = v;
}

// y = -L x (positive definite form), partial sums of x.y
__global__ void negLapKernel(const double *x, double *y, int n, double h,
                             double *partials) {
  __shared__ double sh[256];
  const size_t ns = (size_t)n * n * n;
  const double hh = h * h;
  const double c0 = (90.0 / 12.0) / hh, c1 = -(16.0 / 12.0) / hh,
               c2 = (1.0 / 12.0) / hh;
  double acc = 0;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < ns;
       p += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(p % n), j = (int)((p / n) % n), k = (int)(p / ((size_t)n * n));
    const size_t sy = n, sz = (size_t)n * n;
    double s = c0 * x[p];
    if (i >= 1) s += c1 * x[p - 1];
    if (i >= 2) s += c2 * x[p - 2];
    if (i + 1 < n) s += c1 * x[p + 1];
    if (i + 2 < n) s += c2 * x[p + 2];
    if (j >= 1) s += c1 * x[p - sy];
    if (j >= 2) s += c2 * x[p - 2 * sy];
    if (j + 1 < n) s += c1 * x[p + sy];
    if (j + 2 < n) s += c2 * x[p + 2 * sy];
    if (k >= 1) s += c1 * x[p - sz];
    if (k >= 2) s += c2 * x[p - 2 * sz];
    if (k + 1 < n) s += c1 * x[p + sz];
    if (k + 2 < n) s += c2 * x[p + 2 * sz];
    y[p] = s;
    acc += x[p] * s;
  }
  double t = blockReduce(acc, sh);
  if (partials && threadIdx.x == 0) partials[blockIdx.x] = t;
}

// r = b - (-L) U from y = -L U ; partials |r|^2, |b|^2 ; p = r
__global__ void cgInitKernel(const double *rhs, const double *y, double *r,
                             double *p, size_t ns, double *partials) {
  __shared__ double sh[256];
  double rr = 0, bb = 0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < ns;
       e += (size_t)gridDim.x * blockDim.x) {
    const double b = -rhs[e];
    const double v = b - y[e];
    r[e] = v;
    p[e] = v;
    rr += v * v;
    bb += b * b;
  }
  double s0 = blockReduce(rr, sh), s1 = blockReduce(bb, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = s0;
    partials[gridDim.x + blockIdx.x] = s1;
  }
}

// scalars: s[0] = rr, s[1] = bb, s[2] = pAp, s[3] = done
__global__ void cgScalarInit(const double *partials, int nblk, double *s) {
  if (threadIdx.x) return;
  double rr = 0, bb = 0;
  for (int b = 0; b < nblk; ++b) {
    rr += partials[b];
    bb += partials[nblk + b];
  }
  s[0] = rr;
  s[1] = bb;
  s[3] = (bb == 0.0) ? 1.0 : 0.0;
}

// alpha = rr / pAp; x += alpha p; r -= alpha Ap; partial |r|^2
__global__ void cgUpdateKernel(double *x, double *r, const double *p,
                               const double *Ap, size_t ns,
                               const double *pApPartials, int nblk,
                               const double *s, double *partials) {
  __shared__ double sh[256];
  __shared__ double alpha;
  if (s[3] != 0.0) return;
  if (threadIdx.x == 0) {
    double pAp = 0;
    for (int b = 0; b < nblk; ++b) pAp += pApPartials[b];
    alpha = s[0] / pAp;
  }
  __syncthreads();
  const double al = alpha;
  double rr = 0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < ns;
       e += (size_t)gridDim.x * blockDim.x) {
    x[e] += al * p[e];
    const double v = r[e] - al * Ap[e];
    r[e] = v;
    rr += v * v;
  }
  double t = blockReduce(rr, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

// beta = rr_new / rr; p = r + beta p; s[0] = rr_new; done when below tol
__global__ void cgDirKernel(double *p, const double *r, size_t ns,
                            const double *partials, int nblk, double *s,
                            double tol2) {
  __shared__ double beta, rrn;
  if (s[3] != 0.0) return;
  if (threadIdx.x == 0) {
    double v = 0;
    for (int b = 0; b < nblk; ++b) v += partials[b];
    rrn = v;
    beta = v / s[0];
  }
  __syncthreads();
  const double bt = beta;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < ns;
       e += (size_t)gridDim.x * blockDim.x)
    p[e] = r[e] + bt * p[e];
  // Blocks of this launch still read s[0], so the new residual goes to s[4]
  // and cgCommit (the next launch) moves it into place.
  __syncthreads();
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    s[4] = rrn;
    s[5] = (rrn <= tol2 * s[1]) ? 1.0 : 0.0;
  }
}

__global__ void cgCommit(double *s) {
  if (threadIdx.x) return;
  if (s[3] != 0.0) return;
  s[0] = s[4];
  s[3] = s[5];
}

// One axis of the separable transform of the fast solver: out[p] =
// sum_t C[a][t] in[p with its axis-`axis` index a replaced by t], with C = W^T
// (forward) or W (inverse), W the eigenvectors of the 1-D operator (column j
// = eigenvector j, column-major, n x n). scaleD: divide by the eigenvalue sum
// (d_i + d_j + d_k) / h^2 (last forward pass); accum: out[p] += result (last
// inverse pass, into the potential) instead of out[p] = result.
__global__ void axisTransformKernel(const double *__restrict__ in,
                                    double *__restrict__ out,
                                    const double *__restrict__ Wd, int n,
                                    int axis, int inverse, int scaleD,
                                    double hh, int accum) {
  extern __shared__ double cs[]; // cs[t n + a] = C[a][t], then d (n)
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int t = e / n, a = e % n;
    cs[e] = inverse ? Wd[(size_t)t * n + a] : Wd[(size_t)a * n + t];
  }
  for (int e = threadIdx.x; e < n; e += blockDim.x) cs[n * n + e] = Wd[n * n + e];
  __syncthreads();
  const size_t ns = (size_t)n * n * n;
  const size_t stride = axis == 0 ? 1 : (axis == 1 ? (size_t)n : (size_t)n * n);
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < ns;
       p += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(p % n), j = (int)((p / n) % n),
              k = (int)(p / ((size_t)n * n));
    const int a = axis == 0 ? i : (axis == 1 ? j : k);
    const double *base = in + (p - (size_t)a * stride);
    double v = 0.0;
    for (int t = 0; t < n; ++t) v = fma(cs[t * n + a], base[(size_t)t * stride], v);
    if (scaleD) v /= (cs[n * n + i] + cs[n * n + j] + cs[n * n + k]) / hh;
    if (accum)
      out[p] += v;
    else
      out[p] = v;
  }
}

// 1-D operator of the fast solver at h = 1 as a Hermitian matrix for heig:
// 30/12 on the diagonal, -16/12 and 1/12 on the first and second
// off-diagonals, rows truncated at the ends (the Dirichlet truncation of -L)
__global__ void oneDimOperatorKernel(int n, double2 *T) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * n) return;
  const int r = e % n, c = e / n, d = r > c ? r - c : c - r;
  const double v = d == 0 ? 30.0 / 12.0
                          : (d == 1 ? -16.0 / 12.0 : (d == 2 ? 1.0 / 12.0 : 0.0));
  T[e] = make_double2(v, 0.0);
}
__global__ void realPartsKernel(const double2 *V, const double *w, int n,
                                double *Wd) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n * n) Wd[e] = V[e].x;
  if (e < n) Wd[n * n + e] = w[e];
}

__global__ void exchangeKernel(const double *rhoP, const double *Ud,
                               double *UC, size_t ns) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= ns) return;
  double v = 0.0;
  v -= kE2Poisson * pow(3.0 / M_PI, 1.0 / 3.0) * pow(rhoP[e], 1.0 / 3.0);
  UC[e] = Ud[e] + v;
}

} // namespace

// -L is the Kronecker sum T (+) T (+) T of one 1-D operator T / h^2 (the
// 13-point stencil truncated at the box edge on every axis), so with
// T = W D W^T (a one-off n x n eigenproblem per lattice size, kept per device)
// (-L)^-1 = (W (x) W (x) W) diag(h^2 / (d_i + d_j + d_k)) (W (x) W (x) W)^T:
// six passes of n x n products along the axes. It preconditions an iterative
// refinement x += M^-1 (b + L x) that reaches the 1e-13 residual in one or
// two steps; plain CG continues if it does not.
struct PoissonEigen {
  int dev, n;
  double *Wd; // device: W (n x n), then the n eigenvalues of T at h = 1
};
std::vector<PoissonEigen> g_peig;
std::mutex g_peigMutex;

// The dynamic shared-memory limit of axisTransformKernel is an attribute of
// each device: it is raised once on every device that runs the fast solver.
// False when it cannot be raised (the caller then solves with CG only).
std::vector<int> g_axisAttrDevs;
bool axisTransformReady() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  std::lock_guard<std::mutex> lock(g_peigMutex);
  for (int d : g_axisAttrDevs)
    if (d == dev) return true;
  if (cudaFuncSetAttribute(axisTransformKernel,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (80 * 80 + 80) * (int)sizeof(double)) !=
      cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  g_axisAttrDevs.push_back(dev);
  return true;
}

const double *poissonEigen(int n, cudaStream_t s) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(g_peigMutex);
  for (auto &e : g_peig)
    if (e.dev == dev && e.n == n) return e.Wd;
  if (n > 80) return nullptr; // the shared-memory tier of the eigensolver
  double *Wd = nullptr;
  char *tmp = nullptr;
  const size_t mat = (size_t)n * n * sizeof(double2);
  if (cudaMalloc(&Wd, ((size_t)n * n + n) * sizeof(double)) != cudaSuccess)
    return nullptr;
  if (cudaMalloc(&tmp, 3 * mat + n * sizeof(double) + 2 * n * sizeof(int) +
                           64) != cudaSuccess) {
    cudaFree(Wd);
    return nullptr;
  }
  double2 *T = reinterpret_cast<double2 *>(tmp), *work = T + (size_t)n * n,
          *V = work + (size_t)n * n;
  double *w = reinterpret_cast<double *>(V + (size_t)n * n);
  int *perm = reinterpret_cast<int *>(w + n), *status = perm + n;
  oneDimOperatorKernel<<<(n * n + 127) / 128, 128, 0, s>>>(n, T);
  heig(T, n, n, work, V, w, perm, status, s);
  realPartsKernel<<<(n * n + 127) / 128, 128, 0, s>>>(V, w, n, Wd);
  int hs = 1;
  cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, s);
  const bool ok = cudaStreamSynchronize(s) == cudaSuccess && hs == 0;
  cudaFree(tmp);
  if (!ok) {
    cudaFree(Wd);
    return nullptr;
  }
  g_peig.push_back({dev, n, Wd});
  return Wd;
}

int poissonSolve(const PoissonArgs &P, cudaStream_t s, int *iterations) {
  const int n = P.n;
  const size_t ns = (size_t)n * n * n;
  const int nblk = 120;
  double *q = P.work;                 // 2
  double *sc = P.work + 8;            // 8 scalars
  double *part = P.work + 16;         // 2 * nblk
  double *part2 = part + 2 * nblk;    // nblk
  double *rhs = P.work + 16 + 4 * nblk;
  double *r = rhs + ns, *p = r + ns, *Ap = p + ns;
  quadKernel<<<nblk, 256, 0, s>>>(P.rhoP, n, P.a, P.h, part);
  // reduce Q20, Q22 (2 values)
  {
    std::vector<double> hp(2 * nblk);
    cudaMemcpyAsync(hp.data(), part, sizeof(double) * 2 * nblk,
                    cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return NCGM_ERR_CUDA;
    double qq[2] = {0, 0};
    for (int b = 0; b < nblk; ++b) {
      qq[0] += hp[b];
      qq[1] += hp[nblk + b];
    }
    cudaMemcpyAsync(q, qq, sizeof(double) * 2, cudaMemcpyHostToDevice, s);
  }
  rhsKernel<<<(unsigned)((ns + 255) / 256), 256, 0, s>>>(P.rhoP, n, P.a, P.h,
                                                          P.Z, q, rhs);
  if (!P.warm) cudaMemsetAsync(P.U, 0, ns * sizeof(double), s);
  negLapKernel<<<nblk, 256, 0, s>>>(P.U, Ap, n, P.h, nullptr);
  cgInitKernel<<<nblk, 256, 0, s>>>(rhs, Ap, r, p, ns, part);
  cgScalarInit<<<1, 32, 0, s>>>(part, nblk, sc);
  const double tol2 = P.tol * P.tol;
  int it = 0;
  const int maxit = std::max(100, (int)std::min<size_t>(4 * ns, 20000));
  // fast solver: refinement steps with the separable inverse (p and Ap serve
  // as the transform's temporaries); NCGM_POISSON_FAST=0 keeps plain CG
  const char *fenv = std::getenv("NCGM_POISSON_FAST");
  const double *Wd = (fenv && fenv[0] == '0') ? nullptr : poissonEigen(n, s);
  bool solved = false;
  if (Wd && axisTransformReady()) {
    const size_t smem = ((size_t)n * n + n) * sizeof(double);
    const double hh = P.h * P.h;
    for (int ref = 0; ref < 4; ++ref) {
      double hs2[2];
      cudaMemcpyAsync(hs2, sc, sizeof(double) * 2, cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return NCGM_ERR_CUDA;
      if (!std::isfinite(hs2[0])) return NCGM_ERR_NAN;
      if (hs2[1] == 0.0 || hs2[0] <= tol2 * hs2[1]) {
        solved = true;
        break;
      }
      axisTransformKernel<<<nblk, 256, smem, s>>>(r, p, Wd, n, 0, 0, 0, hh, 0);
      axisTransformKernel<<<nblk, 256, smem, s>>>(p, Ap, Wd, n, 1, 0, 0, hh, 0);
      axisTransformKernel<<<nblk, 256, smem, s>>>(Ap, p, Wd, n, 2, 0, 1, hh, 0);
      axisTransformKernel<<<nblk, 256, smem, s>>>(p, Ap, Wd, n, 0, 1, 0, hh, 0);
      axisTransformKernel<<<nblk, 256, smem, s>>>(Ap, p, Wd, n, 1, 1, 0, hh, 0);
      axisTransformKernel<<<nblk, 256, smem, s>>>(p, P.U, Wd, n, 2, 1, 0, hh, 1);
      // a failed launch leaves U as it was (all six passes share one
      // configuration): rebuild the residual from U and finish with CG
      const bool launched = cudaGetLastError() == cudaSuccess;
      negLapKernel<<<nblk, 256, 0, s>>>(P.U, Ap, n, P.h, nullptr);
      cgInitKernel<<<nblk, 256, 0, s>>>(rhs, Ap, r, p, ns, part);
      cgScalarInit<<<1, 32, 0, s>>>(part, nblk, sc);
      if (!launched) break;
      ++it;
    }
  }

  double hs[8];
  double best = 1e300;
  int sinceBest = 0;
  // a block of 16 CG iterations (64 launches with fixed arguments) is
  // captured once per solve into a CUDA graph and replayed; the host checks
  // convergence between blocks. NCGM_POISSON_GRAPH=0 keeps direct launches.
  auto block = [&]() {
    for (int b = 0; b < 16; ++b) {
      negLapKernel<<<nblk, 256, 0, s>>>(p, Ap, n, P.h, part2);
      cgUpdateKernel<<<nblk, 256, 0, s>>>(P.U, r, p, Ap, ns, part2, nblk, sc,
                                          part);
      cgDirKernel<<<nblk, 256, 0, s>>>(p, r, ns, part, nblk, sc, tol2);
      cgCommit<<<1, 32, 0, s>>>(sc);
    }
  };
  const char *genv = std::getenv("NCGM_POISSON_GRAPH");
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  if (!solved && !(genv && genv[0] == '0') &&
      cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) ==
          cudaSuccess) {
    block();
    if (cudaStreamEndCapture(s, &graph) != cudaSuccess ||
        cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess)
      exec = nullptr;
    cudaGetLastError();
  }
  struct GraphGuard {
    cudaGraph_t &g;
    cudaGraphExec_t &e;
    ~GraphGuard() {
      if (e) cudaGraphExecDestroy(e);
      if (g) cudaGraphDestroy(g);
    }
  } guard{graph, exec};
  for (; !solved && it < maxit;) {
    if (exec)
      cudaGraphLaunch(exec, s);
    else
      block();
    it += 16;
    cudaMemcpyAsync(hs, sc, sizeof(double) * 8, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return NCGM_ERR_CUDA;
    if (!std::isfinite(hs[0])) return NCGM_ERR_NAN;
    if (hs[3] != 0.0) break;
    // stagnation guard: rounding floor reached
    if (hs[0] < 0.5 * best) {
      best = hs[0];
      sinceBest = 0;
    } else if (++sinceBest > 8) {
      break;
    }
  }
  exchangeKernel<<<(unsigned)((ns + 255) / 256), 256, 0, s>>>(P.rhoP, P.U,
                                                               P.UC, ns);
  if (iterations) *iterations = it;
  return cudaGetLastError() == cudaSuccess ? NCGM_OK : NCGM_ERR_CUDA;
}

size_t poissonWorkDoubles(int n) {
  const size_t ns = (size_t)n * n * n;
  return 16 + 4 * 120 + 4 * ns + 64;
}

// ---------------------------------------------------------------------------
// Allocation-free variant. Its scratch (right-hand side, CG vectors and
// reduction partials) lives in this file-scope device array, sized for
// lattices up to NCGM_POISSON_NOALLOC_MAX_N points per axis; every GPU that
// loads the library holds it until the process exits. Host code never uses
// the symbol's host-side name as a device address: the address is looked up
// once per device with cudaGetSymbolAddress and handed to the kernels.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocMaxN = NCGM_POISSON_NOALLOC_MAX_N;
constexpr size_t kNoAllocDoubles =
    16 + 4 * 120 + 4 * kNoAllocMaxN * kNoAllocMaxN * kNoAllocMaxN + 64;
static __device__ __align__(256) double g_poissonScratch[kNoAllocDoubles];

constexpr int kMaxDevices = 64;
double *g_scratchAddr[kMaxDevices] = {nullptr};
std::mutex g_scratchMutex; // first calls on a device from several threads

// device address of the static scratch on the current device (set-up on the
// first call per device)
int staticScratch(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return NCGM_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return NCGM_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_scratchMutex);
  if (!g_scratchAddr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_poissonScratch);
    if (e != cudaSuccess || !p) return NCGM_ERR_CUDA;
    g_scratchAddr[dev] = static_cast<double *>(p);
  }
  *out = g_scratchAddr[dev];
  return NCGM_OK;
}

// The CG path of poissonSolve (the separable-inverse refinement, which needs
// the per-lattice eigenvectors in allocated memory, is not used), with the
// host-side reduction buffers on the stack instead of the heap. Both stop at
// the same 1e-13 relative residual, so their results agree to that level,
// not bit for bit.
int poissonSolveNoAlloc(const PoissonArgs &P, cudaStream_t s,
                        int *iterations) {
  const int n = P.n;
  const size_t ns = (size_t)n * n * n;
  constexpr int nblk = 120;
  double *q = P.work;
  double *sc = P.work + 8;
  double *part = P.work + 16;
  double *part2 = part + 2 * nblk;
  double *rhs = P.work + 16 + 4 * nblk;
  double *r = rhs + ns, *p = r + ns, *Ap = p + ns;
  quadKernel<<<nblk, 256, 0, s>>>(P.rhoP, n, P.a, P.h, part);
  double hp[2 * nblk];
  if (cudaMemcpyAsync(hp, part, sizeof(hp), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return NCGM_ERR_CUDA;
  double qq[2] = {0, 0};
  for (int b = 0; b < nblk; ++b) {
    qq[0] += hp[b];
    qq[1] += hp[nblk + b];
  }
  if (cudaMemcpyAsync(q, qq, sizeof(qq), cudaMemcpyHostToDevice, s) !=
      cudaSuccess)
    return NCGM_ERR_CUDA;
  rhsKernel<<<(unsigned)((ns + 255) / 256), 256, 0, s>>>(P.rhoP, n, P.a, P.h,
                                                          P.Z, q, rhs);
  negLapKernel<<<nblk, 256, 0, s>>>(P.U, Ap, n, P.h, nullptr);
  cgInitKernel<<<nblk, 256, 0, s>>>(rhs, Ap, r, p, ns, part);
  cgScalarInit<<<1, 32, 0, s>>>(part, nblk, sc);
  const double tol2 = P.tol * P.tol;
  int it = 0;
  const int maxit = std::max(100, (int)std::min<size_t>(4 * ns, 20000));
  double hs[8];
  double best = 1e300;
  int sinceBest = 0;
  for (; it < maxit;) {
    for (int b = 0; b < 16; ++b, ++it) {
      negLapKernel<<<nblk, 256, 0, s>>>(p, Ap, n, P.h, part2);
      cgUpdateKernel<<<nblk, 256, 0, s>>>(P.U, r, p, Ap, ns, part2, nblk, sc,
                                          part);
      cgDirKernel<<<nblk, 256, 0, s>>>(p, r, ns, part, nblk, sc, tol2);
      cgCommit<<<1, 32, 0, s>>>(sc);
    }
    if (cudaMemcpyAsync(hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return NCGM_ERR_CUDA;
    if (!std::isfinite(hs[0])) return NCGM_ERR_NAN;
    if (hs[3] != 0.0) break;
    if (hs[0] < 0.5 * best) {
      best = hs[0];
      sinceBest = 0;
    } else if (++sinceBest > 8) {
      break;
    }
  }
  if (P.UC)
    exchangeKernel<<<(unsigned)((ns + 255) / 256), 256, 0, s>>>(P.rhoP, P.U,
                                                                 P.UC, ns);
  if (iterations) *iterations = it;
  return cudaGetLastError() == cudaSuccess ? NCGM_OK : NCGM_ERR_CUDA;
}

bool onDevice(const void *p) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

} // namespace

void setError(const std::string &msg);

} // namespace ncgm

// Allocation-free Coulomb Poisson solve (see ncgm.h). For callers that cannot
// allocate device memory; the scratch is the static array above, shared by
// every call on a device, so calls that overlap on the GPU race.
extern "C" int ncgm_poisson_noalloc(int n, double a, const double *rhoP,
                                    int Z, const double *U_guess,
                                    double *U_out, double *UC_out,
                                    void *stream, int *iterations) {
  using namespace ncgm;
  if (n < 2 || !(a > 0) || !rhoP || !U_out) {
    setError("ncgm_poisson_noalloc: need n >= 2, a > 0, rhoP and U_out");
    return NCGM_ERR_ARG;
  }
  if ((size_t)n > kNoAllocMaxN) {
    setError("ncgm_poisson_noalloc: n = " + std::to_string(n) +
             " exceeds the static scratch limit of " +
             std::to_string(kNoAllocMaxN) + " points per axis");
    return NCGM_ERR_ARG;
  }
  if (!onDevice(rhoP) || !onDevice(U_out) || (UC_out && !onDevice(UC_out)) ||
      (U_guess && !onDevice(U_guess))) {
    setError("ncgm_poisson_noalloc: all buffers must be device memory");
    return NCGM_ERR_ARG;
  }
  double *scratch = nullptr;
  int st = staticScratch(&scratch);
  if (st != NCGM_OK) {
    setError("ncgm_poisson_noalloc: static scratch address lookup failed");
    return st;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t ns = (size_t)n * n * n;
  // the solver iterates in place on U_out: start from the guess or from zero
  if (U_guess && U_guess != U_out) {
    if (cudaMemcpyAsync(U_out, U_guess, ns * sizeof(double),
                        cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return NCGM_ERR_CUDA;
  } else if (!U_guess) {
    if (cudaMemsetAsync(U_out, 0, ns * sizeof(double), s) != cudaSuccess)
      return NCGM_ERR_CUDA;
  }
  PoissonArgs P;
  P.n = n;
  P.a = a;
  P.h = 2.0 * a / (n - 1);
  P.Z = Z;
  P.rhoP = rhoP;
  P.U = U_out;
  P.UC = UC_out;
  P.warm = 1;
  P.tol = 1e-13;
  P.work = scratch;
  st = poissonSolveNoAlloc(P, s, iterations);
  if (st != NCGM_OK) {
    setError("ncgm_poisson_noalloc: solve failed");
    return st;
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return NCGM_ERR_CUDA;
  return NCGM_OK;
}
