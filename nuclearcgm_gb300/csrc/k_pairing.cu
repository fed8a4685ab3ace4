// Pairing and guess kernels of the self-consistent loop:
//  * time reversal T psi = i sigma_y psi^* (Wavefunction::timeReverse,
//    src/util/wavefunction.cpp:554-580);
//  * BCS with state-dependent G_pq = V0 int rho_p rho_q (BCS::compute_G_pairing
//    and solveBCS, src/util/bcs.cpp:10-254): the density Gram on the lattice
//    and the gap/Fermi-level iteration in one CTA;
//  * HFB pairing field kappa(r) and pairing matrix Delta_ab
//    (kappa_field / delta_matrix, src/util/iteration_data.cpp:467-538) as
//    one N x nS product and one weighted Gram over the lattice points;
//  * spherical harmonic-oscillator spinor guess (harmonic_oscillator_guess,
//    src/solver/guess.cpp:10-248).
#include "k_pairing.cuh"
#include "k_dense.cuh"

#include <cfloat>
#include <cmath>

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

__global__ void timeReverseKernel(const double2 *X, double2 *Y, size_t ns,
                                  int ncols, size_t ld, int oddOnly) {
  const int c = blockIdx.y;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < ns;
       p += (size_t)gridDim.x * blockDim.x) {
    if (oddOnly) {
      // numericalTR (iteration_data.cpp:577-587): odd columns are the time
      // reverse of the preceding even column, even columns are copied
      const double2 *src = X + (size_t)(c % 2 ? c - 1 : c) * ld;
      double2 a = src[2 * p], b = src[2 * p + 1];
      if (c % 2) {
        Y[(size_t)c * ld + 2 * p] = make_double2(b.x, -b.y);
        Y[(size_t)c * ld + 2 * p + 1] = make_double2(-a.x, a.y);
      } else {
        Y[(size_t)c * ld + 2 * p] = a;
        Y[(size_t)c * ld + 2 * p + 1] = b;
      }
    } else {
      const double2 *src = X + (size_t)c * ld;
      double2 a = src[2 * p], b = src[2 * p + 1];
      // i sigma_y (a*, b*) = (b*, -a*)
      Y[(size_t)c * ld + 2 * p] = make_double2(b.x, -b.y);
      Y[(size_t)c * ld + 2 * p + 1] = make_double2(-a.x, a.y);
    }
  }
}

// G_pq = V0 int rho_p rho_q, rho_p = |phi_{cols[p]}|^2 ; one block per (p,q)
__global__ void densityGramKernel(const double2 *X, size_t ld, const int *cols,
                                  int np, int n, double h, double V0,
                                  double *G) {
  __shared__ double sh[256];
  const int p = blockIdx.x, q = blockIdx.y;
  const size_t ns = (size_t)n * n * n;
  const double2 *a = X + (size_t)cols[p] * ld, *b = X + (size_t)cols[q] * ld;
  const double hhh = h * h * h;
  double acc = 0;
  for (size_t e = threadIdx.x; e < ns; e += blockDim.x) {
    double2 a0 = a[2 * e], a1 = a[2 * e + 1], b0 = b[2 * e], b1 = b[2 * e + 1];
    double ra = (a0.x * a0.x + a0.y * a0.y) + (a1.x * a1.x + a1.y * a1.y);
    double rb = (b0.x * b0.x + b0.y * b0.y) + (b1.x * b1.x + b1.y * b1.y);
    acc += (ra * rb) * hhh * trapW(e, n);
  }
  double s = blockReduce(acc, sh);
  if (threadIdx.x == 0) G[(size_t)q * np + p] = V0 * s;
}

// solveBCS (bcs.cpp:107-254) in one CTA. Gp: np x np (already symmetrised
// 0.5 (G + G^T)); eps: pair energies. out: u2, v2, Delta (np each),
// scal[0] = lambda, scal[1] = Epair.
__global__ void bcsKernel(const double *eps, const double *Gp, int np, int A,
                          double window, int windowBoth, const double *oldDelta,
                          int useOld, double oldLambda, double *u2, double *v2,
                          double *Delta, double *scal, double *work) {
  __shared__ double sh[256];
  __shared__ double lam, raw, stop;
  const int tid = threadIdx.x, nt = blockDim.x;
  double *ww = work, *Eqp = work + np, *Dn = work + 2 * np, *D = Delta;
  const double ws = window / 10.0;
  const double EPS_SMALL = 1e-12;
  for (int p = tid; p < np; p += nt) D[p] = useOld ? oldDelta[p] : 1.0;
  if (tid == 0) {
    double l = oldLambda;
    if (!isfinite(l)) {
      int mid = (A / 2) - 1;
      mid = mid < 0 ? 0 : (mid > np - 1 ? np - 1 : mid);
      l = eps[mid];
    }
    lam = l;
  }
  __syncthreads();
  for (int iter = 0; iter < 2000; ++iter) {
    const double prev = lam;
    double s1 = 0, sI = 0;
    for (int p = tid; p < np; p += nt) {
      double w = 1.0 / (1.0 + exp((eps[p] - prev - window) / ws));
      if (windowBoth) w *= 1.0 / (1.0 + exp(-(eps[p] - prev + window) / ws));
      ww[p] = w;
      double xi = eps[p] - prev;
      double E = sqrt(xi * xi + D[p] * D[p] * w);
      Eqp[p] = E;
      s1 += (1.0 - eps[p] / E);
      sI += 1.0 / E;
    }
    s1 = blockReduce(s1, sh);
    sI = blockReduce(sI, sh);
    if (tid == 0) {
      raw = (sI < EPS_SMALL) ? prev : ((double)A - s1) / sI;
      lam = 0.9 * raw + (1.0 - 0.9) * prev;
    }
    __syncthreads();
    double dn = 0;
    for (int p = tid; p < np; p += nt) {
      double sum = 0;
      for (int q = 0; q < np; ++q)
        if (ww[q] > EPS_SMALL) sum += (0.5 * Gp[(size_t)q * np + p]) * ww[q] * D[q] / Eqp[q];
      Dn[p] = sum;
    }
    __syncthreads();
    for (int p = tid; p < np; p += nt) {
      double mixed = (1.0 - 0.9) * D[p] + 0.9 * Dn[p];
      dn += (mixed - D[p]) * (mixed - D[p]);
      Dn[p] = mixed;
    }
    dn = blockReduce(dn, sh);
    for (int p = tid; p < np; p += nt) D[p] = Dn[p];
    if (tid == 0) stop = (fabs(raw - prev) < 1e-10 && sqrt(dn) < 1e-10) ? 1 : 0;
    __syncthreads();
    if (stop) break;
  }
  const double l = lam;
  for (int p = tid; p < np; p += nt) {
    double w = 1.0 / (1.0 + exp((eps[p] - l - window) / ws));
    if (windowBoth) w *= 1.0 / (1.0 + exp(-(eps[p] - l + window) / ws));
    ww[p] = w;
    double xi = eps[p] - l;
    Eqp[p] = sqrt(xi * xi + D[p] * D[p] * w);
    double v = 0.5 * (1 - xi / Eqp[p]);
    v = fmin(fmax(v, 0.0), 1.0);
    v2[p] = v;
    u2[p] = 1 - v;
  }
  __syncthreads();
  double ep = 0;
  for (int p = tid; p < np; p += nt)
    for (int q = 0; q < np; ++q)
      if (ww[q] > EPS_SMALL)
        ep += -0.5 * ww[q] * ww[p] * D[p] * D[q] * (0.5 * Gp[(size_t)q * np + p]) /
              Eqp[p] / Eqp[q];
  ep = blockReduce(ep, sh);
  if (tid == 0) {
    scal[0] = l;
    scal[1] = ep;
  }
}

// C (nS x nS, complex, col-major) = Kff^T: column a of Q = Phi C is
// sum_b K_ab phi_b (Kff already carries f_a f_b)
__global__ void kffTransposeKernel(const double *Kff, int nS, double2 *C) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nS * nS) return;
  const int b = e % nS, a = e / nS; // C(b, a) = K(a, b) = Kff[b nS + a]
  C[e] = make_double2(Kff[(size_t)b * nS + a], 0.0);
}

// kappa(r) = sum_a Re(phi_a(r,1) Q_a(r,0) - phi_a(r,0) Q_a(r,1)), the
// reference's double sum over (a, b) with the b sum done by the product
// Q = Phi Kff^T; consecutive threads take consecutive points
__global__ void kappaReduceKernel(const double2 *Phi, size_t ld,
                                  const double2 *Q, size_t ldq, int nS,
                                  size_t ns, double *kappa) {
  const size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (p >= ns) return;
  double acc = 0;
  for (int a = 0; a < nS; ++a) {
    const double2 a0 = Phi[(size_t)a * ld + 2 * p],
                  a1 = Phi[(size_t)a * ld + 2 * p + 1];
    const double2 q0 = Q[(size_t)a * ldq + 2 * p],
                  q1 = Q[(size_t)a * ldq + 2 * p + 1];
    acc += (a1.x * q0.x - a1.y * q0.y) - (a0.x * q1.x - a0.y * q1.y);
  }
  kappa[p] = acc;
}

// The two spin planes of the Delta Gram: A0 = conj(phi(r, 0)) and
// B1 = h^3 w(r) kappa(r) phi(r, 1), ns x nS each (ld ns), so that
// (A0^H B1)_ab = int phi_a(r,0) kappa(r) phi_b(r,1)
__global__ void deltaOperandsKernel(const double2 *Phi, size_t ld, int nS,
                                    const double *kappa, int n, double h,
                                    double2 *A0, double2 *B1) {
  const size_t ns = (size_t)n * n * n;
  const size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const int a = blockIdx.y;
  if (p >= ns || a >= nS) return;
  const double2 v0 = Phi[(size_t)a * ld + 2 * p],
                v1 = Phi[(size_t)a * ld + 2 * p + 1];
  const double d = kappa[p] * h * h * h * trapW(p, n);
  A0[(size_t)a * ns + p] = make_double2(v0.x, -v0.y);
  B1[(size_t)a * ns + p] = make_double2(d * v1.x, d * v1.y);
}

// Delta_ab = 0.5 V0 f_a f_b Re int (phi_a(0) phi_b(1) - phi_a(1) phi_b(0))
// kappa = 0.5 V0 f_a f_b Re(G_ab - G_ba) with G = A0^H B1 (antisymmetric,
// zero diagonal)
__global__ void deltaFromGramKernel(const double2 *G, int nS, const double *ff,
                                    double V0, double *Delta) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nS * nS) return;
  const int a = e % nS, b = e / nS;
  Delta[e] = a == b ? 0.0
                    : 0.5 * V0 * ff[a] * ff[b] *
                          (G[(size_t)b * nS + a].x - G[(size_t)a * nS + b].x);
}

// --- HFB quasiparticle step (iteration_data.cpp:605-850) on the device ----
// Matrices are col-major; M x M state matrices (U, V, kappa) index the whole
// basis, nS x nS window matrices the states start .. start + nS - 1.

// Kff(a, b) = kappa(start + a, start + b) f_a f_b
__global__ void hfbKffKernel(const double *kappa, int M, int start, int nS,
                             const double *ff, double *Kff) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nS * nS) return;
  const int a = e % nS, b = e / nS;
  Kff[e] = kappa[(size_t)(start + b) * M + start + a] * ff[a] * ff[b];
}

// out[0] = sum of squares of the nS x nS entries (one block)
__global__ void hfbNorm2Kernel(const double *D, int nS, double *out) {
  __shared__ double sh[256];
  double acc = 0;
  for (int e = threadIdx.x; e < nS * nS; e += blockDim.x) acc += D[e] * D[e];
  acc = blockReduce(acc, sh);
  if (threadIdx.x == 0) out[0] = acc;
}

// H = [[e - lambda, Delta], [-Delta, -(e - lambda)]] (2nS x 2nS, complex
// storage of the real symmetric matrix)
__global__ void hfbMatrixKernel(const double *e, const double *Delta, int nS,
                                double lambda, double2 *H) {
  const int m2 = 2 * nS;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= m2 * m2) return;
  const int i = idx % m2, j = idx / m2;
  double v = 0.0;
  if (i < nS && j < nS) {
    if (i == j) v = e[i] - lambda;
  } else if (i >= nS && j >= nS) {
    if (i == j) v = -(e[i - nS] - lambda);
  } else if (i < nS) {
    v = Delta[(size_t)(j - nS) * nS + i];
  } else {
    v = -Delta[(size_t)j * nS + (i - nS)];
  }
  H[idx] = make_double2(v, 0.0);
}

// The positive-energy half of the eigenvectors (ascending eigenvalues:
// columns nS .. 2nS-1): U = upper block, V = lower block, and
// num[0] = sum V^2 (NaN when the eigensolver reported failure). One block.
__global__ void hfbExtractKernel(const double2 *Ev, int nS, const int *status,
                                 double *Uw, double *Vw, double *num) {
  __shared__ double sh[256];
  const int m2 = 2 * nS;
  double acc = 0;
  for (int e = threadIdx.x; e < nS * nS; e += blockDim.x) {
    const int i = e % nS, k = e / nS;
    const double u = Ev[(size_t)(k + nS) * m2 + i].x,
                 v = Ev[(size_t)(k + nS) * m2 + nS + i].x;
    Uw[e] = u;
    Vw[e] = v;
    acc += v * v;
  }
  acc = blockReduce(acc, sh);
  if (threadIdx.x == 0) num[0] = (*status != 0) ? nan("") : acc;
}

// U, V on the whole basis: the window blocks, V = 1 below the window and
// U = 1 above it (iteration_data.cpp: the padded amplitude matrices)
__global__ void hfbPadKernel(const double *Uw, const double *Vw, int nS,
                             int start, int M, double *U, double *V) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= M * M) return;
  const int r = idx % M, c = idx / M;
  const int end = start + nS - 1;
  double u = 0.0, v = 0.0;
  if (r >= start && r <= end && c >= start && c <= end) {
    const size_t w = (size_t)(c - start) * nS + (r - start);
    u = Uw[w];
    v = Vw[w];
  } else if (r == c) {
    if (r < start) v = 1.0;
    if (r > end) u = 1.0;
  }
  U[idx] = u;
  V[idx] = v;
}

// kappa = U V^T (M x M)
__global__ void hfbKappaKernel(const double *U, const double *V, int M,
                               double *kappa) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= M * M) return;
  const int i = idx % M, j = idx / M;
  double acc = 0;
  for (int k = 0; k < M; ++k)
    acc += U[(size_t)k * M + i] * V[(size_t)k * M + j];
  kappa[idx] = acc;
}

// pe[0] = 0.5 sum_ij Delta(i, j) (V U^T)(i, j) over the window, where
// (V U^T)(i, j) = kappa(start + j, start + i). One block.
__global__ void hfbPairEnergyKernel(const double *Delta, const double *kappa,
                                    int M, int start, int nS, double *pe) {
  __shared__ double sh[256];
  double acc = 0;
  for (int e = threadIdx.x; e < nS * nS; e += blockDim.x) {
    const int i = e % nS, j = e / nS;
    acc += Delta[e] * kappa[(size_t)(start + i) * M + start + j];
  }
  acc = blockReduce(acc, sh);
  if (threadIdx.x == 0) pe[0] = 0.5 * acc;
}

// U = 0, V = 1 on the first `target` states, kappa = 0 (the unpaired
// amplitudes)
__global__ void hfbNullKernel(int M, int target, double *U, double *V,
                              double *kappa) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= M * M) return;
  const int r = idx % M, c = idx / M;
  U[idx] = 0.0;
  kappa[idx] = 0.0;
  V[idx] = (r == c && r < target) ? 1.0 : 0.0;
}

// rho = V V^T (complex storage for the Hermitian eigensolver)
__global__ void hfbDensityMatrixKernel(const double *V, int M, double2 *rho) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= M * M) return;
  const int i = idx % M, j = idx / M;
  double acc = 0;
  for (int k = 0; k < M; ++k)
    acc += V[(size_t)k * M + i] * V[(size_t)k * M + j];
  rho[idx] = make_double2(acc, 0.0);
}

// T = W diag(sqrt(w)) with occupations below 1e-12 set to zero (the natural
// orbitals weighted by their occupation, iteration_data.cpp:326-338)
__global__ void hfbNaturalKernel(const double2 *W, const double *w, int M,
                                 double2 *T) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= M * M) return;
  const int j = idx / M;
  const double x = w[j] < 1e-12 ? 0.0 : w[j];
  const double sq = sqrt(x);
  T[idx] = make_double2(W[idx].x * sq, W[idx].y * sq);
}

// spherical HO spinor (nr, l, j2, mj2) on the lattice, unnormalised
struct Orb {
  int nr, l, j2, mj2;
};
__device__ double factorialD(int n) {
  double r = 1.0;
  for (int i = 2; i <= n; i++) r *= i;
  return r;
}
__device__ double assocLegendre(int l, int m, double x) {
  double pmm = 1.0;
  if (m > 0) {
    double fact = 1.0;
    for (int i = 1; i <= 2 * m - 1; i += 2) fact *= i;
    pmm = fact * pow(1.0 - x * x, m / 2.0);
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
__device__ double2 ylm(int l, int m, double theta, double phi) {
  int mm = abs(m);
  double norm = sqrt(((2.0 * l + 1.0) / (4.0 * M_PI)) *
                     (factorialD(l - mm) / factorialD(l + mm)));
  double leg = assocLegendre(l, mm, cos(theta));
  double sg = (mm % 2) ? -1.0 : 1.0;
  double re = sg * norm * leg * cos(mm * phi), im = sg * norm * leg * sin(mm * phi);
  if (m < 0) return make_double2(sg * re, -sg * im);
  return make_double2(re, im);
}
__device__ double laguerre(int n, double alpha, double x) {
  if (n == 0) return 1.0;
  if (n == 1) return 1.0 + alpha - x;
  double Lm2 = 1.0, Lm1 = 1.0 + alpha - x, L = 0.0;
  for (int k = 2; k <= n; ++k) {
    L = ((2.0 * k - 1.0 + alpha - x) * Lm1 - (k - 1.0 + alpha) * Lm2) / k;
    Lm2 = Lm1;
    Lm1 = L;
  }
  return L;
}

__global__ void hoGuessKernel(const int4 *orbs, int nev, int n, double a,
                              double h, double b, double2 *X, size_t ld) {
  const size_t ns = (size_t)n * n * n;
  const int c = blockIdx.y;
  const int4 o = orbs[c];
  const int nr = o.x, l = o.y, j2 = o.z, mj2 = o.w;
  const double mj = mj2 * 0.5, denom = 2.0 * l + 1.0;
  double Cu, Cd;
  if (j2 == 2 * l + 1) {
    Cu = sqrt((l + mj + 0.5) / denom);
    Cd = sqrt((l - mj + 0.5) / denom);
  } else {
    Cu = sqrt((l - mj + 0.5) / denom);
    Cd = -sqrt((l + mj - 0.5) / denom);
  }
  const int mlu = (mj2 - 1) / 2, mld = (mj2 + 1) / 2;
  const bool hu = abs(mlu) <= l, hd = abs(mld) <= l;
  const double norm = sqrt(2.0 * tgamma(nr + 1.0) /
                           (b * b * b * tgamma(nr + l + 1.5)));
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < ns;
       p += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(p % n), jg = (int)((p / n) % n), k = (int)(p / ((size_t)n * n));
    const double x = -a + i * h, y = -a + jg * h, z = -a + k * h;
    const double r = sqrt(x * x + y * y + z * z);
    const double theta = (r > 1e-12) ? acos(z / r) : 0.0;
    const double phi = atan2(y, x);
    const double rho = r / b;
    const double R = norm * pow(rho, l) * laguerre(nr, l + 0.5, rho * rho) *
                     exp(-0.5 * rho * rho);
    double2 up = make_double2(0, 0), dn = make_double2(0, 0);
    if (hu) {
      double2 y = ylm(l, mlu, theta, phi);
      up = make_double2(Cu * R * y.x, Cu * R * y.y);
    }
    if (hd) {
      double2 y = ylm(l, mld, theta, phi);
      dn = make_double2(Cd * R * y.x, Cd * R * y.y);
    }
    X[(size_t)c * ld + 2 * p] = up;
    X[(size_t)c * ld + 2 * p + 1] = dn;
  }
}

__global__ void colNorm2Kernel(const double2 *X, size_t ld, size_t N,
                               double *out) {
  __shared__ double sh[256];
  const int c = blockIdx.x;
  double a = 0;
  for (size_t e = threadIdx.x; e < N; e += blockDim.x) {
    double2 v = X[(size_t)c * ld + e];
    a += v.x * v.x + v.y * v.y;
  }
  double s = blockReduce(a, sh);
  if (threadIdx.x == 0) out[c] = s;
}

__global__ void scaleColsKernel(double2 *X, size_t ld, size_t N,
                                const double *norm2) {
  const int c = blockIdx.y;
  const double n2 = norm2[c];
  if (!(n2 > 0.0)) return; // Eigen normalize() leaves a zero column alone
  const double s = sqrt(n2);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N;
       e += (size_t)gridDim.x * blockDim.x) {
    double2 v = X[(size_t)c * ld + e];
    X[(size_t)c * ld + e] = make_double2(v.x / s, v.y / s);
  }
}

} // namespace

void timeReverse(const double2 *X, double2 *Y, size_t ns, int ncols, size_t ld,
                 bool oddOnly, cudaStream_t s) {
  if (ncols <= 0) return;
  dim3 grid((unsigned)std::min<size_t>(512, (ns + 255) / 256), ncols);
  timeReverseKernel<<<grid, 256, 0, s>>>(X, Y, ns, ncols, ld, oddOnly ? 1 : 0);
}

void densityGram(const double2 *X, size_t ld, const int *cols, int np, int n,
                 double h, double V0, double *G, cudaStream_t s) {
  if (np <= 0) return;
  dim3 grid(np, np);
  densityGramKernel<<<grid, 256, 0, s>>>(X, ld, cols, np, n, h, V0, G);
}

void bcsSolve(const double *eps, const double *Gp, int np, int A,
              double window, int windowBoth, const double *oldDelta,
              bool useOld, double oldLambda, double *u2, double *v2,
              double *Delta, double *scal, double *work, cudaStream_t s) {
  bcsKernel<<<1, 256, 0, s>>>(eps, Gp, np, A, window, windowBoth, oldDelta,
                              useOld ? 1 : 0, oldLambda, u2, v2, Delta, scal,
                              work);
}

void kappaFieldGemm(const double2 *Phi, size_t ld, int nS, const double *Kff,
                    size_t ns, double *kappa, double2 *Q, double2 *C,
                    const PairingGemm &g, cudaStream_t s) {
  if (nS <= 0) return;
  const size_t N = 2 * ns;
  kffTransposeKernel<<<(nS * nS + 255) / 256, 256, 0, s>>>(Kff, nS, C);
  if (g.exactScratch)
    gemmVCExact(Phi, ld, nS, C, nS, nS, Q, N, N, g.exactScratch, s);
  else
    gemmVC(Phi, ld, nS, C, nS, nS, Q, N, N, 0.0, s);
  kappaReduceKernel<<<(unsigned)((ns + 255) / 256), 256, 0, s>>>(
      Phi, ld, Q, N, nS, ns, kappa);
}

void deltaMatrixGemm(const double2 *Phi, size_t ld, int nS, const double *ff,
                     const double *kappa, int n, double h, double V0,
                     double *Delta, double2 *work, double2 *G,
                     const PairingGemm &g, cudaStream_t s) {
  if (nS <= 0) return;
  const size_t ns = (size_t)n * n * n;
  double2 *A0 = work, *B1 = work + ns * nS;
  dim3 grid((unsigned)((ns + 255) / 256), nS);
  deltaOperandsKernel<<<grid, 256, 0, s>>>(Phi, ld, nS, kappa, n, h, A0, B1);
  if (g.exactScratch)
    gramTCExact(A0, ns, nS, B1, ns, nS, ns, G, nS,
                static_cast<double *>(g.exactScratch), s);
  else
    gram(A0, ns, nS, B1, ns, nS, ns, G, nS, g.partials, g.maxChunks, s);
  deltaFromGramKernel<<<(nS * nS + 255) / 256, 256, 0, s>>>(G, nS, ff, V0,
                                                           Delta);
}

namespace {
inline unsigned blocksFor(size_t n) { return (unsigned)((n + 255) / 256); }
} // namespace

void hfbKff(const double *kappa, int M, int start, int nS, const double *ff,
            double *Kff, cudaStream_t s) {
  if (nS <= 0) return;
  hfbKffKernel<<<blocksFor((size_t)nS * nS), 256, 0, s>>>(kappa, M, start, nS,
                                                          ff, Kff);
}

void hfbNorm2(const double *D, int nS, double *out, cudaStream_t s) {
  hfbNorm2Kernel<<<1, 256, 0, s>>>(D, nS, out);
}

void hfbMatrix(const double *e, const double *Delta, int nS, double lambda,
               double2 *H, cudaStream_t s) {
  hfbMatrixKernel<<<blocksFor(4 * (size_t)nS * nS), 256, 0, s>>>(
      e, Delta, nS, lambda, H);
}

void hfbExtract(const double2 *Ev, int nS, const int *status, double *Uw,
                double *Vw, double *num, cudaStream_t s) {
  hfbExtractKernel<<<1, 256, 0, s>>>(Ev, nS, status, Uw, Vw, num);
}

void hfbAmplitudes(const double *Uw, const double *Vw, int nS, int start,
                   int M, double *U, double *V, double *kappa,
                   cudaStream_t s) {
  const unsigned b = blocksFor((size_t)M * M);
  hfbPadKernel<<<b, 256, 0, s>>>(Uw, Vw, nS, start, M, U, V);
  hfbKappaKernel<<<b, 256, 0, s>>>(U, V, M, kappa);
}

void hfbPairEnergy(const double *Delta, const double *kappa, int M, int start,
                   int nS, double *pe, cudaStream_t s) {
  hfbPairEnergyKernel<<<1, 256, 0, s>>>(Delta, kappa, M, start, nS, pe);
}

void hfbNull(int M, int target, double *U, double *V, double *kappa,
             cudaStream_t s) {
  hfbNullKernel<<<blocksFor((size_t)M * M), 256, 0, s>>>(M, target, U, V,
                                                         kappa);
}

void hfbDensityMatrix(const double *V, int M, double2 *rho, cudaStream_t s) {
  hfbDensityMatrixKernel<<<blocksFor((size_t)M * M), 256, 0, s>>>(V, M, rho);
}

void hfbNatural(const double2 *W, const double *w, int M, double2 *T,
                cudaStream_t s) {
  hfbNaturalKernel<<<blocksFor((size_t)M * M), 256, 0, s>>>(W, w, M, T);
}

void hoGuess(const int4 *orbs, int nev, int n, double a, double h, double b,
             double2 *X, size_t ld, double *work, cudaStream_t s) {
  const size_t ns = (size_t)n * n * n;
  dim3 grid((unsigned)std::min<size_t>(256, (ns + 127) / 128), nev);
  hoGuessKernel<<<grid, 128, 0, s>>>(orbs, nev, n, a, h, b, X, ld);
  normalizeEuclid(X, ld, 2 * ns, nev, work, s);
}

void normalizeEuclid(double2 *X, size_t ld, size_t N, int ncols, double *work,
                     cudaStream_t s) {
  if (ncols <= 0) return;
  colNorm2Kernel<<<ncols, 256, 0, s>>>(X, ld, N, work);
  dim3 grid((unsigned)std::min<size_t>(512, (N + 255) / 256), ncols);
  scaleColsKernel<<<grid, 256, 0, s>>>(X, ld, N, work);
}

} // namespace ncgm
