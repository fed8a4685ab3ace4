// Hermitian eigensolver for projected problems above the shared-memory
// tier (m > 80): the GCG's Rayleigh-Ritz matrices (m = 3 nev, up to 480 at
// 160 states) and the HFB matrices. The one-CTA Jacobi runs those from
// global memory on one SM's FP64 pipe (2 FMAs per clock on GB300): seconds
// at m = 480. Here the work is spread over the whole GPU, in the order of
// the classical dense method (the reference's Eigen SelfAdjointEigenSolver
// is also tridiagonalisation based):
//  1. Householder tridiagonalisation of the full Hermitian matrix, one step
//     per column: the reflector (one block), the matrix-vector product
//     p = tau A22 v split over row blocks and column chunks, w = p - tau/2
//     (p^H v) v, and the rank-2 update A22 -= v w^H + w v^H over the whole
//     grid. Reflectors H = I - tau v v^H with real beta (the LAPACK
//     convention), so the tridiagonal matrix is real.
//  2. Eigenvalues of the real tridiagonal by multisection on Sturm counts,
//     one warp per eigenvalue.
//  3. Eigenvectors by inverse iteration (tridiagonal LU with partial
//     pivoting, three solves from a hashed start vector), then modified
//     Gram-Schmidt inside clusters of equal eigenvalues (Kramers pairs are
//     exactly degenerate).
//  4. Back-transformation X = H_0 ... H_{m-2} Z, one reflector at a time.
// A numpy restatement of these steps gives eigenvalues to 2e-15 and
// orthonormality to 7e-13 relative, also with twofold degenerate spectra.
#include "k_dense.cuh"
#include "df64.cuh"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstdint>

namespace ncgm {

namespace {

constexpr int kT = 256;
constexpr int kJC = 32; // column chunks of the matrix-vector product

__device__ __forceinline__ double2 cmulD(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconjmulD(double2 a, double2 b) {
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ double blockSumD(double v, double *sh) {
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

// full Hermitian copy from the lower triangle of Ain
__global__ void fullCopyKernel(const double2 *Ain, int lda, int m,
                               double2 *A) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m * m) return;
  const int i = e % m, j = e / m;
  double2 v;
  if (i > j) v = Ain[(size_t)j * lda + i];
  else if (i < j) {
    const double2 l = Ain[(size_t)i * lda + j];
    v = make_double2(l.x, -l.y);
  } else v = make_double2(Ain[(size_t)j * lda + i].x, 0.0);
  A[e] = v;
}

// step k: reflector of x = A[k+1:, k] into Vr[:, k], tau[k], d[k], e[k]
__global__ void hhVectorKernel(const double2 *A, int m, int k, double2 *Vr,
                               double2 *tau, double *d, double *e) {
  __shared__ double sh[kT];
  __shared__ double2 sc;   // 1 / (alpha - beta)
  __shared__ int skip;
  const int L = m - k - 1;
  const double2 *x = A + (size_t)k * m + k + 1;
  double loc = 0;
  for (int i = 1 + threadIdx.x; i < L; i += blockDim.x)
    loc += x[i].x * x[i].x + x[i].y * x[i].y;
  const double xn2 = blockSumD(loc, sh);
  if (threadIdx.x == 0) {
    const double2 al = x[0];
    d[k] = A[(size_t)k * m + k].x;
    if (xn2 == 0.0 && al.y == 0.0) {
      tau[k] = make_double2(0.0, 0.0);
      e[k] = al.x;
      skip = 1;
    } else {
      const double beta =
          -(al.x >= 0.0 ? 1.0 : -1.0) * sqrt(al.x * al.x + al.y * al.y + xn2);
      tau[k] = make_double2((beta - al.x) / beta, -al.y / beta);
      e[k] = beta;
      // 1 / (alpha - beta)
      const double2 den = make_double2(al.x - beta, al.y);
      const double dd = den.x * den.x + den.y * den.y;
      sc = make_double2(den.x / dd, -den.y / dd);
      skip = 0;
    }
  }
  __syncthreads();
  double2 *v = Vr + (size_t)k * m;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    double2 r = make_double2(0.0, 0.0);
    if (!skip && i > k) r = (i == k + 1) ? make_double2(1.0, 0.0)
                                        : cmulD(x[i - k - 1], sc);
    v[i] = r;
  }
}

// partial products P[c][i] = sum_{j in chunk c} A22[i][j] v_j (rows k+1..)
__global__ void hhMatvecKernel(const double2 *A, int m, int k,
                               const double2 *Vr, double2 *P) {
  const int L = m - k - 1;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i >= L) return;
  const int per = (L + kJC - 1) / kJC;
  const int j0 = c * per, j1 = min(L, j0 + per);
  const double2 *v = Vr + (size_t)k * m + k + 1;
  double2 s = make_double2(0.0, 0.0);
  for (int j = j0; j < j1; ++j) {
    const double2 a = A[(size_t)(k + 1 + j) * m + (k + 1 + i)];
    const double2 t = cmulD(a, v[j]);
    s.x += t.x;
    s.y += t.y;
  }
  P[(size_t)c * m + i] = s;
}

// w = p - tau/2 (p^H v) v with p = tau sum_c P[c] (one block)
__global__ void hhWKernel(int m, int k, const double2 *P, const double2 *Vr,
                          const double2 *tau, double2 *Wv) {
  __shared__ double sh[kT];
  const int L = m - k - 1;
  const double2 t = tau[k];
  const double2 *v = Vr + (size_t)k * m + k + 1;
  double re = 0, im = 0;
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    double2 p = make_double2(0.0, 0.0);
    for (int c = 0; c < kJC; ++c) {
      p.x += P[(size_t)c * m + i].x;
      p.y += P[(size_t)c * m + i].y;
    }
    p = cmulD(t, p);
    Wv[i] = p;
    const double2 pv = cconjmulD(p, v[i]); // conj(p) v
    re += pv.x;
    im += pv.y;
  }
  re = blockSumD(re, sh);
  im = blockSumD(im, sh);
  // alpha2 = -1/2 tau (p^H v)
  const double2 a2 = cmulD(make_double2(-0.5 * t.x, -0.5 * t.y),
                           make_double2(re, im));
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    const double2 av = cmulD(a2, v[i]);
    Wv[i].x += av.x;
    Wv[i].y += av.y;
  }
}

// A22[i][j] -= v_i conj(w_j) + w_i conj(v_j)
__global__ void hhUpdateKernel(double2 *A, int m, int k, const double2 *Vr,
                               const double2 *Wv, const double2 *tau) {
  const double2 t = tau[k];
  if (t.x == 0.0 && t.y == 0.0) return;
  const int L = m - k - 1;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= L || j >= L) return;
  const double2 *v = Vr + (size_t)k * m + k + 1;
  const double2 a = cconjmulD(Wv[j], v[i]); // v_i conj(w_j)
  const double2 b = cconjmulD(v[j], Wv[i]); // w_i conj(v_j)
  double2 &x = A[(size_t)(k + 1 + j) * m + (k + 1 + i)];
  x.x -= a.x + b.x;
  x.y -= a.y + b.y;
}

__global__ void lastDiagKernel(const double2 *A, int m, double *d) {
  if (threadIdx.x == 0 && blockIdx.x == 0)
    d[m - 1] = A[(size_t)(m - 1) * m + (m - 1)].x;
}

// number of eigenvalues of the tridiagonal (d, e) below x (the quotient
// form of the Sturm sequence, with a pivot floor)
__device__ int sturmCount(const double *d, const double *e, int m, double x,
                          double pivmin) {
  double q = d[0] - x;
  int c = q < 0.0 ? 1 : 0;
  for (int i = 1; i < m; ++i) {
    if (fabs(q) < pivmin) q = -pivmin;
    q = d[i] - x - e[i - 1] * e[i - 1] / q;
    if (q < 0.0) ++c;
  }
  return c;
}

// eigenvalue j (ascending) by multisection from the Gershgorin bounds, one
// warp per eigenvalue: each step the 32 lanes count the eigenvalues below
// 32 equally spaced points of the bracket (Sturm counts), which shrinks it
// 33-fold, so about 11 steps reach the 2.3e-16 relative tolerance where
// bisection takes ~55
__global__ void multisectKernel(const double *d, const double *e, int m,
                                double *w) {
  const int j = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x % 32;
  if (j >= m) return;
  double lo = 1e300, hi = -1e300, emax = 0;
  for (int i = lane; i < m; i += 32) {
    double r = 0;
    if (i > 0) r += fabs(e[i - 1]);
    if (i + 1 < m) r += fabs(e[i]);
    lo = fmin(lo, d[i] - r);
    hi = fmax(hi, d[i] + r);
    if (i + 1 < m) emax = fmax(emax, fabs(e[i]));
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    emax = fmax(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  }
  const double scale = fmax(fabs(lo), fabs(hi));
  const double pivmin = fmax(1e-300, 2.3e-308 * fmax(1.0, emax * emax));
  const double tol = 2.3e-16 * scale;
  for (int it = 0; it < 64; ++it) {
    if (hi - lo <= 2.0 * tol) break;
    const double step = (hi - lo) / 33.0;
    const double x = lo + (lane + 1) * step;
    const bool below =
        x > lo && x < hi && sturmCount(d, e, m, x, pivmin) <= j;
    // the bracket is [x_k, x_{k+1}] for the last lane k whose point has at
    // most j eigenvalues below it (the counts grow with the lane)
    const unsigned mask = __ballot_sync(0xffffffffu, below);
    const int k = mask ? 31 - __clz(mask) : -1;
    const double nlo = k >= 0 ? lo + (k + 1) * step : lo;
    const double nhi = k < 31 ? lo + (k + 2) * step : hi;
    if (nlo == lo && nhi == hi) break; // no representable progress
    lo = nlo;
    hi = fmin(nhi, hi);
  }
  if (lane == 0) w[j] = 0.5 * (lo + hi);
}

__device__ __forceinline__ double hashUniform(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  x ^= x >> 31;
  return (double)(x >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// inverse iteration for eigenvalue j: three solves of (T - w_j) z = b with
// one LU factorisation with partial pivoting of the tridiagonal; column j of
// Z. The factors live in column j of the scratch arrays F (5 x m x m): the
// reciprocal pivots, the two upper diagonals of U, the multipliers and the
// row swaps. Divisions (slow on the FP64 pipe) are made once per row in the
// factorisation; the solves multiply.
__global__ void invIterKernel(const double *d, const double *e, int m,
                              const double *w, double *Z, double *F) {
  // one eigenvalue per block (its FP64 chain on an SM of its own)
  const int j = blockIdx.x;
  if (j >= m || threadIdx.x != 0) return;
  const size_t mm = (size_t)m * m;
  double *rb = F + (size_t)j * m, *c = F + mm + (size_t)j * m,
         *u2 = F + 2 * mm + (size_t)j * m, *l = F + 3 * mm + (size_t)j * m,
         *sw = F + 4 * mm + (size_t)j * m;
  double *z = Z + (size_t)j * m;
  double scale = 0;
  for (int i = 0; i < m; ++i) scale = fmax(scale, fabs(d[i]));
  for (int i = 0; i + 1 < m; ++i) scale = fmax(scale, fabs(e[i]));
  const double eps = 2.3e-16 * fmax(scale, 1e-300);
  const double lam = w[j];
  // factorisation: row i of U is (b0, c0, u0) after elimination
  {
    double b0 = d[0] - lam, c0 = m > 1 ? e[0] : 0.0, u0 = 0.0;
    for (int i = 0; i + 1 < m; ++i) {
      double a1 = e[i], b1 = d[i + 1] - lam, c1 = (i + 2 < m) ? e[i + 1] : 0.0;
      double u1 = 0.0;
      const bool swap = fabs(a1) > fabs(b0);
      if (swap) {
        double t;
        t = b0; b0 = a1; a1 = t;
        t = c0; c0 = b1; b1 = t;
        t = u0; u0 = c1; c1 = t;
      }
      if (b0 == 0.0) b0 = eps;
      const double li = a1 / b0;
      b1 -= li * c0;
      c1 -= li * u0;
      rb[i] = 1.0 / b0;
      c[i] = c0;
      u2[i] = u0;
      l[i] = li;
      sw[i] = swap ? 1.0 : 0.0;
      b0 = b1;
      c0 = c1;
      u0 = u1;
    }
    if (b0 == 0.0) b0 = eps;
    rb[m - 1] = 1.0 / b0;
  }
  for (int i = 0; i < m; ++i)
    z[i] = hashUniform(((uint64_t)j << 32) ^ (uint64_t)i);
  for (int rep = 0; rep < 3; ++rep) {
    // forward: the recorded swaps and multipliers on the right-hand side
    double y0 = z[0];
    for (int i = 0; i + 1 < m; ++i) {
      double y1 = z[i + 1];
      if (sw[i] != 0.0) {
        const double t = y0;
        y0 = y1;
        y1 = t;
      }
      z[i] = y0;
      y0 = y1 - l[i] * y0;
    }
    z[m - 1] = y0;
    // back substitution
    double nrm = 0;
    for (int i = m - 1; i >= 0; --i) {
      double sacc = z[i];
      if (i + 1 < m) sacc -= c[i] * z[i + 1];
      if (i + 2 < m) sacc -= u2[i] * z[i + 2];
      z[i] = sacc * rb[i];
      nrm += z[i] * z[i];
    }
    const double inv = 1.0 / sqrt(nrm);
    for (int i = 0; i < m; ++i) z[i] *= inv;
  }
}

// The same multisection with the Sturm counts in double-float arithmetic
// (heigMid): a quotient costs a few dependent FP32 operations where an FP64
// division takes ~600 cycles on GB300. The bracket stops at 2^-44 of the
// spectrum's scale (the double-float resolution), so the eigenvalues are good
// to about 1e-13 relative. d, e2: the diagonal and the squared off-diagonal
// in double-float (dfl), staged in shared memory.
constexpr int kDfSturmMax = 512;
__global__ void __launch_bounds__(32)
    multisectDfKernel(const double *d, const double *e, int m, double *w) {
  __shared__ dfl dd[kDfSturmMax], ee[kDfSturmMax];
  const int j = blockIdx.x, lane = threadIdx.x;
  if (j >= m) return;
  double lo = 1e300, hi = -1e300, emax = 0;
  for (int i = lane; i < m; i += 32) {
    double r = 0;
    if (i > 0) r += fabs(e[i - 1]);
    if (i + 1 < m) r += fabs(e[i]);
    lo = fmin(lo, d[i] - r);
    hi = fmax(hi, d[i] + r);
    dd[i] = dfFrom(d[i]);
    if (i + 1 < m) {
      emax = fmax(emax, fabs(e[i]));
      const dfl ei = dfFrom(e[i]);
      ee[i] = dfMul(ei, ei);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    emax = fmax(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  }
  __syncwarp();
  const double scale = fmax(fabs(lo), fabs(hi));
  const float pivmin = (float)fmax(1e-30, 5.7e-14 * fmax(1.0, emax * emax));
  const double tol = 5.7e-14 * scale;
  for (int it = 0; it < 64; ++it) {
    if (hi - lo <= 2.0 * tol) break;
    const double step = (hi - lo) / 33.0;
    const double x = lo + (lane + 1) * step;
    bool below = false;
    if (x > lo && x < hi) {
      const dfl xd = dfFrom(x);
      dfl q = dfSub(dd[0], xd);
      int c = q.hi < 0.f ? 1 : 0;
      for (int i = 1; i < m; ++i) {
        if (fabsf(q.hi) < pivmin) q = {-pivmin, 0.f};
        q = dfSub(dfSub(dd[i], xd), dfDiv(ee[i - 1], q));
        if (q.hi < 0.f) ++c;
      }
      below = c <= j;
    }
    const unsigned mask = __ballot_sync(0xffffffffu, below);
    const int k = mask ? 31 - __clz(mask) : -1;
    const double nlo = k >= 0 ? lo + (k + 1) * step : lo;
    const double nhi = k < 31 ? lo + (k + 2) * step : hi;
    if (nlo == lo && nhi == hi) break;
    lo = nlo;
    hi = fmin(nhi, hi);
  }
  if (lane == 0) w[j] = 0.5 * (lo + hi);
}

// modified Gram-Schmidt inside each cluster of equal eigenvalues (one block
// per cluster head)
__global__ void clusterMgsKernel(const double *w, int m, double *Z) {
  __shared__ double sh[kT];
  const int j = blockIdx.x;
  double scale = 0;
  for (int i = 0; i < m; ++i) scale = fmax(scale, fabs(w[i]));
  const double gap = 1e-8 * fmax(scale, 1e-300);
  if (j > 0 && w[j] - w[j - 1] <= gap) return; // not a cluster head
  int k = j + 1;
  while (k < m && w[k] - w[k - 1] <= gap) ++k;
  if (k == j + 1) return; // a single eigenvalue
  for (int a = j; a < k; ++a) {
    double *za = Z + (size_t)a * m;
    for (int b = j; b < a; ++b) {
      const double *zb = Z + (size_t)b * m;
      double loc = 0;
      for (int i = threadIdx.x; i < m; i += blockDim.x) loc += zb[i] * za[i];
      const double dot = blockSumD(loc, sh);
      for (int i = threadIdx.x; i < m; i += blockDim.x) za[i] -= dot * zb[i];
      __syncthreads();
    }
    double loc = 0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) loc += za[i] * za[i];
    const double inv = 1.0 / sqrt(blockSumD(loc, sh));
    for (int i = threadIdx.x; i < m; i += blockDim.x) za[i] *= inv;
    __syncthreads();
  }
}

// One-CTA tridiagonalisation for m <= kMidMax: the same reflectors as steps
// hhVector / hhMatvec / hhW / hhUpdate, with the full Hermitian matrix in
// shared memory and __syncthreads between the phases of a step, so the
// whole reduction is one launch instead of four per column. The
// matrix-vector product reads column i of A22 (contiguous in shared memory)
// and uses A22 v = conj(A22^H) v: the rank-2 updates keep A exactly
// Hermitian, element (j, i) being computed as the conjugate of (i, j) with
// the same roundings.
constexpr int kMidMax = 112; // 112^2 x 16 B = 196 KB of shared memory
constexpr int kMidT = 512;
__global__ void __launch_bounds__(kMidT, 1)
    hhTridiagSmemKernel(const double2 *Ain, int lda, int m, double2 *Vr,
                        double2 *tau, double *d, double *e) {
  extern __shared__ double2 Ash[];
  __shared__ double2 vs[kMidMax], ps[kMidMax];
  __shared__ double sh[kMidT];
  __shared__ double2 sc;
  __shared__ int skip;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int warp = tid / 32, lane = tid % 32, nw = nt / 32;
  for (int q = tid; q < m * m; q += nt) {
    const int i = q % m, j = q / m;
    double2 v;
    if (i > j) v = Ain[(size_t)j * lda + i];
    else if (i < j) {
      const double2 l = Ain[(size_t)i * lda + j];
      v = make_double2(l.x, -l.y);
    } else v = make_double2(Ain[(size_t)j * lda + i].x, 0.0);
    Ash[q] = v;
  }
  __syncthreads();
  for (int k = 0; k + 1 < m; ++k) {
    const int L = m - k - 1;
    const double2 *x = Ash + (size_t)k * m + k + 1;
    double loc = 0;
    for (int i = 1 + tid; i < L; i += nt)
      loc += x[i].x * x[i].x + x[i].y * x[i].y;
    const double xn2 = blockSumD(loc, sh);
    if (tid == 0) {
      const double2 al = x[0];
      d[k] = Ash[(size_t)k * m + k].x;
      if (xn2 == 0.0 && al.y == 0.0) {
        tau[k] = make_double2(0.0, 0.0);
        e[k] = al.x;
        skip = 1;
      } else {
        const double beta =
            -(al.x >= 0.0 ? 1.0 : -1.0) * sqrt(al.x * al.x + al.y * al.y + xn2);
        tau[k] = make_double2((beta - al.x) / beta, -al.y / beta);
        e[k] = beta;
        const double2 den = make_double2(al.x - beta, al.y);
        const double dd = den.x * den.x + den.y * den.y;
        sc = make_double2(den.x / dd, -den.y / dd);
        skip = 0;
      }
    }
    __syncthreads();
    const bool sk = skip != 0;
    const double2 t = tau[k]; // written by thread 0 before the barrier
    double2 *vg = Vr + (size_t)k * m;
    for (int i = tid; i < m; i += nt) {
      double2 r = make_double2(0.0, 0.0);
      if (!sk && i > k) r = (i == k + 1) ? make_double2(1.0, 0.0)
                                         : cmulD(x[i - k - 1], sc);
      vg[i] = r;
      if (i > k) vs[i - k - 1] = r;
    }
    __syncthreads();
    if (sk || L < 2) continue; // uniform: skip and L are shared
    // p = tau A22 v, one warp per row; A22[i][j] = conj(A22[j][i]) read
    // along column i
    for (int i = warp; i < L; i += nw) {
      const double2 *col = Ash + (size_t)(k + 1 + i) * m + k + 1;
      double re = 0, im = 0;
      for (int j = lane; j < L; j += 32) {
        const double2 a = col[j], v = vs[j]; // conj(a) v
        re += a.x * v.x + a.y * v.y;
        im += a.x * v.y - a.y * v.x;
      }
      for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
      }
      if (lane == 0) ps[i] = cmulD(t, make_double2(re, im));
    }
    __syncthreads();
    // w = p - tau/2 (p^H v) v
    double re = 0, im = 0;
    for (int i = tid; i < L; i += nt) {
      const double2 pv = cconjmulD(ps[i], vs[i]);
      re += pv.x;
      im += pv.y;
    }
    re = blockSumD(re, sh);
    im = blockSumD(im, sh);
    const double2 a2 =
        cmulD(make_double2(-0.5 * t.x, -0.5 * t.y), make_double2(re, im));
    for (int i = tid; i < L; i += nt) {
      const double2 av = cmulD(a2, vs[i]);
      ps[i].x += av.x;
      ps[i].y += av.y;
    }
    __syncthreads();
    // A22[i][j] -= v_i conj(w_j) + w_i conj(v_j)
    for (int q = tid; q < L * L; q += nt) {
      const int i = q % L, j = q / L;
      const double2 a = cconjmulD(ps[j], vs[i]);
      const double2 b = cconjmulD(vs[j], ps[i]);
      double2 &y = Ash[(size_t)(k + 1 + j) * m + (k + 1 + i)];
      y.x -= a.x + b.x;
      y.y -= a.y + b.y;
    }
    __syncthreads();
  }
  if (tid == 0) d[m - 1] = Ash[(size_t)(m - 1) * m + (m - 1)].x;
}

// sum over the block with two barriers: warp shuffles, then the warps'
// partial sums (red: 32 doubles per value)
__device__ __forceinline__ double2 blockSum2(double a, double b, double *red) {
  const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if (lane == 0) {
    red[warp] = a;
    red[32 + warp] = b;
  }
  __syncthreads();
  // one warp sums the warps' partials (FP64 work stays off the other 15
  // warps: the FP64 pipe retires 2 operations per clock per SM)
  if (warp == 0) {
    const int nw = blockDim.x / 32;
    double ra = lane < nw ? red[lane] : 0.0;
    double rb = lane < nw ? red[32 + lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      ra += __shfl_xor_sync(0xffffffffu, ra, o);
      rb += __shfl_xor_sync(0xffffffffu, rb, o);
    }
    if (lane == 0) {
      red[0] = ra;
      red[32] = rb;
    }
  }
  __syncthreads();
  const double2 r = make_double2(red[0], red[32]);
  __syncthreads();
  return r;
}

// The same reduction as hhTridiagSmemKernel with the matrix held in
// double-float (df64) form: the O(L^2) parts of a step (the matrix-vector
// product, one thread per row, and the rank-2 update) and the reflector's
// square root and quotients run on the FP32 pipe; p^H v and w in FP64.
// About 1e-14 relative accuracy of the tridiagonal form.
__global__ void __launch_bounds__(kMidT, 1)
    hhTridiagDfKernel(const double2 *Ain, int lda, int m, double2 *Vr,
                      double2 *tau, double *d, double *e) {
  extern __shared__ dfc Adf[];
  __shared__ dfc vsd[kMidMax], wsd[kMidMax];
  __shared__ double2 v64[kMidMax], p64[kMidMax];
  __shared__ double red[64];
  __shared__ double2 sc, taus;
  __shared__ int skip;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int q = tid; q < m * m; q += nt) {
    const int i = q % m, j = q / m;
    double2 v;
    if (i > j) v = Ain[(size_t)j * lda + i];
    else if (i < j) {
      const double2 l = Ain[(size_t)i * lda + j];
      v = make_double2(l.x, -l.y);
    } else v = make_double2(Ain[(size_t)j * lda + i].x, 0.0);
    Adf[q] = dfcFrom(v);
  }
  __syncthreads();
  for (int k = 0; k + 1 < m; ++k) {
    const int L = m - k - 1;
    const dfc *x = Adf + (size_t)k * m + k + 1;
    double loc = 0;
    for (int i = 1 + tid; i < L; i += nt) {
      const double2 xi = dfcTo(x[i]);
      loc += xi.x * xi.x + xi.y * xi.y;
    }
    const double xn2 = blockSum2(loc, 0.0, red).x;
    if (tid == 0) {
      // the reflector in double-float: an FP64 square root or quotient takes
      // ~650 cycles on GB300's FP64 pipe
      const dfc al = x[0];
      d[k] = dfTo(Adf[(size_t)k * m + k].re);
      if (xn2 == 0.0 && al.im.hi == 0.f) {
        tau[k] = make_double2(0.0, 0.0);
        taus = make_double2(0.0, 0.0);
        e[k] = dfTo(al.re);
        skip = 1;
      } else {
        const dfl n2 = dfAdd(dfAdd(dfMul(al.re, al.re), dfMul(al.im, al.im)),
                             dfFrom(xn2));
        dfl beta = dfSqrt(n2);
        if (al.re.hi >= 0.f) beta = dfNeg(beta);
        const dfl rb = dfDiv(dfl{1.f, 0.f}, beta);
        const double2 tv = make_double2(dfTo(dfMul(dfSub(beta, al.re), rb)),
                                        -dfTo(dfMul(al.im, rb)));
        tau[k] = tv;
        taus = tv;
        e[k] = dfTo(beta);
        const dfl dr = dfSub(al.re, beta);
        const dfl rdd = dfDiv(dfl{1.f, 0.f},
                              dfAdd(dfMul(dr, dr), dfMul(al.im, al.im)));
        sc = make_double2(dfTo(dfMul(dr, rdd)), -dfTo(dfMul(al.im, rdd)));
        skip = 0;
      }
    }
    __syncthreads();
    const bool sk = skip != 0;
    const double2 t = taus;
    // the reflectors go out in double-float form (a dfc is 16 bytes, as a
    // double2) for the double-float back-transformation
    dfc *vg = reinterpret_cast<dfc *>(Vr) + (size_t)k * m;
    for (int i = tid; i < m; i += nt) {
      double2 r = make_double2(0.0, 0.0);
      if (!sk && i > k) r = (i == k + 1) ? make_double2(1.0, 0.0)
                                         : cmulD(dfcTo(x[i - k - 1]), sc);
      const dfc rd = dfcFrom(r);
      vg[i] = rd;
      if (i > k) {
        v64[i - k - 1] = r;
        vsd[i - k - 1] = rd;
      }
    }
    __syncthreads();
    if (sk || L < 2) continue; // uniform: skip and L are shared
    // p = tau A22 v in df64: a thread per row, over the row (consecutive
    // threads read consecutive elements of each column), two accumulators
    for (int i = tid; i < L; i += nt) {
      const dfc *row = Adf + (size_t)(k + 1) * m + k + 1 + i;
      dfc a0 = {{0.f, 0.f}, {0.f, 0.f}}, a1 = a0;
      int j = 0;
      for (; j + 1 < L; j += 2) {
        a0 = dfcAdd(a0, dfcMul(row[(size_t)j * m], vsd[j]));
        a1 = dfcAdd(a1, dfcMul(row[(size_t)(j + 1) * m], vsd[j + 1]));
      }
      if (j < L) a0 = dfcAdd(a0, dfcMul(row[(size_t)j * m], vsd[j]));
      p64[i] = cmulD(t, dfcTo(dfcAdd(a0, a1)));
    }
    __syncthreads();
    // w = p - tau/2 (p^H v) v (FP64), then its df64 copy
    double re = 0, im = 0;
    for (int i = tid; i < L; i += nt) {
      const double2 pv = cconjmulD(p64[i], v64[i]);
      re += pv.x;
      im += pv.y;
    }
    const double2 pv = blockSum2(re, im, red);
    const double2 a2 = cmulD(make_double2(-0.5 * t.x, -0.5 * t.y), pv);
    for (int i = tid; i < L; i += nt) {
      const double2 av = cmulD(a2, v64[i]);
      wsd[i] = dfcFrom(make_double2(p64[i].x + av.x, p64[i].y + av.y));
    }
    __syncthreads();
    // A22[i][j] -= v_i conj(w_j) + w_i conj(v_j)
    for (int q = tid; q < L * L; q += nt) {
      const int i = q % L, j = q / L;
      const dfc u = dfcAdd(dfcMulConj(vsd[i], wsd[j]),
                           dfcMulConj(wsd[i], vsd[j]));
      dfc &y = Adf[(size_t)(k + 1 + j) * m + (k + 1 + i)];
      y = dfcSub(y, u);
    }
    __syncthreads();
  }
  if (tid == 0) d[m - 1] = dfTo(Adf[(size_t)(m - 1) * m + (m - 1)].re);
}

// X = H_0 H_1 ... H_{m-2} Z for the real tridiagonal eigenvectors Z, one
// warp per column with the column in shared memory: the reflectors are
// applied from the last to the first (y = v_k^H x, x -= tau_k v_k y)
constexpr int kBtWarps = 1; // a column per SM: FP64-pipe bound
__global__ void __launch_bounds__(32 * kBtWarps)
    btColumnsKernel(const double *Z, int m, const double2 *Vr,
                    const double2 *tau, double2 *X) {
  extern __shared__ double2 xs[]; // kBtWarps x m
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int c = blockIdx.x * kBtWarps + warp;
  if (c >= m) return;
  double2 *x = xs + (size_t)warp * m;
  for (int i = lane; i < m; i += 32)
    x[i] = make_double2(Z[(size_t)c * m + i], 0.0);
  __syncwarp();
  for (int k = m - 2; k >= 0; --k) {
    const double2 t = tau[k];
    if (t.x == 0.0 && t.y == 0.0) continue;
    const int L = m - k - 1;
    const double2 *v = Vr + (size_t)k * m + k + 1;
    double2 *xx = x + k + 1;
    double re = 0, im = 0;
    for (int i = lane; i < L; i += 32) {
      const double2 p = cconjmulD(v[i], xx[i]);
      re += p.x;
      im += p.y;
    }
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, o);
      im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    const double2 ty = cmulD(t, make_double2(re, im));
    for (int i = lane; i < L; i += 32) {
      const double2 u = cmulD(v[i], ty);
      xx[i].x -= u.x;
      xx[i].y -= u.y;
    }
    __syncwarp();
  }
  for (int i = lane; i < m; i += 32) X[(size_t)c * m + i] = x[i];
}

// btColumnsKernel in double-float arithmetic, for the reflectors of
// hhTridiagDfKernel (stored as dfc): a warp per column, the column in shared
// memory as dfc. The dependent chain of a reflector (dot, warp reduction,
// update) runs on the FP32 pipe instead of the FP64 pipe (64-cycle latency).
__global__ void __launch_bounds__(32)
    btColumnsDfKernel(const double *Z, int m, const dfc *Vr,
                      const double2 *tau, double2 *X) {
  extern __shared__ dfc xd[];
  const int c = blockIdx.x, lane = threadIdx.x;
  if (c >= m) return;
  for (int i = lane; i < m; i += 32)
    xd[i] = {dfFrom(Z[(size_t)c * m + i]), {0.f, 0.f}};
  __syncwarp();
  for (int k = m - 2; k >= 0; --k) {
    const double2 t = tau[k];
    if (t.x == 0.0 && t.y == 0.0) continue;
    const int L = m - k - 1;
    const dfc *v = Vr + (size_t)k * m + k + 1;
    dfc *xx = xd + k + 1;
    dfc acc = {{0.f, 0.f}, {0.f, 0.f}};
    for (int i = lane; i < L; i += 32) acc = dfcAdd(acc, dfcConjMul(v[i], xx[i]));
    for (int o = 16; o > 0; o >>= 1) {
      dfc oth;
      oth.re.hi = __shfl_xor_sync(0xffffffffu, acc.re.hi, o);
      oth.re.lo = __shfl_xor_sync(0xffffffffu, acc.re.lo, o);
      oth.im.hi = __shfl_xor_sync(0xffffffffu, acc.im.hi, o);
      oth.im.lo = __shfl_xor_sync(0xffffffffu, acc.im.lo, o);
      acc = dfcAdd(acc, oth);
    }
    const dfc ty = dfcMul(dfcFrom(t), acc);
    for (int i = lane; i < L; i += 32) xx[i] = dfcSub(xx[i], dfcMul(v[i], ty));
    __syncwarp();
  }
  for (int i = lane; i < m; i += 32) X[(size_t)c * m + i] = dfcTo(xd[i]);
}

__global__ void finishKernel(int m, int *perm, int *status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) perm[i] = i;
  if (i == 0) *status = 0;
}

} // namespace

size_t heigLargeScratchBytes(int m) {
  const size_t mm = (size_t)m * m;
  return 2 * mm * sizeof(double2)                // A, Vr
         + (size_t)kJC * m * sizeof(double2)     // P
         + (size_t)m * sizeof(double2)           // Wv
         + (size_t)m * sizeof(double2)           // tau
         + 2 * (size_t)m * sizeof(double)        // d, e
         + 6 * mm * sizeof(double) + 1024;       // Z, F (5)
}

// w ascending, V eigenvectors (m x m, column-major); scratch holds
// heigLargeScratchBytes(m) bytes
void heigLarge(const double2 *Ain, int lda, int m, double2 *V, double *w,
               int *perm, int *status, void *scratch, cudaStream_t s) {
  const size_t mm = (size_t)m * m;
  char *p = static_cast<char *>(scratch);
  auto take = [&](size_t bytes) {
    char *r = p;
    p += (bytes + 255) & ~(size_t)255;
    return r;
  };
  double2 *A = reinterpret_cast<double2 *>(take(mm * sizeof(double2)));
  double2 *Vr = reinterpret_cast<double2 *>(take(mm * sizeof(double2)));
  double2 *P = reinterpret_cast<double2 *>(take((size_t)kJC * m * sizeof(double2)));
  double2 *Wv = reinterpret_cast<double2 *>(take(m * sizeof(double2)));
  double2 *tau = reinterpret_cast<double2 *>(take(m * sizeof(double2)));
  double *d = reinterpret_cast<double *>(take(m * sizeof(double)));
  double *e = reinterpret_cast<double *>(take(m * sizeof(double)));
  double *Z = reinterpret_cast<double *>(take(mm * sizeof(double)));
  double *F = reinterpret_cast<double *>(take(5 * mm * sizeof(double)));
  const unsigned gm = (unsigned)((mm + kT - 1) / kT);
  fullCopyKernel<<<gm, kT, 0, s>>>(Ain, lda, m, A);
  for (int k = 0; k + 1 < m; ++k) {
    const int L = m - k - 1;
    hhVectorKernel<<<1, kT, 0, s>>>(A, m, k, Vr, tau, d, e);
    if (L < 2) continue; // the last reflector only makes e[m-2] real
    hhMatvecKernel<<<dim3((L + 127) / 128, kJC), 128, 0, s>>>(A, m, k, Vr, P);
    hhWKernel<<<1, kT, 0, s>>>(m, k, P, Vr, tau, Wv);
    hhUpdateKernel<<<dim3((L + 127) / 128, L), 128, 0, s>>>(A, m, k, Vr, Wv,
                                                            tau);
  }
  lastDiagKernel<<<1, 32, 0, s>>>(A, m, d);
  multisectKernel<<<m, 32, 0, s>>>(d, e, m, w);
  invIterKernel<<<m, 32, 0, s>>>(d, e, m, w, Z, F);
  clusterMgsKernel<<<m, kT, 0, s>>>(w, m, Z);
  btColumnsKernel<<<(m + kBtWarps - 1) / kBtWarps, 32 * kBtWarps,
                    kBtWarps * (size_t)m * sizeof(double2), s>>>(Z, m, Vr, tau,
                                                                 V);
  finishKernel<<<(m + 255) / 256, 256, 0, s>>>(m, perm, status);
}

// NCGM_HEIG_MID_FP64=1 keeps the FP64 reduction (comparisons)
static bool heigMidFp64() {
  static const bool v = [] {
    const char *e = std::getenv("NCGM_HEIG_MID_FP64");
    return e && e[0] == '1';
  }();
  return v;
}

size_t heigMidScratchBytes(int m) {
  const size_t mm = (size_t)m * m;
  return mm * sizeof(double2) + 256         // Vr
         + (size_t)m * sizeof(double2) + 256 // tau
         + 2 * ((size_t)m * sizeof(double) + 256) // d, e
         + 6 * mm * sizeof(double) + 1024;  // Z, F (5)
}
int heigMidMax() { return kMidMax; }

// The Householder method of heigLarge with the tridiagonalisation in one CTA
// (m <= kMidMax): one launch for the reduction, then multisection, inverse
// iteration, cluster orthogonalisation and the per-column
// back-transformation.
void heigMid(const double2 *Ain, int lda, int m, double2 *V, double *w,
             int *perm, int *status, void *scratch, cudaStream_t s) {
  const size_t mm = (size_t)m * m;
  char *p = static_cast<char *>(scratch);
  auto take = [&](size_t bytes) {
    char *r = p;
    p += (bytes + 255) & ~(size_t)255;
    return r;
  };
  double2 *Vr = reinterpret_cast<double2 *>(take(mm * sizeof(double2)));
  double2 *tau = reinterpret_cast<double2 *>(take(m * sizeof(double2)));
  double *d = reinterpret_cast<double *>(take(m * sizeof(double)));
  double *e = reinterpret_cast<double *>(take(m * sizeof(double)));
  double *Z = reinterpret_cast<double *>(take(mm * sizeof(double)));
  double *F = reinterpret_cast<double *>(take(5 * mm * sizeof(double)));
  // the dynamic shared-memory limit is a per-device attribute: set on every
  // call (a driver call of about a microsecond)
  if (heigMidFp64()) {
    cudaFuncSetAttribute(hhTridiagSmemKernel,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kMidMax * kMidMax * (int)sizeof(double2));
    hhTridiagSmemKernel<<<1, kMidT, mm * sizeof(double2), s>>>(Ain, lda, m,
                                                               Vr, tau, d, e);
  } else {
    cudaFuncSetAttribute(hhTridiagDfKernel,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kMidMax * kMidMax * (int)sizeof(dfc));
    hhTridiagDfKernel<<<1, kMidT, mm * sizeof(dfc), s>>>(Ain, lda, m, Vr, tau,
                                                         d, e);
  }
  // eigenvalues by double-float multisection; the eigenvectors by FP64
  // inverse iteration (its backward error sets the orthogonality between
  // clusters: a double-float solve left 1e-11 there)
  if (heigMidFp64())
    multisectKernel<<<m, 32, 0, s>>>(d, e, m, w);
  else
    multisectDfKernel<<<m, 32, 0, s>>>(d, e, m, w);
  invIterKernel<<<m, 32, 0, s>>>(d, e, m, w, Z, F);
  clusterMgsKernel<<<m, kT, 0, s>>>(w, m, Z);
  if (heigMidFp64())
    btColumnsKernel<<<(m + kBtWarps - 1) / kBtWarps, 32 * kBtWarps,
                      kBtWarps * (size_t)m * sizeof(double2), s>>>(Z, m, Vr,
                                                                   tau, V);
  else
    btColumnsDfKernel<<<m, 32, (size_t)m * sizeof(dfc), s>>>(
        Z, m, reinterpret_cast<const dfc *>(Vr), tau, V);
  finishKernel<<<(m + 255) / 256, 256, 0, s>>>(m, perm, status);
}

} // namespace ncgm
