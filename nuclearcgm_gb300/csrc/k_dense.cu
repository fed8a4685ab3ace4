// Tall-skinny and small dense FP64 complex linear algebra for the block GCG
// eigensolver (gcgm_complex_no_B_lock, src/solver/solver.cpp:642-959):
//  * gram:      C = A^H B for N x p, N x q blocks (row chunks, deterministic
//               two-pass reduction, no atomics);
//  * gemmVC:    Y = V C for N x m times m x k;
//  * cholDrop:  one-CTA Cholesky of a Gram matrix with the modified
//               Gram-Schmidt column-drop rule (|v_j| after projection below
//               1e-12 -> column dropped, solver.cpp:404-407), returning the
//               inverse factor so that Q = V R^{-1};
//  * heig:      one-CTA cyclic Jacobi Hermitian eigensolver reading the lower
//               triangle (as SelfAdjointEigenSolver does), ascending order.
#include "k_dense.cuh"
#include "df64.cuh"

#include <algorithm>
#include <cstdlib>
#include <cmath>

namespace ncgm {

namespace {

constexpr int kTile = 16;  // gram output tile
constexpr int kRows = 32;  // rows staged per smem pass

__global__ void gramKernel(const double2 *__restrict__ A, size_t lda, int p,
                           const double2 *__restrict__ B, size_t ldb, int q,
                           size_t N, size_t rowsPerChunk, double2 *partials) {
  __shared__ double2 As[kRows][kTile + 1];
  __shared__ double2 Bs[kRows][kTile + 1];
  const int ti = threadIdx.x % kTile, tj = threadIdx.x / kTile;
  const int i0 = blockIdx.x * kTile, j0 = blockIdx.y * kTile;
  const size_t r0 = blockIdx.z * rowsPerChunk;
  const size_t r1 = min(N, r0 + rowsPerChunk);
  double2 acc = make_double2(0.0, 0.0);
  for (size_t rb = r0; rb < r1; rb += kRows) {
    // load kRows x kTile of A and B (column-major: consecutive rows)
    for (int e = threadIdx.x; e < kRows * kTile; e += blockDim.x) {
      int rr = e % kRows, cc = e / kRows;
      size_t r = rb + rr;
      int ia = i0 + cc, jb = j0 + cc;
      As[rr][cc] = (r < r1 && ia < p) ? A[ia * lda + r] : make_double2(0, 0);
      Bs[rr][cc] = (r < r1 && jb < q) ? B[jb * ldb + r] : make_double2(0, 0);
    }
    __syncthreads();
#pragma unroll 8
    for (int rr = 0; rr < kRows; ++rr) {
      double2 a = As[rr][ti], b = Bs[rr][tj];
      // conj(a) * b
      acc.x += a.x * b.x + a.y * b.y;
      acc.y += a.x * b.y - a.y * b.x;
    }
    __syncthreads();
  }
  const int i = i0 + ti, j = j0 + tj;
  if (i < p && j < q)
    partials[(size_t)blockIdx.z * p * q + (size_t)j * p + i] = acc;
}

__global__ void reducePartials(const double2 *partials, int chunks, int count,
                               double2 *out, int ldo, int p) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= count) return;
  double2 s = make_double2(0, 0);
  for (int c = 0; c < chunks; ++c) {
    double2 v = partials[(size_t)c * count + e];
    s.x += v.x;
    s.y += v.y;
  }
  int i = e % p, j = e / p;
  out[(size_t)j * ldo + i] = s;
}

// Y(:, j) = sum_l V(:, l) C(l, j) (+ beta Y) ; C in shared memory
__global__ void gemmVCKernel(const double2 *__restrict__ V, size_t ldv, int m,
                             const double2 *__restrict__ Cm, int ldc, int k,
                             double2 *Y, size_t ldy, size_t N, double beta) {
  extern __shared__ double2 Cs[];
  for (int e = threadIdx.x; e < m * k; e += blockDim.x) {
    int l = e % m, j = e / m;
    Cs[e] = Cm[(size_t)j * ldc + l];
  }
  __syncthreads();
  const size_t r = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (r >= N) return;
  const int j0 = blockIdx.y * 8;
  const int j1 = min(k, j0 + 8);
  double2 acc[8];
#pragma unroll
  for (int t = 0; t < 8; ++t) acc[t] = make_double2(0, 0);
  for (int l = 0; l < m; ++l) {
    double2 v = V[l * ldv + r];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      if (j0 + t < j1) {
        double2 c = Cs[(size_t)(j0 + t) * m + l];
        acc[t].x += v.x * c.x - v.y * c.y;
        acc[t].y += v.x * c.y + v.y * c.x;
      }
    }
  }
  for (int t = 0; t < 8; ++t)
    if (j0 + t < j1) {
      double2 *y = Y + (size_t)(j0 + t) * ldy + r;
      if (beta != 0.0) {
        double2 o = *y;
        acc[t].x += beta * o.x;
        acc[t].y += beta * o.y;
      }
      *y = acc[t];
    }
}

__device__ inline double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ inline double2 cconjmul(double2 a, double2 b) { // conj(a) b
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// One CTA. G (m x m, col-major, Hermitian, upper triangle used) ->
// R upper with G = R^H R, columns whose pivot <= dropTol are dropped (their
// row/column of R zero). Writes T = R^{-1} (m x m, zero rows/cols for dropped
// columns) and keep[j] (1 kept, 0 dropped). Work arrays in global memory.
__global__ void cholDropKernel(const double2 *G, int ldg, int m,
                               double dropTol, double2 *R, double2 *T,
                               int *keep) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < m * m; e += nt) {
    R[e] = make_double2(0, 0);
    T[e] = make_double2(0, 0);
  }
  __syncthreads();
  __shared__ double piv;
  for (int j = 0; j < m; ++j) {
    // pivot: d = G_jj - sum_{k<j} |R_kj|^2
    if (tid == 0) {
      double d = G[(size_t)j * ldg + j].x;
      for (int k = 0; k < j; ++k) {
        double2 r = R[(size_t)j * m + k];
        d -= r.x * r.x + r.y * r.y;
      }
      // The Gram pivot carries a rounding floor of ~eps * G_jj, so a column
      // whose residual is below that floor is dependent to working precision
      // and is dropped, as MGS drops residual norms below 1e-12.
      const double floor = fmax(dropTol, 64.0 * 2.220446049250313e-16 *
                                             G[(size_t)j * ldg + j].x);
      const int kp = (d > floor) ? 1 : 0;
      piv = kp ? d : 0.0;
      keep[j] = kp;
      if (kp) R[(size_t)j * m + j] = make_double2(sqrt(d), 0.0);
    }
    __syncthreads();
    if (piv > 0.0) {
      const double rjj = sqrt(piv);
      // R_ji = (G_ji - sum_{k<j} conj(R_kj) R_ki) / R_jj, i > j
      for (int i = j + 1 + tid; i < m; i += nt) {
        double2 s = G[(size_t)i * ldg + j];
        for (int k = 0; k < j; ++k) {
          double2 t = cconjmul(R[(size_t)j * m + k], R[(size_t)i * m + k]);
          s.x -= t.x;
          s.y -= t.y;
        }
        R[(size_t)i * m + j] = make_double2(s.x / rjj, s.y / rjj);
      }
    }
    __syncthreads();
  }
  // T = R^{-1} restricted to kept columns: solve R T = I column by column
  // (upper triangular back substitution), one thread per column of T.
  for (int c = tid; c < m; c += nt) {
    if (!keep[c]) continue;
    for (int i = c; i >= 0; --i) {
      if (!keep[i]) continue;
      double2 s = make_double2(i == c ? 1.0 : 0.0, 0.0);
      for (int k = i + 1; k <= c; ++k) {
        if (!keep[k]) continue;
        double2 t = cmul(R[(size_t)k * m + i], T[(size_t)c * m + k]);
        s.x -= t.x;
        s.y -= t.y;
      }
      double rii = R[(size_t)i * m + i].x;
      T[(size_t)c * m + i] = make_double2(s.x / rii, s.y / rii);
    }
  }
}

// FP64 cyclic Jacobi sweeps sweep0 .. 59 on the Hermitian A (m x m,
// column-major), rotations accumulated into Vm (round-robin pairing: every
// round rotates m/2 disjoint (p,q) pairs at once). Returns 1 on convergence.
__device__ int jacobiSweeps64(double2 *A, double2 *Vm, int m, double fro,
                              int sweep0, int *P, int *Q, double *C,
                              double *S, double2 *E, double *red) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int mp = (m % 2) ? m + 1 : m; // players incl. a dummy for odd m
  const int npairs = mp / 2;
  int converged = 0;
  for (int sweep = sweep0; sweep < 60; ++sweep) {
    double loc = 0;
    for (int e = tid; e < m * m; e += nt) {
      int i = e % m, j = e / m;
      if (i > j) loc += A[e].x * A[e].x + A[e].y * A[e].y;
    }
    red[tid] = loc;
    __syncthreads();
    for (int st = nt / 2; st > 0; st >>= 1) {
      if (tid < st) red[tid] += red[tid + st];
      __syncthreads();
    }
    double off = red[0];
    __syncthreads();
    if (off <= 1e-32 * fro || off == 0.0) {
      converged = 1;
      break;
    }
    for (int r = 0; r < mp - 1; ++r) {
      // pairing of this round and rotation parameters, one thread per pair
      for (int k = tid; k < npairs; k += nt) {
        int a, b;
        if (k == 0) {
          a = mp - 1;
          b = r;
        } else {
          a = (r + k) % (mp - 1);
          b = (r - k + (mp - 1)) % (mp - 1);
        }
        int p = min(a, b), q = max(a, b);
        P[k] = p;
        Q[k] = q;
        C[k] = 1.0;
        S[k] = 0.0;
        E[k] = make_double2(1.0, 0.0);
        if (q < m) {
          double2 apq = A[(size_t)q * m + p];
          double mag = sqrt(apq.x * apq.x + apq.y * apq.y);
          double app = A[(size_t)p * m + p].x, aqq = A[(size_t)q * m + q].x;
          if (mag != 0.0 &&
              !(sweep > 3 && mag < 1e-18 * sqrt(fabs(app * aqq)) + 1e-300)) {
            double tau = (aqq - app) / (2.0 * mag);
            double t = (tau >= 0 ? 1.0 : -1.0) /
                       (fabs(tau) + sqrt(1.0 + tau * tau));
            C[k] = 1.0 / sqrt(1.0 + t * t);
            S[k] = t * C[k];
            E[k] = make_double2(apq.x / mag, apq.y / mag);
          }
        }
      }
      __syncthreads();
      // A <- A U and V <- V U: thread per (row, pair)
      for (int e = tid; e < m * npairs; e += nt) {
        int row = e % m, k = e / m;
        int p = P[k], q = Q[k];
        if (q >= m || S[k] == 0.0) continue;
        double c = C[k], s = S[k];
        double2 ec = make_double2(E[k].x, -E[k].y);
        double2 arp = A[(size_t)p * m + row], arq = A[(size_t)q * m + row];
        double2 t1 = cmul(ec, arq);
        A[(size_t)p * m + row] = make_double2(c * arp.x - s * t1.x, c * arp.y - s * t1.y);
        A[(size_t)q * m + row] = make_double2(s * arp.x + c * t1.x, s * arp.y + c * t1.y);
        double2 vrp = Vm[(size_t)p * m + row], vrq = Vm[(size_t)q * m + row];
        double2 t2 = cmul(ec, vrq);
        Vm[(size_t)p * m + row] = make_double2(c * vrp.x - s * t2.x, c * vrp.y - s * t2.y);
        Vm[(size_t)q * m + row] = make_double2(s * vrp.x + c * t2.x, s * vrp.y + c * t2.y);
      }
      __syncthreads();
      // A <- U^H A: thread per (pair, column)
      for (int e = tid; e < m * npairs; e += nt) {
        int col = e % m, k = e / m;
        int p = P[k], q = Q[k];
        if (q >= m || S[k] == 0.0) continue;
        double c = C[k], s = S[k];
        double2 ee = E[k];
        double2 apr = A[(size_t)col * m + p], aqr = A[(size_t)col * m + q];
        double2 t1 = cmul(ee, aqr);
        A[(size_t)col * m + p] = make_double2(c * apr.x - s * t1.x, c * apr.y - s * t1.y);
        A[(size_t)col * m + q] = make_double2(s * apr.x + c * t1.x, s * apr.y + c * t1.y);
      }
      __syncthreads();
      for (int k = tid; k < npairs; k += nt) {
        int p = P[k], q = Q[k];
        if (q >= m || S[k] == 0.0) continue;
        A[(size_t)q * m + p] = make_double2(0, 0);
        A[(size_t)p * m + q] = make_double2(0, 0);
        A[(size_t)p * m + p].y = 0.0;
        A[(size_t)q * m + q].y = 0.0;
      }
      __syncthreads();
    }
  }
  return converged;
}

// ascending order of the diagonal (stable insertion sort by thread 0),
// eigenvalues w, status, and the permuted eigenvectors written to Vg (A is
// reused as the staging copy)
__device__ void jacobiFinish(double2 *A, const double2 *Vm, int m,
                             int converged, double2 *Vg, double *w, int *perm,
                             int *status) {
  const int tid = threadIdx.x, nt = blockDim.x;
  // sort ascending (stable insertion sort by thread 0), permute eigenvectors
  if (tid == 0) {
    for (int i = 0; i < m; ++i) perm[i] = i;
    for (int i = 1; i < m; ++i) {
      int pi = perm[i];
      double key = A[(size_t)pi * m + pi].x;
      int k = i - 1;
      while (k >= 0 && A[(size_t)perm[k] * m + perm[k]].x > key) {
        perm[k + 1] = perm[k];
        --k;
      }
      perm[k + 1] = pi;
    }
    for (int i = 0; i < m; ++i) w[i] = A[(size_t)perm[i] * m + perm[i]].x;
    *status = converged ? 0 : 1;
  }
  __syncthreads();
  for (int e = tid; e < m * m; e += nt) {
    int r = e % m, c = e / m;
    A[e] = Vm[(size_t)perm[c] * m + r];
  }
  __syncthreads();
  for (int e = tid; e < m * m; e += nt) Vg[e] = A[e];
}


// One CTA parallel-order Jacobi (round-robin pairing: every round rotates
// m/2 disjoint (p,q) pairs at once, m-1 rounds per sweep) on a Hermitian
// m x m matrix whose lower triangle is read. A, Vm: m x m workspaces;
// w: eigenvalues ascending; Vm: eigenvectors in the same order.
__global__ void heigKernel(const double2 *Ain, int lda, int m, double2 *Ag,
                           double2 *Vg, double *w, int *perm, int *status,
                           int useSmem) {
  // working copies in shared memory when they fit: useSmem 2 = A and V
  // (m <= 81), 1 = A only (m <= 114), 0 = both in the global work buffers
  extern __shared__ double2 hsm[];
  double2 *A = useSmem ? hsm : Ag;
  double2 *Vm = useSmem == 2 ? hsm + (size_t)m * m : Vg;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < m * m; e += nt) {
    int i = e % m, j = e / m;
    double2 v;
    if (i > j) v = Ain[(size_t)j * lda + i];
    else if (i < j) {
      double2 l = Ain[(size_t)i * lda + j];
      v = make_double2(l.x, -l.y);
    } else v = make_double2(Ain[(size_t)j * lda + i].x, 0.0);
    A[e] = v;
    Vm[e] = make_double2(i == j ? 1.0 : 0.0, 0.0);
  }
  __shared__ int P[256], Q[256];
  __shared__ double C[256], S[256];
  __shared__ double2 E[256];
  __shared__ double red[512]; // blockDim.x <= 512
  __syncthreads();
  double fro = 0;
  {
    double loc = 0;
    for (int e = tid; e < m * m; e += nt) loc += A[e].x * A[e].x + A[e].y * A[e].y;
    red[tid] = loc;
    __syncthreads();
    for (int st = nt / 2; st > 0; st >>= 1) {
      if (tid < st) red[tid] += red[tid + st];
      __syncthreads();
    }
    fro = red[0];
    __syncthreads();
  }
  const int converged =
      jacobiSweeps64(A, Vm, m, fro, 0, P, Q, C, S, E, red);
  jacobiFinish(A, Vm, m, converged, Vg, w, perm, status);
}

// ---- double-float (df64) form of the Jacobi eigensolver ----
// GB300's FP64 pipe retires 2 FMAs per clock per SM, its FP32 pipe 128, so
// the one-CTA Jacobi is FP64-throughput-bound (about 19 k cycles per round at
// m = 60). Here the rotation updates, most of the work, run in double-float
// arithmetic: a value is an unevaluated sum hi + lo of two floats (~48-bit
// significand), with Knuth's two-sum and the FMA two-product (Dekker; Hida,
// Li and Bailey's double-double algorithms, restated for float pairs). The
// rotation parameters and the convergence test stay FP64. Accumulated
// rounding over a few hundred rotations per element: ~1e-13 relative. The
// sweeps stop at an off-diagonal norm of 3e-13 relative (the FP64 Jacobi
// stops at 1e-16); the matrices are then converted in place to FP64 for the
// output, and only if that level was not reached do FP64 sweeps continue.
// c x - s (w y), s x + c (w y) for complex x, y, w and real c, s
__device__ __forceinline__ void dfRot(dfc &x, dfc &y, dfl c, dfl s, dfc w) {
  const dfc t = {dfAdd(dfMul(w.re, y.re), dfNeg(dfMul(w.im, y.im))),
                 dfAdd(dfMul(w.re, y.im), dfMul(w.im, y.re))};
  const dfc nx = {dfAdd(dfMul(c, x.re), dfNeg(dfMul(s, t.re))),
                  dfAdd(dfMul(c, x.im), dfNeg(dfMul(s, t.im)))};
  const dfc ny = {dfAdd(dfMul(s, x.re), dfMul(c, t.re)),
                  dfAdd(dfMul(s, x.im), dfMul(c, t.im))};
  x = nx;
  y = ny;
}

constexpr int kHeigDfMax = 80; // A and V in shared memory: 2 m^2 x 16 B
// Same algorithm, pairing and output as heigKernel, with A and V held as
// double-float complex values in shared memory.
__global__ void heigDfKernel(const double2 *Ain, int lda, int m, double2 *Vg,
                             double *w, int *perm, int *status) {
  extern __shared__ dfc dsm[];
  dfc *A = dsm, *Vm = dsm + (size_t)m * m;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < m * m; e += nt) {
    const int i = e % m, j = e / m;
    double2 v;
    if (i > j) v = Ain[(size_t)j * lda + i];
    else if (i < j) {
      const double2 l = Ain[(size_t)i * lda + j];
      v = make_double2(l.x, -l.y);
    } else v = make_double2(Ain[(size_t)j * lda + i].x, 0.0);
    A[e] = {dfFrom(v.x), dfFrom(v.y)};
    Vm[e] = {{i == j ? 1.f : 0.f, 0.f}, {0.f, 0.f}};
  }
  const int mp = (m % 2) ? m + 1 : m;
  const int npairs = mp / 2;
  __shared__ int P[kHeigDfMax / 2 + 1], Q[kHeigDfMax / 2 + 1];
  __shared__ dfl C[kHeigDfMax / 2 + 1], S[kHeigDfMax / 2 + 1];
  __shared__ dfc E[kHeigDfMax / 2 + 1];
  __shared__ int act[kHeigDfMax / 2 + 1];
  __shared__ double red[512];
  __syncthreads();
  auto mag2 = [](const dfc &a) {
    const double x = dfTo(a.re), y = dfTo(a.im);
    return x * x + y * y;
  };
  double fro;
  {
    double loc = 0;
    for (int e = tid; e < m * m; e += nt) loc += mag2(A[e]);
    red[tid] = loc;
    __syncthreads();
    for (int st = nt / 2; st > 0; st >>= 1) {
      if (tid < st) red[tid] += red[tid + st];
      __syncthreads();
    }
    fro = red[0];
    __syncthreads();
  }
  int dfSweeps = 0, dfConverged = 0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double loc = 0;
    for (int e = tid; e < m * m; e += nt) {
      const int i = e % m, j = e / m;
      if (i > j) loc += mag2(A[e]);
    }
    red[tid] = loc;
    __syncthreads();
    for (int st = nt / 2; st > 0; st >>= 1) {
      if (tid < st) red[tid] += red[tid + st];
      __syncthreads();
    }
    const double off = red[0];
    __syncthreads();
    if (off <= 1e-25 * fro || off == 0.0) {
      dfConverged = 1;
      break;
    }
    ++dfSweeps;
    for (int r = 0; r < mp - 1; ++r) {
      for (int k = tid; k < npairs; k += nt) {
        int a, b;
        if (k == 0) {
          a = mp - 1;
          b = r;
        } else {
          a = (r + k) % (mp - 1);
          b = (r - k + (mp - 1)) % (mp - 1);
        }
        const int p = min(a, b), q = max(a, b);
        P[k] = p;
        Q[k] = q;
        act[k] = 0;
        if (q < m) {
          const dfc apqd = A[(size_t)q * m + p];
          const double ax = dfTo(apqd.re), ay = dfTo(apqd.im);
          const double mag = sqrt(ax * ax + ay * ay);
          const double app = dfTo(A[(size_t)p * m + p].re),
                       aqq = dfTo(A[(size_t)q * m + q].re);
          if (mag != 0.0 &&
              !(sweep > 3 && mag < 1e-18 * sqrt(fabs(app * aqq)) + 1e-300)) {
            const double tau = (aqq - app) / (2.0 * mag);
            const double t = (tau >= 0 ? 1.0 : -1.0) /
                             (fabs(tau) + sqrt(1.0 + tau * tau));
            const double c = 1.0 / sqrt(1.0 + t * t);
            C[k] = dfFrom(c);
            S[k] = dfFrom(t * c);
            E[k] = {dfFrom(ax / mag), dfFrom(ay / mag)};
            act[k] = 1;
          }
        }
      }
      __syncthreads();
      // A <- A U and V <- V U: thread per (row, pair); U mixes columns p, q
      // with conj(e) on column q
      for (int e = tid; e < m * npairs; e += nt) {
        const int row = e % m, k = e / m;
        if (!act[k]) continue;
        const int p = P[k], q = Q[k];
        const dfc ec = {E[k].re, dfNeg(E[k].im)};
        dfRot(A[(size_t)p * m + row], A[(size_t)q * m + row], C[k], S[k], ec);
        dfRot(Vm[(size_t)p * m + row], Vm[(size_t)q * m + row], C[k], S[k],
              ec);
      }
      __syncthreads();
      // A <- U^H A: thread per (pair, column); rows p, q with e on row q
      for (int e = tid; e < m * npairs; e += nt) {
        const int col = e % m, k = e / m;
        if (!act[k]) continue;
        const int p = P[k], q = Q[k];
        dfRot(A[(size_t)col * m + p], A[(size_t)col * m + q], C[k], S[k],
              E[k]);
      }
      __syncthreads();
      for (int k = tid; k < npairs; k += nt) {
        if (!act[k]) continue;
        const int p = P[k], q = Q[k];
        A[(size_t)q * m + p] = {{0.f, 0.f}, {0.f, 0.f}};
        A[(size_t)p * m + q] = {{0.f, 0.f}, {0.f, 0.f}};
        A[(size_t)p * m + p].im = {0.f, 0.f};
        A[(size_t)q * m + q].im = {0.f, 0.f};
      }
      __syncthreads();
    }
  }
  // in place to FP64 (a dfc and a double2 are both 16 bytes; every thread
  // converts the elements it reads), then the FP64 sweeps
  double2 *A64 = reinterpret_cast<double2 *>(A);
  double2 *V64 = reinterpret_cast<double2 *>(Vm);
  for (int e = tid; e < m * m; e += nt) {
    const dfc a = A[e], v = Vm[e];
    A64[e] = make_double2(dfTo(a.re), dfTo(a.im));
    V64[e] = make_double2(dfTo(v.re), dfTo(v.im));
  }
  __syncthreads();
  __shared__ double C64[kHeigDfMax / 2 + 1], S64[kHeigDfMax / 2 + 1];
  __shared__ double2 E64[kHeigDfMax / 2 + 1];
  const int converged =
      dfConverged ? 1
                  : jacobiSweeps64(A64, V64, m, fro, dfSweeps, P, Q, C64, S64,
                                   E64, red);
  jacobiFinish(A64, V64, m, converged, Vg, w, perm, status);
}

} // namespace

void gram(const double2 *A, size_t lda, int p, const double2 *B, size_t ldb,
          int q, size_t N, double2 *C, int ldc, double2 *partials,
          int maxChunks, cudaStream_t s) {
  if (p == 0 || q == 0) return;
  int chunks = (int)std::min<size_t>(maxChunks, std::max<size_t>(1, N / 256));
  size_t rows = (N + chunks - 1) / chunks;
  rows = ((rows + kRows - 1) / kRows) * kRows;
  chunks = (int)((N + rows - 1) / rows);
  dim3 grid((p + kTile - 1) / kTile, (q + kTile - 1) / kTile, chunks);
  gramKernel<<<grid, kTile * kTile, 0, s>>>(A, lda, p, B, ldb, q, N, rows,
                                            partials);
  int count = p * q;
  reducePartials<<<(count + 127) / 128, 128, 0, s>>>(partials, chunks, count,
                                                     C, ldc, p);
}

int gramMaxChunks() { return 256; }

void gemmVC(const double2 *V, size_t ldv, int m, const double2 *Cm, int ldc,
            int k, double2 *Y, size_t ldy, size_t N, double beta,
            cudaStream_t s) {
  if (k == 0) return;
  if (m == 0) {
    // Y = beta Y; only used with beta = 0 -> zero
    for (int j = 0; j < k; ++j)
      cudaMemsetAsync(Y + (size_t)j * ldy, 0, N * sizeof(double2), s);
    return;
  }
  static const bool attr = [] {
    cudaFuncSetAttribute(gemmVCKernel,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         200 * 1024);
    return true;
  }();
  (void)attr;
  // C is staged in shared memory: blocks of kt columns with m * kt * 16
  // bytes <= 200 KB (kt a multiple of 8)
  int kt = (int)((200 * 1024) / ((size_t)m * sizeof(double2)));
  kt = std::max(8, kt / 8 * 8);
  for (int j0 = 0; j0 < k; j0 += kt) {
    const int kb = std::min(kt, k - j0);
    const size_t smem = (size_t)m * kb * sizeof(double2);
    dim3 grid((unsigned)((N + 127) / 128), (kb + 7) / 8);
    gemmVCKernel<<<grid, 128, smem, s>>>(V, ldv, m, Cm + (size_t)j0 * ldc,
                                         ldc, kb, Y + (size_t)j0 * ldy, ldy, N,
                                         beta);
  }
}

// Same factorisation in shared memory, right-looking: at step j the pivot is
// the updated diagonal A_jj = G_jj - sum_{k<j} |R_kj|^2, row j of R is
// A_j. / R_jj, and the trailing upper triangle takes the rank-1 update
// A_ab -= conj(R_ja) R_jb in parallel (one barrier-separated phase per
// step instead of a serial dot product per element). The drop rule and
// T = R^{-1} are those of cholDropKernel.
constexpr int kCholSmemMax = 80; // 2 m^2 double2 <= 200 KB
// The FP32 forms' CholQR factor with the matrix held as double-float in
// shared memory: the O(m^3) trailing updates and R^-1 run on the FP32 pipe
// (an FP64 FMA has 64-cycle latency and the FP64 pipe 2 per clock per SM on
// GB300), the pivot test in FP64. About 1e-14 relative accuracy; the second
// CholQR pass absorbs it. Same drop rule, outputs and layout as
// cholDropSmemKernel.
__global__ void cholDropDfKernel(const double2 *G, int ldg, int m,
                                 double dropTol, double2 *R, double2 *T,
                                 int *keep) {
  extern __shared__ dfc cdf[];
  dfc *A = cdf;              // m x m column-major; upper triangle -> R
  dfc *Ts = cdf + m * m;     // T
  __shared__ int kp[kCholSmemMax];
  __shared__ double gd[kCholSmemMax]; // the Gram diagonal (drop floor)
  __shared__ dfl rinv[kCholSmemMax];
  __shared__ int pivOk;
  const int tid = threadIdx.x, nt = blockDim.x;
  const dfc zero = {{0.f, 0.f}, {0.f, 0.f}};
  for (int e = tid; e < m * m; e += nt) {
    const double2 g = G[(size_t)(e / m) * ldg + (e % m)];
    A[e] = dfcFrom(g);
    Ts[e] = zero;
    if (e / m == e % m) gd[e % m] = g.x;
  }
  __syncthreads();
  for (int j = 0; j < m; ++j) {
    if (tid == 0) {
      const double d = dfTo(A[(size_t)j * m + j].re);
      const double floor =
          fmax(dropTol, 64.0 * 2.220446049250313e-16 * gd[j]);
      pivOk = (d > floor) ? 1 : 0;
      kp[j] = pivOk;
    }
    __syncthreads();
    if (pivOk) {
      const dfl sq = dfSqrt(A[(size_t)j * m + j].re);
      const dfl inv = dfDiv(dfl{1.f, 0.f}, sq);
      for (int i = j + 1 + tid; i < m; i += nt) {
        dfc &a = A[(size_t)i * m + j];
        a = {dfMul(a.re, inv), dfMul(a.im, inv)};
      }
      if (tid == 0) {
        A[(size_t)j * m + j] = {sq, {0.f, 0.f}};
        rinv[j] = inv;
      }
      __syncthreads();
      const int w = m - j - 1;
      for (int e = tid; e < w * w; e += nt) {
        const int a = j + 1 + e % w, b = j + 1 + e / w;
        if (a <= b) {
          const dfc t = dfcConjMul(A[(size_t)a * m + j], A[(size_t)b * m + j]);
          dfc &x = A[(size_t)b * m + a];
          x = dfcSub(x, t);
        }
      }
    } else {
      for (int i = j + tid; i < m; i += nt) A[(size_t)i * m + j] = zero;
      if (tid == 0) rinv[j] = {0.f, 0.f};
    }
    __syncthreads();
  }
  // T = R^{-1} on the kept columns, one thread per column; dropped rows and
  // columns hold zeros in R and T, so they add nothing to the sums
  for (int c = tid; c < m; c += nt) {
    if (!kp[c]) continue;
    for (int i = c; i >= 0; --i) {
      if (!kp[i]) continue;
      dfc s0 = {{i == c ? 1.f : 0.f, 0.f}, {0.f, 0.f}}, s1 = zero;
      int k = i + 1;
      for (; k + 1 <= c; k += 2) {
        s0 = dfcSub(s0, dfcMul(A[(size_t)k * m + i], Ts[(size_t)c * m + k]));
        s1 = dfcSub(s1, dfcMul(A[(size_t)(k + 1) * m + i],
                               Ts[(size_t)c * m + k + 1]));
      }
      if (k <= c)
        s0 = dfcSub(s0, dfcMul(A[(size_t)k * m + i], Ts[(size_t)c * m + k]));
      const dfc sum = dfcAdd(s0, s1);
      Ts[(size_t)c * m + i] = {dfMul(sum.re, rinv[i]), dfMul(sum.im, rinv[i])};
    }
  }
  __syncthreads();
  for (int e = tid; e < m * m; e += nt) {
    const int row = e % m, col = e / m;
    R[e] = row <= col ? dfcTo(A[e]) : make_double2(0, 0);
    T[e] = dfcTo(Ts[e]);
  }
  for (int j = tid; j < m; j += nt) keep[j] = kp[j];
}

__global__ void cholDropSmemKernel(const double2 *G, int ldg, int m,
                                   double dropTol, double2 *R, double2 *T,
                                   int *keep) {
  extern __shared__ double2 csm[];
  double2 *A = csm;          // m x m column-major; upper triangle -> R
  double2 *Ts = csm + m * m; // T
  __shared__ int kp[kCholSmemMax];
  __shared__ double gd[kCholSmemMax]; // the Gram diagonal (drop floor)
  __shared__ double piv;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < m * m; e += nt) {
    const double2 g = G[(size_t)(e / m) * ldg + (e % m)];
    A[e] = g;
    Ts[e] = make_double2(0, 0);
    if (e / m == e % m) gd[e % m] = g.x;
  }
  __syncthreads();
  for (int j = 0; j < m; ++j) {
    if (tid == 0) {
      const double d = A[(size_t)j * m + j].x;
      const double floor =
          fmax(dropTol, 64.0 * 2.220446049250313e-16 * gd[j]);
      const int k = (d > floor) ? 1 : 0;
      kp[j] = k;
      piv = k ? d : 0.0;
    }
    __syncthreads();
    const double pv = piv;
    if (pv > 0.0) {
      const double rjj = sqrt(pv);
      for (int i = j + 1 + tid; i < m; i += nt) {
        const double2 a = A[(size_t)i * m + j];
        A[(size_t)i * m + j] = make_double2(a.x / rjj, a.y / rjj);
      }
      if (tid == 0) A[(size_t)j * m + j] = make_double2(rjj, 0.0);
      __syncthreads();
      const int w = m - j - 1;
      for (int e = tid; e < w * w; e += nt) {
        const int a = j + 1 + e % w, b = j + 1 + e / w;
        if (a <= b) {
          const double2 t = cconjmul(A[(size_t)a * m + j], A[(size_t)b * m + j]);
          double2 &x = A[(size_t)b * m + a];
          x.x -= t.x;
          x.y -= t.y;
        }
      }
    } else {
      for (int i = j + tid; i < m; i += nt) A[(size_t)i * m + j] = make_double2(0, 0);
    }
    __syncthreads();
  }
  // T = R^{-1} on the kept columns, one thread per column of T
  for (int c = tid; c < m; c += nt) {
    if (!kp[c]) continue;
    for (int i = c; i >= 0; --i) {
      if (!kp[i]) continue;
      double2 sum = make_double2(i == c ? 1.0 : 0.0, 0.0);
      for (int k = i + 1; k <= c; ++k) {
        if (!kp[k]) continue;
        const double2 t = cmul(A[(size_t)k * m + i], Ts[(size_t)c * m + k]);
        sum.x -= t.x;
        sum.y -= t.y;
      }
      const double rii = A[(size_t)i * m + i].x;
      Ts[(size_t)c * m + i] = make_double2(sum.x / rii, sum.y / rii);
    }
  }
  __syncthreads();
  for (int e = tid; e < m * m; e += nt) {
    const int row = e % m, col = e / m;
    R[e] = row <= col ? A[e] : make_double2(0, 0);
    T[e] = Ts[e];
  }
  for (int j = tid; j < m; j += nt) keep[j] = kp[j];
}

// Large m (> 80): the same right-looking factorisation in global memory with
// one launch pair per column (pivot and row scaling in one block, the rank-1
// update of the trailing triangle over the whole GPU), then T = R^{-1} one
// thread per column. G's diagonal (drop floor) and the pivots are kept in
// T's first 2m entries until T is computed.
__global__ void cholCopyKernel(const double2 *G, int ldg, int m, double2 *R,
                               double2 *T) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m * m) return;
  const int row = e % m, col = e / m;
  const double2 g = G[(size_t)col * ldg + row];
  R[e] = g;
  if (row == col) T[row] = make_double2(g.x, 0.0);
}
__global__ void cholPivotKernel(double2 *R, int m, int j, double dropTol,
                                double2 *T, int *keep) {
  __shared__ double piv;
  if (threadIdx.x == 0) {
    const double d = R[(size_t)j * m + j].x;
    const double floor =
        fmax(dropTol, 64.0 * 2.220446049250313e-16 * T[j].x);
    const int k = (d > floor) ? 1 : 0;
    keep[j] = k;
    piv = k ? d : 0.0;
    T[m + j] = make_double2(piv, 0.0);
  }
  __syncthreads();
  if (piv > 0.0) {
    const double rjj = sqrt(piv);
    for (int i = j + 1 + threadIdx.x; i < m; i += blockDim.x) {
      const double2 a = R[(size_t)i * m + j];
      R[(size_t)i * m + j] = make_double2(a.x / rjj, a.y / rjj);
    }
    if (threadIdx.x == 0) R[(size_t)j * m + j] = make_double2(rjj, 0.0);
  } else {
    for (int i = j + threadIdx.x; i < m; i += blockDim.x)
      R[(size_t)i * m + j] = make_double2(0, 0);
  }
}
__global__ void cholUpdateKernel(double2 *R, int m, int j, const double2 *T) {
  if (T[m + j].x <= 0.0) return;
  const int a = j + 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int b = j + 1 + blockIdx.y;
  if (a >= m || a > b) return;
  const double2 t = cconjmul(R[(size_t)a * m + j], R[(size_t)b * m + j]);
  double2 &x = R[(size_t)b * m + a];
  x.x -= t.x;
  x.y -= t.y;
}
__global__ void cholFinishKernel(double2 *R, int m, double2 *T) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m * m) return;
  if (e % m > e / m) R[e] = make_double2(0, 0); // lower triangle
  T[e] = make_double2(0, 0);
}
__global__ void cholInvKernel(const double2 *R, int m, const int *keep,
                              double2 *T) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m || !keep[c]) return;
  for (int i = c; i >= 0; --i) {
    if (!keep[i]) continue;
    double2 sum = make_double2(i == c ? 1.0 : 0.0, 0.0);
    for (int k = i + 1; k <= c; ++k) {
      if (!keep[k]) continue;
      const double2 t = cmul(R[(size_t)k * m + i], T[(size_t)c * m + k]);
      sum.x -= t.x;
      sum.y -= t.y;
    }
    const double rii = R[(size_t)i * m + i].x;
    T[(size_t)c * m + i] = make_double2(sum.x / rii, sum.y / rii);
  }
}

void cholDrop(const double2 *G, int ldg, int m, double dropTol, double2 *R,
              double2 *T, int *keep, cudaStream_t s, bool fast) {
  if (m > kCholSmemMax) {
    const unsigned gm = (unsigned)(((size_t)m * m + 255) / 256);
    cholCopyKernel<<<gm, 256, 0, s>>>(G, ldg, m, R, T);
    for (int j = 0; j < m; ++j) {
      cholPivotKernel<<<1, 128, 0, s>>>(R, m, j, dropTol, T, keep);
      const int w = m - j - 1;
      if (w > 0)
        cholUpdateKernel<<<dim3((w + 127) / 128, w), 128, 0, s>>>(R, m, j, T);
    }
    cholFinishKernel<<<gm, 256, 0, s>>>(R, m, T);
    cholInvKernel<<<(m + 63) / 64, 64, 0, s>>>(R, m, keep, T);
    return;
  }
  if (m <= kCholSmemMax) {
    static const bool attr = [] {
      cudaFuncSetAttribute(cholDropSmemKernel,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           2 * kCholSmemMax * kCholSmemMax * (int)sizeof(double2));
      return true;
    }();
    (void)attr;
    const size_t smem = 2 * (size_t)m * m * sizeof(double2);
    static const bool dfAttr = [] {
      cudaFuncSetAttribute(cholDropDfKernel,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           2 * kCholSmemMax * kCholSmemMax * (int)sizeof(dfc));
      return true;
    }();
    (void)dfAttr;
    if (fast)
      cholDropDfKernel<<<1, 256, 2 * (size_t)m * m * sizeof(dfc), s>>>(
          G, ldg, m, dropTol, R, T, keep);
    else
      cholDropSmemKernel<<<1, 256, smem, s>>>(G, ldg, m, dropTol, R, T, keep);
    return;
  }
  cholDropKernel<<<1, 256, 0, s>>>(G, ldg, m, dropTol, R, T, keep);
}

// NCGM_HEIG_FP64=1 keeps the one-CTA FP64 Jacobi for every size
// (comparisons)
static bool heigFp64Only() {
  static const bool v = [] {
    const char *e = std::getenv("NCGM_HEIG_FP64");
    return e && e[0] == '1';
  }();
  return v;
}

// NCGM_HEIG_MID=0 keeps the double-float Jacobi for the fast path's
// projected problems up to m = 80 instead of the one-CTA Householder method
// (comparisons)
static bool heigMidOn() {
  static const bool v = [] {
    const char *e = std::getenv("NCGM_HEIG_MID");
    return !(e && e[0] == '0');
  }();
  return v;
}

size_t heigScratchBytes(int m) {
  return std::max(heigMidScratchBytes(m), heigLargeScratchBytes(m));
}

void heig(const double2 *A, int lda, int m, double2 *work, double2 *V,
          double *w, int *perm, int *status, cudaStream_t s, bool fast,
          void *scratch, size_t scratchBytes) {
  // the Householder methods' scratch: the caller's, or stream-ordered
  auto withScratch = [&](size_t need, auto &&run) {
    if (scratch && scratchBytes >= need) {
      run(scratch);
      return true;
    }
    void *scr = nullptr;
    if (cudaMallocAsync(&scr, need, s) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    run(scr);
    cudaFreeAsync(scr, s);
    return true;
  };
  // the round-robin tables hold up to 256 pairs (m <= 512)
  constexpr size_t kMaxDyn = 210 * 1024; // + 14 KB static <= 227 KB
  static const bool attr = [] {
    cudaFuncSetAttribute(heigKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)kMaxDyn);
    return true;
  }();
  (void)attr;
  if (fast && m <= heigMidMax() && !heigFp64Only() && heigMidOn() &&
      withScratch(heigMidScratchBytes(m), [&](void *scr) {
        heigMid(A, lda, m, V, w, perm, status, scr, s);
      }))
    return;
  if (fast && m <= kHeigDfMax && !heigFp64Only()) {
    static const bool dfAttr = [] {
      cudaFuncSetAttribute(heigDfKernel,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           2 * kHeigDfMax * kHeigDfMax * (int)sizeof(dfc));
      return true;
    }();
    (void)dfAttr;
    const int threads = m <= 32 ? 128 : (m <= 48 ? 256 : 512);
    heigDfKernel<<<1, threads, 2 * (size_t)m * m * sizeof(dfc), s>>>(
        A, lda, m, V, w, perm, status);
    return;
  }
  // above the shared-memory tier: the multi-kernel solver over the whole
  // GPU
  if (m > kHeigDfMax && !heigFp64Only() &&
      withScratch(heigLargeScratchBytes(m), [&](void *scr) {
        heigLarge(A, lda, m, V, w, perm, status, scr, s);
      }))
    return;
  const size_t mat = (size_t)m * m * sizeof(double2);
  const int sm = 2 * mat <= kMaxDyn ? 2 : (mat <= kMaxDyn ? 1 : 0);
  const size_t smem = sm == 2 ? 2 * mat : (sm == 1 ? mat : 0);
  // a round updates m x m/2 elements between barriers: small problems run
  // with fewer warps, so each of the ~4 barriers per round is cheaper
  const int threads = m <= 32 ? 128 : (m <= 48 ? 256 : 512);
  heigKernel<<<1, threads, smem, s>>>(A, lda, m, work, V, w, perm, status,
                                      sm);
}

} // namespace ncgm
