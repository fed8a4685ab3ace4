// Batched Jacobi-preconditioned conjugate gradients: the GCG correction step
// of gcgm_complex_no_B_lock (src/solver/solver.cpp:723-745), one independent
// system (A + shift I) w_k = x_k (lambda_k + shift) per active column with
// initial guess x_k. The iteration and stopping rule are those of Eigen's
// ConjugateGradient with DiagonalPreconditioner (textbook PCG, Saad Alg. 9.1):
// stop when |r|^2 < max(tol^2 |b|^2, DBL_MIN) or after cg_steps iterations.
// All columns advance together; a converged column is frozen by its flag.
// Reductions are deterministic (per-block partials summed in a fixed order).
// Vectors are FP64 (plain form) or FP32 (mixed form, dots in FP64).
#include "k_pcg.cuh"

#include <type_traits>

#include <cfloat>
#include <chrono>
#include <cstdlib>
#include <mutex>
#include <vector>

namespace ncgm {

namespace {

constexpr int kThreads = 256;

template <class T> struct C2;
template <> struct C2<double> { using type = double2; };
template <> struct C2<float> { using type = float2; };

__device__ double blockSum(double v, double *sh) {
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

// inverse Jacobi diagonal: diag = c0 + shift, c0 = U + UC + 7.5 f / h^2
// (the diagonal of H, one double per lattice point)
__device__ inline double invDiag(const double *c0, size_t p, double shift) {
  double d = c0[p] + shift;
  return d != 0.0 ? 1.0 / d : 1.0;
}

// Last-block test of a per-column reduction: every block has written its
// partial before it arrives; the block that arrives last sees all of them
// and resets the counter for the next use.
__device__ inline bool lastArrival(unsigned *counter, int nblk) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned prev = atomicAdd(counter, 1u);
    last = (prev == (unsigned)nblk - 1);
    if (last) *counter = 0;
  }
  __syncthreads();
  if (last) __threadfence();
  return last;
}

// r = b - T, b = x (lam+shift), z = Minv r, p = z, w = x; partials |b|^2,
// |r|^2, Re(r^H z).
template <class T>
__global__ void pcgInitKernel(const typename C2<T>::type *X, size_t ldx,
                              const typename C2<T>::type *Tx,
                              typename C2<T>::type *Wv,
                              typename C2<T>::type *R, typename C2<T>::type *Z,
                              typename C2<T>::type *P, size_t N,
                              const double *lamShift, const double *coef,
                              double shift, double *partials, int nblk) {
  __shared__ double sh[kThreads];
  const int col = blockIdx.y;
  const double ls = lamShift[col];
  double bb = 0, rr = 0, rz = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x) {
    size_t o = (size_t)col * N + i;
    auto x = X[(size_t)col * ldx + i];
    auto t = Tx[o];
    double bx = (double)x.x * ls, by = (double)x.y * ls;
    double rx = bx - (double)t.x, ry = by - (double)t.y;
    double m = invDiag(coef, i / 2, shift);
    double zx = m * rx, zy = m * ry;
    bb += bx * bx + by * by;
    rr += rx * rx + ry * ry;
    rz += rx * zx + ry * zy;
    Wv[o] = x;
    R[o] = {(T)rx, (T)ry};
    Z[o] = {(T)zx, (T)zy};
    P[o] = {(T)zx, (T)zy};
  }
  double s0 = blockSum(bb, sh), s1 = blockSum(rr, sh), s2 = blockSum(rz, sh);
  if (threadIdx.x == 0) {
    double *pp = partials + (size_t)col * nblk * 3;
    pp[blockIdx.x] = s0;
    pp[nblk + blockIdx.x] = s1;
    pp[2 * nblk + blockIdx.x] = s2;
  }
}

// Correction form (mixed precision): solve (A + shift) d = b - (A + shift) x
// from d = 0 with the initial residual r0 = x lam - A x evaluated in FP64
// (b = x (lam + shift)); algebraically the same iterates as PCG on w with
// guess x, w = x + d, but d carries only the correction so its FP32 rounding
// stays relative to the correction, not to w.
template <class T>
__global__ void pcgInitCorrKernel(const double2 *X64, const double2 *AX64,
                                  typename C2<T>::type *Dv,
                                  typename C2<T>::type *R,
                                  typename C2<T>::type *Z,
                                  typename C2<T>::type *P, size_t N,
                                  const double *lamShift, const double *coef,
                                  double shift, double *partials, int nblk) {
  __shared__ double sh[kThreads];
  const int col = blockIdx.y;
  const double ls = lamShift[col], lam = ls - shift;
  double bb = 0, rr = 0, rz = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x) {
    size_t o = (size_t)col * N + i;
    double2 x = X64[o], ax = AX64[o];
    double bx = x.x * ls, by = x.y * ls;
    double rx = x.x * lam - ax.x, ry = x.y * lam - ax.y;
    double m = invDiag(coef, i / 2, shift);
    double zx = m * rx, zy = m * ry;
    bb += bx * bx + by * by;
    rr += rx * rx + ry * ry;
    rz += rx * zx + ry * zy;
    Dv[o] = {(T)0, (T)0};
    R[o] = {(T)rx, (T)ry};
    Z[o] = {(T)zx, (T)zy};
    P[o] = {(T)zx, (T)zy};
  }
  double s0 = blockSum(bb, sh), s1 = blockSum(rr, sh), s2 = blockSum(rz, sh);
  if (threadIdx.x == 0) {
    double *pp = partials + (size_t)col * nblk * 3;
    pp[blockIdx.x] = s0;
    pp[nblk + blockIdx.x] = s1;
    pp[2 * nblk + blockIdx.x] = s2;
  }
}

// partials of Re(d0^H r0) and Re(d0^H T) per column, r0 = x lam - A x
// (FP64), T = (A + shift) d0 for the learned initial correction d0
template <class T>
__global__ void pcgNetNormKernel(const double2 *X64, const double2 *AX64,
                                 const typename C2<T>::type *D0,
                                 const typename C2<T>::type *Td, size_t N,
                                 const double *lamShift, double shift,
                                 double *partials, int nblk) {
  __shared__ double sh[kThreads];
  const int col = blockIdx.y;
  const double lam = lamShift[col] - shift;
  double a = 0, b = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x) {
    size_t o = (size_t)col * N + i;
    double2 x = X64[o], ax = AX64[o];
    auto d = D0[o];
    auto t = Td[o];
    double rx = x.x * lam - ax.x, ry = x.y * lam - ax.y;
    a += (double)d.x * rx + (double)d.y * ry;
    b += (double)d.x * t.x + (double)d.y * t.y;
  }
  double s0 = blockSum(a, sh), s1 = blockSum(b, sh);
  if (threadIdx.x == 0) {
    double *pp = partials + (size_t)col * nblk * 2;
    pp[blockIdx.x] = s0;
    pp[nblk + blockIdx.x] = s1;
  }
}

// Correction-form start from the learned d0, scaled by the step that
// minimises the CG energy Phi(d) = d^H (A + shift) d / 2 - Re(d^H r0) along
// d0: alpha = Re(d0^H r0) / Re(d0^H (A + shift) d0). Phi(alpha d0) <= Phi(0),
// so the start is never worse than the reference's d = 0 in the A-norm the
// PCG minimises; a column with alpha <= 0 (or a non-positive curvature)
// starts from 0. d = alpha d0, r = r0 - alpha T, z = Minv r, p = z.
template <class T>
__global__ void pcgInitNetKernel(const double2 *X64, const double2 *AX64,
                                 const typename C2<T>::type *D0,
                                 const typename C2<T>::type *Td,
                                 typename C2<T>::type *Dv,
                                 typename C2<T>::type *R,
                                 typename C2<T>::type *Z,
                                 typename C2<T>::type *P, size_t N,
                                 const double *lamShift, const double *coef,
                                 double shift, const double *normPart,
                                 double *partials, int nblk, int *useNet) {
  __shared__ double sh[kThreads];
  __shared__ double alpha;
  const int col = blockIdx.y;
  if (threadIdx.x == 0) {
    const double *pp = normPart + (size_t)col * nblk * 2;
    double dr = 0, dad = 0;
    for (int k = 0; k < nblk; ++k) {
      dr += pp[k];
      dad += pp[nblk + k];
    }
    alpha = (dr > 0.0 && dad > 0.0) ? dr / dad : 0.0;
    if (blockIdx.x == 0 && useNet) useNet[col] = alpha > 0.0;
  }
  __syncthreads();
  const double al = alpha;
  const double ls = lamShift[col], lam = ls - shift;
  double bb = 0, rr = 0, rz = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x) {
    size_t o = (size_t)col * N + i;
    double2 x = X64[o], ax = AX64[o];
    double bx = x.x * ls, by = x.y * ls;
    double rx = x.x * lam - ax.x, ry = x.y * lam - ax.y;
    auto d0 = D0[o];
    auto t = Td[o];
    rx -= al * (double)t.x;
    ry -= al * (double)t.y;
    double m = invDiag(coef, i / 2, shift);
    double zx = m * rx, zy = m * ry;
    bb += bx * bx + by * by;
    rr += rx * rx + ry * ry;
    rz += rx * zx + ry * zy;
    Dv[o] = {(T)(al * (double)d0.x), (T)(al * (double)d0.y)};
    R[o] = {(T)rx, (T)ry};
    Z[o] = {(T)zx, (T)zy};
    P[o] = {(T)zx, (T)zy};
  }
  double s0 = blockSum(bb, sh), s1 = blockSum(rr, sh), s2 = blockSum(rz, sh);
  if (threadIdx.x == 0) {
    double *pp = partials + (size_t)col * nblk * 3;
    pp[blockIdx.x] = s0;
    pp[nblk + blockIdx.x] = s1;
    pp[2 * nblk + blockIdx.x] = s2;
  }
}

// w = x + d (FP64 result); a column with b = 0 returns w = 0
template <class T>
__global__ void pcgCombineKernel(const double2 *X64,
                                 const typename C2<T>::type *Dv, double2 *W64,
                                 size_t N, const PcgCol *st, int onlyD) {
  const int col = blockIdx.y;
  const bool zero = st[col].zero;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x) {
    size_t o = (size_t)col * N + i;
    auto d = Dv[o];
    double2 x = onlyD ? make_double2(0.0, 0.0) : X64[o];
    W64[o] = zero ? make_double2(0.0, 0.0)
                  : make_double2(x.x + (double)d.x, x.y + (double)d.y);
  }
}

__global__ void pcgInitFinish(PcgCol *st, const double *partials, int nblk,
                              double tol, int *ndone) {
  const int col = blockIdx.x;
  if (threadIdx.x != 0) return;
  const double *pp = partials + (size_t)col * nblk * 3;
  double bb = 0, rr = 0, rz = 0;
  for (int b = 0; b < nblk; ++b) {
    bb += pp[b];
    rr += pp[nblk + b];
    rz += pp[2 * nblk + b];
  }
  PcgCol c;
  c.rhsNorm2 = bb;
  c.thr = fmax(tol * tol * bb, DBL_MIN);
  c.absNew = rz;
  c.absOld = rz;
  c.beta = 0;
  c.iters = 0;
  c.zero = (bb == 0.0);
  c.done = (bb == 0.0) || (rr < c.thr);
  st[col] = c;
  if (c.done && ndone) atomicAdd(ndone, 1);
}

// partial p^H Ap (complex)
template <class T>
__global__ void pcgDotKernel(const typename C2<T>::type *P,
                             const typename C2<T>::type *AP, size_t N,
                             PcgCol *st, double *partials, int nblk,
                             unsigned *arrive) {
  __shared__ double sh[kThreads];
  const int col = blockIdx.y;
  if (st[col].done) return;
  double re = 0, im = 0;
  if (std::is_same<T, float>::value) {
    // FP32 form: per-thread sums in FP32, block sums in FP64
    float re32 = 0.f, im32 = 0.f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
         i += (size_t)gridDim.x * blockDim.x) {
      const size_t o = (size_t)col * N + i;
      const auto p = P[o];
      const auto a = AP[o];
      re32 += (float)p.x * (float)a.x + (float)p.y * (float)a.y;
      im32 += (float)p.x * (float)a.y - (float)p.y * (float)a.x;
    }
    re = re32;
    im = im32;
  } else {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
         i += (size_t)gridDim.x * blockDim.x) {
      size_t o = (size_t)col * N + i;
      auto p = P[o];
      auto a = AP[o];
      re += (double)p.x * a.x + (double)p.y * a.y;
      im += (double)p.x * a.y - (double)p.y * a.x;
    }
  }
  double s0 = blockSum(re, sh), s1 = blockSum(im, sh);
  double *pp = partials + (size_t)col * nblk * 3;
  if (threadIdx.x == 0) {
    pp[blockIdx.x] = s0;
    pp[nblk + blockIdx.x] = s1;
  }
  // the last block sums the partials in block order: alpha = absNew / p^H Ap
  // the last block sums the partials. FP32 plans: with all its threads (one
  // L2 round trip, then a fixed-order tree; a serial sum was a chain of
  // ~nblk L2 latencies per PCG step). FP64 plans keep the serial block order,
  // the rounding path the FP64 parity tests were validated on.
  if (lastArrival(&arrive[col], nblk)) {
    double r = 0, m = 0;
    if (std::is_same<T, float>::value) {
      for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
        r += __ldcg(pp + b);
        m += __ldcg(pp + nblk + b);
      }
      r = blockSum(r, sh);
      m = blockSum(m, sh);
    } else if (threadIdx.x == 0) {
      for (int b = 0; b < nblk; ++b) {
        r += ((volatile double *)pp)[b];
        m += ((volatile double *)pp)[nblk + b];
      }
    }
    if (threadIdx.x == 0) {
      const double den = r * r + m * m;
      const double a = st[col].absNew;
      st[col].alphaR = a * r / den;
      st[col].alphaI = -a * m / den;
    }
  }
}

// w += alpha p; r -= alpha Ap; z = Minv r; partials |r|^2 and Re(r^H z);
// the last block to finish a column takes the stopping decision and the
// next beta (the column's finish step)
template <class T>
__global__ void pcgUpdateKernel(typename C2<T>::type *Wv,
                                typename C2<T>::type *R,
                                typename C2<T>::type *Z,
                                const typename C2<T>::type *P,
                                const typename C2<T>::type *AP, size_t N,
                                PcgCol *st, const double *diag, double shift,
                                const float *invd, double *partials2,
                                int nblk, unsigned *arrive, int *live,
                                int *ndone) {
  __shared__ double sh[kThreads];
  const int col = blockIdx.y;
  if (st[col].done) return;
  const double alr = st[col].alphaR, ali = st[col].alphaI;
  double rr = 0, rz = 0;
  if (std::is_same<T, float>::value && invd) {
    // FP32 form: the element arithmetic in FP32 (the vectors are FP32; the
    // FP64 pipe of GB300 retires 2 FMAs per clock per SM), per-thread sums
    // in FP32 over a handful of elements, block sums in FP64
    const float fr = (float)alr, fi = (float)ali;
    float rr32 = 0.f, rz32 = 0.f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
         i += (size_t)gridDim.x * blockDim.x) {
      const size_t o = (size_t)col * N + i;
      const auto p = P[o];
      const auto a = AP[o];
      const auto w = Wv[o];
      const auto r = R[o];
      const float wx = (float)w.x + (fr * (float)p.x - fi * (float)p.y);
      const float wy = (float)w.y + (fr * (float)p.y + fi * (float)p.x);
      const float rx = (float)r.x - (fr * (float)a.x - fi * (float)a.y);
      const float ry = (float)r.y - (fr * (float)a.y + fi * (float)a.x);
      const float m = invd[i / 2];
      const float zx = m * rx, zy = m * ry;
      Wv[o] = {(T)wx, (T)wy};
      R[o] = {(T)rx, (T)ry};
      Z[o] = {(T)zx, (T)zy};
      rr32 += rx * rx + ry * ry;
      rz32 += rx * zx + ry * zy;
    }
    rr = rr32;
    rz = rz32;
  } else {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
         i += (size_t)gridDim.x * blockDim.x) {
      size_t o = (size_t)col * N + i;
      auto p = P[o];
      auto a = AP[o];
      auto w = Wv[o];
      auto r = R[o];
      double px = p.x, py = p.y, ax = a.x, ay = a.y;
      double wx = (double)w.x + (alr * px - ali * py);
      double wy = (double)w.y + (alr * py + ali * px);
      double rx = (double)r.x - (alr * ax - ali * ay);
      double ry = (double)r.y - (alr * ay + ali * ax);
      double m = invDiag(diag, i / 2, shift);
      double zx = m * rx, zy = m * ry;
      Wv[o] = {(T)wx, (T)wy};
      R[o] = {(T)rx, (T)ry};
      Z[o] = {(T)zx, (T)zy};
      rr += rx * rx + ry * ry;
      rz += rx * zx + ry * zy;
    }
  }
  double s0 = blockSum(rr, sh), s1 = blockSum(rz, sh);
  double *pp = partials2 + (size_t)col * nblk * 2;
  if (threadIdx.x == 0) {
    pp[blockIdx.x] = s0;
    pp[nblk + blockIdx.x] = s1;
  }
  if (lastArrival(&arrive[col], nblk)) {
    double tr = 0, tz = 0;
    if (std::is_same<T, float>::value) { // see pcgDotKernel
      for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
        tr += __ldcg(pp + b);
        tz += __ldcg(pp + nblk + b);
      }
      tr = blockSum(tr, sh);
      tz = blockSum(tz, sh);
    } else if (threadIdx.x == 0) {
      for (int b = 0; b < nblk; ++b) {
        tr += ((volatile double *)pp)[b];
        tz += ((volatile double *)pp)[nblk + b];
      }
    }
    if (threadIdx.x != 0) return;
    PcgCol c = st[col];
    if (tr < c.thr) {
      c.done = 1;
      if (ndone) atomicAdd(ndone, 1);
    } else {
      c.absOld = c.absNew;
      c.absNew = tz;
      c.beta = c.absNew / c.absOld;
      c.iters += 1;
      atomicAdd(live, 1);
    }
    st[col] = c;
  }
}

template <class T>
__global__ void pcgPKernel(typename C2<T>::type *P,
                           const typename C2<T>::type *Z, size_t N,
                           const PcgCol *st) {
  const int col = blockIdx.y;
  if (st[col].done) return;
  const double b = st[col].beta;
  const float b32 = (float)b;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x) {
    size_t o = (size_t)col * N + i;
    auto z = Z[o];
    auto p = P[o];
    if (std::is_same<T, float>::value)
      P[o] = {(T)((float)z.x + b32 * (float)p.x),
              (T)((float)z.y + b32 * (float)p.y)};
    else
      P[o] = {(T)((double)z.x + b * p.x), (T)((double)z.y + b * p.y)};
  }
}

template <class T>
__global__ void pcgZeroKernel(typename C2<T>::type *Wv, size_t N,
                              const PcgCol *st) {
  const int col = blockIdx.y;
  if (!st[col].zero) return;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x)
    Wv[(size_t)col * N + i] = {(T)0, (T)0};
}

} // namespace

constexpr int kLag = 2, kPollSlots = 4096;
struct ExitPoll {
  int device = -1;
  int *host = nullptr;        // pinned, kPollSlots
  int *hostDev = nullptr;     // the device's address of host
  int *counter = nullptr;     // device: the next slot to write
  cudaEvent_t done = nullptr; // after the last write of the previous user
};
// A pool of pinned slot arrays and event rings, per device: a PCG run takes
// one out and returns it when it ends. The pool outlives short-lived host
// threads (the HF driver solves the protons on a new thread each iteration),
// so nothing is allocated per thread.
std::mutex g_pollMutex;
std::vector<ExitPoll *> g_pollFree;

ExitPoll *exitPollTake() {
  int dev = 0;
  cudaGetDevice(&dev);
  {
    std::lock_guard<std::mutex> lock(g_pollMutex);
    for (size_t i = 0; i < g_pollFree.size(); ++i)
      if (g_pollFree[i]->device == dev) {
        ExitPoll *p = g_pollFree[i];
        g_pollFree.erase(g_pollFree.begin() + (long)i);
        // the previous user's last copies into p->host have landed
        cudaEventSynchronize(p->done);
        return p;
      }
  }
  auto *p = new ExitPoll;
  p->device = dev;
  if (cudaHostAlloc(reinterpret_cast<void **>(&p->host),
                    sizeof(int) * kPollSlots, cudaHostAllocMapped) !=
          cudaSuccess ||
      cudaHostGetDevicePointer(reinterpret_cast<void **>(&p->hostDev),
                               p->host, 0) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void **>(&p->counter), sizeof(int)) !=
          cudaSuccess) {
    cudaGetLastError();
    if (p->host) cudaFreeHost(p->host);
    delete p;
    return nullptr;
  }
  cudaEventCreateWithFlags(&p->done, cudaEventDisableTiming);
  return p;
}

// back to the pool once the copies queued on s have completed
void exitPollGive(ExitPoll *p, cudaStream_t s) {
  if (!p) return;
  cudaEventRecord(p->done, s);
  std::lock_guard<std::mutex> lock(g_pollMutex);
  g_pollFree.push_back(p);
}

namespace {
// the count of finished columns into the next host slot (one thread, after
// a step's kernels): the host reads it without a copy or an event
__global__ void pcgMarkKernel(const int *ndone, int *hostSlots,
                              int *counter) {
  const int k = *counter;
  *counter = k + 1;
  if (k < kPollSlots) {
    *(volatile int *)(hostSlots + k) = *(volatile const int *)ndone;
    __threadfence_system();
  }
}

__global__ void invDiag32Kernel(const double *c0, double shift, size_t ns,
                                float *inv) {
  const size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (p < ns) inv[p] = (float)invDiag(c0, p, shift);
}
} // namespace

void inverseDiagonal32(const double *c0, double shift, size_t ns, float *inv,
                       cudaStream_t s) {
  invDiag32Kernel<<<(unsigned)((ns + 255) / 256), 256, 0, s>>>(c0, shift, ns,
                                                               inv);
}

int pcgBlocks(size_t N) {
  size_t b = (N + kThreads * 4 - 1) / (kThreads * 4);
  if (b > 128) b = 128;
  if (b < 1) b = 1;
  return (int)b;
}

template <class T>
void pcgRun(const PcgPlan<T> &pl, cudaStream_t s) {
  const int nblk = pcgBlocks(pl.N);
  dim3 grid(nblk, pl.ncols);
  using V = typename C2<T>::type;
  if (pl.AX64 && pl.D0) {
    // T = (A + shift) d0 into AP (free until the first step)
    pl.apply(pl.D0, pl.N, pl.AP, pl.ncols, pl.shift, s);
    pcgNetNormKernel<T><<<grid, kThreads, 0, s>>>(
        pl.X64, pl.AX64, reinterpret_cast<const V *>(pl.D0),
        reinterpret_cast<const V *>(pl.AP), pl.N, pl.lamShift, pl.shift,
        pl.partials2, nblk);
    pcgInitNetKernel<T><<<grid, kThreads, 0, s>>>(
        pl.X64, pl.AX64, reinterpret_cast<const V *>(pl.D0),
        reinterpret_cast<const V *>(pl.AP), reinterpret_cast<V *>(pl.W),
        reinterpret_cast<V *>(pl.R), reinterpret_cast<V *>(pl.Z),
        reinterpret_cast<V *>(pl.P), pl.N, pl.lamShift, pl.coef, pl.shift,
        pl.partials2, pl.partials, nblk, pl.useNet);
  } else if (pl.AX64) {
    pcgInitCorrKernel<T><<<grid, kThreads, 0, s>>>(
        pl.X64, pl.AX64, reinterpret_cast<V *>(pl.W),
        reinterpret_cast<V *>(pl.R), reinterpret_cast<V *>(pl.Z),
        reinterpret_cast<V *>(pl.P), pl.N, pl.lamShift, pl.coef, pl.shift,
        pl.partials, nblk);
  } else {
    // T = (A + shift) X
    pl.apply(pl.X, pl.ldx, pl.AP, pl.ncols, pl.shift, s);
    pcgInitKernel<T><<<grid, kThreads, 0, s>>>(
        reinterpret_cast<const V *>(pl.X), pl.ldx,
        reinterpret_cast<const V *>(pl.AP), reinterpret_cast<V *>(pl.W),
        reinterpret_cast<V *>(pl.R), reinterpret_cast<V *>(pl.Z),
        reinterpret_cast<V *>(pl.P), pl.N, pl.lamShift, pl.coef, pl.shift,
        pl.partials, nblk);
  }
  if (pl.ndone) cudaMemsetAsync(pl.ndone, 0, sizeof(int), s);
  cudaMemsetAsync(pl.arrive, 0, 2 * sizeof(unsigned) * pl.ncols, s);
  pcgInitFinish<<<pl.ncols, 32, 0, s>>>(pl.st, pl.partials, nblk, pl.tol,
                                        pl.ndone);
  // Early exit: after the init and after every step a one-thread kernel
  // writes the count of finished columns into the next slot of mapped
  // pinned host memory (slot 0 after the init, it + 1 after step it); the
  // host marks a slot unwritten (-1) before it launches the step that
  // writes it. Before step `it` the host reads the slot of step it - kLag
  // (so the device queue never drains) and stops issuing steps once every
  // column has finished. Later steps would only launch no-op kernels.
  ExitPoll *poll = pl.ndone ? exitPollTake() : nullptr;
  auto mark = [&]() {
    if (poll) pcgMarkKernel<<<1, 1, 0, s>>>(pl.ndone, poll->hostDev,
                                           poll->counter);
  };
  if (poll) {
    cudaMemsetAsync(poll->counter, 0, sizeof(int), s);
    poll->host[0] = -1;
    poll->host[1] = -1;
  }
  mark();
  // waits (bounded, ~10 s, then for the stream) until the slot is written
  auto readSlot = [&](int slot) -> int {
    volatile int *h = poll->host + slot;
    const auto t0 = std::chrono::steady_clock::now();
    for (unsigned spin = 0; *h == -1; ++spin) {
      if ((spin & 1023u) == 0 &&
          std::chrono::steady_clock::now() - t0 > std::chrono::seconds(10)) {
        cudaStreamSynchronize(s);
        break;
      }
    }
    return *h;
  };
  auto step = [&]() {
    pl.apply(pl.P, pl.N, pl.AP, pl.ncols, pl.shift, s);
    pcgDotKernel<T><<<grid, kThreads, 0, s>>>(
        reinterpret_cast<const V *>(pl.P), reinterpret_cast<const V *>(pl.AP),
        pl.N, pl.st, pl.partials, nblk, pl.arrive);
    pcgUpdateKernel<T><<<grid, kThreads, 0, s>>>(
        reinterpret_cast<V *>(pl.W), reinterpret_cast<V *>(pl.R),
        reinterpret_cast<V *>(pl.Z), reinterpret_cast<const V *>(pl.P),
        reinterpret_cast<const V *>(pl.AP), pl.N, pl.st, pl.coef, pl.shift,
        pl.invd, pl.partials2, nblk, pl.arrive + pl.ncols, pl.live,
        pl.ndone);
    pcgPKernel<T><<<grid, kThreads, 0, s>>>(
        reinterpret_cast<V *>(pl.P), reinterpret_cast<const V *>(pl.Z), pl.N,
        pl.st);
    mark();
  };
  // One step is the same five launches with the same arguments every time:
  // after a first direct step (which also settles the stencil's tuned
  // shape), it is captured once into a CUDA graph and replayed, one graph
  // launch per step. NCGM_PCG_GRAPH=0 keeps direct launches.
  const char *genv = std::getenv("NCGM_PCG_GRAPH");
  const bool useGraph = !(genv && genv[0] == '0');
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool graphFailed = false;
  for (int it = 0; it < pl.maxSteps; ++it) {
    if (poll && it + 1 - kLag >= 0 && it + 1 - kLag < kPollSlots &&
        readSlot(it + 1 - kLag) >= pl.ncols)
      break;
    if (poll && it + 2 < kPollSlots) poll->host[it + 2] = -1;
    if (useGraph && it > 0 && !exec && !graphFailed) {
      if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) ==
          cudaSuccess) {
        step();
        if (cudaStreamEndCapture(s, &graph) != cudaSuccess ||
            cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
          graphFailed = true;
          exec = nullptr;
        }
      } else {
        graphFailed = true;
      }
      cudaGetLastError();
    }
    if (exec)
      cudaGraphLaunch(exec, s);
    else
      step();
  }
  exitPollGive(poll, s);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (pl.AX64)
    pcgCombineKernel<T><<<grid, kThreads, 0, s>>>(
        pl.X64, reinterpret_cast<const V *>(pl.W), pl.W64, pl.N, pl.st,
        pl.onlyCorrection ? 1 : 0);
  else
    pcgZeroKernel<T><<<grid, kThreads, 0, s>>>(reinterpret_cast<V *>(pl.W),
                                               pl.N, pl.st);
}

template void pcgRun<double>(const PcgPlan<double> &, cudaStream_t);
template void pcgRun<float>(const PcgPlan<float> &, cudaStream_t);

} // namespace ncgm
