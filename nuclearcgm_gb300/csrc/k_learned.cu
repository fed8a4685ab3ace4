// Learned preconditioner for the GCG correction step.
//
// The reference corrects each Ritz vector with Jacobi-preconditioned CG on
// (A + shift) w = x (lambda + shift) (src/solver/solver.cpp:723-745). In
// correction form that is (A + shift) d = r, r = x lambda - A x, w = x + d.
// Here a small 3-D convolutional network maps r (one real component at a
// time, scaled to unit RMS) together with the local fields (U + shift and
// the kinetic coefficient f / h^2) to an estimate d0 of d. The PCG then starts
// from alpha d0 instead of 0, alpha the step along d0 that minimises the CG
// energy (so the start is never worse than 0 in the A-norm the PCG
// minimises); a column with alpha <= 0 starts from 0 as before. The
// unmodified Jacobi PCG then runs to the reference's tolerance and the GCG
// still locks on the FP64 residual.
//
// Network: a 4-level U-Net, BF16 weights (round-to-nearest-even copies of
// FP32 master weights), FP32 activations and accumulation:
//   e0 = relu(conv3(x;  3->16))          D0 = n
//   e1 = relu(conv3(pool(e0); 16->16))   D1 = (D0+1)/2
//   e2 = relu(conv3(pool(e1); 16->32))   D2
//   e3 = relu(conv1(pool(e2); 32->64))   D3
//   g3 = relu(conv1(e3; 64->32))
//   g2 = relu(conv3(e2 + up(g3); 32->16))
//   g1 = relu(conv3(e1 + up(g2); 16->16))
//   y  = conv3(e0 + up(g1); 16->1)
// 47,489 parameters. Training (forward, backward, Adam) runs on the device
// with the kernels of this file on residual / exact-correction pairs that
// the solver itself produces (ncgm_lp_collect).
#include "k_learned.cuh"
#include "k_pcg.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

namespace ncgm {

bool isDevicePtr(const void *p);

namespace {

constexpr float kU = 50.f;   // MeV: scale of U + shift at the input
// MeV: scale of f / h^2 at the input (20.7 MeV fm^2 at h = 0.5 fm), so the
// network sees the kinetic scale of the lattice it runs on
constexpr float kK = 82.8f;
constexpr float kE = 10.f;   // MeV: d is predicted as d kE / rms(r)
constexpr int kNL = 8;

struct LayerDef {
  int cin, cout, k;
};
constexpr LayerDef kLayers[kNL] = {{3, 16, 3},  {16, 16, 3}, {16, 32, 3},
                                   {32, 64, 1}, {64, 32, 1}, {32, 16, 3},
                                   {16, 16, 3}, {16, 1, 3}};

int layerW(int l) {
  return kLayers[l].cout * kLayers[l].cin * kLayers[l].k * kLayers[l].k *
         kLayers[l].k;
}
int layerOff(int l) { // offset of layer l's weights (bias follows)
  int o = 0;
  for (int i = 0; i < l; ++i) o += layerW(i) + kLayers[i].cout;
  return o;
}
int numParams() { return layerOff(kNL); }

// ---------------------------------------------------------------- kernels
// 3x3x3 taps in (dk, dj, di) lexicographic order; tap t and 26 - t are
// opposite offsets.
__device__ __forceinline__ bool tapIndex(int i, int j, int k, int t, int D,
                                         int &q) {
  const int di = t % 3 - 1, dj = (t / 3) % 3 - 1, dk = t / 9 - 1;
  const int ii = i + di, jj = j + dj, kk = k + dk;
  if ((unsigned)ii >= (unsigned)D || (unsigned)jj >= (unsigned)D ||
      (unsigned)kk >= (unsigned)D)
    return false;
  q = (kk * D + jj) * D + ii;
  return true;
}

// out[b][o][p] = bias[o] + sum_c sum_t w(o, c, t) in[b][c][p + off_t]
// w(o, c, t) = W[o][c][t] (forward) or W[c][o][KK-1-t] (transposed: the
// data gradient of the layer, whose output channels are the layer's inputs)
template <int K, int COT>
__global__ void convKernel(const float *__restrict__ in, int Cin, int D,
                           const __nv_bfloat16 *__restrict__ Wq,
                           const float *__restrict__ bias, int Cout,
                           float *__restrict__ out, int relu, int transposed,
                           int layerCin, int layerCout) {
  constexpr int KK = K * K * K;
  extern __shared__ float ws[]; // [c][t][o], Cin * KK * COT
  const int o0 = blockIdx.y * COT, b = blockIdx.z;
  const int V = D * D * D;
  for (int e = threadIdx.x; e < Cin * KK * COT; e += blockDim.x) {
    const int o = e % COT, t = (e / COT) % KK, c = e / (COT * KK);
    float w = 0.f;
    if (o0 + o < Cout) {
      size_t idx = transposed
                       ? ((size_t)c * layerCin + (o0 + o)) * KK + (KK - 1 - t)
                       : ((size_t)(o0 + o) * layerCin + c) * KK + t;
      w = __bfloat162float(Wq[idx]);
    }
    ws[e] = w;
  }
  (void)layerCout;
  __syncthreads();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= V) return;
  const int i = p % D, j = (p / D) % D, k = p / (D * D);
  float acc[COT];
#pragma unroll
  for (int o = 0; o < COT; ++o)
    acc[o] = (bias && o0 + o < Cout) ? bias[o0 + o] : 0.f;
  for (int c = 0; c < Cin; ++c) {
    const float *src = in + ((size_t)b * Cin + c) * V;
#pragma unroll
    for (int t = 0; t < KK; ++t) {
      int q = p;
      float v = 0.f;
      if (K == 1 || tapIndex(i, j, k, t, D, q)) v = __ldg(src + q);
      const float *w = ws + ((size_t)c * KK + t) * COT;
#pragma unroll
      for (int o = 0; o < COT; ++o) acc[o] = fmaf(w[o], v, acc[o]);
    }
  }
#pragma unroll
  for (int o = 0; o < COT; ++o)
    if (o0 + o < Cout) {
      float r = acc[o];
      if (relu) r = fmaxf(r, 0.f);
      out[((size_t)b * Cout + o0 + o) * V + p] = r;
    }
}

// Partial weight/bias gradients of one (o, c) pair over one chunk of the
// (batch, voxel) range: part[(o Cin + c) nChunk + chunk][t], and for c == 0
// bpart[o nChunk + chunk].
template <int K>
__global__ void convWGradKernel(const float *__restrict__ dOut,
                                const float *__restrict__ in, int D, int B,
                                int Cin, int Cout, int nChunk,
                                float *__restrict__ part,
                                float *__restrict__ bpart) {
  constexpr int KK = K * K * K;
  __shared__ float red[8][KK + 1];
  const int oc = blockIdx.x, o = oc / Cin, c = oc % Cin;
  const int chunk = blockIdx.y;
  const int V = D * D * D;
  const long long total = (long long)B * V;
  const long long e0 = chunk * total / nChunk, e1 = (chunk + 1) * total / nChunk;
  float acc[KK + 1];
#pragma unroll
  for (int t = 0; t <= KK; ++t) acc[t] = 0.f;
  for (long long e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const int b = (int)(e / V), p = (int)(e % V);
    const float g = dOut[((size_t)b * Cout + o) * V + p];
    acc[KK] += g;
    const float *src = in + ((size_t)b * Cin + c) * V;
    const int i = p % D, j = (p / D) % D, k = p / (D * D);
#pragma unroll
    for (int t = 0; t < KK; ++t) {
      int q = p;
      if (K == 1 || tapIndex(i, j, k, t, D, q))
        acc[t] = fmaf(g, __ldg(src + q), acc[t]);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t <= KK; ++t) {
    float v = acc[t];
    for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
    if (lane == 0) red[warp][t] = v;
  }
  __syncthreads();
  const int nw = blockDim.x >> 5;
  if (threadIdx.x <= KK) {
    float v = 0.f;
    for (int w = 0; w < nw; ++w) v += red[w][threadIdx.x];
    if (threadIdx.x < KK)
      part[((size_t)oc * nChunk + chunk) * KK + threadIdx.x] = v;
    else if (c == 0)
      bpart[(size_t)o * nChunk + chunk] = v;
  }
}

__global__ void wGradReduce(const float *__restrict__ part,
                            const float *__restrict__ bpart, int nW, int KK,
                            int nChunk, int Cout, float *__restrict__ gW,
                            float *__restrict__ gB) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nW) {
    const int oc = e / KK, t = e % KK;
    float s = 0.f;
    for (int ch = 0; ch < nChunk; ++ch)
      s += part[((size_t)oc * nChunk + ch) * KK + t];
    gW[e] = s;
  } else if (e < nW + Cout) {
    const int o = e - nW;
    float s = 0.f;
    for (int ch = 0; ch < nChunk; ++ch) s += bpart[(size_t)o * nChunk + ch];
    gB[o] = s;
  }
}

// coarse q <- (1/8) sum of its children inside the fine lattice
__global__ void poolKernel(const float *__restrict__ in, int D, int Dc,
                           long long total, float *__restrict__ out) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       e < total; e += (long long)gridDim.x * blockDim.x) {
    const int Vc = Dc * Dc * Dc;
    const long long bc = e / Vc;
    const int q = (int)(e % Vc);
    const int i = q % Dc, j = (q / Dc) % Dc, k = q / (Dc * Dc);
    const float *src = in + bc * (long long)D * D * D;
    float s = 0.f;
    for (int dk = 0; dk < 2; ++dk)
      for (int dj = 0; dj < 2; ++dj)
        for (int di = 0; di < 2; ++di) {
          const int ii = 2 * i + di, jj = 2 * j + dj, kk = 2 * k + dk;
          if (ii < D && jj < D && kk < D) s += src[(kk * D + jj) * D + ii];
        }
    out[e] = s * 0.125f;
  }
}

__device__ __forceinline__ int parentOf(int p, int D, int Dc) {
  const int i = p % D, j = (p / D) % D, k = p / (D * D);
  return ((k >> 1) * Dc + (j >> 1)) * Dc + (i >> 1);
}

// out = a + up(c)  (fine lattice D, coarse Dc); total = B*C*D^3
__global__ void upAddKernel(const float *__restrict__ a,
                            const float *__restrict__ c, int D, int Dc,
                            long long total, float *__restrict__ out) {
  const int V = D * D * D, Vc = Dc * Dc * Dc;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       e < total; e += (long long)gridDim.x * blockDim.x) {
    const long long bc = e / V;
    const int p = (int)(e % V);
    out[e] = a[e] + c[bc * Vc + parentOf(p, D, Dc)];
  }
}

// g[q] = (sum over fine children of d) * (act[q] > 0), coarse total
__global__ void upBwdMaskKernel(const float *__restrict__ d, int D, int Dc,
                                const float *__restrict__ act, long long total,
                                float *__restrict__ g) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       e < total; e += (long long)gridDim.x * blockDim.x) {
    const int Vc = Dc * Dc * Dc;
    const long long bc = e / Vc;
    const int q = (int)(e % Vc);
    const int i = q % Dc, j = (q / Dc) % Dc, k = q / (Dc * Dc);
    const float *src = d + bc * (long long)D * D * D;
    float s = 0.f;
    for (int dk = 0; dk < 2; ++dk)
      for (int dj = 0; dj < 2; ++dj)
        for (int di = 0; di < 2; ++di) {
          const int ii = 2 * i + di, jj = 2 * j + dj, kk = 2 * k + dk;
          if (ii < D && jj < D && kk < D) s += src[(kk * D + jj) * D + ii];
        }
    g[e] = act[e] > 0.f ? s : 0.f;
  }
}

// d[p] = (d[p] + (1/8) c[parent(p)]) * (act[p] > 0); fine total
__global__ void poolBwdMaskKernel(float *__restrict__ d,
                                  const float *__restrict__ c, int D, int Dc,
                                  const float *__restrict__ act,
                                  long long total) {
  const int V = D * D * D, Vc = Dc * Dc * Dc;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       e < total; e += (long long)gridDim.x * blockDim.x) {
    const long long bc = e / V;
    const int p = (int)(e % V);
    const float v = d[e] + 0.125f * c[bc * Vc + parentOf(p, D, Dc)];
    d[e] = act[e] > 0.f ? v : 0.f;
  }
}

__global__ void reluMaskKernel(float *__restrict__ d,
                               const float *__restrict__ act, long long total) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       e < total; e += (long long)gridDim.x * blockDim.x)
    if (!(act[e] > 0.f)) d[e] = 0.f;
}

// per instance: loss_b = |y - t|^2 / (|t|^2 + 1e-30); dy = 2 (y - t) /
// ((|t|^2 + 1e-30) B). One block per instance, fixed-order reduction.
__global__ void lossKernel(const float *__restrict__ y,
                           const float *__restrict__ t, int V, int B,
                           float *__restrict__ dy, float *__restrict__ lossB) {
  __shared__ double sh[2][256];
  const int b = blockIdx.x;
  const float *yb = y + (size_t)b * V, *tb = t + (size_t)b * V;
  double num = 0, den = 0;
  for (int p = threadIdx.x; p < V; p += blockDim.x) {
    const double r = (double)yb[p] - tb[p];
    num += r * r;
    den += (double)tb[p] * tb[p];
  }
  sh[0][threadIdx.x] = num;
  sh[1][threadIdx.x] = den;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + s];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  const double dn = sh[1][0] + 1e-30;
  if (threadIdx.x == 0) lossB[b] = (float)(sh[0][0] / dn);
  if (dy) {
    const float sc = (float)(2.0 / (dn * B));
    for (int p = threadIdx.x; p < V; p += blockDim.x)
      dy[(size_t)b * V + p] = sc * (yb[p] - tb[p]);
  }
}

__global__ void meanKernel(const float *__restrict__ v, int n,
                           float *__restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += v[i];
    *out = (float)(s / n);
  }
}

__global__ void adamKernel(float *__restrict__ w, __nv_bfloat16 *__restrict__ wq,
                           float *__restrict__ m, float *__restrict__ v,
                           const float *__restrict__ g, int n, float lr,
                           float c1, float c2) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float gi = g[e];
  const float mi = b1 * m[e] + (1.f - b1) * gi;
  const float vi = b2 * v[e] + (1.f - b2) * gi * gi;
  m[e] = mi;
  v[e] = vi;
  const float wi = w[e] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[e] = wi;
  wq[e] = __float2bfloat16_rn(wi);
}

__global__ void quantKernel(const float *__restrict__ w,
                            __nv_bfloat16 *__restrict__ wq, int n) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) wq[e] = __float2bfloat16_rn(w[e]);
}

// RMS of each real component c of r = x lam - A x, one block per (col, c)
__global__ void residualRmsKernel(const double2 *__restrict__ X,
                                  const double2 *__restrict__ AX,
                                  const double *__restrict__ lam, size_t N,
                                  size_t ns, float *__restrict__ scale) {
  __shared__ double sh[256];
  const int jc = blockIdx.x, j = jc / 4, c = jc % 4;
  const int spin = c / 2, im = c % 2;
  const double l = lam[j];
  double s = 0;
  for (size_t p = threadIdx.x; p < ns; p += blockDim.x) {
    const size_t o = (size_t)j * N + 2 * p + spin;
    const double2 x = X[o], ax = AX[o];
    const double r = im ? x.y * l - ax.y : x.x * l - ax.x;
    s += r * r;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) scale[jc] = (float)sqrt(sh[0] / (double)ns);
}

// network inputs of instance b = 4 j + c: r_c / rms, (U + UC + shift) / kU,
// (f / h^2) / kK (U + UC = c0 - 7.5 c1 and f / h^2 = c1 from the
// coefficient table)
__global__ void packInputKernel(const double2 *__restrict__ X,
                                const double2 *__restrict__ AX,
                                const double *__restrict__ lam,
                                const float *__restrict__ scale,
                                const double *__restrict__ coef, double h2,
                                double shift, size_t N, size_t ns, int ncols,
                                float *__restrict__ x, size_t instStride) {
  const long long total = (long long)ncols * 4 * ns;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       e < total; e += (long long)gridDim.x * blockDim.x) {
    const int jc = (int)(e / ns);
    const size_t p = (size_t)(e % ns);
    const int j = jc / 4, c = jc % 4, spin = c / 2, im = c % 2;
    const size_t o = (size_t)j * N + 2 * p + spin;
    const double2 xv = X[o], ax = AX[o];
    const double r = im ? xv.y * lam[j] - ax.y : xv.x * lam[j] - ax.x;
    const float s = scale[jc];
    float *dst = x + (size_t)jc * instStride;
    dst[p] = s > 0.f ? (float)(r / s) : 0.f;
    const double c0 = coef[8 * p], c1 = coef[8 * p + 1];
    dst[ns + p] = (float)((c0 - 7.5 * c1 + shift) / kU);
    dst[2 * ns + p] = (float)(c1 / kK);
  }
}

// target of instance b = 4 j + c: (w - x)_c kE / rms
__global__ void packTargetKernel(const double2 *__restrict__ X,
                                 const double2 *__restrict__ Wv,
                                 const float *__restrict__ scale, size_t N,
                                 size_t ns, int ncols, float *__restrict__ t,
                                 size_t instStride) {
  const long long total = (long long)ncols * 4 * ns;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       e < total; e += (long long)gridDim.x * blockDim.x) {
    const int jc = (int)(e / ns);
    const size_t p = (size_t)(e % ns);
    const int j = jc / 4, c = jc % 4, spin = c / 2, im = c % 2;
    const size_t o = (size_t)j * N + 2 * p + spin;
    const double d = im ? Wv[o].y - X[o].y : Wv[o].x - X[o].x;
    const float s = scale[jc];
    t[(size_t)jc * instStride + p] = s > 0.f ? (float)(d * kE / s) : 0.f;
  }
}

template <class T> struct Cplx;
template <> struct Cplx<float> { using type = float2; };
template <> struct Cplx<double> { using type = double2; };

// d0 (column j, component c) = y[4 j + c] rms / kE
template <class T>
__global__ void unpackKernel(const float *__restrict__ y,
                             const float *__restrict__ scale, size_t N,
                             size_t ns, int ncols,
                             typename Cplx<T>::type *__restrict__ D0) {
  const long long total = (long long)ncols * ns * 2;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       e < total; e += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(e / (2 * ns));
    const size_t r = (size_t)(e % (2 * ns)), p = r / 2;
    const int spin = (int)(r % 2);
    const int c0 = 4 * j + 2 * spin;
    const float s0 = scale[c0] / kE, s1 = scale[c0 + 1] / kE;
    D0[(size_t)j * N + r] = {(T)(y[(size_t)c0 * ns + p] * s0),
                             (T)(y[(size_t)(c0 + 1) * ns + p] * s1)};
  }
}

// gather training instances idx[0..B) of a group into x (B x 3 x V) and
// t (B x V); the group stores [cap][4][V] (3 inputs then the target)
__global__ void gatherInstKernel(const float *__restrict__ data,
                                 const int *__restrict__ idx, int B, size_t V,
                                 float *__restrict__ x, float *__restrict__ t) {
  const long long total = (long long)B * 4 * V;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
       e < total; e += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(e / (4 * V));
    const size_t r = (size_t)(e % (4 * V));
    const float v = data[(size_t)idx[b] * 4 * V + r];
    if (r < 3 * V)
      x[(size_t)b * 3 * V + r] = v;
    else
      t[(size_t)b * V + (r - 3 * V)] = v;
  }
}

int blocksFor(long long total) {
  long long b = (total + 255) / 256;
  return (int)std::max<long long>(1, std::min<long long>(b, 4096));
}

} // namespace

// ------------------------------------------------------------- network
struct LpAct {
  int n = 0, B = 0;
  int D[4] = {0, 0, 0, 0};
  std::vector<float *> bufs;
  float *x, *e0, *d0, *y, *p1, *e1, *d1, *g1, *p2, *e2, *d2, *g2, *p3, *e3,
      *g3;
  // gradients
  float *dy, *dd0, *dg1, *dd1, *dg2, *dd2, *dg3, *de3, *dp3, *dp2, *dp1;
  float *t, *lossB;
  float *part = nullptr, *bpart = nullptr;
  size_t partCap = 0;
};

struct LpGroup {
  int n = 0, count = 0, cap = 0;
  float *data = nullptr; // [cap][4][n^3]
};

} // namespace ncgm

struct ncgm_lp {
  int device = 0;
  int P = 0;
  float *w = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;
  __nv_bfloat16 *wq = nullptr;
  int step = 0;
  cudaStream_t s = nullptr;
  std::map<std::pair<int, int>, ncgm::LpAct *> acts;
  std::vector<ncgm::LpGroup> groups;
  float *scratch = nullptr;
  size_t scratchCap = 0;
  float *dLoss = nullptr;
  int *dIdx = nullptr;
  int idxCap = 0;
  std::mutex mu; // one user at a time (batched runs may share a network)
  // recorded after each inference on the caller's stream: the next caller,
  // possibly on another stream, waits for it before reusing the activations
  cudaEvent_t done = nullptr;
  bool doneRecorded = false;
};

namespace ncgm {

namespace {

float *devAlloc(size_t count) {
  void *p = nullptr;
  if (cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(float)) !=
      cudaSuccess)
    return nullptr;
  return static_cast<float *>(p);
}

LpAct *actsFor(ncgm_lp *lp, int n, int B) {
  auto key = std::make_pair(n, B);
  auto it = lp->acts.find(key);
  if (it != lp->acts.end()) return it->second;
  auto *a = new LpAct;
  a->n = n;
  a->B = B;
  a->D[0] = n;
  for (int l = 1; l < 4; ++l) a->D[l] = (a->D[l - 1] + 1) / 2;
  size_t V[4];
  for (int l = 0; l < 4; ++l) V[l] = (size_t)a->D[l] * a->D[l] * a->D[l];
  bool ok = true;
  auto take = [&](size_t count) {
    float *p = devAlloc(count);
    if (!p) ok = false;
    a->bufs.push_back(p);
    return p;
  };
  const size_t b = B;
  a->x = take(b * 3 * V[0]);
  a->e0 = take(b * 16 * V[0]);
  a->d0 = take(b * 16 * V[0]);
  a->y = take(b * V[0]);
  a->p1 = take(b * 16 * V[1]);
  a->e1 = take(b * 16 * V[1]);
  a->d1 = take(b * 16 * V[1]);
  a->g1 = take(b * 16 * V[1]);
  a->p2 = take(b * 16 * V[2]);
  a->e2 = take(b * 32 * V[2]);
  a->d2 = take(b * 32 * V[2]);
  a->g2 = take(b * 16 * V[2]);
  a->p3 = take(b * 32 * V[3]);
  a->e3 = take(b * 64 * V[3]);
  a->g3 = take(b * 32 * V[3]);
  a->dy = take(b * V[0]);
  a->dd0 = take(b * 16 * V[0]);
  a->dg1 = take(b * 16 * V[1]);
  a->dd1 = take(b * 16 * V[1]);
  a->dg2 = take(b * 16 * V[2]);
  a->dd2 = take(b * 32 * V[2]);
  a->dg3 = take(b * 32 * V[3]);
  a->de3 = take(b * 64 * V[3]);
  a->dp3 = take(b * 32 * V[3]);
  a->dp2 = take(b * 16 * V[2]);
  a->dp1 = take(b * 16 * V[1]);
  a->t = take(b * V[0]);
  a->lossB = take(b);
  if (!ok) {
    for (float *p : a->bufs) cudaFree(p);
    delete a;
    return nullptr;
  }
  lp->acts[key] = a;
  return a;
}

template <int K, int COT>
void launchConv(const float *in, int Cin, int D, int B,
                const __nv_bfloat16 *Wq, const float *bias, int Cout,
                float *out, bool relu, bool transposed, int layerCin,
                int layerCout, cudaStream_t s) {
  const int V = D * D * D;
  const size_t smem = (size_t)Cin * K * K * K * COT * sizeof(float);
  static const bool attr = [] {
    cudaFuncSetAttribute(convKernel<K, COT>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         100 * 1024);
    return true;
  }();
  (void)attr;
  dim3 grid((V + 127) / 128, (Cout + COT - 1) / COT, B);
  convKernel<K, COT><<<grid, 128, smem, s>>>(in, Cin, D, Wq, bias, Cout, out,
                                             relu ? 1 : 0, transposed ? 1 : 0,
                                             layerCin, layerCout);
}

// forward of layer l: in (B, cin, D) -> out (B, cout, D)
void convFwd(ncgm_lp *lp, int l, const float *in, int D, int B, float *out,
             bool relu, cudaStream_t s) {
  const LayerDef L = kLayers[l];
  const __nv_bfloat16 *Wq = lp->wq + layerOff(l);
  const float *bias = lp->w + layerOff(l) + layerW(l);
  if (L.k == 3) {
    if (L.cout % 16 == 0)
      launchConv<3, 16>(in, L.cin, D, B, Wq, bias, L.cout, out, relu, false,
                        L.cin, L.cout, s);
    else
      launchConv<3, 1>(in, L.cin, D, B, Wq, bias, L.cout, out, relu, false,
                       L.cin, L.cout, s);
  } else {
    launchConv<1, 16>(in, L.cin, D, B, Wq, bias, L.cout, out, relu, false,
                      L.cin, L.cout, s);
  }
}

// data gradient of layer l: dOut (B, cout, D) -> dIn (B, cin, D)
void convBwdData(ncgm_lp *lp, int l, const float *dOut, int D, int B,
                 float *dIn, cudaStream_t s) {
  const LayerDef L = kLayers[l];
  const __nv_bfloat16 *Wq = lp->wq + layerOff(l);
  if (L.k == 3)
    launchConv<3, 16>(dOut, L.cout, D, B, Wq, nullptr, L.cin, dIn, false, true,
                      L.cin, L.cout, s);
  else
    launchConv<1, 16>(dOut, L.cout, D, B, Wq, nullptr, L.cin, dIn, false, true,
                      L.cin, L.cout, s);
}

// weight and bias gradients of layer l into lp->g
int convBwdW(ncgm_lp *lp, LpAct *a, int l, const float *dOut, const float *in,
             int D, int B, cudaStream_t s) {
  const LayerDef L = kLayers[l];
  const int KK = L.k * L.k * L.k;
  const int pairs = L.cout * L.cin;
  const long long total = (long long)B * D * D * D;
  int nChunk = (int)std::max<long long>(
      1, std::min<long long>({(608 + pairs - 1) / pairs, 64, total / 256}));
  const size_t need = (size_t)pairs * nChunk * KK, needB = (size_t)L.cout * nChunk;
  if (a->partCap < need + needB) {
    if (a->part) cudaFree(a->part);
    a->part = devAlloc(need + needB);
    if (!a->part) {
      a->partCap = 0;
      return NCGM_ERR_NOMEM;
    }
    a->partCap = need + needB;
  }
  a->bpart = a->part + need;
  dim3 grid(pairs, nChunk);
  if (L.k == 3)
    convWGradKernel<3><<<grid, 256, 0, s>>>(dOut, in, D, B, L.cin, L.cout,
                                            nChunk, a->part, a->bpart);
  else
    convWGradKernel<1><<<grid, 256, 0, s>>>(dOut, in, D, B, L.cin, L.cout,
                                            nChunk, a->part, a->bpart);
  const int nW = layerW(l);
  float *gW = lp->g + layerOff(l);
  wGradReduce<<<(nW + L.cout + 255) / 256, 256, 0, s>>>(
      a->part, a->bpart, nW, KK, nChunk, L.cout, gW, gW + nW);
  return NCGM_OK;
}

// x (B x 3 x n^3) already in a->x; result y in a->y
void forward(ncgm_lp *lp, LpAct *a, cudaStream_t s) {
  const int B = a->B;
  const int *D = a->D;
  auto V = [&](int l) { return (long long)D[l] * D[l] * D[l]; };
  convFwd(lp, 0, a->x, D[0], B, a->e0, true, s);
  poolKernel<<<blocksFor(B * 16 * V(1)), 256, 0, s>>>(a->e0, D[0], D[1],
                                                      B * 16 * V(1), a->p1);
  convFwd(lp, 1, a->p1, D[1], B, a->e1, true, s);
  poolKernel<<<blocksFor(B * 16 * V(2)), 256, 0, s>>>(a->e1, D[1], D[2],
                                                      B * 16 * V(2), a->p2);
  convFwd(lp, 2, a->p2, D[2], B, a->e2, true, s);
  poolKernel<<<blocksFor(B * 32 * V(3)), 256, 0, s>>>(a->e2, D[2], D[3],
                                                      B * 32 * V(3), a->p3);
  convFwd(lp, 3, a->p3, D[3], B, a->e3, true, s);
  convFwd(lp, 4, a->e3, D[3], B, a->g3, true, s);
  upAddKernel<<<blocksFor(B * 32 * V(2)), 256, 0, s>>>(
      a->e2, a->g3, D[2], D[3], B * 32 * V(2), a->d2);
  convFwd(lp, 5, a->d2, D[2], B, a->g2, true, s);
  upAddKernel<<<blocksFor(B * 16 * V(1)), 256, 0, s>>>(
      a->e1, a->g2, D[1], D[2], B * 16 * V(1), a->d1);
  convFwd(lp, 6, a->d1, D[1], B, a->g1, true, s);
  upAddKernel<<<blocksFor(B * 16 * V(0)), 256, 0, s>>>(
      a->e0, a->g1, D[0], D[1], B * 16 * V(0), a->d0);
  convFwd(lp, 7, a->d0, D[0], B, a->y, false, s);
}

// loss of a->y against a->t; gradients of every parameter into lp->g
int backward(ncgm_lp *lp, LpAct *a, float *lossOut, cudaStream_t s) {
  const int B = a->B;
  const int *D = a->D;
  auto V = [&](int l) { return (long long)D[l] * D[l] * D[l]; };
  lossKernel<<<B, 256, 0, s>>>(a->y, a->t, (int)V(0), B, a->dy, a->lossB);
  if (lossOut) meanKernel<<<1, 32, 0, s>>>(a->lossB, B, lossOut);
  // y = conv(d0; W7)
  NCGM_TRY(convBwdW(lp, a, 7, a->dy, a->d0, D[0], B, s));
  convBwdData(lp, 7, a->dy, D[0], B, a->dd0, s); // = de0 (skip) + up-path
  upBwdMaskKernel<<<blocksFor(B * 16 * V(1)), 256, 0, s>>>(
      a->dd0, D[0], D[1], a->g1, B * 16 * V(1), a->dg1);
  // g1 = relu(conv(d1; W6))
  NCGM_TRY(convBwdW(lp, a, 6, a->dg1, a->d1, D[1], B, s));
  convBwdData(lp, 6, a->dg1, D[1], B, a->dd1, s);
  upBwdMaskKernel<<<blocksFor(B * 16 * V(2)), 256, 0, s>>>(
      a->dd1, D[1], D[2], a->g2, B * 16 * V(2), a->dg2);
  // g2 = relu(conv(d2; W5))
  NCGM_TRY(convBwdW(lp, a, 5, a->dg2, a->d2, D[2], B, s));
  convBwdData(lp, 5, a->dg2, D[2], B, a->dd2, s);
  upBwdMaskKernel<<<blocksFor(B * 32 * V(3)), 256, 0, s>>>(
      a->dd2, D[2], D[3], a->g3, B * 32 * V(3), a->dg3);
  // g3 = relu(conv1(e3; W4))
  NCGM_TRY(convBwdW(lp, a, 4, a->dg3, a->e3, D[3], B, s));
  convBwdData(lp, 4, a->dg3, D[3], B, a->de3, s);
  reluMaskKernel<<<blocksFor(B * 64 * V(3)), 256, 0, s>>>(a->de3, a->e3,
                                                         B * 64 * V(3));
  // e3 = relu(conv1(p3; W3))
  NCGM_TRY(convBwdW(lp, a, 3, a->de3, a->p3, D[3], B, s));
  convBwdData(lp, 3, a->de3, D[3], B, a->dp3, s);
  // de2 = (dd2 + poolT(dp3)) * (e2 > 0)
  poolBwdMaskKernel<<<blocksFor(B * 32 * V(2)), 256, 0, s>>>(
      a->dd2, a->dp3, D[2], D[3], a->e2, B * 32 * V(2));
  NCGM_TRY(convBwdW(lp, a, 2, a->dd2, a->p2, D[2], B, s));
  convBwdData(lp, 2, a->dd2, D[2], B, a->dp2, s);
  poolBwdMaskKernel<<<blocksFor(B * 16 * V(1)), 256, 0, s>>>(
      a->dd1, a->dp2, D[1], D[2], a->e1, B * 16 * V(1));
  NCGM_TRY(convBwdW(lp, a, 1, a->dd1, a->p1, D[1], B, s));
  convBwdData(lp, 1, a->dd1, D[1], B, a->dp1, s);
  poolBwdMaskKernel<<<blocksFor(B * 16 * V(0)), 256, 0, s>>>(
      a->dd0, a->dp1, D[0], D[1], a->e0, B * 16 * V(0));
  NCGM_TRY(convBwdW(lp, a, 0, a->dd0, a->x, D[0], B, s));
  return NCGM_OK;
}

float *scratch(ncgm_lp *lp, size_t count) {
  if (lp->scratchCap < count) {
    if (lp->scratch) cudaFree(lp->scratch);
    lp->scratch = devAlloc(count);
    lp->scratchCap = lp->scratch ? count : 0;
  }
  return lp->scratch;
}

uint64_t splitmix(uint64_t &st) {
  uint64_t z = (st += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double uniform01(uint64_t &st) {
  return ((splitmix(st) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

LpGroup *groupFor(ncgm_lp *lp, int n) {
  for (auto &g : lp->groups)
    if (g.n == n) return &g;
  lp->groups.push_back(LpGroup{n, 0, 0, nullptr});
  return &lp->groups.back();
}

bool growGroup(LpGroup &g, int need) {
  if (g.count + need <= g.cap) return true;
  const size_t V = (size_t)g.n * g.n * g.n;
  int cap = std::max(g.cap * 2, g.count + need);
  cap = std::max(cap, 64);
  float *p = devAlloc((size_t)cap * 4 * V);
  if (!p) return false;
  if (g.data) {
    cudaMemcpy(p, g.data, (size_t)g.count * 4 * V * sizeof(float),
               cudaMemcpyDeviceToDevice);
    cudaFree(g.data);
  }
  g.data = p;
  g.cap = cap;
  return true;
}

} // namespace

template <class T>
int lpInitialCorrection(ncgm_lp *lp, ncgm_ctx *ctx, int species,
                        const double2 *X, const double2 *AX, const double *lam,
                        double shift, int ncols, T *D0, cudaStream_t s) {
  if (!lp) {
    setError("learned preconditioner: no network bound to the context");
    return NCGM_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(lp->mu);
  const int n = ctx->n;
  const size_t ns = ctx->ns, N = ctx->N;
  const int B = 4 * ncols;
  LpAct *a = actsFor(lp, n, B);
  float *scale = scratch(lp, (size_t)B);
  if (!a || !scale) return NCGM_ERR_NOMEM;
  if (lp->doneRecorded) NCGM_CUDA(cudaStreamWaitEvent(s, lp->done, 0));
  residualRmsKernel<<<B, 256, 0, s>>>(X, AX, lam, N, ns, scale);
  packInputKernel<<<blocksFor((long long)B * ns), 256, 0, s>>>(
      X, AX, lam, scale, ctx->sp[species].coef64, ctx->h * ctx->h, shift, N,
      ns, ncols, a->x, 3 * ns);
  forward(lp, a, s);
  unpackKernel<T><<<blocksFor((long long)ncols * 2 * ns), 256, 0, s>>>(
      a->y, scale, N, ns, ncols,
      reinterpret_cast<typename Cplx<T>::type *>(D0));
  NCGM_CUDA(cudaGetLastError());
  NCGM_CUDA(cudaEventRecord(lp->done, s));
  lp->doneRecorded = true;
  return NCGM_OK;
}

template int lpInitialCorrection<float>(ncgm_lp *, ncgm_ctx *, int,
                                        const double2 *, const double2 *,
                                        const double *, double, int, float *,
                                        cudaStream_t);
template int lpInitialCorrection<double>(ncgm_lp *, ncgm_ctx *, int,
                                         const double2 *, const double2 *,
                                         const double *, double, int,
                                         double *, cudaStream_t);

} // namespace ncgm

using namespace ncgm;

namespace {

bool onLpDevice(ncgm_lp *lp) {
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != lp->device) {
    setError("learned preconditioner: called on another device");
    return false;
  }
  return true;
}

int copyIn(float *dst, const float *src, size_t count, cudaStream_t s) {
  NCGM_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(float),
                            isDevicePtr(src) ? cudaMemcpyDeviceToDevice
                                       : cudaMemcpyHostToDevice,
                            s));
  return NCGM_OK;
}
int copyOut(float *dst, const float *src, size_t count, cudaStream_t s) {
  NCGM_CUDA(cudaMemcpyAsync(dst, src, count * sizeof(float),
                            isDevicePtr(dst) ? cudaMemcpyDeviceToDevice
                                       : cudaMemcpyDeviceToHost,
                            s));
  return NCGM_OK;
}

} // namespace

extern "C" {

int ncgm_lp_num_params(void) { return numParams(); }

int ncgm_lp_create(ncgm_lp **out, unsigned long long seed) {
  if (!out) {
    setError("ncgm_lp_create: null handle");
    return NCGM_ERR_ARG;
  }
  *out = nullptr;
  auto *lp = new ncgm_lp;
  cudaGetDevice(&lp->device);
  lp->P = numParams();
  lp->w = devAlloc(lp->P);
  lp->m = devAlloc(lp->P);
  lp->v = devAlloc(lp->P);
  lp->g = devAlloc(lp->P);
  lp->dLoss = devAlloc(1 << 16);
  void *q = nullptr;
  const bool ok = lp->w && lp->m && lp->v && lp->g && lp->dLoss &&
                  cudaMalloc(&q, lp->P * sizeof(__nv_bfloat16)) == cudaSuccess &&
                  cudaStreamCreateWithFlags(&lp->s, cudaStreamNonBlocking) ==
                      cudaSuccess &&
                  cudaEventCreateWithFlags(&lp->done, cudaEventDisableTiming) ==
                      cudaSuccess;
  lp->wq = static_cast<__nv_bfloat16 *>(q);
  if (!ok) {
    ncgm_lp_destroy(lp);
    setError("ncgm_lp_create: device allocation failed");
    return NCGM_ERR_NOMEM;
  }
  // He-normal weights (splitmix64 + Box-Muller), zero biases
  std::vector<float> h(lp->P, 0.f);
  uint64_t st = seed ? seed : 0x5eedull;
  for (int l = 0; l < kNL; ++l) {
    const int fan = kLayers[l].cin * kLayers[l].k * kLayers[l].k * kLayers[l].k;
    const double sd = std::sqrt(2.0 / fan);
    float *w = h.data() + layerOff(l);
    for (int e = 0; e < layerW(l); ++e) {
      const double u1 = uniform01(st), u2 = uniform01(st);
      w[e] = (float)(sd * std::sqrt(-2.0 * std::log(u1)) *
                     std::cos(6.283185307179586 * u2));
    }
  }
  int rc = ncgm_lp_set_params(lp, h.data());
  if (rc != NCGM_OK) {
    ncgm_lp_destroy(lp);
    return rc;
  }
  *out = lp;
  return NCGM_OK;
}

int ncgm_lp_destroy(ncgm_lp *lp) {
  if (!lp) return NCGM_OK;
  cudaFree(lp->w);
  cudaFree(lp->m);
  cudaFree(lp->v);
  cudaFree(lp->g);
  cudaFree(lp->wq);
  cudaFree(lp->dLoss);
  cudaFree(lp->dIdx);
  cudaFree(lp->scratch);
  for (auto &kv : lp->acts) {
    for (float *p : kv.second->bufs) cudaFree(p);
    cudaFree(kv.second->part);
    delete kv.second;
  }
  for (auto &g : lp->groups) cudaFree(g.data);
  if (lp->s) cudaStreamDestroy(lp->s);
  if (lp->done) cudaEventDestroy(lp->done);
  delete lp;
  return NCGM_OK;
}

int ncgm_lp_set_params(ncgm_lp *lp, const float *theta) {
  if (!lp || !theta) {
    setError("ncgm_lp_set_params: bad argument");
    return NCGM_ERR_ARG;
  }
  if (!onLpDevice(lp)) return NCGM_ERR_ARG;
  NCGM_TRY(copyIn(lp->w, theta, lp->P, lp->s));
  quantKernel<<<(lp->P + 255) / 256, 256, 0, lp->s>>>(lp->w, lp->wq, lp->P);
  NCGM_CUDA(cudaMemsetAsync(lp->m, 0, lp->P * sizeof(float), lp->s));
  NCGM_CUDA(cudaMemsetAsync(lp->v, 0, lp->P * sizeof(float), lp->s));
  lp->step = 0;
  NCGM_CUDA(cudaStreamSynchronize(lp->s));
  return NCGM_OK;
}

int ncgm_lp_get_params(ncgm_lp *lp, float *theta) {
  if (!lp || !theta) {
    setError("ncgm_lp_get_params: bad argument");
    return NCGM_ERR_ARG;
  }
  if (!onLpDevice(lp)) return NCGM_ERR_ARG;
  NCGM_TRY(copyOut(theta, lp->w, lp->P, lp->s));
  NCGM_CUDA(cudaStreamSynchronize(lp->s));
  return NCGM_OK;
}

int ncgm_lp_forward(ncgm_lp *lp, int n, int batch, const float *x, float *y) {
  if (!lp || n < 2 || batch < 1 || !x || !y) {
    setError("ncgm_lp_forward: bad argument");
    return NCGM_ERR_ARG;
  }
  if (!onLpDevice(lp)) return NCGM_ERR_ARG;
  LpAct *a = actsFor(lp, n, batch);
  if (!a) return NCGM_ERR_NOMEM;
  const size_t V = (size_t)n * n * n;
  NCGM_TRY(copyIn(a->x, x, (size_t)batch * 3 * V, lp->s));
  forward(lp, a, lp->s);
  NCGM_TRY(copyOut(y, a->y, (size_t)batch * V, lp->s));
  NCGM_CUDA(cudaStreamSynchronize(lp->s));
  NCGM_CUDA(cudaGetLastError());
  return NCGM_OK;
}

int ncgm_lp_gradient(ncgm_lp *lp, int n, int batch, const float *x,
                     const float *t, float *loss, float *grad) {
  if (!lp || n < 2 || batch < 1 || !x || !t || !grad) {
    setError("ncgm_lp_gradient: bad argument");
    return NCGM_ERR_ARG;
  }
  if (!onLpDevice(lp)) return NCGM_ERR_ARG;
  LpAct *a = actsFor(lp, n, batch);
  if (!a) return NCGM_ERR_NOMEM;
  const size_t V = (size_t)n * n * n;
  NCGM_TRY(copyIn(a->x, x, (size_t)batch * 3 * V, lp->s));
  NCGM_TRY(copyIn(a->t, t, (size_t)batch * V, lp->s));
  forward(lp, a, lp->s);
  NCGM_TRY(backward(lp, a, lp->dLoss, lp->s));
  NCGM_TRY(copyOut(grad, lp->g, lp->P, lp->s));
  float l = 0;
  NCGM_CUDA(cudaMemcpyAsync(&l, lp->dLoss, sizeof(float),
                            cudaMemcpyDeviceToHost, lp->s));
  NCGM_CUDA(cudaStreamSynchronize(lp->s));
  NCGM_CUDA(cudaGetLastError());
  if (loss) *loss = l;
  return NCGM_OK;
}

int ncgm_lp_collect(ncgm_lp *lp, ncgm_ctx *ctx, int species, const double *X,
                    int ncols, const double *lambda, double shift,
                    int cg_steps, double cg_tol) {
  if (!lp || !ctx || species < 0 || species > 1 || !X || !lambda ||
      ncols < 1 || ncols > ctx->max_cols || cg_steps < 1 || cg_tol < 0) {
    setError("ncgm_lp_collect: bad argument");
    return NCGM_ERR_ARG;
  }
  if (!ctx->sp[species].ready) {
    setError("ncgm_lp_collect: fields not set for this species");
    return NCGM_ERR_ARG;
  }
  if (!onLpDevice(lp)) return NCGM_ERR_ARG;
  std::lock_guard<std::mutex> lock(lp->mu);
  cudaStream_t s = ctx->stream;
  const size_t N = ctx->N, ns = ctx->ns;
  // device copies of X and the exact-correction workspace
  double2 *buf = static_cast<double2 *>(
      ctx->buf(30, N * (size_t)ncols * sizeof(double2) * 8 + 4096 * 16));
  if (!buf) return NCGM_ERR_NOMEM;
  double2 *Xd = buf, *AX = Xd + N * ncols, *Wv = AX + N * ncols,
          *R = Wv + N * ncols, *Z = R + N * ncols, *Pp = Z + N * ncols,
          *AP = Pp + N * ncols, *Wd = AP + N * ncols;
  char *tail = reinterpret_cast<char *>(Wd + N * ncols);
  double *dLs = reinterpret_cast<double *>(tail);
  double *dLam = dLs + ncols;
  PcgCol *st = reinterpret_cast<PcgCol *>(dLam + ncols);
  const int nblk = pcgBlocks(N);
  double *pp1 = static_cast<double *>(ctx->buf(
      31, sizeof(double) * ((size_t)ncols * nblk * 5 + 64 + ncols)));
  // (live and the finished-column counter follow the partial sums)
  if (!pp1) return NCGM_ERR_NOMEM;
  double *pp2 = pp1 + (size_t)ncols * nblk * 3;
  int *live = reinterpret_cast<int *>(pp2 + (size_t)ncols * nblk * 2);
  NCGM_CUDA(cudaMemcpyAsync(Xd, X, N * ncols * sizeof(double2),
                            cudaMemcpyDefault, s));
  std::vector<double> ls(ncols);
  for (int j = 0; j < ncols; ++j) ls[j] = lambda[j] + shift;
  NCGM_CUDA(cudaMemcpyAsync(dLs, ls.data(), ncols * sizeof(double),
                            cudaMemcpyHostToDevice, s));
  NCGM_CUDA(cudaMemcpyAsync(dLam, lambda, ncols * sizeof(double),
                            cudaMemcpyDefault, s));
  NCGM_CUDA(cudaMemsetAsync(live, 0, 2 * sizeof(int), s));
  applyH64(ctx, species, Xd, AX, ncols, 0.0, s);
  // exact correction: FP64 correction-form PCG run to a tight tolerance
  PcgPlan<double> pl;
  pl.N = N;
  pl.ncols = ncols;
  pl.X = Xd;
  pl.ldx = N;
  pl.X64 = Xd;
  pl.AX64 = AX;
  pl.W64 = Wv;
  pl.W = Wd;
  pl.R = R;
  pl.Z = Z;
  pl.P = Pp;
  pl.AP = AP;
  pl.lamShift = dLs;
  pl.coef = jacobiDiagonal(ctx, species, s);
  pl.arrive = reinterpret_cast<unsigned *>(live + 2);
  if (!pl.coef) return NCGM_ERR_NOMEM;
  pl.shift = shift;
  pl.tol = cg_tol;
  pl.maxSteps = cg_steps;
  pl.st = st;
  pl.partials = pp1;
  pl.partials2 = pp2;
  pl.live = live;
  pl.ndone = live + 1;
  pl.apply = [&](const void *Xi, size_t, void *Yo, int cols, double sh,
                 cudaStream_t stm) {
    applyH64(ctx, species, static_cast<const double2 *>(Xi),
             static_cast<double2 *>(Yo), cols, sh, stm);
  };
  pcgRun<double>(pl, s);
  // append 4 ncols instances to the lattice group
  LpGroup *g = groupFor(lp, ctx->n);
  NCGM_CUDA(cudaStreamSynchronize(s));
  if (!growGroup(*g, 4 * ncols)) return NCGM_ERR_NOMEM;
  float *scale = scratch(lp, (size_t)4 * ncols);
  if (!scale) return NCGM_ERR_NOMEM;
  const size_t V = ns;
  float *base = g->data + (size_t)g->count * 4 * V;
  residualRmsKernel<<<4 * ncols, 256, 0, s>>>(Xd, AX, dLam, N, ns, scale);
  packInputKernel<<<blocksFor((long long)4 * ncols * ns), 256, 0, s>>>(
      Xd, AX, dLam, scale, ctx->sp[species].coef64, ctx->h * ctx->h, shift, N,
      ns, ncols, base, 4 * V);
  packTargetKernel<<<blocksFor((long long)4 * ncols * ns), 256, 0, s>>>(
      Xd, Wv, scale, N, ns, ncols, base + 3 * V, 4 * V);
  // keep the columns whose exact solve converged (an indefinite H + shift,
  // e.g. far from the eigenpairs, gives no usable target)
  std::vector<PcgCol> hs(ncols);
  NCGM_CUDA(cudaMemcpyAsync(hs.data(), st, sizeof(PcgCol) * ncols,
                            cudaMemcpyDeviceToHost, s));
  NCGM_CUDA(cudaStreamSynchronize(s));
  int kept = 0;
  for (int j = 0; j < ncols; ++j) {
    if (!hs[j].done || hs[j].zero) continue;
    if (kept != j)
      NCGM_CUDA(cudaMemcpyAsync(base + (size_t)kept * 16 * V,
                                base + (size_t)j * 16 * V,
                                sizeof(float) * 16 * V,
                                cudaMemcpyDeviceToDevice, s));
    ++kept;
  }
  NCGM_CUDA(cudaStreamSynchronize(s));
  NCGM_CUDA(cudaGetLastError());
  g->count += 4 * kept;
  return NCGM_OK;
}

int ncgm_lp_dataset_size(ncgm_lp *lp, int n) {
  if (!lp) return 0;
  for (auto &g : lp->groups)
    if (g.n == n) return g.count;
  return 0;
}

int ncgm_lp_train(ncgm_lp *lp, int steps, int batch, double lr,
                  unsigned long long seed, float *loss_curve) {
  if (!lp || steps < 1 || steps > (1 << 16) || batch < 1 || lr <= 0) {
    setError("ncgm_lp_train: bad argument");
    return NCGM_ERR_ARG;
  }
  if (!onLpDevice(lp)) return NCGM_ERR_ARG;
  long long total = 0;
  for (auto &g : lp->groups) total += g.count;
  if (total == 0) {
    setError("ncgm_lp_train: no training pairs (ncgm_lp_collect first)");
    return NCGM_ERR_ARG;
  }
  if (lp->idxCap < batch) {
    cudaFree(lp->dIdx);
    void *p = nullptr;
    if (cudaMalloc(&p, sizeof(int) * batch) != cudaSuccess)
      return NCGM_ERR_NOMEM;
    lp->dIdx = static_cast<int *>(p);
    lp->idxCap = batch;
  }
  uint64_t st = seed ? seed : 1;
  std::vector<int> idx(batch);
  cudaStream_t s = lp->s;
  for (int it = 0; it < steps; ++it) {
    // group with probability proportional to its pair count
    long long pick = (long long)(uniform01(st) * total);
    LpGroup *g = &lp->groups[0];
    for (auto &gg : lp->groups) {
      if (pick < gg.count) {
        g = &gg;
        break;
      }
      pick -= gg.count;
    }
    for (int b = 0; b < batch; ++b)
      idx[b] = std::min(g->count - 1, (int)(uniform01(st) * g->count));
    LpAct *a = actsFor(lp, g->n, batch);
    if (!a) return NCGM_ERR_NOMEM;
    NCGM_CUDA(cudaMemcpyAsync(lp->dIdx, idx.data(), sizeof(int) * batch,
                              cudaMemcpyHostToDevice, s));
    const size_t V = (size_t)g->n * g->n * g->n;
    gatherInstKernel<<<blocksFor((long long)batch * 4 * V), 256, 0, s>>>(
        g->data, lp->dIdx, batch, V, a->x, a->t);
    forward(lp, a, s);
    NCGM_TRY(backward(lp, a, lp->dLoss + it, s));
    lp->step += 1;
    const float c1 = 1.f - std::pow(0.9f, (float)lp->step);
    const float c2 = 1.f - std::pow(0.999f, (float)lp->step);
    adamKernel<<<(lp->P + 255) / 256, 256, 0, s>>>(
        lp->w, lp->wq, lp->m, lp->v, lp->g, lp->P, (float)lr, c1, c2);
    // the host index list is reused next step
    NCGM_CUDA(cudaStreamSynchronize(s));
  }
  if (loss_curve)
    NCGM_CUDA(cudaMemcpy(loss_curve, lp->dLoss, sizeof(float) * steps,
                         cudaMemcpyDeviceToHost));
  NCGM_CUDA(cudaGetLastError());
  return NCGM_OK;
}

int ncgm_lp_eval(ncgm_lp *lp, int n, double *mean_loss) {
  if (!lp || !mean_loss) {
    setError("ncgm_lp_eval: bad argument");
    return NCGM_ERR_ARG;
  }
  if (!onLpDevice(lp)) return NCGM_ERR_ARG;
  LpGroup *g = nullptr;
  for (auto &gg : lp->groups)
    if (gg.n == n) g = &gg;
  if (!g || g->count == 0) {
    setError("ncgm_lp_eval: no pairs for this lattice");
    return NCGM_ERR_ARG;
  }
  const int B = std::min(g->count, 64);
  LpAct *a = actsFor(lp, n, B);
  if (!a) return NCGM_ERR_NOMEM;
  if (lp->idxCap < B) {
    cudaFree(lp->dIdx);
    void *p = nullptr;
    if (cudaMalloc(&p, sizeof(int) * B) != cudaSuccess) return NCGM_ERR_NOMEM;
    lp->dIdx = static_cast<int *>(p);
    lp->idxCap = B;
  }
  const size_t V = (size_t)n * n * n;
  double sum = 0;
  int done = 0;
  std::vector<int> idx(B);
  std::vector<float> lb(B);
  cudaStream_t s = lp->s;
  while (done < g->count) {
    const int cnt = std::min(B, g->count - done);
    for (int b = 0; b < B; ++b) idx[b] = done + std::min(b, cnt - 1);
    NCGM_CUDA(cudaMemcpyAsync(lp->dIdx, idx.data(), sizeof(int) * B,
                              cudaMemcpyHostToDevice, s));
    gatherInstKernel<<<blocksFor((long long)B * 4 * V), 256, 0, s>>>(
        g->data, lp->dIdx, B, V, a->x, a->t);
    forward(lp, a, s);
    lossKernel<<<B, 256, 0, s>>>(a->y, a->t, (int)V, B, nullptr, a->lossB);
    NCGM_CUDA(cudaMemcpyAsync(lb.data(), a->lossB, sizeof(float) * B,
                              cudaMemcpyDeviceToHost, s));
    NCGM_CUDA(cudaStreamSynchronize(s));
    for (int b = 0; b < cnt; ++b) sum += lb[b];
    done += cnt;
  }
  *mean_loss = sum / g->count;
  return NCGM_OK;
}

int ncgm_set_lp(ncgm_ctx *ctx, ncgm_lp *lp) {
  if (!ctx) {
    setError("ncgm_set_lp: null context");
    return NCGM_ERR_ARG;
  }
  ctx->lp = lp;
  return NCGM_OK;
}

} // extern "C"
