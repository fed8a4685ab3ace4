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
// Two kernels:
//  * stencilPoint<T>: one thread per (point, column), neighbours through the
//    L1/L2 caches. Used for FP64, where GB300's FP64 pipe (not HBM) bounds it.
//  * stencilPlanes32: the FP32 HBM-bound kernel. A CTA owns one column, a
//    band of TY lattice rows and a chunk of z planes; each (sub)plane of the
//    band (+-2 halo rows) is contiguous in the Eigen layout and is fetched with
//    one TMA bulk copy (cp.async.bulk + mbarrier) into a shared-memory ring.
//    Outputs stream back with coalesced 16-byte stores.
#include "ncgm_internal.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

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

template <class T> struct Spinor {
  T r0, i0, r1, i1;
};

template <class T>
__device__ __forceinline__ Spinor<T> ldSpinor(const typename V4<T>::type *p) {
  typename V4<T>::type v = *p;
  return {v.x, v.y, v.z, v.w};
}

// Core arithmetic of one output point. c: coefficients (see
// SpeciesFields), v: centre, xp/xm/... neighbours (zero outside the box).
template <class T>
__device__ __forceinline__ Spinor<T>
pointH(const T c[8], T shift, const Spinor<T> &v, const Spinor<T> &xp1,
       const Spinor<T> &xm1, const Spinor<T> &xp2, const Spinor<T> &xm2,
       const Spinor<T> &yp1, const Spinor<T> &ym1, const Spinor<T> &yp2,
       const Spinor<T> &ym2, const Spinor<T> &zp1, const Spinor<T> &zm1,
       const Spinor<T> &zp2, const Spinor<T> &zm2) {
  const T d = c[0] + shift, fk = c[1];
  const T gx = c[2], gy = c[3], gz = c[4];
  const T wx = c[5], wy = c[6], wz = c[7];
  const T c43 = T(4) / T(3), c112 = T(1) / T(12);
  Spinor<T> o;
#define NCGM_COMP(m)                                                           \
  {                                                                            \
    T s1 = (xp1.m + xm1.m) + (yp1.m + ym1.m) + (zp1.m + zm1.m);                \
    T s2 = (xp2.m + xm2.m) + (yp2.m + ym2.m) + (zp2.m + zm2.m);                \
    o.m = d * v.m - fk * (c43 * s1 - c112 * s2);                               \
  }
  NCGM_COMP(r0)
  NCGM_COMP(i0)
  NCGM_COMP(r1)
  NCGM_COMP(i1)
#undef NCGM_COMP
  Spinor<T> Dx, Dy, Dz;
#define NCGM_D(D, p1, m1, p2, m2, m)                                           \
  D.m = T(8) * (p1.m - m1.m) - (p2.m - m2.m);
  NCGM_D(Dx, xp1, xm1, xp2, xm2, r0) NCGM_D(Dx, xp1, xm1, xp2, xm2, i0)
  NCGM_D(Dx, xp1, xm1, xp2, xm2, r1) NCGM_D(Dx, xp1, xm1, xp2, xm2, i1)
  NCGM_D(Dy, yp1, ym1, yp2, ym2, r0) NCGM_D(Dy, yp1, ym1, yp2, ym2, i0)
  NCGM_D(Dy, yp1, ym1, yp2, ym2, r1) NCGM_D(Dy, yp1, ym1, yp2, ym2, i1)
  NCGM_D(Dz, zp1, zm1, zp2, zm2, r0) NCGM_D(Dz, zp1, zm1, zp2, zm2, i0)
  NCGM_D(Dz, zp1, zm1, zp2, zm2, r1) NCGM_D(Dz, zp1, zm1, zp2, zm2, i1)
#undef NCGM_D
  // non-local kinetic: -grad f . D psi
  o.r0 += gx * Dx.r0 + gy * Dy.r0 + gz * Dz.r0;
  o.i0 += gx * Dx.i0 + gy * Dy.i0 + gz * Dz.i0;
  o.r1 += gx * Dx.r1 + gy * Dy.r1 + gz * Dz.r1;
  o.i1 += gx * Dx.i1 + gy * Dy.i1 + gz * Dz.i1;
  // spin-orbit: -i sum_a (sigma x W)_a D_a psi
  // x: -i(sy Wz - sz Wy) = [[i Wy, -Wz], [Wz, -i Wy]]
  o.r0 += -wy * Dx.i0 - wz * Dx.r1;
  o.i0 += wy * Dx.r0 - wz * Dx.i1;
  o.r1 += wz * Dx.r0 + wy * Dx.i1;
  o.i1 += wz * Dx.i0 - wy * Dx.r1;
  // y: -i(sz Wx - sx Wz) = [[-i Wx, i Wz], [i Wz, i Wx]]
  o.r0 += wx * Dy.i0 - wz * Dy.i1;
  o.i0 += -wx * Dy.r0 + wz * Dy.r1;
  o.r1 += -wz * Dy.i0 - wx * Dy.i1;
  o.i1 += wz * Dy.r0 + wx * Dy.r1;
  // z: -i(sx Wy - sy Wx) = [[0, Wx - i Wy], [-Wx - i Wy, 0]]
  o.r0 += wx * Dz.r1 + wy * Dz.i1;
  o.i0 += wx * Dz.i1 - wy * Dz.r1;
  o.r1 += -wx * Dz.r0 + wy * Dz.i0;
  o.i1 += -wx * Dz.i0 - wy * Dz.r0;
  return o;
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

// ---- FP32 plane kernel: TMA bulk copies into a shared-memory ring ---------
__device__ __forceinline__ uint32_t smemAddr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbarInit(uint64_t *bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)),
               "r"(count));
}
__device__ __forceinline__ void mbarExpectTx(uint64_t *bar, uint32_t bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
          smemAddr(bar)),
      "r"(bytes)
      : "memory");
}
// Bounded wait on an mbarrier phase. Returns false after `limit` polls.
__device__ __forceinline__ bool mbarWait(uint64_t *bar, uint32_t phase,
                                         uint32_t limit) {
  uint32_t done = 0;
  for (uint32_t it = 0; it < limit; ++it) {
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smemAddr(bar)), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Tensor-map TMA (cp.async.bulk.tensor.5d) into a shared-memory ring.
// The 5-D map views X as [col][k][j][i][4 floats]; one box is a padded
// (TY+4) x (n+4) sub-plane that starts at i = -2, j = y0 - 2. Out-of-box
// coordinates are zero-filled by the TMA unit, which is exactly the
// reference's Dirichlet truncation, so the compute loop has no bounds checks.
__device__ __forceinline__ void tmaTileLoad5(void *dst, const CUtensorMap *map,
                                             int c0, int c1, int c2, int c3,
                                             int c4, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::"
      "complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(
          smemAddr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2),
      "r"(c3), "r"(c4), "r"(smemAddr(bar))
      : "memory");
}

struct TileArgs {
  float4 *Y;
  const float4 *coef;
  int n;
  size_t ns;
  float shift;
  int TY;     // rows per band
  int kchunk; // output planes per CTA
  int ring;   // ring slots (>= 6)
  int *err;   // device error word (timeout)
};

constexpr int kMaxPts = 8; // owned points per thread (bandPts <= 8*threads)

// grid: x = band * nchunks + chunk, y = column
__global__ void __launch_bounds__(256)
    stencilTiles32(const __grid_constant__ CUtensorMap map, TileArgs A) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int n = A.n, W = n + 4;
  const int nchunks = (n + A.kchunk - 1) / A.kchunk;
  const int band = blockIdx.x / nchunks, chunk = blockIdx.x % nchunks;
  const int col = blockIdx.y;
  const int y0 = band * A.TY;
  const int ty = min(A.TY, n - y0);
  // a slot holds one box; slots start on 128-byte boundaries (TMA dst rule)
  const int boxElems = (A.TY + 4) * W;
  const int slotElems = (boxElems + 7) & ~7;
  const uint32_t boxBytes = boxElems * 16u;
  float4 *ring = reinterpret_cast<float4 *>(smem_raw);
  uint64_t *bars = reinterpret_cast<uint64_t *>(
      smem_raw + (size_t)A.ring * slotElems * 16u);
  const int k0 = chunk * A.kchunk, k1 = min(n, k0 + A.kchunk);
  const int zlo = k0 - 2, zhi = k1 + 2; // planes loaded (OOB -> zeros)

  // owned points of the band (same for every plane)
  int lr[kMaxPts], gq[kMaxPts];
  const int bandPts = ty * n;
  int np = 0;
#pragma unroll
  for (int t = 0; t < kMaxPts; ++t) {
    int q = threadIdx.x + t * blockDim.x;
    lr[t] = 0;
    gq[t] = 0;
    if (q < bandPts) {
      int jj = q / n, i = q - jj * n;
      lr[t] = (jj + 2) * W + (i + 2);
      gq[t] = (y0 + jj) * n + i;
      np = t + 1;
    }
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < A.ring; ++s) mbarInit(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int z) {
    int s = (z - zlo) % A.ring;
    mbarExpectTx(&bars[s], boxBytes);
    tmaTileLoad5(ring + (size_t)s * slotElems, &map, 0, -2, y0 - 2, z, col,
                 &bars[s]);
  };
  int nextLoad = zlo;
  if (threadIdx.x == 0)
    for (; nextLoad < zhi && nextLoad - zlo < A.ring; ++nextLoad) issue(nextLoad);
  bool ok = true;
  const uint32_t kLimit = 1u << 22;
  int waitedUpTo = zlo - 1;
  const size_t plane = (size_t)n * n;
  float4 *Yc = A.Y + (size_t)col * A.ns;
  for (int k = k0; k < k1; ++k) {
    while (ok && waitedUpTo < k + 2) {
      int z = waitedUpTo + 1;
      int s = (z - zlo) % A.ring;
      uint32_t phase = ((z - zlo) / A.ring) & 1u;
      if (!mbarWait(&bars[s], phase, kLimit)) ok = false;
      else waitedUpTo = z;
    }
    ok = __syncthreads_and(ok); // block-uniform decision
    if (!ok) break;
    const float4 *pm2 = ring + (size_t)((k - 2 - zlo) % A.ring) * slotElems;
    const float4 *pm1 = ring + (size_t)((k - 1 - zlo) % A.ring) * slotElems;
    const float4 *pc = ring + (size_t)((k - zlo) % A.ring) * slotElems;
    const float4 *pp1 = ring + (size_t)((k + 1 - zlo) % A.ring) * slotElems;
    const float4 *pp2 = ring + (size_t)((k + 2 - zlo) % A.ring) * slotElems;
#pragma unroll
    for (int t = 0; t < kMaxPts; ++t) {
      if (t < np) {
        const int l = lr[t];
        const size_t gp = (size_t)k * plane + gq[t];
        const float4 *c2 = A.coef + 2 * gp;
        float4 ca = __ldg(c2), cb = __ldg(c2 + 1);
        float c[8] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w};
        auto S = [](float4 v) { return Spinor<float>{v.x, v.y, v.z, v.w}; };
        Spinor<float> o = pointH<float>(
            c, A.shift, S(pc[l]), S(pc[l + 1]), S(pc[l - 1]), S(pc[l + 2]),
            S(pc[l - 2]), S(pc[l + W]), S(pc[l - W]), S(pc[l + 2 * W]),
            S(pc[l - 2 * W]), S(pp1[l]), S(pm1[l]), S(pp2[l]), S(pm2[l]));
        Yc[gp] = make_float4(o.r0, o.i0, o.r1, o.i1);
      }
    }
    __syncthreads(); // plane k-2 is free after this
    if (threadIdx.x == 0)
      while (nextLoad < zhi && nextLoad < k - 1 + A.ring) issue(nextLoad++);
  }
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(A.err, 1);
    for (int z = waitedUpTo + 1; z < nextLoad; ++z) {
      int s = (z - zlo) % A.ring;
      mbarWait(&bars[s], ((z - zlo) / A.ring) & 1u, kLimit);
    }
  }
}

// ---- coefficient builders -------------------------------------------------
__global__ void buildCoefKernel(const double *f, const double *gf,
                                const double *U, const double *W,
                                const double *UC, size_t ns, double h,
                                double *c64, float *c32) {
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

int *errWord() {
  static int *d = nullptr;
  if (!d) {
    cudaMalloc(&d, sizeof(int));
    cudaMemset(d, 0, sizeof(int));
  }
  return d;
}

struct ShapeCache {
  ncgm_ctx *ctx = nullptr;
  StencilShape s;
  bool tuned = false;
};
ShapeCache g_shape[8];

size_t tileSmem(int n, int TY, int ring) {
  size_t slot = (((size_t)(TY + 4) * (n + 4) + 7) & ~size_t(7)) * 16;
  return (size_t)ring * slot + (size_t)ring * 8;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no
// direct libcuda link).
PFN_cuTensorMapEncodeTiled_v12000 encodeFn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void *p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                         cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

struct MapKey {
  const void *ptr;
  int n, ncols, TY;
};
struct MapEntry {
  MapKey k;
  CUtensorMap map;
};
std::vector<MapEntry> g_maps;

// 5-D map of X: dims (4 floats, i, j, k, col), box (4, n+4, TY+4, 1, 1).
bool tensorMapFor(const void *X, int n, int ncols, int TY, CUtensorMap *out) {
  for (auto &e : g_maps)
    if (e.k.ptr == X && e.k.n == n && e.k.ncols == ncols && e.k.TY == TY) {
      *out = e.map;
      return true;
    }
  auto fn = encodeFn();
  if (!fn) return false;
  cuuint64_t dims[5] = {4, (cuuint64_t)n, (cuuint64_t)n, (cuuint64_t)n,
                        (cuuint64_t)ncols};
  cuuint64_t strides[4] = {16, (cuuint64_t)16 * n, (cuuint64_t)16 * n * n,
                           (cuuint64_t)16 * n * n * n};
  cuuint32_t box[5] = {4, (cuuint32_t)(n + 4), (cuuint32_t)(TY + 4), 1, 1};
  cuuint32_t es[5] = {1, 1, 1, 1, 1};
  CUtensorMap m;
  CUresult r = fn(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5, const_cast<void *>(X),
                  dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return false;
  if (g_maps.size() > 64) g_maps.erase(g_maps.begin());
  g_maps.push_back({{X, n, ncols, TY}, m});
  *out = m;
  return true;
}

} // namespace

StencilShape &stencilShape32(ncgm_ctx *ctx) {
  for (auto &c : g_shape)
    if (c.ctx == ctx) return c.s;
  for (auto &c : g_shape)
    if (c.ctx == nullptr) {
      c.ctx = ctx;
      c.s.kchunk = 8;
      c.s.threads = 256;
      return c.s;
    }
  g_shape[0].ctx = ctx;
  return g_shape[0].s;
}

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
  }
  buildCoefKernel<<<(unsigned)((ctx->ns + 255) / 256), 256, 0, ctx->stream>>>(
      f, gradf, U, W, UC, ctx->ns, ctx->h, F.coef64, F.coef32);
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

// Rows per band: a candidate list for the autotuner; the ring holds the 5
// planes of the stencil plus prefetch.
static int bandRowsDefault(int n) {
  int TY = n;
  while (TY > 4 && tileSmem(n, TY, 6) > 110 * 1024) TY = (TY + 1) / 2;
  return TY;
}

static bool launchTiles(ncgm_ctx *ctx, int species, const float2 *X,
                        float2 *Y, int ncols, float shift, cudaStream_t s,
                        const StencilShape &sh) {
  const int n = ctx->n;
  const int TY = sh.rows > 0 ? std::min(sh.rows, n) : bandRowsDefault(n);
  if ((size_t)TY * n > (size_t)kMaxPts * sh.threads) return false;
  CUtensorMap map;
  if (!tensorMapFor(X, n, ncols, TY, &map)) return false;
  TileArgs A;
  A.Y = reinterpret_cast<float4 *>(Y);
  A.coef = reinterpret_cast<const float4 *>(ctx->sp[species].coef32);
  A.n = n;
  A.ns = ctx->ns;
  A.shift = shift;
  A.TY = TY;
  A.kchunk = sh.kchunk;
  A.ring = sh.ring;
  A.err = errWord();
  const int nbands = (n + TY - 1) / TY;
  const int nchunks = (n + sh.kchunk - 1) / sh.kchunk;
  dim3 grid(nbands * nchunks, ncols);
  stencilTiles32<<<grid, sh.threads, tileSmem(n, TY, sh.ring), s>>>(map, A);
  return true;
}

void applyH32(ncgm_ctx *ctx, int species, const float2 *X, float2 *Y,
              int ncols, float shift, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(stencilTiles32,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         220 * 1024);
    attr = true;
  }
  StencilShape &sh0 = stencilShape32(ctx);
  if (!sh0.tuned && !sh0.tuning) {
    // first FP32 apply on this context: pick the launch shape by timing
    sh0.tuning = true;
    autotuneStencil32(ctx, species, ncols);
    sh0.tuning = false;
    sh0.tuned = true;
  }
  if (!launchTiles(ctx, species, X, Y, ncols, shift, s, sh0)) {
    // shape not launchable on this lattice: default shape
    StencilShape d;
    d.threads = 256;
    d.rows = bandRowsDefault(ctx->n);
    while ((size_t)d.rows * ctx->n > (size_t)kMaxPts * d.threads && d.rows > 1)
      d.rows = (d.rows + 1) / 2;
    if (!launchTiles(ctx, species, X, Y, ncols, shift, s, d))
      setError("FP32 stencil: tensor map encoding failed");
  }
}

// Project autotuner for the FP32 stencil launch shape: times each candidate
// (z-chunk length x threads per CTA) on the context's own lattice with CUDA
// events and keeps the fastest. Runs once per context.
int autotuneStencil32(ncgm_ctx *ctx, int species, int ncols) {
  StencilShape &best = stencilShape32(ctx);
  ncols = std::max(1, std::min(ncols, ctx->max_cols));
  size_t bytes = ctx->N * ncols * sizeof(float2);
  float2 *X = static_cast<float2 *>(ctx->buf(1, bytes));
  float2 *Y = static_cast<float2 *>(ctx->buf(2, bytes));
  if (!X || !Y) return NCGM_ERR_NOMEM;
  NCGM_CUDA(cudaMemsetAsync(X, 0, bytes, ctx->stream));
  const int n = ctx->n;
  std::vector<int> rowsC;
  for (int r = n; r >= 4; r = (r + 1) / 2) {
    rowsC.push_back(r);
    if (r == 4) break;
  }
  const int chunks[] = {4, 8, 16};
  const int threads[] = {128, 256};
  const int rings[] = {6, 8};
  float bestMs = 1e30f;
  StencilShape keep = best;
  bool any = false;
  for (int rw : rowsC)
    for (int kc : chunks)
      for (int th : threads)
        for (int rg : rings) {
          if (tileSmem(n, rw, rg) > 200 * 1024) continue;
          if ((size_t)rw * n > (size_t)kMaxPts * th) continue;
          StencilShape cand = best;
          cand.kchunk = kc;
          cand.threads = th;
          cand.rows = rw;
          cand.ring = rg;
          best.kchunk = kc;
          best.threads = th;
          best.rows = rw;
          best.ring = rg;
          if (!launchTiles(ctx, species, X, Y, ncols, 0.f, ctx->stream, best))
            continue; // warm
          cudaEventRecord(ctx->ev0, ctx->stream);
          for (int r = 0; r < 3; ++r)
            launchTiles(ctx, species, X, Y, ncols, 0.f, ctx->stream, best);
          cudaEventRecord(ctx->ev1, ctx->stream);
          NCGM_CUDA(cudaEventSynchronize(ctx->ev1));
          float ms = 0;
          cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
          if (ms < bestMs) {
            bestMs = ms;
            keep = cand;
            any = true;
          }
        }
  if (!any) keep = StencilShape();
  best.rows = keep.rows;
  best.ring = keep.ring;
  best.kchunk = keep.kchunk;
  best.threads = keep.threads;
  NCGM_CUDA(cudaGetLastError());
  return NCGM_OK;
}

int stencilErrorFlag() {
  int h = 0;
  cudaMemcpy(&h, errWord(), sizeof(int), cudaMemcpyDeviceToHost);
  return h;
}

} // namespace ncgm
