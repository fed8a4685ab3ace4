// FP64-accurate Gram products on the tensor cores: C = A^H B for complex FP64
// blocks A (N x p), B (N x q), with the error-free splitting of Ozaki, Ogita,
// Oishi and Rump (Numer. Algorithms 59, 2012) mapped onto tcgen05 BF16 MMAs.
//
// The complex product is one real product of the interleaved blocks S (N x
// 2p, column 2c = Re A_c, 2c + 1 = Im A_c) and T (N x 2q, same for B). Every
// column c of S and T is scaled by a power of two 2^-e_c that brings its
// entries into [-1, 1] (e_c from the column's max-abs, exact), and each
// scaled value is written as a sum of kDig signed 7-bit integer digits,
//   x 2^-e = sum_t a_t 2^(-7t),  |a_1| <= 128, |a_t| <= 64 (t > 1),
// all exactly representable in BF16. A product of two digits is an integer
// below 2^14; the MMAs of one "level" l = t + u (pairs with the same scale
// 2^(-7l)) accumulate in FP32 tensor memory over 256 rows, so every partial
// sum is an integer below 2^24 and the FP32 accumulation is exact. After each
// 256-row block the levels are combined in FP64 (shared-memory accumulators),
// and the CTA's FP64 partial is summed with the other row chunks in a fixed
// order. Levels above kDig + 1 are dropped: the truncation error is ~2^(-7
// kDig) of the column max per element (kDig = 6: ~2e-13 relative).
//
// Tile: M = 128 rows of S^T, N = 64 columns of T; 8 warps stage 32-row slabs
// (double-buffered, K-major core matrices, no swizzle), one thread issues the
// MMAs (instruction K = 16, 2 per slab per digit pair) and commits them, and
// after every 8 slabs the warps fold the level accumulators (tcgen05.ld) into
// FP64. Every wait is bounded.
#include "ncgm_internal.cuh"

#include <cuda_bf16.h>

#include <algorithm>

namespace ncgm {

namespace {

constexpr int kDig = 6;                  // digits per value
constexpr int kM = 128, kN = 64;         // D tile
constexpr int kSlab = 32;                // K rows per stage (2 MMAs of K 16)
constexpr int kFold = 8;                 // slabs per exact accumulation block
constexpr int kThr = 256;
constexpr int kABytes = kM * kSlab * 2;  // one digit plane of A: 8 KB
constexpr int kBBytes = kN * kSlab * 2;  // one digit plane of B: 4 KB
constexpr int kBuf = kDig * (kABytes + kBBytes); // 72 KB
constexpr int kAccLd = kN + 1;                   // padded row: no bank conflicts
constexpr int kAccBytes = kM * kAccLd * 8;       // FP64 tile: 65 KB
constexpr int kSmem = 2 * kBuf + kAccBytes + 64;
constexpr uint32_t kLBO = 128, kSBO = 512;       // 8 rows x 16 B cores; K 32
constexpr uint32_t kTmemCols = 512; // kDig levels x kN = 384 -> 512

__device__ __forceinline__ uint32_t sAddr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((kLBO >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((kSBO >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}
// D FP32, A/B BF16, K-major, M = 128, N = 64
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) |
                            ((uint32_t)(kN >> 3) << 17) |
                            ((uint32_t)(kM >> 4) << 24);

// byte offset of element (row, k) in a K-major tile with 32 BF16 per row:
// core matrices of 8 rows x 8 elements (16 B); 4 cores along K
__device__ __forceinline__ uint32_t off16(int row, int k) {
  return (uint32_t)(row >> 3) * kSBO + (uint32_t)(k >> 3) * kLBO +
         (uint32_t)(row & 7) * 16u + (uint32_t)(k & 7) * 2u;
}

__device__ __forceinline__ bool waitBar(uint64_t *bar, uint32_t phase) {
  for (uint32_t it = 0; it < (1u << 20); ++it) {
    uint32_t done;
    asm volatile("{\n .reg .pred p;\n"
                 " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
                 " selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(done)
                 : "r"(sAddr(bar)), "r"(phase), "r"(1000u)
                 : "memory");
    if (done) return true;
  }
  return false;
}


// digits of a scaled value: w = round(x 2^(42-e)), |w| < 2^42, written as
// sum_t a_t 2^(42-7t) with |a_1| <= 128 and |a_t| <= 64, by integer rounding
// divisions (exact; the digits are integers, exact in BF16). One 64-bit
// rounding split w = h 2^21 + l (|l| <= 2^20) leaves 32-bit work: three
// digits from each half, and 32-bit integer-to-float conversions (the
// 64-bit conversion runs on the slow FP64 pipe).
static_assert(kDig == 6, "digits() splits 42 bits as 3 + 3 digits");
__device__ __forceinline__ void digits(long long w, float d[kDig]) {
  const long long hh = (w + (1ll << 20)) >> 21;
  int l = (int)(w - (hh << 21));
  int h = (int)hh;
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    const int sh = 14 - 7 * t;
    const int a = (h + (1 << (sh - 1))) >> sh;
    d[t] = (float)a;
    h -= a << sh;
    const int b = (l + (1 << (sh - 1))) >> sh;
    d[3 + t] = (float)b;
    l -= b << sh;
  }
  d[2] = (float)h;
  d[5] = (float)l;
}

// w = round(x 2^(42 - e)) for |x| < 2^e, from the bits of x with integer
// operations only (round half away from zero; the FP64 pipe is slow)
__device__ __forceinline__ long long scaledInt(double x, int e) {
  const long long bits = __double_as_longlong(x);
  const int ex = (int)((bits >> 52) & 0x7FF);
  if (ex == 0) return 0; // zero or subnormal: below 2^-1022
  const long long mant = (bits & 0xFFFFFFFFFFFFFll) | (1ll << 52);
  // x = mant 2^(ex - 1075); the result is mant 2^(ex - 1033 - e), where the
  // shift is <= -11 since |x| < 2^e
  const int sh = 1033 + e - ex;
  if (sh >= 63) return 0;
  const long long w = (mant + (1ll << (sh - 1))) >> sh;
  return bits < 0 ? -w : w;
}

// per column c of the interleaved block X (N x 2p): the power of two
// sc[c] = 2^e above its max-abs, and e = ex[c]. Pass 1: blocks (complex
// column, row chunk) fold |Re| and |Im| maxima into sc as IEEE bit patterns
// (for non-negative doubles the integer order is the numeric order); pass
// 2 turns them into exponents.
__global__ void colMaxKernel(const double2 *X, size_t ld, int p, size_t N,
                             size_t rowsPerBlock, double *sc) {
  __shared__ double sh[2][256];
  const int c = blockIdx.x;
  const size_t r0 = (size_t)blockIdx.y * rowsPerBlock;
  const size_t r1 = r0 + rowsPerBlock < N ? r0 + rowsPerBlock : N;
  double mr = 0, mi = 0;
  for (size_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const double2 v = X[(size_t)c * ld + r];
    mr = fmax(mr, fabs(v.x));
    mi = fmax(mi, fabs(v.y));
  }
  sh[0][threadIdx.x] = mr;
  sh[1][threadIdx.x] = mi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sh[0][threadIdx.x] = fmax(sh[0][threadIdx.x], sh[0][threadIdx.x + s]);
      sh[1][threadIdx.x] = fmax(sh[1][threadIdx.x], sh[1][threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x < 2)
    atomicMax(reinterpret_cast<unsigned long long *>(sc) + 2 * c + threadIdx.x,
              (unsigned long long)__double_as_longlong(sh[threadIdx.x][0]));
}
__global__ void colExpKernel(int cols, double *sc, int *exq) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  const double m = sc[c]; // the bit pattern written by colMaxKernel
  int e = 0;
  if (m > 0) frexp(m, &e); // m < 2^e
  sc[c] = ldexp(1.0, e);   // column scale: entries / sc in (-1, 1)
  exq[c] = e;
}
// column maxima of the p complex columns of X (2p interleaved real columns)
void colMax(const double2 *X, size_t ld, int p, size_t N, double *sc, int *ex,
            cudaStream_t s) {
  const int chunks = (int)std::min<size_t>(16, (N + 4095) / 4096);
  const size_t rows = (N + chunks - 1) / chunks;
  cudaMemsetAsync(sc, 0, 2 * (size_t)p * sizeof(double), s);
  colMaxKernel<<<dim3(p, chunks), 256, 0, s>>>(X, ld, p, N, rows, sc);
  colExpKernel<<<(2 * p + 127) / 128, 128, 0, s>>>(2 * p, sc, ex);
}

__global__ void __launch_bounds__(kThr, 1)
    exactGramKernel(const double2 *__restrict__ A, size_t lda, int p,
                    const double2 *__restrict__ B, size_t ldb, int q, size_t N,
                    const double *__restrict__ scA,
                    const int *__restrict__ eA,
                    const double *__restrict__ scB,
                    const int *__restrict__ eB, int rowsPerChunk,
                    double *__restrict__ part, int *err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  double *acc = reinterpret_cast<double *>(sm + 2 * kBuf);
  uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + 2 * kBuf + kAccBytes);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int mt = blockIdx.x, nt = blockIdx.y, chunk = blockIdx.z;
  const size_t r0 = (size_t)chunk * rowsPerChunk;
  const size_t r1 = (r0 + (size_t)rowsPerChunk < N) ? r0 + rowsPerChunk : N;
  const int nslab = (int)((r1 - r0 + kSlab - 1) / kSlab);

  if (warp == 0) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::
            "r"(sAddr(tslot)),
        "r"(kTmemCols)
        : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;"
                 ::
                     : "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sAddr(&mbar[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sAddr(&mbar[1])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int e = tid; e < kM * kAccLd; e += kThr) acc[e] = 0.0;
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t taddr = *tslot;
  bool ok = true;
  __shared__ int nCommitted;
  int committed = 0;

  for (int s = 0; s < nslab && ok; ++s) {
    const int b = s & 1;
    if (s >= 2 && !waitBar(&mbar[b], ((s - 2) >> 1) & 1)) ok = false;
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    unsigned char *buf = sm + b * kBuf;
    // stage the digit planes. One warp step covers 8 complex columns x 8
    // rows: lane (cc = lane >> 2, kp = lane & 3) loads rows 2kp, 2kp + 1 of
    // complex column cc as double2 (4 lanes read 128 contiguous bytes) and
    // writes the digits of interleaved rows 2cc (Re) and 2cc + 1 (Im) at
    // those two k. Steps: 32 for the A tile (64 complex columns x 32 rows),
    // 16 for B; all of a warp's loads are issued before its digit work.
    {
      constexpr int kStepsA = (kM / 16) * (kSlab / 8), kSteps =
          kStepsA + (kN / 16) * (kSlab / 8);
      constexpr int kPer = kSteps / (kThr / 32); // 6 steps per warp
      const int cc = lane >> 2, kp = lane & 3;
      double2 v[kPer][2];
#pragma unroll
      for (int i = 0; i < kPer; ++i) {
        const int g = warp + i * (kThr / 32);
        const bool isA = g < kStepsA;
        const int gg = isA ? g : g - kStepsA;
        const int col = (gg >> 2) * 8 + cc;        // complex column in tile
        const int k = (gg & 3) * 8 + 2 * kp;       // slab row
        const int gcol = isA ? mt * (kM / 2) + col : nt * (kN / 2) + col;
        const int ncol = isA ? p : q;
        const double2 *X = isA ? A : B;
        const size_t ld = isA ? lda : ldb;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const size_t r = r0 + (size_t)s * kSlab + k + h;
          v[i][h] = (gcol < ncol && r < r1) ? X[(size_t)gcol * ld + r]
                                            : make_double2(0.0, 0.0);
        }
      }
#pragma unroll
      for (int i = 0; i < kPer; ++i) {
        const int g = warp + i * (kThr / 32);
        const bool isA = g < kStepsA;
        const int gg = isA ? g : g - kStepsA;
        const int col = (gg >> 2) * 8 + cc;
        const int k = (gg & 3) * 8 + 2 * kp;
        const int gcol = isA ? mt * (kM / 2) + col : nt * (kN / 2) + col;
        const int ncol = isA ? p : q;
#pragma unroll
        for (int part = 0; part < 2; ++part) { // 0: Re, 1: Im
          const int row = 2 * col + part;        // interleaved tile row
          const int e = gcol < ncol ? (isA ? eA : eB)[2 * gcol + part] : 0;
          float d0[kDig], d1[kDig];
          digits(scaledInt(part ? v[i][0].y : v[i][0].x, e), d0);
          digits(scaledInt(part ? v[i][1].y : v[i][1].x, e), d1);
          const uint32_t o = off16(row, k);
#pragma unroll
          for (int t = 0; t < kDig; ++t) {
            unsigned char *plane =
                isA ? buf + t * kABytes : buf + kDig * kABytes + t * kBBytes;
            *reinterpret_cast<__nv_bfloat162 *>(plane + o) =
                __floats2bfloat162_rn(d0[t], d1[t]);
          }
        }
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t base = sAddr(buf);
      const bool first = (s % kFold) == 0;
      for (int ks = 0; ks < kSlab / 16; ++ks) {
        const uint32_t kofs = ks * 2 * kLBO; // 16 K = 2 core matrices
        for (int t = 0; t < kDig; ++t)
          for (int u = 0; u + t < kDig; ++u) {
            const int lev = t + u; // level index 0 .. kDig-1
            const uint64_t ad = smemDesc(base + t * kABytes + kofs);
            const uint64_t bd =
                smemDesc(base + kDig * kABytes + u * kBBytes + kofs);
            // the first MMA of each level in a fold block overwrites (in this
            // loop order a level's first pair is (0, lev))
            const uint32_t accum = (first && ks == 0 && t == 0) ? 0u : 1u;
            const uint32_t td = taddr + (uint32_t)(lev * kN);
            asm volatile("{\n .reg .pred pa;\n setp.ne.b32 pa, %4, 0;\n"
                         " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, "
                         "%3, pa;\n}\n" ::"r"(td),
                         "l"(ad), "l"(bd), "r"(kIdesc), "r"(accum)
                         : "memory");
          }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::"
                   "cluster.b64 [%0];" ::"r"(sAddr(&mbar[b]))
                   : "memory");
      committed = s + 1;
    }
    // fold the exact level sums into FP64 at the end of each block
    if ((s % kFold) == kFold - 1 || s == nslab - 1) {
      if (!waitBar(&mbar[b], (s >> 1) & 1)) ok = false;
      if (!__syncthreads_and(ok)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int lw = warp & 3, row = lw * 32 + lane;
      const int cBeg = (warp >> 2) * (kN / 2);
      for (int c0 = cBeg; c0 < cBeg + kN / 2; c0 += 16) {
        // the level sums are integers below 2^24: combine them exactly in
        // 64-bit integers (sum_l L_l 2^(7 (kDig-1-l)) < 2^60), then one
        // conversion to FP64 per element
        long long sum[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) sum[j] = 0;
        for (int lev = 0; lev < kDig; ++lev) {
          uint32_t v[16];
          const uint32_t ta =
              taddr + ((uint32_t)(lw * 32) << 16) + (uint32_t)(lev * kN + c0);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, "
              "%5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
              : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]),
                "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]),
                "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                "=r"(v[14]), "=r"(v[15])
              : "r"(ta));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int j = 0; j < 16; ++j)
            sum[j] = sum[j] * 128 + (long long)__float2int_rn(
                                         __uint_as_float(v[j]));
        }
        // sum = sum_l L_l 2^(7 (kDig-1-l)); value = sum 2^(-7 (kDig+1))
        const double w = ldexp(1.0, -7 * (kDig + 1));
#pragma unroll
        for (int j = 0; j < 16; ++j)
          acc[row * kAccLd + c0 + j] += (double)sum[j] * w;
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
    }
  }
  if (tid == 0) nCommitted = committed;
  __syncthreads();
  if (!ok && nCommitted > 0) {
    const int last = nCommitted - 1;
    waitBar(&mbar[last & 1], (last >> 1) & 1);
  }
  ok = __syncthreads_and(ok);
  if (ok) {
    for (int e = tid; e < kM * kN; e += kThr) {
      const int row = e / kN, col = e % kN;
      const int gr = mt * kM + row, gc = nt * kN + col;
      if (gr < 2 * p && gc < 2 * q)
        part[((size_t)chunk * 2 * p + gr) * (2 * q) + gc] =
            acc[row * kAccLd + col] * scA[gr] * scB[gc];
    }
  } else if (tid == 0) {
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(
                     taddr),
                 "r"(kTmemCols)
                 : "memory");
}

// one warp per output element: lane l sums chunks l, l + 32, ...; the lane
// sums are combined in a fixed shuffle order (deterministic)
__global__ void exactGramReduce(const double *__restrict__ part, int chunks,
                                int p, int q, double2 *__restrict__ C,
                                int ldc) {
  const int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (e >= p * q) return;
  const int i = e % p, j = e / p;
  const size_t W = 2 * (size_t)q, H = 2 * (size_t)p;
  double re = 0, im = 0;
  for (int ch = lane; ch < chunks; ch += 32) {
    const double *P = part + (size_t)ch * H * W;
    re += P[(size_t)(2 * i) * W + 2 * j] + P[(size_t)(2 * i + 1) * W + 2 * j + 1];
    im += P[(size_t)(2 * i) * W + 2 * j + 1] - P[(size_t)(2 * i + 1) * W + 2 * j];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  if (lane == 0) C[(size_t)j * ldc + i] = make_double2(re, im);
}

// ---------------------------------------------------------------------------
// Y = V C (V: N x m, C: m x k, complex FP64) with the same exact digit
// products. Real form: A = V interleaved (N x 2m, column 2c = Re V_c,
// 2c + 1 = Im V_c), B (2m x 2k) with B[2c][2j] = Re C_cj, B[2c+1][2j] =
// -Im C_cj, B[2c][2j+1] = Im C_cj, B[2c+1][2j+1] = Re C_cj, so that column
// 2j of A B is Re Y_j and 2j + 1 is Im Y_j. A's columns are scaled by powers
// of two 2^-eA (colMaxKernel); the scales move into B, whose columns are
// scaled again by 2^-eB, and the digits of that B are precomputed once
// (vcPrepKernel) in the shared-memory image the MMAs read. The reduction
// (K = 2m <= 512) is a few 32-row slabs; every 8 slabs the level sums fold
// into FP64. Each CTA owns 128 rows of Y and 64 of its 2k real columns.

// digits of B = diag(2^eA) B0 2^-eB, laid out per (column tile, slab, digit)
// as the K-major core-matrix image of one 64 x 32 BF16 plane
__global__ void vcMaxKernel(const double2 *__restrict__ Cm, int ldc, int m,
                            int k, const int *__restrict__ eA, double *scB,
                            int *eB) {
  const int jr = blockIdx.x * blockDim.x + threadIdx.x; // real column of B
  if (jr >= 2 * k) return;
  const int j = jr >> 1, b = jr & 1;
  int emax = -100000;
  for (int c = 0; c < m; ++c) {
    const double2 t = Cm[(size_t)j * ldc + c];
    // rows 2c, 2c+1 of column jr: (Re, -Im) for b = 0, (Im, Re) for b = 1
    const double v0 = b ? t.y : t.x, v1 = b ? t.x : -t.y;
    int e0 = -100000, e1 = -100000;
    if (v0 != 0.0) { frexp(v0, &e0); e0 += eA[2 * c]; }
    if (v1 != 0.0) { frexp(v1, &e1); e1 += eA[2 * c + 1]; }
    emax = max(emax, max(e0, e1));
  }
  if (emax == -100000) emax = 0; // an all-zero column
  eB[jr] = emax;                  // |B[., jr]| 2^eA < 2^emax
  scB[jr] = ldexp(1.0, emax);
}

__global__ void vcPrepKernel(const double2 *__restrict__ Cm, int ldc, int m,
                             int k, const int *__restrict__ eA,
                             const int *__restrict__ eB, int nslab,
                             unsigned char *__restrict__ dig) {
  const int ntile = (2 * k + kN - 1) / kN;
  const size_t total = (size_t)nslab * kSlab * ntile * kN;
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= total) return;
  const int cr = (int)(e % ((size_t)nslab * kSlab)); // row of B (K index)
  const int jr = (int)(e / ((size_t)nslab * kSlab)); // column of B
  long long w = 0;
  if (cr < 2 * m && jr < 2 * k) {
    const int c = cr >> 1, a = cr & 1, j = jr >> 1, b = jr & 1;
    const double2 t = Cm[(size_t)j * ldc + c];
    const double v = b ? (a ? t.x : t.y) : (a ? -t.y : t.x);
    // v 2^eA[cr] 2^-eB[jr] scaled to 42 bits: scaledInt(v, eB - eA)
    w = scaledInt(v, eB[jr] - eA[cr]);
  }
  float d[kDig];
  digits(w, d);
  const int s = cr / kSlab, kk = cr % kSlab, nt = jr / kN, jj = jr % kN;
  unsigned char *base =
      dig + ((size_t)(nt * nslab + s) * kDig) * (size_t)kBBytes;
  const uint32_t o = off16(jj, kk);
#pragma unroll
  for (int t = 0; t < kDig; ++t)
    *reinterpret_cast<__nv_bfloat16 *>(base + (size_t)t * kBBytes + o) =
        __float2bfloat16_rn(d[t]);
}

__global__ void __launch_bounds__(kThr, 1)
    exactVCKernel(const double2 *__restrict__ V, size_t ldv, int m,
                  const int *__restrict__ eA,
                  const unsigned char *__restrict__ dig,
                  const double *__restrict__ scB, int k, int nslab,
                  double2 *__restrict__ Y, size_t ldy, size_t N, int accum,
                  int *err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  double *acc = reinterpret_cast<double *>(sm + 2 * kBuf);
  uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + 2 * kBuf + kAccBytes);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int mt = blockIdx.x, nt = blockIdx.y;
  const size_t r0 = (size_t)mt * kM;

  if (warp == 0) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::
            "r"(sAddr(tslot)),
        "r"(kTmemCols)
        : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;"
                 ::
                     : "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sAddr(&mbar[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sAddr(&mbar[1])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int e = tid; e < kM * kAccLd; e += kThr) acc[e] = 0.0;
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t taddr = *tslot;
  bool ok = true;
  __shared__ int nCommitted;
  int committed = 0;

  for (int s = 0; s < nslab && ok; ++s) {
    const int b = s & 1;
    if (s >= 2 && !waitBar(&mbar[b], ((s - 2) >> 1) & 1)) ok = false;
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    unsigned char *buf = sm + b * kBuf;
    // A digits: 128 rows x 16 complex columns. A warp step covers 8 rows x
    // 4 complex columns (one core matrix): lane (r8 = lane >> 2, kp =
    // lane & 3) loads V[col, row] and writes the (Re, Im) digit pair at
    // k = 2 col. 64 steps, 8 per warp; loads first.
    {
      constexpr int kPer = (kM / 8) * (kSlab / 8) / (kThr / 32);
      const int r8 = lane >> 2, kp = lane & 3;
      double2 v[kPer];
#pragma unroll
      for (int i = 0; i < kPer; ++i) {
        const int g = warp + i * (kThr / 32);
        const int row = (g >> 2) * 8 + r8, col = (g & 3) * 4 + kp;
        const int gc = s * (kSlab / 2) + col;
        const size_t r = r0 + row;
        v[i] = (gc < m && r < N) ? V[(size_t)gc * ldv + r]
                                 : make_double2(0.0, 0.0);
      }
#pragma unroll
      for (int i = 0; i < kPer; ++i) {
        const int g = warp + i * (kThr / 32);
        const int row = (g >> 2) * 8 + r8, col = (g & 3) * 4 + kp;
        const int gc = s * (kSlab / 2) + col;
        float d0[kDig], d1[kDig];
        if (gc < m) {
          digits(scaledInt(v[i].x, eA[2 * gc]), d0);
          digits(scaledInt(v[i].y, eA[2 * gc + 1]), d1);
        } else {
          digits(0, d0);
          digits(0, d1);
        }
        const uint32_t o = off16(row, 2 * col);
#pragma unroll
        for (int t = 0; t < kDig; ++t)
          *reinterpret_cast<__nv_bfloat162 *>(buf + t * kABytes + o) =
              __floats2bfloat162_rn(d0[t], d1[t]);
      }
    }
    // B digits: the precomputed image of this (column tile, slab)
    {
      const uint4 *src = reinterpret_cast<const uint4 *>(
          dig + ((size_t)(nt * nslab + s) * kDig) * (size_t)kBBytes);
      uint4 *dst = reinterpret_cast<uint4 *>(buf + kDig * kABytes);
      for (int e = tid; e < kDig * kBBytes / 16; e += kThr) dst[e] = src[e];
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t base = sAddr(buf);
      const bool first = (s % kFold) == 0;
      for (int ks = 0; ks < kSlab / 16; ++ks) {
        const uint32_t kofs = ks * 2 * kLBO;
        for (int t = 0; t < kDig; ++t)
          for (int u = 0; u + t < kDig; ++u) {
            const int lev = t + u;
            const uint64_t ad = smemDesc(base + t * kABytes + kofs);
            const uint64_t bd =
                smemDesc(base + kDig * kABytes + u * kBBytes + kofs);
            const uint32_t accum = (first && ks == 0 && t == 0) ? 0u : 1u;
            const uint32_t td = taddr + (uint32_t)(lev * kN);
            asm volatile("{\n .reg .pred pa;\n setp.ne.b32 pa, %4, 0;\n"
                         " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, "
                         "%3, pa;\n}\n" ::"r"(td),
                         "l"(ad), "l"(bd), "r"(kIdesc), "r"(accum)
                         : "memory");
          }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::"
                   "cluster.b64 [%0];" ::"r"(sAddr(&mbar[b]))
                   : "memory");
      committed = s + 1;
    }
    if ((s % kFold) == kFold - 1 || s == nslab - 1) {
      if (!waitBar(&mbar[b], (s >> 1) & 1)) ok = false;
      if (!__syncthreads_and(ok)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int lw = warp & 3, row = lw * 32 + lane;
      const int cBeg = (warp >> 2) * (kN / 2);
      for (int c0 = cBeg; c0 < cBeg + kN / 2; c0 += 16) {
        long long sum[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) sum[j] = 0;
        for (int lev = 0; lev < kDig; ++lev) {
          uint32_t v[16];
          const uint32_t ta =
              taddr + ((uint32_t)(lw * 32) << 16) + (uint32_t)(lev * kN + c0);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, "
              "%5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
              : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]),
                "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]),
                "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                "=r"(v[14]), "=r"(v[15])
              : "r"(ta));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int j = 0; j < 16; ++j)
            sum[j] = sum[j] * 128 + (long long)__float2int_rn(
                                         __uint_as_float(v[j]));
        }
        const double w = ldexp(1.0, -7 * (kDig + 1));
#pragma unroll
        for (int j = 0; j < 16; ++j)
          acc[row * kAccLd + c0 + j] += (double)sum[j] * w;
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
    }
  }
  if (tid == 0) nCommitted = committed;
  __syncthreads();
  if (!ok && nCommitted > 0) {
    const int last = nCommitted - 1;
    waitBar(&mbar[last & 1], (last >> 1) & 1);
  }
  ok = __syncthreads_and(ok);
  if (ok) {
    // Y[j][r] = (acc[r][2j] 2^eB[2j], acc[r][2j+1] 2^eB[2j+1])
    for (int e = tid; e < kM * (kN / 2); e += kThr) {
      const int row = e % kM, jc = e / kM;
      const size_t r = r0 + row;
      const int jr = nt * kN + 2 * jc;
      if (r < N && jr < 2 * k) {
        double2 v = make_double2(acc[row * kAccLd + 2 * jc] * scB[jr],
                                 acc[row * kAccLd + 2 * jc + 1] * scB[jr + 1]);
        double2 &y = Y[(size_t)(jr >> 1) * ldy + r];
        if (accum) {
          v.x += y.x;
          v.y += y.y;
        }
        y = v;
      }
    }
  } else if (tid == 0) {
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(
                     taddr),
                 "r"(kTmemCols)
                 : "memory");
}

int chunkRows(size_t N, int p, int q) {
  const int tiles = ((2 * p + kM - 1) / kM) * ((2 * q + kN - 1) / kN);
  size_t rows = (N * tiles + 303) / 304;
  const size_t blk = (size_t)kSlab * kFold;
  rows = ((rows + blk - 1) / blk) * blk;
  if (rows < blk) rows = blk;
  return (int)rows;
}

} // namespace

// Scratch of gramTCExact for any p' <= p, q' <= q columns: column scales
// 2(p+q) doubles, exponents 2(p+q) ints and chunks x 2p' x 2q' partials. The
// row chunking gives a product with fewer output tiles more chunks, so a
// narrower product can need more partials than the widest one; the bound is
// the largest over every (M tiles, N tiles) count up to those of (p, q), each
// with its widest p', q'.
size_t exactGramScratchDoubles(size_t N, int p, int q) {
  const int mtiles = (2 * p + kM - 1) / kM, ntiles = (2 * q + kN - 1) / kN;
  size_t part = 0;
  for (int a = 1; a <= mtiles; ++a)
    for (int b = 1; b <= ntiles; ++b) {
      const int pp = std::min(p, a * kM / 2), qq = std::min(q, b * kN / 2);
      const size_t rows = chunkRows(N, pp, qq);
      const size_t chunks = (N + rows - 1) / rows;
      part = std::max(part, chunks * 4 * (size_t)pp * qq);
    }
  return part + 4 * (size_t)(p + q) + 8;
}

int *exactGramErrWord() {
  static int *d = [] {
    int *x = nullptr;
    if (cudaMalloc(&x, sizeof(int)) == cudaSuccess)
      cudaMemset(x, 0, sizeof(int));
    return x;
  }();
  return d;
}

// C = A^H B on the tensor cores to ~1e-13 relative (see the file comment);
// scratch holds exactGramScratchDoubles(N, p, q) doubles.
void gramTCExact(const double2 *A, size_t lda, int p, const double2 *B,
                 size_t ldb, int q, size_t N, double2 *C, int ldc,
                 double *scratch, cudaStream_t s) {
  if (p == 0 || q == 0 || N == 0) return;
  static const bool attr = [] {
    cudaFuncSetAttribute(exactGramKernel,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    return true;
  }();
  (void)attr;
  double *scA = scratch, *scB = scA + 2 * (size_t)p;
  int *eA = reinterpret_cast<int *>(scB + 2 * (size_t)q);
  int *eB = eA + 2 * (size_t)p;
  double *part = scB + 4 * (size_t)q + 2 * (size_t)p + 8;
  colMax(A, lda, p, N, scA, eA, s);
  colMax(B, ldb, q, N, scB, eB, s);
  const int rows = chunkRows(N, p, q);
  const int chunks = (int)((N + rows - 1) / rows);
  dim3 grid((2 * p + kM - 1) / kM, (2 * q + kN - 1) / kN, chunks);
  exactGramKernel<<<grid, kThr, kSmem, s>>>(A, lda, p, B, ldb, q, N, scA, eA,
                                            scB, eB, rows, part,
                                            exactGramErrWord());
  exactGramReduce<<<(unsigned)(((size_t)p * q * 32 + 255) / 256), 256, 0, s>>>(
      part, chunks, p, q, C, ldc);
}

// scratch of gemmVCExact in bytes: A column scales / exponents (2m), B
// column scales / exponents (2k), the digit image of B
size_t exactVCScratchBytes(int m, int k) {
  const size_t nslab = (2 * (size_t)m + kSlab - 1) / kSlab;
  const size_t ntile = (2 * (size_t)k + kN - 1) / kN;
  return 256 + 16 * (size_t)(2 * m + 2 * k) + ntile * nslab * kDig * kBBytes;
}

// Y = V C (accum: Y += V C) to ~1e-12 relative of the column maxima (see
// above)
void gemmVCExact(const double2 *V, size_t ldv, int m, const double2 *Cm,
                 int ldc, int k, double2 *Y, size_t ldy, size_t N,
                 void *scratch, cudaStream_t s, bool accum) {
  if (k == 0 || N == 0) return;
  if (m == 0) {
    if (accum) return;
    for (int j = 0; j < k; ++j)
      cudaMemsetAsync(Y + (size_t)j * ldy, 0, N * sizeof(double2), s);
    return;
  }
  static const bool attr = [] {
    cudaFuncSetAttribute(exactVCKernel,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    return true;
  }();
  (void)attr;
  const int nslab = (2 * m + kSlab - 1) / kSlab;
  const int ntile = (2 * k + kN - 1) / kN;
  unsigned char *base = static_cast<unsigned char *>(scratch);
  double *scA = reinterpret_cast<double *>(base);
  double *scB = scA + 2 * (size_t)m;
  int *eA = reinterpret_cast<int *>(scB + 2 * (size_t)k);
  int *eB = eA + 2 * (size_t)m;
  unsigned char *dig =
      base + (((size_t)16 * (2 * m + 2 * k) + 255) & ~(size_t)255);
  colMax(V, ldv, m, N, scA, eA, s);
  vcMaxKernel<<<(2 * k + 127) / 128, 128, 0, s>>>(Cm, ldc, m, k, eA, scB, eB);
  const size_t total = (size_t)nslab * kSlab * ntile * kN;
  vcPrepKernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(
      Cm, ldc, m, k, eA, eB, nslab, dig);
  dim3 grid((unsigned)((N + kM - 1) / kM), ntile);
  exactVCKernel<<<grid, kThr, kSmem, s>>>(V, ldv, m, eA, dig, scB, k, nslab, Y,
                                          ldy, N, accum ? 1 : 0,
                                          exactGramErrWord());
}

} // namespace ncgm
