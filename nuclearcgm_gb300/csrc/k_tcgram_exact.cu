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
// 256-row block the levels are combined exactly in 64-bit integers (held in
// registers over at most 16 blocks), converted to FP64 once per CTA, and the
// CTA's FP64 partial is summed with the other row chunks in a fixed order.
// Levels above kDig + 1 are dropped: the truncation error is ~2^(-7 kDig) of
// the column max per element (kDig = 6: ~2e-13 relative).
//
// Two passes per product:
//  1. A digitising kernel writes each operand's digits once, as the exact
//     K-major core-matrix image of the 128 x 32 BF16 tiles that the MMAs
//     read (48 KB per tile, kDig planes). It runs at full occupancy, so the
//     integer work of the splitting hides the memory latency.
//  2. The MMA kernel streams those tiles into shared memory with 16-byte
//     cp.async copies through a three-stage ring: the copies of slab s + 2
//     are in flight while the tensor cores work on slab s. One thread issues
//     the MMAs (tile M = 128, N = 64, instruction K = 16, two per slab per
//     digit pair) and commits them to the stage's mbarrier; after every 8
//     slabs all warps fold the level accumulators (tcgen05.ld) into their
//     64-bit sums. Every wait is bounded.
#include "ncgm_internal.cuh"

#include <cuda_bf16.h>

#include <algorithm>

namespace ncgm {

int smCount();

namespace {

constexpr int kDig = 6;                  // digits per value
constexpr int kM = 128, kN = 64;         // D tile
constexpr int kSlab = 32;                // K rows per stage (2 MMAs of K 16)
constexpr int kFold = 8;                 // slabs per exact accumulation block
constexpr int kMaxFolds = 16;            // fold blocks per 64-bit sum
constexpr int kThr = 256;
constexpr int kABytes = kM * kSlab * 2;  // one digit plane of A: 8 KB
constexpr int kBBytes = kN * kSlab * 2;  // one digit plane of B: 4 KB
constexpr int kTile = kDig * kABytes;    // a digitised 128 x 32 tile: 48 KB
constexpr int kBuf = kDig * (kABytes + kBBytes); // one stage: 72 KB
constexpr int kStages = 3;
constexpr int kSmem = kStages * kBuf + 128; // + barriers, TMEM slot
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

// the same wait without the suspend-time hint, bounded by the SM clock
// (~1 s): for the one thread whose waits gate the next MMAs
__device__ __forceinline__ bool waitSpin(uint64_t *bar, uint32_t phase) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t done;
    asm volatile("{\n .reg .pred p;\n"
                 " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                 " selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(done)
                 : "r"(sAddr(bar)), "r"(phase)
                 : "memory");
    if (done) return true;
    if (clock64() - t0 > (1ll << 31)) return false;
  }
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
  const double2 *col = X + (size_t)c * ld;
  size_t r = r0 + threadIdx.x;
  for (; r + 3 * blockDim.x < r1; r += 4 * blockDim.x) {
    double2 v[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = col[r + i * blockDim.x];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      mr = fmax(mr, fabs(v[i].x));
      mi = fmax(mi, fabs(v[i].y));
    }
  }
  for (; r < r1; r += blockDim.x) {
    const double2 v = col[r];
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
  const int chunks = (int)std::min<size_t>(
      std::max<size_t>(1, (size_t)(4 * smCount()) / (size_t)std::max(p, 1)),
      (N + 4095) / 4096);
  const size_t rows = (N + chunks - 1) / chunks;
  cudaMemsetAsync(sc, 0, 2 * (size_t)p * sizeof(double), s);
  colMaxKernel<<<dim3(p, chunks), 256, 0, s>>>(X, ld, p, N, rows, sc);
  colExpKernel<<<(2 * p + 127) / 128, 128, 0, s>>>(2 * p, sc, ex);
}

// packs the BF16 digits t of 8 consecutive values into one 16-byte row of a
// core matrix (element k at byte 2k)
__device__ __forceinline__ uint4 packRow(const float (*d)[kDig], int t) {
  uint4 w;
  __nv_bfloat162 b;
  b = __floats2bfloat162_rn(d[0][t], d[1][t]);
  w.x = *reinterpret_cast<uint32_t *>(&b);
  b = __floats2bfloat162_rn(d[2][t], d[3][t]);
  w.y = *reinterpret_cast<uint32_t *>(&b);
  b = __floats2bfloat162_rn(d[4][t], d[5][t]);
  w.z = *reinterpret_cast<uint32_t *>(&b);
  b = __floats2bfloat162_rn(d[6][t], d[7][t]);
  w.w = *reinterpret_cast<uint32_t *>(&b);
  return w;
}

// Digit image of the interleaved block S (N x 2p) for the Gram: the tile (M
// tile mt, slab s) holds real columns 128 mt .. 128 mt + 127 as tile rows
// and lattice rows 32 s .. 32 s + 31 as K, at img + (mt nslab + s) kTile.
// Thread (complex column cc of the tile, 8-row group kq) loads 8 consecutive
// entries (4 lanes read 512 contiguous bytes) and writes one 16-byte core
// row per digit for Re (tile row 2 cc) and Im (2 cc + 1). Rows past N and
// columns past p are zero digits.
__global__ void __launch_bounds__(256)
    digitizeGramKernel(const double2 *__restrict__ X, size_t ld, int p,
                       size_t N, const int *__restrict__ ex, int nslab,
                       unsigned char *__restrict__ img) {
  const int s = blockIdx.x, mt = blockIdx.y;
  const int kq = threadIdx.x & 3, cc = threadIdx.x >> 2;
  const int c = mt * (kM / 2) + cc;
  const size_t r0 = (size_t)s * kSlab + 8 * kq;
  double2 v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
    v[i] = (c < p && r0 + i < N) ? X[(size_t)c * ld + r0 + i]
                                 : make_double2(0.0, 0.0);
  unsigned char *base = img + ((size_t)mt * nslab + s) * (size_t)kTile;
#pragma unroll
  for (int part = 0; part < 2; ++part) {
    const int e = c < p ? ex[2 * c + part] : 0;
    float d[8][kDig];
#pragma unroll
    for (int i = 0; i < 8; ++i)
      digits(scaledInt(part ? v[i].y : v[i].x, e), d[i]);
    const uint32_t o = off16(2 * cc + part, 8 * kq);
#pragma unroll
    for (int t = 0; t < kDig; ++t)
      *reinterpret_cast<uint4 *>(base + (size_t)t * kABytes + o) =
          packRow(d, t);
  }
}

// Digit image of the interleaved block V (N x 2m) for Y = V C: the tile (row
// tile mt, K slab s) holds lattice rows 128 mt .. 128 mt + 127 as tile rows
// and real columns 32 s .. 32 s + 31 as K, at img + (mt nslab + s) kTile.
// Task (row, 8-column group kq): 4 complex entries of one lattice row (a
// warp reads 512 contiguous bytes per column), one 16-byte core row per
// digit.
__global__ void __launch_bounds__(256)
    digitizeVCKernel(const double2 *__restrict__ V, size_t ld, int m,
                     size_t N, const int *__restrict__ ex, int nslab,
                     unsigned char *__restrict__ img) {
  const int mt = blockIdx.x, s = blockIdx.y;
  unsigned char *base = img + ((size_t)mt * nslab + s) * (size_t)kTile;
  for (int task = threadIdx.x; task < kM * (kSlab / 8); task += 256) {
    const int row = task % kM, kq = task / kM;
    const size_t r = (size_t)mt * kM + row;
    const int c0 = s * (kSlab / 2) + 4 * kq;
    double2 v[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
      v[i] = (c0 + i < m && r < N) ? V[(size_t)(c0 + i) * ld + r]
                                   : make_double2(0.0, 0.0);
    float d[8][kDig];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const bool in = c0 + i < m;
      digits(scaledInt(v[i].x, in ? ex[2 * (c0 + i)] : 0), d[2 * i]);
      digits(scaledInt(v[i].y, in ? ex[2 * (c0 + i) + 1] : 0), d[2 * i + 1]);
    }
    const uint32_t o = off16(row, 8 * kq);
#pragma unroll
    for (int t = 0; t < kDig; ++t)
      *reinterpret_cast<uint4 *>(base + (size_t)t * kABytes + o) =
          packRow(d, t);
  }
}

// instruction descriptor: D FP32, A/B BF16, K-major, M = 128, N = n
__host__ __device__ constexpr uint32_t idescN(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(kM >> 4) << 24);
}

__device__ __forceinline__ void mmaIssue(uint32_t td, uint64_t ad,
                                         uint64_t bd, uint32_t idesc,
                                         uint32_t accum) {
  asm volatile("{\n .reg .pred pa;\n setp.ne.b32 pa, %4, 0;\n"
               " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, pa;\n"
               "}\n" ::"r"(td),
               "l"(ad), "l"(bd), "r"(idesc), "r"(accum)
               : "memory");
}

// the MMAs of one 32-row slab. Level l = t + u collects the products of A
// digit t and B digit u. B's digit planes lie 4 KB (8 row groups) apart, so
// planes u0 .. u1 read as one B operand of N = 64 (u1 - u0 + 1) rows, and
// one MMA with A digit t writes the levels t + u0 .. t + u1 into their
// adjacent 64-column blocks of tensor memory: per 16 K, A digit 0 takes B
// digits 0-3 and 4-5, digit 1 takes 0-3 and 4, digits 2 .. 5 take 0 ..
// 5 - t (8 MMAs instead of 21). aBase / bBase: shared addresses of digit
// plane 0 of A and B. first: the slab opens a fold block (A digit 0 writes
// every level first and overwrites). Descriptors are the plane-0
// descriptor plus a constant: the start-address field holds address / 16
// and shared addresses stay below 256 KB, so the addition never carries.
__device__ __forceinline__ void issueSlab(uint32_t taddr, uint32_t aBase,
                                          uint32_t bBase, bool first) {
  static_assert(kDig == 6 && kBBytes == 8 * kSBO, "stacked B planes");
  const uint64_t a0 = smemDesc(aBase), b0 = smemDesc(bBase);
#pragma unroll
  for (int ks = 0; ks < kSlab / 16; ++ks) {
    const uint32_t ko = ks * 2 * kLBO;
    const uint32_t acc0 = (ks == 0 && first) ? 0u : 1u;
#pragma unroll
    for (int t = 0; t < kDig; ++t) {
      const uint64_t ad = a0 + ((t * kABytes + ko) >> 4);
      // runs of B digits [u0, u1] with at most 4 planes (N <= 256)
#pragma unroll
      for (int u0 = 0; u0 < kDig - t; u0 += 4) {
        const int u1 = min(u0 + 3, kDig - 1 - t);
        const uint64_t bd = b0 + ((u0 * kBBytes + ko) >> 4);
        mmaIssue(taddr + (uint32_t)((t + u0) * kN), ad, bd,
                 idescN(kN * (u1 - u0 + 1)), t == 0 ? acc0 : 1u);
      }
    }
  }
}

// adds the level sums of the finished fold block, combined exactly, to the
// 64-bit sums of TMEM lane row (lw 32 + lane), columns cBeg .. cBeg + 31:
// sum_l L_l 2^(7 (kDig-1-l)) = (L0 2^7 + L1) 2^28 + (L2 2^7 + L3) 2^14 +
// (L4 2^7 + L5), each pair in 32 bits (|L_l| < 2^23), the sum below 2^58.1,
// so kMaxFolds = 16 blocks stay below 2^63. Two levels per load wait.
static_assert(kDig == 6, "foldLevels combines three level pairs");
__device__ __forceinline__ void tmemLoad16(uint32_t ta, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, "
      "%7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]),
        "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]),
        "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
        "=r"(v[15])
      : "r"(ta));
}
__device__ __forceinline__ void foldLevels(uint32_t taddr, int lw, int cBeg,
                                           long long acc[32]) {
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const uint32_t ta =
        taddr + ((uint32_t)(lw * 32) << 16) + (uint32_t)(cBeg + 16 * h);
    int pr[3][16];
#pragma unroll
    for (int pl = 0; pl < 3; ++pl) {
      uint32_t hi[16], lo[16];
      tmemLoad16(ta + (uint32_t)(2 * pl * kN), hi);
      tmemLoad16(ta + (uint32_t)((2 * pl + 1) * kN), lo);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int j = 0; j < 16; ++j)
        pr[pl][j] = __float2int_rn(__uint_as_float(hi[j])) * 128 +
                    __float2int_rn(__uint_as_float(lo[j]));
    }
#pragma unroll
    for (int j = 0; j < 16; ++j)
      acc[16 * h + j] += ((long long)pr[0][j] << 28) +
                         ((long long)pr[1][j] << 14) + (long long)pr[2][j];
  }
}

// a 2^e rounded to the nearest double (ties to even) with integer
// operations, equal to (double)a * 2^e (the FP64 pipe retires two
// operations per clock per SM); results outside the normal range take the
// FP64 path
__device__ __forceinline__ double scaledDouble(long long a, int e) {
  if (a == 0) return 0.0;
  const unsigned long long sign = a < 0 ? 1ull << 63 : 0ull;
  unsigned long long m = a < 0 ? 0ull - (unsigned long long)a
                               : (unsigned long long)a;
  const int lz = __clzll(m);
  m <<= lz; // leading one at bit 63
  unsigned long long keep = m >> 11;
  const unsigned long long rest = m & 0x7FFull;
  keep += (rest > 0x400ull || (rest == 0x400ull && (keep & 1ull))) ? 1ull
                                                                    : 0ull;
  int ex = 63 - lz + e;
  if (keep >> 53) {
    keep >>= 1;
    ++ex;
  }
  if (ex < -1022 || ex > 1023) return ldexp((double)a, e);
  return __longlong_as_double((long long)(sign |
                                          ((unsigned long long)(ex + 1023)
                                           << 52) |
                                          (keep & 0xFFFFFFFFFFFFFull)));
}

__device__ __forceinline__ void tmemAlloc(uint32_t *slot) {
  asm volatile(
      "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::
          "r"(sAddr(slot)),
      "r"(kTmemCols)
      : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::
                   : "memory");
}
__device__ __forceinline__ void tmemFree(uint32_t taddr) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(
                   taddr),
               "r"(kTmemCols)
               : "memory");
}

// a 1-D bulk copy global -> shared that completes on an mbarrier's tx count
__device__ __forceinline__ void bulkCopy(uint32_t dst, const void *src,
                                         uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::"
               "bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// The copy / MMA pipeline of one CTA. Barriers after the stages: mma[st]
// (MMA commits of the slab in stage st), full[st] (its bulk copies, tx
// count), fold (one commit after each fold block's last slab). Thread 0
// issues copies and MMAs and waits on every phase of mma and full in order;
// the other threads wait only on fold, once per block, and every block ends
// with a CTA barrier, so no barrier runs two phases ahead of a waiter.
struct Pipe {
  uint64_t *bar;
  uint32_t *tslot;
  int committed = 0, landedN = 0, issued = 0; // thread 0's counts of slabs
  __device__ explicit Pipe(unsigned char *sm)
      : bar(reinterpret_cast<uint64_t *>(sm + kStages * kBuf)),
        tslot(reinterpret_cast<uint32_t *>(bar + 2 * kStages + 1)) {}
  __device__ uint32_t full(int st) const { return sAddr(bar + kStages + st); }
  __device__ void init(int warp, int tid) {
    if (warp == 0) tmemAlloc(tslot);
    if (tid == 0) {
      for (int i = 0; i < 2 * kStages + 1; ++i)
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(
            sAddr(bar + i)));
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  __device__ uint32_t taddr() const { return *tslot; }
  __device__ void expect(int st, uint32_t bytes) const {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::
                     "r"(full(st)),
                 "r"(bytes)
                 : "memory");
  }
  // the copies of slab s have landed (thread 0, in slab order)
  __device__ bool landed(int s) {
    if (!waitSpin(bar + kStages + s % kStages, (s / kStages) & 1))
      return false;
    landedN = s + 1;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    return true;
  }
  __device__ void commit(int s, bool foldPt) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one."
                 "shared::cluster.b64 [%0];" ::"r"(sAddr(bar + s % kStages))
                 : "memory");
    if (foldPt)
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one."
                   "shared::cluster.b64 [%0];" ::"r"(sAddr(bar + 2 * kStages))
                   : "memory");
    committed = s + 1;
  }
  // the MMAs of slab s are complete (thread 0, in slab order)
  __device__ bool mmaDone(int s) const {
    return waitSpin(bar + s % kStages, (s / kStages) & 1);
  }
  // all threads: fold block f's MMAs are complete. A thread 0 that gave up
  // arrives itself, so the others return at once; false ends the loop.
  __device__ bool foldWait(int tid, bool ok, int f) {
    if (tid == 0 && !ok)
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                       sAddr(bar + 2 * kStages))
                   : "memory");
    if (ok && !waitBar(bar + 2 * kStages, f & 1)) ok = false;
    if (!__syncthreads_and(ok)) return false;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncwarp();
    return true;
  }
  // the block's accumulators are read: thread 0 may overwrite them
  __device__ void foldDone() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  // drains what thread 0 left in flight (after an early exit) and returns
  // the CTA-wide status
  __device__ bool finish(int tid, bool ok) {
    if (tid == 0) {
      for (int s = landedN; s < issued; ++s)
        waitBar(bar + kStages + s % kStages, (s / kStages) & 1);
      if (committed > 0) mmaDone(committed - 1);
    }
    return __syncthreads_and(ok);
  }
  __device__ void release(int warp, uint32_t taddr) {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) tmemFree(taddr);
  }
};


// C partials of one (M tile mt, N tile nt, row chunk): the digit tiles of
// S^T (imgA, tile mt) and T^T (imgB, half nt & 1 of tile nt >> 1) over the
// chunk's slabs (for a Gram of a block with itself imgB is imgA). Thread 0
// runs the pipeline (bulk copies, MMAs, commits); all warps join at the
// folds.
__global__ void __launch_bounds__(kThr, 1)
    exactGramKernel(const unsigned char *__restrict__ imgA,
                    const unsigned char *__restrict__ imgB, int p, int q,
                    int nslab, int slabsPerChunk,
                    const int *__restrict__ eA,
                    const int *__restrict__ eB, double *__restrict__ part,
                    int *err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  Pipe P(sm);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int mt = blockIdx.x, nt = blockIdx.y, chunk = blockIdx.z;
  const int g0 = chunk * slabsPerChunk;
  const int ns = min(nslab, g0 + slabsPerChunk) - g0;
  const unsigned char *srcA = imgA + ((size_t)mt * nslab + g0) * kTile;
  const unsigned char *srcB =
      imgB + ((size_t)(nt >> 1) * nslab + g0) * kTile + (nt & 1) * kBBytes;
  // slab s of the chunk into stage s % kStages (thread 0)
  auto copySlab = [&](int s) {
    const int st = s % kStages;
    const uint32_t dst = sAddr(sm + st * kBuf);
    P.expect(st, kTile + kDig * kBBytes);
    bulkCopy(dst, srcA + (size_t)s * kTile, kTile, P.full(st));
    for (int t = 0; t < kDig; ++t)
      bulkCopy(dst + kDig * kABytes + t * kBBytes,
               srcB + (size_t)s * kTile + (size_t)t * kABytes, kBBytes,
               P.full(st));
  };
  P.init(warp, tid);
  if (tid == 0) {
    copySlab(0);
    if (ns > 1) copySlab(1);
    P.issued = ns > 1 ? 2 : 1;
  }
  const uint32_t taddr = P.taddr();
  const int lw = warp & 3, cBeg = (warp >> 2) * (kN / 2);
  long long acc[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) acc[j] = 0;
  bool ok = true;
  int fold = 0;

  for (int s = 0; s < ns; ++s) {
    const int st = s % kStages;
    const bool foldPt = s % kFold == kFold - 1 || s == ns - 1;
    // warp 0's other lanes wait at the warp barrier while lane 0 works
    if (warp == 0) {
      if (lane == 0 && ok) {
        const uint32_t base = sAddr(sm + st * kBuf);
        if (!P.landed(s)) {
          ok = false;
        } else {
          issueSlab(taddr, base, base + kDig * kABytes, s % kFold == 0);
          P.commit(s, foldPt);
          // refill: slab s + 2 goes to the stage that the MMAs of slab s - 1
          // read
          if (s + 2 < ns) {
            if (s >= 1 && !P.mmaDone(s - 1))
              ok = false;
            else {
              copySlab(s + 2);
              ++P.issued;
            }
          }
        }
      }
      __syncwarp();
    }
    if (foldPt) {
      if (!P.foldWait(tid, ok, fold++)) {
        ok = false;
        break;
      }
      foldLevels(taddr, lw, cBeg, acc);
      P.foldDone();
    }
  }
  ok = P.finish(tid, ok);
  if (ok) {
    // value = sum 2^(eA + eB - 7 (kDig+1))
    const int gr = mt * kM + lw * 32 + lane;
    if (gr < 2 * p) {
      double *dst = part + ((size_t)chunk * 2 * p + gr) * (2 * q);
      const int er = eA[gr] - 7 * (kDig + 1);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int gc = nt * kN + cBeg + j;
        if (gc < 2 * q) dst[gc] = scaledDouble(acc[j], er + eB[gc]);
      }
    }
  } else if (tid == 0) {
    atomicExch(err, 1);
  }
  P.release(warp, taddr);
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
// one warp per real column jr of B: lanes take rows c = lane, lane + 32, ...
// and the largest exponent is reduced over the warp
__global__ void vcMaxKernel(const double2 *__restrict__ Cm, int ldc, int m,
                            int k, const int *__restrict__ eA, double *scB,
                            int *eB) {
  const int jr = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (jr >= 2 * k) return;
  const int j = jr >> 1, b = jr & 1;
  int emax = -100000;
  for (int c = lane; c < m; c += 32) {
    const double2 t = Cm[(size_t)j * ldc + c];
    // rows 2c, 2c+1 of column jr: (Re, -Im) for b = 0, (Im, Re) for b = 1
    const double v0 = b ? t.y : t.x, v1 = b ? t.x : -t.y;
    int e0 = -100000, e1 = -100000;
    if (v0 != 0.0) { frexp(v0, &e0); e0 += eA[2 * c]; }
    if (v1 != 0.0) { frexp(v1, &e1); e1 += eA[2 * c + 1]; }
    emax = max(emax, max(e0, e1));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  if (lane == 0) {
    if (emax == -100000) emax = 0; // an all-zero column
    eB[jr] = emax;                  // |B[., jr]| 2^eA < 2^emax
    scB[jr] = ldexp(1.0, emax);
  }
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

// Y tiles (row tile mt of 128 rows, column tile nt of 64 real columns), tile
// index mt ntiles + nt; CTA b takes tiles b, b + G, b + 2G, ... (G CTAs, one
// per SM) and runs the slabs of all its tiles through one copy/MMA pipeline,
// so the copies of the next tile overlap the fold and the stores of the
// current one. A: the digit image of V (imgV, tile (mt, s)); B: the
// precomputed digit image of C (dig, tile (nt, s)).
__global__ void __launch_bounds__(kThr, 1)
    exactVCKernel(const unsigned char *__restrict__ imgV,
                  const unsigned char *__restrict__ dig,
                  const int *__restrict__ eB, int k, int nslab,
                  int ntiles, int tiles, double2 *__restrict__ Y, size_t ldy,
                  size_t N, int accum, int *err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  Pipe P(sm);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int G = gridDim.x;
  const int myTiles = (tiles - (int)blockIdx.x + G - 1) / G;
  const int total = myTiles * nslab;
  // step i of the CTA's sequence (tile i / nslab, slab i % nslab) into stage
  // i % kStages (thread 0)
  auto copyStep = [&](int i) {
    const int tile = (int)blockIdx.x + (i / nslab) * G, s = i % nslab;
    const int mt = tile / ntiles, nt = tile % ntiles;
    const int st = i % kStages;
    const uint32_t dst = sAddr(sm + st * kBuf);
    P.expect(st, kTile + kDig * kBBytes);
    bulkCopy(dst, imgV + ((size_t)mt * nslab + s) * kTile, kTile, P.full(st));
    bulkCopy(dst + kDig * kABytes,
             dig + ((size_t)nt * nslab + s) * (size_t)(kDig * kBBytes),
             kDig * kBBytes, P.full(st));
  };
  P.init(warp, tid);
  if (tid == 0 && total > 0) {
    copyStep(0);
    if (total > 1) copyStep(1);
    P.issued = total > 1 ? 2 : 1;
  }
  const uint32_t taddr = P.taddr();
  const int lw = warp & 3, cBeg = (warp >> 2) * (kN / 2);
  long long acc[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) acc[j] = 0;
  bool ok = true;
  int fold = 0;

  for (int i = 0; i < total; ++i) {
    const int st = i % kStages, s = i % nslab;
    const bool foldPt = s % kFold == kFold - 1 || s == nslab - 1;
    if (warp == 0) {
      if (lane == 0 && ok) {
        const uint32_t base = sAddr(sm + st * kBuf);
        if (!P.landed(i)) {
          ok = false;
        } else {
          issueSlab(taddr, base, base + kDig * kABytes, s % kFold == 0);
          P.commit(i, foldPt);
          if (i + 2 < total) {
            if (i >= 1 && !P.mmaDone(i - 1))
              ok = false;
            else {
              copyStep(i + 2);
              ++P.issued;
            }
          }
        }
      }
      __syncwarp();
    }
    if (foldPt) {
      if (!P.foldWait(tid, ok, fold++)) {
        ok = false;
        break;
      }
      foldLevels(taddr, lw, cBeg, acc);
      P.foldDone();
      if (s == nslab - 1) {
        // Y[j][r] = (acc[2j] 2^eB[2j], acc[2j+1] 2^eB[2j+1]) 2^(-7 (kDig+1))
        constexpr int ew = -7 * (kDig + 1);
        const int tile = (int)blockIdx.x + (i / nslab) * G;
        const int mt = tile / ntiles, nt = tile % ntiles;
        const size_t r = (size_t)mt * kM + lw * 32 + lane;
        if (r < N) {
#pragma unroll
          for (int j = 0; j < 32; j += 2) {
            const int jr = nt * kN + cBeg + j;
            if (jr < 2 * k) {
              double2 v = make_double2(scaledDouble(acc[j], ew + eB[jr]),
                                       scaledDouble(acc[j + 1], ew + eB[jr + 1]));
              double2 &y = Y[(size_t)(jr >> 1) * ldy + r];
              if (accum) {
                v.x += y.x;
                v.y += y.y;
              }
              y = v;
            }
          }
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) acc[j] = 0;
      }
    }
  }
  ok = P.finish(tid, ok);
  if (!ok && tid == 0) atomicExch(err, 1);
  P.release(warp, taddr);
}

// rows per chunk of the Gram grid: a multiple of one fold block and at most
// kMaxFolds blocks (the 64-bit sums), chosen to minimise the waves of one
// CTA per SM times the rows of a chunk (plus a fixed cost per CTA)
int chunkRows(size_t N, int p, int q) {
  const size_t tiles =
      (size_t)((2 * p + kM - 1) / kM) * (size_t)((2 * q + kN - 1) / kN);
  const size_t blk = (size_t)kSlab * kFold;
  const size_t sms = (size_t)smCount();
  size_t best = blk;
  double bestCost = 1e300;
  for (size_t rows = blk; rows <= kMaxFolds * blk; rows += blk) {
    const size_t chunks = (N + rows - 1) / rows;
    const size_t waves = (chunks * tiles + sms - 1) / sms;
    const double cost = (double)waves * (double)(std::min(rows, N) + 2 * kSlab);
    if (cost <= bestCost) { // ties: the longer chunks (fewer partials)
      bestCost = cost;
      best = rows;
    }
    if (rows >= N) break;
  }
  return (int)best;
}

size_t gramImageBytes(size_t N, int p) {
  const size_t nslab = (N + kSlab - 1) / kSlab;
  return nslab * (size_t)((2 * p + kM - 1) / kM) * kTile;
}
size_t gramHeaderBytes(int p, int q) {
  return ((sizeof(double) * (4 * (size_t)(p + q) + 8)) + 255) & ~(size_t)255;
}

} // namespace

// Scratch of gramTCExact for any p' <= p, q' <= q columns: column scales and
// exponents, the digit images of both operands, and chunks x 2p' x 2q'
// partials. The row chunking gives a product with fewer output tiles more
// chunks, so a narrower product can need more partials than the widest one;
// the bound is the largest over every (M tiles, N tiles) count up to those
// of (p, q), each with its widest p', q'.
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
  const size_t bytes = gramHeaderBytes(p, q) + gramImageBytes(N, p) +
                       gramImageBytes(N, q) + sizeof(double) * part + 256;
  return (bytes + sizeof(double) - 1) / sizeof(double);
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
// scratch holds exactGramScratchDoubles(N, p, q) doubles (256-byte aligned).
// A Gram of a block with itself (A == B, same ld and width) digitises it once.
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
  const bool self = A == B && lda == ldb && p == q;
  double *scA = scratch, *scB = scA + 2 * (size_t)p;
  int *eA = reinterpret_cast<int *>(scB + 2 * (size_t)q);
  int *eB = eA + 2 * (size_t)p;
  unsigned char *imgA =
      reinterpret_cast<unsigned char *>(scratch) + gramHeaderBytes(p, q);
  unsigned char *imgB = imgA + gramImageBytes(N, p);
  double *part = reinterpret_cast<double *>(imgB + gramImageBytes(N, q));
  const int nslab = (int)((N + kSlab - 1) / kSlab);
  colMax(A, lda, p, N, scA, eA, s);
  digitizeGramKernel<<<dim3(nslab, (2 * p + kM - 1) / kM), 256, 0, s>>>(
      A, lda, p, N, eA, nslab, imgA);
  if (self) {
    imgB = imgA;
    eB = eA;
  } else {
    colMax(B, ldb, q, N, scB, eB, s);
    digitizeGramKernel<<<dim3(nslab, (2 * q + kM - 1) / kM), 256, 0, s>>>(
        B, ldb, q, N, eB, nslab, imgB);
  }
  const int rows = chunkRows(N, p, q);
  const int spc = rows / kSlab;
  const int chunks = (nslab + spc - 1) / spc;
  dim3 grid((2 * p + kM - 1) / kM, (2 * q + kN - 1) / kN, chunks);
  exactGramKernel<<<grid, kThr, kSmem, s>>>(imgA, imgB, p, q, nslab, spc,
                                            eA, eB, part,
                                            exactGramErrWord());
  exactGramReduce<<<(unsigned)(((size_t)p * q * 32 + 255) / 256), 256, 0, s>>>(
      part, chunks, p, q, C, ldc);
}

// scratch of gemmVCExact in bytes: A column scales / exponents (2m), B
// column scales / exponents (2k), the digit image of B and that of V
size_t exactVCScratchBytes(size_t N, int m, int k) {
  const size_t nslab = (2 * (size_t)m + kSlab - 1) / kSlab;
  const size_t ntile = (2 * (size_t)k + kN - 1) / kN;
  const size_t mtile = (N + kM - 1) / kM;
  return 512 + 16 * (size_t)(2 * m + 2 * k) + ntile * nslab * kDig * kBBytes +
         mtile * nslab * kTile;
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
  const int mtile = (int)((N + kM - 1) / kM);
  unsigned char *base = static_cast<unsigned char *>(scratch);
  double *scA = reinterpret_cast<double *>(base);
  double *scB = scA + 2 * (size_t)m;
  int *eA = reinterpret_cast<int *>(scB + 2 * (size_t)k);
  int *eB = eA + 2 * (size_t)m;
  unsigned char *dig =
      base + (((size_t)16 * (2 * m + 2 * k) + 255) & ~(size_t)255);
  unsigned char *imgV = dig + (size_t)ntile * nslab * kDig * kBBytes;
  colMax(V, ldv, m, N, scA, eA, s);
  vcMaxKernel<<<(2 * k + 3) / 4, 128, 0, s>>>(Cm, ldc, m, k, eA, scB, eB);
  const size_t total = (size_t)nslab * kSlab * ntile * kN;
  vcPrepKernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(
      Cm, ldc, m, k, eA, eB, nslab, dig);
  digitizeVCKernel<<<dim3(mtile, nslab), 256, 0, s>>>(V, ldv, m, N, eA, nslab,
                                                      imgV);
  const int tiles = mtile * ntile;
  const int G = std::min(tiles, smCount());
  exactVCKernel<<<G, kThr, kSmem, s>>>(imgV, dig, eB, k, nslab, ntile, tiles,
                                       Y, ldy, N, accum ? 1 : 0,
                                       exactGramErrWord());
}

} // namespace ncgm
