// Tensor-core (tcgen05, kind::tf32) Gram products for the mixed-precision
// GCG: C = A^H B for complex FP64 column blocks A (N x p) and B (N x q).
//
// The complex product is one real product of the stacked blocks
//   [Re A; Im A]^T-rows (2p x N)  times  [Re B; Im B] (N x 2q),
//   C_re = D[i][j] + D[p+i][q+j],  C_im = D[i][q+j] - D[p+i][j].
// Every FP64 value is rounded to FP32 and split into two TF32 parts
// (hi = tf32(x), lo = tf32(x - hi)); a D tile accumulates hi*hi + hi*lo +
// lo*hi in FP32 in tensor memory (TMEM) over one chunk of rows, and the
// chunk partials are summed in FP64 in a fixed order. The result carries
// FP32-level relative error (~1e-7 of the entries), which is what the
// mixed-precision form accepts for its Gram products; the projected
// eigenproblem and the Cholesky factorisation stay in FP64.
//
// One CTA of 8 warps computes one 128 x 128 tile of D over one chunk of rows:
// all threads stage 32-row slabs of both operands into shared memory
// (double-buffered, core-matrix layout without swizzle), one thread issues
// the tcgen05.mma instructions and commits them to an mbarrier, and after
// the last slab the warps read the accumulator out of TMEM (tcgen05.ld
// 32x32b; a warp may read only its quarter of the TMEM lanes, so warps w and
// w + 4 split the columns of lanes 32 (w % 4) ..). Every wait is bounded; on a timeout the CTA records
// an error, waits (bounded) for its own MMAs and frees its TMEM.
#include "ncgm_internal.cuh"

#include <algorithm>

namespace ncgm {

namespace {

constexpr int kTile = 128;     // rows of a D tile (M) and columns (N)
constexpr int kSlab = 32;      // K rows staged per step
constexpr int kTileBytes = kTile * kSlab * 4;       // one operand part
constexpr int kBufBytes = 4 * kTileBytes;           // A hi/lo, B hi/lo
constexpr int kSmemBytes = 2 * kBufBytes + 64;      // two buffers + barriers
constexpr uint32_t kLBO = 128;  // bytes between K-adjacent core matrices
constexpr uint32_t kSBO = 1024; // bytes between M/N-adjacent 8-row groups

__device__ __forceinline__ uint32_t sAddr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor: K-major, no swizzle (core matrices of
// 8 rows x 16 bytes), start address, LBO (K direction), SBO (M/N direction)
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((kLBO >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((kSBO >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46; // descriptor version for tcgen05
  return d;              // base offset 0, swizzle none
}

// instruction descriptor: D FP32, A/B TF32, both K-major, M = N = 128
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) |
                            ((uint32_t)(kTile >> 3) << 17) |
                            ((uint32_t)(kTile >> 4) << 24);

// byte offset of element (row, k) of a 128 x 32 operand tile
__device__ __forceinline__ uint32_t tileOff(int row, int k) {
  return (uint32_t)(row >> 3) * kSBO + (uint32_t)(k >> 2) * kLBO +
         (uint32_t)(row & 7) * 16u + (uint32_t)(k & 3) * 4u;
}

__device__ __forceinline__ float tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void mbarInitT(uint64_t *bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sAddr(bar)),
               "r"(count));
}
__device__ __forceinline__ bool mbarWaitT(uint64_t *bar, uint32_t phase) {
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

// element of the stacked real block: real row c in [0, 2p) of column block X
__device__ __forceinline__ float stacked(const double2 *X, size_t ld, int p,
                                         int c, size_t r) {
  if (c < p) return (float)X[(size_t)c * ld + r].x;
  if (c < 2 * p) return (float)X[(size_t)(c - p) * ld + r].y;
  return 0.f;
}

constexpr int kThreads = 256; // 8 warps: staging by all, epilogue split

__global__ void __launch_bounds__(kThreads, 1)
    tcGramKernel(const double2 *__restrict__ A, size_t lda, int p,
                 const double2 *__restrict__ B, size_t ldb, int q, size_t N,
                 int rowsPerChunk, float *__restrict__ part, int *err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + 2 * kBufBytes);
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
        "r"(kTile)
        : "memory");
    asm volatile(
        "tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::
            : "memory");
  }
  if (tid == 0) {
    mbarInitT(&mbar[0], 1);
    mbarInitT(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t taddr = *tslot;
  bool ok = true;
  int committed = 0; // commits issued (thread 0)

  for (int s = 0; s < nslab && ok; ++s) {
    const int b = s & 1;
    if (s >= 2 && !mbarWaitT(&mbar[b], ((s - 2) >> 1) & 1)) ok = false;
    if (!__syncthreads_and(ok)) {
      ok = false;
      break;
    }
    unsigned char *buf = sm + b * kBufBytes;
    // a warp stages one 8 x 4 core matrix per step: lane = (row & 7, k & 3),
    // so its 32 stores fill 128 contiguous bytes (no bank conflicts) and
    // every 4 lanes read 4 consecutive rows of one column; all the slab's
    // loads of a thread are issued before any is used
    constexpr int kPer = (kTile / 8) * (kSlab / 4) / (kThreads / 32);
    const int r8 = lane >> 2, k4 = lane & 3;
    float va[kPer], vb[kPer];
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int g = warp + (kThreads / 32) * i;
      const int row = (g >> 3) * 8 + r8, k = (g & 7) * 4 + k4;
      const size_t r = r0 + (size_t)s * kSlab + k;
      const bool rv = r < r1;
      va[i] = rv ? stacked(A, lda, p, mt * kTile + row, r) : 0.f;
      vb[i] = rv ? stacked(B, ldb, q, nt * kTile + row, r) : 0.f;
    }
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const int g = warp + (kThreads / 32) * i;
      const int row = (g >> 3) * 8 + r8, k = (g & 7) * 4 + k4;
      const float ah = tf32(va[i]), al = tf32(va[i] - ah);
      const float bh = tf32(vb[i]), bl = tf32(vb[i] - bh);
      const uint32_t o = tileOff(row, k);
      *reinterpret_cast<float *>(buf + o) = ah;
      *reinterpret_cast<float *>(buf + kTileBytes + o) = al;
      *reinterpret_cast<float *>(buf + 2 * kTileBytes + o) = bh;
      *reinterpret_cast<float *>(buf + 3 * kTileBytes + o) = bl;
    }
    // generic-proxy stores -> async proxy (tensor core operand reads)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t base = sAddr(buf);
      for (int ks = 0; ks < kSlab / 8; ++ks) {
        const uint32_t kofs = ks * 2 * kLBO;
        const uint64_t ah = smemDesc(base + kofs);
        const uint64_t al = smemDesc(base + kTileBytes + kofs);
        const uint64_t bh = smemDesc(base + 2 * kTileBytes + kofs);
        const uint64_t bl = smemDesc(base + 3 * kTileBytes + kofs);
        const uint64_t as[3] = {ah, ah, al}, bs[3] = {bh, bl, bh};
        for (int t = 0; t < 3; ++t) {
          const uint32_t acc = (s > 0 || ks > 0 || t > 0) ? 1u : 0u;
          asm volatile("{\n .reg .pred pa;\n setp.ne.b32 pa, %4, 0;\n"
                       " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, "
                       "%3, pa;\n}\n" ::"r"(taddr),
                       "l"(as[t]), "l"(bs[t]), "r"(kIdesc), "r"(acc)
                       : "memory");
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::"
                   "cluster.b64 [%0];" ::"r"(sAddr(&mbar[b]))
                   : "memory");
      committed = s + 1;
    }
  }
  // wait for the last commit (it tracks every earlier MMA of thread 0)
  __shared__ int nCommitted;
  if (tid == 0) nCommitted = committed;
  __syncthreads();
  if (nCommitted > 0) {
    const int last = nCommitted - 1;
    if (!mbarWaitT(&mbar[last & 1], (last >> 1) & 1)) ok = false;
  }
  ok = __syncthreads_and(ok) && nCommitted == nslab;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok && nslab > 0) {
    // (every thread of the CTA takes this branch together)
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (D rows), warps
    // 0-3 the first 64 columns and warps 4-7 the last 64
    const int lw = warp & 3;
    const int row = mt * kTile + lw * 32 + lane;
    const int cBeg = (warp >> 2) * (kTile / 2);
    for (int c0 = cBeg; c0 < cBeg + kTile / 2; c0 += 16) {
      uint32_t v[16];
      const uint32_t ta = taddr + ((uint32_t)(lw * 32) << 16) + c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, "
          "%6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]),
            "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]),
            "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
            "=r"(v[15])
          : "r"(ta));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < 2 * p)
        for (int j = 0; j < 16; ++j) {
          const int col = nt * kTile + c0 + j;
          if (col < 2 * q)
            part[((size_t)chunk * 2 * p + row) * (2 * q) + col] =
                __uint_as_float(v[j]);
        }
    }
  } else if (!ok && tid == 0) {
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(
                     taddr),
                 "r"(kTile)
                 : "memory");
}

// C (p x q, ld ldc) from the chunk partials of the stacked real product
__global__ void tcGramReduce(const float *__restrict__ part, int chunks,
                             int p, int q, double2 *__restrict__ C, int ldc) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= p * q) return;
  const int i = e % p, j = e / p;
  const size_t W = 2 * (size_t)q, H = 2 * (size_t)p;
  double re = 0, im = 0;
  for (int ch = 0; ch < chunks; ++ch) {
    const float *P = part + (size_t)ch * H * W;
    re += (double)P[(size_t)i * W + j] + (double)P[(size_t)(p + i) * W + q + j];
    im += (double)P[(size_t)i * W + q + j] - (double)P[(size_t)(p + i) * W + j];
  }
  C[(size_t)j * ldc + i] = make_double2(re, im);
}

} // namespace

// Rows per chunk so that the grid covers the GPU about twice.
int tcGramChunkRows(size_t N, int p, int q) {
  const int tiles = ((2 * p + kTile - 1) / kTile) * ((2 * q + kTile - 1) / kTile);
  size_t rows = (N * tiles + 303) / 304;
  rows = std::max<size_t>(256, (rows + kSlab - 1) / kSlab * kSlab);
  return (int)rows;
}

size_t tcGramPartialFloats(size_t N, int p, int q) {
  const size_t rows = tcGramChunkRows(N, p, q);
  const size_t chunks = (N + rows - 1) / rows;
  return chunks * 4 * (size_t)p * q;
}

int *tcGramErrWord() {
  static int *d = [] {
    int *x = nullptr;
    if (cudaMalloc(&x, sizeof(int)) == cudaSuccess)
      cudaMemset(x, 0, sizeof(int));
    return x;
  }();
  return d;
}

// C = A^H B on the tensor cores (see the file comment); part holds
// tcGramPartialFloats(N, p, q) floats.
void gramTC(const double2 *A, size_t lda, int p, const double2 *B, size_t ldb,
            int q, size_t N, double2 *C, int ldc, float *part,
            cudaStream_t s) {
  if (p == 0 || q == 0 || N == 0) return;
  static const bool attr = [] {
    cudaFuncSetAttribute(tcGramKernel,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kSmemBytes);
    return true;
  }();
  (void)attr;
  const int rows = tcGramChunkRows(N, p, q);
  const int chunks = (int)((N + rows - 1) / rows);
  dim3 grid((2 * p + kTile - 1) / kTile, (2 * q + kTile - 1) / kTile, chunks);
  tcGramKernel<<<grid, kThreads, kSmemBytes, s>>>(A, lda, p, B, ldb, q, N,
                                                  rows, part, tcGramErrWord());
  tcGramReduce<<<(p * q + 127) / 128, 128, 0, s>>>(part, chunks, p, q, C,
                                                   ldc);
}

} // namespace ncgm
