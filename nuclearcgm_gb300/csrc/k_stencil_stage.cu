// FP32 H.X stencil, staged-coefficient form (launch kind 2).
//
// The operator and the plane pipeline are those of stencilStream32
// (k_stencil32.cu): a persistent grid, a CTA streams its contiguous range of
// output band-planes through a ring of TMA-loaded X planes (zero fill
// outside the lattice = the reference's Dirichlet truncation), warp 0
// produces, mbarrier waits carry iteration limits. What differs:
//  * The per-point field coefficients of each output band-plane are copied
//    by TMA into a second shared-memory ring, from the split coefficient
//    table (the lo float4 of every point, then the hi float4). Warp 1 is
//    their producer. Consumers issue no global loads, so no long-latency
//    waits sit in the compute loop, and the coefficient reads cost shared
//    wavefronts instead of L1 global wavefronts.
//  * A consumer thread owns YR consecutive rows at one x of the band and
//    keeps their y-window (YR + 4 points) in registers: 8 + (YR + 4) / YR
//    shared loads per point instead of 13.
//  * One X box holds NC adjacent columns (spinors); both are computed with
//    the same coefficient registers.
//  * Launch kind 3 (ZQ) also keeps the z-neighbours of a thread's own points
//    in registers (planes k-2, k-1, k+1), so a plane is read from shared
//    memory only as the centre plane and once as plane k+2. Consumers then
//    hold three planes of the ring instead of five: with a ring of 8 the
//    producer runs five planes ahead instead of three.
// Adjacent consumer threads take adjacent x, so the 16-byte shared loads of
// a warp are contiguous runs (conflict-free).
#include "ncgm_internal.cuh"
#include "stencil32.cuh"

#include <algorithm>

namespace ncgm {

int *stencilErrWord();

namespace {

using namespace s32;

struct StageArgs {
  float4 *Y;
  int n, TY, nbands, ring, cring, ncols;
  size_t ns;
  long long total; // column groups * nbands * n output band-planes
  float shift;
  int *err;
  int xflat, cflat; // flat 4-D forms of the X and coefficient maps
};

// block-size limit per variant (register budget 102 at 640 threads, 128 at
// 512, 168 at 384: the multi-row, two-column and z-queue forms hold larger
// register windows)
constexpr int stageMaxThreads(int yr, int nc, bool zq = false) {
  return zq ? (yr >= 4 ? 384 : 512) : ((yr >= 2 || nc == 2) ? 512 : 640);
}
constexpr int kStageItems = 2; // items per consumer thread at most

template <int YR, int NC, int WFIX, bool ZQ>
__global__ void __launch_bounds__(stageMaxThreads(YR, NC, ZQ), 1)
    stencilStage32(const __grid_constant__ CUtensorMap xmap,
                   const __grid_constant__ CUtensorMap cmap, StageArgs A) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ Run runs[kMaxRuns];
  __shared__ int nruns, totalSeq, failed;
  const int n = A.n, TY = A.TY, W = WFIX ? WFIX : n + 4;
  const int boxElems = (TY + 4) * W;
  const int slotElems = (NC * boxElems + 7) & ~7; // 128-byte aligned slots
  const uint32_t boxBytes = (uint32_t)(NC * boxElems) * 16u;
  const int cHalf = TY * n;
  const int cElems = (2 * cHalf + 7) & ~7;
  const uint32_t cBytes = (uint32_t)(2 * cHalf) * 16u;
  const int nCons = blockDim.x / 32 - 2; // consumer warps
  const int rmask = A.ring - 1, rlog = __ffs(A.ring) - 1;   // ring = 2^rlog
  const int cmask = A.cring - 1, clog = __ffs(A.cring) - 1; // cring = 2^clog
  float4 *xr = reinterpret_cast<float4 *>(smem_raw);
  float4 *cr = xr + (size_t)A.ring * slotElems;
  uint64_t *full = reinterpret_cast<uint64_t *>(cr + (size_t)A.cring * cElems);
  uint64_t *empty = full + A.ring;
  uint64_t *cfull = empty + A.ring;
  uint64_t *cempty = cfull + A.cring;
  const long long t0 = (long long)blockIdx.x * A.total / gridDim.x;
  const long long t1 = (long long)(blockIdx.x + 1) * A.total / gridDim.x;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const uint32_t kLimit = 1u << 20; // x ~1 us suspend hint: bounded (~1 s)

  if (threadIdx.x == 0) {
    int r = 0, seq = 0;
    for (long long t = t0; t < t1 && r < kMaxRuns;) {
      const int cb = (int)(t / n), ka = (int)(t % n);
      const long long rem = t1 - t;
      const int kb = (rem < (long long)(n - ka)) ? ka + (int)rem : n;
      runs[r] = {cb, ka, kb, seq};
      seq += kb - ka + 4;
      t += kb - ka;
      ++r;
    }
    nruns = r;
    totalSeq = seq;
    failed = 0;
    for (int s = 0; s < A.ring; ++s) {
      mbarInit(&full[s], 1);
      mbarInit(&empty[s], nCons);
    }
    for (int s = 0; s < A.cring; ++s) {
      mbarInit(&cfull[s], 1);
      mbarInit(&cempty[s], nCons);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int NR = nruns, TS = totalSeq;

  if (warp == 0) {
    // ---- X producer: the plane sequence of every run (4 halo planes) ----
    if (lane == 0) {
      int pr = 0, pz = (NR > 0) ? runs[0].ka - 2 : 0;
      int issued = 0;
      bool ok = true;
      for (int s = 0; s < TS; ++s) {
        const int slot = s & rmask;
        if (s >= A.ring) {
          if (!mbarWaitSleep(&empty[slot], ((s >> rlog) - 1) & 1u, kLimit) ||
              *(volatile int *)&failed) {
            ok = false;
            break;
          }
        }
        const Run &R = runs[pr];
        const int cg = R.cb / A.nbands, band = R.cb % A.nbands;
        mbarExpectTx(&full[slot], boxBytes);
        tmaBand(xr + (size_t)slot * slotElems, &xmap, A.xflat, -2,
                band * TY - 2, pz, cg * NC, &full[slot]);
        issued = s + 1;
        if (++pz >= R.kb + 2 && pr + 1 < NR) {
          ++pr;
          pz = runs[pr].ka - 2;
        }
      }
      if (!ok) {
        atomicExch(A.err, 1);
        *(volatile int *)&failed = 1;
        for (int s = (issued > A.ring ? issued - A.ring : 0); s < issued; ++s)
          mbarWaitSleep(&full[s & rmask], (s >> rlog) & 1u, kLimit);
      }
    }
    return;
  }
  if (warp == 1) {
    // ---- coefficient producer: one band-plane per output plane ----
    if (lane == 0) {
      int c = 0;
      bool ok = true;
      for (int r = 0; r < NR && ok; ++r) {
        const Run R = runs[r];
        const int band = R.cb % A.nbands;
        for (int k = R.ka; k < R.kb; ++k) {
          const int slot = c & cmask;
          if (c >= A.cring) {
            if (!mbarWaitSleep(&cempty[slot], ((c >> clog) - 1) & 1u,
                               kLimit) ||
                *(volatile int *)&failed) {
              ok = false;
              break;
            }
          }
          mbarExpectTx(&cfull[slot], cBytes);
          tmaBand(cr + (size_t)slot * cElems, &cmap, A.cflat, 0, band * TY, k,
                  0, &cfull[slot]);
          ++c;
        }
      }
      if (!ok) {
        atomicExch(A.err, 1);
        *(volatile int *)&failed = 1;
        for (int s = (c > A.cring ? c - A.cring : 0); s < c; ++s)
          mbarWaitSleep(&cfull[s & cmask], (s >> clog) & 1u, kLimit);
      }
    }
    return;
  }

  // ---- consumers: item it -> (x = it % n, rows rb .. rb + YR - 1) ----
  const int ct = threadIdx.x - 64, nct = nCons * 32;
  const int nC = WFIX ? WFIX - 4 : n; // compile-time lattice size if known
  const int items = (TY / YR) * nC;
  if constexpr (ZQ) {
    // one item per thread; zm2/zm1/zp1 hold the own points of planes k-2,
    // k-1 and k+1 while the thread marches in z through a run
    static_assert(NC == 1, "the z-queue form takes one column per box");
    const bool has = ct < items;
    const int x = ct % nC, rb = (ct / nC) * YR;
    const int wo = rb * W + x + 2, co = rb * nC + x;
    float4 zm2[YR], zm1[YR], zp1[YR];
    int waited = -1, c = 0;
    const float shift = A.shift;
    for (int r = 0; r < NR; ++r) {
      const Run R = runs[r];
      const int cg = R.cb / A.nbands, band = R.cb % A.nbands;
      const int y0 = band * TY;
      const int rowsValid = min(TY, n - y0);
      float4 *Yb = A.Y + (size_t)cg * A.ns + (size_t)y0 * n;
      for (int k = R.ka; k < R.kb; ++k) {
        const int s0 = R.base + (k - R.ka);
        bool ok = true;
        while (waited < s0 + 4) {
          const int s = waited + 1;
          if (!mbarWaitBackoff(&full[s & rmask], (s >> rlog) & 1u, kLimit,
                               kPollNs)) {
            ok = false;
            break;
          }
          waited = s;
        }
        if (ok && !mbarWaitBackoff(&cfull[c & cmask], (c >> clog) & 1u,
                                   kLimit, kPollNs))
          ok = false;
        if (!ok || *(volatile int *)&failed) {
          if (lane == 0) {
            atomicExch(A.err, 1);
            *(volatile int *)&failed = 1;
          }
          return;
        }
        const float4 *pc = xr + (size_t)((s0 + 2) & rmask) * slotElems;
        const float4 *pp2 = xr + (size_t)((s0 + 4) & rmask) * slotElems;
        const float4 *cs = cr + (size_t)(c & cmask) * cElems;
        float4 *Yk = Yb + (size_t)k * nC * nC;
        if (has) {
          if (k == R.ka) {
            const float4 *pm2 = xr + (size_t)(s0 & rmask) * slotElems;
            const float4 *pm1 = xr + (size_t)((s0 + 1) & rmask) * slotElems;
            const float4 *pp1 = xr + (size_t)((s0 + 3) & rmask) * slotElems;
#pragma unroll
            for (int t = 0; t < YR; ++t) {
              const int l = wo + (t + 2) * W;
              zm2[t] = pm2[l];
              zm1[t] = pm1[l];
              zp1[t] = pp1[l];
            }
          }
          float4 win[YR + 4];
#pragma unroll
          for (int q = 0; q < YR + 4; ++q) win[q] = pc[wo + q * W];
#pragma unroll
          for (int t = 0; t < YR; ++t) {
            const int ci = co + t * nC;
            const float4 ca = cs[ci], cb = cs[cHalf + ci];
            const int l = wo + (t + 2) * W;
            const float4 zp2 = pp2[l];
            const float4 o = pointH2(ca, cb, shift, win[t + 2], pc[l + 1],
                                     pc[l - 1], pc[l + 2], pc[l - 2],
                                     win[t + 3], win[t + 1], win[t + 4],
                                     win[t], zp1[t], zm1[t], zp2, zm2[t]);
            if (rb + t < rowsValid) Yk[ci] = o;
            zm2[t] = zm1[t];
            zm1[t] = win[t + 2];
            zp1[t] = zp2;
          }
        }
        // release: the centre plane; at the start of a run also the two
        // planes below it, at the end also the two above
        __syncwarp();
        if (lane == 0) {
          const int first = (k == R.ka) ? s0 : s0 + 2;
          const int last = (k + 1 < R.kb) ? s0 + 2 : s0 + 4;
          for (int s = first; s <= last; ++s) mbarArrive(&empty[s & rmask]);
          mbarArrive(&cempty[c & cmask]);
        }
        ++c;
      }
    }
    return;
  }
  // A thread owns items ct and ct + nct (launch shapes give at most two);
  // their slot and table offsets are fixed for the whole kernel.
  int woff[kStageItems], coff[kStageItems], row0[kStageItems];
#pragma unroll
  for (int m = 0; m < kStageItems; ++m) {
    const int it = ct + m * nct;
    const int x = it % nC, rb = (it / nC) * YR;
    row0[m] = it < items ? rb : 0x7fffffff; // past every band: no item
    woff[m] = rb * W + x + 2;  // window start (row rb - 2 of the band)
    coff[m] = rb * nC + x;     // coefficient / output offset of row rb
  }
  int waited = -1, c = 0;
  const float shift = A.shift;
  const size_t ns = A.ns;
  for (int r = 0; r < NR; ++r) {
    const Run R = runs[r];
    const int cg = R.cb / A.nbands, band = R.cb % A.nbands;
    const int y0 = band * TY;
    const int rowsValid = min(TY, n - y0);
    const int col0 = cg * NC;
    const int ncv = min(NC, A.ncols - col0);
    float4 *Yb = A.Y + (size_t)col0 * A.ns + (size_t)y0 * n;
    for (int k = R.ka; k < R.kb; ++k) {
      const int s0 = R.base + (k - R.ka);
      bool ok = true;
      while (waited < s0 + 4) {
        const int s = waited + 1;
        if (!mbarWaitBackoff(&full[s & rmask], (s >> rlog) & 1u, kLimit,
                             kPollNs)) {
          ok = false;
          break;
        }
        waited = s;
      }
      if (ok && !mbarWaitBackoff(&cfull[c & cmask], (c >> clog) & 1u, kLimit,
                                 kPollNs))
        ok = false;
      if (!ok || *(volatile int *)&failed) {
        if (lane == 0) {
          atomicExch(A.err, 1);
          *(volatile int *)&failed = 1;
        }
        return;
      }
      const float4 *pm2 = xr + (size_t)(s0 & rmask) * slotElems;
      const float4 *pm1 = xr + (size_t)((s0 + 1) & rmask) * slotElems;
      const float4 *pc = xr + (size_t)((s0 + 2) & rmask) * slotElems;
      const float4 *pp1 = xr + (size_t)((s0 + 3) & rmask) * slotElems;
      const float4 *pp2 = xr + (size_t)((s0 + 4) & rmask) * slotElems;
      const float4 *cs = cr + (size_t)(c & cmask) * cElems;
      float4 *Yk = Yb + (size_t)k * nC * nC;
#pragma unroll
      for (int m = 0; m < kStageItems; ++m) {
        if (row0[m] >= TY) break;
        float4 win[NC][YR + 4];
#pragma unroll
        for (int j = 0; j < NC; ++j)
          if (j < ncv) {
#pragma unroll
            for (int q = 0; q < YR + 4; ++q)
              win[j][q] = pc[j * boxElems + woff[m] + q * W];
          }
#pragma unroll
        for (int t = 0; t < YR; ++t) {
          const int ci = coff[m] + t * nC;
          const float4 ca = cs[ci], cb = cs[cHalf + ci];
#pragma unroll
          for (int j = 0; j < NC; ++j)
            if (j < ncv) {
              const int l = j * boxElems + woff[m] + (t + 2) * W;
              const float4 o = pointH2(
                  ca, cb, shift, win[j][t + 2], pc[l + 1], pc[l - 1],
                  pc[l + 2], pc[l - 2], win[j][t + 3], win[j][t + 1],
                  win[j][t + 4], win[j][t], pp1[l], pm1[l], pp2[l], pm2[l]);
              if (row0[m] + t < rowsValid) Yk[(size_t)j * ns + ci] = o;
            }
        }
      }
      // release the X planes this warp no longer needs (seq s0, or all five
      // at the end of the run) and the coefficient slot
      __syncwarp();
      if (lane == 0) {
        const int last = (k + 1 < R.kb) ? s0 : s0 + 4;
        for (int s = s0; s <= last; ++s) mbarArrive(&empty[s & rmask]);
        mbarArrive(&cempty[c & cmask]);
      }
      ++c;
    }
  }
}

using StageKernel = void (*)(const CUtensorMap, const CUtensorMap, StageArgs);
constexpr int kStageWidths[] = {0, 34, 36, 40, 44, 52};
template <int YR, int NC, bool ZQ> StageKernel pickStageW(int W) {
  switch (W) {
  case 34: return stencilStage32<YR, NC, 34, ZQ>;
  case 36: return stencilStage32<YR, NC, 36, ZQ>;
  case 40: return stencilStage32<YR, NC, 40, ZQ>;
  case 44: return stencilStage32<YR, NC, 44, ZQ>;
  case 52: return stencilStage32<YR, NC, 52, ZQ>;
  default: return stencilStage32<YR, NC, 0, ZQ>;
  }
}
StageKernel pickStage(int yr, int nc, int W, bool zq) {
  if (zq) {
    if (yr == 1) return pickStageW<1, 1, true>(W);
    if (yr == 2) return pickStageW<2, 1, true>(W);
    return pickStageW<4, 1, true>(W);
  }
  if (nc == 2) // 4 rows x 2 columns does not fit the register budget
    return yr == 1 ? pickStageW<1, 2, false>(W) : pickStageW<2, 2, false>(W);
  if (yr == 1) return pickStageW<1, 1, false>(W);
  if (yr == 2) return pickStageW<2, 1, false>(W);
  return pickStageW<4, 1, false>(W);
}

size_t stageSmem(int n, int TY, int ring, int cring, int nc) {
  const size_t slot = (((size_t)nc * (TY + 4) * (n + 4) + 7) & ~size_t(7)) * 16;
  const size_t cslot = (((size_t)2 * TY * n + 7) & ~size_t(7)) * 16;
  return (size_t)ring * slot + (size_t)cring * cslot +
         (size_t)(2 * ring + 2 * cring) * 8;
}

} // namespace

bool validStage(int n, int TY, int ring, int cring, int yr, int nc, int cps,
                bool zq, int &threads) {
  if (!(yr == 1 || yr == 2 || yr == 4) || !(nc == 1 || nc == 2)) return false;
  if (yr == 4 && nc == 2) return false;
  if (zq && nc != 1) return false;
  if (TY < yr || TY > n || TY % yr || cps < 1) return false;
  if (ring < 8 || ring > 64 || (ring & (ring - 1))) return false;
  if (cring < 2 || cring > 16 || (cring & (cring - 1))) return false;
  if (TY + 4 > 256 || n + 4 > 256) return false;
  const int items = (TY / yr) * n;
  const int maxWarps = (stageMaxThreads(yr, nc, zq) - 64) / 32;
  threads = 64 + std::min((items + 31) / 32, maxWarps) * 32;
  if (items > (zq ? 1 : kStageItems) * (threads - 64)) return false;
  return stageSmem(n, TY, ring, cring, nc) * cps <= 220 * 1024;
}

bool launchStage(ncgm_ctx *ctx, int species, const float2 *X, float2 *Y,
                 int ncols, float shift, cudaStream_t st, int TY, int ring,
                 int cring, int yr, int nc, int cps, bool zq) {
  static const bool attr = [] {
    for (int w : kStageWidths)
      for (int y : {1, 2, 4}) {
        for (int c : {1, 2})
          if (!(y == 4 && c == 2))
            cudaFuncSetAttribute(pickStage(y, c, w, false),
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 220 * 1024);
        cudaFuncSetAttribute(pickStage(y, 1, w, true),
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             220 * 1024);
      }
    return true;
  }();
  (void)attr;
  const int n = ctx->n;
  if (nc > ncols) nc = 1; // a single column: no box wider than the block
  int threads = 0;
  if (!validStage(n, TY, ring, cring, yr, nc, cps, zq, threads)) return false;
  const float *cs = ctx->sp[species].coef32s;
  if (!cs) return false;
  CUtensorMap xmap, cmap;
  bool xflat = false, cflat = false;
  if (!tensorMapX(X, n, ncols, n + 4, TY + 4, nc, xflat, &xmap)) return false;
  if (!tensorMapX(cs, n, 2, n, TY, 2, cflat, &cmap)) return false;
  StageArgs A;
  A.Y = reinterpret_cast<float4 *>(Y);
  A.n = n;
  A.TY = TY;
  A.nbands = (n + TY - 1) / TY;
  A.ring = ring;
  A.cring = cring;
  A.ncols = ncols;
  A.ns = ctx->ns;
  A.total = (long long)((ncols + nc - 1) / nc) * A.nbands * n;
  A.shift = shift;
  A.err = stencilErrWord();
  A.xflat = xflat;
  A.cflat = cflat;
  // enough CTAs that no CTA holds more than kMaxRuns runs
  long long ctas = (long long)smCount() * cps;
  const long long minCtas = (A.total + (long long)(kMaxRuns - 2) * n - 1) /
                            ((long long)(kMaxRuns - 2) * n);
  ctas = std::max(ctas, minCtas);
  ctas = std::min<long long>(ctas, A.total);
  pickStage(yr, nc, n + 4, zq)<<<(unsigned)ctas, threads,
                             stageSmem(n, TY, ring, cring, nc), st>>>(xmap,
                                                                      cmap, A);
  return true;
}

} // namespace ncgm
