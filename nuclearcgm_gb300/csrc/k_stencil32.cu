// FP32 H.X stencil: persistent streaming kernel on TMA tensor tiles.
//
// Same operator as stencilPoint in k_hamiltonian.cu (the matrix-free form of
// Hamiltonian::buildMatrix, src/hamiltonian/hamiltonian.cpp:303-372), built
// for HBM bandwidth on GB300:
//  * A 5-D tensor map views X as [col][k][j][i][4 floats]. One TMA box is a
//    padded (TY+4) x (n+4) band of one z plane starting at i = -2,
//    j = y0 - 2; out-of-range coordinates (also z < 0, z >= n) are zero-filled
//    by the TMA unit, which is the reference's Dirichlet truncation, so the
//    arithmetic has no bounds checks.
//  * The grid is a fixed number of CTAs per SM. The (column, band, z) output
//    planes are flattened and split into equal contiguous ranges, one per
//    CTA; a CTA streams its range through a shared-memory ring with one TMA
//    pipeline that runs across column/band boundaries (4 extra halo planes
//    at each boundary), so loads stay `ring - 5` planes ahead of the compute.
//  * Every thread owns fixed in-band points; the per-point field coefficients
//    (L2 resident, shared by all columns) are loaded before the plane wait.
//  * mbarrier waits are bounded: on timeout the CTA records an error flag,
//    drains its own copies (bounded) and returns.
#include "ncgm_internal.cuh"
#include "stencil32.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdio>
#include <mutex>
#include <string>
#include <cstdlib>
#include <vector>

namespace ncgm {

int *stencilErrWord();

namespace {

using namespace s32;

// Warp-specialised form. Warp 0 is the producer: one lane issues the TMA
// loads of the CTA's plane sequence, waiting on the slot's `empty` barrier
// before reusing it. Warps 1..C are consumers: each waits on the `full`
// barrier of the planes it needs, computes its points and releases the
// planes it no longer needs with one arrive per warp. No CTA-wide barrier
// in the loop. PPT: points per consumer thread; WFIX: padded row width
// n + 4 fixed at compile time (0: runtime), making +-W offsets immediates.
// block-size limit per variant: the 1- and 2-point forms fit in 102
// registers, so up to 640 threads (20 warps) per SM; the 4-point form 512
constexpr int streamMaxThreads(int ppt) { return ppt == 4 ? 512 : 640; }

template <int PPT, int WFIX>
__global__ void __launch_bounds__(streamMaxThreads(PPT), 1)
    stencilStream32(const __grid_constant__ CUtensorMap map, StreamArgs A) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ Run runs[kMaxRuns];
  __shared__ int nruns, totalSeq, failed;
  const int n = A.n, W = WFIX ? WFIX : n + 4;
  const int boxElems = (A.TY + 4) * W;
  const int slotElems = (boxElems + 7) & ~7; // 128-byte aligned slots
  const uint32_t boxBytes = boxElems * 16u;
  const int nCons = blockDim.x / 32 - 1;      // consumer warps
  const int rmask = A.ring - 1, rlog = __ffs(A.ring) - 1; // ring = 2^rlog
  float4 *ring = reinterpret_cast<float4 *>(smem_raw);
  uint64_t *full = reinterpret_cast<uint64_t *>(
      smem_raw + (size_t)A.ring * slotElems * 16u);
  uint64_t *empty = full + A.ring;
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
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int NR = nruns, TS = totalSeq;

  if (warp == 0) {
    // ---- producer ----
    if (lane == 0) {
      int pr = 0, pz = (NR > 0) ? runs[0].ka - 2 : 0;
      int issued = 0;
      bool ok = true;
      for (int s = 0; s < TS; ++s) {
        const int slot = s & rmask;
        if (s >= A.ring) {
          // slot reuse: every consumer warp released seq s - ring
          if (!mbarWaitSleep(&empty[slot], ((s >> rlog) - 1) & 1u, kLimit) ||
              *(volatile int *)&failed) {
            ok = false;
            break;
          }
        }
        const Run &R = runs[pr];
        const int col = R.cb / A.nbands, band = R.cb % A.nbands;
        mbarExpectTx(&full[slot], boxBytes);
        tmaBand(ring + (size_t)slot * slotElems, &map, A.flat, -2,
                band * A.TY - 2,
                 pz, col, &full[slot]);
        issued = s + 1;
        if (++pz >= R.kb + 2 && pr + 1 < NR) {
          ++pr;
          pz = runs[pr].ka - 2;
        }
      }
      if (!ok) {
        atomicExch(A.err, 1);
        *(volatile int *)&failed = 1;
        // drain: wait (bounded) for every copy this CTA issued
        for (int s = (issued > A.ring ? issued - A.ring : 0); s < issued; ++s)
          mbarWaitSleep(&full[s & rmask], (s >> rlog) & 1u, kLimit);
      }
    }
    return;
  }

  // ---- consumers ----
  const int ct = threadIdx.x - 32; // consumer thread index
  const int nct = nCons * 32;
  int qv[PPT], lr[PPT];
#pragma unroll
  for (int t = 0; t < PPT; ++t) {
    int q = ct + t * nct;
    if (q >= A.TY * n) q = 0x7fffffff;
    qv[t] = q;
    lr[t] = (q == 0x7fffffff) ? 0 : ((q / n) + 2) * W + (q % n) + 2;
  }
  // with A.cpa: per-thread coefficient staging (two planes x PPT points x
  // 2 float4) after the ring; the next plane's coefficients are copied with
  // cp.async while the current plane is computed
  float4 *stage = reinterpret_cast<float4 *>(
      smem_raw + (size_t)A.ring * slotElems * 16u + (size_t)A.ring * 16u);
  auto stg = [&](int buf, int t, int h) {
    return stage + ((buf * PPT + t) * 2 + h) * nct + ct;
  };
  auto prefetch = [&](unsigned pb, int tyn, int buf) {
#pragma unroll
    for (int t = 0; t < PPT; ++t)
      if (qv[t] < tyn) {
        const float4 *c2 = A.coef + 2 * (size_t)(pb + qv[t]);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                         smemAddr(stg(buf, t, 0))),
                     "l"(c2)
                     : "memory");
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                         smemAddr(stg(buf, t, 1))),
                     "l"(c2 + 1)
                     : "memory");
      }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  int waited = -1, sc = 0;
  for (int r = 0; r < NR; ++r) {
    const Run R = runs[r];
    const int col = R.cb / A.nbands, band = R.cb % A.nbands;
    const int y0 = band * A.TY;
    const int tyn = min(A.TY, n - y0) * n;
    float4 *Yc = A.Y + (size_t)col * A.ns;
    if (A.cpa)
      prefetch((unsigned)R.ka * (unsigned)(n * n) + (unsigned)(y0 * n), tyn,
               sc & 1);
    for (int k = R.ka; k < R.kb; ++k) {
      const int s0 = R.base + (k - R.ka);
      const unsigned pbase = (unsigned)k * (unsigned)(n * n) + (unsigned)(y0 * n);
      float4 ca[PPT], cbv[PPT];
      if (A.cpa) {
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        const int cur = sc & 1;
#pragma unroll
        for (int t = 0; t < PPT; ++t)
          if (qv[t] < tyn) {
            ca[t] = *stg(cur, t, 0);
            cbv[t] = *stg(cur, t, 1);
          }
        if (k + 1 < R.kb) prefetch(pbase + (unsigned)(n * n), tyn, cur ^ 1);
        ++sc;
      } else {
#pragma unroll
        for (int t = 0; t < PPT; ++t)
          if (qv[t] < tyn) {
            const float4 *c2 = A.coef + 2 * (size_t)(pbase + qv[t]);
            ca[t] = __ldg(c2);
            cbv[t] = __ldg(c2 + 1);
          }
      }
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
      if (!ok || *(volatile int *)&failed) {
        if (lane == 0) {
          atomicExch(A.err, 1);
          *(volatile int *)&failed = 1;
        }
        return;
      }
      const float4 *pm2 = ring + ((s0) & rmask) * slotElems;
      const float4 *pm1 = ring + ((s0 + 1) & rmask) * slotElems;
      const float4 *pc = ring + ((s0 + 2) & rmask) * slotElems;
      const float4 *pp1 = ring + ((s0 + 3) & rmask) * slotElems;
      const float4 *pp2 = ring + ((s0 + 4) & rmask) * slotElems;
#pragma unroll
      for (int t = 0; t < PPT; ++t)
        if (qv[t] < tyn) {
          const int l = lr[t];
          Yc[pbase + qv[t]] = pointH2(
              ca[t], cbv[t], A.shift, pc[l], pc[l + 1], pc[l - 1], pc[l + 2],
              pc[l - 2], pc[l + W], pc[l - W], pc[l + 2 * W], pc[l - 2 * W],
              pp1[l], pm1[l], pp2[l], pm2[l]);
        }
      // release the planes this warp no longer needs: seq s0, or all five at
      // the end of the run
      __syncwarp();
      if (lane == 0) {
        const int last = (k + 1 < R.kb) ? s0 : s0 + 4;
        for (int s = s0; s <= last; ++s) mbarArrive(&empty[s & rmask]);
      }
    }
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// z-marching form. Same producer and plane sequence as stencilStream32, but
// every consumer thread owns one point of the band and keeps its z-column
// (z-2 .. z+2) in registers while it walks the planes of a run: per step it
// reads the new plane z+2 at its point and the x/y neighbours in the centre
// plane (9 shared loads per point instead of 13), and releases the centre
// plane as soon as the step is done. The
// per-point field coefficients of the next plane are copied one step ahead
// into a per-thread shared staging buffer (cp.async), so no global-load
// latency sits on the step's critical path.
// Release rule per warp and run (seq base <-> plane ka-2): base and base+1
// after the window load, base+2+m after step ka+m, base+len+2 and base+len+3
// after the last step.
constexpr int kMarchThreads = 512;
template <int WFIX>
__global__ void __launch_bounds__(kMarchThreads, 1)
    stencilMarch32(const __grid_constant__ CUtensorMap map, StreamArgs A) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ Run runs[kMaxRuns];
  __shared__ int nruns, totalSeq, failed;
  const int n = A.n, W = WFIX ? WFIX : n + 4;
  const int boxElems = (A.TY + 4) * W;
  const int slotElems = (boxElems + 7) & ~7;
  const uint32_t boxBytes = boxElems * 16u;
  const int nCons = blockDim.x / 32 - 1;
  const int rmask = A.ring - 1, rlog = __ffs(A.ring) - 1;
  float4 *ring = reinterpret_cast<float4 *>(smem_raw);
  uint64_t *full = reinterpret_cast<uint64_t *>(
      smem_raw + (size_t)A.ring * slotElems * 16u);
  uint64_t *empty = full + A.ring;
  const long long t0 = (long long)blockIdx.x * A.total / gridDim.x;
  const long long t1 = (long long)(blockIdx.x + 1) * A.total / gridDim.x;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const uint32_t kLimit = 1u << 20;

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
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int NR = nruns, TS = totalSeq;

  if (warp == 0) {
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
        const int col = R.cb / A.nbands, band = R.cb % A.nbands;
        mbarExpectTx(&full[slot], boxBytes);
        tmaBand(ring + (size_t)slot * slotElems, &map, A.flat, -2,
                band * A.TY - 2,
                 pz, col, &full[slot]);
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

  // ---- consumers: thread ct owns point (i, j) of the band ----
  // (adjacent threads take adjacent i: conflict-free 16-byte shared loads)
  const int ct = threadIdx.x - 32, nct = blockDim.x - 32;
  const bool own = ct < A.TY * n;
  const int ii = own ? ct % n : 0, jj = own ? ct / n : 0;
  const int l = (jj + 2) * W + ii + 2;
  // per-thread coefficient staging, two buffers x 2 float4 (cp.async)
  float4 *stage = reinterpret_cast<float4 *>(
      smem_raw + (size_t)A.ring * slotElems * 16u + (size_t)A.ring * 16u);
  const uint32_t stage0 = smemAddr(stage + ct), dstep = nct * 16u;
  auto prefetch = [&](bool act, unsigned pidx, int buf) {
    if (act) {
      const float4 *c0 = A.coef + 2 * (size_t)pidx;
      const uint32_t d0 = stage0 + buf * 2 * dstep;
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d0),
                   "l"(c0)
                   : "memory");
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                       d0 + dstep),
                   "l"(c0 + 1)
                   : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  int waited = -1, sc = 0; // sc: running step count (staging buffer parity)
  bool ok = true;
  auto waitTo = [&](int upto) {
    while (waited < upto) {
      const int s = waited + 1;
      if (!mbarWaitBackoff(&full[s & rmask], (s >> rlog) & 1u, kLimit,
                           kPollNs))
        return false;
      waited = s;
    }
    return !*(volatile int *)&failed;
  };
  auto slotp = [&](int s) {
    return (const float4 *)(ring + (size_t)(s & rmask) * slotElems);
  };
  auto release = [&](int s) {
    __syncwarp();
    if (lane == 0) mbarArrive(&empty[s & rmask]);
  };
  for (int r = 0; r < NR && ok; ++r) {
    const Run R = runs[r];
    const int col = R.cb / A.nbands, band = R.cb % A.nbands;
    const int y0 = band * A.TY;
    const bool act = own && (y0 + jj) < n;
    float4 *Yc = A.Y + (size_t)col * A.ns;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const unsigned rowOff = (unsigned)((y0 + jj) * n + ii);
    const unsigned nn = (unsigned)(n * n);
    prefetch(act, (unsigned)R.ka * nn + rowOff, sc & 1);
    float4 a[5]; // z-window of the point, rotating by 5
    if (!waitTo(R.base + 3)) {
      ok = false;
      break;
    }
#pragma unroll
    for (int d = 0; d < 4; ++d) a[d] = act ? slotp(R.base + d)[l] : z4;
    a[4] = z4;
    release(R.base);
    if (lane == 0) mbarArrive(&empty[(R.base + 1) & rmask]);
    int k = R.ka;
#define NCGM_MARCH_STEP(P)                                                     \
  {                                                                            \
    const int s0 = R.base + (k - R.ka);                                        \
    const unsigned pidx = (unsigned)k * nn + rowOff;                           \
    asm volatile("cp.async.wait_group 0;" ::: "memory");                       \
    const int cur = sc & 1;                                                    \
    float4 ca, cb;                                                             \
    if (act) {                                                                 \
      ca = stage[(cur * 2) * nct + ct];                                        \
      cb = stage[(cur * 2 + 1) * nct + ct];                                    \
    }                                                                          \
    if (k + 1 < R.kb) prefetch(act, pidx + nn, cur ^ 1);                       \
    ++sc;                                                                      \
    if (!waitTo(s0 + 4)) {                                                     \
      ok = false;                                                              \
      break;                                                                   \
    }                                                                          \
    if (act) {                                                                 \
      const float4 *pc = slotp(s0 + 2);                                        \
      a[(P + 4) % 5] = slotp(s0 + 4)[l];                                       \
      Yc[pidx] = pointH2(ca, cb, A.shift, a[(P + 2) % 5], pc[l + 1],           \
                         pc[l - 1], pc[l + 2], pc[l - 2], pc[l + W],           \
                         pc[l - W], pc[l + 2 * W], pc[l - 2 * W],              \
                         a[(P + 3) % 5], a[(P + 1) % 5], a[(P + 4) % 5],       \
                         a[P % 5]);                                            \
    }                                                                          \
    release(s0 + 2);                                                           \
    if (k + 1 == R.kb && lane == 0) {                                          \
      mbarArrive(&empty[(s0 + 3) & rmask]);                                    \
      mbarArrive(&empty[(s0 + 4) & rmask]);                                    \
    }                                                                          \
    if (++k >= R.kb) break;                                                    \
  }
    while (true) {
      NCGM_MARCH_STEP(0)
      NCGM_MARCH_STEP(1)
      NCGM_MARCH_STEP(2)
      NCGM_MARCH_STEP(3)
      NCGM_MARCH_STEP(4)
    }
#undef NCGM_MARCH_STEP
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  if (!ok && lane == 0) {
    atomicExch(A.err, 1);
    *(volatile int *)&failed = 1;
  }
}

using StreamKernel = void (*)(const CUtensorMap, StreamArgs);
constexpr int kWidths[] = {0, 34, 36, 40, 44, 52};
template <int PPT> StreamKernel pickW(int W) {
  switch (W) {
  case 34: return stencilStream32<PPT, 34>;
  case 36: return stencilStream32<PPT, 36>;
  case 40: return stencilStream32<PPT, 40>;
  case 44: return stencilStream32<PPT, 44>;
  case 52: return stencilStream32<PPT, 52>;
  default: return stencilStream32<PPT, 0>;
  }
}
StreamKernel pickMarch(int W) {
  switch (W) {
  case 34: return stencilMarch32<34>;
  case 36: return stencilMarch32<36>;
  case 40: return stencilMarch32<40>;
  case 44: return stencilMarch32<44>;
  case 52: return stencilMarch32<52>;
  default: return stencilMarch32<0>;
  }
}
// kind 0: stencilStream32 with `ppt` points per thread; kind 1: z-marching
StreamKernel pickKernel(int kind, int ppt, int W) {
  static const bool attr = [] {
    for (int w : kWidths) {
      cudaFuncSetAttribute(pickW<1>(w), cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
      cudaFuncSetAttribute(pickW<2>(w), cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
      cudaFuncSetAttribute(pickW<4>(w), cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
      cudaFuncSetAttribute(pickMarch(w), cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    }
    return true;
  }();
  (void)attr;
  if (kind == 1) return pickMarch(W);
  if (ppt == 1) return pickW<1>(W);
  if (ppt == 2) return pickW<2>(W);
  return pickW<4>(W);
}

PFN_cuTensorMapEncodeTiled_v12000 encodeFn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    PFN_cuTensorMapEncodeTiled_v12000 f = nullptr;
    cudaDriverEntryPointQueryResult q;
    void *p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                         cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      f = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    return f;
  }();
  return fn;
}

struct MapEntry {
  const void *ptr;
  int n, d4, boxW, boxRows, boxD4;
  bool flat;
  CUtensorMap map;
};
std::vector<MapEntry> g_maps;
std::mutex g_mapsMutex; // contexts may run on several host threads

} // namespace

bool tensorMapX(const void *base, int n, int d4, int boxW, int boxRows,
                int boxD4, bool &flat, CUtensorMap *out) {
  std::lock_guard<std::mutex> lock(g_mapsMutex);
  for (auto &e : g_maps)
    if (e.ptr == base && e.n == n && e.d4 == d4 && e.boxW == boxW &&
        e.boxRows == boxRows && e.boxD4 == boxD4) {
      flat = e.flat;
      *out = e.map;
      return true;
    }
  auto fn = encodeFn();
  if (!fn) return false;
  const bool fl = 4 * boxW <= 256;
  const cuuint64_t nn = (cuuint64_t)n;
  cuuint64_t dims5[5] = {4, nn, nn, nn, (cuuint64_t)d4};
  cuuint64_t dims4[4] = {4 * nn, nn, nn, (cuuint64_t)d4};
  cuuint64_t str5[4] = {16, 16 * nn, 16 * nn * nn, 16 * nn * nn * nn};
  cuuint64_t str4[3] = {16 * nn, 16 * nn * nn, 16 * nn * nn * nn};
  cuuint32_t box5[5] = {4, (cuuint32_t)boxW, (cuuint32_t)boxRows, 1,
                        (cuuint32_t)boxD4};
  cuuint32_t box4[4] = {(cuuint32_t)(4 * boxW), (cuuint32_t)boxRows, 1,
                        (cuuint32_t)boxD4};
  cuuint32_t es[5] = {1, 1, 1, 1, 1};
  CUtensorMap m;
  CUresult r = fn(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, fl ? 4 : 5,
                  const_cast<void *>(base), fl ? dims4 : dims5,
                  fl ? str4 : str5, fl ? box4 : box5, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return false;
  if (g_maps.size() > 64) g_maps.erase(g_maps.begin());
  g_maps.push_back({base, n, d4, boxW, boxRows, boxD4, fl, m});
  flat = fl;
  *out = m;
  return true;
}

int smCount() {
  static const int c = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  return c;
}

namespace {

// map of X with one (n+4) x (TY+4) band box of one column
bool tensorMapFor(const void *X, int n, int ncols, int TY, bool &flat,
                  CUtensorMap *out) {
  return tensorMapX(X, n, ncols, n + 4, TY + 4, 1, flat, out);
}

size_t streamSmem(int n, int TY, int ring) {
  size_t slot = (((size_t)(TY + 4) * (n + 4) + 7) & ~size_t(7)) * 16;
  return (size_t)ring * slot + (size_t)ring * 16; // slots + full/empty bars
}
// coefficient staging per consumer thread: the z-marching kernel 2 x 2
// float4, the streaming kernel with prefetch 2 x ppt x 2 float4
size_t kernelSmem(int kind, int n, int TY, int ring, int threads, int ppt,
                  int cpa) {
  size_t st = 0;
  if (kind == 1) st = (size_t)64 * (threads - 32);
  else if (cpa) st = (size_t)64 * ppt * (threads - 32);
  return streamSmem(n, TY, ring) + st;
}

struct Shape {
  int TY, ring, ppt, ctasPerSM;
  int kind; // 0: stencilStream32, 1: stencilMarch32 (ppt unused),
            // 2: stencilStage32 (ppt = rows per thread),
            // 3: stencilStage32 with the z-neighbours in registers
  int cpa;  // kind 0: coefficients prefetched with cp.async;
            // kinds 2, 3: coefficient ring depth
  int nc;   // kind 2: columns per X box (kind 3: 1)
};

bool validShape(int n, const Shape &s, int &threads) {
  if (s.kind == 2 || s.kind == 3)
    return validStage(n, s.TY, s.ring, s.cpa, s.ppt, s.nc, s.ctasPerSM,
                      s.kind == 3, threads);
  if (s.TY < 1 || s.TY > n || s.ring < 4 || (s.ring & (s.ring - 1)) ||
      s.ring > 64 || s.ctasPerSM < 1)
    return false;
  if (s.TY + 4 > 256 || n + 4 > 256) return false;
  if (s.kind == 1) {
    // one point per consumer thread
    threads = 32 + ((s.TY * n) + 31) / 32 * 32;
    if (threads > kMarchThreads) return false;
  } else {
    if (s.kind != 0 || s.ring < 8 || !(s.ppt == 1 || s.ppt == 2 || s.ppt == 4))
      return false;
    const int pts = s.TY * n;
    // one producer warp + consumer warps covering the band
    threads = 32 + ((pts + s.ppt - 1) / s.ppt + 31) / 32 * 32;
    if (threads > streamMaxThreads(s.ppt)) return false;
  }
  if (threads < 64) return false;
  if (kernelSmem(s.kind, n, s.TY, s.ring, threads, s.ppt, s.cpa) *
          s.ctasPerSM >
      220 * 1024)
    return false;
  return true;
}

bool launchStream(ncgm_ctx *ctx, int species, const float2 *X, float2 *Y,
                  int ncols, float shift, cudaStream_t st, const Shape &sh) {
  const int n = ctx->n;
  int threads = 0;
  if (!validShape(n, sh, threads)) return false;
  if (sh.kind == 2 || sh.kind == 3)
    return launchStage(ctx, species, X, Y, ncols, shift, st, sh.TY, sh.ring,
                       sh.cpa, sh.ppt, sh.nc, sh.ctasPerSM, sh.kind == 3);
  CUtensorMap map;
  bool flat = false;
  if (!tensorMapFor(X, n, ncols, sh.TY, flat, &map)) return false;
  StreamArgs A;
  A.Y = reinterpret_cast<float4 *>(Y);
  A.coef = reinterpret_cast<const float4 *>(ctx->sp[species].coef32);
  A.n = n;
  A.TY = sh.TY;
  A.nbands = (n + sh.TY - 1) / sh.TY;
  A.ring = sh.ring;
  A.ppt = sh.ppt;
  A.ns = ctx->ns;
  A.total = (long long)ncols * A.nbands * n;
  A.shift = shift;
  A.err = stencilErrWord();
  A.cpa = sh.kind == 0 ? sh.cpa : 0;
  A.flat = flat ? 1 : 0;
  // enough CTAs that no CTA holds more than kMaxRuns runs
  long long ctas = (long long)smCount() * sh.ctasPerSM;
  const long long minCtas = (A.total + (long long)(kMaxRuns - 2) * n - 1) /
                            ((long long)(kMaxRuns - 2) * n);
  ctas = std::max(ctas, minCtas);
  ctas = std::min<long long>(ctas, A.total);
  StreamKernel kern = pickKernel(sh.kind, sh.ppt, n + 4);
  kern<<<(unsigned)ctas, threads,
         kernelSmem(sh.kind, n, sh.TY, sh.ring, threads, sh.ppt, sh.cpa),
         st>>>(map, A);
  return true;
}

// Tuned launch shapes, one per lattice size (and shape override string):
// contexts on the same lattice share the first context's measurement.
struct TunedShape {
  int n;
  std::string env;
  Shape s;
};
std::vector<TunedShape> g_tuned;
std::mutex g_tunedMutex;

Shape defaultShape(int n) {
  Shape s{n, 8, 4, 1, 0, 0, 1};  // ring: a power of two
  int th;
  while (!validShape(n, s, th) && s.TY > 1) {
    if (s.TY * n > 512 * s.ppt && s.ppt < kPPT) {
      s.ppt *= 2;
      continue;
    }
    s.TY = (s.TY + 1) / 2;
  }
  return s;
}

} // namespace

// Project autotuner for the FP32 stencil: times candidate (band rows, ring
// depth, points per thread, CTAs per SM) on the context's own lattice with
// CUDA events and keeps the fastest. Runs once per context.
static Shape tune(ncgm_ctx *ctx, int species, int ncols) {
  const int n = ctx->n;
  ncols = std::max(1, std::min(ncols, ctx->max_cols));
  size_t bytes = ctx->N * ncols * sizeof(float2);
  float2 *X = static_cast<float2 *>(ctx->buf(1, bytes));
  float2 *Y = static_cast<float2 *>(ctx->buf(2, bytes));
  Shape best = defaultShape(n);
  if (!X || !Y) return best;
  cudaMemsetAsync(X, 0, bytes, ctx->stream);
  std::vector<int> rows;
  for (int r = n;; r = (r + 1) / 2) {
    rows.push_back(r);
    if (r <= 4) break;
  }
  float bestMs = 1e30f;
  // NCGM_TUNE_LOG=1 prints every candidate's time to stderr
  const char *lg = std::getenv("NCGM_TUNE_LOG");
  const bool log = lg && lg[0] == '1';
  auto trial = [&](const Shape &s) {
    int th;
    if (!validShape(n, s, th)) return;
    if (!launchStream(ctx, species, X, Y, ncols, 0.f, ctx->stream, s)) return;
    cudaEventRecord(ctx->ev0, ctx->stream);
    for (int r = 0; r < 3; ++r)
      launchStream(ctx, species, X, Y, ncols, 0.f, ctx->stream, s);
    cudaEventRecord(ctx->ev1, ctx->stream);
    if (cudaEventSynchronize(ctx->ev1) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    if (log)
      std::fprintf(stderr,
                   "[ncgm tune] n=%d cols=%d kind=%d rows=%d ring=%d ppt=%d "
                   "ctas/SM=%d cpa=%d nc=%d: %.1f us\n",
                   n, ncols, s.kind, s.TY, s.ring, s.ppt, s.ctasPerSM, s.cpa,
                   s.nc, 1e3f * ms / 3);
    if (ms < bestMs) {
      bestMs = ms;
      best = s;
    }
  };
  // plus, per points-per-thread, the tallest band one block can cover
  for (int ppt : {1, 2, 4}) {
    const int ty = ((streamMaxThreads(ppt) - 32) * ppt) / n;
    if (ty >= 1 && ty < n &&
        std::find(rows.begin(), rows.end(), ty) == rows.end())
      rows.push_back(ty);
  }
  for (int TY : rows) {
    for (int ring : {8, 16})
      for (int ppt : {1, 2, 4})
        for (int cps : {1, 2, 4})
          for (int cpa : {0, 1}) trial(Shape{TY, ring, ppt, cps, 0, cpa, 1});
    for (int ring : {4, 8, 16})
      for (int cps : {1, 2, 4}) trial(Shape{TY, ring, 1, cps, 1, 0, 1});
  }
  // staged-coefficient kernel: band rows a multiple of the rows per thread
  std::vector<int> srows;
  for (int TY = 2; TY <= std::min(n, 40); TY += 2) srows.push_back(TY);
  for (int TY : srows)
    for (int yr : {1, 2, 4})
      for (int ring : {8, 16})
        for (int cring : {2, 4, 8})
          for (int cps : {1, 2, 3, 4}) {
            for (int nc : {1, 2})
              trial(Shape{TY, ring, yr, cps, 2, cring, nc});
            trial(Shape{TY, ring, yr, cps, 3, cring, 1});
          }
  return best;
}

void applyH32(ncgm_ctx *ctx, int species, const float2 *X, float2 *Y,
              int ncols, float shift, cudaStream_t s) {
  // NCGM_STENCIL_SHAPE="rows,ring,ppt,ctasPerSM[,kind[,cpa[,nc]]]" fixes the
  // shape
  const char *envp = std::getenv("NCGM_STENCIL_SHAPE");
  const std::string env = envp ? envp : "";
  Shape sh{};
  {
    std::lock_guard<std::mutex> lock(g_tunedMutex);
    bool found = false;
    for (auto &t : g_tuned)
      if (t.n == ctx->n && t.env == env) {
        sh = t.s;
        found = true;
      }
    if (!found) {
      Shape fixed{};
      fixed.nc = 1;
      int th = 0;
      if (!env.empty() &&
          std::sscanf(env.c_str(), "%d,%d,%d,%d,%d,%d,%d", &fixed.TY,
                      &fixed.ring, &fixed.ppt, &fixed.ctasPerSM, &fixed.kind,
                      &fixed.cpa, &fixed.nc) >= 4 &&
          validShape(ctx->n, fixed, th))
        sh = fixed;
      else
        sh = tune(ctx, species, ncols);
      g_tuned.push_back({ctx->n, env, sh});
    }
  }
  if (!launchStream(ctx, species, X, Y, ncols, shift, s, sh))
    setError("FP32 stencil: launch shape or tensor map unavailable");
}

} // namespace ncgm
