// Device helpers shared by the FP32 stencil kernels (k_stencil32.cu,
// k_stencil_stage.cu): mbarrier waits with iteration limits, 5-D TMA tile
// loads, packed f32x2 arithmetic and the per-point operator pointH2.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

struct ncgm_ctx;

namespace ncgm {
namespace s32 {

constexpr int kPPT = 4;       // max owned points per thread
constexpr int kMaxRuns = 48;  // (column, band) runs per CTA

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
__device__ __forceinline__ bool mbarWait(uint64_t *bar, uint32_t phase,
                                         uint32_t limit) {
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t done;
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
__device__ __forceinline__ void tmaTile5(void *dst, const CUtensorMap *map,
                                         int c1, int c2, int c3, int c4,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::"
      "complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(
          smemAddr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(c1), "r"(c2), "r"(c3),
      "r"(c4), "r"(smemAddr(bar))
      : "memory");
}

__device__ __forceinline__ void tmaTile4(void *dst, const CUtensorMap *map,
                                         int c0, int c1, int c2, int c3,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::"
      "complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(
          smemAddr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
      "r"(smemAddr(bar))
      : "memory");
}
// One band-plane box of a map made by tensorMapX: point coordinate i0 (a
// multiple-of-16-byte float offset 4 * i0 in the flat form), row j, plane k,
// column (or table half) d4.
__device__ __forceinline__ void tmaBand(void *dst, const CUtensorMap *map,
                                        bool flat, int i0, int j, int k,
                                        int d4, uint64_t *bar) {
  if (flat)
    tmaTile4(dst, map, 4 * i0, j, k, d4, bar);
  else
    tmaTile5(dst, map, i0, j, k, d4, bar);
}

struct StreamArgs {
  float4 *Y;
  const float4 *coef;
  int n, TY, nbands, ring, ppt;
  size_t ns;
  long long total; // ncols * nbands * n output band-planes
  float shift;
  int *err;
  int cpa; // stencilStream32: coefficients prefetched one plane ahead
  int flat; // X map is the flat 4-D form (see tensorMapX)
};

struct Run {
  int cb, ka, kb, base;
};

__device__ __forceinline__ void mbarArrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smemAddr(bar))
               : "memory");
}
// bounded wait that lets the warp sleep between polls (suspend-time hint)
__device__ __forceinline__ bool mbarWaitSleep(uint64_t *bar, uint32_t phase,
                                              uint32_t limit) {
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smemAddr(bar)), "r"(phase), "r"(1000u)
        : "memory");
    if (done) return true;
  }
  return false;
}

// bounded wait polling with plain try_wait and a nanosleep of `ns` between
// polls; ns = 0 selects the suspend-hint wait above. Consumer warps wait
// this way: with the suspend hint they resumed measurably later after the
// phase completed (5-7 % of the stencil time at 40^3 x 64).
constexpr uint32_t kPollNs = 32;
__device__ __forceinline__ bool mbarWaitBackoff(uint64_t *bar, uint32_t phase,
                                                uint32_t limit, uint32_t ns) {
  if (ns == 0) return mbarWaitSleep(bar, phase, limit);
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smemAddr(bar)), "r"(phase)
        : "memory");
    if (done) return true;
    __nanosleep(ns);
  }
  return false;
}

// ---- packed FP32 pair arithmetic (f32x2: one instruction, two lanes) ----
using f2x = unsigned long long;
__device__ __forceinline__ f2x pk(float a, float b) {
  f2x r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float2 upk(f2x v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
__device__ __forceinline__ f2x add2(f2x a, f2x b) {
  f2x r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f2x sub2(f2x a, f2x b) {
  f2x r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f2x mul2(f2x a, f2x b) {
  f2x r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f2x fma2(f2x a, f2x b, f2x c) {
  f2x r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
__device__ __forceinline__ f2x bc(float a) { return pk(a, a); }

// pointH (stencil_core.cuh) with each spin component held as one (re, im)
// pair: the kinetic, derivative and gradient terms are real coefficients
// times pairs; the spin-orbit matrix is split as A + iB (A, B real), so
// (A + iB) D = A D + i (B D) and only one i-rotation per spin is needed.
__device__ __forceinline__ float4 pointH2(const float4 ca, const float4 cb,
                                          float shift, float4 v, float4 xp1,
                                          float4 xm1, float4 xp2, float4 xm2,
                                          float4 yp1, float4 ym1, float4 yp2,
                                          float4 ym2, float4 zp1, float4 zm1,
                                          float4 zp2, float4 zm2) {
  const f2x D = bc(ca.x + shift), NF = bc(-ca.y);
  const f2x GX = bc(ca.z), GY = bc(ca.w), GZ = bc(cb.x);
  const f2x WX = bc(cb.y), WY = bc(cb.z), WZ = bc(cb.w);
  const f2x NWX = bc(-cb.y), NWY = bc(-cb.z), NWZ = bc(-cb.w);
  const f2x C43 = bc(4.0f / 3.0f), NC112 = bc(-1.0f / 12.0f), EIGHT = bc(8.f);
  f2x o[2], Dx[2], Dy[2], Dz[2];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    auto A = [s](float4 q) { return s ? pk(q.z, q.w) : pk(q.x, q.y); };
    const f2x a_xp1 = A(xp1), a_xm1 = A(xm1), a_xp2 = A(xp2), a_xm2 = A(xm2);
    const f2x a_yp1 = A(yp1), a_ym1 = A(ym1), a_yp2 = A(yp2), a_ym2 = A(ym2);
    const f2x a_zp1 = A(zp1), a_zm1 = A(zm1), a_zp2 = A(zp2), a_zm2 = A(zm2);
    f2x s1 = add2(add2(add2(a_xp1, a_xm1), add2(a_yp1, a_ym1)),
                  add2(a_zp1, a_zm1));
    f2x s2 = add2(add2(add2(a_xp2, a_xm2), add2(a_yp2, a_ym2)),
                  add2(a_zp2, a_zm2));
    f2x t = fma2(C43, s1, mul2(NC112, s2));
    f2x os = fma2(NF, t, mul2(D, A(v)));
    Dx[s] = fma2(EIGHT, sub2(a_xp1, a_xm1), sub2(a_xm2, a_xp2));
    Dy[s] = fma2(EIGHT, sub2(a_yp1, a_ym1), sub2(a_ym2, a_yp2));
    Dz[s] = fma2(EIGHT, sub2(a_zp1, a_zm1), sub2(a_zm2, a_zp2));
    os = fma2(GX, Dx[s], os);
    os = fma2(GY, Dy[s], os);
    o[s] = fma2(GZ, Dz[s], os);
  }
  // spin-orbit: real parts (A) into o, imaginary parts (B) into u, o += i u
  o[0] = fma2(NWZ, Dx[1], o[0]);
  o[0] = fma2(WX, Dz[1], o[0]);
  f2x u0 = mul2(WY, Dx[0]);
  u0 = fma2(NWX, Dy[0], u0);
  u0 = fma2(WZ, Dy[1], u0);
  u0 = fma2(NWY, Dz[1], u0);
  o[1] = fma2(WZ, Dx[0], o[1]);
  o[1] = fma2(NWX, Dz[0], o[1]);
  f2x u1 = mul2(NWY, Dx[1]);
  u1 = fma2(WZ, Dy[0], u1);
  u1 = fma2(WX, Dy[1], u1);
  u1 = fma2(NWY, Dz[0], u1);
  const float2 p0 = upk(o[0]), p1 = upk(o[1]), q0 = upk(u0), q1 = upk(u1);
  return make_float4(p0.x - q0.y, p0.y + q0.x, p1.x - q1.y, p1.y + q1.x);
}


} // namespace s32

// host helpers of the FP32 stencil launchers (k_stencil32.cu)
int smCount();
// Tensor map over a column-major block of float4 points [d4][k][j][i], box
// (boxW points, boxRows rows, 1 plane, boxD4 columns); cached per argument
// set. Flat form (flat = true) when 4 * boxW <= 256: dims (4n floats, j, k,
// d4), so each box row is one contiguous run of 16 * boxW bytes; otherwise
// dims (4 floats, i, j, k, d4) with 16-byte box rows. Both fill the same
// shared-memory layout [d4][row][point][4 floats].
bool tensorMapX(const void *base, int n, int d4, int boxW, int boxRows,
                int boxD4, bool &flat, CUtensorMap *out);

// staged-coefficient kernel (k_stencil_stage.cu): TY band rows, X ring and
// coefficient ring depths, YR rows per thread, NC columns per box, CTAs/SM
bool validStage(int n, int TY, int ring, int cring, int yr, int nc, int cps,
                bool zq, int &threads);
bool launchStage(ncgm_ctx *ctx, int species, const float2 *X, float2 *Y,
                 int ncols, float shift, cudaStream_t st, int TY, int ring,
                 int cring, int yr, int nc, int cps, bool zq);
} // namespace ncgm
