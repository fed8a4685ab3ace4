// Arithmetic of one output point of the matrix-free Hamiltonian, shared by
// the FP64 (k_hamiltonian.cu) and FP32 (k_stencil32.cu) stencil kernels.
#pragma once
#include <cuda_runtime.h>

namespace ncgm {

template <class T> struct Spinor {
  T r0, i0, r1, i1;
};

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


} // namespace ncgm
