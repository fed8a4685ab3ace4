// Density and mean-field accumulation of IterationData::updateQuantities
// (src/util/iteration_data.cpp:852-1125), fused per lattice point:
//  * densityKernel: rho, tau, J_{mu nu} and div J from a block of occupied
//    spinor columns in one pass (Wavefunction::density / kineticDensity /
//    soDensity / divJ, src/util/wavefunction.cpp:21-44,348-360,421-517), the
//    spinor gradients taken with the order-dropping 9-point stencils of
//    Operators::derivative (src/operators/differential_operators.cpp:482-543);
//  * gradLapKernel: grad rho and lap rho (gradNoSpin / lapNoSpin, 295-316,
//    356-417, 545-610, keeping the first-derivative formula that derivative2
//    uses at the two box faces);
//  * fieldsKernel: effective mass f_q and grad f_q (src/util/
//    effective_mass.cpp:7-34), Skyrme field U_q (wavefunction.cpp:264-310)
//    and spin-orbit field W_q (iteration_data.cpp:1094-1122);
//  * energyKernel: the trapezoid-weighted energy integrals of
//    iteration_data.cpp:153-271 and iteration_data_integrals.cpp:95-262.
// All FP64: these feed the fixed point whose energies are compared at keV.
#include "fd_deriv.cuh"
#include "k_density.cuh"

namespace ncgm {

namespace {

using fd::d1;

__device__ __forceinline__ double d2(const double *v, size_t base,
                                     size_t stride, int pos, int n, double h) {
  auto g = [&](int p) { return v[base + (size_t)p * stride]; };
  if (pos == 0) {
    return (g(pos + 1) - g(pos)) / (h);
  } else if (pos == 1 || pos == n - 2) {
    return (g(pos - 1) - 2.0 * g(pos) + g(pos + 1)) / (h * h);
  } else if (pos == n - 1) {
    return (g(pos) - g(pos - 1)) / (h);
  } else if (pos == 2 || pos == n - 3) {
    double f_2 = g(pos - 2), f_1 = g(pos - 1), f0 = g(pos), f1 = g(pos + 1),
           f2 = g(pos + 2);
    return (-f2 + 16.0 * f1 - 30.0 * f0 + 16.0 * f_1 - f_2) / (12.0 * h * h);
  } else if (pos == 3 || pos == n - 4) {
    double f_3 = g(pos - 3), f_2 = g(pos - 2), f_1 = g(pos - 1), f0 = g(pos);
    double f1 = g(pos + 1), f2 = g(pos + 2), f3 = g(pos + 3);
    return (2.0 * f3 - 27.0 * f2 + 270.0 * f1 + -490.0 * f0 + 270.0 * f_1 -
            27.0 * f_2 + 2.0 * f_3) /
           (180.0 * h * h);
  } else {
    double f_4 = g(pos - 4), f_3 = g(pos - 3), f_2 = g(pos - 2),
           f_1 = g(pos - 1), f0 = g(pos);
    double f1 = g(pos + 1), f2 = g(pos + 2), f3 = g(pos + 3), f4 = g(pos + 4);
    return (-9.0 * f_4 + 128.0 * f_3 - 1008.0 * f_2 + 8064.0 * f_1 -
            14350.0 * f0 + 8064.0 * f1 - 1008.0 * f2 + 128.0 * f3 - 9.0 * f4) /
           (5040.0 * h * h);
  }
}

struct Cx {
  double x, y;
  __device__ Cx operator+(Cx o) const { return {x + o.x, y + o.y}; }
  __device__ Cx operator-(Cx o) const { return {x - o.x, y - o.y}; }
  __device__ Cx operator-() const { return {-x, -y}; }
  __device__ Cx operator/(double d) const { return {x / d, y / d}; }
  __device__ friend Cx operator*(double a, Cx c) { return {a * c.x, a * c.y}; }
};
__device__ __forceinline__ Cx cmul(Cx a, Cx b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
__device__ __forceinline__ Cx conjmul(Cx a, Cx b) { // conj(a) * b
  return {a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x};
}
// sigma_nu (a, b): x, y, z Pauli matrices
__device__ __forceinline__ void pauli(int nu, Cx a, Cx b, Cx &o0, Cx &o1) {
  if (nu == 0) {
    o0 = b;
    o1 = a;
  } else if (nu == 1) {
    o0 = {b.y, -b.x}; // -i b
    o1 = {-a.y, a.x}; //  i a
  } else {
    o0 = a;
    o1 = -b;
  }
}
__device__ __forceinline__ Cx scrub(Cx v) {
  return (isnan(v.x) || isnan(v.y)) ? Cx{0, 0} : v;
}

__global__ void densityKernel(const double2 *__restrict__ Phi, size_t ldphi,
                              int M, int n, double h, double *rho, double *tau,
                              double *J9, double *divJ) {
  const size_t ns = (size_t)n * n * n;
  const size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (p >= ns) return;
  const int i = (int)(p % n), j = (int)((p / n) % n), k = (int)(p / ((size_t)n * n));
  const size_t sy = n, sz = (size_t)n * n;
  double r = 0, t = 0, dj = 0;
  double J[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) J[q] = 0.0;
  for (int c = 0; c < M; ++c) {
    const double2 *ps = Phi + (size_t)c * ldphi;
    auto at = [&](size_t q, int s) {
      double2 v = ps[2 * q + s];
      return Cx{v.x, v.y};
    };
    Cx psi[2] = {at(p, 0), at(p, 1)};
    Cx g[3][2];
    for (int s = 0; s < 2; ++s) {
      g[0][s] = scrub(d1<Cx>(
          [&](int q) { return at(p - i + q, s); }, i, n, h));
      g[1][s] = scrub(d1<Cx>(
          [&](int q) { return at(p + ((long long)q - j) * (long long)sy, s); },
          j, n, h));
      g[2][s] = scrub(d1<Cx>(
          [&](int q) { return at(p + ((long long)q - k) * (long long)sz, s); },
          k, n, h));
    }
    // density: sum_s |psi_s|^2
    r += psi[0].x * psi[0].x + psi[0].y * psi[0].y;
    r += psi[1].x * psi[1].x + psi[1].y * psi[1].y;
    // kinetic density
    double m0 = 0, m1 = 0;
    for (int mu = 0; mu < 3; ++mu) {
      m0 += g[mu][0].x * g[mu][0].x + g[mu][0].y * g[mu][0].y;
      m1 += g[mu][1].x * g[mu][1].x + g[mu][1].y * g[mu][1].y;
    }
    t += m0 + m1;
    // spin-orbit density J_{mu nu} = Im(psi^* sigma_nu d_mu psi)
    for (int mu = 0; mu < 3; ++mu)
      for (int nu = 0; nu < 3; ++nu) {
        Cx q0, q1;
        pauli(nu, g[mu][0], g[mu][1], q0, q1);
        J[mu * 3 + nu] += psi[0].x * q0.y - psi[0].y * q0.x + psi[1].x * q1.y -
                          psi[1].y * q1.x;
      }
    // div J: -sum eps_{mu nu la} Im(d_nu psi^H sigma_la d_mu psi)
    Cx sum = {0, 0};
    const int tri[6][4] = {{0, 1, 2, 1},  {1, 2, 0, 1},  {2, 0, 1, 1},
                           {2, 1, 0, -1}, {0, 2, 1, -1}, {1, 0, 2, -1}};
    // reference loop order is (mu, nu, la) ascending; visit in that order
    const int ord[6] = {0, 4, 5, 1, 2, 3};
    for (int e = 0; e < 6; ++e) {
      const int *tr = tri[ord[e]];
      int mu = tr[0], nu = tr[1], la = tr[2];
      double eps = tr[3];
      Cx q0, q1;
      pauli(la, g[mu][0], g[mu][1], q0, q1);
      Cx term = conjmul(g[nu][0], q0) + conjmul(g[nu][1], q1);
      sum = sum + eps * term;
    }
    dj += sum.y;
  }
  rho[p] = r;
  tau[p] = t;
  for (int q = 0; q < 9; ++q) J9[q * ns + p] = J[q];
  divJ[p] = -dj;
}

__global__ void gradLapKernel(const double *v, int n, double h, double *g3,
                              double *lap) {
  const size_t ns = (size_t)n * n * n;
  const size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (p >= ns) return;
  const int i = (int)(p % n), j = (int)((p / n) % n), k = (int)(p / ((size_t)n * n));
  const size_t sy = n, sz = (size_t)n * n;
  const size_t bx = p - i, by = p - (size_t)j * sy, bz = p - (size_t)k * sz;
  if (g3) {
    double gx = d1<double>([&](int q) { return v[bx + q]; }, i, n, h);
    double gy = d1<double>([&](int q) { return v[by + (size_t)q * sy]; }, j, n, h);
    double gz = d1<double>([&](int q) { return v[bz + (size_t)q * sz]; }, k, n, h);
    g3[p] = isnan(gx) ? 0.0 : gx;
    g3[ns + p] = isnan(gy) ? 0.0 : gy;
    g3[2 * ns + p] = isnan(gz) ? 0.0 : gz;
  }
  if (lap) {
    double acc = 0.0;
    acc += d2(v, bx, 1, i, n, h);
    acc += d2(v, by, sy, j, n, h);
    acc += d2(v, bz, sz, k, n, h);
    lap[p] = acc;
  }
}

__global__ void mixKernel(double *old, const double *nw, double mu,
                          size_t count, int first) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= count) return;
  old[e] = first ? nw[e] : old[e] * (1.0 - mu) + nw[e] * mu;
}

__global__ void fieldsKernel(FieldsIn in, FieldsOut out) {
  const size_t ns = in.ns;
  const size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (p >= ns) return;
  const ncgm_edf &P = in.edf;
  const double rN = in.rhoN[p], rP = in.rhoP[p], rho = rN + rP;
  const double tN = in.tauN[p], tP = in.tauP[p], tau = tN + tP;
  const double lN = in.lapN[p], lP = in.lapP[p], lap = lN + lP;
  const double dN = in.spinOrbit ? in.divJN[p] : 0.0;
  const double dP = in.spinOrbit ? in.divJP[p] : 0.0;
  const double dJ = dN + dP;
  const double t3 = 48 * P.C0Drr / 3;
  const double x3 = -0.5 - 24 * P.C1Drr / t3;
  const double sg = P.sigma;
  const double base = 1.0 * in.hbar2m; // hbar^2 / (2 m_corr)
  for (int q = 0; q < 2; ++q) {
    const double rq = q ? rP : rN, tq = q ? tP : tN, lq = q ? lP : lN,
                 dq = q ? dP : dN;
    // EffectiveMass
    double f = 0.0;
    f += base;
    f += (P.C0rt - P.C1rt) * rho + 2 * P.C1rt * rq;
    (q ? out.fP : out.fN)[p] = f;
    for (int a = 0; a < 3; ++a) {
      double gr = in.gN[a * ns + p] + in.gP[a * ns + p];
      double gq = (q ? in.gP : in.gN)[a * ns + p];
      (q ? out.gfP : out.gfN)[a * ns + p] =
          (P.C0rt - P.C1rt) * gr + 2 * P.C1rt * gq;
    }
    // Wavefunction::field
    double U = 0.0;
    U += (2 * P.C0rr - 2 * P.C1rr) * rho + 4 * P.C1rr * rq;
    U += (P.C0rt - P.C1rt) * tau + 2 * P.C1rt * tq;
    U += (2 * P.C0rdr - 2 * P.C1rdr) * lap + 4 * P.C1rdr * lq;
    U += (P.C0nJ - P.C1nJ) * dJ + 2 * P.C1nJ * dq;
    double rm = rho - rq;
    U += (t3 / 12.0) * pow(rho, sg - 1.0) *
         ((1.0 + 0.5 * x3) * (sg + 2.0) * pow(rho, 2.0) -
          (x3 + 0.5) * (sg * (rq * rq + rm * rm) + 2.0 * rho * rq));
    (q ? out.UP : out.UN)[p] = U;
    // spin-orbit field W_q (B in the reference)
    for (int a = 0; a < 3; ++a) {
      double w = 0.0;
      double gs = in.gN[a * ns + p] + in.gP[a * ns + p];
      double gq = (q ? in.gP : in.gN)[a * ns + p];
      if (in.spinOrbit) {
        w += -(P.C0nJ - P.C1nJ) * gs;
        w += -2 * P.C1nJ * gq;
      }
      if (in.useJ) {
        // J vector by the Levi-Civita contraction (common_operators.cpp:24-38)
        auto jv = [&](const double *J9, int c) {
          const int A[3][2] = {{5, 7}, {6, 2}, {1, 3}};
          return J9[A[c][0] * ns + p] - J9[A[c][1] * ns + p];
        };
        double js = jv(in.JN, a) + jv(in.JP, a);
        double jq = jv(q ? in.JP : in.JN, a);
        w += 2 * (P.C0J2 - P.C1J2) * js;
        w += 4 * P.C1J2 * jq;
      }
      (q ? out.WP : out.WN)[a * ns + p] = w;
    }
  }
}

// trapezoid weight of point p (half per boundary face index)
__device__ __forceinline__ double trapW(size_t p, int n) {
  const int i = (int)(p % n), j = (int)((p / n) % n), k = (int)(p / ((size_t)n * n));
  double w = 1.0;
  if (i == 0 || i == n - 1) w *= 0.5;
  if (j == 0 || j == n - 1) w *= 0.5;
  if (k == 0 || k == n - 1) w *= 0.5;
  return w;
}

__device__ double blockReduce(double v, double *sh) {
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

// Per-point energy densities -> per-block partial integrals (kEnergyTerms).
__global__ void energyKernel(EnergyIn in, double *partials) {
  __shared__ double sh[256];
  const size_t ns = in.ns;
  const ncgm_edf &P = in.edf;
  const double hhh = in.h * in.h * in.h;
  double acc[kEnergyTerms];
#pragma unroll
  for (int t = 0; t < kEnergyTerms; ++t) acc[t] = 0.0;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < ns;
       p += (size_t)gridDim.x * blockDim.x) {
    const double w = trapW(p, in.n) * hhh;
    const double rN = in.rhoN[p], rP = in.rhoP[p];
    const double r0 = rN + rP, r1 = rN - rP;
    const double t0 = in.tauN[p] + in.tauP[p], t1 = in.tauN[p] - in.tauP[p];
    const double l0 = in.lapN[p] + in.lapP[p], l1 = in.lapN[p] - in.lapP[p];
    const double rs = pow(r0, P.sigma);
    double j0 = 0, j1 = 0;
    for (int a = 0; a < 3; ++a) {
      const int A[3][2] = {{5, 7}, {6, 2}, {1, 3}};
      double jn = in.JN[A[a][0] * ns + p] - in.JN[A[a][1] * ns + p];
      double jp = in.JP[A[a][0] * ns + p] - in.JP[A[a][1] * ns + p];
      j0 += (jn + jp) * (jn + jp);
      j1 += (jn - jp) * (jn - jp);
    }
    const double dj0 = in.divJN[p] + in.divJP[p],
                 dj1 = in.divJN[p] - in.divJP[p];
    const double sl = pow(rP, 4.0 / 3.0) * (-3.0 * kE2 / 4.0) *
                      pow(3.0 / M_PI, 1.0 / 3.0);
    double e[kEnergyTerms];
    e[0] = (P.C0rr * 1.0 + P.C0Drr * rs) * (r0 * r0);
    e[1] = (P.C1rr * 1.0 + P.C1Drr * rs) * (r1 * r1);
    e[2] = P.C0rdr * (r0 * l0);
    e[3] = P.C1rdr * (l1 * r1);
    e[4] = P.C0rt * (t0 * r0);
    e[5] = P.C1rt * (t1 * r1);
    e[6] = P.C0J2 * j0;
    e[7] = P.C1J2 * j1;
    e[8] = P.C0nJ * (dj0 * r0);
    e[9] = P.C1nJ * (dj1 * r1);
    e[10] = in.UCDir ? rP * in.UCDir[p] : 0.0;
    e[11] = sl;
    e[12] = 0.5 * in.hbar2 * in.tauN[p] / in.massCorr +
            0.5 * in.hbar2 * in.tauP[p] / in.massCorr;
    e[13] = -0.5 * P.sigma *
            (P.C0Drr * pow(r0, P.sigma + 2) + P.C1Drr * pow(r0, P.sigma) *
                                                  (r1 * r1));
#pragma unroll
    for (int t = 0; t < kEnergyTerms; ++t) acc[t] += e[t] * w;
  }
  for (int t = 0; t < kEnergyTerms; ++t) {
    double s = blockReduce(acc[t], sh);
    if (threadIdx.x == 0) partials[(size_t)t * gridDim.x + blockIdx.x] = s;
  }
}

__global__ void sumPartials(const double *partials, int nblk, int terms,
                            double *out) {
  int t = threadIdx.x;
  if (t >= terms) return;
  double s = 0;
  for (int b = 0; b < nblk; ++b) s += partials[(size_t)t * nblk + b];
  out[t] = s;
}

// int O_c(r) rho(r) for several scalar operators (constraints), one block
// partial each; O given as a list of operator ids on the fly.
__global__ void weightedIntegrals(const double *f, const double *g, int n,
                                  double h, double *partials) {
  __shared__ double sh[256];
  const size_t ns = (size_t)n * n * n;
  const double hhh = h * h * h;
  double a = 0;
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < ns;
       p += (size_t)gridDim.x * blockDim.x)
    a += (g ? f[p] * g[p] : f[p]) * hhh * trapW(p, n);
  double s = blockReduce(a, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// per column trapezoid norm of a spinor block, then scale (normalize)
__global__ void columnIntegral(const double2 *X, size_t ld, int n, double h,
                               double *out) {
  __shared__ double sh[256];
  const size_t ns = (size_t)n * n * n;
  const int c = blockIdx.x;
  const double2 *x = X + (size_t)c * ld;
  const double hhh = h * h * h;
  double a = 0;
  for (size_t p = threadIdx.x; p < ns; p += blockDim.x) {
    double2 u = x[2 * p], d = x[2 * p + 1];
    double den = (u.x * u.x + u.y * u.y) + (d.x * d.x + d.y * d.y);
    a += den * hhh * trapW(p, n);
  }
  double s = blockReduce(a, sh);
  if (threadIdx.x == 0) out[c] = s;
}

__global__ void scaleColumns(double2 *X, size_t ld, size_t N, const double *I,
                             int sqrtInv) {
  const int c = blockIdx.y;
  const double s = sqrt(I[c]);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < N;
       e += (size_t)gridDim.x * blockDim.x) {
    double2 v = X[(size_t)c * ld + e];
    X[(size_t)c * ld + e] = make_double2(v.x / s, v.y / s);
  }
}

} // namespace

void densities(const double2 *Phi, size_t ld, int M, int n, double h,
               double *rho, double *tau, double *J9, double *divJ,
               cudaStream_t s) {
  const size_t ns = (size_t)n * n * n;
  densityKernel<<<(unsigned)((ns + 127) / 128), 128, 0, s>>>(
      Phi, ld, M, n, h, rho, tau, J9, divJ);
}

void gradLap(const double *v, int n, double h, double *g3, double *lap,
             cudaStream_t s) {
  const size_t ns = (size_t)n * n * n;
  gradLapKernel<<<(unsigned)((ns + 255) / 256), 256, 0, s>>>(v, n, h, g3, lap);
}

void mix(double *old, const double *nw, double mu, size_t count, bool first,
         cudaStream_t s) {
  mixKernel<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(old, nw, mu, count,
                                                           first ? 1 : 0);
}

void meanFields(const FieldsIn &in, const FieldsOut &out, cudaStream_t s) {
  fieldsKernel<<<(unsigned)((in.ns + 127) / 128), 128, 0, s>>>(in, out);
}

void energyIntegrals(const EnergyIn &in, double *partials, double *out,
                     cudaStream_t s) {
  const int nblk = 120;
  energyKernel<<<nblk, 256, 0, s>>>(in, partials);
  sumPartials<<<1, 32, 0, s>>>(partials, nblk, kEnergyTerms, out);
}

void integral(const double *f, const double *g, int n, double h,
              double *partials, double *out, cudaStream_t s) {
  const int nblk = 120;
  weightedIntegrals<<<nblk, 256, 0, s>>>(f, g, n, h, partials);
  sumPartials<<<1, 32, 0, s>>>(partials, nblk, 1, out);
}

void normalizeColumns(double2 *X, size_t ld, int ncols, int n, double h,
                      double *work, cudaStream_t s) {
  if (ncols <= 0) return;
  columnIntegral<<<ncols, 256, 0, s>>>(X, ld, n, h, work);
  const size_t N = 2 * (size_t)n * n * n;
  dim3 grid((unsigned)std::min<size_t>(512, (N + 255) / 256), ncols);
  scaleColumns<<<grid, 256, 0, s>>>(X, ld, N, work, 1);
}

} // namespace ncgm
