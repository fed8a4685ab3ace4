// The self-consistent Hartree-Fock(-Bogoliubov) iteration on the device:
// the GB300 form of main()'s run loop (src/main.cpp:59-342) with
// IterationData::updateQuantities (src/util/iteration_data.cpp:852-1125),
// the energies (iteration_data.cpp:153-271, iteration_data_integrals.cpp),
// the Woods-Saxon + harmonic-oscillator guess (main.cpp:72-111) and the
// augmented-Lagrangian constraints (src/skyrme/*_constraint.cpp).
//
// Lattice-sized data never leaves the device. The host keeps the O(M^2)
// bookkeeping the reference does with scalars and small matrices: Kramers
// pair matching, locking, constraint multipliers, bisection brackets.
#include "k_dense.cuh"
#include "k_density.cuh"
#include "k_pairing.cuh"
#include "k_poisson.cuh"
#include "ncgm_internal.cuh"

#include <algorithm>
#include <atomic>
#include <thread>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <tuple>
#include <vector>

namespace ncgm {

bool isDevicePtr(const void *p);
int gcgRun(ncgm_ctx *ctx, int species, const double2 *Xinit, int xcols,
           const double2 *ConjDir, int pcols, int nev,
           const ncgm_gcg_params &prm, double2 *Xout, double *lamOut,
           ncgm_gcg_stats *stats);

namespace {

constexpr double kHbar = 197.327053;
constexpr double kMass = 938.91869;

double now() {
  return std::chrono::duration<double>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// constraint operators O(r) (xcm/ycm/zcm, x^2-y^2, 2xy, r^3 Y30, Q20)
// SphericalHarmonics::Y (spherical_harmonics.cpp:14-99): associated
// Legendre by the upward recurrence (no Condon-Shortley sign inside), the
// (-1)^|m| factor and e^{i |m| phi}, conjugated with (-1)^|m| for m < 0
__device__ double2 ylmDev(int l, int m, double theta, double phi) {
  const int mm = m < 0 ? -m : m;
  double fl = 1.0, fh = 1.0;
  for (int i = 2; i <= l - mm; ++i) fl *= i;
  for (int i = 2; i <= l + mm; ++i) fh *= i;
  const double norm = sqrt(((2.0 * l + 1.0) / (4.0 * M_PI)) * (fl / fh));
  const double x = cos(theta);
  double pmm = 1.0;
  if (mm > 0) {
    double fact = 1.0;
    for (int i = 1; i <= 2 * mm - 1; i += 2) fact *= i;
    pmm = fact * pow(1.0 - x * x, mm / 2.0);
  }
  double leg = pmm;
  if (l > mm) {
    double p1 = x * (2 * mm + 1) * pmm, p2 = pmm;
    leg = p1;
    for (int ll = mm + 2; ll <= l; ++ll) {
      const double pll = ((2 * ll - 1) * x * p1 - (ll + mm - 1) * p2) / (ll - mm);
      p2 = p1;
      p1 = pll;
      leg = pll;
    }
  }
  const double sgn = (mm % 2) ? -1.0 : 1.0;
  const double re = sgn * norm * leg * cos(mm * phi),
               im = sgn * norm * leg * sin(mm * phi);
  return m < 0 ? make_double2(sgn * re, -sgn * im) : make_double2(re, im);
}

// MultipoleConstraint's operator X_lm r^l (multipole_constraint.cpp:24-27):
// X_lm = sqrt2 Re Y_l,-m (m > 0), sqrt2 Im Y_lm (m < 0), Re Y_l0
// (spherical_harmonics.cpp:45-58); NaN at the origin, as acos(0/0)
__device__ double multipoleOp(int l, int m, double x, double y, double z) {
  const double r = sqrt(x * x + y * y + z * z);
  const double theta = acos(z / r), phi = atan2(y, x);
  double X;
  if (m > 0) X = 2.0 * ylmDev(l, -m, theta, phi).x / sqrt(2.0);
  else if (m < 0) X = 2.0 * ylmDev(l, m, theta, phi).y / sqrt(2.0);
  else X = ylmDev(l, 0, theta, phi).x;
  return X * pow(fabs(r), (double)l);
}

// multipole constraints carry kind = kMultipoleKind + 100 l + (m + 50)
constexpr int kMultipoleKind = 1000;

__device__ double constraintOp(int kind, double x, double y, double z) {
  if (kind >= kMultipoleKind) {
    const int lm = kind - kMultipoleKind;
    return multipoleOp(lm / 100, lm % 100 - 50, x, y, z);
  }
  switch (kind) {
  case 0: return x;
  case 1: return y;
  case 2: return z;
  case 3: return x * x - y * y;
  case 4: return 2.0 * x * y;
  case 5: {
    double r = sqrt(x * x + y * y + z * z);
    double ct = z / r;
    return r * r * r * sqrt(7.0 / (4.0 * M_PI)) * 0.5 * (5.0 * ct * ct * ct - 3.0 * ct);
  }
  default:
    return 0.25 * sqrt(5 / (M_PI)) * (2.0 * z * z - y * y - x * x);
  }
}

__device__ __forceinline__ double trapWd(size_t p, int n) {
  const int i = (int)(p % n), j = (int)((p / n) % n), k = (int)(p / ((size_t)n * n));
  double w = 1.0;
  if (i == 0 || i == n - 1) w *= 0.5;
  if (j == 0 || j == n - 1) w *= 0.5;
  if (k == 0 || k == n - 1) w *= 0.5;
  return w;
}

// partials[c * nblk + b] = int O_c (rhoN + rhoP), c < nc
__global__ void constraintQ(const double *rN, const double *rP, int n,
                            double a, double h, const int *kinds, int nc,
                            double *partials) {
  __shared__ double sh[256];
  const size_t ns = (size_t)n * n * n;
  const double hhh = h * h * h;
  for (int c = 0; c < nc; ++c) {
    double acc = 0;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < ns;
         p += (size_t)gridDim.x * blockDim.x) {
      const int i = (int)(p % n), j = (int)((p / n) % n), k = (int)(p / ((size_t)n * n));
      double O = constraintOp(kinds[c], -a + i * h, -a + j * h, -a + k * h);
      acc += (O * (rN[p] + rP[p])) * hhh * trapWd(p, n);
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) partials[(size_t)c * gridDim.x + blockIdx.x] = sh[0];
    __syncthreads();
  }
}

// Uconstr = sum_c coef_c O_c ; UN += Uconstr ; UP += Uconstr
__global__ void constraintField(const int *kinds, const double *coef, int nc,
                                int n, double a, double h, double *UC,
                                double *UN, double *UP) {
  const size_t ns = (size_t)n * n * n;
  const size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (p >= ns) return;
  const int i = (int)(p % n), j = (int)((p / n) % n), k = (int)(p / ((size_t)n * n));
  double v = 0;
  for (int c = 0; c < nc; ++c)
    v += coef[c] * constraintOp(kinds[c], -a + i * h, -a + j * h, -a + k * h);
  UC[p] = v;
  UN[p] += v;
  UP[p] += v;
}

__global__ void zeroKernel(double *x, size_t n) {
  size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e < n) x[e] = 0.0;
}

struct Constraint {
  int kind;
  double target, C, gamma, lambda = 0, value = 0;
  bool first = true;
  double error() const {
    if (kind <= 2) return 0.0; // COM constraints (xcm_constraint.cpp:13)
    double t = (kind == 6 || kind >= kMultipoleKind) ? target : 0.0;
    if (std::abs(t) <= 1e-12) return std::abs(value);
    return std::abs(value / t - 1.0);
  }
};

Constraint makeConstraint(int kind, double target) {
  Constraint c;
  c.kind = kind;
  c.target = target;
  c.C = (kind <= 2) ? 0.05 : (kind == 5 ? 0.001 : 0.005);
  c.gamma = (kind <= 2) ? 0.2 : 0.3;
  return c;
}

struct BCSRes {
  std::vector<double> u2, v2, Delta, qp;
  double lambda = 0, Epair = 0;
};
// HFB amplitudes of one species on the device (M x M, col-major); `ready`
// once the HFB branch has started (startHFBIter)
struct HFBRes {
  double *U = nullptr, *V = nullptr, *kappa = nullptr;
  int M = 0;
  bool ready = false;
  double lambda = 0, energy = 0;
};

// Device workspace of the HFB step, shared by both species (they run one
// after the other on the main stream); M = the larger basis
struct HfbWork {
  int M = 0;
  double2 *gemmW = nullptr, *gemmParts = nullptr; // kappa / Delta products
  void *gemmExact = nullptr; // exact-digit scratch (tensor-core form)
  double *e = nullptr, *ff = nullptr, *Kff = nullptr, *Delta = nullptr,
         *Uw = nullptr, *Vw = nullptr, *eig = nullptr, *scal = nullptr;
  double2 *C = nullptr, *G = nullptr, *H = nullptr, *Hwork = nullptr,
          *Hv = nullptr, *rho = nullptr, *Wm = nullptr, *T = nullptr;
  int *perm = nullptr, *status = nullptr;
  void *heigScr = nullptr; // the eigensolvers' workspace (up to 2M)
  size_t heigScrB = 0;
  static constexpr int kChunks = 64;
};

struct Species {
  int orb = 0;
  double2 *X = nullptr, *Xn = nullptr, *CD = nullptr, *Phi = nullptr,
          *TX = nullptr;
  std::vector<double> e;
  int cdCols = 0;
  BCSRes bcs;
  HFBRes hfb, hfbNew; // current amplitudes and the next step's candidate
  ncgm_pairing par;
};

struct Run {
  ncgm_ctx *ctx = nullptr;
  // proton context: its own stream and workspace, so that the two species'
  // eigenproblems of an HF iteration run on two host threads at once
  // (null when the species run one after the other on ctx)
  ncgm_ctx *ctxP = nullptr;
  cudaEvent_t evFields = nullptr, evProtons = nullptr;
  ncgm_hf_config cfg;
  int n = 0;
  size_t ns = 0, N = 0;
  double a = 0, h = 0;
  cudaStream_t s = nullptr;
  // lattice state
  double *rho[2], *tau[2], *J9[2], *divJ[2], *g[2], *lap[2];
  double *f[2], *gf[2], *U[2], *W[2];
  double *UCdir = nullptr, *UCoul = nullptr, *UConstr = nullptr;
  double *nrho = nullptr, *ntau = nullptr, *nJ9 = nullptr, *ndivJ = nullptr;
  double *scratch = nullptr, *poissonWork = nullptr, *energy = nullptr;
  double2 *cplx = nullptr; // small complex matrices
  double *small = nullptr; // small real matrices
  int *ismall = nullptr;
  bool have = false, haveCoul = false;
  double massCorr = kMass, energyDiff = 1.0;
  Species sp[2];
  std::vector<Constraint> cons;
  double tPair = 0, tFields = 0, tPoisson = 0, tGcg = 0;
  double constraintEnergy = 0; // of the last energy evaluation
  std::vector<void *> allocs;
  // tensor-core form: scratch of the exact-digit Gram / V C products of the
  // driver's own overlaps and rotations (allocated on first use)
  void *tcScr = nullptr;
  bool tc() const { return cfg.hf_gcg.precision == NCGM_FP32_TC; }
  void *tcScratch() {
    if (!tcScr) {
      int M = std::max(sp[0].orb, sp[1].orb);
      size_t b = std::max(exactGramScratchDoubles(N, M, M) * sizeof(double),
                          exactVCScratchBytes(N, M, M));
      tcScr = alloc<char>(b + 1024);
    }
    return tcScr;
  }

  // HFB workspace and both species' amplitude matrices (first use)
  HfbWork hw;
  HfbWork *hfbWork() {
    if (hw.gemmW) return &hw;
    const int M = std::max(sp[0].orb, sp[1].orb);
    const size_t MM = (size_t)M * M;
    HfbWork w;
    w.M = M;
    w.gemmParts = alloc<double2>(HfbWork::kChunks * MM);
    if (tc()) {
      // both bounds hold for every window size nS <= M
      const size_t b =
          std::max(exactGramScratchDoubles(ns, M, M) * sizeof(double),
                   exactVCScratchBytes(N, M, M));
      w.gemmExact = alloc<char>(b + 1024);
      if (!w.gemmExact) return nullptr;
    }
    double *d = alloc<double>(4 * (size_t)M + 4 * MM + 2 * (size_t)M + 16);
    double2 *c = alloc<double2>(2 * MM + 3 * 4 * MM + 3 * MM);
    int *iw = alloc<int>(2 * (size_t)M + 16);
    for (int q = 0; q < 2; ++q)
      for (HFBRes *h : {&sp[q].hfb, &sp[q].hfbNew}) {
        const size_t mq = (size_t)sp[q].orb * sp[q].orb;
        h->U = alloc<double>(mq);
        h->V = alloc<double>(mq);
        h->kappa = alloc<double>(mq);
        if (!h->kappa) return nullptr;
      }
    w.gemmW = alloc<double2>(N * (size_t)M);
    w.heigScrB = heigScratchBytes(2 * M);
    w.heigScr = alloc<char>(w.heigScrB);
    if (!w.gemmParts || !d || !c || !iw || !w.gemmW || !w.heigScr)
      return nullptr;
    w.e = d;
    w.ff = w.e + M;
    w.eig = w.ff + M; // 2M
    w.Kff = w.eig + 2 * (size_t)M;
    w.Delta = w.Kff + MM;
    w.Uw = w.Delta + MM;
    w.Vw = w.Uw + MM;
    w.scal = w.Vw + MM;
    w.C = c;
    w.G = w.C + MM;
    w.H = w.G + MM;
    w.Hwork = w.H + 4 * MM;
    w.Hv = w.Hwork + 4 * MM;
    w.rho = w.Hv + 4 * MM;
    w.Wm = w.rho + MM;
    w.T = w.Wm + MM;
    w.perm = iw;
    w.status = iw + 2 * M + 8;
    hw = w;
    return &hw;
  }
  PairingGemm pairingGemm() const {
    PairingGemm g;
    if (tc()) g.exactScratch = hw.gemmExact;
    g.partials = hw.gemmParts;
    g.maxChunks = HfbWork::kChunks;
    return g;
  }

  template <class T> T *alloc(size_t count) {
    void *p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess)
      return nullptr;
    allocs.push_back(p);
    return static_cast<T *>(p);
  }
  ~Run() {
    if (ctxP) cudaStreamSynchronize(ctxP->stream);
    for (void *p : allocs) cudaFree(p);
    if (evFields) cudaEventDestroy(evFields);
    if (evProtons) cudaEventDestroy(evProtons);
    if (ctxP) ncgm_destroy(ctxP);
    if (ctx) ncgm_destroy(ctx);
  }
};

// NCGM_HF_PHASE_SYNC=1: synchronise both species' streams after every phase
// of an HF iteration and name the phase in the error, so that a failing
// kernel is attributed to its phase (diagnostics; off by default)
bool phaseSyncOn() {
  static const bool v = [] {
    const char *e = std::getenv("NCGM_HF_PHASE_SYNC");
    return e && e[0] == '1';
  }();
  return v;
}
int phaseSync(Run &R, const char *phase, int it) {
  if (!phaseSyncOn()) return NCGM_OK;
  cudaError_t e = cudaStreamSynchronize(R.s);
  if (e == cudaSuccess && R.ctxP) e = cudaStreamSynchronize(R.ctxP->stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    setError(std::string("hf: iteration ") + std::to_string(it) + ", " +
             phase + ": " + cudaGetErrorString(e));
    return NCGM_ERR_CUDA;
  }
  return NCGM_OK;
}

int sync(Run &R) {
  cudaError_t e = cudaStreamSynchronize(R.s);
  if (e != cudaSuccess) {
    setError(std::string("hf: ") + cudaGetErrorString(e));
    return NCGM_ERR_CUDA;
  }
  return NCGM_OK;
}

// gram of columns (N rows): C = A^H B into host matrix (p x q)
int hostGram(Run &R, const double2 *A, int p, const double2 *B, int q,
             std::vector<double2> &C) {
  static thread_local double2 *parts = nullptr;
  static thread_local size_t cap = 0;
  const int maxChunks = 64;
  size_t need = (size_t)maxChunks * p * q;
  if (cap < need) {
    if (parts) cudaFree(parts);
    if (cudaMalloc(&parts, need * sizeof(double2)) != cudaSuccess) {
      parts = nullptr;
      cap = 0;
      return NCGM_ERR_NOMEM;
    }
    cap = need;
  }
  if (R.tc() && R.tcScratch())
    gramTCExact(A, R.N, p, B, R.N, q, R.N, R.cplx, p,
                static_cast<double *>(R.tcScratch()), R.s);
  else
    gram(A, R.N, p, B, R.N, q, R.N, R.cplx, p, parts, maxChunks, R.s);
  C.resize((size_t)p * q);
  cudaMemcpyAsync(C.data(), R.cplx, sizeof(double2) * p * q,
                  cudaMemcpyDeviceToHost, R.s);
  return sync(R);
}

// --- BCS (iteration_data.cpp:384-465, bcs.cpp:65-321) ----------------------
BCSRes nullBCS(const std::vector<double> &e, int num) {
  BCSRes b;
  const int M = (int)e.size();
  b.u2.assign(M, 1.0);
  b.v2.assign(M, 0.0);
  for (int i = 0; i < num && i < M; ++i) {
    b.u2[i] = 0.0;
    b.v2[i] = 1.0;
  }
  b.Delta.assign(num, 0.0);
  b.qp.resize(M);
  for (int i = 0; i < M; ++i) b.qp[i] = b.v2[i] * e[i];
  return b;
}

int bcsIter(Run &R, Species &S, int A, const std::vector<double> &oldDelta,
            double oldLambda, BCSRes &out) {
  const int M = S.orb;
  // pair overlaps |phi^H T phi|^2 (bcs.cpp:65-70)
  timeReverse(S.X, S.TX, R.ns, M, R.N, false, R.s);
  std::vector<double2> ov;
  NCGM_TRY(hostGram(R, S.X, M, S.TX, M, ov));
  // match_time_reversal (bcs.cpp:71-105)
  std::vector<std::tuple<double, int, int>> list;
  for (int k = 0; k < M; ++k)
    for (int j = 0; j < M; ++j) {
      double2 z = ov[(size_t)j * M + k];
      double v = z.x * z.x + z.y * z.y;
      if (std::abs(v) > 1e-6) list.emplace_back(v, k, j);
    }
  std::stable_sort(list.begin(), list.end(), [](const auto &x, const auto &y) {
    return std::get<0>(x) > std::get<0>(y);
  });
  std::vector<int> partner(M, -1);
  std::vector<char> used(M, 0);
  for (auto &t : list) {
    int k = std::get<1>(t), j = std::get<2>(t);
    if (used[k] || used[j] || k == j) continue;
    partner[k] = j;
    partner[j] = k;
    used[k] = used[j] = 1;
  }
  std::vector<int> unique, s2p(M, 0);
  std::vector<bool> visited(M, false);
  for (int i = 0; i < M; ++i)
    if (!visited[i]) {
      int pt = partner[i];
      if (pt != i && pt != -1) {
        int pi = (int)unique.size();
        unique.push_back(i);
        s2p[i] = s2p[pt] = pi;
        visited[i] = visited[pt] = true;
      }
    }
  const int np = (int)unique.size();
  std::vector<double> eps(np);
  for (int p = 0; p < np; ++p) eps[p] = S.e[unique[p]];
  std::vector<double> oldU;
  if ((int)oldDelta.size() == np * 2) {
    oldU.resize(std::min(M / 2, np));
    for (size_t i = 0; i < oldU.size(); ++i) oldU[i] = oldDelta[unique[i]];
  } else {
    oldU = oldDelta;
  }
  bool useOld = (int)oldU.size() == np && np > 0 &&
                *std::max_element(oldU.begin(), oldU.end()) > 1e-3;
  // device work
  int *dCols = R.ismall;
  double *dG = R.small, *dEps = dG + (size_t)np * np, *dOld = dEps + np,
         *du2 = dOld + np, *dv2 = du2 + np, *dD = dv2 + np, *dSc = dD + np,
         *dW = dSc + 4;
  cudaMemcpyAsync(dCols, unique.data(), sizeof(int) * np,
                  cudaMemcpyHostToDevice, R.s);
  densityGram(S.X, R.N, dCols, np, R.n, R.h, S.par.V0, dG, R.s);
  std::vector<double> G((size_t)np * np);
  cudaMemcpyAsync(G.data(), dG, sizeof(double) * np * np,
                  cudaMemcpyDeviceToHost, R.s);
  NCGM_TRY(sync(R));
  std::vector<double> Gs((size_t)np * np);
  for (int p = 0; p < np; ++p)
    for (int q = 0; q < np; ++q)
      Gs[(size_t)q * np + p] = 0.5 * (G[(size_t)q * np + p] + G[(size_t)p * np + q]);
  cudaMemcpyAsync(dG, Gs.data(), sizeof(double) * np * np,
                  cudaMemcpyHostToDevice, R.s);
  cudaMemcpyAsync(dEps, eps.data(), sizeof(double) * np, cudaMemcpyHostToDevice,
                  R.s);
  if (useOld)
    cudaMemcpyAsync(dOld, oldU.data(), sizeof(double) * np,
                    cudaMemcpyHostToDevice, R.s);
  bcsSolve(dEps, dG, np, A, S.par.window, S.par.window_both, dOld, useOld,
           oldLambda, du2, dv2, dD, dSc, dW, R.s);
  std::vector<double> u2(np), v2(np), D(np), sc(2);
  cudaMemcpyAsync(u2.data(), du2, sizeof(double) * np, cudaMemcpyDeviceToHost, R.s);
  cudaMemcpyAsync(v2.data(), dv2, sizeof(double) * np, cudaMemcpyDeviceToHost, R.s);
  cudaMemcpyAsync(D.data(), dD, sizeof(double) * np, cudaMemcpyDeviceToHost, R.s);
  cudaMemcpyAsync(sc.data(), dSc, sizeof(double) * 2, cudaMemcpyDeviceToHost, R.s);
  NCGM_TRY(sync(R));
  out.u2.assign(M, 0.0);
  out.v2.assign(M, 0.0);
  out.Delta.assign(M, 0.0);
  for (int i = 0; i < M; ++i)
    if (visited[i]) {
      int pi = s2p[i];
      out.u2[i] = u2[pi];
      out.v2[i] = v2[pi];
      out.Delta[i] = D[pi];
    }
  out.qp.resize(M);
  for (int i = 0; i < M; ++i) out.qp[i] = S.e[i] * out.v2[i];
  out.lambda = sc[0];
  out.Epair = sc[1];
  return NCGM_OK;
}

int solvePairingBCS(Run &R) {
  const int A = R.cfg.A, Z = R.cfg.Z, N = A - Z;
  BCSRes nN = nullBCS(R.sp[0].e, N), nP = nullBCS(R.sp[1].e, Z);
  auto &sn = R.sp[0], &spp = R.sp[1];
  if (R.cfg.pairing_type == NCGM_PAIRING_NONE) {
    sn.bcs = nN;
    spp.bcs = nP;
  } else if (!R.have) {
    std::vector<double> tmp(1, 0.0);
    if (sn.par.active) {
      NCGM_TRY(bcsIter(R, sn, N, tmp, 0.5 * (sn.e[N - 1] + sn.e[N]), sn.bcs));
    } else sn.bcs = nN;
    if (spp.par.active) {
      NCGM_TRY(bcsIter(R, spp, Z, tmp, 0.5 * (spp.e[Z - 1] + spp.e[Z]), spp.bcs));
    } else spp.bcs = nP;
  } else {
    if (sn.par.active) {
      BCSRes o;
      NCGM_TRY(bcsIter(R, sn, N, sn.bcs.Delta, sn.bcs.lambda, o));
      sn.bcs = o;
    } else sn.bcs = nN;
    if (spp.par.active) {
      BCSRes o;
      NCGM_TRY(bcsIter(R, spp, Z, spp.bcs.Delta, spp.bcs.lambda, o));
      spp.bcs = o;
    } else spp.bcs = nP;
  }
  double a = 0, b = 0;
  for (double v : sn.bcs.v2) a += v;
  for (double v : spp.bcs.v2) b += v;
  if (std::isnan(a) || std::isnan(b)) {
    sn.bcs = nN;
    spp.bcs = nP;
  }
  return NCGM_OK;
}

// --- HFB (iteration_data.cpp:605-850) ---------------------------------------
// Everything runs on the device; the host keeps the Fermi-level search
// (which trial lambda comes next) and reads one scalar per trial.
int readScalar(Run &R, const double *d, double &v) {
  NCGM_CUDA(cudaMemcpyAsync(&v, d, sizeof(double), cudaMemcpyDeviceToHost,
                            R.s));
  return sync(R);
}

void nullHFB(Run &R, int M, int target, const std::vector<double> &e,
             HFBRes &h) {
  h.M = M;
  h.ready = true;
  h.lambda = e[target - 1];
  h.energy = 0.0;
  hfbNull(M, target, h.U, h.V, h.kappa, R.s);
}

int hfbSpecies(Run &R, Species &S, int target, HFBRes &out) {
  const HFBRes &prev = S.hfb;
  const int M = S.orb;
  HfbWork *w = R.hfbWork();
  if (!w) {
    setError("hfb: device allocation failed");
    return NCGM_ERR_NOMEM;
  }
  const double window = S.par.window, smooth = window / 10.0;
  auto fac = [&](double en, double lam) {
    double v = 1.0 / (1.0 + std::exp((en - lam - window) / smooth));
    v *= 1.0 / (1.0 + std::exp(-(en - lam + window) / smooth));
    return std::sqrt(v);
  };
  double lambda = prev.lambda;
  std::vector<double> ff(M);
  for (int i = 0; i < M; ++i) ff[i] = fac(S.e[i], lambda);
  int start = 0, end = M - 1;
  for (int i = 0; i < M; i += 2)
    if (ff[i] > R.cfg.pairing_threshold) {
      start = i;
      break;
    }
  for (int i = start; i < M; i += 2)
    if (ff[i] < R.cfg.pairing_threshold) {
      end = i;
      break;
    }
  const int nS = end - start + 1;
  // phi_rev = numericalTR(phi)
  timeReverse(S.X, S.TX, R.ns, M, R.N, true, R.s);
  // the window's levels and factors, then K_ab f_a f_b from the previous
  // kappa, kappa(r) and Delta_ab (one N x nS product and one weighted Gram;
  // exact-digit tensor-core forms in the tensor-core precision form)
  NCGM_CUDA(cudaMemcpyAsync(w->e, S.e.data() + start, sizeof(double) * nS,
                            cudaMemcpyHostToDevice, R.s));
  NCGM_CUDA(cudaMemcpyAsync(w->ff, ff.data() + start, sizeof(double) * nS,
                            cudaMemcpyHostToDevice, R.s));
  hfbKff(prev.kappa, M, start, nS, w->ff, w->Kff, R.s);
  const PairingGemm g = R.pairingGemm();
  const double2 *Phi0 = S.TX + (size_t)start * R.N;
  double *dkap = R.scratch;
  kappaFieldGemm(Phi0, R.N, nS, w->Kff, R.ns, dkap, w->gemmW, w->C, g, R.s);
  deltaMatrixGemm(Phi0, R.N, nS, w->ff, dkap, R.n, R.h, S.par.V0, w->Delta,
                  w->gemmW, w->G, g, R.s);
  hfbNorm2(w->Delta, nS, w->scal, R.s);
  double dn = 0;
  NCGM_TRY(readScalar(R, w->scal, dn));
  if (std::sqrt(dn) < 1e-3) {
    nullHFB(R, M, target, S.e, out);
    return NCGM_OK;
  }
  // Fermi level: N(lambda) - target = 0 inside [lambda - 1.7, lambda + 1.7]
  // to |N - target| < 1e-12, as the reference's bisection
  // (iteration_data.cpp:605-850). The first trial is the previous lambda;
  // once both signs are known the next trial is the Illinois regula falsi
  // point (Dowell and Jarratt 1971) instead of the midpoint, so a converged
  // HF run needs a few eigensolves per step instead of ~45.
  double bmin = lambda - 1.7, bmax = lambda + 1.7, cur = lambda;
  double flo = 0, fhi = 0;
  bool haveLo = false, haveHi = false;
  int side = 0; // Illinois: which end was kept last
  const int m2 = 2 * nS;
  for (int it = 0; it < 100; ++it) {
    hfbMatrix(w->e, w->Delta, nS, cur, w->H, R.s);
    heig(w->H, m2, m2, w->Hwork, w->Hv, w->eig, w->perm, w->status, R.s,
         false, w->heigScr, w->heigScrB);
    hfbExtract(w->Hv, nS, w->status, w->Uw, w->Vw, w->scal + 1, R.s);
    double num = 0;
    NCGM_TRY(readScalar(R, w->scal + 1, num));
    if (std::isnan(num)) {
      setError("hfb: dense eigensolver did not converge");
      return NCGM_ERR_EIG;
    }
    num += start;
    double diff = num - target;
    if (std::abs(diff) < 1e-12) break;
    if (diff > 0) {
      bmax = cur;
      fhi = diff;
      haveHi = true;
      if (side == 1) flo *= 0.5;
      side = 1;
    } else {
      bmin = cur;
      flo = diff;
      haveLo = true;
      if (side == -1) fhi *= 0.5;
      side = -1;
    }
    double next = (bmax + bmin) / 2.0;
    if (haveLo && haveHi && fhi != flo) {
      const double rf = bmin - flo * (bmax - bmin) / (fhi - flo);
      if (rf > bmin && rf < bmax) next = rf;
    }
    if (next == cur || bmax - bmin <= 1e-15 * std::max(1.0, std::abs(cur)))
      break;
    cur = next;
  }
  // amplitudes on the whole basis, kappa = U V^T and the pairing energy
  hfbAmplitudes(w->Uw, w->Vw, nS, start, M, out.U, out.V, out.kappa, R.s);
  hfbPairEnergy(w->Delta, out.kappa, M, start, nS, w->scal + 2, R.s);
  double pe = 0;
  NCGM_TRY(readScalar(R, w->scal + 2, pe));
  out.M = M;
  out.ready = true;
  out.lambda = cur;
  out.energy = pe;
  return NCGM_OK;
}

// Phi = phi * T (occupation transform), T on the device (M x M, col-major)
int occupyDev(Run &R, Species &S, const double2 *T) {
  const int M = S.orb;
  if (R.tc() && R.tcScratch())
    gemmVCExact(S.X, R.N, M, T, M, M, S.Phi, R.N, R.N, R.tcScratch(), R.s);
  else
    gemmVC(S.X, R.N, M, T, M, M, S.Phi, R.N, R.N, 0.0, R.s);
  return NCGM_OK;
}

// Phi = phi * T with T given on the host
int occupy(Run &R, Species &S, const std::vector<double2> &T) {
  const int M = S.orb;
  NCGM_CUDA(cudaMemcpyAsync(R.cplx, T.data(), sizeof(double2) * M * M,
                            cudaMemcpyHostToDevice, R.s));
  return occupyDev(R, S, R.cplx);
}

int occupiedOrbitals(Run &R, int q, bool bcsOcc, int &ncols,
                     const double2 *&Phi) {
  Species &S = R.sp[q];
  const int M = S.orb;
  const bool pairing = R.cfg.pairing_type != NCGM_PAIRING_NONE;
  // a run that ends before startHFBIter has BCS occupations only: the
  // output step then occupies with those (no HFB amplitudes exist yet)
  const bool hfbReady = S.hfb.ready;
  if (pairing && S.par.active && R.cfg.pairing_type == NCGM_PAIRING_HFB &&
      !hfbReady) {
    if (S.bcs.v2.size() != (size_t)M) {
      setError("hf: no pairing occupations to occupy the orbitals with");
      return NCGM_ERR_ARG;
    }
    bcsOcc = true;
  }
  if (bcsOcc || (pairing && S.par.active &&
                 R.cfg.pairing_type == NCGM_PAIRING_BCS)) {
    std::vector<double2> T((size_t)M * M, make_double2(0, 0));
    for (int c = 0; c < M; ++c)
      T[(size_t)c * M + c] = make_double2(std::sqrt(S.bcs.v2[c]), 0);
    NCGM_TRY(occupy(R, S, T));
    Phi = S.Phi;
    ncols = M;
    return NCGM_OK;
  }
  if (pairing && S.par.active && R.cfg.pairing_type == NCGM_PAIRING_HFB) {
    // natural orbitals of rho = V V^T (iteration_data.cpp:326-338)
    HfbWork *w = R.hfbWork();
    if (!w) {
      setError("hfb: device allocation failed");
      return NCGM_ERR_NOMEM;
    }
    hfbDensityMatrix(S.hfb.V, M, w->rho, R.s);
    heig(w->rho, M, M, w->Hwork, w->Wm, w->eig, w->perm, w->status, R.s,
         false, w->heigScr, w->heigScrB);
    hfbNatural(w->Wm, w->eig, M, w->T, R.s);
    int st = 0;
    NCGM_CUDA(cudaMemcpyAsync(&st, w->status, sizeof(int),
                              cudaMemcpyDeviceToHost, R.s));
    NCGM_TRY(occupyDev(R, S, w->T));
    NCGM_TRY(sync(R));
    if (st != 0) {
      setError("hfb: dense eigensolver did not converge (natural orbitals)");
      return NCGM_ERR_EIG;
    }
    Phi = S.Phi;
    ncols = M;
    return NCGM_OK;
  }
  // phi * nullOcc(particles) (iteration_data.cpp:290-294, 319-323): all
  // columns without pairing (the basis is the particle number); the first
  // `particles` columns when HFB pairing was switched off during the run,
  // as the reference's release build (no size check) computes that product
  const int particles = q == 0 ? R.cfg.A - R.cfg.Z : R.cfg.Z;
  Phi = S.X;
  ncols = std::min(M, std::max(particles, 0));
  return NCGM_OK;
}

int updateQuantities(Run &R, int iter) {
  const ncgm_hf_config &C = R.cfg;
  const double mu = C.density_mix;
  double t0 = now();
  bool bcsOcc = false;
  if (C.pairing_type == NCGM_PAIRING_HFB) {
    if (iter < C.start_hfb_iter) {
      NCGM_TRY(solvePairingBCS(R));
      bcsOcc = true;
    } else {
      if (iter == C.start_hfb_iter) {
        // kappa_ii+1 = -kappa_i+1i = sqrt(u2 v2) of the BCS pairs, V = 0
        if (!R.hfbWork()) {
          setError("hfb: device allocation failed");
          return NCGM_ERR_NOMEM;
        }
        for (int q = 0; q < 2; ++q) {
          Species &S = R.sp[q];
          const int M = S.orb;
          std::vector<double> kap((size_t)M * M, 0.0);
          for (int i = 0; i < M - 1; ++i)
            if (i % 2 == 0) {
              double uv = std::sqrt(S.bcs.u2[i] * S.bcs.v2[i]);
              kap[(size_t)(i + 1) * M + i] = uv;
              kap[(size_t)i * M + i + 1] = -1.0 * uv;
            }
          NCGM_CUDA(cudaMemcpyAsync(S.hfb.kappa, kap.data(),
                                    sizeof(double) * M * M,
                                    cudaMemcpyHostToDevice, R.s));
          NCGM_CUDA(cudaMemsetAsync(S.hfb.U, 0, sizeof(double) * M * M, R.s));
          NCGM_CUDA(cudaMemsetAsync(S.hfb.V, 0, sizeof(double) * M * M, R.s));
          S.hfb.M = M;
          S.hfb.ready = true;
          S.hfb.lambda = S.bcs.lambda;
        }
      }
      const int targets[2] = {C.A - C.Z, C.Z};
      for (int q = 0; q < 2; ++q) {
        Species &S = R.sp[q];
        if (!S.par.active) continue;
        HFBRes &nw = S.hfbNew;
        NCGM_TRY(hfbSpecies(R, S, targets[q], nw));
        if (std::isnan(nw.energy)) {
        } else if (std::abs(nw.energy) < 1e-12) {
          S.par.active = 0;
        } else {
          std::swap(S.hfb, S.hfbNew);
        }
      }
    }
  } else {
    NCGM_TRY(solvePairingBCS(R));
  }
  R.tPair += now() - t0;
  t0 = now();
  const bool first = !R.have;
  for (int q = 0; q < 2; ++q) {
    int nc = 0;
    const double2 *Phi = nullptr;
    NCGM_TRY(occupiedOrbitals(R, q, bcsOcc, nc, Phi));
    densities(Phi, R.N, nc, R.n, R.h, R.nrho, R.ntau, R.nJ9, R.ndivJ, R.s);
    mix(R.rho[q], R.nrho, mu, R.ns, first, R.s);
    mix(R.tau[q], R.ntau, mu, R.ns, first, R.s);
    mix(R.J9[q], R.nJ9, mu, 9 * R.ns, first, R.s);
    mix(R.divJ[q], R.ndivJ, mu, R.ns, first, R.s);
  }
  for (int q = 0; q < 2; ++q) gradLap(R.rho[q], R.n, R.h, R.g[q], R.lap[q], R.s);
  FieldsIn in;
  in.ns = R.ns;
  in.edf = C.edf;
  in.hbar2m = kHbar * kHbar / (2 * R.massCorr);
  in.spinOrbit = C.spin_orbit;
  in.useJ = C.use_j;
  in.rhoN = R.rho[0];
  in.rhoP = R.rho[1];
  in.tauN = R.tau[0];
  in.tauP = R.tau[1];
  in.lapN = R.lap[0];
  in.lapP = R.lap[1];
  in.divJN = R.divJ[0];
  in.divJP = R.divJ[1];
  in.gN = R.g[0];
  in.gP = R.g[1];
  in.JN = R.J9[0];
  in.JP = R.J9[1];
  FieldsOut out{R.f[0], R.f[1], R.gf[0], R.gf[1], R.U[0], R.U[1], R.W[0], R.W[1]};
  meanFields(in, out, R.s);
  // constraints (iteration_data.cpp:1031-1038,1079-1086)
  const int nc = (int)R.cons.size();
  if (iter > 0 && nc > 0) {
    std::vector<int> kinds(nc);
    for (int c = 0; c < nc; ++c) kinds[c] = R.cons[c].kind;
    const int nblk = 120;
    cudaMemcpyAsync(R.ismall, kinds.data(), sizeof(int) * nc,
                    cudaMemcpyHostToDevice, R.s);
    constraintQ<<<nblk, 256, 0, R.s>>>(R.rho[0], R.rho[1], R.n, R.a, R.h,
                                       R.ismall, nc, R.small);
    std::vector<double> part((size_t)nc * nblk);
    cudaMemcpyAsync(part.data(), R.small, sizeof(double) * nc * nblk,
                    cudaMemcpyDeviceToHost, R.s);
    NCGM_TRY(sync(R));
    std::vector<double> coef(nc);
    for (int c = 0; c < nc; ++c) {
      double Q = 0;
      for (int b = 0; b < nblk; ++b) Q += part[(size_t)c * nblk + b];
      Constraint &k = R.cons[c];
      double m;
      if (k.kind >= kMultipoleKind) {
        // MultipoleConstraint::getField (multipole_constraint.cpp:18-40):
        // the multiplier moves every iteration
        k.lambda += k.gamma * 2.0 * k.C * (Q - k.target);
        m = k.target - k.lambda / (2.0 * k.C);
        k.value = Q;
      } else if (k.first) {
        k.first = false;
        m = (k.kind == 6) ? k.target - k.lambda / (2.0 * k.C) : k.target;
      } else {
        if (k.kind > 2 || R.energyDiff < 5e-3)
          k.lambda += k.gamma * 2.0 * k.C * (Q - k.target);
        m = k.target - k.lambda / (2.0 * k.C);
        k.value = Q;
      }
      coef[c] = 2.0 * k.C * (Q - m);
    }
    cudaMemcpyAsync(R.small + nc * nblk, coef.data(), sizeof(double) * nc,
                    cudaMemcpyHostToDevice, R.s);
    constraintField<<<(unsigned)((R.ns + 255) / 256), 256, 0, R.s>>>(
        R.ismall, R.small + nc * nblk, nc, R.n, R.a, R.h, R.UConstr, R.U[0],
        R.U[1]);
  } else {
    zeroKernel<<<(unsigned)((R.ns + 255) / 256), 256, 0, R.s>>>(R.UConstr,
                                                                 R.ns);
  }
  NCGM_TRY(sync(R));
  R.tFields += now() - t0;
  if (C.use_coulomb) {
    t0 = now();
    PoissonArgs P;
    P.n = R.n;
    P.a = R.a;
    P.h = R.h;
    P.Z = C.Z;
    P.rhoP = R.rho[1];
    P.U = R.UCdir;
    P.UC = R.UCoul;
    P.warm = R.haveCoul;
    P.tol = 1e-13;
    P.work = R.poissonWork;
    int its = 0;
    int st = poissonSolve(P, R.s, &its);
    if (st != NCGM_OK) {
      setError("hf: Poisson solve failed");
      return st;
    }
    R.haveCoul = true;
    NCGM_TRY(sync(R));
    R.tPoisson += now() - t0;
  }
  R.have = true;
  return NCGM_OK;
}

double epair(Run &R, int q) {
  const ncgm_hf_config &C = R.cfg;
  if (C.pairing_type == NCGM_PAIRING_NONE) return 0.0;
  if (!R.sp[q].par.active) return 0.0;
  if (C.pairing_type == NCGM_PAIRING_HFB) return R.sp[q].hfb.energy;
  return R.sp[q].bcs.Epair;
}

// the energy integrals (iteration_data_integrals.cpp:95-262) of the run's
// densities, with tau, J and the Laplacian of rho given; copied to e
// (kEnergyTerms values) on the run's stream, not synchronised
void energyTerms(Run &R, double *const tau[2], double *const J9[2],
                 double *const lap[2], double *e) {
  const ncgm_hf_config &C = R.cfg;
  EnergyIn in;
  in.ns = R.ns;
  in.n = R.n;
  in.h = R.h;
  in.edf = C.edf;
  in.hbar2 = kHbar * kHbar;
  in.massCorr = R.massCorr;
  in.rhoN = R.rho[0];
  in.rhoP = R.rho[1];
  in.tauN = tau[0];
  in.tauP = tau[1];
  in.lapN = lap[0];
  in.lapP = lap[1];
  in.divJN = R.divJ[0];
  in.divJP = R.divJ[1];
  in.JN = J9[0];
  in.JP = J9[1];
  in.UCDir = C.use_coulomb ? R.UCdir : nullptr;
  energyIntegrals(in, R.scratch, R.energy, R.s);
  cudaMemcpyAsync(e, R.energy, sizeof(double) * kEnergyTerms,
                  cudaMemcpyDeviceToHost, R.s);
}

// kinetic + totalEnergyIntegral (main.cpp:300-301) from the terms
double integratedEnergy(Run &R, const double *e) {
  const ncgm_hf_config &C = R.cfg;
  const double cd = C.use_coulomb ? 0.5 * e[10] : 0.0;
  const double sl = C.use_coulomb ? e[11] : 0.0;
  const double total = e[0] + e[1] + e[2] + e[3] + e[4] + e[5] + cd +
                       epair(R, 0) + epair(R, 1) + sl + e[6] + e[7] + e[8] +
                       e[9];
  return total + e[12];
}

int energies(Run &R, double &Eint, double &EHF) {
  const ncgm_hf_config &C = R.cfg;
  double e[kEnergyTerms];
  energyTerms(R, R.tau, R.J9, R.lap, e);
  // constraint energies need int O rho with the current densities
  const int nc = (int)R.cons.size();
  std::vector<double> Qs(nc, 0.0);
  if (nc) {
    std::vector<int> kinds(nc);
    for (int c = 0; c < nc; ++c) kinds[c] = R.cons[c].kind;
    const int nblk = 120;
    cudaMemcpyAsync(R.ismall, kinds.data(), sizeof(int) * nc,
                    cudaMemcpyHostToDevice, R.s);
    constraintQ<<<nblk, 256, 0, R.s>>>(R.rho[0], R.rho[1], R.n, R.a, R.h,
                                       R.ismall, nc, R.small);
    std::vector<double> part((size_t)nc * nblk);
    cudaMemcpyAsync(part.data(), R.small, sizeof(double) * nc * nblk,
                    cudaMemcpyDeviceToHost, R.s);
    NCGM_TRY(sync(R));
    for (int c = 0; c < nc; ++c)
      for (int b = 0; b < nblk; ++b) Qs[c] += part[(size_t)c * nblk + b];
  }
  NCGM_TRY(sync(R));
  const double sl = C.use_coulomb ? e[11] : 0.0;
  const double kin = e[12];
  Eint = integratedEnergy(R, e);
  double ce = 0;
  for (int c = 0; c < nc; ++c) {
    const Constraint &k = R.cons[c];
    ce += k.C * std::pow(Qs[c] - k.target, 2) + k.lambda * (Qs[c] - k.target);
  }
  R.constraintEnergy = ce;
  double qN = 0, qP = 0;
  for (double v : R.sp[0].bcs.qp) qN += v;
  for (double v : R.sp[1].bcs.qp) qP += v;
  EHF = ce + 0.5 * (qN + qP + kin) + e[13] + sl / 3.0 + epair(R, 0) +
        epair(R, 1);
  return NCGM_OK;
}

// Output::shellsToFile's Lagrange-mesh recompute (output.cpp:252-256,
// iteration_data.cpp:346-382): tau, J and the Laplacian of rho from the
// final occupied orbitals with Lagrange-mesh derivatives, rho and div J as
// they are, then kinetic + totalEnergyIntegral ("EintLag").
// With out, the recomputed tau and the Lagrange-mesh gradient of rho (the
// fields the reference's output step writes after the recompute) are copied
// to it as well.
int lagrangeEnergy(Run &R, double &E, ncgm_hf_outputs *out) {
  const size_t ns = R.ns;
  double *w = R.alloc<double>(28 * ns);
  void *scr = R.alloc<char>(lagrangeScratchBytes(R.n));
  if (!w || !scr) {
    setError("hf: device allocation for the Lagrange recompute failed");
    return NCGM_ERR_NOMEM;
  }
  double *tau[2] = {w, w + ns}, *J9[2] = {w + 2 * ns, w + 11 * ns},
         *lap[2] = {w + 20 * ns, w + 21 * ns},
         *g3[2] = {w + 22 * ns, w + 25 * ns};
  for (int q = 0; q < 2; ++q) {
    int nc = 0;
    const double2 *Phi = nullptr;
    NCGM_TRY(occupiedOrbitals(R, q, false, nc, Phi));
    NCGM_TRY(lagrangeDensities(Phi, R.N, nc, R.n, R.h, R.rho[q], tau[q],
                               J9[q], lap[q], out ? g3[q] : nullptr, scr,
                               R.s));
  }
  double e[kEnergyTerms];
  energyTerms(R, tau, J9, lap, e);
  NCGM_TRY(sync(R));
  E = integratedEnergy(R, e);
  if (out) {
    double *const dt[2] = {out->tau_n, out->tau_p};
    double *const dg[2] = {out->grad_rho_n, out->grad_rho_p};
    for (int q = 0; q < 2; ++q) {
      if (dt[q])
        NCGM_CUDA(cudaMemcpyAsync(dt[q], tau[q], ns * sizeof(double),
                                  cudaMemcpyDefault, R.s));
      if (dg[q])
        NCGM_CUDA(cudaMemcpyAsync(dg[q], g3[q], 3 * ns * sizeof(double),
                                  cudaMemcpyDefault, R.s));
    }
    NCGM_TRY(sync(R));
  }
  return NCGM_OK;
}

// the output step's energy table (output.cpp:205-236, printed before the
// Lagrange recompute), the final orbitals and the mean fields
int fillOutputs(Run &R, ncgm_hf_outputs *out) {
  const ncgm_hf_config &C = R.cfg;
  double e[kEnergyTerms];
  energyTerms(R, R.tau, R.J9, R.lap, e);
  NCGM_TRY(sync(R));
  double *t = out->terms;
  t[0] = e[12];
  t[1] = e[0];
  t[2] = e[1];
  t[3] = e[2];
  t[4] = e[3];
  t[5] = e[4];
  t[6] = e[5];
  t[7] = e[8];
  t[8] = e[9];
  t[9] = e[6];
  t[10] = e[7];
  t[11] = C.use_coulomb ? 0.5 * e[10] : 0.0;
  t[12] = epair(R, 0);
  t[13] = epair(R, 1);
  t[14] = C.use_coulomb ? e[11] : 0.0;
  t[15] = e[13];
  out->constraints_energy = R.constraintEnergy;
  double *const orb[2] = {out->orbitals_n, out->orbitals_p};
  double *const U[2] = {out->U_n, out->U_p};
  for (int q = 0; q < 2; ++q) {
    if (orb[q])
      NCGM_CUDA(cudaMemcpyAsync(orb[q], R.sp[q].X,
                                R.N * R.sp[q].orb * sizeof(double2),
                                cudaMemcpyDefault, R.s));
    if (U[q])
      NCGM_CUDA(cudaMemcpyAsync(U[q], R.U[q], R.ns * sizeof(double),
                                cudaMemcpyDefault, R.s));
  }
  return sync(R);
}

// Wavefunction::TROrder (wavefunction.cpp:581-635)
int trOrder(Run &R, Species &S, double2 *X) {
  const int M = S.orb;
  timeReverse(X, S.TX, R.ns, M, R.N, false, R.s);
  std::vector<double2> ord;
  NCGM_TRY(hostGram(R, X, M, S.TX, M, ord));
  std::vector<bool> used(M, false);
  std::vector<int> order;
  int slot = 0;
  bool fail = false;
  for (int i = 0; i < M && !fail; ++i) {
    if (used[i]) continue;
    order.push_back(i);
    used[i] = true;
    int best = -1;
    double mx = -1.0;
    for (int j = 0; j < M; ++j) {
      if (used[j]) continue;
      double2 z = ord[(size_t)j * M + i];
      double ov = std::sqrt(z.x * z.x + z.y * z.y);
      if (ov > mx) {
        mx = ov;
        best = j;
      }
    }
    if (best < 0) {
      fail = true;
      break;
    }
    order.push_back(best);
    used[best] = true;
    slot += 2;
    if (slot >= M) break;
  }
  if (fail || (int)order.size() != M) return NCGM_OK; // keep psi as is
  // gather columns in `order` (through TX as staging)
  for (int c = 0; c < M; ++c)
    cudaMemcpyAsync(S.TX + (size_t)c * R.N, X + (size_t)order[c] * R.N,
                    sizeof(double2) * R.N, cudaMemcpyDeviceToDevice, R.s);
  cudaMemcpyAsync(X, S.TX, sizeof(double2) * R.N * M, cudaMemcpyDeviceToDevice,
                  R.s);
  return sync(R);
}

// P = Xnew - Xold (Xold^H Xnew), columns normalised (main.cpp:267-282)
int conjDir(Run &R, Species &S) {
  const int M = S.orb;
  std::vector<double2> tmp;
  NCGM_TRY(hostGram(R, S.X, M, S.Xn, M, tmp));
  for (auto &z : tmp) z = make_double2(-z.x, -z.y);
  cudaMemcpyAsync(R.cplx, tmp.data(), sizeof(double2) * M * M,
                  cudaMemcpyHostToDevice, R.s);
  cudaMemcpyAsync(S.CD, S.Xn, sizeof(double2) * R.N * M,
                  cudaMemcpyDeviceToDevice, R.s);
  if (R.tc() && R.tcScratch())
    gemmVCExact(S.X, R.N, M, R.cplx, M, M, S.CD, R.N, R.N, R.tcScratch(),
                R.s, true);
  else
    gemmVC(S.X, R.N, M, R.cplx, M, M, S.CD, R.N, R.N, 1.0, R.s);
  normalizeEuclid(S.CD, R.N, R.N, M, R.small, R.s);
  S.cdCols = M;
  return sync(R);
}

void quadDef(Run &R, double &beta, double &gamma) {
  // output only: beta2 and gamma from the total density
  const int nblk = 120;
  int kinds[2] = {6, 3};
  cudaMemcpyAsync(R.ismall, kinds, sizeof(kinds), cudaMemcpyHostToDevice,
                  R.s);
  cudaStreamSynchronize(R.s); // kinds is a stack array
  constraintQ<<<nblk, 256, 0, R.s>>>(R.rho[0], R.rho[1], R.n, R.a, R.h,
                                     R.ismall, 2, R.small);
  std::vector<double> part(2 * nblk);
  cudaMemcpyAsync(part.data(), R.small, sizeof(double) * 2 * nblk,
                  cudaMemcpyDeviceToHost, R.s);
  cudaStreamSynchronize(R.s);
  double q20 = 0, x2y2 = 0;
  for (int b = 0; b < nblk; ++b) {
    q20 += part[b];
    x2y2 += part[nblk + b];
  }
  // a20 = sqrt(5/16pi) (2z^2-x^2-y^2) = q20 * sqrt(5/16pi)/(0.25 sqrt(5/pi))
  double a20 = q20 * std::sqrt(5.0 / (16.0 * M_PI)) / (0.25 * std::sqrt(5 / M_PI));
  double a22 = x2y2 * std::sqrt(15.0 / (32.0 * M_PI));
  double Rr = 1.2 * std::pow(R.cfg.A, 1.0 / 3.0);
  gamma = std::atan2(std::sqrt(2) * a22, a20);
  beta = 4 * M_PI * a20 / (3 * R.cfg.A * Rr * Rr);
}

std::vector<int4> hoOrbitals(int nev) {
  std::vector<int4> orbs;
  for (int Nsh = 0; (int)orbs.size() < nev; ++Nsh)
    for (int nr = 0; nr <= Nsh / 2 && (int)orbs.size() < nev; ++nr) {
      int l = Nsh - 2 * nr;
      int jp = 2 * l + 1;
      for (int m = 1; m <= jp && (int)orbs.size() < nev; m += 2) {
        orbs.push_back(make_int4(nr, l, jp, m));
        if ((int)orbs.size() < nev) orbs.push_back(make_int4(nr, l, jp, -m));
      }
      if (l > 0) {
        int jm = 2 * l - 1;
        for (int m = 1; m <= jm && (int)orbs.size() < nev; m += 2) {
          orbs.push_back(make_int4(nr, l, jm, m));
          if ((int)orbs.size() < nev) orbs.push_back(make_int4(nr, l, jm, -m));
        }
      }
    }
  return orbs;
}

// main.cpp:201-207: at HF iteration 1 each "constraints" entry becomes a
// MultipoleConstraint. Its constructor (multipole_constraint.cpp:7-16)
// evaluates C (Q - target)^2 with C = 1 on the current densities and sets
// C = 0.01 / that value.
int addMultipoles(Run &R) {
  const ncgm_hf_config &C = R.cfg;
  const int nm = std::min(C.n_multipole, NCGM_MAX_MULTIPOLE);
  std::vector<int> kinds(nm);
  for (int i = 0; i < nm; ++i) {
    if (C.mp_l[i] < 0 || C.mp_l[i] > 9 || std::abs(C.mp_m[i]) > C.mp_l[i]) {
      setError("hf: multipole constraint needs 0 <= l <= 9, |m| <= l");
      return NCGM_ERR_ARG;
    }
    kinds[i] = kMultipoleKind + 100 * C.mp_l[i] + (C.mp_m[i] + 50);
  }
  const int nblk = 120;
  cudaMemcpyAsync(R.ismall, kinds.data(), sizeof(int) * nm,
                  cudaMemcpyHostToDevice, R.s);
  constraintQ<<<nblk, 256, 0, R.s>>>(R.rho[0], R.rho[1], R.n, R.a, R.h,
                                     R.ismall, nm, R.small);
  std::vector<double> part((size_t)nm * nblk);
  cudaMemcpyAsync(part.data(), R.small, sizeof(double) * nm * nblk,
                  cudaMemcpyDeviceToHost, R.s);
  NCGM_TRY(sync(R));
  for (int i = 0; i < nm; ++i) {
    double Q = 0;
    for (int b = 0; b < nblk; ++b) Q += part[(size_t)i * nblk + b];
    Constraint c;
    c.kind = kinds[i];
    c.target = C.mp_target[i];
    c.gamma = 0.3;
    c.C = 0.01 / std::pow(Q - c.target, 2);
    c.first = false;
    R.cons.push_back(c);
  }
  return NCGM_OK;
}

// The run's lattice state, contexts and constraint list for cfg
// (IterationData's constructor, iteration_data.cpp:9-151, and the constraint
// set-up of main.cpp:164-185). twoContexts: a second context for the protons'
// concurrent eigenproblem when the species differ (unless NCGM_HF_SERIAL=1).
int setupRun(Run &R, const ncgm_hf_config &cfg, bool twoContexts) {
  R.cfg = cfg;
  R.n = cfg.n;
  R.a = cfg.box_size / 2.0;
  R.h = 2.0 * R.a / (R.n - 1);
  R.ns = (size_t)R.n * R.n * R.n;
  R.N = 2 * R.ns;
  const int A = cfg.A, Z = cfg.Z, N = A - Z;
  const bool pairing = cfg.pairing_type != NCGM_PAIRING_NONE;
  const int orbN = pairing && cfg.pair_n.active ? cfg.pair_n.basis_size : N;
  const int orbP = pairing && cfg.pair_p.active ? cfg.pair_p.basis_size : Z;
  const int mx = std::max(orbN, orbP);
  NCGM_TRY(ncgm_create(&R.ctx, R.n, R.a, 4 * mx + 8, 0));
  R.s = R.ctx->stream;
  if (cfg.hf_gcg.precond == NCGM_PRECOND_LEARNED && !cfg.lp) {
    setError("hf: learned preconditioner requested without a network");
    return NCGM_ERR_ARG;
  }
  R.ctx->lp = cfg.lp;
  // Both species need their own eigenproblem when the Coulomb field or N != Z
  // makes them differ. Each HF iteration then solves them concurrently, on
  // two contexts and host threads; NCGM_HF_SERIAL=1 solves them one after
  // the other on one context. Either way each species runs the same kernels
  // on the same inputs, so the results are the same.
  const bool twoSpecies = twoContexts && (cfg.use_coulomb || N != Z);
  {
    const char *ser = std::getenv("NCGM_HF_SERIAL");
    if (twoSpecies && !(ser && ser[0] == '1')) {
      NCGM_TRY(ncgm_create(&R.ctxP, R.n, R.a, 4 * mx + 8, 0));
      R.ctxP->lp = cfg.lp;
      NCGM_CUDA(cudaEventCreateWithFlags(&R.evFields, cudaEventDisableTiming));
      NCGM_CUDA(
          cudaEventCreateWithFlags(&R.evProtons, cudaEventDisableTiming));
    }
  }
  R.sp[0].orb = orbN;
  R.sp[1].orb = orbP;
  R.sp[0].par = cfg.pair_n;
  R.sp[1].par = cfg.pair_p;
  if (!pairing) R.sp[0].par.active = R.sp[1].par.active = 0;
  for (int q = 0; q < 2; ++q) {
    R.rho[q] = R.alloc<double>(R.ns);
    R.tau[q] = R.alloc<double>(R.ns);
    R.J9[q] = R.alloc<double>(9 * R.ns);
    R.divJ[q] = R.alloc<double>(R.ns);
    R.g[q] = R.alloc<double>(3 * R.ns);
    R.lap[q] = R.alloc<double>(R.ns);
    R.f[q] = R.alloc<double>(R.ns);
    R.gf[q] = R.alloc<double>(3 * R.ns);
    R.U[q] = R.alloc<double>(R.ns);
    R.W[q] = R.alloc<double>(3 * R.ns);
    Species &S = R.sp[q];
    S.X = R.alloc<double2>(R.N * mx);
    S.Xn = R.alloc<double2>(R.N * mx);
    S.CD = R.alloc<double2>(R.N * mx);
    S.Phi = R.alloc<double2>(R.N * mx);
    S.TX = R.alloc<double2>(R.N * mx);
    if (!S.TX) {
      setError("hf: device allocation failed");
      return NCGM_ERR_NOMEM;
    }
  }
  R.UCdir = R.alloc<double>(R.ns);
  R.UCoul = R.alloc<double>(R.ns);
  R.UConstr = R.alloc<double>(R.ns);
  R.nrho = R.alloc<double>(R.ns);
  R.ntau = R.alloc<double>(R.ns);
  R.nJ9 = R.alloc<double>(9 * R.ns);
  R.ndivJ = R.alloc<double>(R.ns);
  R.scratch = R.alloc<double>(std::max<size_t>(R.ns, 64 * 1024));
  R.poissonWork = R.alloc<double>(poissonWorkDoubles(R.n));
  R.energy = R.alloc<double>(64);
  const size_t sm = std::max<size_t>((size_t)4 * mx * mx + 64, 3 * 4 * 512 * 512);
  R.cplx = R.alloc<double2>(sm);
  R.small = R.alloc<double>(std::max<size_t>(sm, 16 * 1024));
  R.ismall = R.alloc<int>(16 * 1024);
  if (!R.ismall) {
    setError("hf: device allocation failed");
    return NCGM_ERR_NOMEM;
  }
  R.massCorr = cfg.com_corr ? kMass * ((double)A) / ((double)(A - 1)) : kMass;
  if (cfg.constrain_com)
    for (int k = 0; k < 3; ++k) R.cons.push_back(makeConstraint(k, 0.0));
  if (cfg.curve_mode) {
    for (int k = 0; k < 3; ++k) R.cons.push_back(makeConstraint(k, 0.0));
    R.cons.push_back(makeConstraint(3, 0.0));
    R.cons.push_back(makeConstraint(4, 0.0));
    R.cons.push_back(makeConstraint(5, 0.0));
    R.cons.push_back(makeConstraint(6, cfg.mu20));
  }
  return NCGM_OK;
}

int hfRun(const ncgm_hf_config &cfg, ncgm_hf_result &res, double *spe_n,
          double *spe_p, double *rho_n, double *rho_p, double *energiesOut,
          ncgm_hf_outputs *out) {
  const double tStart = now();
  Run R;
  NCGM_TRY(setupRun(R, cfg, true));
  const int A = cfg.A, Z = cfg.Z, N = A - Z;
  const bool pairing = cfg.pairing_type != NCGM_PAIRING_NONE;
  const int orbN = R.sp[0].orb, orbP = R.sp[1].orb;
  const int mx = std::max(orbN, orbP);
  const bool twoSpecies = cfg.use_coulomb || N != Z;

  // --- Woods-Saxon guess (main.cpp:72-111) ---------------------------------
  double t0 = now();
  NCGM_TRY(ncgm_set_woods_saxon(R.ctx, 0, A, Z, cfg.ws_V0, cfg.ws_r0,
                                cfg.ws_diff, cfg.ws_kappa, cfg.initial_beta,
                                cfg.beta3, cfg.wsso_V0, cfg.spin_orbit));
  {
    std::vector<int4> orbs = hoOrbitals(mx);
    int4 *dOrbs = reinterpret_cast<int4 *>(R.ismall);
    cudaMemcpyAsync(dOrbs, orbs.data(), sizeof(int4) * mx,
                    cudaMemcpyHostToDevice, R.s);
    const double nucR = std::pow(A, 0.3333333) * 1.20;
    hoGuess(dOrbs, mx, R.n, R.a, R.h, nucR, R.sp[1].Phi, R.N, R.small, R.s);
    NCGM_TRY(sync(R));
    std::vector<double> lam(mx);
    NCGM_TRY(gcgRun(R.ctx, 0, R.sp[1].Phi, mx, nullptr, 0, mx, cfg.ws_gcg,
                    R.sp[0].Phi, lam.data(), nullptr));
    // neutrons/protons from the same eigenpairs (main.cpp:100-108)
    for (int q = 0; q < 2; ++q) {
      Species &S = R.sp[q];
      const int cols = (q == 0) ? (N >= Z ? mx : orbN) : (N >= Z ? orbP : mx);
      cudaMemcpyAsync(S.X, R.sp[0].Phi, sizeof(double2) * R.N * cols,
                      cudaMemcpyDeviceToDevice, R.s);
      S.e.assign(lam.begin(), lam.begin() + cols);
      normalizeColumns(S.X, R.N, cols, R.n, R.h, R.small, R.s);
    }
    NCGM_TRY(sync(R));
  }
  R.tGcg += now() - t0;

  double Eint = 0.0, EHF = 0.0, lastdE = 0.0;
  int it = 0;
  bool conv = false;
  ncgm_gcg_params hp = cfg.hf_gcg;
  for (it = 0; it < cfg.max_iterations; ++it) {
    if (it == 1 && cfg.n_multipole > 0) NCGM_TRY(addMultipoles(R));
    NCGM_TRY(updateQuantities(R, it));
    NCGM_TRY(phaseSync(R, "densities, fields and pairing", it));
    NCGM_TRY(buildCoefficients(R.ctx, 0, R.f[0], R.gf[0], R.U[0],
                               cfg.spin_orbit ? R.W[0] : nullptr, nullptr));
    // the proton context's stream waits for this iteration's fields and
    // orbitals, which were made on the main stream
    ncgm_ctx *const ctxP = R.ctxP ? R.ctxP : R.ctx;
    if (R.ctxP) {
      NCGM_CUDA(cudaEventRecord(R.evFields, R.s));
      NCGM_CUDA(cudaStreamWaitEvent(R.ctxP->stream, R.evFields, 0));
    }
    NCGM_TRY(buildCoefficients(ctxP, 1, R.f[1], R.gf[1], R.U[1],
                               cfg.spin_orbit ? R.W[1] : nullptr,
                               cfg.use_coulomb ? R.UCoul : nullptr));
    t0 = now();
    std::vector<double> lamN(orbN), lamP(orbP);
    Species &Sn = R.sp[0], &Sp = R.sp[1];
    if (twoSpecies && R.ctxP) {
      int stP = NCGM_OK;
      std::string errP;
      // exceptions stay on their own thread: the proton thread turns them
      // into a status, and the main thread joins before rethrowing
      std::thread protons([&] {
        try {
          cudaSetDevice(R.ctx->device);
          stP = gcgRun(R.ctxP, 1, Sp.X, orbP, Sp.cdCols ? Sp.CD : nullptr,
                       Sp.cdCols, orbP, hp, Sp.Xn, lamP.data(), nullptr);
          if (stP != NCGM_OK) errP = ncgm_last_error();
        } catch (const std::exception &e) {
          stP = NCGM_ERR_ARG;
          errP = std::string("hf (protons): ") + e.what();
        }
      });
      int stN = NCGM_OK;
      try {
        stN = gcgRun(R.ctx, 0, Sn.X, orbN, Sn.cdCols ? Sn.CD : nullptr,
                     Sn.cdCols, orbN, hp, Sn.Xn, lamN.data(), nullptr);
      } catch (...) {
        protons.join();
        throw;
      }
      protons.join();
      if (stN != NCGM_OK) return stN;
      if (stP != NCGM_OK) {
        setError(errP);
        return stP;
      }
      NCGM_CUDA(cudaEventRecord(R.evProtons, R.ctxP->stream));
      NCGM_CUDA(cudaStreamWaitEvent(R.s, R.evProtons, 0));
    } else if (twoSpecies) {
      NCGM_TRY(gcgRun(R.ctx, 0, Sn.X, orbN, Sn.cdCols ? Sn.CD : nullptr,
                      Sn.cdCols, orbN, hp, Sn.Xn, lamN.data(), nullptr));
      NCGM_TRY(gcgRun(R.ctx, 1, Sp.X, orbP, Sp.cdCols ? Sp.CD : nullptr,
                      Sp.cdCols, orbP, hp, Sp.Xn, lamP.data(), nullptr));
    } else {
      NCGM_TRY(gcgRun(R.ctx, 0, Sn.X, orbN, Sn.cdCols ? Sn.CD : nullptr,
                      Sn.cdCols, orbN, hp, Sn.Xn, lamN.data(), nullptr));
      cudaMemcpyAsync(Sp.Xn, Sn.Xn, sizeof(double2) * R.N * orbP,
                      cudaMemcpyDeviceToDevice, R.s);
      std::copy(lamN.begin(), lamN.begin() + orbP, lamP.begin());
    }
    R.tGcg += now() - t0;
    NCGM_TRY(phaseSync(R, "eigensolver", it));
    // training pairs for the learned preconditioner: the new eigenpairs on
    // this iteration's Hamiltonians, with the shift the next GCG call uses
    if (cfg.lp && cfg.lp_collect_every > 0 && it % cfg.lp_collect_every == 0) {
      const double shN = (lamN.back() - 100.0 * lamN[0]) / 99.0;
      const double shP = (lamP.back() - 100.0 * lamP[0]) / 99.0;
      NCGM_TRY(ncgm_lp_collect(cfg.lp, R.ctx, 0,
                               reinterpret_cast<const double *>(Sn.Xn), orbN,
                               lamN.data(), shN, 2000, 1e-10));
      NCGM_TRY(ncgm_lp_collect(cfg.lp, ctxP, 1,
                               reinterpret_cast<const double *>(Sp.Xn), orbP,
                               lamP.data(), shP, 2000, 1e-10));
    }
    double maxd = 0;
    for (int i = 0; i < orbN; ++i) maxd = std::max(maxd, std::abs(lamN[i] - Sn.e[i]));
    for (int i = 0; i < orbP; ++i) maxd = std::max(maxd, std::abs(lamP[i] - Sp.e[i]));
    normalizeColumns(Sn.Xn, R.N, orbN, R.n, R.h, R.small, R.s);
    normalizeColumns(Sp.Xn, R.N, orbP, R.n, R.h, R.small, R.s);
    if (pairing) {
      NCGM_TRY(trOrder(R, Sn, Sn.Xn));
      NCGM_TRY(trOrder(R, Sp, Sp.Xn));
    }
    NCGM_TRY(phaseSync(R, "normalisation and time-reversal order", it));
    if (it > 0) {
      NCGM_TRY(conjDir(R, Sn));
      NCGM_TRY(conjDir(R, Sp));
    }
    NCGM_TRY(phaseSync(R, "conjugate directions", it));
    std::swap(Sn.X, Sn.Xn);
    std::swap(Sp.X, Sp.Xn);
    Sn.e = lamN;
    Sp.e = lamP;
    double nE = 0, nH = 0;
    NCGM_TRY(energies(R, nE, nH));
    NCGM_TRY(phaseSync(R, "energies", it));
    bool cconv = true;
    for (auto &c : R.cons)
      if (c.error() != 0.0) cconv = cconv && (c.error() < cfg.constraints_tol);
    if (energiesOut) {
      energiesOut[2 * it] = nE;
      energiesOut[2 * it + 1] = nH;
    }
    lastdE = std::abs(nE - Eint);
    if (!std::isfinite(nE) || !std::isfinite(nH)) {
      setError("hf: non-finite energy");
      return NCGM_ERR_NAN;
    }
    const bool speOk = cfg.spe_tol <= 0 || maxd < cfg.spe_tol;
    if (std::abs(nE - Eint) < cfg.energy_tol &&
        std::abs(nH - EHF) < cfg.energy_tol && cconv && speOk) {
      Eint = nE;
      EHF = nH;
      conv = true;
      ++it;
      break;
    }
    R.energyDiff = std::abs(nH - EHF);
    Eint = nE;
    EHF = nH;
  }
  if (out) NCGM_TRY(fillOutputs(R, out));
  NCGM_TRY(lagrangeEnergy(R, res.E_int_lagrange, out));
  res.iterations = it;
  res.converged = conv;
  res.E_int = Eint;
  res.E_HF = EHF;
  res.E_pair_n = epair(R, 0);
  res.E_pair_p = epair(R, 1);
  res.lambda_n = cfg.pairing_type == NCGM_PAIRING_HFB ? R.sp[0].hfb.lambda
                                                       : R.sp[0].bcs.lambda;
  res.lambda_p = cfg.pairing_type == NCGM_PAIRING_HFB ? R.sp[1].hfb.lambda
                                                       : R.sp[1].bcs.lambda;
  quadDef(R, res.beta, res.gamma);
  res.last_dE = lastdE;
  res.t_gcg_s = R.tGcg;
  res.t_fields_s = R.tFields;
  res.t_poisson_s = R.tPoisson;
  res.t_pairing_s = R.tPair;
  if (spe_n) std::copy(R.sp[0].e.begin(), R.sp[0].e.end(), spe_n);
  if (spe_p) std::copy(R.sp[1].e.begin(), R.sp[1].e.end(), spe_p);
  if (rho_n)
    NCGM_CUDA(cudaMemcpyAsync(rho_n, R.rho[0], sizeof(double) * R.ns,
                              cudaMemcpyDeviceToHost, R.s));
  if (rho_p)
    NCGM_CUDA(cudaMemcpyAsync(rho_p, R.rho[1], sizeof(double) * R.ns,
                              cudaMemcpyDeviceToHost, R.s));
  NCGM_TRY(sync(R));
  res.wall_s = now() - tStart;
  return NCGM_OK;
}

} // namespace
} // namespace ncgm

using namespace ncgm;

extern "C" int ncgm_hf_run(const ncgm_hf_config *cfg, ncgm_hf_result *res,
                           double *spe_n, double *spe_p, double *rho_n,
                           double *rho_p, double *energies) {
  try {
    if (!cfg || !res || cfg->n < 4 || cfg->box_size <= 0 || cfg->A < 2 ||
        cfg->Z < 0 || cfg->Z > cfg->A || cfg->max_iterations < 0) {
      setError("ncgm_hf_run: bad configuration");
      return NCGM_ERR_ARG;
    }
    std::memset(res, 0, sizeof(*res));
    return hfRun(*cfg, *res, spe_n, spe_p, rho_n, rho_p, energies, nullptr);
  } catch (const std::exception &e) {
    setError(e.what());
    return NCGM_ERR_ARG;
  }
}

extern "C" int ncgm_hf_run_ex(const ncgm_hf_config *cfg, ncgm_hf_result *res,
                              double *spe_n, double *spe_p, double *rho_n,
                              double *rho_p, double *energies,
                              ncgm_hf_outputs *out) {
  try {
    if (!cfg || !res || !out || cfg->n < 4 || cfg->box_size <= 0 ||
        cfg->A < 2 || cfg->Z < 0 || cfg->Z > cfg->A ||
        cfg->max_iterations < 0) {
      setError("ncgm_hf_run_ex: bad configuration");
      return NCGM_ERR_ARG;
    }
    std::memset(res, 0, sizeof(*res));
    std::memset(out->terms, 0, sizeof(out->terms));
    return hfRun(*cfg, *res, spe_n, spe_p, rho_n, rho_p, energies, out);
  } catch (const std::exception &e) {
    setError(e.what());
    return NCGM_ERR_ARG;
  }
}

extern "C" int ncgm_shell_observables(ncgm_ctx *ctx, const double *Psi,
                                      int ncols, double *obs) {
  try {
    if (!ctx || !Psi || ncols < 1 || !obs) {
      setError("ncgm_shell_observables: bad argument");
      return NCGM_ERR_ARG;
    }
    const size_t N = ctx->N;
    double2 *dX = static_cast<double2 *>(ctx->buf(26, N * ncols * sizeof(double2)));
    void *scr = ctx->buf(27, shellScratchBytes(ctx->n));
    if (!dX || !scr) return NCGM_ERR_NOMEM;
    NCGM_CUDA(cudaMemcpyAsync(dX, Psi, N * ncols * sizeof(double2),
                              cudaMemcpyDefault, ctx->stream));
    return shellObservables(dX, N, ncols, ctx->n, ctx->a, scr, obs,
                            ctx->stream);
  } catch (const std::exception &e) {
    setError(e.what());
    return NCGM_ERR_ARG;
  }
}

extern "C" int ncgm_densities(ncgm_ctx *ctx, const double *Phi, int ncols,
                              double *rho, double *tau, double *J9,
                              double *divJ) {
  try {
    if (!ctx || !Phi || ncols < 1 || !rho || !tau || !J9 || !divJ) {
      setError("ncgm_densities: bad argument");
      return NCGM_ERR_ARG;
    }
    const size_t N = ctx->N, ns = ctx->ns;
    double2 *dX = static_cast<double2 *>(ctx->buf(23, N * ncols * sizeof(double2)));
    double *d = static_cast<double *>(ctx->buf(24, 12 * ns * sizeof(double)));
    if (!dX || !d) return NCGM_ERR_NOMEM;
    NCGM_CUDA(cudaMemcpyAsync(dX, Phi, N * ncols * sizeof(double2),
                              cudaMemcpyDefault, ctx->stream));
    densities(dX, N, ncols, ctx->n, ctx->h, d, d + ns, d + 2 * ns, d + 11 * ns,
              ctx->stream);
    NCGM_CUDA(cudaMemcpyAsync(rho, d, ns * sizeof(double), cudaMemcpyDefault,
                              ctx->stream));
    NCGM_CUDA(cudaMemcpyAsync(tau, d + ns, ns * sizeof(double),
                              cudaMemcpyDefault, ctx->stream));
    NCGM_CUDA(cudaMemcpyAsync(J9, d + 2 * ns, 9 * ns * sizeof(double),
                              cudaMemcpyDefault, ctx->stream));
    NCGM_CUDA(cudaMemcpyAsync(divJ, d + 11 * ns, ns * sizeof(double),
                              cudaMemcpyDefault, ctx->stream));
    NCGM_CUDA(cudaStreamSynchronize(ctx->stream));
    return NCGM_OK;
  } catch (const std::exception &e) {
    setError(e.what());
    return NCGM_ERR_ARG;
  }
}

extern "C" int ncgm_lagrange_densities(ncgm_ctx *ctx, const double *Phi,
                                       int ncols, const double *rho,
                                       double *tau, double *J9, double *lap) {
  try {
    if (!ctx || !Phi || ncols < 1 || !tau || !J9 || (!rho != !lap)) {
      setError("ncgm_lagrange_densities: bad argument");
      return NCGM_ERR_ARG;
    }
    const size_t N = ctx->N, ns = ctx->ns;
    double2 *dX = static_cast<double2 *>(ctx->buf(26, N * ncols * sizeof(double2)));
    double *d = static_cast<double *>(ctx->buf(
        27, 12 * ns * sizeof(double) + lagrangeScratchBytes(ctx->n)));
    if (!dX || !d) return NCGM_ERR_NOMEM;
    NCGM_CUDA(cudaMemcpyAsync(dX, Phi, N * ncols * sizeof(double2),
                              cudaMemcpyDefault, ctx->stream));
    if (rho)
      NCGM_CUDA(cudaMemcpyAsync(d + 11 * ns, rho, ns * sizeof(double),
                                cudaMemcpyDefault, ctx->stream));
    NCGM_TRY(lagrangeDensities(dX, N, ncols, ctx->n, ctx->h,
                               rho ? d + 11 * ns : nullptr, d, d + ns,
                               rho ? d + 10 * ns : nullptr, nullptr,
                               d + 12 * ns, ctx->stream));
    NCGM_CUDA(cudaMemcpyAsync(tau, d, ns * sizeof(double), cudaMemcpyDefault,
                              ctx->stream));
    NCGM_CUDA(cudaMemcpyAsync(J9, d + ns, 9 * ns * sizeof(double),
                              cudaMemcpyDefault, ctx->stream));
    if (lap)
      NCGM_CUDA(cudaMemcpyAsync(lap, d + 10 * ns, ns * sizeof(double),
                                cudaMemcpyDefault, ctx->stream));
    NCGM_CUDA(cudaStreamSynchronize(ctx->stream));
    return NCGM_OK;
  } catch (const std::exception &e) {
    setError(e.what());
    return NCGM_ERR_ARG;
  }
}

extern "C" int ncgm_poisson(ncgm_ctx *ctx, const double *rhoP, int Z,
                            const double *U_guess, double *U_out,
                            double *UC_out, int *iterations) {
  try {
    if (!ctx || !rhoP || !U_out) {
      setError("ncgm_poisson: bad argument");
      return NCGM_ERR_ARG;
    }
    const size_t ns = ctx->ns;
    double *d = static_cast<double *>(
        ctx->buf(25, (3 * ns + poissonWorkDoubles(ctx->n)) * sizeof(double)));
    if (!d) return NCGM_ERR_NOMEM;
    NCGM_CUDA(cudaMemcpyAsync(d, rhoP, ns * sizeof(double), cudaMemcpyDefault,
                              ctx->stream));
    if (U_guess)
      NCGM_CUDA(cudaMemcpyAsync(d + ns, U_guess, ns * sizeof(double),
                                cudaMemcpyDefault, ctx->stream));
    PoissonArgs P;
    P.n = ctx->n;
    P.a = ctx->a;
    P.h = ctx->h;
    P.Z = Z;
    P.rhoP = d;
    P.U = d + ns;
    P.UC = d + 2 * ns;
    P.warm = U_guess != nullptr;
    P.tol = 1e-13;
    P.work = d + 3 * ns;
    int its = 0;
    NCGM_TRY(poissonSolve(P, ctx->stream, &its));
    NCGM_CUDA(cudaMemcpyAsync(U_out, d + ns, ns * sizeof(double),
                              cudaMemcpyDefault, ctx->stream));
    if (UC_out)
      NCGM_CUDA(cudaMemcpyAsync(UC_out, d + 2 * ns, ns * sizeof(double),
                                cudaMemcpyDefault, ctx->stream));
    NCGM_CUDA(cudaStreamSynchronize(ctx->stream));
    if (iterations) *iterations = its;
    return NCGM_OK;
  } catch (const std::exception &e) {
    setError(e.what());
    return NCGM_ERR_ARG;
  }
}

// Batch of independent runs (constraint points of a deformation curve, or
// different nuclei) on one GPU: every configuration runs the full HF loop on
// its own host thread, context and non-blocking stream, so the small,
// latency-bound launches of the different runs overlap on the device. Each
// run is bit-for-bit the run ncgm_hf_run gives for that configuration.
extern "C" int ncgm_hf_run_batch(const ncgm_hf_config *cfgs, int count,
                                 int max_concurrent, ncgm_hf_result *res,
                                 int *status, double *const *rho_n,
                                 double *const *rho_p) {
  if (!cfgs || !res || count < 1) {
    setError("ncgm_hf_run_batch: bad argument");
    return NCGM_ERR_ARG;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    setError("ncgm_hf_run_batch: no CUDA device");
    return NCGM_ERR_CUDA;
  }
  const int width =
      max_concurrent > 0 ? std::min(max_concurrent, count) : count;
  std::vector<int> st(count, NCGM_OK);
  std::vector<std::string> err(count);
  std::atomic<int> next{0};
  auto worker = [&]() {
    cudaSetDevice(dev);
    for (int i = next++; i < count; i = next++) {
      st[i] = ncgm_hf_run(&cfgs[i], &res[i], nullptr, nullptr,
                          rho_n ? rho_n[i] : nullptr,
                          rho_p ? rho_p[i] : nullptr, nullptr);
      if (st[i] != NCGM_OK) err[i] = ncgm_last_error();
    }
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < width; ++t) pool.emplace_back(worker);
  for (auto &t : pool) t.join();
  int first = NCGM_OK;
  for (int i = 0; i < count; ++i) {
    if (status) status[i] = st[i];
    if (st[i] != NCGM_OK && first == NCGM_OK) {
      first = st[i];
      setError("ncgm_hf_run_batch: configuration " + std::to_string(i) +
               ": " + err[i]);
    }
  }
  return first;
}


// ---------------------------------------------------------------------------
// IterationData as a handle (include/util/iteration_data.hpp:81-137): the
// densities with their mixing history, the mean fields, the Coulomb field,
// the constraints and the pairing state of one self-consistent run, updated
// from eigenpairs the caller solved for (ncgm_state_update =
// IterationData::updateQuantities, src/util/iteration_data.cpp:852-1125).
// ---------------------------------------------------------------------------
struct ncgm_state {
  ncgm::Run R;
  bool multipolesAdded = false;
  double lastEHF = 0.0; // E_HF of the previous ncgm_state_energy call
};

namespace {
int checkState(ncgm_state *st, const char *who) {
  if (!st) {
    setError(std::string(who) + ": null state");
    return NCGM_ERR_ARG;
  }
  return NCGM_OK;
}
} // namespace

extern "C" int ncgm_state_create(ncgm_state **out, const ncgm_hf_config *cfg) {
  try {
    if (!out || !cfg || cfg->n < 4 || cfg->box_size <= 0 || cfg->A < 2 ||
        cfg->Z < 0 || cfg->Z > cfg->A) {
      setError("ncgm_state_create: bad configuration");
      return NCGM_ERR_ARG;
    }
    *out = nullptr;
    auto *st = new ncgm_state();
    const int rc = setupRun(st->R, *cfg, false);
    if (rc != NCGM_OK) {
      delete st;
      return rc;
    }
    *out = st;
    return NCGM_OK;
  } catch (const std::exception &e) {
    setError(e.what());
    return NCGM_ERR_ARG;
  }
}

extern "C" int ncgm_state_destroy(ncgm_state *st) {
  delete st;
  return NCGM_OK;
}

extern "C" int ncgm_state_update(ncgm_state *st, const double *Xn,
                                 const double *en, int ncols_n,
                                 const double *Xp, const double *ep,
                                 int ncols_p, int iter, int flags) {
  try {
    NCGM_TRY(checkState(st, "ncgm_state_update"));
    Run &R = st->R;
    const double *X[2] = {Xn, Xp}, *e[2] = {en, ep};
    const int cols[2] = {ncols_n, ncols_p};
    for (int q = 0; q < 2; ++q)
      if (!X[q] || !e[q] || cols[q] != R.sp[q].orb || iter < 0) {
        setError("ncgm_state_update: need both species' eigenpairs with " +
                 std::to_string(R.sp[0].orb) + " and " +
                 std::to_string(R.sp[1].orb) + " columns, iter >= 0");
        return NCGM_ERR_ARG;
      }
    const bool pairing = R.cfg.pairing_type != NCGM_PAIRING_NONE;
    for (int q = 0; q < 2; ++q) {
      Species &S = R.sp[q];
      NCGM_CUDA(cudaMemcpyAsync(S.X, X[q], sizeof(double2) * R.N * cols[q],
                                cudaMemcpyDefault, R.s));
      S.e.assign(e[q], e[q] + cols[q]);
      // main.cpp:254-263 before the next update
      if (flags & NCGM_UPDATE_NORMALIZE)
        normalizeColumns(S.X, R.N, cols[q], R.n, R.h, R.small, R.s);
      if ((flags & NCGM_UPDATE_TRORDER) && pairing)
        NCGM_TRY(trOrder(R, S, S.X));
    }
    // the input's multipole constraints join at HF iteration 1
    // (main.cpp:201-207)
    if (iter >= 1 && R.cfg.n_multipole > 0 && !st->multipolesAdded) {
      NCGM_TRY(addMultipoles(R));
      st->multipolesAdded = true;
    }
    NCGM_TRY(updateQuantities(R, iter));
    return sync(R);
  } catch (const std::exception &e) {
    setError(e.what());
    return NCGM_ERR_ARG;
  }
}

extern "C" int ncgm_state_fields(ncgm_state *st, int species, double *f,
                                 double *gradf, double *U, double *W,
                                 double *UC) {
  NCGM_TRY(checkState(st, "ncgm_state_fields"));
  if (species != NCGM_NEUTRON && species != NCGM_PROTON) {
    setError("ncgm_state_fields: bad species");
    return NCGM_ERR_ARG;
  }
  Run &R = st->R;
  const int q = species;
  const size_t b = sizeof(double) * R.ns;
  if (f) NCGM_CUDA(cudaMemcpyAsync(f, R.f[q], b, cudaMemcpyDefault, R.s));
  if (gradf)
    NCGM_CUDA(cudaMemcpyAsync(gradf, R.gf[q], 3 * b, cudaMemcpyDefault, R.s));
  if (U) NCGM_CUDA(cudaMemcpyAsync(U, R.U[q], b, cudaMemcpyDefault, R.s));
  if (W) NCGM_CUDA(cudaMemcpyAsync(W, R.W[q], 3 * b, cudaMemcpyDefault, R.s));
  if (UC) {
    if (q == NCGM_PROTON && R.cfg.use_coulomb && R.haveCoul)
      NCGM_CUDA(cudaMemcpyAsync(UC, R.UCoul, b, cudaMemcpyDefault, R.s));
    else
      NCGM_CUDA(cudaMemsetAsync(UC, 0, b, R.s));
  }
  return sync(R);
}

extern "C" int ncgm_state_densities(ncgm_state *st, int species, double *rho,
                                    double *tau) {
  NCGM_TRY(checkState(st, "ncgm_state_densities"));
  if (species != NCGM_NEUTRON && species != NCGM_PROTON) {
    setError("ncgm_state_densities: bad species");
    return NCGM_ERR_ARG;
  }
  Run &R = st->R;
  const size_t b = sizeof(double) * R.ns;
  if (rho)
    NCGM_CUDA(cudaMemcpyAsync(rho, R.rho[species], b, cudaMemcpyDefault, R.s));
  if (tau)
    NCGM_CUDA(cudaMemcpyAsync(tau, R.tau[species], b, cudaMemcpyDefault, R.s));
  return sync(R);
}

extern "C" int ncgm_state_energy(ncgm_state *st, const double *en,
                                 const double *ep, double *E_int,
                                 double *E_HF) {
  try {
    NCGM_TRY(checkState(st, "ncgm_state_energy"));
    Run &R = st->R;
    if (!en || !ep || !E_int || !E_HF) {
      setError("ncgm_state_energy: null argument");
      return NCGM_ERR_ARG;
    }
    R.sp[0].e.assign(en, en + R.sp[0].orb);
    R.sp[1].e.assign(ep, ep + R.sp[1].orb);
    NCGM_TRY(energies(R, *E_int, *E_HF));
    // data.energyDiff, read by the constraints' multiplier updates
    R.energyDiff = std::abs(*E_HF - st->lastEHF);
    st->lastEHF = *E_HF;
    return NCGM_OK;
  } catch (const std::exception &e) {
    setError(e.what());
    return NCGM_ERR_ARG;
  }
}
