// Block GCG eigensolver with locking on the device: the GB300 form of
// gcgm_complex_no_B_lock (src/solver/solver.cpp:642-959) as called by
// Utilities::solve (src/util/utilities.cpp:20-36).
//
// Steps per outer iteration (reference line numbers in brackets):
//   shift = (L_last - 100 L_0)/99                       [719-722]
//   W = PCG correction of every active column           [723-745]  (k_pcg.cu)
//   V = [X0 | X | P | W], orthonormalised, tiny columns dropped [747-764]
//       -> CholQR2 whose Cholesky pivots follow the MGS drop rule
//   Rayleigh-Ritz on (A + shift): lower triangle of V^H A V [766-777]
//   residuals, absolute-tolerance locking              [796-825]
// and the final assembly/sort of locked + active pairs [838-959].
// Everything runs on the device; the host keeps only O(m) scalars (Ritz
// values, residual norms) to take the locking decisions.
#include "k_dense.cuh"
#include "k_learned.cuh"
#include "k_pcg.cuh"
#include "ncgm_internal.cuh"

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cmath>
#include <numeric>
#include <vector>

namespace ncgm {

bool isDevicePtr(const void *p);

namespace {

__global__ void gatherCols(const double2 *src, size_t lds, const int *idx,
                           int k, double2 *dst, size_t ldd, size_t N) {
  const int c = blockIdx.y;
  if (c >= k) return;
  const double2 *s = src + (size_t)idx[c] * lds;
  double2 *d = dst + (size_t)c * ldd;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x)
    d[i] = s[i];
}

__global__ void scatterCols(const double2 *src, size_t lds, const int *idx,
                            int k, double2 *dst, size_t ldd, size_t N) {
  const int c = blockIdx.y;
  if (c >= k) return;
  const double2 *sp = src + (size_t)c * lds;
  double2 *d = dst + (size_t)idx[c] * ldd;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x)
    d[i] = sp[i];
}

// small matrix: dst(:, c) = src(:, idx[c]) for an m-row matrix
__global__ void gatherSmall(const double2 *src, int lds, int rows,
                            const int *idx, int k, double2 *dst, int ldd) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < rows * k;
       e += gridDim.x * blockDim.x) {
    int r = e % rows, c = e / rows;
    dst[(size_t)c * ldd + r] = src[(size_t)idx[c] * lds + r];
  }
}

// Y = Y + a X  (columns of length N, k columns, per-column scale a[c] * s)
__global__ void axpyCols(double2 *Y, const double2 *X, size_t N, int k,
                         double s) {
  const int c = blockIdx.y;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x) {
    double2 x = X[(size_t)c * N + i];
    double2 y = Y[(size_t)c * N + i];
    Y[(size_t)c * N + i] = make_double2(y.x + s * x.x, y.y + s * x.y);
  }
}

// per column: partial sums of |AX_c - L_c X_c|^2 and Re(X_c^H AX_c) over
// the rows of one block (grid: blocks x columns); colStatsFinish adds the
// partials of each column in a fixed order
__global__ void colStatsPart(const double2 *X, const double2 *AX, size_t N,
                             const double *L, double *part, int nb) {
  __shared__ double s0[256], s1[256];
  const int c = blockIdx.y;
  const double l = L[c];
  double a = 0, b = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N;
       i += (size_t)gridDim.x * blockDim.x) {
    double2 x = X[(size_t)c * N + i], y = AX[(size_t)c * N + i];
    double rx = y.x - l * x.x, ry = y.y - l * x.y;
    a += rx * rx + ry * ry;
    b += x.x * y.x + x.y * y.y;
  }
  s0[threadIdx.x] = a;
  s1[threadIdx.x] = b;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      s0[threadIdx.x] += s0[threadIdx.x + st];
      s1[threadIdx.x] += s1[threadIdx.x + st];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[((size_t)c * nb + blockIdx.x) * 2] = s0[0];
    part[((size_t)c * nb + blockIdx.x) * 2 + 1] = s1[0];
  }
}

__global__ void colStatsFinish(const double *part, int nb, double *res2,
                               double *xax) {
  const int c = blockIdx.x;
  if (threadIdx.x != 0) return;
  double a = 0, b = 0;
  for (int k = 0; k < nb; ++k) {
    a += part[((size_t)c * nb + k) * 2];
    b += part[((size_t)c * nb + k) * 2 + 1];
  }
  res2[c] = a;
  xax[c] = b;
}

__global__ void extractDiag(const double *coef, size_t ns, double *d) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < ns;
       p += (size_t)gridDim.x * blockDim.x)
    d[p] = coef[8 * p];
}

struct Carve {
  char *p;
  size_t off = 0;
  template <class T> T *take(size_t count) {
    off = (off + 255) & ~size_t(255);
    T *r = reinterpret_cast<T *>(p + off);
    off += count * sizeof(T);
    return r;
  }
};

double msSince(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now() - t0)
      .count();
}

} // namespace

// Orthonormalise the k columns of V (N x k, ld N) into Q with MGS-equivalent
// dropping (pivot <= 1e-24). Returns kept column count; Q gets them compacted.
// reads and clears the error word of the exact-digit tensor-core kernels
static int takeExactErr() {
  int flag = 0, zero = 0;
  if (cudaMemcpy(&flag, exactGramErrWord(), sizeof(int),
                 cudaMemcpyDeviceToHost) != cudaSuccess)
    return 1;
  if (flag)
    cudaMemcpy(exactGramErrWord(), &zero, sizeof(int), cudaMemcpyHostToDevice);
  return flag;
}

static int cholQR2(ncgm_ctx *ctx, const double2 *V, int k, double2 *Q,
                   double2 *Q1, double2 *small, double2 *partials,
                   int maxChunks, int *dKeep, int *dIdx, cudaStream_t s,
                   std::vector<int> *keptOrig = nullptr,
                   float *tcPart = nullptr, void *vcPart = nullptr,
                   bool fast = false) {
  const size_t N = ctx->N;
  double2 *G = small, *R = small + (size_t)k * k, *T = small + 2 * (size_t)k * k,
          *Tk = small + 3 * (size_t)k * k;
  std::vector<int> keep(k), idx;
  const double2 *src = V;
  double2 *dst = Q1;
  int cols = k;
  std::vector<int> orig(k);
  std::iota(orig.begin(), orig.end(), 0);
  for (int pass = 0; pass < 2; ++pass) {
    // tensor-core form: both passes' Grams on the tensor cores with exact
    // digit products (~1e-12 relative; the basis is orthonormal to that
    // level); otherwise FP64
    if (tcPart)
      gramTCExact(src, N, cols, src, N, cols, N, G, cols,
                  reinterpret_cast<double *>(tcPart), s);
    else
      gram(src, N, cols, src, N, cols, N, G, cols, partials, maxChunks, s);
    cholDrop(G, cols, cols, 1e-24, R, T, dKeep, s, fast);
    cudaError_t e = cudaMemcpyAsync(keep.data(), dKeep, sizeof(int) * cols,
                                    cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      setError(std::string("ncgm_gcg: orthonormalisation pass ") +
               std::to_string(pass) + " of " + std::to_string(k) +
               " columns: " + cudaGetErrorString(e));
      return -1;
    }
    idx.clear();
    for (int j = 0; j < cols; ++j)
      if (keep[j]) idx.push_back(j);
    const int kept = (int)idx.size();
    if (kept == 0) return 0;
    std::vector<int> o2(kept);
    for (int j = 0; j < kept; ++j) o2[j] = orig[idx[j]];
    orig.swap(o2);
    cudaMemcpyAsync(dIdx, idx.data(), sizeof(int) * kept,
                    cudaMemcpyHostToDevice, s);
    gatherSmall<<<(cols * kept + 255) / 256, 256, 0, s>>>(T, cols, cols, dIdx,
                                                          kept, Tk, cols);
    double2 *out = (pass == 0) ? dst : Q;
    if (vcPart)
      gemmVCExact(src, N, cols, Tk, cols, kept, out, N, N, vcPart, s);
    else
      gemmVC(src, N, cols, Tk, cols, kept, out, N, N, 0.0, s);
    src = out;
    cols = kept;
  }
  if (keptOrig) *keptOrig = orig;
  return cols;
}

double *jacobiDiagonal(ncgm_ctx *ctx, int species, cudaStream_t s) {
  double *d = static_cast<double *>(
      ctx->buf(12 + species, ctx->ns * sizeof(double)));
  if (!d) return nullptr;
  extractDiag<<<(unsigned)std::min<size_t>(1024, (ctx->ns + 255) / 256), 256,
                0, s>>>(ctx->sp[species].coef64, ctx->ns, d);
  return d;
}

int gcgRun(ncgm_ctx *ctx, int species, const double2 *Xinit, int xcols,
           const double2 *ConjDir, int pcols, int nev,
           const ncgm_gcg_params &prm, double2 *Xout, double *lamOut,
           ncgm_gcg_stats *stats) {
  const auto tStart = std::chrono::steady_clock::now();
  cudaStream_t s = ctx->stream;
  const size_t N = ctx->N;
  const int vmax = 3 * nev + pcols;
  const int mx = std::max(vmax, 4);
  const size_t maxChunks = std::max<size_t>(
      1, std::min<size_t>(256, (size_t)8 * 1024 * 1024 / ((size_t)mx * mx)));
  const bool fp32 =
      prm.precision == NCGM_FP32 || prm.precision == NCGM_FP32_TC;
  const bool learned = prm.precond == NCGM_PRECOND_LEARNED;
  // tensor-core Gram products of the search space (FP32-level accuracy)
  const bool tc = prm.precision == NCGM_FP32_TC;
  if (learned && !ctx->lp) {
    setError("ncgm_gcg: learned preconditioner requested but no network set "
             "(ncgm_set_lp)");
    return NCGM_ERR_ARG;
  }
  // workspace
  size_t need = 0;
  need += N * (size_t)vmax * sizeof(double2) * 3; // V, Q, AV
  need += N * (size_t)vmax * sizeof(double2);     // Q1 (CholQR pass 1)
  need += N * (size_t)nev * sizeof(double2) * 5;  // Xa, X0, Xn, AXn, AXa
  need += N * (size_t)nev * (fp32 ? sizeof(float2) : sizeof(double2)) * 7;
  need += (size_t)mx * mx * sizeof(double2) * 8;  // small matrices
  need += maxChunks * (size_t)mx * mx * sizeof(double2);
  need += (size_t)nev * 128 * 5 * sizeof(double) + 64 * 1024;
  need += ctx->ns * sizeof(float) + 256; // FP32 inverse Jacobi diagonal
  char *base = static_cast<char *>(ctx->buf(10, need + 64 * 4096));
  if (!base) return NCGM_ERR_NOMEM;
  float *tcPart = nullptr;
  void *vcPart = nullptr;
  if (tc) {
    tcPart = static_cast<float *>(ctx->buf(
        11, sizeof(double) * exactGramScratchDoubles(N, vmax, vmax) + 256));
    vcPart = ctx->buf(31, exactVCScratchBytes(N, vmax, vmax));
    if (!tcPart || !vcPart) return NCGM_ERR_NOMEM;
  }
  // the projected eigensolver's workspace (Householder methods)
  const size_t heigScrB = heigScratchBytes(mx);
  void *heigScr = ctx->buf(32, heigScrB);
  if (!heigScr) return NCGM_ERR_NOMEM;
  Carve ar{base};
  double2 *V = ar.take<double2>(N * vmax), *Q = ar.take<double2>(N * vmax),
          *AV = ar.take<double2>(N * vmax), *Q1 = ar.take<double2>(N * vmax);
  double2 *Xa = ar.take<double2>(N * nev), *X0 = ar.take<double2>(N * nev),
          *Xn = ar.take<double2>(N * nev), *AXn = ar.take<double2>(N * nev),
          *AXa = ar.take<double2>(N * nev);
  const size_t vbytes = fp32 ? sizeof(float2) : sizeof(double2);
  char *pv = ar.take<char>(N * nev * vbytes * 7);
  void *pX = pv, *pW = pv + N * nev * vbytes, *pR = pv + 2 * N * nev * vbytes,
       *pZ = pv + 3 * N * nev * vbytes, *pP = pv + 4 * N * nev * vbytes,
       *pAP = pv + 5 * N * nev * vbytes, *pD0 = pv + 6 * N * nev * vbytes;
  double2 *small = ar.take<double2>((size_t)mx * mx * 8);
  double2 *partials = ar.take<double2>(maxChunks * (size_t)mx * mx);
  double *dW = ar.take<double>(mx), *dL = ar.take<double>(mx),
         *dRes = ar.take<double>(mx), *dXax = ar.take<double>(mx),
         *dLs = ar.take<double>(mx);
  int *dKeep = ar.take<int>(mx), *dIdx = ar.take<int>(mx),
      *dPerm = ar.take<int>(mx), *dStat = ar.take<int>(4),
      *dUse = ar.take<int>(mx);
  PcgCol *dSt = ar.take<PcgCol>(nev);
  double *pp1 = ar.take<double>((size_t)nev * 128 * 3),
         *pp2 = ar.take<double>((size_t)nev * 128 * 2);
  int *dLive = ar.take<int>(1), *dNdone = ar.take<int>(1);
  unsigned *dArrive = ar.take<unsigned>(2 * (size_t)nev);
  float *dInv32 = ar.take<float>(ctx->ns);
  double2 *Gs = small, *Cw = small + 4 * (size_t)mx * mx,
          *Ev = small + 5 * (size_t)mx * mx, *Ap = small + 6 * (size_t)mx * mx;

  auto gridN = [&](int cols) {
    return dim3((unsigned)std::min<size_t>(1024, (N + 255) / 256), cols);
  };
  auto applyA = [&](const double2 *X, double2 *Y, int cols, double sh) {
    applyH64(ctx, species, X, Y, cols, sh, s);
  };
  NCGM_CUDA(cudaMemsetAsync(dLive, 0, sizeof(int), s));
  const double *dDiag = jacobiDiagonal(ctx, species, s);
  if (!dDiag) return NCGM_ERR_NOMEM;
  if (fp32) inverseDiagonal32(dDiag, prm.shift, ctx->ns, dInv32, s);

  // X = X_init.leftCols(nev), orthonormalised (solver.cpp:669,677)
  NCGM_CUDA(cudaMemcpyAsync(V, Xinit, N * (size_t)nev * sizeof(double2),
                            cudaMemcpyDeviceToDevice, s));
  std::vector<int> keptInit;
  int nkept = cholQR2(ctx, V, nev, Q, Q1, Gs, partials, (int)maxChunks, dKeep,
                      dIdx, s, &keptInit, tcPart, vcPart, fp32);
  if (nkept < 0) return NCGM_ERR_CUDA;
  if (nkept == 0) {
    setError("ncgm_gcg: initial block has no independent columns");
    return NCGM_ERR_RANK;
  }
  // MGS keeps dropped columns as zero columns in place (solver.cpp:404-407)
  NCGM_CUDA(cudaMemsetAsync(Xa, 0, N * (size_t)nev * sizeof(double2), s));
  {
    std::vector<int> dst(keptInit);
    NCGM_CUDA(cudaMemcpyAsync(dIdx, dst.data(), sizeof(int) * nkept,
                              cudaMemcpyHostToDevice, s));
    scatterCols<<<gridN(nkept), 256, 0, s>>>(Q, N, dIdx, nkept, Xa, N, N);
  }
  const int nx = nev;
  double shift = prm.shift;
  std::vector<double> hw(mx), hres(mx), hxax(mx);
  std::vector<double> Lambda;
  // initial Rayleigh-Ritz (rayleighRitz_complex_no_B, solver.cpp:418-463)
  {
    applyA(Xa, AV, nx, shift);
    if (tc)
      gramTCExact(Xa, N, nx, AV, N, nx, N, Ap, nx,
                  reinterpret_cast<double *>(tcPart), s);
    else
      gram(Xa, N, nx, AV, N, nx, N, Ap, nx, partials, (int)maxChunks, s);
    heig(Ap, nx, nx, Cw, Ev, dW, dPerm, dStat, s, fp32, heigScr, heigScrB);
    if (tc)
      gemmVCExact(Xa, N, nx, Ev, nx, nx, Xn, N, N, vcPart, s);
    else
      gemmVC(Xa, N, nx, Ev, nx, nx, Xn, N, N, 0.0, s);
    NCGM_CUDA(cudaMemcpyAsync(Xa, Xn, N * (size_t)nx * sizeof(double2),
                              cudaMemcpyDeviceToDevice, s));
    // A X of the rotated block (shift removed), kept for the FP32 correction
    if (tc)
      gemmVCExact(AV, N, nx, Ev, nx, nx, AXa, N, N, vcPart, s);
    else
      gemmVC(AV, N, nx, Ev, nx, nx, AXa, N, N, 0.0, s);
    if (shift != 0.0)
      axpyCols<<<gridN(nx), 256, 0, s>>>(AXa, Xa, N, nx, -shift);
    NCGM_CUDA(cudaMemcpyAsync(hw.data(), dW, sizeof(double) * nx,
                              cudaMemcpyDeviceToHost, s));
    NCGM_CUDA(cudaStreamSynchronize(s));
    Lambda.resize(nx);
    for (int i = 0; i < nx; ++i) Lambda[i] = hw[i] - shift;
  }
  int nconv = 0, nact = nx;
  std::vector<double> x0lam; // Re(x^H A x) of the locked columns
  bool early = false;
  double msPcg = 0;
  int iterations = 0, lastBasis = 0, pcgMax = 0, lpCols = 0;
  int pc = pcols;
  for (int iter = 0; iter < prm.max_iter; ++iter) {
    if (nconv == nev) {
      early = true;
      break;
    }
    if (Lambda.size() > 1)
      shift = (Lambda[Lambda.size() - 1] - 100.0 * Lambda[0]) / 99.0;
    // assemble V = [X0 | X | P | W]
    size_t o = 0;
    if (nconv)
      NCGM_CUDA(cudaMemcpyAsync(V, X0, N * (size_t)nconv * sizeof(double2),
                                cudaMemcpyDeviceToDevice, s));
    o += nconv;
    NCGM_CUDA(cudaMemcpyAsync(V + o * N, Xa, N * (size_t)nact * sizeof(double2),
                              cudaMemcpyDeviceToDevice, s));
    o += nact;
    if (pc > 0)
      NCGM_CUDA(cudaMemcpyAsync(V + o * N, ConjDir,
                                N * (size_t)pc * sizeof(double2),
                                cudaMemcpyDeviceToDevice, s));
    o += pc;
    double2 *Wd = V + o * N;
    if (nact > 0) {
      std::vector<double> ls(nact);
      for (int k = 0; k < nact; ++k) ls[k] = Lambda[k] + shift;
      NCGM_CUDA(cudaMemcpyAsync(dLs, ls.data(), sizeof(double) * nact,
                                cudaMemcpyHostToDevice, s));
      auto tp = std::chrono::steady_clock::now();
      if (learned) {
        // network start d0 = N(x lambda - A x) for every active column
        NCGM_CUDA(cudaMemcpyAsync(dL, Lambda.data(), sizeof(double) * nact,
                                  cudaMemcpyHostToDevice, s));
        int rc = fp32 ? lpInitialCorrection<float>(
                            ctx->lp, ctx, species, Xa, AXa, dL, shift, nact,
                            static_cast<float *>(pD0), s)
                      : lpInitialCorrection<double>(
                            ctx->lp, ctx, species, Xa, AXa, dL, shift, nact,
                            static_cast<double *>(pD0), s);
        if (rc != NCGM_OK) return rc;
      }
      if (!fp32 && learned) {
        PcgPlan<double> pl;
        pl.N = N;
        pl.ncols = nact;
        pl.X = Xa;
        pl.ldx = N;
        pl.X64 = Xa;
        pl.AX64 = AXa;
        pl.W64 = Wd;
        pl.W = pW;
        pl.R = pR;
        pl.Z = pZ;
        pl.P = pP;
        pl.AP = pAP;
        pl.D0 = pD0;
        pl.useNet = dUse;
        pl.lamShift = dLs;
        pl.coef = dDiag;
        pl.arrive = dArrive;
        pl.shift = shift;
        pl.tol = prm.cg_tol;
        pl.maxSteps = prm.cg_steps;
        pl.st = dSt;
        pl.partials = pp1;
        pl.partials2 = pp2;
        pl.live = dLive;
        pl.ndone = dNdone;
        pl.apply = [&](const void *X, size_t, void *Y, int cols, double sh,
                       cudaStream_t st) {
          applyH64(ctx, species, static_cast<const double2 *>(X),
                   static_cast<double2 *>(Y), cols, sh, st);
        };
        pcgRun<double>(pl, s);
      } else if (!fp32) {
        PcgPlan<double> pl;
        pl.N = N;
        pl.ncols = nact;
        pl.X = Xa;
        pl.ldx = N;
        pl.W = Wd;
        pl.R = pR;
        pl.Z = pZ;
        pl.P = pP;
        pl.AP = pAP;
        pl.lamShift = dLs;
        pl.coef = dDiag;
        pl.arrive = dArrive;
        pl.shift = shift;
        pl.tol = prm.cg_tol;
        pl.maxSteps = prm.cg_steps;
        pl.st = dSt;
        pl.partials = pp1;
        pl.partials2 = pp2;
        pl.live = dLive;
        pl.ndone = dNdone;
        pl.apply = [&](const void *X, size_t, void *Y, int cols, double sh,
                       cudaStream_t st) {
          applyH64(ctx, species, static_cast<const double2 *>(X),
                   static_cast<double2 *>(Y), cols, sh, st);
        };
        pcgRun<double>(pl, s);
      } else {
        PcgPlan<float> pl;
        pl.N = N;
        pl.ncols = nact;
        pl.X = pX;
        pl.ldx = N;
        pl.X64 = Xa;
        pl.AX64 = AXa;
        pl.W64 = Wd;
        pl.W = pW;
        pl.R = pR;
        pl.Z = pZ;
        pl.P = pP;
        pl.AP = pAP;
        if (learned) {
          pl.D0 = pD0;
          pl.useNet = dUse;
        }
        // the search space takes the correction d itself: the same span as
        // w = x + d, but not nearly dependent on x, so the orthonormalisation
        // keeps d's direction to full precision (with w = x + d it would
        // lose the digits of d that FP32 rounding already made noisy)
        pl.onlyCorrection = true;
        pl.lamShift = dLs;
        pl.coef = dDiag;
        pl.invd = dInv32;
        pl.arrive = dArrive;
        pl.shift = shift;
        pl.tol = prm.cg_tol;
        pl.maxSteps = prm.cg_steps;
        pl.st = dSt;
        pl.partials = pp1;
        pl.partials2 = pp2;
        pl.live = dLive;
        pl.ndone = dNdone;
        pl.apply = [&](const void *X, size_t, void *Y, int cols, double sh,
                       cudaStream_t st) {
          applyH32(ctx, species, static_cast<const float2 *>(X),
                   static_cast<float2 *>(Y), cols, (float)sh, st);
        };
        pcgRun<float>(pl, s);
      }
      if (stats) {
        std::vector<PcgCol> hs(nact);
        NCGM_CUDA(cudaMemcpyAsync(hs.data(), dSt, sizeof(PcgCol) * nact,
                                  cudaMemcpyDeviceToHost, s));
        NCGM_CUDA(cudaStreamSynchronize(s));
        for (auto &c : hs) pcgMax = std::max(pcgMax, c.iters);
        if (learned) {
          std::vector<int> hu(nact);
          NCGM_CUDA(cudaMemcpyAsync(hu.data(), dUse, sizeof(int) * nact,
                                    cudaMemcpyDeviceToHost, s));
          NCGM_CUDA(cudaStreamSynchronize(s));
          for (int u : hu) lpCols += u;
        }
      }
      msPcg += msSince(tp);
    }
    const int vcols = nconv + nact + pc + nact;
    int m = cholQR2(ctx, V, vcols, Q, Q1, Gs, partials, (int)maxChunks, dKeep,
                    dIdx, s, nullptr, tcPart, vcPart, fp32);
    if (m < 0) return NCGM_ERR_CUDA;
    if (m == 0) {
      setError("ncgm_gcg: search space collapsed");
      return NCGM_ERR_RANK;
    }
    lastBasis = m;
    // Rayleigh-Ritz on A_shifted
    applyA(Q, AV, m, shift);
    if (tc)
      gramTCExact(Q, N, m, AV, N, m, N, Ap, m,
                  reinterpret_cast<double *>(tcPart), s);
    else
      gram(Q, N, m, AV, N, m, N, Ap, m, partials, (int)maxChunks, s);
    heig(Ap, m, m, Cw, Ev, dW, dPerm, dStat, s, fp32, heigScr, heigScrB);
    const int rr = std::min(nev, m);
    if (tc) {
      gemmVCExact(Q, N, m, Ev, m, rr, Xn, N, N, vcPart, s);
      gemmVCExact(AV, N, m, Ev, m, rr, AXn, N, N, vcPart, s);
    } else {
      gemmVC(Q, N, m, Ev, m, rr, Xn, N, N, 0.0, s);
      gemmVC(AV, N, m, Ev, m, rr, AXn, N, N, 0.0, s);
    }
    axpyCols<<<gridN(rr), 256, 0, s>>>(AXn, Xn, N, rr, -shift); // = A Xn
    NCGM_CUDA(cudaMemcpyAsync(hw.data(), dW, sizeof(double) * m,
                              cudaMemcpyDeviceToHost, s));
    std::vector<double> Lnew(rr);
    NCGM_CUDA(cudaStreamSynchronize(s));
    int hstat = 0;
    NCGM_CUDA(cudaMemcpyAsync(&hstat, dStat, sizeof(int),
                              cudaMemcpyDeviceToHost, s));
    NCGM_CUDA(cudaStreamSynchronize(s));
    if (hstat != 0) {
      setError("ncgm_gcg: projected eigensolver did not converge");
      return NCGM_ERR_EIG;
    }
    for (int i = 0; i < rr; ++i) Lnew[i] = hw[i] - shift;
    NCGM_CUDA(cudaMemcpyAsync(dL, Lnew.data(), sizeof(double) * rr,
                              cudaMemcpyHostToDevice, s));
    {
      const int nb = pcgBlocks(N);
      double *part = reinterpret_cast<double *>(partials);
      colStatsPart<<<dim3(nb, rr), 256, 0, s>>>(Xn, AXn, N, dL, part, nb);
      colStatsFinish<<<rr, 32, 0, s>>>(part, nb, dRes, dXax);
    }
    NCGM_CUDA(cudaMemcpyAsync(hres.data(), dRes, sizeof(double) * rr,
                              cudaMemcpyDeviceToHost, s));
    NCGM_CUDA(cudaMemcpyAsync(hxax.data(), dXax, sizeof(double) * rr,
                              cudaMemcpyDeviceToHost, s));
    NCGM_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < rr; ++i) {
      if (!std::isfinite(hres[i]) || !std::isfinite(Lnew[i])) {
        setError("ncgm_gcg: NaN in Ritz pairs");
        return NCGM_ERR_NAN;
      }
    }
    // locking (solver.cpp:804-835)
    std::vector<int> newly, next;
    for (int i = nconv; i < rr; ++i) {
      if (std::sqrt(hres[i]) < prm.tol && (nconv + (int)newly.size() < nev))
        newly.push_back(i);
      else
        next.push_back(i);
    }
    std::vector<int> x0idx(nconv);
    std::iota(x0idx.begin(), x0idx.end(), 0);
    for (int i : newly) x0idx.push_back(i);
    if (!x0idx.empty()) {
      NCGM_CUDA(cudaMemcpyAsync(dIdx, x0idx.data(), sizeof(int) * x0idx.size(),
                                cudaMemcpyHostToDevice, s));
      gatherCols<<<gridN((int)x0idx.size()), 256, 0, s>>>(
          Xn, N, dIdx, (int)x0idx.size(), X0, N, N);
    }
    if (!next.empty()) {
      NCGM_CUDA(cudaStreamSynchronize(s));
      NCGM_CUDA(cudaMemcpyAsync(dIdx, next.data(), sizeof(int) * next.size(),
                                cudaMemcpyHostToDevice, s));
      gatherCols<<<gridN((int)next.size()), 256, 0, s>>>(
          Xn, N, dIdx, (int)next.size(), Xa, N, N);
      gatherCols<<<gridN((int)next.size()), 256, 0, s>>>(
          AXn, N, dIdx, (int)next.size(), AXa, N, N);
    }
    NCGM_CUDA(cudaStreamSynchronize(s));
    nconv = (int)x0idx.size();
    nact = (int)next.size();
    Lambda.resize(nact);
    for (int i = 0; i < nact; ++i) Lambda[i] = Lnew[next[i]];
    // X0 eigenvalue estimates Re(x^H A x) (solver.cpp:840-842,921-923)
    x0lam.resize(nconv);
    for (int i = 0; i < nconv; ++i) x0lam[i] = hxax[x0idx[i]];
    pc = 0; // P is used in the first iteration only
    iterations = iter + 1;
  }
  // final assembly (solver.cpp:838-959)
  const int take = std::min(nact, nev - nconv);
  std::vector<double> finalL(nev, 0.0);
  for (int i = 0; i < nconv; ++i) finalL[i] = x0lam[i];
  for (int i = 0; i < take; ++i) finalL[nconv + i] = Lambda[i];
  std::vector<int> order(nev);
  std::iota(order.begin(), order.end(), 0);
  if (prm.ordering == NCGM_ORDER_ASCENDING || early)
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return finalL[a] < finalL[b]; });
  // finalX = [X0 | Xa(:, :take) | 0] gathered in `order` into Xout
  NCGM_CUDA(cudaMemsetAsync(Q, 0, N * (size_t)nev * sizeof(double2), s));
  if (nconv)
    NCGM_CUDA(cudaMemcpyAsync(Q, X0, N * (size_t)nconv * sizeof(double2),
                              cudaMemcpyDeviceToDevice, s));
  if (take)
    NCGM_CUDA(cudaMemcpyAsync(Q + (size_t)nconv * N, Xa,
                              N * (size_t)take * sizeof(double2),
                              cudaMemcpyDeviceToDevice, s));
  NCGM_CUDA(cudaMemcpyAsync(dIdx, order.data(), sizeof(int) * nev,
                            cudaMemcpyHostToDevice, s));
  gatherCols<<<gridN(nev), 256, 0, s>>>(Q, N, dIdx, nev, Xout, N, N);
  for (int k = 0; k < nev; ++k) lamOut[k] = finalL[order[k]];
  NCGM_CUDA(cudaStreamSynchronize(s));
  NCGM_CUDA(cudaGetLastError());
  if (tc && takeExactErr()) {
    setError("ncgm_gcg: tensor-core kernel wait timed out");
    return NCGM_ERR_TIMEOUT;
  }
  if (stats) {
    int live = 0;
    cudaMemcpyAsync(&live, dLive, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    stats->iterations = iterations;
    stats->converged = nconv;
    stats->pcg_steps_max = pcgMax;
    stats->pcg_steps_total = live;
    stats->basis_cols = lastBasis;
    double mr = 0;
    for (int i = 0; i < std::min(nev, (int)hres.size()); ++i)
      mr = std::max(mr, std::sqrt(std::max(0.0, hres[i])));
    stats->max_residual = mr;
    stats->ms_total = msSince(tStart);
    stats->ms_pcg = msPcg;
    stats->lp_columns = lpCols;
  }
  return NCGM_OK;
}

} // namespace ncgm

using namespace ncgm;

extern "C" int ncgm_gcg(ncgm_ctx *ctx, int species, const double *X_init,
                        int xcols, const double *ConjDir, int pcols, int nev,
                        const ncgm_gcg_params *params, double *X_out,
                        double *lambda_out, ncgm_gcg_stats *stats) {
  try {
    if (!ctx || species < 0 || species > 1 || !X_init || !X_out ||
        !lambda_out || !params || nev < 1 || xcols < nev || pcols < 0 ||
        (pcols > 0 && !ConjDir) || 3 * nev + pcols > 1024 ||
        params->max_iter < 0 || params->cg_steps < 0) {
      setError("ncgm_gcg: bad argument");
      return NCGM_ERR_ARG;
    }
    if (!ctx->sp[species].ready) {
      setError("ncgm_gcg: fields not set for this species");
      return NCGM_ERR_ARG;
    }
    const size_t N = ctx->N;
    cudaStream_t s = ctx->stream;
    const double2 *Xd = reinterpret_cast<const double2 *>(X_init);
    const double2 *Pd = reinterpret_cast<const double2 *>(ConjDir);
    if (!isDevicePtr(X_init)) {
      double2 *b = static_cast<double2 *>(ctx->buf(20, N * nev * sizeof(double2)));
      if (!b) return NCGM_ERR_NOMEM;
      NCGM_CUDA(cudaMemcpyAsync(b, X_init, N * nev * sizeof(double2),
                                cudaMemcpyHostToDevice, s));
      Xd = b;
    }
    if (pcols > 0 && !isDevicePtr(ConjDir)) {
      double2 *b =
          static_cast<double2 *>(ctx->buf(21, N * pcols * sizeof(double2)));
      if (!b) return NCGM_ERR_NOMEM;
      NCGM_CUDA(cudaMemcpyAsync(b, ConjDir, N * pcols * sizeof(double2),
                                cudaMemcpyHostToDevice, s));
      Pd = b;
    }
    const bool devOut = isDevicePtr(X_out);
    double2 *Xo = reinterpret_cast<double2 *>(X_out);
    if (!devOut) {
      Xo = static_cast<double2 *>(ctx->buf(22, N * nev * sizeof(double2)));
      if (!Xo) return NCGM_ERR_NOMEM;
    }
    std::vector<double> lam(nev);
    int st = gcgRun(ctx, species, Xd, xcols, Pd, pcols, nev, *params, Xo,
                    lam.data(), stats);
    if (st != NCGM_OK) return st;
    if (!devOut)
      NCGM_CUDA(cudaMemcpy(X_out, Xo, N * nev * sizeof(double2),
                           cudaMemcpyDeviceToHost));
    if (isDevicePtr(lambda_out))
      NCGM_CUDA(cudaMemcpy(lambda_out, lam.data(), nev * sizeof(double),
                           cudaMemcpyHostToDevice));
    else
      std::copy(lam.begin(), lam.end(), lambda_out);
    return NCGM_OK;
  } catch (const std::exception &e) {
    setError(e.what());
    return NCGM_ERR_ARG;
  }
}

extern "C" int ncgm_gram(ncgm_ctx *ctx, const double *A, int p,
                         const double *B, int q, double *C, int precision) {
  if (!ctx || !A || !B || !C || p < 1 || q < 1 || p > 4096 || q > 4096 ||
      (precision != NCGM_FP64 && precision != NCGM_FP32 &&
       precision != NCGM_FP32_TC)) {
    setError("ncgm_gram: bad argument");
    return NCGM_ERR_ARG;
  }
  const size_t N = ctx->N;
  cudaStream_t s = ctx->stream;
  auto stage = [&](const double *h, int cols, int slot) -> const double2 * {
    if (isDevicePtr(h)) return reinterpret_cast<const double2 *>(h);
    auto *d = static_cast<double2 *>(ctx->buf(slot, N * cols * sizeof(double2)));
    if (d && cudaMemcpyAsync(d, h, N * cols * sizeof(double2),
                             cudaMemcpyHostToDevice, s) != cudaSuccess)
      return nullptr;
    return d;
  };
  // a Gram of a block with itself stages it once (the tensor-core form then
  // digitises it once)
  const double2 *dA = stage(A, p, 26);
  const double2 *dB = (B == A && q == p) ? dA : stage(B, q, 27);
  if (!dA || !dB) return NCGM_ERR_NOMEM;
  const bool devOut = isDevicePtr(C);
  double2 *dC = devOut ? reinterpret_cast<double2 *>(C)
                       : static_cast<double2 *>(
                             ctx->buf(28, (size_t)p * q * sizeof(double2)));
  if (!dC) return NCGM_ERR_NOMEM;
  if (precision == NCGM_FP32) {
    float *part = static_cast<float *>(
        ctx->buf(29, sizeof(float) * tcGramPartialFloats(N, p, q) + 256));
    if (!part) return NCGM_ERR_NOMEM;
    gramTC(dA, N, p, dB, N, q, N, dC, p, part, s);
  } else if (precision == NCGM_FP32_TC) {
    double *part = static_cast<double *>(
        ctx->buf(29, sizeof(double) * exactGramScratchDoubles(N, p, q) + 256));
    if (!part) return NCGM_ERR_NOMEM;
    gramTCExact(dA, N, p, dB, N, q, N, dC, p, part, s);
  } else {
    const int chunks = gramMaxChunks();
    auto *part = static_cast<double2 *>(
        ctx->buf(29, sizeof(double2) * (size_t)chunks * p * q));
    if (!part) return NCGM_ERR_NOMEM;
    gram(dA, N, p, dB, N, q, N, dC, p, part, chunks, s);
  }
  if (!devOut)
    NCGM_CUDA(cudaMemcpyAsync(C, dC, (size_t)p * q * sizeof(double2),
                              cudaMemcpyDeviceToHost, s));
  NCGM_CUDA(cudaStreamSynchronize(s));
  NCGM_CUDA(cudaGetLastError());
  int flag = 0;
  if (precision == NCGM_FP32_TC) flag = takeExactErr();
  if (precision == NCGM_FP32)
    NCGM_CUDA(cudaMemcpy(&flag, tcGramErrWord(), sizeof(int),
                         cudaMemcpyDeviceToHost));
  if (precision != NCGM_FP64) {
    if (flag) {
      setError("ncgm_gram: tensor-core kernel wait timed out");
      return NCGM_ERR_TIMEOUT;
    }
  }
  return NCGM_OK;
}

extern "C" int ncgm_vc(ncgm_ctx *ctx, const double *V, int m, const double *C,
                       int k, double *Y, int precision) {
  if (!ctx || !V || !C || !Y || m < 1 || k < 1 || m > 4096 || k > 4096 ||
      (precision != NCGM_FP64 && precision != NCGM_FP32_TC)) {
    setError("ncgm_vc: bad argument");
    return NCGM_ERR_ARG;
  }
  using namespace ncgm;
  const size_t N = ctx->N;
  cudaStream_t s = ctx->stream;
  auto stage = [&](const double *h, size_t count, int slot) -> double2 * {
    if (isDevicePtr(h)) return reinterpret_cast<double2 *>(const_cast<double *>(h));
    auto *d = static_cast<double2 *>(ctx->buf(slot, count * sizeof(double2)));
    if (d && cudaMemcpyAsync(d, h, count * sizeof(double2),
                             cudaMemcpyHostToDevice, s) != cudaSuccess)
      return nullptr;
    return d;
  };
  const double2 *dV = stage(V, N * (size_t)m, 26);
  const double2 *dC = stage(C, (size_t)m * k, 27);
  if (!dV || !dC) return NCGM_ERR_NOMEM;
  const bool devOut = isDevicePtr(Y);
  double2 *dY = devOut ? reinterpret_cast<double2 *>(Y)
                       : static_cast<double2 *>(
                             ctx->buf(28, N * (size_t)k * sizeof(double2)));
  if (!dY) return NCGM_ERR_NOMEM;
  if (precision == NCGM_FP32_TC) {
    void *part = ctx->buf(29, exactVCScratchBytes(N, m, k));
    if (!part) return NCGM_ERR_NOMEM;
    gemmVCExact(dV, N, m, dC, m, k, dY, N, N, part, s);
  } else {
    gemmVC(dV, N, m, dC, m, k, dY, N, N, 0.0, s);
  }
  if (!devOut)
    NCGM_CUDA(cudaMemcpyAsync(Y, dY, N * (size_t)k * sizeof(double2),
                              cudaMemcpyDeviceToHost, s));
  NCGM_CUDA(cudaStreamSynchronize(s));
  NCGM_CUDA(cudaGetLastError());
  if (precision == NCGM_FP32_TC && takeExactErr()) {
    setError("ncgm_vc: tensor-core kernel wait timed out");
    return NCGM_ERR_TIMEOUT;
  }
  return NCGM_OK;
}

extern "C" int ncgm_heig(ncgm_ctx *ctx, const double *A, int m, double *w,
                         double *V, int precision) {
  if (!ctx || !A || !w || !V || m < 1 || m > 1024 ||
      (precision != NCGM_FP64 && precision != NCGM_FP32 &&
       precision != NCGM_FP32_TC)) {
    setError("ncgm_heig: bad argument");
    return NCGM_ERR_ARG;
  }
  using namespace ncgm;
  cudaStream_t s = ctx->stream;
  const size_t mm = (size_t)m * m;
  char *base = static_cast<char *>(ctx->buf(
      30, 3 * mm * sizeof(double2) + m * (sizeof(double) + sizeof(int)) + 1024));
  if (!base) return NCGM_ERR_NOMEM;
  double2 *dA = reinterpret_cast<double2 *>(base);
  double2 *work = dA + mm, *dV = work + mm;
  double *dw = reinterpret_cast<double *>(dV + mm);
  int *perm = reinterpret_cast<int *>(dw + m), *st = perm + m;
  NCGM_CUDA(cudaMemcpyAsync(dA, A, mm * sizeof(double2), cudaMemcpyDefault, s));
  heig(dA, m, m, work, dV, dw, perm, st, s, precision != NCGM_FP64);
  int hs = 0;
  NCGM_CUDA(cudaMemcpyAsync(w, dw, m * sizeof(double), cudaMemcpyDefault, s));
  NCGM_CUDA(cudaMemcpyAsync(V, dV, mm * sizeof(double2), cudaMemcpyDefault, s));
  NCGM_CUDA(cudaMemcpyAsync(&hs, st, sizeof(int), cudaMemcpyDeviceToHost, s));
  NCGM_CUDA(cudaStreamSynchronize(s));
  NCGM_CUDA(cudaGetLastError());
  if (hs != 0) {
    setError("ncgm_heig: eigensolver did not converge");
    return NCGM_ERR_EIG;
  }
  return NCGM_OK;
}
