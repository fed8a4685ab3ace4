// C ABI of the GB300 nuclearcgm library (include/ncgm.h): context, field
// upload, Hamiltonian apply. Every entry point returns a status code and never
// lets a C++ exception cross the boundary.
#include "ncgm_internal.cuh"

#include <cstdlib>

#include <algorithm>

#include <cstring>
#include <exception>
#include <string>

namespace ncgm {
namespace {
thread_local std::string g_err;
}
void setError(const std::string &msg) { g_err = msg; }
const char *lastError() { return g_err.c_str(); }

// Is `p` device-accessible memory? (host pointers are staged by copies)
bool isDevicePtr(const void *p) {
  if (!p) return false;
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

} // namespace ncgm

void *ncgm_ctx::buf(int slot, size_t bytes) {
  if ((int)bufs.size() <= slot) bufs.resize(slot + 1, {nullptr, 0});
  auto &b = bufs[slot];
  if (b.second < bytes) {
    if (b.first) cudaFree(b.first);
    b.first = nullptr;
    b.second = 0;
    if (cudaMalloc(&b.first, bytes) != cudaSuccess) {
      cudaGetLastError();
      ncgm::setError("device allocation of " + std::to_string(bytes) +
                     " bytes failed");
      return nullptr;
    }
    b.second = bytes;
  }
  return b.first;
}

using namespace ncgm;

#define NCGM_GUARD_BEGIN try {
#define NCGM_GUARD_END                                                         \
  }                                                                            \
  catch (const std::exception &e) {                                            \
    setError(e.what());                                                        \
    return NCGM_ERR_ARG;                                                       \
  }                                                                            \
  catch (...) {                                                                \
    setError("unknown C++ exception");                                         \
    return NCGM_ERR_ARG;                                                       \
  }

extern "C" {

const char *ncgm_last_error(void) { return lastError(); }

int ncgm_edf_from_skyrme(const ncgm_skyrme *in, ncgm_edf *out) {
  if (!in || !out) {
    setError("null argument");
    return NCGM_ERR_ARG;
  }
  // EDF::setFromInteraction (src/skyrme/EDF.cpp:61-103)
  const double t0 = in->t0, t1 = in->t1, t2 = in->t2, t3 = in->t3;
  const double x0 = in->x0, x1 = in->x1, x2 = in->x2, x3 = in->x3;
  out->sigma = in->sigma;
  out->C0rr = 3 * t0 / 8;
  out->C1rr = -t0 * (0.5 + x0) / 4;
  out->C0Drr = 3 * t3 / 48;
  out->C1Drr = -t3 * (0.5 + x3) / 24;
  out->C0rt = 3 * t1 / 16 + t2 * (5.0 / 4.0 + x2) / 4;
  out->C1rt = -t1 * (0.5 + x1) / 8 + t2 * (0.5 + x2) / 8;
  out->C0rdr = -9 * t1 / 64 + t2 * (5.0 / 4.0 + x2) / 16;
  out->C1rdr = 3 * t1 * (0.5 + x1) / 32 + t2 * (0.5 + x2) / 32;
  out->C0nJ = -0.5 * in->W0 - 0.25 * in->W0_pr;
  out->C1nJ = -0.5 * in->W0;
  const double C0T = -(t1 * (1 - 2 * x1) - t2 * (1 + 2 * x2)) / 16;
  const double C1T = -(t1 - t2) / 16;
  const double C0F = -3 * (in->te + 3 * in->to) / 8;
  const double C1F = -3 * (in->te - in->to) / 8;
  out->C0J2 = -0.5 * (C0T - 0.5 * C0F);
  out->C1J2 = -0.5 * (C1T - 0.5 * C1F);
  return NCGM_OK;
}

int ncgm_create(ncgm_ctx **out, int n, double a, int max_cols, int flags) {
  NCGM_GUARD_BEGIN
  (void)flags;
  if (!out || n < 2 || !(a > 0) || max_cols < 1) {
    setError("ncgm_create: need n >= 2, a > 0, max_cols >= 1");
    return NCGM_ERR_ARG;
  }
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    setError("ncgm_create: no CUDA device");
    return NCGM_ERR_CUDA;
  }
  auto *ctx = new ncgm_ctx();
  ctx->n = n;
  ctx->a = a;
  ctx->h = 2.0 * a / (n - 1); // Grid::Grid (src/grid/grid.cpp:16)
  ctx->max_cols = max_cols;
  ctx->ns = (size_t)n * n * n;
  ctx->N = 2 * ctx->ns;
  cudaGetDevice(&ctx->device);
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) !=
          cudaSuccess ||
      cudaEventCreate(&ctx->ev0) != cudaSuccess ||
      cudaEventCreate(&ctx->ev1) != cudaSuccess) {
    setError(std::string("ncgm_create: ") +
             cudaGetErrorString(cudaGetLastError()));
    delete ctx;
    return NCGM_ERR_CUDA;
  }
  *out = ctx;
  return NCGM_OK;
  NCGM_GUARD_END
}

int ncgm_destroy(ncgm_ctx *ctx) {
  if (!ctx) return NCGM_OK;
  cudaStreamSynchronize(ctx->stream);
  for (auto &b : ctx->bufs)
    if (b.first) cudaFree(b.first);
  for (auto &s : ctx->sp) {
    if (s.coef64) cudaFree(s.coef64);
    if (s.coef32) cudaFree(s.coef32);
    if (s.coef32s) cudaFree(s.coef32s);
  }
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  for (auto e : ctx->xev) cudaEventDestroy(e);
  if (ctx->xin) cudaStreamDestroy(ctx->xin);
  if (ctx->xout) cudaStreamDestroy(ctx->xout);
  if (ctx->ownStream) ctx->stream = ctx->ownStream;
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return NCGM_OK;
}

int ncgm_sync(ncgm_ctx *ctx) {
  if (!ctx) return NCGM_ERR_ARG;
  NCGM_CUDA(cudaStreamSynchronize(ctx->stream));
  NCGM_CUDA(cudaGetLastError());
  return NCGM_OK;
}

int ncgm_set_fields(ncgm_ctx *ctx, int species, const double *f,
                    const double *gradf, const double *U, const double *W,
                    const double *UC) {
  NCGM_GUARD_BEGIN
  if (!ctx || species < 0 || species > 1 || !f || !gradf || !U) {
    setError("ncgm_set_fields: bad argument");
    return NCGM_ERR_ARG;
  }
  const size_t ns = ctx->ns;
  // staging: f, gradf(3), U, W(3), UC -> 9 ns doubles
  double *d = static_cast<double *>(ctx->buf(0, 9 * ns * sizeof(double)));
  if (!d) return NCGM_ERR_NOMEM;
  double *df = d, *dg = d + ns, *dU = d + 4 * ns, *dW = d + 5 * ns,
         *dC = d + 8 * ns;
  auto put = [&](double *dst, const double *src, size_t cnt) {
    return cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyDefault,
                           ctx->stream);
  };
  NCGM_CUDA(put(df, f, ns));
  NCGM_CUDA(put(dg, gradf, 3 * ns));
  NCGM_CUDA(put(dU, U, ns));
  if (W) NCGM_CUDA(put(dW, W, 3 * ns));
  if (UC) NCGM_CUDA(put(dC, UC, ns));
  NCGM_TRY(buildCoefficients(ctx, species, df, dg, dU, W ? dW : nullptr,
                             UC ? dC : nullptr));
  NCGM_CUDA(cudaStreamSynchronize(ctx->stream));
  return NCGM_OK;
  NCGM_GUARD_END
}

int ncgm_set_woods_saxon(ncgm_ctx *ctx, int species, int A, int Z, double V0,
                         double r0, double diff, double kappa, double beta,
                         double beta3, double so_V0, int spin_orbit) {
  NCGM_GUARD_BEGIN
  if (!ctx || species < 0 || species > 1 || A <= 0) {
    setError("ncgm_set_woods_saxon: bad argument");
    return NCGM_ERR_ARG;
  }
  NCGM_TRY(buildWoodsSaxon(ctx, species, A, Z, V0, r0, diff, kappa, beta,
                           beta3, so_V0, spin_orbit));
  NCGM_CUDA(cudaStreamSynchronize(ctx->stream));
  return NCGM_OK;
  NCGM_GUARD_END
}

int ncgm_apply_h(ncgm_ctx *ctx, int species, const double *X, double *Y,
                 int ncols, int precision) {
  NCGM_GUARD_BEGIN
  if (!ctx || species < 0 || species > 1 || !X || !Y || ncols < 1 ||
      ncols > ctx->max_cols ||
      (precision != NCGM_FP64 && precision != NCGM_FP32)) {
    setError("ncgm_apply_h: bad argument (species, pointers, ncols <= "
             "max_cols, precision)");
    return NCGM_ERR_ARG;
  }
  if (!ctx->sp[species].ready) {
    setError("ncgm_apply_h: fields not set for this species");
    return NCGM_ERR_ARG;
  }
  const size_t cnt = ctx->N * (size_t)ncols; // complex entries
  const bool dX = isDevicePtr(X), dY = isDevicePtr(Y);
  // Host in and out with several columns: a three-stage pipeline over
  // column chunks of ~16 MB (copy in on one stream, convert and apply on the
  // context stream, copy out on a third), so the host<->device copies of
  // consecutive chunks overlap each other and the compute. Every column is
  // computed by the same kernels as in one launch (columns are independent),
  // so the results are identical.
  // NCGM_PIPE_CHUNK_MB sets the chunk size (default 16 MB)
  size_t chunkBytes = (size_t)16 << 20;
  if (const char *e = std::getenv("NCGM_PIPE_CHUNK_MB")) {
    const long v = std::atol(e);
    if (v >= 1 && v <= 4096) chunkBytes = (size_t)v << 20;
  }
  const int chunkCols = std::max<int>(
      1, (int)std::min<size_t>(ncols, chunkBytes /
                                          (ctx->N * sizeof(double2))));
  if (!dX && !dY && ncols > chunkCols) {
    const int nch = (ncols + chunkCols - 1) / chunkCols;
    if (!ctx->xin)
      NCGM_CUDA(cudaStreamCreateWithFlags(&ctx->xin, cudaStreamNonBlocking));
    if (!ctx->xout)
      NCGM_CUDA(cudaStreamCreateWithFlags(&ctx->xout, cudaStreamNonBlocking));
    while ((int)ctx->xev.size() < 2 * nch + 1) {
      cudaEvent_t e;
      NCGM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      ctx->xev.push_back(e);
    }
    auto *Xs = static_cast<double2 *>(ctx->buf(3, cnt * sizeof(double2)));
    auto *Ys = static_cast<double2 *>(ctx->buf(4, cnt * sizeof(double2)));
    float2 *x32 = nullptr, *y32 = nullptr;
    if (precision == NCGM_FP32) {
      x32 = static_cast<float2 *>(ctx->buf(5, cnt * sizeof(float2)));
      y32 = static_cast<float2 *>(ctx->buf(6, cnt * sizeof(float2)));
    }
    if (!Xs || !Ys || (precision == NCGM_FP32 && (!x32 || !y32)))
      return NCGM_ERR_NOMEM;
    // the copy streams start after earlier work on the context stream
    NCGM_CUDA(cudaEventRecord(ctx->xev[0], ctx->stream));
    NCGM_CUDA(cudaStreamWaitEvent(ctx->xin, ctx->xev[0], 0));
    NCGM_CUDA(cudaStreamWaitEvent(ctx->xout, ctx->xev[0], 0));
    const double2 *Xh = reinterpret_cast<const double2 *>(X);
    double2 *Yh = reinterpret_cast<double2 *>(Y);
    for (int c = 0; c < nch; ++c) {
      const int c0 = c * chunkCols, cc = std::min(chunkCols, ncols - c0);
      const size_t off = (size_t)c0 * ctx->N, len = (size_t)cc * ctx->N;
      cudaEvent_t in = ctx->xev[1 + 2 * c], done = ctx->xev[2 + 2 * c];
      NCGM_CUDA(cudaMemcpyAsync(Xs + off, Xh + off, len * sizeof(double2),
                                cudaMemcpyHostToDevice, ctx->xin));
      NCGM_CUDA(cudaEventRecord(in, ctx->xin));
      NCGM_CUDA(cudaStreamWaitEvent(ctx->stream, in, 0));
      if (precision == NCGM_FP64) {
        applyH64(ctx, species, Xs + off, Ys + off, cc, 0.0, ctx->stream);
      } else {
        convert64to32(Xs + off, x32 + off, len, ctx->stream);
        applyH32(ctx, species, x32 + off, y32 + off, cc, 0.f, ctx->stream);
        convert32to64(y32 + off, Ys + off, len, ctx->stream);
      }
      NCGM_CUDA(cudaGetLastError());
      NCGM_CUDA(cudaEventRecord(done, ctx->stream));
      NCGM_CUDA(cudaStreamWaitEvent(ctx->xout, done, 0));
      NCGM_CUDA(cudaMemcpyAsync(Yh + off, Ys + off, len * sizeof(double2),
                                cudaMemcpyDeviceToHost, ctx->xout));
    }
    NCGM_CUDA(cudaStreamSynchronize(ctx->xout));
    NCGM_CUDA(cudaStreamSynchronize(ctx->stream));
    return NCGM_OK;
  }
  const double2 *Xd = reinterpret_cast<const double2 *>(X);
  double2 *Yd = reinterpret_cast<double2 *>(Y);
  if (!dX) {
    double2 *s = static_cast<double2 *>(ctx->buf(3, cnt * sizeof(double2)));
    if (!s) return NCGM_ERR_NOMEM;
    NCGM_CUDA(cudaMemcpyAsync(s, X, cnt * sizeof(double2),
                              cudaMemcpyHostToDevice, ctx->stream));
    Xd = s;
  }
  if (!dY) {
    Yd = static_cast<double2 *>(ctx->buf(4, cnt * sizeof(double2)));
    if (!Yd) return NCGM_ERR_NOMEM;
  }
  if (precision == NCGM_FP64) {
    applyH64(ctx, species, Xd, Yd, ncols, 0.0, ctx->stream);
  } else {
    float2 *x32 = static_cast<float2 *>(ctx->buf(5, cnt * sizeof(float2)));
    float2 *y32 = static_cast<float2 *>(ctx->buf(6, cnt * sizeof(float2)));
    if (!x32 || !y32) return NCGM_ERR_NOMEM;
    convert64to32(Xd, x32, cnt, ctx->stream);
    applyH32(ctx, species, x32, y32, ncols, 0.f, ctx->stream);
    convert32to64(y32, Yd, cnt, ctx->stream);
  }
  NCGM_CUDA(cudaGetLastError());
  if (!dY)
    NCGM_CUDA(cudaMemcpyAsync(Y, Yd, cnt * sizeof(double2),
                              cudaMemcpyDeviceToHost, ctx->stream));
  NCGM_CUDA(cudaStreamSynchronize(ctx->stream));
  return NCGM_OK;
  NCGM_GUARD_END
}

int ncgm_apply_h_device(ncgm_ctx *ctx, int species, const void *X, void *Y,
                        int ncols, int precision, double shift) {
  NCGM_GUARD_BEGIN
  if (!ctx || species < 0 || species > 1 || !X || !Y || ncols < 1 ||
      ncols > ctx->max_cols ||
      (precision != NCGM_FP64 && precision != NCGM_FP32)) {
    setError("ncgm_apply_h_device: bad argument");
    return NCGM_ERR_ARG;
  }
  if (!ctx->sp[species].ready) {
    setError("ncgm_apply_h_device: fields not set for this species");
    return NCGM_ERR_ARG;
  }
  if (precision == NCGM_FP64)
    applyH64(ctx, species, static_cast<const double2 *>(X),
             static_cast<double2 *>(Y), ncols, shift, ctx->stream);
  else
    applyH32(ctx, species, static_cast<const float2 *>(X),
             static_cast<float2 *>(Y), ncols, (float)shift, ctx->stream);
  NCGM_CUDA(cudaGetLastError());
  return NCGM_OK;
  NCGM_GUARD_END
}

int ncgm_set_stream(ncgm_ctx *ctx, void *stream) {
  if (!ctx) {
    setError("ncgm_set_stream: null context");
    return NCGM_ERR_ARG;
  }
  if (stream) {
    if (!ctx->ownStream) ctx->ownStream = ctx->stream;
    ctx->stream = static_cast<cudaStream_t>(stream);
  } else if (ctx->ownStream) {
    ctx->stream = ctx->ownStream;
  }
  return NCGM_OK;
}

} // extern "C"
