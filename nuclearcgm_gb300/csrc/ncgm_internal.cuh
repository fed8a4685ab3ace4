// Internal declarations of the GB300 (sm_103a) nuclearcgm library: device
// context, error plumbing and kernel entry points shared by the .cu files.
#pragma once
#include "../../include/ncgm.h"

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace ncgm {

// Thread-local text of the last failure (ncgm_last_error).
void setError(const std::string &msg);

#define NCGM_CUDA(call)                                                        \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      ::ncgm::setError(std::string(#call) + ": " + cudaGetErrorString(e_));    \
      return NCGM_ERR_CUDA;                                                    \
    }                                                                          \
  } while (0)

#define NCGM_TRY(call)                                                         \
  do {                                                                         \
    int s_ = (call);                                                           \
    if (s_ != NCGM_OK) return s_;                                              \
  } while (0)

// Per-point Hamiltonian coefficients (matrix-free form of the reference
// term list). For each lattice point p:
//   c[0] = U + UC + 7.5 f / h^2     (diagonal, shift added at apply time)
//   c[1] = f / h^2                  (multiplies the 4/3, -1/12 neighbours)
//   c[2..4] = -grad_a f / (12 h)    (non-local kinetic, per axis)
//   c[5..7] = W_a / (12 h)          (spin-orbit field, per axis)
// stored as two 4-vectors per point: lo = c[0..3], hi = c[4..7].
struct SpeciesFields {
  double *coef64 = nullptr; // ns x 8
  float *coef32 = nullptr;  // ns x 8
  float *coef32s = nullptr; // 2 x ns x 4: lo halves of all points, then hi
  bool ready = false;
};

// Device workspace arena: one allocation, carved by ncgm_ctx on demand.
struct Arena {
  char *base = nullptr;
  size_t cap = 0, off = 0;
};

} // namespace ncgm

struct ncgm_ctx {
  int n = 0;
  double a = 0, h = 0;
  int max_cols = 0;
  size_t ns = 0, N = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t ownStream = nullptr; // set while a caller stream is in use
  ncgm::SpeciesFields sp[2];
  // scratch buffers, grown on demand (device)
  std::vector<std::pair<void *, size_t>> bufs;
  void *buf(int slot, size_t bytes);
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  ncgm_lp *lp = nullptr; // learned preconditioner (not owned)
  // host-buffer applies: copy-in / copy-out streams and their events,
  // created on first use
  cudaStream_t xin = nullptr, xout = nullptr;
  std::vector<cudaEvent_t> xev;
};

namespace ncgm {

// ---- Hamiltonian (k_hamiltonian.cu) -------------------------------------
int buildCoefficients(ncgm_ctx *ctx, int species, const double *f,
                      const double *gradf, const double *U, const double *W,
                      const double *UC);
int buildWoodsSaxon(ncgm_ctx *ctx, int species, int A, int Z, double V0,
                    double r0, double diff, double kappa, double beta,
                    double beta3, double so_V0, int spin_orbit);
// Y = (H + shift) X on device buffers, ncols columns, leading dim N.
void applyH64(ncgm_ctx *ctx, int species, const double2 *X, double2 *Y,
              int ncols, double shift, cudaStream_t s);
void applyH32(ncgm_ctx *ctx, int species, const float2 *X, float2 *Y,
              int ncols, float shift, cudaStream_t s);
// Non-zero when a stencil's bounded wait gave up since the last reset.
int stencilErrorFlag();

void convert64to32(const double2 *in, float2 *out, size_t count,
                   cudaStream_t s);
void convert32to64(const float2 *in, double2 *out, size_t count,
                   cudaStream_t s);

} // namespace ncgm
