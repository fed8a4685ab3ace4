// Learned preconditioner of the GCG correction step (see k_learned.cu).
#pragma once
#include "ncgm_internal.cuh"

namespace ncgm {

// Initial corrections d0 = N(r) of the correction-form PCG for `ncols`
// columns: r = x lam - A x from the FP64 block X (N x ncols, ld N), A X (same
// layout, shift removed) and lam (device, ncols). D0 receives d0 in the PCG
// precision (T = float or double, interleaved complex, ld N). Returns NCGM_OK
// or an error status (no network bound, allocation failure).
template <class T>
int lpInitialCorrection(ncgm_lp *lp, ncgm_ctx *ctx, int species,
                        const double2 *X, const double2 *AX, const double *lam,
                        double shift, int ncols, T *D0, cudaStream_t s);

} // namespace ncgm
