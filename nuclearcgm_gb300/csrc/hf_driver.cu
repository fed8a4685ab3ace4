// Placeholder translation unit for the eigensolver and self-consistent driver
// entry points; filled in by the GCG / HF implementation.
#include "ncgm_internal.cuh"

extern "C" int ncgm_hf_run(const ncgm_hf_config *, ncgm_hf_result *, double *,
                           double *, double *, double *, double *) {
  ncgm::setError("ncgm_hf_run: not available in this build");
  return NCGM_ERR_ARG;
}
