// cleanup.cu -- PSD cleanup and Davidson entry points (kernels land with the cleanup stage).
#include "ss_common.cuh"
#include "ss_context.cuh"
extern "C" {
int ss_psd_clean(ss_ctx*, double*, int, int, int, int, uint64_t, int*) {
  ss_set_error_msg("ss_psd_clean: not available in this build");
  return SS_ERR_UNSUPPORTED;
}
int ss_davidson(ss_ctx*, const double*, int, int, double, int, double*, double*) {
  ss_set_error_msg("ss_davidson: not available in this build");
  return SS_ERR_UNSUPPORTED;
}
}
