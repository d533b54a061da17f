// sg_filter_spec64.cu -- the noise filter split at the spectrum (double): forward real FFT
// to a half spectrum, or inverse real FFT from one (kernel in sg_filter.cuh).
#include "sg_filter.cuh"

namespace sg {

template <>
cudaError_t filter_spec_launch<double>(const FilterArgs<double>& a, int logm, int S, int nclusters,
                                    cudaStream_t st) {
  const int logr = (logm + 1) / 2, logc = logm / 2;
  const bool out = a.spec_out != nullptr;
  if (out == (a.spec_in != nullptr)) return cudaErrorInvalidValue;  // exactly one of them
#define SG_CASE(TT, LR, LC, SS)                                        \
  if (logr == LR && logc == LC && S == SS)                             \
    return out ? launch_one<TT, LR, LC, SS, kSpecOut>(a, nclusters, st) \
               : launch_one<TT, LR, LC, SS, kSpecIn>(a, nclusters, st);
  SG_FILTER_CASES_F64(SG_CASE)
#undef SG_CASE
  return cudaErrorInvalidValue;
}

}  // namespace sg
