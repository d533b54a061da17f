// sg_filter.cu -- the fused noise filter's launches (kernel in sg_filter.cuh)
#include <algorithm>
#include <vector>

#include "sg_filter.cuh"

namespace sg {

size_t filter_smem_bytes(int logm, int S, int esize) {
  const int logr = (logm + 1) / 2, logc = logm / 2;
  const size_t R = 1u << logr, C = 1u << logc, M = R * C;
  const size_t C2 = C >> ((logc + 1) / 2);
  const size_t buf = std::max(R * (C / S + 1), C * (R / S + 1));
  return (size_t)esize * 2 * (buf + kTwLo + M / kTwLo + R + C + C2);
}

// frequency k of every spectrum slot of the spectrum-split filter variants
// (the unit order of sg_filter.cuh), slot M the Nyquist bin
void spec_slot_freq(int logm, int S, std::vector<int>& kfreq) {
  const int logr = (logm + 1) / 2, logc = logm / 2;
  const long long R = 1LL << logr, C = 1LL << logc, M = R * C;
  const long long C1 = 1LL << ((logc + 1) / 2), Rs = R / S;
  kfreq.assign(M + 1, 0);
  for (long long s = 0; s < M; s++) {
    const long long t = s % Rs, j = (s / Rs) % S, rest = s / (Rs * S);
    const long long ka = rest % C1, i = rest / C1;
    const long long r = j * Rs + t;  // row list index -> row k1 (rows 0, R/2, then pairs)
    const long long p = r >> 1;
    const long long k1 = r == 0 ? 0 : (r == 1 ? R / 2 : ((r & 1) ? R - p : p));
    kfreq[s] = (int)(k1 + R * ka + R * C1 * i);
  }
  kfreq[M] = (int)M;
}

int filter_cluster_size(int logm, int esize) {
  const long M = 1L << logm;
  const long emax = esize == 4 ? 8192 : 4096;
  return (int)(M / emax > 1 ? M / emax : 1);
}

template <>
cudaError_t filter_launch<float>(const FilterArgs<float>& a, int logm, int S, int nclusters,
                                 cudaStream_t st) {
  const int logr = (logm + 1) / 2, logc = logm / 2;
#define SG_CASE(TT, LR, LC, SS) \
  if (logr == LR && logc == LC && S == SS) return launch_one<TT, LR, LC, SS, kFused>(a, nclusters, st);
  SG_FILTER_CASES_F32(SG_CASE)
#undef SG_CASE
  return cudaErrorInvalidValue;
}

template <>
cudaError_t filter_launch<double>(const FilterArgs<double>& a, int logm, int S, int nclusters,
                                  cudaStream_t st) {
  const int logr = (logm + 1) / 2, logc = logm / 2;
#define SG_CASE(TT, LR, LC, SS) \
  if (logr == LR && logc == LC && S == SS) return launch_one<TT, LR, LC, SS, kFused>(a, nclusters, st);
  SG_FILTER_CASES_F64(SG_CASE)
#undef SG_CASE
  return cudaErrorInvalidValue;
}

template <>
int filter_max_clusters<float>(int logm, int S) {
  const int logr = (logm + 1) / 2, logc = logm / 2;
#define SG_CASE(TT, LR, LC, SS) \
  if (logr == LR && logc == LC && S == SS) return max_clusters_one<TT, LR, LC, SS, kFused>();
  SG_FILTER_CASES_F32(SG_CASE)
#undef SG_CASE
  return 0;
}

template <>
int filter_max_clusters<double>(int logm, int S) {
  const int logr = (logm + 1) / 2, logc = logm / 2;
#define SG_CASE(TT, LR, LC, SS) \
  if (logr == LR && logc == LC && S == SS) return max_clusters_one<TT, LR, LC, SS, kFused>();
  SG_FILTER_CASES_F64(SG_CASE)
#undef SG_CASE
  return 0;
}

}  // namespace sg
