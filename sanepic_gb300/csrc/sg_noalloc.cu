// sg_noalloc.cu -- the noise weighting N^-1 on caller-owned device buffers,
// allocating no GPU memory at all.
//
// Who needs this: code that cannot call cudaMalloc -- a host application
// whose GPU memory is owned by its own pool or arena (a fixed-budget
// acquisition or streaming pipeline), a caller that is in the middle of
// capturing a CUDA graph (allocation calls are not allowed in a global-mode
// capture), or a real-time loop that cannot afford the implicit device
// synchronisation cudaMalloc/cudaFree may cause.  The regular path
// (sg_noise_filter) needs a context, whose set-up allocates.
//
// The only memory the kernel needs beyond its inputs and outputs is the FFT
// twiddle table of the tile length.  It lives in the file-scope array below,
// sized for the largest supported tile (ns = 131072 samples: 64 + 1024
// complex FP32 entries, 8.5 KiB), which every GPU that loads this library
// holds until the process exits.  Host code never dereferences the array's
// name (on the host it is only a stand-in symbol); the first call on each
// device resolves its device address with cudaGetSymbolAddress, with that
// device current, and caches it, and the first call for each tile length
// sets that kernel's launch attributes (and may load it).  So make one call
// per device and tile length before any stream capture begins.  All calls share the table and rewrite it
// for their own tile length, so two calls that overlap on the GPU (different
// streams, different lengths) race on it; nothing in it has to start at zero.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <mutex>

#include "../../include/sanepic_gpu.h"
#include "sg_kernels.h"

namespace {

constexpr long kNoAllocMaxNs = 131072;
constexpr int kTwLoN = 64;
constexpr int kScratchEntries = kTwLoN + (int)(kNoAllocMaxNs / 2 / kTwLoN);

// W_M^j for j < 64, then W_M^{64 j} for j < M/64 (M = ns/2).
static __device__ __align__(256) cplx<float> g_noalloc_twiddles[kScratchEntries];

__global__ void k_fill_twiddles(int M) {
  const int n = kTwLoN + M / kTwLoN;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double j = i < kTwLoN ? (double)i : (double)kTwLoN * (double)(i - kTwLoN);
    double s, c;
    sincospi(2.0 * j / (double)M, &s, &c);
    g_noalloc_twiddles[i] = cplx<float>{(float)c, (float)-s};
  }
}

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

}  // namespace

extern "C" int sg_noise_filter_noalloc(const float* in, float* out, const float* filt, long ns,
                                       long ntiles, long tiles_per_filter, void* stream) {
  if (!in || !out || !filt || ntiles < 1 || tiles_per_filter < 1) return SG_ERR_ARG;
  if (ns < 256 || (ns & (ns - 1)) != 0 || ns > kNoAllocMaxNs) return SG_ERR_UNSUPPORTED;
  // every tile index is below ntiles, so a larger group size only ever selects
  // row 0: clamp it before it is narrowed to the kernel's int
  if (tiles_per_filter > ntiles) tiles_per_filter = ntiles;
  if (tiles_per_filter > INT_MAX) return SG_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SG_ERR_CUDA;
  void* addr = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_twiddles) != cudaSuccess) return SG_ERR_CUDA;
      g_scratch_addr[dev] = p;
    }
    addr = g_scratch_addr[dev];
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const long M = ns / 2;
  int logm = 0;
  while ((1L << logm) < M) logm++;
  const int S = (int)(M / 8192 > 1 ? M / 8192 : 1);
  const int ncl = sg::filter_max_clusters<float>(logm, S);
  if (ncl <= 0) return SG_ERR_CUDA;
  k_fill_twiddles<<<(kTwLoN + M / kTwLoN + 255) / 256, 256, 0, st>>>((int)M);
  if (cudaGetLastError() != cudaSuccess) return SG_ERR_CUDA;
  sg::FilterArgs<float> a{};
  a.ntiles = ntiles;
  a.nseg = (int)tiles_per_filter;
  a.mode = sg::kLoadTod;
  a.filt_abs = 0;
  a.tod = in;
  a.filt = filt;
  a.out = out;
  a.tw_lo = reinterpret_cast<const cplx<float>*>(addr);
  a.tw_hi = reinterpret_cast<const cplx<float>*>(addr) + kTwLoN;
  const double a1 = 6.2831853071795864769252867665590057683943387987502 / (double)ns;
  a.wn1 = cplx<float>{(float)std::cos(a1), (float)-std::sin(a1)};
  const int launch_cl = (int)(ntiles < ncl ? ntiles : ncl);
  if (sg::filter_launch<float>(a, logm, S, launch_cl, st) != cudaSuccess) return SG_ERR_CUDA;
  return SG_OK;
}
