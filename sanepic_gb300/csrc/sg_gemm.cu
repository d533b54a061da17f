// sg_gemm.cu -- BF16 GEMM on the 5th-generation tensor cores for the learned
// preconditioner's MLP (no reference counterpart: the reference has no
// learned component).
//
//   C[M x N] (FP32)  = A[M x K] . B[N x K]^T        (beta = 0)
//   C[M x N] (FP32) += A[M x K] . B[N x K]^T        (beta = 1)
//
// A and B are row-major BF16 with K contiguous.  One CTA computes a 128 x BN
// tile: a TMA producer thread streams 128 x 64 (A) and BN x 64 (B) boxes with
// the 128-byte swizzle into a 4-stage shared-memory ring; one thread issues
// tcgen05.mma (kind::f16, BF16 inputs, FP32 accumulate) into a TMEM
// accumulator of 128 lanes x BN columns; stage reuse and the epilogue are
// ordered by mbarriers that tcgen05.commit arrives on; the four warps then
// read their 32 TMEM lanes with tcgen05.ld and store FP32 rows.
//
// Every mbarrier wait is bounded: on timeout the kernel records an error code
// in *err, skips the rest of its work, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <mutex>

#include <cstdint>

#include "sg_kernels.h"

namespace sg {

cudaError_t gemm_prepare();

namespace {

constexpr int kBM = 128, kBK = 64, kStages = 4, kGemmThreads = 128;
constexpr int kWaitLimit = 1 << 20;  // try_wait polls before giving up

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes)
               : "memory");
}

// true when the phase of parity `parity` has completed; false after the limit
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int i = 0; i < kWaitLimit; i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];\n" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// UMMA shared-memory descriptor of a K-major tile stored as TMA wrote it with
// the 128-byte swizzle: rows of 128 B, 8-row atoms 1024 B apart (SBO), start
// address >> 4 in bits 0-13, descriptor version 1 (bits 46-47), layout
// SWIZZLE_128B (2) in bits 61-63.  LBO is unused for this layout.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// instruction descriptor, kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 in bits 17-22, M >> 4 in
// bits 24-28
template <int BN>
__device__ __forceinline__ uint32_t idesc_bf16() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
         ((uint32_t)(kBM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}

// 32 lanes x 32 consecutive 32-bit columns: thread t of the warp gets lane
// (warp's base lane + t), columns col .. col+31
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, "
      "%29, %30, %31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

template <int BN>
constexpr size_t gemm_smem_bytes() {
  return 1024 + (size_t)kStages * (kBM * kBK * 2 + BN * kBK * 2) + 8 * (2 * kStages + 1) + 16;
}

template <int BN>
__global__ void __launch_bounds__(kGemmThreads, 1)
    k_gemm_bf16(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
                float* __restrict__ C, int ldc, int K, int beta, int* err) {
  constexpr int A_BYTES = kBM * kBK * 2, B_BYTES = BN * kBK * 2;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~uintptr_t(1023));
  uint8_t* sA = base;
  uint8_t* sB = base + kStages * A_BYTES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sB + kStages * B_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kStages + 1);
  const uint32_t full0 = smem_addr(bars), empty0 = full0 + 8 * kStages,
                 accum = full0 + 16 * kStages;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tm = blockIdx.x, tn = blockIdx.y;
  const int nk = K / kBK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; s++) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    mbar_init(accum, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  }
  __syncwarp();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_addr(tmem_slot)),
                 "r"(BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // TMA producer
    for (int kb = 0; kb < nk; kb++) {
      const int s = kb % kStages;
      if (kb >= kStages && !mbar_wait(empty0 + 8 * s, ((kb / kStages) - 1) & 1)) {
        atomicExch(err, 1);
        break;
      }
      mbar_expect_tx(full0 + 8 * s, A_BYTES + B_BYTES);
      tma_load_2d(smem_addr(sA + s * A_BYTES), &ta, kb * kBK, tm * kBM, full0 + 8 * s);
      tma_load_2d(smem_addr(sB + s * B_BYTES), &tb, kb * kBK, tn * BN, full0 + 8 * s);
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    const uint32_t idesc = idesc_bf16<BN>();
    for (int kb = 0; kb < nk; kb++) {
      const int s = kb % kStages;
      if (!mbar_wait(full0 + 8 * s, (kb / kStages) & 1)) {
        atomicExch(err, 2);
        break;
      }
      tc_fence_after();
      const uint32_t a0 = smem_addr(sA + s * A_BYTES), b0 = smem_addr(sB + s * B_BYTES);
#pragma unroll
      for (int k = 0; k < kBK / 16; k++)  // 16 BF16 = 32 bytes per MMA along K
        mma_bf16(tmem, desc_sw128(a0 + 32 * k), desc_sw128(b0 + 32 * k), idesc,
                 (kb > 0 || k > 0) ? 1u : 0u);
      mma_commit(empty0 + 8 * s);
    }
    mma_commit(accum);
  }
  __syncwarp();

  // epilogue: warp w owns TMEM lanes (rows) 32w .. 32w+31
  const bool ok = __all_sync(0xffffffffu, mbar_wait(accum, 0));  // warp-uniform for tcgen05.ld
  if (!ok && lane == 0) atomicExch(err, 3);
  tc_fence_after();
  if (ok) {
    const int row = tm * kBM + warp * 32 + lane;
    float* dst = C + (size_t)row * ldc + (size_t)tn * BN;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 32) {
      uint32_t r[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
      float4* d4 = reinterpret_cast<float4*>(dst + c0);
#pragma unroll
      for (int i = 0; i < 8; i++) {
        float4 v = make_float4(__uint_as_float(r[4 * i]), __uint_as_float(r[4 * i + 1]),
                               __uint_as_float(r[4 * i + 2]), __uint_as_float(r[4 * i + 3]));
        if (beta) {
          const float4 o = d4[i];
          v.x += o.x;
          v.y += o.y;
          v.z += o.z;
          v.w += o.w;
        }
        d4[i] = v;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(BN)
                 : "memory");
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// row-major BF16 [rows x cols] (cols contiguous), box of box_rows x 64
bool make_map(CUtensorMap* m, const void* ptr, int rows, int cols, int box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box,
            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the large dynamic shared-memory opt-in, once per device (before any graph
// capture uses the kernels); contexts on several host threads share it
std::mutex g_prepared_mu;
bool g_prepared[64] = {};

template <int BN>
cudaError_t launch_bn(const CUtensorMap& ta, const CUtensorMap& tb, float* C, int ldc, int M,
                      int N, int K, int beta, int* err, cudaStream_t st) {
  const size_t smem = gemm_smem_bytes<BN>();
  cudaError_t e = gemm_prepare();
  if (e != cudaSuccess) return e;
  dim3 grid(M / kBM, N / BN);
  k_gemm_bf16<BN><<<grid, kGemmThreads, smem, st>>>(ta, tb, C, ldc, K, beta, err);
  return cudaGetLastError();
}

}  // namespace

cudaError_t gemm_prepare() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(g_prepared_mu);
  if (dev >= 0 && dev < 64 && g_prepared[dev]) return cudaSuccess;
  e = cudaFuncSetAttribute(k_gemm_bf16<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)gemm_smem_bytes<128>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_gemm_bf16<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)gemm_smem_bytes<256>());
  if (e == cudaSuccess && dev >= 0 && dev < 64) g_prepared[dev] = true;
  return e;
}

bool gemm_shape_ok(int M, int N, int K) {
  return M > 0 && N > 0 && K > 0 && M % kBM == 0 && N % 128 == 0 && K % kBK == 0;
}

cudaError_t gemm_bf16(const void* A, const void* B, float* C, int M, int N, int K, int beta,
                      int* err, cudaStream_t st) {
  if (!gemm_shape_ok(M, N, K)) return cudaErrorInvalidValue;
  const int bn = (N % 256 == 0) ? 256 : 128;
  CUtensorMap ta, tb;
  if (!make_map(&ta, A, M, K, kBM) || !make_map(&tb, B, N, K, bn)) return cudaErrorInvalidValue;
  return bn == 256 ? launch_bn<256>(ta, tb, C, N, M, N, K, beta, err, st)
                   : launch_bn<128>(ta, tb, C, N, M, N, K, beta, err, st);
}

}  // namespace sg
