// mcx_tcmlp.cu -- batched evaluation of the learned proposal's network
// (mcx_mlp_forward): on the 5th-generation tensor cores (k_mlp_tc:
// tcgen05.mma, accumulators in TMEM; mcx_tcmlp.cuh) or with the warp-level
// mma.sync network of the learned passes (k_mlp_warp; mcx_mlp.cuh).  No
// counterpart in the reference.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mcx_kernels.cuh"
#include "mcx_tcmlp.cuh"

namespace mcx {

constexpr int kTcThreads = 128;
constexpr int kTcFwdSmem = kTcWBytes + kTcXBytes + kTcHBytes + 64;
constexpr uint32_t kTcFwdCols = 64;  // one tile's accumulators (64 FP32 columns)

// One row of network inputs (19 floats) as 32 BF16, packed in pairs.
__device__ __forceinline__ void pack_inputs(const float *in, bool live, uint32_t w[16]) {
#pragma unroll
  for (int q = 0; q < 16; q++) {
    const float a = live && 2 * q < 19 ? in[2 * q] : 0.f;
    const float b = live && 2 * q + 1 < 19 ? in[2 * q + 1] : 0.f;
    w[q] = pack_bf16(a, b);
  }
}

// Persistent CTAs over tiles of 128 rows; thread t is row t of a tile.
__global__ void __launch_bounds__(kTcThreads, 1) k_mlp_tc(const uint8_t *mlp, const float *in, int n, float *out,
                                                          unsigned *err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  uint8_t *W = sm, *X = sm + kTcWBytes, *H = X + kTcXBytes;
  uint64_t *bar = reinterpret_cast<uint64_t *>(H + kTcHBytes);
  uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 1);
  const int t = threadIdx.x;
  tc_load_weights(mlp, W, kTcThreads);
  if (t == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (t < 32) tc_alloc(slot, kTcFwdCols);
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  uint32_t phase = 0;
#pragma unroll 1
  for (int tile = blockIdx.x; tile * 128 < n; tile += gridDim.x) {
    const int row = tile * 128 + t;
    uint32_t w[16];
    pack_inputs(in + (size_t)row * 19, row < n, w);
    tc_store_row32(X, t, w);
    fence_proxy_async();
    __syncthreads();
    float y[2][4];
    if (!tc_mlp(W, X, H, 1, tmem, bar, phase, y, err)) break;
    if (row < n)
#pragma unroll
      for (int q = 0; q < 4; q++) out[(size_t)row * 4 + q] = y[0][q];
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (t < 32) tc_dealloc(tmem, kTcFwdCols);
}

// The same network with the learned passes' warp-level code: each warp
// evaluates 64 rows (mlp_warp).
constexpr int kWarpFwdSmem = kMlpBytes + (kTcThreads / 32) * (64 * kXs * 2 + 64 * 4 * 4);

__global__ void __launch_bounds__(kTcThreads) k_mlp_warp(const uint8_t *mlp, const float *in, int n, float *out) {
  extern __shared__ __align__(16) uint8_t sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint8_t *W = sm;
  __nv_bfloat16 *X = reinterpret_cast<__nv_bfloat16 *>(sm + kMlpBytes) + (size_t)warp * 64 * kXs;
  float *Y = reinterpret_cast<float *>(sm + kMlpBytes + (kTcThreads / 32) * 64 * kXs * 2) + (size_t)warp * 64 * 4;
  for (int i = threadIdx.x; i < kMlpBytes / 16; i += kTcThreads)
    reinterpret_cast<int4 *>(W)[i] = reinterpret_cast<const int4 *>(mlp)[i];
  __syncthreads();
  const int warps = gridDim.x * (kTcThreads / 32);
#pragma unroll 1
  for (int base = (blockIdx.x * (kTcThreads / 32) + warp) * 64; base < n; base += warps * 64) {
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int row = base + 2 * lane + h;
      uint32_t w[16];
      pack_inputs(in + (size_t)row * 19, row < n, w);
      uint32_t *r = reinterpret_cast<uint32_t *>(X + (size_t)(2 * lane + h) * kXs);
#pragma unroll
      for (int q = 0; q < 16; q++) r[q] = w[q];
    }
    __syncwarp();
    mlp_warp(W, X, Y);
    __syncwarp();
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int row = base + 2 * lane + h;
      if (row < n)
#pragma unroll
        for (int q = 0; q < 4; q++) out[(size_t)row * 4 + q] = Y[(2 * lane + h) * 4 + q];
    }
    __syncwarp();
  }
}

cudaError_t launch_mlp_forward(const uint8_t *mlp, const float *in, int n, float *out, int tensor_cores,
                               unsigned *err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (tensor_cores) {
    cudaError_t r = cudaFuncSetAttribute(k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcFwdSmem);
    if (r != cudaSuccess) return r;
    const int tiles = (n + 127) / 128;
    k_mlp_tc<<<tiles < nsm ? tiles : nsm, kTcThreads, kTcFwdSmem, st>>>(mlp, in, n, out, err);
  } else {
    cudaError_t r = cudaFuncSetAttribute(k_mlp_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, kWarpFwdSmem);
    if (r != cudaSuccess) return r;
    const int blocks = (n + 255) / 256;
    k_mlp_warp<<<blocks < 4 * nsm ? blocks : 4 * nsm, kTcThreads, kWarpFwdSmem, st>>>(mlp, in, n, out);
  }
  return cudaGetLastError();
}

}  // namespace mcx
