// mcx_tcmlp.cuh -- the learned proposal's network on the 5th-generation
// tensor cores: tcgen05.mma with operands in shared memory and FP32
// accumulators in tensor memory (TMEM), read back with tcgen05.ld (no
// counterpart in the reference).
//
// One CTA of 128 threads evaluates the 19 -> 64 -> 64 -> 4 network for a tile
// of M = 128 rows (sites): thread t owns row t, which is TMEM lane t, so
// tcgen05.ld of the 32x32b shape hands every thread its own row's
// accumulators (warp w reads lanes 32w .. 32w + 31).  Per layer one elected
// thread issues the K = 16 MMAs (kind::f16: BF16 operands, FP32 accumulate)
// and commits them to an mbarrier; the other threads wait on it (bounded),
// load their row's accumulators, add the bias, apply the GELU in packed BF16
// (gelu_bf16x2, mcx_mlp.cuh: the same arithmetic as the mma.sync path) and
// store the BF16 activations as the next layer's A operand.
//
// Operand layout in shared memory: the canonical K-major layout without
// swizzle -- 8 x 16-byte core matrices (8 rows x 8 BF16 along K), stored
// [row group][K group][8 rows][8 elements]: the K-adjacent core matrices are
// 128 bytes apart (the descriptor's leading-dimension offset) and the
// row-adjacent groups (K / 8) x 128 bytes apart (its stride offset).  The
// weights are the B operands, N x K (transposed, as in mcx_mlp.cuh); layer 3
// runs at N = 16 (outputs 8 .. 15 zero).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "mcx_mlp.cuh"
#include "mcx_tma.cuh"

namespace mcx {

// Canonical-layout byte offset of element (row, k) of a K-major operand with
// K columns.
__host__ __device__ constexpr int tc_off(int row, int k, int K) {
  return (row >> 3) * (K >> 3) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}

// Shared-memory image of the network for the tensor-core path (bytes).
constexpr int kTcW1 = 0;                     // 64 x 32 BF16
constexpr int kTcW2 = kTcW1 + 64 * 32 * 2;   // 64 x 64 BF16
constexpr int kTcW3 = kTcW2 + 64 * 64 * 2;   // 16 x 64 BF16 (rows 8 .. 15 zero)
constexpr int kTcB1 = kTcW3 + 16 * 64 * 2;   // 64 floats
constexpr int kTcB2 = kTcB1 + 64 * 4;        // 64 floats
constexpr int kTcB3 = kTcB2 + 64 * 4;        // 8 floats
constexpr int kTcWBytes = 15360;             // rounded up to 1 KB
static_assert(kTcB3 + 8 * 4 <= kTcWBytes, "network image");
constexpr int kTcXBytes = 128 * 32 * 2;      // one input tile (M = 128, K = 32)
constexpr int kTcHBytes = 128 * 64 * 2;      // one activation tile (M = 128, K = 64)

// Shared-memory matrix descriptor (tcgen05): start address, leading- and
// stride-dimension byte offsets (all >> 4), version 1, no swizzle.
__device__ __forceinline__ uint64_t tc_desc(const void *p, uint32_t lbo, uint32_t sbo) {
  const uint64_t a = (smem_u32(p) >> 4) & 0x3FFFu;
  return a | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N and M.
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
      : "memory");
}

// Arrives on `bar` once every tcgen05 operation this thread issued has
// completed.
__device__ __forceinline__ void tc_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// TMEM columns for the CTA (one warp: every lane calls); the base address is
// written to *slot.
__device__ __forceinline__ void tc_alloc(uint32_t *slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc_dealloc(uint32_t base, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// The network image in shared memory from the mma.sync layout of mcx_mlp.cuh
// (W1t [64][kW1s], W2t [64][kW2s], W3t [8][kW3s] BF16 rows n holding k; the
// biases): every thread of the CTA takes a share.
__device__ __forceinline__ void tc_load_weights(const uint8_t *src, uint8_t *W, int nthreads) {
  const uint16_t *w1 = reinterpret_cast<const uint16_t *>(src + kMlpW1);
  const uint16_t *w2 = reinterpret_cast<const uint16_t *>(src + kMlpW2);
  const uint16_t *w3 = reinterpret_cast<const uint16_t *>(src + kMlpW3);
  for (int i = threadIdx.x; i < 64 * 32; i += nthreads) {
    const int n = i >> 5, k = i & 31;
    *reinterpret_cast<uint16_t *>(W + kTcW1 + tc_off(n, k, 32)) = w1[n * kW1s + k];
  }
  for (int i = threadIdx.x; i < 64 * 64; i += nthreads) {
    const int n = i >> 6, k = i & 63;
    *reinterpret_cast<uint16_t *>(W + kTcW2 + tc_off(n, k, 64)) = w2[n * kW2s + k];
  }
  for (int i = threadIdx.x; i < 16 * 64; i += nthreads) {
    const int n = i >> 6, k = i & 63;
    *reinterpret_cast<uint16_t *>(W + kTcW3 + tc_off(n, k, 64)) = n < 8 ? w3[n * kW3s + k] : (uint16_t)0;
  }
  const float *b = reinterpret_cast<const float *>(src + kMlpB1);
  float *bd = reinterpret_cast<float *>(W + kTcB1);
  for (int i = threadIdx.x; i < 64 + 64 + 8; i += nthreads) bd[i] = b[i];
}

// Row t of an input tile (K = 32): 32 BF16 (the 19 inputs then zeros) as 16
// packed words, stored as four 16-byte pieces.
__device__ __forceinline__ void tc_store_row32(uint8_t *X, int t, const uint32_t w[16]) {
#pragma unroll
  for (int g = 0; g < 4; g++)
    *reinterpret_cast<uint4 *>(X + tc_off(t, 8 * g, 32)) = make_uint4(w[4 * g], w[4 * g + 1], w[4 * g + 2], w[4 * g + 3]);
}

// Issues one layer for `ntiles` tiles: D[tile] (TMEM columns dcol + tile *
// dstride) = A[tile] (M = 128, K) x B^T (N x K); one thread.
__device__ __forceinline__ void tc_issue_layer(uint32_t tmem, int dcol, int dstride, const uint8_t *A, int abytes,
                                               int ntiles, const uint8_t *B, int K, int N) {
  const uint32_t idesc = tc_idesc(128, N);
#pragma unroll 1
  for (int tile = 0; tile < ntiles; tile++)
#pragma unroll 1
    for (int ks = 0; ks < K / 16; ks++)
      tc_mma(tmem + (uint32_t)(dcol + tile * dstride), tc_desc(A + tile * abytes + ks * 256, 128, (K / 8) * 128),
             tc_desc(B + ks * 256, 128, (K / 8) * 128), idesc, ks > 0);
}

// Accumulators of one hidden layer (64 columns at TMEM column `col` of this
// thread's lane) -> bias -> twice the GELU in BF16 -> row t of the next
// layer's A operand H (K = 64).
__device__ __forceinline__ void tc_hidden_to_smem(uint32_t lane_addr, int col, const float *bias, uint8_t *H, int t) {
#pragma unroll
  for (int c = 0; c < 4; c++) {
    float v[16];
    tc_ld16(lane_addr + (uint32_t)(col + 16 * c), v);
    uint32_t w[8];
#pragma unroll
    for (int i = 0; i < 8; i++) w[i] = gelu_bf16x2(v[2 * i] + bias[16 * c + 2 * i], v[2 * i + 1] + bias[16 * c + 2 * i + 1]);
    *reinterpret_cast<uint4 *>(H + tc_off(t, 16 * c, 64)) = make_uint4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<uint4 *>(H + tc_off(t, 16 * c + 8, 64)) = make_uint4(w[4], w[5], w[6], w[7]);
  }
}

// A wait ran out: set the error flag and wait (bounded) once more for the
// MMAs in flight, so that the caller can free the TMEM they write.
__device__ __forceinline__ void tc_give_up(uint64_t *bar, uint32_t phase, unsigned *err) {
  if (threadIdx.x == 0) {
    atomicOr(err, 4u);
    mbar_wait(bar, phase ^ 1u);
  }
  __syncthreads();
}

// The network for `ntiles` (1 or 2) tiles of 128 rows whose inputs are in X
// (ntiles x kTcXBytes, already stored and made visible: fence_proxy_async +
// __syncthreads by the caller), with H (ntiles x kTcHBytes) as activation
// space and TMEM columns [tmem, tmem + 64 ntiles).  Every one of the 128
// threads calls; thread t receives the 4 outputs of row t of each tile in
// y[tile].  *phase is the mbarrier's parity, advanced per layer.  Returns
// false when a wait ran out (the error flag is set; the caller stops).
__device__ __forceinline__ bool tc_mlp(const uint8_t *W, const uint8_t *X, uint8_t *H, int ntiles, uint32_t tmem,
                                       uint64_t *bar, uint32_t &phase, float y[2][4], unsigned *err) {
  const int t = threadIdx.x;
  const uint32_t lane_addr = tmem + ((uint32_t)((t >> 5) * 32) << 16);
  const float *b1 = reinterpret_cast<const float *>(W + kTcB1);
  const float *b2 = reinterpret_cast<const float *>(W + kTcB2);
  const float *b3 = reinterpret_cast<const float *>(W + kTcB3);
  int ok = 1;
  // layer 1
  if (t == 0) {
    tc_fence_after();
    tc_issue_layer(tmem, 0, 64, X, kTcXBytes, ntiles, W + kTcW1, 32, 64);
    tc_commit(bar);
  }
  ok = mbar_wait(bar, phase);
  phase ^= 1u;
  tc_fence_after();
  if (ok)
    for (int tile = 0; tile < ntiles; tile++) tc_hidden_to_smem(lane_addr, 64 * tile, b1, H + tile * kTcHBytes, t);
  fence_proxy_async();
  tc_fence_before();
  if (!__syncthreads_and(ok)) {
    tc_give_up(bar, phase, err);
    return false;
  }
  // layer 2
  if (t == 0) {
    tc_fence_after();
    tc_issue_layer(tmem, 0, 64, H, kTcHBytes, ntiles, W + kTcW2, 64, 64);
    tc_commit(bar);
  }
  ok = mbar_wait(bar, phase);
  phase ^= 1u;
  tc_fence_after();
  // every thread's loads of layer 2 and its stores into H (the operand of the
  // MMAs just completed) come before the next barrier
  if (ok)
    for (int tile = 0; tile < ntiles; tile++) tc_hidden_to_smem(lane_addr, 64 * tile, b2, H + tile * kTcHBytes, t);
  fence_proxy_async();
  tc_fence_before();
  if (!__syncthreads_and(ok)) {
    tc_give_up(bar, phase, err);
    return false;
  }
  // layer 3 (N = 16; outputs 0 .. 3 used)
  if (t == 0) {
    tc_fence_after();
    tc_issue_layer(tmem, 0, 64, H, kTcHBytes, ntiles, W + kTcW3, 64, 16);
    tc_commit(bar);
  }
  ok = mbar_wait(bar, phase);
  phase ^= 1u;
  tc_fence_after();
  if (ok)
    for (int tile = 0; tile < ntiles; tile++) {
      float v[16];
      tc_ld16(lane_addr + (uint32_t)(64 * tile), v);
#pragma unroll
      for (int q = 0; q < 4; q++) y[tile][q] = v[q] + b3[q];
    }
  tc_fence_before();
  if (!__syncthreads_and(ok)) {
    tc_give_up(bar, phase, err);
    return false;
  }
  return true;
}

}  // namespace mcx
