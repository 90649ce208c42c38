// mcx_mlp.cuh -- the learned proposal's network on the tensor cores, and its
// von Mises-Fisher mixture proposal (no counterpart in the reference).
//
// Network: 19 inputs (six neighbour directors, T) -> 64 -> 64 -> 4 outputs
// (mean axis mu, log kappa), GELU (tanh form) between layers, BF16 weights and
// activations, FP32 accumulation; the GELU itself in packed BF16 arithmetic.  One warp evaluates it for 64 sites as four
// 16-row tiles with mma.sync m16n8k16 (BF16 in, FP32 out); a layer's FP32
// accumulator fragments become the next layer's BF16 A fragments in
// registers, so only the inputs and the 4 outputs pass through shared memory.
//
// Shared-memory weight layout (also the device buffer's layout, bytes):
//   W1t [64][40] bf16   W1 transposed: row n holds k = 0..31 (19..31 zero), 8 pad
//   W2t [64][72] bf16   W2 transposed and halved (gelu_bf16x2 returns twice the GELU), 8 pad
//   W3t [ 8][72] bf16   W3 transposed and halved (n = 0..7, outputs 4..7 zero)
//   b1 [64], b2 [64], b3 [8] float
// The row pads keep the B-fragment loads of a warp on 32 distinct banks.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace mcx {

constexpr int kMlpIn = 32, kMlpH = 64, kMlpOut = 8;
constexpr int kW1s = 40, kW2s = 72, kW3s = 72, kXs = 40;
constexpr int kMlpW1 = 0;
constexpr int kMlpW2 = kMlpW1 + kMlpH * kW1s * 2;
constexpr int kMlpW3 = kMlpW2 + kMlpH * kW2s * 2;
constexpr int kMlpB1 = kMlpW3 + kMlpOut * kW3s * 2;
constexpr int kMlpB2 = kMlpB1 + kMlpH * 4;
constexpr int kMlpB3 = kMlpB2 + kMlpH * 4;
constexpr int kMlpBytes = kMlpB3 + kMlpOut * 4;  // 16032
constexpr float kLogKMin = -4.0f, kLogKMax = 6.0f;

__device__ __forceinline__ void mma_bf16(float d[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// GELU, tanh form: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))).
__device__ __forceinline__ float gelu(float x) {
  const float u = 0.7978845608028654f * fmaf(0.044715f * x * x, x, x);
  return 0.5f * x * (1.0f + tanh_approx(u));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&v);
}

// Twice the GELU of two FP32 pre-activations, evaluated in packed BF16
// arithmetic and returned packed (the next layer's operand).  Each step
// rounds to BF16:
//   x = bf16(a), x2 = x*x, t = x2*(c*0.044715) + c, u = x*t,
//   th = tanh(u) (hardware approximation), y = x*th + x
// with c = sqrt(2/pi) and the constants rounded to BF16.  y is exactly twice
// the GELU's h*th + h with h = x*0.5 (a power-of-two scale commutes with each
// rounding), and the next layer's weights are packed at half scale
// (pack_mlp_weights), so the products, and everything after them, are those
// of the GELU itself.  Half the SFU operations of the FP32 form.
__device__ __forceinline__ uint32_t gelu_bf16x2(float a, float b) {
  const uint32_t kC = 0x3F4C3F4Cu;    // bf16(0.7978845608) = 0.796875, twice
  const uint32_t kC3 = 0x3D123D12u;   // bf16(0.7978845608 * 0.044715) = 0.03564453125, twice
  const uint32_t x = pack_bf16(a, b);
  uint32_t x2, t, u, th, y;
  asm("mul.rn.bf16x2 %0, %1, %1;" : "=r"(x2) : "r"(x));
  asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(t) : "r"(x2), "r"(kC3), "r"(kC));
  asm("mul.rn.bf16x2 %0, %1, %2;" : "=r"(u) : "r"(x), "r"(t));
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(th) : "r"(u));
  asm("fma.rn.bf16x2 %0, %1, %2, %1;" : "=r"(y) : "r"(x), "r"(th));
  return y;
}

__device__ __forceinline__ uint32_t lds32(const uint8_t *p) { return *reinterpret_cast<const uint32_t *>(p); }

// B fragments of two adjacent n-tiles for one 16-wide k-tile, from a
// transposed weight block (row n holds the k values): four 8x8 matrices, rows
// n0..n0+7 at k and k+8, rows n0+8..n0+15 at k and k+8.  Lane l supplies the
// row address of matrix l/8; the result is {b0, b1} of n-tile n0/8 and of the
// next one, exactly the words two LDS.32 per fragment would read.
__device__ __forceinline__ void ldsm_b2(const uint8_t *wt, int stride_elems, int n0, int k0, uint32_t b[4]) {
  const int lane = threadIdx.x & 31;
  const int row = n0 + (lane & 7) + ((lane >> 4) << 3);
  const int col = k0 + (((lane >> 3) & 1) << 3);
  const uint32_t addr = (uint32_t)__cvta_generic_to_shared(wt + ((size_t)row * stride_elems + col) * 2);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(b[0]), "=r"(b[1]), "=r"(b[2]), "=r"(b[3])
               : "r"(addr));
}

// The network for 64 rows of X (bf16, row stride kXs) -> Y (64 x 4 floats),
// by one warp.  Rows are sites; all 32 lanes must call.
__device__ __forceinline__ void mlp_warp(const uint8_t *W, const __nv_bfloat16 *X, float *Y) {
  const int lane = threadIdx.x & 31, g = lane >> 2, tg = lane & 3;
  const uint8_t *W1 = W + kMlpW1, *W2 = W + kMlpW2, *W3 = W + kMlpW3;
  const float *b1 = reinterpret_cast<const float *>(W + kMlpB1);
  const float *b2 = reinterpret_cast<const float *>(W + kMlpB2);
  const float *b3 = reinterpret_cast<const float *>(W + kMlpB3);
#pragma unroll 1
  for (int mt = 0; mt < 4; mt++) {
    const __nv_bfloat16 *Xr = X + (size_t)(16 * mt) * kXs;
    // layer 1: 2 k-tiles x 8 n-tiles
    uint32_t a1[2][4];
#pragma unroll
    for (int kt = 0; kt < 2; kt++) {
      a1[kt][0] = *reinterpret_cast<const uint32_t *>(Xr + g * kXs + kt * 16 + 2 * tg);
      a1[kt][1] = *reinterpret_cast<const uint32_t *>(Xr + (g + 8) * kXs + kt * 16 + 2 * tg);
      a1[kt][2] = *reinterpret_cast<const uint32_t *>(Xr + g * kXs + kt * 16 + 8 + 2 * tg);
      a1[kt][3] = *reinterpret_cast<const uint32_t *>(Xr + (g + 8) * kXs + kt * 16 + 8 + 2 * tg);
    }
    uint32_t a2[4][4];  // layer-2 A fragments (k-tile q = layer-1 n-tiles 2q, 2q+1)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      float h[2][4];
#pragma unroll
      for (int half = 0; half < 2; half++) {
        const int nt = 2 * q + half;
        const float bb0 = b1[nt * 8 + 2 * tg], bb1 = b1[nt * 8 + 2 * tg + 1];
        h[half][0] = bb0;
        h[half][1] = bb1;
        h[half][2] = bb0;
        h[half][3] = bb1;
      }
#pragma unroll
      for (int kt = 0; kt < 2; kt++) {
        uint32_t bf[4];
        ldsm_b2(W1, kW1s, 16 * q, kt * 16, bf);
        mma_bf16(h[0], a1[kt], bf[0], bf[1]);
        mma_bf16(h[1], a1[kt], bf[2], bf[3]);
      }
      a2[q][0] = gelu_bf16x2(h[0][0], h[0][1]);
      a2[q][1] = gelu_bf16x2(h[0][2], h[0][3]);
      a2[q][2] = gelu_bf16x2(h[1][0], h[1][1]);
      a2[q][3] = gelu_bf16x2(h[1][2], h[1][3]);
    }
    // layer 2 in pairs of n-tiles, each pair feeding one layer-3 k-tile
    float y[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 4; q++) {
      float h[2][4];
#pragma unroll
      for (int half = 0; half < 2; half++) {
        const int nt = 2 * q + half;
        const float bb0 = b2[nt * 8 + 2 * tg], bb1 = b2[nt * 8 + 2 * tg + 1];
        h[half][0] = bb0;
        h[half][1] = bb1;
        h[half][2] = bb0;
        h[half][3] = bb1;
      }
#pragma unroll
      for (int kt = 0; kt < 4; kt++) {
        uint32_t bf[4];
        ldsm_b2(W2, kW2s, 16 * q, kt * 16, bf);
        mma_bf16(h[0], a2[kt], bf[0], bf[1]);
        mma_bf16(h[1], a2[kt], bf[2], bf[3]);
      }
      uint32_t a3[4];
      a3[0] = gelu_bf16x2(h[0][0], h[0][1]);
      a3[1] = gelu_bf16x2(h[0][2], h[0][3]);
      a3[2] = gelu_bf16x2(h[1][0], h[1][1]);
      a3[3] = gelu_bf16x2(h[1][2], h[1][3]);
      const uint8_t *wr = W3 + (g * kW3s + q * 16 + 2 * tg) * 2;
      mma_bf16(y, a3, lds32(wr), lds32(wr + 16));
    }
    if (tg < 2) {
      const int c0 = 2 * tg;
      float *Y0 = Y + (16 * mt + g) * 4, *Y1 = Y + (16 * mt + g + 8) * 4;
      Y0[c0] = y[0] + b3[c0];
      Y0[c0 + 1] = y[1] + b3[c0 + 1];
      Y1[c0] = y[2] + b3[c0];
      Y1[c0 + 1] = y[3] + b3[c0 + 1];
    }
  }
}

// log cosh, stable: |x| + log(1 + exp(-2|x|)) (the -log 2 cancels in ratios).
__device__ __forceinline__ float log_cosh_shift(float x) {
  const float a = fabsf(x);
  return __fadd_rn(a, log1pf(__expf(__fmul_rn(-2.f, a))));
}

// The mixture's mean axis and concentration from the network outputs.
__device__ __forceinline__ void vmf_params(const float y[4], float mu[3], float &kappa) {
  const float nm2 = fmaf(y[2], y[2], fmaf(y[1], y[1], __fmul_rn(y[0], y[0])));
  if (nm2 > 1e-24f) {
    const float inv = rsqrtf(nm2);
    mu[0] = y[0] * inv;
    mu[1] = y[1] * inv;
    mu[2] = y[2] * inv;
  } else {
    mu[0] = 0.f;
    mu[1] = 0.f;
    mu[2] = 1.f;
  }
  kappa = __expf(fminf(fmaxf(y[3], kLogKMin), kLogKMax));
}

// A draw from half vMF(mu, kappa) + half vMF(-mu, kappa): w = cos(angle to mu)
// by the exact inverse CDF w = 1 + log(1 - (1-u)(1 - exp(-2 kappa)))/kappa,
// azimuth 2 pi u_phi in the basis e1 = normalize(mu x a), e2 = mu x e1
// (a = x-axis unless |mu_x| >= 0.9, then y-axis), sign flipped when
// u_sign >= 1/2.
__device__ __forceinline__ void vmf_sample(const float mu[3], float kappa, float u_w, float u_phi, float u_sign,
                                           float v[3]) {
  float w = 1.f + log1pf(-(1.f - u_w) * (-expm1f(-2.f * kappa))) / kappa;
  w = fminf(1.f, fmaxf(-1.f, w));
  const bool ax = fabsf(mu[0]) < 0.9f;
  const float a0 = ax ? 1.f : 0.f, a1 = ax ? 0.f : 1.f;
  // e1 = mu x a
  float e1x = mu[1] * 0.f - mu[2] * a1, e1y = mu[2] * a0 - mu[0] * 0.f, e1z = mu[0] * a1 - mu[1] * a0;
  const float in1 = rsqrtf(e1x * e1x + e1y * e1y + e1z * e1z);
  e1x *= in1;
  e1y *= in1;
  e1z *= in1;
  const float e2x = mu[1] * e1z - mu[2] * e1y, e2y = mu[2] * e1x - mu[0] * e1z, e2z = mu[0] * e1y - mu[1] * e1x;
  float sp, cp;
  sincospif(2.f * u_phi, &sp, &cp);
  const float r = sqrtf(fmaxf(0.f, 1.f - w * w));
  float x = w * mu[0] + r * (cp * e1x + sp * e2x);
  float y = w * mu[1] + r * (cp * e1y + sp * e2y);
  float z = w * mu[2] + r * (cp * e1z + sp * e2z);
  const float inv = rsqrtf(x * x + y * y + z * z);
  const float sg = u_sign < 0.5f ? inv : -inv;
  v[0] = x * sg;
  v[1] = y * sg;
  v[2] = z * sg;
}

}  // namespace mcx
