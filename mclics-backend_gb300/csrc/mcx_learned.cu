// mcx_learned.cu -- the direct pass with the learned proposal (instantiations
// of k_pass<..., LEARN = true>, mcx_pass.cuh) and the packing of the
// network's weights into the layout its tensor-core code reads
// (mcx_mlp.cuh).  No counterpart in the reference.
#include <cuda_runtime.h>
#include <string.h>

#include "mcx_device.cuh"
#include "mcx_kernels.cuh"
#include "mcx_mlp.cuh"
#include "mcx_pass.cuh"

namespace mcx {

template <int POT, bool MASK, bool FIELD>
static const void *learned_fn(int mode) {
  switch (mode) {
    case MODE_SWEEP: return (const void *)k_pass<POT, MASK, FIELD, MODE_SWEEP, true>;
    case MODE_SWEEP_MEASURE: return (const void *)k_pass<POT, MASK, FIELD, MODE_SWEEP_MEASURE, true>;
    default: return (const void *)k_pass<POT, MASK, FIELD, MODE_TRACE, true>;
  }
}

static const void *learned_select(const Variant &v, int mode) {
  if (v.pot == POT_LL) {
    if (v.mask) return v.field ? learned_fn<POT_LL, true, true>(mode) : learned_fn<POT_LL, true, false>(mode);
    return v.field ? learned_fn<POT_LL, false, true>(mode) : learned_fn<POT_LL, false, false>(mode);
  }
  if (v.mask) return v.field ? learned_fn<POT_GHRL, true, true>(mode) : learned_fn<POT_GHRL, true, false>(mode);
  return v.field ? learned_fn<POT_GHRL, false, true>(mode) : learned_fn<POT_GHRL, false, false>(mode);
}

int pass_learned_blocks_per_sm(const Variant &v, int mode) {
  const void *fn = learned_select(v, mode);
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kLearnSmem) != cudaSuccess) return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kPB, kLearnSmem) != cudaSuccess) return 0;
  return n;
}

template <int POT, bool MASK, bool FIELD>
static void launch_l(int mode, const PassArgs &a, int nb, cudaStream_t st) {
  switch (mode) {
    case MODE_SWEEP: k_pass<POT, MASK, FIELD, MODE_SWEEP, true><<<nb, kPB, kLearnSmem, st>>>(a); break;
    case MODE_SWEEP_MEASURE: k_pass<POT, MASK, FIELD, MODE_SWEEP_MEASURE, true><<<nb, kPB, kLearnSmem, st>>>(a); break;
    default: k_pass<POT, MASK, FIELD, MODE_TRACE, true><<<nb, kPB, kLearnSmem, st>>>(a); break;
  }
}

void launch_pass_learned(const Variant &v, int mode, const PassArgs &a, int nb, cudaStream_t st) {
  if (v.pot == POT_LL) {
    if (v.mask) {
      if (v.field) launch_l<POT_LL, true, true>(mode, a, nb, st);
      else launch_l<POT_LL, true, false>(mode, a, nb, st);
    } else {
      if (v.field) launch_l<POT_LL, false, true>(mode, a, nb, st);
      else launch_l<POT_LL, false, false>(mode, a, nb, st);
    }
  } else {
    if (v.mask) {
      if (v.field) launch_l<POT_GHRL, true, true>(mode, a, nb, st);
      else launch_l<POT_GHRL, true, false>(mode, a, nb, st);
    } else {
      if (v.field) launch_l<POT_GHRL, false, true>(mode, a, nb, st);
      else launch_l<POT_GHRL, false, false>(mode, a, nb, st);
    }
  }
}

int mlp_device_bytes() { return kMlpBytes; }

// Round to the nearest bfloat16, ties to even (the conversion the tensor-core
// path's operands go through).
static uint16_t to_bf16(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7F800000u) == 0x7F800000u) return (uint16_t)(u >> 16);  // inf / nan kept
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

// flat (FP32): W1 [32][64] (input rows 19..31 zero), b1 [64], W2 [64][64],
// b2 [64], W3 [64][8] (output columns 4..7 zero), b3 [8]; row index = input.
void pack_mlp_weights(const float *flat, uint8_t *out) {
  memset(out, 0, kMlpBytes);
  const float *W1 = flat, *b1 = W1 + kMlpIn * kMlpH, *W2 = b1 + kMlpH, *b2 = W2 + kMlpH * kMlpH, *W3 = b2 + kMlpH,
              *b3 = W3 + kMlpH * kMlpOut;
  uint16_t *w1t = reinterpret_cast<uint16_t *>(out + kMlpW1);
  uint16_t *w2t = reinterpret_cast<uint16_t *>(out + kMlpW2);
  uint16_t *w3t = reinterpret_cast<uint16_t *>(out + kMlpW3);
  for (int n = 0; n < kMlpH; n++)
    for (int k = 0; k < kMlpIn; k++) w1t[n * kW1s + k] = to_bf16(W1[k * kMlpH + n]);
  // layers 2 and 3 take twice the GELU (gelu_bf16x2): their weights at half
  // scale, exactly (bf16(w / 2) = bf16(w) / 2 for weights above 1e-38)
  for (int n = 0; n < kMlpH; n++)
    for (int k = 0; k < kMlpH; k++) w2t[n * kW2s + k] = to_bf16(0.5f * W2[k * kMlpH + n]);
  for (int n = 0; n < kMlpOut; n++)
    for (int k = 0; k < kMlpH; k++) w3t[n * kW3s + k] = to_bf16(0.5f * W3[k * kMlpOut + n]);
  memcpy(out + kMlpB1, b1, kMlpH * 4);
  memcpy(out + kMlpB2, b2, kMlpH * 4);
  memcpy(out + kMlpB3, b3, kMlpOut * 4);
}

}  // namespace mcx
