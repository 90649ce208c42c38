// mcx_train.cu -- training of the learned proposal's network on the GPU (no
// counterpart in the reference).
//
//   k_collect   draws training samples from the replicas' current states: a
//               Philox-chosen active site, its six neighbours and T as the 19
//               inputs, its director as the target; optionally a random
//               rotation (Shoemake's uniform quaternion) of the whole
//               neighbourhood and random head-tail flips of every director.
//   k_mlp_grad  loss and gradient of the mean negative log-likelihood of the
//               targets under the antipodal vMF mixture (oracle/mlp.py states
//               it in FP64).  Four warps take 64 samples at a time: each warp
//               runs the forward and backward passes of its 16 samples with
//               mma.sync m16n8k16 (BF16 operands, FP32 accumulation, the
//               layer outputs chained in registers as in inference), then the
//               CTA contracts activations with output gradients over the 64
//               samples -- again on the tensor cores, operands transposed by
//               ldmatrix.trans -- into FP32 weight gradients held in
//               registers; one FP32 atomic per weight and CTA at the end.
//   k_adam      Adam on the FP32 master weights (padding entries stay zero).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "../../include/mcx.h"
#include "mcx_device.cuh"
#include "mcx_kernels.cuh"
#include "mcx_mlp.cuh"

namespace mcx {

constexpr int kSampleF = 24;  // floats per sample: 19 inputs, 3 target, 2 pad
constexpr int kTW = 4;        // warps per CTA of k_mlp_grad
constexpr int kTS = 16 * kTW; // samples per chunk
constexpr int kRowH = 72;     // bf16 row stride of 64-wide tiles (8 pad)
constexpr int kRowY = 24;     // bf16 row stride of the 16-wide output-gradient tile
// flat FP32 parameter offsets (mcx.h layout)
constexpr int kPW1 = 0, kPB1 = kPW1 + kMlpIn * kMlpH, kPW2 = kPB1 + kMlpH, kPB2 = kPW2 + kMlpH * kMlpH,
              kPW3 = kPB2 + kMlpH, kPB3 = kPW3 + kMlpH * kMlpOut, kPTotal = kPB3 + kMlpOut;
static_assert(kPTotal == MCX_MLP_PARAMS, "parameter layout");

// ---------------------------------------------------------------------------
// Sample collection.
// ---------------------------------------------------------------------------
struct CollectArgs {
  const RepDev *reps;
  const RepState *st;
  const float *dir;
  const uint8_t *pt;
  float *out;       // [n][kSampleF]
  const int *rep_of;  // replica of each sample block of 256
  int n;
  uint32_t seed;
  int augment;
};

__device__ __forceinline__ void natural_to_split(const RepDev &R, int i, int j, int k, int &c, int &off, int &offp) {
  c = (i + j + k) & 1;
  const int row = j + R.ny * k;
  off = row * R.hs + (i >> 1);
  offp = row * R.hps + (i >> 1);
}

__device__ __forceinline__ void qrot(const float q[4], float v[3]) {
  // v' = q v q*, q = (w, x, y, z)
  const float w = q[0], x = q[1], y = q[2], z = q[3];
  const float tx = 2.f * (y * v[2] - z * v[1]), ty = 2.f * (z * v[0] - x * v[2]), tz = 2.f * (x * v[1] - y * v[0]);
  const float ox = v[0] + w * tx + (y * tz - z * ty);
  const float oy = v[1] + w * ty + (z * tx - x * tz);
  const float oz = v[2] + w * tz + (x * ty - y * tx);
  v[0] = ox;
  v[1] = oy;
  v[2] = oz;
}

__global__ void k_collect(CollectArgs a) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= a.n) return;
  const int r = a.rep_of[s / 256];
  const RepDev &R = a.reps[r];
  const float T = a.st[r].T;
  const int ntot = R.ntot;
  int site = -1, i = 0, j = 0, k = 0;
  for (int tr = 0; tr < 16 && site < 0; tr++) {
    const uint4 rw = philox4x32_10(make_uint4((uint32_t)s, (uint32_t)tr, 0x5A3Du, 0xC011u), a.seed, (uint32_t)r);
    const int cand = (int)(((unsigned long long)rw.x * (unsigned long long)ntot) >> 32);
    i = cand % R.nx;
    j = (cand / R.nx) % R.ny;
    k = cand / (R.nx * R.ny);
    int c, off, offp;
    natural_to_split(R, i, j, k, c, off, offp);
    if (a.pt == nullptr || a.pt[R.pt_off + (long long)c * R.pplane + offp] != 0) site = cand;
  }
  float *o = a.out + (size_t)s * kSampleF;
  for (int q = 0; q < 22; q++) o[q] = 0.f;
  o[22] = __int_as_float(r);
  o[23] = __int_as_float(site);
  if (site < 0) return;  // no active site found: an all-zero sample (a zero target carries no gradient)
  float f[7][3];          // six neighbours, then the site itself
  const int di[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  const int N[3] = {R.nx, R.ny, R.nz}, B[3] = {R.xb, R.yb, R.zb};
  for (int d = 0; d < 7; d++) {
    int cc[3] = {i, j, k};
    bool ok = true;
    if (d < 6)
      for (int ax = 0; ax < 3; ax++) {
        cc[ax] += di[d][ax];
        if (cc[ax] < 0 || cc[ax] >= N[ax]) {
          if (B[ax] == BOUND_PERIODIC) cc[ax] = (cc[ax] + N[ax]) % N[ax];
          else ok = false;
        }
      }
    f[d][0] = f[d][1] = f[d][2] = 0.f;
    if (!ok) continue;
    int c, off, offp;
    natural_to_split(R, cc[0], cc[1], cc[2], c, off, offp);
    if (d < 6 && a.pt != nullptr && a.pt[R.pt_off + (long long)c * R.pplane + offp] == 0) continue;
    const float *p = a.dir + R.dir_off + (long long)(c * 3) * R.plane + off;
    f[d][0] = p[0];
    f[d][1] = p[R.plane];
    f[d][2] = p[2 * R.plane];
  }
  if (a.augment) {
    const uint4 ra = philox4x32_10(make_uint4((uint32_t)s, 0u, 0xA06Du, 0xC011u), a.seed, (uint32_t)r);
    if (a.augment & MCX_AUG_ROTATE) {
      const float u1 = u01(ra.x), u2 = u01(ra.y), u3 = u01(ra.z);
      const float s1 = sqrtf(1.f - u1), s2 = sqrtf(u1);
      float sa, ca, sb, cb;
      sincospif(2.f * u2, &sa, &ca);
      sincospif(2.f * u3, &sb, &cb);
      const float q[4] = {s2 * cb, s1 * sa, s1 * ca, s2 * sb};
      for (int d = 0; d < 7; d++) qrot(q, f[d]);
    }
    if (a.augment & MCX_AUG_FLIP)
      for (int d = 0; d < 7; d++) {
        const float sg = (ra.w >> d) & 1u ? -1.f : 1.f;
        f[d][0] *= sg;
        f[d][1] *= sg;
        f[d][2] *= sg;
      }
  }
  for (int d = 0; d < 6; d++)
    for (int q = 0; q < 3; q++) o[3 * d + q] = f[d][q];
  o[18] = T;
  o[19] = f[6][0];
  o[20] = f[6][1];
  o[21] = f[6][2];
}

// ---------------------------------------------------------------------------
// Loss and gradient.
// ---------------------------------------------------------------------------
struct GradArgs {
  const float *w;        // FP32 master weights (flat)
  const float *samples;  // [n][kSampleF]
  const int *index;      // sample indices of this batch (null: 0..n-1)
  int n;                 // samples in the batch
  float inv_n;           // 1/n: the loss is a mean
  float *grad;           // FP32 [kPTotal], accumulated
  float *loss;           // accumulated mean loss
};

__device__ __forceinline__ void ldsm_x4_t(uint32_t r[4], const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"((uint32_t)__cvta_generic_to_shared(p)));
}
__device__ __forceinline__ void ldsm_x2_t(uint32_t r[2], const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];"
               : "=r"(r[0]), "=r"(r[1])
               : "r"((uint32_t)__cvta_generic_to_shared(p)));
}

__device__ __forceinline__ float gelu_grad(float x) {
  const float c = 0.7978845608028654f;
  const float t = tanh_approx(c * fmaf(0.044715f * x * x, x, x));
  return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * c * fmaf(3.f * 0.044715f, x * x, 1.f);
}

__device__ __forceinline__ void store_pair(__nv_bfloat16 *base, int row, int stride, int col, float a, float b) {
  *reinterpret_cast<uint32_t *>(base + (size_t)row * stride + col) = pack_bf16(a, b);
}

// dynamic shared memory layout (bytes)
constexpr int kGW1t = 0;                           // [64][40] bf16 (forward)
constexpr int kGW2t = kGW1t + kMlpH * kW1s * 2;    // [64][72] bf16 (forward)
constexpr int kGW3t = kGW2t + kMlpH * kW2s * 2;    // [8][72]  bf16 (forward)
constexpr int kGW2r = kGW3t + kMlpOut * kW3s * 2;  // [64][72] bf16 row = input (backward)
constexpr int kGW3r = kGW2r + kMlpH * kRowH * 2;   // [64][24] bf16 row = hidden, cols = out (backward)
constexpr int kGB = kGW3r + kMlpH * kRowY * 2;     // b1[64] b2[64] b3[8] floats
constexpr int kGX = kGB + (2 * kMlpH + kMlpOut) * 4;  // chunk tiles
constexpr int kGA1 = kGX + kTS * kXs * 2;
constexpr int kGA2 = kGA1 + kTS * kRowH * 2;
constexpr int kGdH1 = kGA2 + kTS * kRowH * 2;
constexpr int kGdH2 = kGdH1 + kTS * kRowH * 2;
constexpr int kGdY = kGdH2 + kTS * kRowH * 2;
constexpr int kGY = kGdY + kTS * kRowY * 2;        // [64][4] float outputs
constexpr int kGSmem = kGY + kTS * 4 * 4;

__global__ void __launch_bounds__(kTW * 32) k_mlp_grad(GradArgs a) {
  extern __shared__ __align__(16) uint8_t sm[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, g = lane >> 2, tg = lane & 3;
  __nv_bfloat16 *W1t = reinterpret_cast<__nv_bfloat16 *>(sm + kGW1t);
  __nv_bfloat16 *W2t = reinterpret_cast<__nv_bfloat16 *>(sm + kGW2t);
  __nv_bfloat16 *W3t = reinterpret_cast<__nv_bfloat16 *>(sm + kGW3t);
  __nv_bfloat16 *W2r = reinterpret_cast<__nv_bfloat16 *>(sm + kGW2r);
  __nv_bfloat16 *W3r = reinterpret_cast<__nv_bfloat16 *>(sm + kGW3r);
  float *bias = reinterpret_cast<float *>(sm + kGB);
  __nv_bfloat16 *X = reinterpret_cast<__nv_bfloat16 *>(sm + kGX);
  __nv_bfloat16 *A1 = reinterpret_cast<__nv_bfloat16 *>(sm + kGA1);
  __nv_bfloat16 *A2 = reinterpret_cast<__nv_bfloat16 *>(sm + kGA2);
  __nv_bfloat16 *dH1 = reinterpret_cast<__nv_bfloat16 *>(sm + kGdH1);
  __nv_bfloat16 *dH2 = reinterpret_cast<__nv_bfloat16 *>(sm + kGdH2);
  __nv_bfloat16 *dY = reinterpret_cast<__nv_bfloat16 *>(sm + kGdY);
  float *Ys = reinterpret_cast<float *>(sm + kGY);
  // weights: FP32 master -> BF16 in the forward (transposed) and backward layouts
  for (int e = tid; e < kMlpH * kW1s; e += kTW * 32) {
    const int n = e / kW1s, k = e % kW1s;
    W1t[e] = __float2bfloat16_rn(k < kMlpIn ? a.w[kPW1 + k * kMlpH + n] : 0.f);
  }
  for (int e = tid; e < kMlpH * kW2s; e += kTW * 32) {
    const int n = e / kW2s, k = e % kW2s;
    W2t[e] = __float2bfloat16_rn(k < kMlpH ? a.w[kPW2 + k * kMlpH + n] : 0.f);
    W2r[e] = __float2bfloat16_rn(k < kMlpH ? a.w[kPW2 + n * kMlpH + k] : 0.f);  // row n = input, col k = output
  }
  for (int e = tid; e < kMlpOut * kW3s; e += kTW * 32) {
    const int n = e / kW3s, k = e % kW3s;
    W3t[e] = __float2bfloat16_rn(k < kMlpH ? a.w[kPW3 + k * kMlpOut + n] : 0.f);
  }
  for (int e = tid; e < kMlpH * kRowY; e += kTW * 32) {
    const int i = e / kRowY, o = e % kRowY;
    W3r[e] = __float2bfloat16_rn(o < kMlpOut ? a.w[kPW3 + i * kMlpOut + o] : 0.f);
  }
  for (int e = tid; e < 2 * kMlpH + kMlpOut; e += kTW * 32)
    bias[e] = e < kMlpH ? a.w[kPB1 + e] : (e < 2 * kMlpH ? a.w[kPB2 + e - kMlpH] : a.w[kPB3 + e - 2 * kMlpH]);
  __syncthreads();
  // weight-gradient accumulators (FP32, fragment layout)
  float gW2[8][4], gWx[8][4];  // gWx: gW1 slice (warps 0,1) or gW3 slices (warps 2,3: [2][4] used)
#pragma unroll
  for (int q = 0; q < 8; q++)
#pragma unroll
    for (int r = 0; r < 4; r++) gW2[q][r] = gWx[q][r] = 0.f;
  float gb = 0.f;  // bias gradient owned by this thread: b1 (tid < 64), b2 (64 <= tid < 128)
  float gb3 = 0.f; // b3 entries (tid < 8)
  float lsum = 0.f;
  const int nchunk = (a.n + kTS - 1) / kTS;
  for (int ch = blockIdx.x; ch < nchunk; ch += gridDim.x) {
    const int row0 = warp * 16;  // this warp's rows in the chunk tiles
    // ---- inputs: lane l fills half a row ----
    {
      const int r = lane >> 1, half = lane & 1;
      const int sidx = ch * kTS + row0 + r;
      float v[16];
      if (sidx < a.n) {
        const float *sp = a.samples + (size_t)(a.index ? a.index[sidx] : sidx) * kSampleF;
        for (int q = 0; q < 16; q++) {
          const int col = half * 16 + q;
          v[q] = col < 19 ? sp[col] : 0.f;
        }
      } else {
        for (int q = 0; q < 16; q++) v[q] = 0.f;
      }
      uint32_t *xr = reinterpret_cast<uint32_t *>(X + (size_t)(row0 + r) * kXs + half * 16);
      for (int q = 0; q < 8; q++) xr[q] = pack_bf16(v[2 * q], v[2 * q + 1]);
    }
    __syncwarp();
    const __nv_bfloat16 *Xr = X + (size_t)row0 * kXs;
    uint32_t a1[2][4];
#pragma unroll
    for (int kt = 0; kt < 2; kt++) {
      a1[kt][0] = *reinterpret_cast<const uint32_t *>(Xr + g * kXs + kt * 16 + 2 * tg);
      a1[kt][1] = *reinterpret_cast<const uint32_t *>(Xr + (g + 8) * kXs + kt * 16 + 2 * tg);
      a1[kt][2] = *reinterpret_cast<const uint32_t *>(Xr + g * kXs + kt * 16 + 8 + 2 * tg);
      a1[kt][3] = *reinterpret_cast<const uint32_t *>(Xr + (g + 8) * kXs + kt * 16 + 8 + 2 * tg);
    }
    // ---- layer 1 ----
    float h1[8][4];
    uint32_t a2[4][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const float bb0 = bias[nt * 8 + 2 * tg], bb1 = bias[nt * 8 + 2 * tg + 1];
      h1[nt][0] = bb0; h1[nt][1] = bb1; h1[nt][2] = bb0; h1[nt][3] = bb1;
#pragma unroll
      for (int kt = 0; kt < 2; kt++) {
        const uint8_t *wr = reinterpret_cast<const uint8_t *>(W1t + (nt * 8 + g) * kW1s + kt * 16 + 2 * tg);
        mma_bf16(h1[nt], a1[kt], lds32(wr), lds32(wr + 16));
      }
      const float g0 = gelu(h1[nt][0]), g1 = gelu(h1[nt][1]), g2 = gelu(h1[nt][2]), g3 = gelu(h1[nt][3]);
      store_pair(A1, row0 + g, kRowH, nt * 8 + 2 * tg, g0, g1);
      store_pair(A1, row0 + g + 8, kRowH, nt * 8 + 2 * tg, g2, g3);
      const int q = nt >> 1;
      if ((nt & 1) == 0) {
        a2[q][0] = pack_bf16(g0, g1);
        a2[q][1] = pack_bf16(g2, g3);
      } else {
        a2[q][2] = pack_bf16(g0, g1);
        a2[q][3] = pack_bf16(g2, g3);
      }
    }
    // ---- layer 2 ----
    float h2[8][4];
    uint32_t a3[4][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const float bb0 = bias[kMlpH + nt * 8 + 2 * tg], bb1 = bias[kMlpH + nt * 8 + 2 * tg + 1];
      h2[nt][0] = bb0; h2[nt][1] = bb1; h2[nt][2] = bb0; h2[nt][3] = bb1;
#pragma unroll
      for (int kt = 0; kt < 4; kt++) {
        const uint8_t *wr = reinterpret_cast<const uint8_t *>(W2t + (nt * 8 + g) * kW2s + kt * 16 + 2 * tg);
        mma_bf16(h2[nt], a2[kt], lds32(wr), lds32(wr + 16));
      }
      const float g0 = gelu(h2[nt][0]), g1 = gelu(h2[nt][1]), g2 = gelu(h2[nt][2]), g3 = gelu(h2[nt][3]);
      store_pair(A2, row0 + g, kRowH, nt * 8 + 2 * tg, g0, g1);
      store_pair(A2, row0 + g + 8, kRowH, nt * 8 + 2 * tg, g2, g3);
      const int q = nt >> 1;
      if ((nt & 1) == 0) {
        a3[q][0] = pack_bf16(g0, g1);
        a3[q][1] = pack_bf16(g2, g3);
      } else {
        a3[q][2] = pack_bf16(g0, g1);
        a3[q][3] = pack_bf16(g2, g3);
      }
    }
    // ---- layer 3 ----
    float y[4] = {bias[2 * kMlpH + 2 * tg], bias[2 * kMlpH + 2 * tg + 1], bias[2 * kMlpH + 2 * tg],
                  bias[2 * kMlpH + 2 * tg + 1]};
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
      const uint8_t *wr = reinterpret_cast<const uint8_t *>(W3t + g * kW3s + kt * 16 + 2 * tg);
      mma_bf16(y, a3[kt], lds32(wr), lds32(wr + 16));
    }
    if (tg < 2) {
      Ys[(row0 + g) * 4 + 2 * tg] = y[0];
      Ys[(row0 + g) * 4 + 2 * tg + 1] = y[1];
      Ys[(row0 + g + 8) * 4 + 2 * tg] = y[2];
      Ys[(row0 + g + 8) * 4 + 2 * tg + 1] = y[3];
    }
    __syncwarp();
    // ---- loss and dL/dY (lanes 0..15, one sample each) ----
    if (lane < 16) {
      const int sidx = ch * kTS + row0 + lane;
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      if (sidx < a.n) {
        const float *sp = a.samples + (size_t)(a.index ? a.index[sidx] : sidx) * kSampleF;
        const float nx = sp[19], ny = sp[20], nz = sp[21];
        const float *yy = Ys + (row0 + lane) * 4;
        const float nm = sqrtf(yy[0] * yy[0] + yy[1] * yy[1] + yy[2] * yy[2]);
        const float inm = nm > 1e-12f ? 1.f / nm : 0.f;
        const float mx = yy[0] * inm, my = yy[1] * inm, mz = yy[2] * inm;
        const bool clamped = yy[3] < kLogKMin || yy[3] > kLogKMax;
        const float l = fminf(fmaxf(yy[3], kLogKMin), kLogKMax);
        const float k = expf(l);
        const float m = mx * nx + my * ny + mz * nz;
        const bool live = nx * nx + ny * ny + nz * nz > 0.5f;
        if (live) {
          // -log q = -log k + log 4 pi + log sinh k - log cosh(k m)
          const float lsinh = k + log1pf(-expf(-2.f * k)) - 0.69314718f;
          const float am = fabsf(k * m);
          const float lcosh = am + log1pf(expf(-2.f * am)) - 0.69314718f;
          lsum += (-logf(k) + 2.53102425f + lsinh - lcosh) * a.inv_n;
          const float th = tanhf(k * m);
          const float dk = (-1.f / k + 1.f / tanhf(k) - m * th) * a.inv_n;
          const float dm = (-k * th) * a.inv_n;
          d[0] = dm * (nx - m * mx) * inm;
          d[1] = dm * (ny - m * my) * inm;
          d[2] = dm * (nz - m * mz) * inm;
          d[3] = clamped ? 0.f : dk * k;
        }
      }
      uint32_t *dr = reinterpret_cast<uint32_t *>(dY + (size_t)(row0 + lane) * kRowY);
      dr[0] = pack_bf16(d[0], d[1]);
      dr[1] = pack_bf16(d[2], d[3]);
      for (int q = 2; q < 8; q++) dr[q] = 0u;
    }
    __syncwarp();
    // ---- dA2 = dY W3^T, dH2 = dA2 * gelu'(H2) ----
    uint32_t ay[4];
    {
      const __nv_bfloat16 *Dr = dY + (size_t)row0 * kRowY;
      ay[0] = *reinterpret_cast<const uint32_t *>(Dr + g * kRowY + 2 * tg);
      ay[1] = *reinterpret_cast<const uint32_t *>(Dr + (g + 8) * kRowY + 2 * tg);
      ay[2] = *reinterpret_cast<const uint32_t *>(Dr + g * kRowY + 8 + 2 * tg);
      ay[3] = *reinterpret_cast<const uint32_t *>(Dr + (g + 8) * kRowY + 8 + 2 * tg);
    }
    uint32_t ad[4][4];  // dH2 as A fragments
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      const uint8_t *wr = reinterpret_cast<const uint8_t *>(W3r + (nt * 8 + g) * kRowY + 2 * tg);
      mma_bf16(d, ay, lds32(wr), lds32(wr + 16));
      d[0] *= gelu_grad(h2[nt][0]);
      d[1] *= gelu_grad(h2[nt][1]);
      d[2] *= gelu_grad(h2[nt][2]);
      d[3] *= gelu_grad(h2[nt][3]);
      store_pair(dH2, row0 + g, kRowH, nt * 8 + 2 * tg, d[0], d[1]);
      store_pair(dH2, row0 + g + 8, kRowH, nt * 8 + 2 * tg, d[2], d[3]);
      const int q = nt >> 1;
      if ((nt & 1) == 0) {
        ad[q][0] = pack_bf16(d[0], d[1]);
        ad[q][1] = pack_bf16(d[2], d[3]);
      } else {
        ad[q][2] = pack_bf16(d[0], d[1]);
        ad[q][3] = pack_bf16(d[2], d[3]);
      }
    }
    // ---- dA1 = dH2 W2^T, dH1 = dA1 * gelu'(H1) ----
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int kt = 0; kt < 4; kt++) {
        const uint8_t *wr = reinterpret_cast<const uint8_t *>(W2r + (nt * 8 + g) * kRowH + kt * 16 + 2 * tg);
        mma_bf16(d, ad[kt], lds32(wr), lds32(wr + 16));
      }
      d[0] *= gelu_grad(h1[nt][0]);
      d[1] *= gelu_grad(h1[nt][1]);
      d[2] *= gelu_grad(h1[nt][2]);
      d[3] *= gelu_grad(h1[nt][3]);
      store_pair(dH1, row0 + g, kRowH, nt * 8 + 2 * tg, d[0], d[1]);
      store_pair(dH1, row0 + g + 8, kRowH, nt * 8 + 2 * tg, d[2], d[3]);
    }
    __syncthreads();
    // ---- weight gradients over the chunk's 64 samples ----
    // mma A = (activations)^T: rows = the weight's input index, k = samples;
    // B = output gradients: k = samples, n = the weight's output index.  Both
    // are stored sample-major, so ldmatrix.trans yields the fragments.
#pragma unroll
    for (int kt = 0; kt < kTS / 16; kt++) {
      const int s0 = kt * 16;
      const int mrow = (lane & 7) + ((lane >> 4) << 3);  // ldmatrix row address: sample
      const int mcol = ((lane >> 3) & 1) << 3;           // column block within 16
      {  // gW2 rows [16 warp, +16)
        uint32_t af[4];
        ldsm_x4_t(af, A1 + (size_t)(s0 + mrow) * kRowH + warp * 16 + mcol);
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
          uint32_t bf[2];
          ldsm_x2_t(bf, dH2 + (size_t)(s0 + (lane & 15)) * kRowH + nt * 8);
          mma_bf16(gW2[nt], af, bf[0], bf[1]);
        }
      }
      if (warp < 2) {  // gW1 rows [16 warp, +16) (input features)
        uint32_t af[4];
        ldsm_x4_t(af, X + (size_t)(s0 + mrow) * kXs + warp * 16 + mcol);
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
          uint32_t bf[2];
          ldsm_x2_t(bf, dH1 + (size_t)(s0 + (lane & 15)) * kRowH + nt * 8);
          mma_bf16(gWx[nt], af, bf[0], bf[1]);
        }
      } else {  // gW3 rows [32 (warp-2), +32): two 16-row tiles, one 8-wide output tile
        uint32_t bf[2];
        ldsm_x2_t(bf, dY + (size_t)(s0 + (lane & 15)) * kRowY);
#pragma unroll
        for (int mt = 0; mt < 2; mt++) {
          uint32_t af[4];
          ldsm_x4_t(af, A2 + (size_t)(s0 + mrow) * kRowH + (warp - 2) * 32 + mt * 16 + mcol);
          mma_bf16(gWx[mt], af, bf[0], bf[1]);
        }
      }
    }
    // bias gradients: column sums of dH1 (tid < 64), dH2 (64..127), dY (tid < 8)
    if (tid < 64) {
      for (int s2 = 0; s2 < kTS; s2++) gb += __bfloat162float(dH1[(size_t)s2 * kRowH + tid]);
    } else {
      for (int s2 = 0; s2 < kTS; s2++) gb += __bfloat162float(dH2[(size_t)s2 * kRowH + tid - 64]);
    }
    if (tid < kMlpOut)
      for (int s2 = 0; s2 < kTS; s2++) gb3 += __bfloat162float(dY[(size_t)s2 * kRowY + tid]);
    __syncthreads();
  }
  // ---- one atomic per weight and CTA ----
#pragma unroll
  for (int nt = 0; nt < 8; nt++) {
    const int o0 = nt * 8 + 2 * tg;
    const int i0 = warp * 16 + g;
    atomicAdd(a.grad + kPW2 + i0 * kMlpH + o0, gW2[nt][0]);
    atomicAdd(a.grad + kPW2 + i0 * kMlpH + o0 + 1, gW2[nt][1]);
    atomicAdd(a.grad + kPW2 + (i0 + 8) * kMlpH + o0, gW2[nt][2]);
    atomicAdd(a.grad + kPW2 + (i0 + 8) * kMlpH + o0 + 1, gW2[nt][3]);
    if (warp < 2) {
      atomicAdd(a.grad + kPW1 + i0 * kMlpH + o0, gWx[nt][0]);
      atomicAdd(a.grad + kPW1 + i0 * kMlpH + o0 + 1, gWx[nt][1]);
      atomicAdd(a.grad + kPW1 + (i0 + 8) * kMlpH + o0, gWx[nt][2]);
      atomicAdd(a.grad + kPW1 + (i0 + 8) * kMlpH + o0 + 1, gWx[nt][3]);
    }
  }
  if (warp >= 2) {
#pragma unroll
    for (int mt = 0; mt < 2; mt++) {
      const int i0 = (warp - 2) * 32 + mt * 16 + g;
      const int o0 = 2 * tg;
      atomicAdd(a.grad + kPW3 + i0 * kMlpOut + o0, gWx[mt][0]);
      atomicAdd(a.grad + kPW3 + i0 * kMlpOut + o0 + 1, gWx[mt][1]);
      atomicAdd(a.grad + kPW3 + (i0 + 8) * kMlpOut + o0, gWx[mt][2]);
      atomicAdd(a.grad + kPW3 + (i0 + 8) * kMlpOut + o0 + 1, gWx[mt][3]);
    }
  }
  atomicAdd(a.grad + (tid < 64 ? kPB1 + tid : kPB2 + tid - 64), gb);
  if (tid < kMlpOut) atomicAdd(a.grad + kPB3 + tid, gb3);
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if (lane == 0) atomicAdd(a.loss, lsum);
}

// Adam (Kingma & Ba 2015) on the FP32 master weights; the layout's padding
// (input rows 19..31 of W1, output columns 4..7 of W3 and b3) stays zero.
__global__ void k_adam(float *w, float *m, float *v, const float *g, int step, float lr, float b1, float b2,
                       float eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kPTotal) return;
  bool pad = false;
  if (i < kPB1) pad = (i - kPW1) / kMlpH >= 19;
  else if (i >= kPW3 && i < kPB3) pad = (i - kPW3) % kMlpOut >= 4;
  else if (i >= kPB3) pad = i - kPB3 >= 4;
  if (pad) {
    w[i] = 0.f;
    return;
  }
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.f - powf(b1, (float)step));
  const float vh = vi / (1.f - powf(b2, (float)step));
  w[i] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void k_batch_index(int *idx, int n, int nsamples, uint32_t seed, uint32_t step) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint4 r = philox4x32_10(make_uint4((uint32_t)i, step, 0xBA7Cu, 0xC011u), seed, 0x7EA1u);
  idx[i] = (int)(((unsigned long long)r.x * (unsigned long long)nsamples) >> 32);
}

}  // namespace mcx

// ---------------------------------------------------------------------------
// Host side (C ABI in mcx_engine.cu calls these).
// ---------------------------------------------------------------------------
namespace mcx {

int train_smem_bytes() { return kGSmem; }
int sample_floats() { return kSampleF; }

cudaError_t launch_collect(const RepDev *reps, const RepState *st, const float *dir, const uint8_t *pt, float *out,
                           const int *rep_of, int n, uint32_t seed, int augment, cudaStream_t s) {
  CollectArgs a{reps, st, dir, pt, out, rep_of, n, seed, augment};
  k_collect<<<(n + 255) / 256, 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_mlp_grad(const float *w, const float *samples, const int *index, int n, float *grad, float *loss,
                            int grid, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaError_t r = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, kGSmem);
    if (r != cudaSuccess) return r;
    attr = true;
  }
  GradArgs a{w, samples, index, n, 1.f / (float)n, grad, loss};
  k_mlp_grad<<<grid, kTW * 32, kGSmem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adam(float *w, float *m, float *v, const float *g, int step, float lr, cudaStream_t s) {
  k_adam<<<(kPTotal + 255) / 256, 256, 0, s>>>(w, m, v, g, step, lr, 0.9f, 0.999f, 1e-8f);
  return cudaGetLastError();
}

cudaError_t launch_batch_index(int *idx, int n, int nsamples, uint32_t seed, uint32_t step, cudaStream_t s) {
  k_batch_index<<<(n + 255) / 256, 256, 0, s>>>(idx, n, nsamples, seed, step);
  return cudaGetLastError();
}

}  // namespace mcx
