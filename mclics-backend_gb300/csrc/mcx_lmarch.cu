// mcx_lmarch.cu -- the learned-proposal pass as a z-march (no counterpart in
// the reference).
//
//   k_lmarch  the z-march of mcx_march.cu with the learned proposal: per
//             plane every thread loads its pair's neighbourhood into
//             registers (the z neighbours come from the march), writes the two
//             sites' network inputs as rows 2*lane and 2*lane+1 of its warp's
//             64-row tile, the warp evaluates the network on the tensor cores
//             (mlp_warp, mcx_mlp.cuh), and each thread draws and accepts its
//             sites' moves (site_update_learned, mcx_pass.cuh).  The network is
//             warp-synchronous, so every lane runs every plane: a thread past
//             the end of the plane contributes zero rows and updates nothing.
//             No shared-memory staging of neighbourhoods: 40 KB per CTA
//             (weights and one input/output tile per warp), four CTAs of 128
//             threads per SM at 128 registers.
//
//             With TC the network runs on the 5th-generation tensor cores
//             instead (tc_mlp, mcx_tcmlp.cuh): per plane the CTA's 128
//             threads store their two sites' input rows as two M = 128 tiles
//             (thread t is row t of each: site A, site B), one thread issues
//             the tcgen05.mma of each layer, the accumulators sit in 128 TMEM
//             columns of the CTA and every thread reads back its own rows.
//             63 KB of shared memory per CTA (three CTAs per SM).
//
// It computes what the learned direct pass (k_pass<LEARN>) computes: the
// same rows reach the network, the same per-site Philox counters drive the
// draws.  Results agree bit for bit except where a decision lies within an
// ulp of its threshold: the compiler fuses multiply-adds per kernel, so such
// a decision (about one in 10^7-10^8 updates) can go the other way.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mcx_march.cuh"
#include "mcx_mlp.cuh"
#include "mcx_tcmlp.cuh"

namespace mcx {

constexpr int kLPB = 128;  // threads per CTA (4 warps)
constexpr int kLmarchSmem = kMlpBytes + (kLPB / 32) * (64 * kXs * 2 + 64 * 4 * 4);
constexpr int kLmarchTcSmem = kTcWBytes + 2 * kTcXBytes + 2 * kTcHBytes + 64;
constexpr uint32_t kLmarchTcCols = 128;  // two tiles of 64 FP32 accumulator columns
#ifndef MCX_LMARCH_MIN_BLOCKS
#define MCX_LMARCH_MIN_BLOCKS 4
#endif

// the tensor-core form holds 63 KB of shared memory: three CTAs per SM, so
// each thread may use up to 170 registers.  ODD: the batch holds an odd nx
// (phantom slots, odd_tail); built only for masked batches that need it.
template <int POT, bool MASK, bool FIELD, int MODE, bool TC, bool ODD>
__global__ void __launch_bounds__(kLPB, TC ? 3 : MCX_LMARCH_MIN_BLOCKS) k_lmarch(PassArgs a) {
  static_assert(MODE == MODE_SWEEP || MODE == MODE_SWEEP_MEASURE, "sweep modes only");
  extern __shared__ __align__(1024) uint8_t dyn[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint8_t *W = dyn;
  __nv_bfloat16 *X = reinterpret_cast<__nv_bfloat16 *>(dyn + kMlpBytes) + (size_t)warp * 64 * kXs;
  float *Y = reinterpret_cast<float *>(dyn + kMlpBytes + (kLPB / 32) * 64 * kXs * 2) + (size_t)warp * 64 * 4;
  // tensor-core form: network image, two input tiles, two activation tiles,
  // the MMA mbarrier and the TMEM address
  uint8_t *TX = dyn + kTcWBytes, *TH = TX + 2 * kTcXBytes;
  uint64_t *tbar = reinterpret_cast<uint64_t *>(TH + 2 * kTcHBytes);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(tbar + 1);
  uint32_t tmem = 0, tphase = 0;
  // the weights are written only between launches (host copies on the stream)
  if (TC) {
    tc_load_weights(a.mlp, W, kLPB);
    if (threadIdx.x == 0) {
      mbar_init(tbar, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tc_alloc(tslot, kLmarchTcCols);
    fence_proxy_async();
    tc_fence_before();
  } else {
    for (int i = threadIdx.x; i < kMlpBytes / 16; i += kLPB)
      reinterpret_cast<int4 *>(W)[i] = reinterpret_cast<const int4 *>(a.mlp)[i];
  }
  const int4 u = a.units[blockIdx.x];
  const int r = u.x, c = a.colour;
  const RepDev &R = a.reps[r];
  const RepState *S = a.st + r;
  const int npp = R.hp * R.ny;
  const bool valid = u.y + (int)threadIdx.x < npp;
  const int p = valid ? u.y + (int)threadIdx.x : npp - 1;  // lanes past the plane shadow the last pair
  March m;
  march_init<MASK, ODD>(a, R, c, p, u.z, m);
  const int nz = R.nz, nx = R.nx;
  const bool zper = R.zb == BOUND_PERIODIC;
  const int kb = u.z, ke = u.z + (u.w & kUnitPlanes);
  unsigned acc = 0;
  float qs[kQ];
#pragma unroll
  for (int q = 0; q < kQ; q++) qs[q] = 0.f;
  __syncthreads();  // weights in shared memory
  if (TC) {
    tc_fence_after();
    tmem = *tslot;
  }
  grid_dependency_wait(m);
  if (MASK && (u.w & kUnitDead)) {  // no active site in or next to the unit: field energies only
    if (valid) dead_unit<FIELD, MODE>(R, m, kb, ke, qs);
  } else {
  const unsigned long long sw = S->sweep;
  const float T = S->T, invT = 1.0f / S->T;
  OPair om, o0, op;
  const bool zm0 = kb > 0 || zper;
  {
    const int wrap = kb == 0 ? nz : 0;
    load_opair_at<MASK>(m, m.off + (wrap - 1) * m.dz, m.offp + (wrap - 1) * m.dzp, zm0, om);
    load_opair_at<MASK>(m, m.off, m.offp, true, o0);
  }
  bool zm = zm0;
  auto wt = [&](float ee, uint8_t pp) { return MASK ? (ee != 0.f && pp != 0 ? 1.f : 0.f) : ee; };
#pragma unroll 1
  for (int k = kb; k < ke; k++) {
    const bool zp = k + 1 < nz || zper;
    const int up = k + 1 < nz ? 1 : 1 - nz;
    load_opair_at<MASK>(m, m.off + up * m.dz, m.offp + up * m.dzp, zp, op);
    const int dx = m.s ? m.dx1 : m.dx0;
    uint16_t pself = 0x0101;
    if (MASK) pself = __ldg(reinterpret_cast<const uint16_t *>(m.PA + m.offp));
    // a warp whose 64 sites are all inactive: nothing moves, so it needs no
    // network, and in an unmeasured sweep nothing is measured either, so it
    // skips the updates too (the tensor-core form evaluates the network per
    // CTA and does not skip)
    const bool idle = !TC && MASK && __all_sync(0xffffffffu, !valid || pself == 0);
    const bool skip = idle && MODE == MODE_SWEEP;
    if (!skip) {
    float2 ax = *reinterpret_cast<const float2 *>(m.A0 + m.off);
    float2 ay = *reinterpret_cast<const float2 *>(m.A1 + m.off);
    float2 az = *reinterpret_cast<const float2 *>(m.A2 + m.off);
    const float exv[3] = {ldo1(m.O0 + m.off + dx), ldo1(m.O1 + m.off + dx), ldo1(m.O2 + m.off + dx)};
    OPair yp, ym;
    load_opair_at<MASK>(m, m.off + m.dyp, m.offp + m.dypp, true, yp);
    load_opair_at<MASK>(m, m.off + m.dym, m.offp + m.dymp, true, ym);
    uint8_t pex = 1;
    if (MASK) pex = __ldg(m.PO + m.offp + dx);
    const int s = m.s;
    const float exe = s ? m.ee1 : m.ee0;
    const float erz[4] = {m.eyp, m.eym, zp ? 1.f : 0.f, zm ? 1.f : 0.f};
    const OPair *rows4[4] = {&yp, &ym, &op, &om};
    const uint8_t lo = (uint8_t)(o0.pt & 0xFF), hi = (uint8_t)(o0.pt >> 8);
    // neighbour slots x+ x- y+ y- z+ z- of both sites (as update_pair)
    float nbA[6][3], wA[6], eA[6], nbB[6][3], wB[6], eB[6];
    if (s == 0) {
      nbA[0][0] = o0.v[0].x; nbA[0][1] = o0.v[1].x; nbA[0][2] = o0.v[2].x; eA[0] = 1.f; wA[0] = wt(1.f, lo);
      nbA[1][0] = exv[0]; nbA[1][1] = exv[1]; nbA[1][2] = exv[2]; eA[1] = exe; wA[1] = wt(exe, pex);
      nbB[0][0] = o0.v[0].y; nbB[0][1] = o0.v[1].y; nbB[0][2] = o0.v[2].y; eB[0] = 1.f; wB[0] = wt(1.f, hi);
      nbB[1][0] = o0.v[0].x; nbB[1][1] = o0.v[1].x; nbB[1][2] = o0.v[2].x; eB[1] = 1.f; wB[1] = wt(1.f, lo);
      // odd nx: the row's last site has no x+ bond (odd_tail, mcx_pass.cuh)
      if (MASK && m.tail == 1) eA[0] = wA[0] = 0.f;
      if (MASK && m.tail == 2) eB[0] = wB[0] = 0.f;
    } else {
      if (m.hasB) {
        nbA[0][0] = o0.v[0].y; nbA[0][1] = o0.v[1].y; nbA[0][2] = o0.v[2].y; eA[0] = 1.f; wA[0] = wt(1.f, hi);
      } else {
        nbA[0][0] = exv[0]; nbA[0][1] = exv[1]; nbA[0][2] = exv[2]; eA[0] = exe; wA[0] = wt(exe, pex);
      }
      nbA[1][0] = o0.v[0].x; nbA[1][1] = o0.v[1].x; nbA[1][2] = o0.v[2].x; eA[1] = 1.f; wA[1] = wt(1.f, lo);
      nbB[0][0] = exv[0]; nbB[0][1] = exv[1]; nbB[0][2] = exv[2]; eB[0] = exe; wB[0] = wt(exe, pex);
      nbB[1][0] = o0.v[0].y; nbB[1][1] = o0.v[1].y; nbB[1][2] = o0.v[2].y; eB[1] = 1.f; wB[1] = wt(1.f, hi);
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const OPair &o = *rows4[q];
      nbA[2 + q][0] = o.v[0].x; nbA[2 + q][1] = o.v[1].x; nbA[2 + q][2] = o.v[2].x;
      nbB[2 + q][0] = o.v[0].y; nbB[2 + q][1] = o.v[1].y; nbB[2 + q][2] = o.v[2].y;
      eA[2 + q] = eB[2 + q] = erz[q];
      wA[2 + q] = wt(erz[q], MASK ? (uint8_t)(o.pt & 0xFF) : 1);
      wB[2 + q] = wt(erz[q], MASK ? (uint8_t)(o.pt >> 8) : 1);
    }
    const int psA = MASK ? (pself & 0xFF) : 1, psB = MASK ? (pself >> 8) : 1;
    float yA[4], yB[4];
    if (TC) {
      // the network for the CTA's 256 sites: two M = 128 tiles on the tensor cores
      uint32_t fw[16];
      feature_words(nbA, wA, T, valid, fw);
      tc_store_row32(TX, threadIdx.x, fw);
      feature_words(nbB, wB, T, valid && m.hasB, fw);
      tc_store_row32(TX + kTcXBytes, threadIdx.x, fw);
      fence_proxy_async();
      __syncthreads();
      float y[2][4];
      if (!tc_mlp(W, TX, TH, 2, tmem, tbar, tphase, y, a.err)) break;  // uniform: every thread saw the same waits
#pragma unroll
      for (int q = 0; q < 4; q++) {
        yA[q] = y[0][q];
        yB[q] = y[1][q];
      }
    } else if (idle) {  // no active site: the outputs are never read
#pragma unroll
      for (int q = 0; q < 4; q++) yA[q] = yB[q] = 0.f;
    } else {
      // the network for the warp's 64 sites
      __syncwarp();
      write_features(X + (size_t)(2 * lane) * kXs, nbA, wA, T, valid);
      write_features(X + (size_t)(2 * lane + 1) * kXs, nbB, wB, T, valid && m.hasB);
      __syncwarp();
      mlp_warp(W, X, Y);
      __syncwarp();
#pragma unroll
      for (int q = 0; q < 4; q++) {
        yA[q] = Y[(2 * lane) * 4 + q];
        yB[q] = Y[(2 * lane + 1) * 4 + q];
      }
    }
    if (valid) {
      // odd nx: the phantom in the last slot of an s = 1 row is skipped
      const bool skipA = MASK && s == 1 && m.tail == 1, skipB = MASK && s == 1 && m.tail == 2;
      if (!skipA) {
        float sx = 0.f, sy = 0.f, sz = 0.f;
        if (MASK && psA > 1) {
          const float *nsb = a.ns + R.ns_off + (long long)(c * 3) * R.plane + m.off;
          sx = __ldg(nsb);
          sy = __ldg(nsb + R.plane);
          sz = __ldg(nsb + 2 * R.plane);
        }
        const uint32_t nat = (uint32_t)(2 * m.h0 + s) + (uint32_t)nx * (uint32_t)m.row;
        acc += site_update_learned<POT, MASK, FIELD, MODE>(R, a, c, ax.x, ay.x, az.x, nbA, wA, eA, psA, sx, sy, sz,
                                                           yA, invT, nat, sw, qs);
      }
      if (m.hasB && !skipB) {
        float sx = 0.f, sy = 0.f, sz = 0.f;
        if (MASK && psB > 1) {
          const float *nsb = a.ns + R.ns_off + (long long)(c * 3) * R.plane + m.off + 1;
          sx = __ldg(nsb);
          sy = __ldg(nsb + R.plane);
          sz = __ldg(nsb + 2 * R.plane);
        }
        const uint32_t nat = (uint32_t)(2 * m.h0 + 2 + s) + (uint32_t)nx * (uint32_t)m.row;
        acc += site_update_learned<POT, MASK, FIELD, MODE>(R, a, c, ax.y, ay.y, az.y, nbB, wB, eB, psB, sx, sy, sz,
                                                           yB, invT, nat, sw, qs);
      }
      *reinterpret_cast<float2 *>(m.A0 + m.off) = ax;
      *reinterpret_cast<float2 *>(m.A1 + m.off) = ay;
      *reinterpret_cast<float2 *>(m.A2 + m.off) = az;
    }
    }  // !skip
    om = o0;
    o0 = op;
    zm = true;
    m.off += m.dz;
    m.offp += m.dzp;
    m.pid += m.dpid;
    m.row += R.ny;
    m.s ^= 1;
  }
  }
  grid_launch_dependents();
  flush_replica<kLPB, MODE>(a, r, 1, (unsigned)R.lcta, acc, qs, MASK);
  if (TC) {  // every TMEM read is done (tc_mlp ends on a fenced barrier; flush_replica syncs again)
    tc_fence_after();
    if (warp == 0) tc_dealloc(tmem, kLmarchTcCols);
  }
}

template <int POT, bool MASK, bool FIELD, bool TC, bool ODD = false>
static const void *lmarch_fn(int mode) {
  return mode == MODE_SWEEP_MEASURE ? (const void *)k_lmarch<POT, MASK, FIELD, MODE_SWEEP_MEASURE, TC, ODD>
                                    : (const void *)k_lmarch<POT, MASK, FIELD, MODE_SWEEP, TC, ODD>;
}

template <int POT, bool FIELD, bool TC>
static const void *lmarch_fn_masked(const Variant &v, int mode) {
  return v.odd ? lmarch_fn<POT, true, FIELD, TC, true>(mode) : lmarch_fn<POT, true, FIELD, TC, false>(mode);
}

template <bool TC>
static const void *lmarch_kernel_tc(const Variant &v, int mode) {
  if (v.pot == POT_LL) {
    if (v.mask) return v.field ? lmarch_fn_masked<POT_LL, true, TC>(v, mode) : lmarch_fn_masked<POT_LL, false, TC>(v, mode);
    return v.field ? lmarch_fn<POT_LL, false, true, TC>(mode) : lmarch_fn<POT_LL, false, false, TC>(mode);
  }
  if (v.mask)
    return v.field ? lmarch_fn_masked<POT_GHRL, true, TC>(v, mode) : lmarch_fn_masked<POT_GHRL, false, TC>(v, mode);
  return v.field ? lmarch_fn<POT_GHRL, false, true, TC>(mode) : lmarch_fn<POT_GHRL, false, false, TC>(mode);
}

static const void *lmarch_kernel(const Variant &v, int mode, bool tc) {
  return tc ? lmarch_kernel_tc<true>(v, mode) : lmarch_kernel_tc<false>(v, mode);
}

static int lmarch_smem(bool tc) { return tc ? kLmarchTcSmem : kLmarchSmem; }

int lmarch_block_threads() { return kLPB; }

bool lmarch_prepare(const Variant &v, bool tc) {
  if (v.pot == POT_PEAR) return false;
  for (int mode : {MODE_SWEEP, MODE_SWEEP_MEASURE})
    if (cudaFuncSetAttribute(lmarch_kernel(v, mode, tc), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             lmarch_smem(tc)) != cudaSuccess)
      return false;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, lmarch_kernel(v, MODE_SWEEP, tc), kLPB, lmarch_smem(tc)) !=
      cudaSuccess)
    return false;
  // the tensor-core form's CTAs must all find their TMEM columns (512 per SM)
  return n > 0 && (!tc || (uint32_t)n * kLmarchTcCols <= 512);
}

void launch_lmarch(const Variant &v, int mode, const PassArgs &a, bool pdl, bool tc, cudaStream_t st) {
  if (v.pot == POT_PEAR) return;  // the learned proposal is refused for Pear
  PassArgs args = a;
  void *params[] = {&args};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(a.nunits);
  cfg.blockDim = dim3(kLPB);
  cfg.dynamicSmemBytes = lmarch_smem(tc);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelExC(&cfg, lmarch_kernel(v, mode, tc), params);
}

}  // namespace mcx
