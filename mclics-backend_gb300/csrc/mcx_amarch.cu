// mcx_amarch.cu -- the z-march of the plain proposal with a per-thread
// cp.async prefetch of the next plane's neighbourhood (k_amarch), and its
// launchers.  Same work units, Philox counters and pair update as k_march
// (mcx_march.cu), so the two agree bit for bit except at decisions within an
// ulp of their threshold (see mcx_march.cu); this form hides each plane's
// load latency behind the arithmetic of the plane before it.
#include <cuda_runtime.h>

#include "mcx_march.cuh"

namespace mcx {

// ---------------------------------------------------------------------------
// The z-march with a per-thread prefetch (k_amarch).  While a thread updates
// its pair in plane k, cp.async copies the neighbourhood of plane k+1 (its
// own pair, the opposite pairs of rows y+1 and y-1, the extra x site, and the
// opposite pair of plane k+2) into the thread's own shared-memory slots of
// the other stage; the load latency of a plane is then hidden behind the
// arithmetic of the one before it.  Every thread reads back only what it
// copied, so cp.async.wait_group alone orders copies and reads: no block
// barrier, no registers held by loads in flight.  Slots are structure-of-
// arrays ([stage][slot][thread]), so the reads are conflict-free.  Unmasked
// lattices; the same inputs to update_pair as k_march.
// ---------------------------------------------------------------------------
constexpr int kAF2 = 12;  // float2 slots per stage: own, y+1, y-1, plane k+1 opposite (x 3 components)
constexpr int kAF1 = 3;   // float slots per stage: the extra x site (3 components)
constexpr int amarch_smem_per_thread() { return 2 * (kAF2 * 8 + kAF1 * 4); }

// Copies the neighbourhood of the plane at offset `off` (own-site parity s;
// the plane after it at `off + up`, absent when !zp) into one stage.
template <int NT>
__device__ __forceinline__ void am_issue(const March &m, int off, int s, int up, bool zp, float2 *f2, float *f1) {
  const int t = threadIdx.x;
  const int dx = s ? m.dx1 : m.dx0;
  const float *Ab[3] = {m.A0, m.A1, m.A2};
  const float *Ob[3] = {m.O0, m.O1, m.O2};
#pragma unroll
  for (int q = 0; q < 3; q++) {
    cp_async(&f2[q * NT + t], Ab[q] + off, 8, true);
    cp_async(&f2[(3 + q) * NT + t], Ob[q] + off + m.dyp, 8, true);
    cp_async(&f2[(6 + q) * NT + t], Ob[q] + off + m.dym, 8, true);
    cp_async(&f2[(9 + q) * NT + t], Ob[q] + (zp ? off + up : off), 8, zp);  // zero-filled when absent
    cp_async(&f1[q * NT + t], Ob[q] + off + dx, 4, true);
  }
}

template <int POT, bool FIELD, int MODE, int NT, bool PER>
__global__ void __launch_bounds__(NT, march_min_blocks<POT, false, NT>()) k_amarch(PassArgs a) {
  static_assert(MODE == MODE_SWEEP || MODE == MODE_SWEEP_MEASURE, "sweep modes only");
  extern __shared__ __align__(16) unsigned char am_smem[];
  float2 *F2 = reinterpret_cast<float2 *>(am_smem);                            // [2][kAF2][NT]
  float *F1 = reinterpret_cast<float *>(am_smem + 2 * kAF2 * NT * sizeof(float2));  // [2][kAF1][NT]
  const int4 u = a.units[blockIdx.x];
  const int r = u.x, c = a.colour;
  const RepDev &R = a.reps[r];
  const RepState *S = a.st + r;
  unsigned acc = 0;
  float qs[kQ];
#pragma unroll
  for (int q = 0; q < kQ; q++) qs[q] = 0.f;
  const int p = u.y + (int)threadIdx.x;
  if (p < R.hp * R.ny) {
    const int nz = R.nz;
    March m;
    march_init<false>(a, R, c, p, u.z, m);
    const bool zper = R.zb == BOUND_PERIODIC;
    const int kb = u.z, ke = u.z + (u.w & kUnitPlanes);
    const uint32_t seed = R.seed, stream = R.stream;
    grid_dependency_wait(m);  // directors and state may be written by the previous pass until here
    const unsigned long long sw = S->sweep;
    const float ang = S->ang_var, invT = 1.0f / S->T;
    OPair om, o0;
    const bool zm0 = kb > 0 || zper;
    {
      const int wrap = kb == 0 ? nz : 0;
      load_opair_at<false>(m, m.off + (wrap - 1) * m.dz, 0, zm0, om);
      load_opair_at<false>(m, m.off, 0, true, o0);
    }
    {
      const bool zp = kb + 1 < nz || zper;
      am_issue<NT>(m, m.off, m.s, (kb + 1 < nz ? 1 : 1 - nz) * m.dz, zp, F2, F1);
    }
    cp_async_commit();
    bool zm = zm0;
    // the draw of the plane being updated; the next plane's is computed
    // alongside this plane's arithmetic (integer and FP32 pipes interleave)
    uint4 rw = pair_draw(m.pid, c, sw, seed, stream);
#pragma unroll 1
    for (int k = kb; k < ke; k++) {
      const int st = (k - kb) & 1;
      if (k + 1 < ke) {  // the next plane's neighbourhood into the other stage
        const bool zp2 = k + 2 < nz || zper;
        am_issue<NT>(m, m.off + m.dz, m.s ^ 1, (k + 2 < nz ? 1 : 1 - nz) * m.dz, zp2, F2 + (st ^ 1) * kAF2 * NT,
                     F1 + (st ^ 1) * kAF1 * NT);
      }
      cp_async_commit();
      cp_async_wait1();  // this plane's stage has landed
      const float2 *f2 = F2 + st * kAF2 * NT + threadIdx.x;
      const float *f1 = F1 + st * kAF1 * NT + threadIdx.x;
      float2 ax = f2[0], ay = f2[NT], az = f2[2 * NT];
      OPair yp, ym, op;
#pragma unroll
      for (int q = 0; q < 3; q++) {
        yp.v[q] = f2[(3 + q) * NT];
        ym.v[q] = f2[(6 + q) * NT];
        op.v[q] = f2[(9 + q) * NT];
      }
      const float exv[3] = {f1[0], f1[NT], f1[2 * NT]};
      const bool zp = k + 1 < nz || zper;
      const uint4 rw_next = pair_draw(m.pid + m.dpid, c, sw, seed, stream);  // unused after the last plane
      update_pair_draw<POT, false, FIELD, MODE, PER>(a, R, c, m.s, m.hasB, m.ee0, m.ee1, m.eyp, m.eym, o0, yp, ym, op,
                                                     om, exv, 0x0101, 1, zp, zm, rw, m.off, ang, invT, ax, ay, az, acc,
                                                     qs);
      if (MODE == MODE_SWEEP_MEASURE && a.meas_both && c == 1) {  // the colour-0 pair of this row (PassArgs::meas_both)
        measure_opposite<FIELD>(R, o0.v[0].x, o0.v[1].x, o0.v[2].x, qs);
        if (m.hasB) measure_opposite<FIELD>(R, o0.v[0].y, o0.v[1].y, o0.v[2].y, qs);
      }
      rw = rw_next;
      *reinterpret_cast<float2 *>(m.A0 + m.off) = ax;
      *reinterpret_cast<float2 *>(m.A1 + m.off) = ay;
      *reinterpret_cast<float2 *>(m.A2 + m.off) = az;
      om = o0;
      o0 = op;
      zm = true;
      m.off += m.dz;
      m.pid += m.dpid;
      m.row += R.ny;
      m.s ^= 1;
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
  }
  grid_dependency_wait();    // threads without a pair reach here without having waited
  grid_launch_dependents();  // the next pass may start its set-up now
  flush_replica<NT, MODE>(a, r, 1, (unsigned)R.mcta, acc, qs, false);
}

template <int POT, bool FIELD, int NT>
static const void *amarch_fn(const Variant &v, int mode) {
  if (mode == MODE_SWEEP_MEASURE)
    return v.per ? (const void *)k_amarch<POT, FIELD, MODE_SWEEP_MEASURE, NT, true>
                 : (const void *)k_amarch<POT, FIELD, MODE_SWEEP_MEASURE, NT, false>;
  return v.per ? (const void *)k_amarch<POT, FIELD, MODE_SWEEP, NT, true>
               : (const void *)k_amarch<POT, FIELD, MODE_SWEEP, NT, false>;
}

template <int NT>
static const void *amarch_fn_v(const Variant &v, int mode) {
  if (v.pot == POT_LL) return v.field ? amarch_fn<POT_LL, true, NT>(v, mode) : amarch_fn<POT_LL, false, NT>(v, mode);
  return v.field ? amarch_fn<POT_GHRL, true, NT>(v, mode) : amarch_fn<POT_GHRL, false, NT>(v, mode);
}

static const void *amarch_kernel(const Variant &v, int mode, int nt) {
  switch (nt) {
    case 64: return amarch_fn_v<64>(v, mode);
    case 256: return amarch_fn_v<256>(v, mode);
    default: return amarch_fn_v<128>(v, mode);
  }
}

int amarch_smem_bytes(int nt) { return nt * amarch_smem_per_thread(); }

bool amarch_prepare(const Variant &v, int nt) {
  if (v.mask || v.pot == POT_PEAR) return false;  // built for unmasked LL and GHRL
  for (int mode : {MODE_SWEEP, MODE_SWEEP_MEASURE})
    if (cudaFuncSetAttribute(amarch_kernel(v, mode, nt), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             amarch_smem_bytes(nt)) != cudaSuccess)
      return false;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, amarch_kernel(v, MODE_SWEEP, nt), nt, amarch_smem_bytes(nt)) !=
      cudaSuccess)
    return false;
  return n > 0;
}

int amarch_blocks_per_sm(const Variant &v, int nt) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, amarch_kernel(v, MODE_SWEEP, nt), nt, amarch_smem_bytes(nt)) !=
      cudaSuccess)
    return 0;
  return n;
}

void launch_amarch(const Variant &v, int mode, const PassArgs &a, int nt, bool pdl, cudaStream_t st) {
  if (v.mask || v.pot == POT_PEAR) return;  // never selected there (amarch_prepare is false)
  PassArgs args = a;
  void *params[] = {&args};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(a.nunits);
  cfg.blockDim = dim3(nt);
  cfg.dynamicSmemBytes = amarch_smem_bytes(nt);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelExC(&cfg, amarch_kernel(v, mode, nt), params);
}

}  // namespace mcx
