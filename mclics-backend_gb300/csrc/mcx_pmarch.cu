// mcx_pmarch.cu -- the plain-proposal z-march as one cooperative launch for a
// run of sweeps (k_pmarch), and its launchers.
//
// A sweep of separate pass launches pays, per pass, the grid's launch and
// ramp, the first plane's load latency and the drain: about 3.7 us on a
// GB300, a third of a 128^3 lattice's pass.  Programmatic dependent launch
// cannot hide it when the pass holds every register of the SM (the next
// grid's CTAs cannot become resident early).  Here every CTA keeps its z-march
// unit (the balanced one-wave plan: one unit per resident CTA) for all the
// passes of the run and the passes are separated by a grid barrier; the
// cooperative launch guarantees that all CTAs are resident, so the barrier
// cannot wait on a CTA that never runs.
//
// The barrier: each CTA's thread 0 publishes the CTA's writes
// (__threadfence), adds 1 to a counter that the host zeroes before the
// launch, and polls it with acquire loads until it reaches the pass's target
// (CTAs x passes done).  Every poll loop is bounded: when the limit runs out
// (or another CTA has flagged an error) the CTA sets bit 2 of the error flag
// and returns, so every CTA leaves and the host reports the error.
//
// Directors and replica state are read with __ldcg (L2, not L1): later passes
// of the launch read what other CTAs wrote in earlier ones, and L1 is not
// coherent between SMs.  Point types and normals never change and keep the
// read-only path.  Per pass the work is that of k_march (mcx_march.cu) with
// the same units, Philox counters and pair update, so results agree with it
// bit for bit (the energy change fixes its roundings: bond_sum in
// mcx_pass.cuh).
#include <cuda_runtime.h>

#include "mcx_march.cuh"

namespace mcx {

constexpr unsigned kBarrierPolls = 1u << 20;  // about a second of polls, far beyond any pass

__device__ __forceinline__ float2 ldcg2(const float *p) { return __ldcg(reinterpret_cast<const float2 *>(p)); }

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid barrier `target` (see above); false when the CTA must stop.
__device__ __forceinline__ bool pm_barrier(unsigned *bar, unsigned target, unsigned *err) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(bar, 1u);
    int ok = 1;
    for (unsigned i = 0;; i++) {
      if (ld_acquire(bar) >= target) break;
      if (i >= kBarrierPolls || ld_acquire(err) != 0u) {
        atomicOr(err, 2u);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

template <bool MASK>
__device__ __forceinline__ void pm_load_opair(const March &m, int off, int offp, bool on, OPair &o) {
  if (on) {
    o.v[0] = ldcg2(m.O0 + off);
    o.v[1] = ldcg2(m.O1 + off);
    o.v[2] = ldcg2(m.O2 + off);
    if (MASK) o.pt = __ldg(reinterpret_cast<const uint16_t *>(m.PO + offp));
  } else {
    o.v[0] = o.v[1] = o.v[2] = make_float2(0.f, 0.f);
    if (MASK) o.pt = 0;
  }
}

// One plane: k_march's march_plane with L2 loads of the directors.
template <int POT, bool MASK, bool FIELD, int MODE, bool PER>
__device__ __forceinline__ void pm_plane(const PassArgs &a, const RepDev &R, int c, const March &m, const OPair &om,
                                         const OPair &o0, const OPair &op, bool zp, bool zm, uint32_t seed,
                                         uint32_t stream, unsigned long long sw, float ang, float invT, unsigned &acc,
                                         float qs[kQ]) {
  float2 ax = ldcg2(m.A0 + m.off);
  float2 ay = ldcg2(m.A1 + m.off);
  float2 az = ldcg2(m.A2 + m.off);
  const int dx = m.s ? m.dx1 : m.dx0;
  const float exv[3] = {__ldcg(m.O0 + m.off + dx), __ldcg(m.O1 + m.off + dx), __ldcg(m.O2 + m.off + dx)};
  OPair yp, ym;
  pm_load_opair<MASK>(m, m.off + m.dyp, m.offp + m.dypp, true, yp);
  pm_load_opair<MASK>(m, m.off + m.dym, m.offp + m.dymp, true, ym);
  uint16_t pself = 0x0101;
  uint8_t pex = 1;
  if (MASK) {
    pself = __ldg(reinterpret_cast<const uint16_t *>(m.PA + m.offp));
    pex = __ldg(m.PO + m.offp + dx);
  }
  update_pair<POT, MASK, FIELD, MODE, PER>(a, R, c, m.s, m.hasB, m.ee0, m.ee1, m.eyp, m.eym, o0, yp, ym, op, om, exv,
                                           pself, pex, zp, zm, m.pid, m.off, seed, stream, sw, ang, invT, ax, ay, az,
                                           acc, qs, m.tail);
  *reinterpret_cast<float2 *>(m.A0 + m.off) = ax;
  *reinterpret_cast<float2 *>(m.A1 + m.off) = ay;
  *reinterpret_cast<float2 *>(m.A2 + m.off) = az;
}

template <int POT, bool MASK, bool FIELD, int MODE, int NT, bool PER>
__global__ void __launch_bounds__(NT, march_min_blocks<POT, MASK, NT>())
    k_pmarch(PassArgs a, int nsweeps, unsigned *bar, unsigned extra) {
  static_assert(MODE == MODE_SWEEP || MODE == MODE_SWEEP_MEASURE, "sweep modes only");
  const int4 u = a.units[blockIdx.x];
  const int r = u.x;
  const RepDev &R = a.reps[r];
  const RepState *S = a.st + r;
  const int p = u.y + (int)threadIdx.x;
  const bool has_pair = p < R.hp * R.ny;
  const int nz = R.nz;
  const bool zper = R.zb == BOUND_PERIODIC;
  const int kb = u.z, ke = u.z + (u.w & kUnitPlanes);
  const bool dead = MASK && (u.w & kUnitDead);
  const uint32_t seed = R.seed, stream = R.stream;
  unsigned target = extra;  // extra > 0 only to test the bounded wait: no barrier completes
#pragma unroll 1
  for (int pass = 0; pass < 2 * nsweeps; pass++) {
    const int c = pass & 1;
    unsigned acc = 0;
    float qs[kQ];
#pragma unroll
    for (int q = 0; q < kQ; q++) qs[q] = 0.f;
    if (has_pair && dead) {
      March m;
      march_init<MASK>(a, R, c, p, kb, m);
      dead_unit<FIELD, MODE>(R, m, kb, ke, qs);
    } else if (has_pair) {
      March m;
      march_init<MASK>(a, R, c, p, kb, m);
      const unsigned long long sw = __ldcg(&S->sweep);
      const float ang = __ldcg(&S->ang_var), invT = 1.0f / __ldcg(&S->T);
      OPair om, o0, op;
      const bool zm0 = kb > 0 || zper;
      {
        const int wrap = kb == 0 ? nz : 0;
        pm_load_opair<MASK>(m, m.off + (wrap - 1) * m.dz, m.offp + (wrap - 1) * m.dzp, zm0, om);
        pm_load_opair<MASK>(m, m.off, m.offp, true, o0);
      }
      bool zm = zm0;
#pragma unroll 1
      for (int k = kb; k < ke; k++) {
        const bool zp = k + 1 < nz || zper;
        const int up = k + 1 < nz ? 1 : 1 - nz;
        pm_load_opair<MASK>(m, m.off + up * m.dz, m.offp + up * m.dzp, zp, op);
        pm_plane<POT, MASK, FIELD, MODE, PER>(a, R, c, m, om, o0, op, zp, zm, seed, stream, sw, ang, invT, acc, qs);
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
    flush_replica<NT, MODE>(a, r, 1, (unsigned)R.mcta, acc, qs, MASK, c);
    target += gridDim.x;
    if (!pm_barrier(bar, target, a.err)) return;
  }
}

// ---------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------
template <int POT, bool MASK, bool FIELD, int NT, bool PER>
static const void *pmarch_fn(int mode) {
  return mode == MODE_SWEEP_MEASURE ? (const void *)k_pmarch<POT, MASK, FIELD, MODE_SWEEP_MEASURE, NT, PER>
                                    : (const void *)k_pmarch<POT, MASK, FIELD, MODE_SWEEP, NT, PER>;
}

template <int POT, int NT>
static const void *pmarch_fn_pot(const Variant &v, int mode) {
  if (v.mask) return v.field ? pmarch_fn<POT, true, true, NT, false>(mode) : pmarch_fn<POT, true, false, NT, false>(mode);
  if (v.per) return v.field ? pmarch_fn<POT, false, true, NT, true>(mode) : pmarch_fn<POT, false, false, NT, true>(mode);
  return v.field ? pmarch_fn<POT, false, true, NT, false>(mode) : pmarch_fn<POT, false, false, NT, false>(mode);
}

template <int NT>
static const void *pmarch_fn_v(const Variant &v, int mode) {
  if (v.pot == POT_LL) return pmarch_fn_pot<POT_LL, NT>(v, mode);
  if (v.pot == POT_PEAR) return pmarch_fn_pot<POT_PEAR, NT>(v, mode);
  return pmarch_fn_pot<POT_GHRL, NT>(v, mode);
}

static const void *pmarch_kernel(const Variant &v, int mode, int nt) {
  return nt == 256 ? pmarch_fn_v<256>(v, mode) : pmarch_fn_v<128>(v, mode);
}

bool pmarch_block_ok(int nt) { return nt == 128 || nt == 256; }

int pmarch_blocks_per_sm(const Variant &v, int nt) {
  if (!pmarch_block_ok(nt)) return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, pmarch_kernel(v, MODE_SWEEP, nt), nt, 0) != cudaSuccess)
    return 0;
  return n;
}

cudaError_t launch_pmarch(const Variant &v, int mode, const PassArgs &a, int nt, int nsweeps, unsigned *bar,
                          cudaStream_t st, unsigned extra) {
  cudaError_t r = cudaMemsetAsync(bar, 0, sizeof(unsigned), st);
  if (r != cudaSuccess) return r;
  PassArgs args = a;
  int n = nsweeps;
  void *params[] = {&args, &n, &bar, &extra};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(a.nunits);
  cfg.blockDim = dim3(nt);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelExC(&cfg, pmarch_kernel(v, mode, nt), params);
}

}  // namespace mcx
