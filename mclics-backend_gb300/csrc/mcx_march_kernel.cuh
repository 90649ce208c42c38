// mcx_march_kernel.cuh -- the z-march pass kernel (k_march) and its plane
// and chunk steps, shared by the translation units that instantiate it:
// mcx_march.cu (unmasked batches, and masked batches without an odd nx) and
// mcx_march_odd.cu (masked batches with an odd nx, whose rows end in phantom
// slots: odd_tail).  The kernel is described in mcx_march.cu.
#pragma once
#include <cuda_runtime.h>

#include "mcx_march.cuh"

namespace mcx {

// One plane of the march: loads (first, so that the Philox rounds overlap
// them), the pair update, the stores.
template <int POT, bool MASK, bool FIELD, int MODE, bool PER>
__device__ __forceinline__ void march_plane(const PassArgs &a, const RepDev &R, int c, const March &m,
                                            const OPair &om, const OPair &o0, const OPair &op, bool zp, bool zm,
                                            uint32_t seed, uint32_t stream, unsigned long long sw, float ang,
                                            float invT, unsigned &acc, float qs[kQ]) {
  float2 ax = *reinterpret_cast<const float2 *>(m.A0 + m.off);
  float2 ay = *reinterpret_cast<const float2 *>(m.A1 + m.off);
  float2 az = *reinterpret_cast<const float2 *>(m.A2 + m.off);
  const int dx = m.s ? m.dx1 : m.dx0;
  const float exv[3] = {ldo1(m.O0 + m.off + dx), ldo1(m.O1 + m.off + dx), ldo1(m.O2 + m.off + dx)};
  OPair yp, ym;
  load_opair_at<MASK>(m, m.off + m.dyp, m.offp + m.dypp, true, yp);
  load_opair_at<MASK>(m, m.off + m.dym, m.offp + m.dymp, true, ym);
  uint16_t pself = 0x0101;
  uint8_t pex = 1;
  if (MASK) {
    pself = __ldg(reinterpret_cast<const uint16_t *>(m.PA + m.offp));
    pex = __ldg(m.PO + m.offp + dx);
    // two inactive sites: nothing moves, and an unmeasured sweep adds nothing
    // (a warp of such pairs skips the draw and the arithmetic)
    if (MODE == MODE_SWEEP && pself == 0) return;
  }
  update_pair<POT, MASK, FIELD, MODE, PER>(a, R, c, m.s, m.hasB, m.ee0, m.ee1, m.eyp, m.eym, o0, yp, ym, op, om, exv,
                                           pself, pex, zp, zm, m.pid, m.off, seed, stream, sw, ang, invT, ax, ay, az,
                                           acc, qs, m.tail);
  if (!MASK && MODE == MODE_SWEEP_MEASURE && a.meas_both && c == 1) {
    // the colour-0 pair of this row (final: its pass is done), as the colour-0
    // pass's site_update would measure it
    measure_opposite<FIELD>(R, o0.v[0].x, o0.v[1].x, o0.v[2].x, qs);
    if (m.hasB) measure_opposite<FIELD>(R, o0.v[0].y, o0.v[1].y, o0.v[2].y, qs);
  }
  *reinterpret_cast<float2 *>(m.A0 + m.off) = ax;
  *reinterpret_cast<float2 *>(m.A1 + m.off) = ay;
  *reinterpret_cast<float2 *>(m.A2 + m.off) = az;
}

// The march of one unit's chunk of planes kb..ke-1 (everything after the
// dependency wait).
template <int POT, bool MASK, bool FIELD, int MODE, bool PER>
__device__ __forceinline__ void march_chunk(const PassArgs &a, const RepDev &R, int c, March &m, int kb, int ke,
                                            const RepState *S, unsigned &acc, float qs[kQ]) {
  const int nz = R.nz;
  const bool zper = R.zb == BOUND_PERIODIC;
  const uint32_t seed = R.seed, stream = R.stream;
  const unsigned long long sw = S->sweep;
  const float ang = S->ang_var, invT = 1.0f / S->T;
  // the z pipeline: opposite pairs of this column at planes k-1, k, k+1
  OPair om, o0, op;
  const bool zm0 = kb > 0 || zper;
  {
    const int wrap = kb == 0 ? nz : 0;  // plane -1 is plane nz-1 when z is periodic
    load_opair_at<MASK>(m, m.off + (wrap - 1) * m.dz, m.offp + (wrap - 1) * m.dzp, zm0, om);
    load_opair_at<MASK>(m, m.off, m.offp, true, o0);
  }
  bool zm = zm0;
#pragma unroll 1
  for (int k = kb; k < ke; k++) {
    const bool zp = k + 1 < nz || zper;
    const int up = k + 1 < nz ? 1 : 1 - nz;
    load_opair_at<MASK>(m, m.off + up * m.dz, m.offp + up * m.dzp, zp, op);
    march_plane<POT, MASK, FIELD, MODE, PER>(a, R, c, m, om, o0, op, zp, zm, seed, stream, sw, ang, invT, acc, qs);
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

template <int POT, bool MASK, bool FIELD, int MODE, int NT, bool PER, bool ODD>
__global__ void __launch_bounds__(NT, march_min_blocks<POT, MASK, NT>()) k_march(PassArgs a) {
  static_assert(MODE == MODE_SWEEP || MODE == MODE_SWEEP_MEASURE, "sweep modes only");
  const int4 u = a.units[blockIdx.x];
  const int r = u.x, c = a.colour;
  const RepDev &R = a.reps[r];
  const RepState *S = a.st + r;
  unsigned acc = 0;
  float qs[kQ];
#pragma unroll
  for (int q = 0; q < kQ; q++) qs[q] = 0.f;
  int slot = -1;  // the sweep's ring slot (measured passes)
  int p = u.y + (int)threadIdx.x;
  bool live = p < R.hp * R.ny;
  if (MASK && (u.w & kUnitTiled)) {  // a tile: kTileW pairs of each of NT / kTileW rows
    const int q = (u.y & ((1 << kTileQBits) - 1)) + ((int)threadIdx.x & (kTileW - 1));
    const int j = (u.y >> kTileQBits) + ((int)threadIdx.x >> kTileLg);
    live = q < R.hp && j < R.ny;
    p = j * R.hp + q;
  }
  if (live) {
    March m;
    march_init<MASK, ODD>(a, R, c, p, u.z, m);
    const int kb = u.z, ke = u.z + (u.w & kUnitPlanes);
    // everything above depends only on constants; the state and the
    // directors may still be written by the previous pass (programmatic
    // dependent launch lets this grid start while that one drains)
    grid_dependency_wait(m);
    // the ring slot read here, off the CTA's tail (headline lattice +0.8%);
    // not in the masked field build, where the live register cost it 1.1%
    if (MODE == MODE_SWEEP_MEASURE && !(MASK && FIELD) && threadIdx.x < kQ) slot = ring_slot(a, S);
    if (MASK && (u.w & kUnitDead))
      dead_unit<FIELD, MODE>(R, m, kb, ke, qs);
    else if (MASK && (u.w & kUnitBulk))  // only bulk sites around: the unmasked update
      march_chunk<POT, false, FIELD, MODE, false>(a, R, c, m, kb, ke, S, acc, qs);
    else
      march_chunk<POT, MASK, FIELD, MODE, PER>(a, R, c, m, kb, ke, S, acc, qs);
  }
  grid_dependency_wait();    // threads without a pair reach here without having waited
  grid_launch_dependents();  // the next pass may start its set-up now
  flush_replica<NT, MODE>(a, r, 1, (unsigned)R.mcta, acc, qs, MASK, -1, slot);
}

}  // namespace mcx
