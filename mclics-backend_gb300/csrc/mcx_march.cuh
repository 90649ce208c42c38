// mcx_march.cuh -- the per-thread state of the z-march passes (the plain
// pass in mcx_march.cu, the learned one in mcx_lmarch.cu): a thread owns one
// same-colour site pair of a row and marches it through a chunk of planes.
#pragma once
#include <cuda_runtime.h>

#include "mcx_pass.cuh"

namespace mcx {

__device__ __forceinline__ float2 ldg2(const float *p) { return __ldg(reinterpret_cast<const float2 *>(p)); }

// Programmatic dependent launch: wait until the preceding grid on the stream
// has completed and its memory is visible (returns at once when the launch
// had no programmatic dependency), and let the following grid be scheduled.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" :::); }

// Opposite-colour pair of one row: 3 components (and point types).
struct OPair {
  float2 v[3];
  uint16_t pt;
};

// Per-thread state of the march.  Offsets are float offsets within a
// (colour, component) plane; the three component planes of a colour are
// reached through three base pointers.
struct March {
  float *A0, *A1, *A2;              // own colour, components x y z
  const float *O0, *O1, *O2;        // opposite colour
  const uint8_t *PA, *PO;           // point types of the two colours (MASK)
  int off, offp;                    // this plane's pair: row * hs + h0, row * hps + h0
  int dz, dzp;                      // one plane further: ny * hs, ny * hps
  int dyp, dym, dypp, dymp;         // rows y+1, y-1 relative to the pair's row
  int dx0, dx1;                     // the extra x neighbour for s = 0, 1
  uint32_t pid, dpid;               // Philox pair counter and its step per plane
  int s;                            // parity of the own sites in this plane
  int h0, row;                      // half-row index of site A; row j + ny * k of this plane
  bool hasB;
  float ee0, ee1, eyp, eym;         // bond present: extra x (s = 0, 1), y+1, y-1
};

template <bool MASK>
__device__ __forceinline__ void load_opair_at(const March &m, int off, int offp, bool on, OPair &o) {
  if (on) {
    o.v[0] = ldg2(m.O0 + off);
    o.v[1] = ldg2(m.O1 + off);
    o.v[2] = ldg2(m.O2 + off);
    if (MASK) o.pt = __ldg(reinterpret_cast<const uint16_t *>(m.PO + offp));
  } else {
    o.v[0] = o.v[1] = o.v[2] = make_float2(0.f, 0.f);
    if (MASK) o.pt = 0;
  }
}

// The thread's march state for pair p of the plane (p < hp * ny) of colour
// c, starting at plane kb: its geometry, y rows, x extras and the offsets of
// plane kb.  Constants only (no director or state reads).
template <bool MASK>
__device__ __forceinline__ void march_init(const PassArgs &a, const RepDev &R, int c, int p, int kb, March &m) {
    const int hs = R.hs, hps = R.hps, ny = R.ny, hx = R.hx;
    const int j = (int)fastdiv((uint32_t)p, R.hp_m, R.hp_p);
    const int h0 = 2 * (p - j * R.hp);
    m.hasB = h0 + 1 < hx;
    // the x neighbour outside the opposite pair: x- of A when s = 0, x+ of B
    // (or of A when the pair has no B) when s = 1
    int ex0 = h0 - 1, ex1 = m.hasB ? h0 + 2 : h0 + 1;
    m.ee0 = m.ee1 = 1.f;
    if (ex0 < 0) { if (R.xb == BOUND_PERIODIC) ex0 = hx - 1; else { m.ee0 = 0.f; ex0 = h0; } }
    if (ex1 == hx) { if (R.xb == BOUND_PERIODIC) ex1 = 0; else { m.ee1 = 0.f; ex1 = h0; } }
    m.dx0 = ex0 - h0;
    m.dx1 = ex1 - h0;
    int jp = j + 1, jm = j - 1;
    m.eyp = m.eym = 1.f;
    if (jp == ny) { if (R.yb == BOUND_PERIODIC) jp = 0; else { m.eyp = 0.f; jp = j; } }
    if (jm < 0) { if (R.yb == BOUND_PERIODIC) jm = ny - 1; else { m.eym = 0.f; jm = j; } }
    m.dyp = (jp - j) * hs;
    m.dym = (jm - j) * hs;
    m.dypp = (jp - j) * hps;
    m.dymp = (jm - j) * hps;
    const int P = R.plane;
    m.A0 = a.dir + R.dir_off + (long long)(c * 3) * P;
    m.A1 = m.A0 + P;
    m.A2 = m.A1 + P;
    m.O0 = a.dir + R.dir_off + (long long)((c ^ 1) * 3) * P;
    m.O1 = m.O0 + P;
    m.O2 = m.O1 + P;
    m.PA = MASK ? a.pt + R.pt_off + (long long)c * R.pplane : nullptr;
    m.PO = MASK ? a.pt + R.pt_off + (long long)(c ^ 1) * R.pplane : nullptr;
    m.dz = ny * hs;
    m.dzp = ny * hps;
    m.off = (j + ny * kb) * hs + h0;
    m.offp = (j + ny * kb) * hps + h0;
    m.pid = (uint32_t)(j + ny * kb) * (uint32_t)R.hp + (uint32_t)(h0 >> 1);
    m.dpid = (uint32_t)ny * (uint32_t)R.hp;
    m.s = (c + j + kb) & 1;
    m.h0 = h0;
    m.row = j + ny * kb;
}

}  // namespace mcx
