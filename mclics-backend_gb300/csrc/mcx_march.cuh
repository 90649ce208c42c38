// mcx_march.cuh -- the per-thread state of the z-march passes (the plain
// pass in mcx_march.cu, the learned one in mcx_lmarch.cu): a thread owns one
// same-colour site pair of a row and marches it through a chunk of planes.
#pragma once
#include <cuda_runtime.h>

#include "mcx_pass.cuh"

namespace mcx {

// Opposite-colour director loads of the z-march passes: L2 loads
// (ld.global.cg).  A pass starts under programmatic dependent launch while
// the previous pass, which writes these directors, drains; after
// griddepcontrol.wait, read-only-path loads (__ldg) were seen to return lines
// that an SM's L1 still held from before the previous pass's writes (the
// chain then differed from a launch-by-launch run), while L2 loads always
// see them.
#ifdef MCX_OPP_L1
__device__ __forceinline__ float2 ldo2(const float *p) { return *reinterpret_cast<const float2 *>(p); }
__device__ __forceinline__ float ldo1(const float *p) { return *p; }
#else
__device__ __forceinline__ float2 ldo2(const float *p) { return __ldcg(reinterpret_cast<const float2 *>(p)); }
__device__ __forceinline__ float ldo1(const float *p) { return __ldcg(p); }
#endif

// Programmatic dependent launch: wait until the preceding grid on the stream
// has completed and its memory is visible (returns at once when the launch
// had no programmatic dependency), and let the following grid be scheduled.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" :::); }

// What a measured pass adds for an active site of an unmasked lattice other
// than its bonds (site_update): its Q-tensor products and field energy.
template <bool FIELD>
__device__ __forceinline__ void measure_opposite(const RepDev &R, float x, float y, float z, float qs[kQ]) {
  qs[2] += x * x;
  qs[3] += x * y;
  qs[4] += x * z;
  qs[5] += y * y;
  qs[6] += y * z;
  if (FIELD) {
    const float ef = field_energy(R, x, y, z);
    qs[0] += ef;
    qs[1] += ef;
  }
}

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
  uint8_t tail;                     // odd nx: 1 / 2 when site A / B sits in the row's last slot (0 otherwise)
  float ee0, ee1, eyp, eym;         // bond present: extra x (s = 0, 1), y+1, y-1
};

// griddepcontrol.wait for a march whose director pointers are in m.  The
// pointers pass through the asm as operands, so every director address is
// computed from values that exist only after the wait, and no load through
// them can be scheduled above it, whatever its cache path.
__device__ __forceinline__ void grid_dependency_wait(March &m) {
  asm volatile("griddepcontrol.wait;"
               : "+l"(m.A0), "+l"(m.A1), "+l"(m.A2), "+l"(m.O0), "+l"(m.O1), "+l"(m.O2)
               :
               : "memory");
}

// A dead unit (kUnitDead) of a masked lattice: in measured sweeps with a
// field, each own (inactive) site adds its field energy, in the order the
// full update adds it; nothing else.
// The slot of a phantom site (odd nx, a row whose own sites are odd) is
// skipped.
template <bool FIELD, int MODE>
__device__ __forceinline__ void dead_unit(const RepDev &R, March &m, int kb, int ke, float qs[kQ]) {
  if (!(FIELD && MODE == MODE_SWEEP_MEASURE)) return;
  int s = m.s;
#pragma unroll 1
  for (int k = kb; k < ke; k++) {
    const float2 x = *reinterpret_cast<const float2 *>(m.A0 + m.off);
    const float2 y = *reinterpret_cast<const float2 *>(m.A1 + m.off);
    const float2 z = *reinterpret_cast<const float2 *>(m.A2 + m.off);
    if (!(s && m.tail == 1)) qs[0] += field_energy(R, x.x, y.x, z.x);
    if (m.hasB && !(s && m.tail == 2)) qs[0] += field_energy(R, x.y, y.y, z.y);
    m.off += m.dz;
    s ^= 1;
  }
}

template <bool MASK>
__device__ __forceinline__ void load_opair_at(const March &m, int off, int offp, bool on, OPair &o) {
  if (on) {
    o.v[0] = ldo2(m.O0 + off);
    o.v[1] = ldo2(m.O1 + off);
    o.v[2] = ldo2(m.O2 + off);
    if (MASK) o.pt = __ldg(reinterpret_cast<const uint16_t *>(m.PO + offp));
  } else {
    o.v[0] = o.v[1] = o.v[2] = make_float2(0.f, 0.f);
    if (MASK) o.pt = 0;
  }
}

// The thread's march state for pair p of the plane (p < hp * ny) of colour
// c, starting at plane kb: its geometry, y rows, x extras and the offsets of
// plane kb.  Constants only (no director or state reads).  ODD false: the
// batch has no odd nx, so no pair has a phantom slot (odd_tail).
template <bool MASK, bool ODD = true>
__device__ __forceinline__ void march_init(const PassArgs &a, const RepDev &R, int c, int p, int kb, March &m) {
    const int hs = R.hs, hps = R.hps, ny = R.ny, hx = R.hx;
    const int j = (int)fastdiv((uint32_t)p, R.hp_m, R.hp_p);
    const int h0 = 2 * (p - j * R.hp);
    m.hasB = h0 + 1 < hx;
    m.tail = odd_tail<MASK, ODD>(R, h0);
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

// Resident CTAs per SM the compiler is asked for (measured best): the
// unmasked Lebwohl-Lasher pass at about 96-113 registers per thread; the GHRL
// and masked variants at 128 (they spill a little there, and still run 1.5x
// faster than unconstrained at 160-206 registers, from the doubled occupancy).
#ifndef MCX_MARCH_LL128_BLOCKS
#define MCX_MARCH_LL128_BLOCKS 6
#endif
#ifndef MCX_MARCH_LL256_BLOCKS
#define MCX_MARCH_LL256_BLOCKS 2
#endif
#ifndef MCX_MARCH_MASK_REGS
#define MCX_MARCH_MASK_REGS 128
#endif
template <int POT, bool MASK, int NT>
constexpr int march_min_blocks() {
  return POT == POT_LL && !MASK ? (NT == 64 ? 9 : (NT == 128 ? MCX_MARCH_LL128_BLOCKS : MCX_MARCH_LL256_BLOCKS))
                                : (MCX_MARCH_MASK_REGS > 0 ? 65536 / (NT * MCX_MARCH_MASK_REGS) : 1);
}

// The update of one same-colour pair from its loaded neighbourhood (shared by
// the z-march and its staged and prefetching forms): own directors (ax, ay,
// az) in and out; o0 the opposite pair of the same row, yp / ym those of rows
// y+1 / y-1, op / om those of the planes above / below (zp / zm: those bonds
// exist), exv the extra x neighbour; s the parity of the own sites in this
// row; rw the pair's Philox draw (pair_draw below).
template <int POT, bool MASK, bool FIELD, int MODE, bool PER>
__device__ __forceinline__ void update_pair_draw(const PassArgs &a, const RepDev &R, int c, int s, bool hasB_,
                                                 float ee0, float ee1, float eyp, float eym, const OPair &o0,
                                                 const OPair &yp, const OPair &ym, const OPair &op, const OPair &om,
                                                 const float exv[3], uint16_t pself, uint8_t pex, bool zp, bool zm,
                                                 const uint4 rw, long long ns_at, float ang, float invT, float2 &ax,
                                                 float2 &ay, float2 &az, unsigned &acc, float qs[kQ],
                                                 int tail = 0) {
  float uA[3], uB[3];
  pair_uniforms(rw, uA, uB);
  auto wt = [&](float ee, uint8_t pp) { return MASK ? (ee != 0.f && pp != 0 ? 1.f : 0.f) : ee; };
  // PER: every bond exists (all axes periodic, pairs always complete)
  const float exe = PER ? 1.f : (s ? ee1 : ee0);
  const float erz[4] = {PER ? 1.f : eyp, PER ? 1.f : eym, PER || zp ? 1.f : 0.f, PER || zm ? 1.f : 0.f};
  const bool hasB = PER || hasB_;
  const OPair *rows4[4] = {&yp, &ym, &op, &om};
  const uint8_t lo = (uint8_t)(o0.pt & 0xFF), hi = (uint8_t)(o0.pt >> 8);
  const int P = R.plane;
  float nb[6][3], w[6], e[6];
  // odd nx (masked only): a phantom in the last slot of an s = 1 row is
  // skipped; the last site of an s = 0 row has no x+ bond
  const bool skipA = MASK && s == 1 && tail == 1, skipB = MASK && s == 1 && tail == 2;
  if (!skipA) {  // site A
    if (s == 0) {
      nb[0][0] = o0.v[0].x; nb[0][1] = o0.v[1].x; nb[0][2] = o0.v[2].x; e[0] = 1.f; w[0] = wt(1.f, lo);
      nb[1][0] = exv[0]; nb[1][1] = exv[1]; nb[1][2] = exv[2]; e[1] = exe; w[1] = wt(exe, pex);
    } else {
      if (hasB) {
        nb[0][0] = o0.v[0].y; nb[0][1] = o0.v[1].y; nb[0][2] = o0.v[2].y; e[0] = 1.f; w[0] = wt(1.f, hi);
      } else {
        nb[0][0] = exv[0]; nb[0][1] = exv[1]; nb[0][2] = exv[2]; e[0] = exe; w[0] = wt(exe, pex);
      }
      nb[1][0] = o0.v[0].x; nb[1][1] = o0.v[1].x; nb[1][2] = o0.v[2].x; e[1] = 1.f; w[1] = wt(1.f, lo);
    }
    if (MASK && s == 0 && tail == 1) e[0] = w[0] = 0.f;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const OPair &o = *rows4[q];
      nb[2 + q][0] = o.v[0].x; nb[2 + q][1] = o.v[1].x; nb[2 + q][2] = o.v[2].x;
      e[2 + q] = erz[q];
      w[2 + q] = wt(erz[q], MASK ? (uint8_t)(o.pt & 0xFF) : 1);
    }
    const int ps = MASK ? (pself & 0xFF) : 1;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    if (MASK && ps > 1) {
      const float *nsb = a.ns + R.ns_off + (long long)(c * 3) * P + ns_at;
      sx = __ldg(nsb);
      sy = __ldg(nsb + P);
      sz = __ldg(nsb + 2 * P);
    }
    acc += site_update<POT, MASK, FIELD, MODE>(R, a, c, ax.x, ay.x, az.x, nb, w, e, ps, sx, sy, sz, uA, ang, invT,
                                               0u, qs);
  }
  if (hasB && !skipB) {  // site B
    if (s == 0) {
      nb[0][0] = o0.v[0].y; nb[0][1] = o0.v[1].y; nb[0][2] = o0.v[2].y; e[0] = 1.f; w[0] = wt(1.f, hi);
      nb[1][0] = o0.v[0].x; nb[1][1] = o0.v[1].x; nb[1][2] = o0.v[2].x; e[1] = 1.f; w[1] = wt(1.f, lo);
      if (MASK && tail == 2) e[0] = w[0] = 0.f;
    } else {
      nb[0][0] = exv[0]; nb[0][1] = exv[1]; nb[0][2] = exv[2]; e[0] = exe; w[0] = wt(exe, pex);
      nb[1][0] = o0.v[0].y; nb[1][1] = o0.v[1].y; nb[1][2] = o0.v[2].y; e[1] = 1.f; w[1] = wt(1.f, hi);
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const OPair &o = *rows4[q];
      nb[2 + q][0] = o.v[0].y; nb[2 + q][1] = o.v[1].y; nb[2 + q][2] = o.v[2].y;
      e[2 + q] = erz[q];
      w[2 + q] = wt(erz[q], MASK ? (uint8_t)(o.pt >> 8) : 1);
    }
    const int ps = MASK ? (pself >> 8) : 1;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    if (MASK && ps > 1) {
      const float *nsb = a.ns + R.ns_off + (long long)(c * 3) * P + ns_at + 1;
      sx = __ldg(nsb);
      sy = __ldg(nsb + P);
      sz = __ldg(nsb + 2 * P);
    }
    acc += site_update<POT, MASK, FIELD, MODE>(R, a, c, ax.y, ay.y, az.y, nb, w, e, ps, sx, sy, sz, uB, ang, invT,
                                               0u, qs);
  }
}

// The pair's Philox draw (counter: pair index, sweep, colour; key: seed,
// stream), and update_pair_draw with it.
__device__ __forceinline__ uint4 pair_draw(uint32_t pid, int c, unsigned long long sw, uint32_t seed, uint32_t stream) {
  return philox4x32_10(make_uint4(pid, (uint32_t)sw, (uint32_t)(sw >> 32), TAG_PLAIN | (uint32_t)c), seed, stream);
}

template <int POT, bool MASK, bool FIELD, int MODE, bool PER>
__device__ __forceinline__ void update_pair(const PassArgs &a, const RepDev &R, int c, int s, bool hasB_, float ee0,
                                            float ee1, float eyp, float eym, const OPair &o0, const OPair &yp,
                                            const OPair &ym, const OPair &op, const OPair &om, const float exv[3],
                                            uint16_t pself, uint8_t pex, bool zp, bool zm, uint32_t pid,
                                            long long ns_at, uint32_t seed, uint32_t stream, unsigned long long sw,
                                            float ang, float invT, float2 &ax, float2 &ay, float2 &az, unsigned &acc,
                                            float qs[kQ], int tail = 0) {
  update_pair_draw<POT, MASK, FIELD, MODE, PER>(a, R, c, s, hasB_, ee0, ee1, eyp, eym, o0, yp, ym, op, om, exv, pself,
                                                pex, zp, zm, pair_draw(pid, c, sw, seed, stream), ns_at, ang, invT, ax,
                                                ay, az, acc, qs, tail);
}

}  // namespace mcx
