// mcx_march.cu -- the plain-proposal red/black pass as a z-march (the sweep
// kernel of mcx_sweep for the reference's rotation move).
//
//   k_march  one red/black half-sweep of every replica (EvolveN::
//            Monte_Carlo_Step, src/evolve.cpp:64-179 of the reference, with 2
//            colours instead of 8).  A CTA owns NT consecutive same-colour
//            site pairs of one z-plane (pairs numbered row-major within the
//            plane) and marches them through a chunk of K planes.  Per plane
//            a thread loads its own pair (3 float2), the opposite colour's
//            pair in the same row (its x neighbours), one extra opposite site
//            (the remaining x neighbour) and the opposite pairs of rows y+1
//            and y-1; the z neighbours are the opposite-colour pairs of the
//            previous and next plane's row, which the march already holds in
//            registers (in the split layout the opposite site above or below
//            a colour-c site has the same half-row index).  The pair's
//            geometry, its y rows and its x extras are computed once per
//            chunk; the Philox key schedule once per thread.
//
// Results are bit-identical to the other passes (same site_update, same
// Philox counter: pair index row * hp + q, sweep, colour).
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

// One plane of the march: the pair at m.off with its z neighbours om (plane
// below) and op (plane above; zp/zm: those bonds exist).
template <int POT, bool MASK, bool FIELD, int MODE, bool PER>
__device__ __forceinline__ void march_plane(const PassArgs &a, const RepDev &R, int c, const March &m,
                                            const OPair &om, const OPair &o0, const OPair &op, bool zp, bool zm,
                                            uint32_t seed, uint32_t stream, unsigned long long sw, float ang,
                                            float invT, unsigned &acc, float qs[kQ]) {
  // loads first, so that the Philox rounds below overlap them
  float2 ax = *reinterpret_cast<const float2 *>(m.A0 + m.off);
  float2 ay = *reinterpret_cast<const float2 *>(m.A1 + m.off);
  float2 az = *reinterpret_cast<const float2 *>(m.A2 + m.off);
  const int dx = m.s ? m.dx1 : m.dx0;
  const float exv[3] = {__ldg(m.O0 + m.off + dx), __ldg(m.O1 + m.off + dx), __ldg(m.O2 + m.off + dx)};
  OPair yp, ym;
  load_opair_at<MASK>(m, m.off + m.dyp, m.offp + m.dypp, true, yp);
  load_opair_at<MASK>(m, m.off + m.dym, m.offp + m.dymp, true, ym);
  uint16_t pself = 0x0101;
  uint8_t pex = 1;
  if (MASK) {
    pself = __ldg(reinterpret_cast<const uint16_t *>(m.PA + m.offp));
    pex = __ldg(m.PO + m.offp + dx);
  }
  const uint4 rw = philox4x32_10(make_uint4(m.pid, (uint32_t)sw, (uint32_t)(sw >> 32), TAG_PLAIN | (uint32_t)c), seed,
                                 stream);
  float uA[3], uB[3];
  pair_uniforms(rw, uA, uB);
  auto wt = [&](float ee, uint8_t pp) { return MASK ? (ee != 0.f && pp != 0 ? 1.f : 0.f) : ee; };
  // PER: every bond exists (all axes periodic, pairs always complete)
  const float exe = PER ? 1.f : (m.s ? m.ee1 : m.ee0);
  const float erz[4] = {PER ? 1.f : m.eyp, PER ? 1.f : m.eym, PER || zp ? 1.f : 0.f, PER || zm ? 1.f : 0.f};
  const bool hasB = PER || m.hasB;
  const OPair *rows4[4] = {&yp, &ym, &op, &om};
  const uint8_t lo = (uint8_t)(o0.pt & 0xFF), hi = (uint8_t)(o0.pt >> 8);
  float nb[6][3], w[6], e[6];
  {  // site A
    if (m.s == 0) {
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
      const float *nsb = a.ns + R.ns_off + (long long)(c * 3) * R.plane + m.off;
      sx = __ldg(nsb);
      sy = __ldg(nsb + R.plane);
      sz = __ldg(nsb + 2 * R.plane);
    }
    acc += site_update<POT, MASK, FIELD, MODE>(R, a, c, ax.x, ay.x, az.x, nb, w, e, ps, sx, sy, sz, uA, ang, invT,
                                               0u, qs);
  }
  if (hasB) {  // site B
    if (m.s == 0) {
      nb[0][0] = o0.v[0].y; nb[0][1] = o0.v[1].y; nb[0][2] = o0.v[2].y; e[0] = 1.f; w[0] = wt(1.f, hi);
      nb[1][0] = o0.v[0].x; nb[1][1] = o0.v[1].x; nb[1][2] = o0.v[2].x; e[1] = 1.f; w[1] = wt(1.f, lo);
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
      const float *nsb = a.ns + R.ns_off + (long long)(c * 3) * R.plane + m.off + 1;
      sx = __ldg(nsb);
      sy = __ldg(nsb + R.plane);
      sz = __ldg(nsb + 2 * R.plane);
    }
    acc += site_update<POT, MASK, FIELD, MODE>(R, a, c, ax.y, ay.y, az.y, nb, w, e, ps, sx, sy, sz, uB, ang, invT,
                                               0u, qs);
  }
  *reinterpret_cast<float2 *>(m.A0 + m.off) = ax;
  *reinterpret_cast<float2 *>(m.A1 + m.off) = ay;
  *reinterpret_cast<float2 *>(m.A2 + m.off) = az;
}

// Resident CTAs per SM the compiler is asked for (measured best): the
// unmasked Lebwohl-Lasher pass at about 96-113 registers per thread; the GHRL
// and masked variants at 128 (they spill a little there, and still run 1.5x
// faster than unconstrained at 160-206 registers, from the doubled occupancy).
#ifndef MCX_MARCH_MASK_REGS
#define MCX_MARCH_MASK_REGS 128
#endif
template <int POT, bool MASK, int NT>
constexpr int march_min_blocks() {
  return POT == POT_LL && !MASK ? (NT == 64 ? 9 : (NT == 128 ? 5 : 2))
                                : (MCX_MARCH_MASK_REGS > 0 ? 65536 / (NT * MCX_MARCH_MASK_REGS) : 1);
}

template <int POT, bool MASK, bool FIELD, int MODE, int NT, bool PER>
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
  const int p = u.y + (int)threadIdx.x;
  if (p < R.hp * R.ny) {
    const int hs = R.hs, hps = R.hps, ny = R.ny, nz = R.nz, hx = R.hx;
    March m;
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
    const bool zper = R.zb == BOUND_PERIODIC;
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
    const int kb = u.z, ke = u.z + u.w;
    m.off = (j + ny * kb) * hs + h0;
    m.offp = (j + ny * kb) * hps + h0;
    m.pid = (uint32_t)(j + ny * kb) * (uint32_t)R.hp + (uint32_t)(h0 >> 1);
    m.dpid = (uint32_t)ny * (uint32_t)R.hp;
    m.s = (c + j + kb) & 1;
    const uint32_t seed = R.seed, stream = R.stream;
    // everything above depends only on constants; the state and the
    // directors may still be written by the previous pass (programmatic
    // dependent launch lets this grid start while that one drains)
    grid_dependency_wait();
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
      m.s ^= 1;
    }
  }
  grid_dependency_wait();    // threads without a pair reach here without having waited
  grid_launch_dependents();  // the next pass may start its set-up now
  flush_replica<NT, MODE>(a, r, 1, (unsigned)R.mcta, acc, qs, MASK);
}

// ---------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------
template <int POT, bool MASK, bool FIELD, int NT, bool PER>
static const void *march_fn(int mode) {
  return mode == MODE_SWEEP_MEASURE ? (const void *)k_march<POT, MASK, FIELD, MODE_SWEEP_MEASURE, NT, PER>
                                    : (const void *)k_march<POT, MASK, FIELD, MODE_SWEEP, NT, PER>;
}

template <int POT, bool FIELD, int NT>
static const void *march_fn_unmasked(const Variant &v, int mode) {
  return v.per ? march_fn<POT, false, FIELD, NT, true>(mode) : march_fn<POT, false, FIELD, NT, false>(mode);
}

template <int NT>
static const void *march_fn_v(const Variant &v, int mode) {
  if (v.pot == POT_LL) {
    if (v.mask)
      return v.field ? march_fn<POT_LL, true, true, NT, false>(mode) : march_fn<POT_LL, true, false, NT, false>(mode);
    return v.field ? march_fn_unmasked<POT_LL, true, NT>(v, mode) : march_fn_unmasked<POT_LL, false, NT>(v, mode);
  }
  if (v.mask)
    return v.field ? march_fn<POT_GHRL, true, true, NT, false>(mode) : march_fn<POT_GHRL, true, false, NT, false>(mode);
  return v.field ? march_fn_unmasked<POT_GHRL, true, NT>(v, mode) : march_fn_unmasked<POT_GHRL, false, NT>(v, mode);
}

static const void *march_kernel(const Variant &v, int mode, int nt) {
  switch (nt) {
    case 64: return march_fn_v<64>(v, mode);
    case 256: return march_fn_v<256>(v, mode);
    default: return march_fn_v<128>(v, mode);
  }
}

bool march_block_ok(int nt) { return nt == 64 || nt == 128 || nt == 256; }

int march_blocks_per_sm(const Variant &v, int mode, int nt) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, march_kernel(v, mode, nt), nt, 0) != cudaSuccess) return 0;
  return n;
}

void launch_march(const Variant &v, int mode, const PassArgs &a, int nt, bool pdl, cudaStream_t st) {
  PassArgs args = a;
  void *params[] = {&args};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(a.nunits);
  cfg.blockDim = dim3(nt);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelExC(&cfg, march_kernel(v, mode, nt), params);
}

}  // namespace mcx
