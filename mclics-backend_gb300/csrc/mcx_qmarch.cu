// mcx_qmarch.cu -- the z-march of the plain proposal with four same-colour
// sites per thread (k_qmarch), and its launchers.
//
// A thread owns two adjacent same-colour site pairs of a row (half-row slots
// h0 .. h0+3, h0 a multiple of 4) and marches them through its unit's chunk
// of planes, as k_march (mcx_march.cu) marches one pair.  Every director row
// segment it needs is one 16-byte load per component: its own four sites,
// the opposite colour's four sites of the same row (their x neighbours), of
// rows y+1 and y-1 and of the planes above and below (the z pipeline keeps
// the last two in registers), plus one extra opposite site for the remaining
// x neighbour -- 15 vector and 3 scalar loads per four site-updates, against
// 15 and 3 per two in k_march.  The two pairs are independent work for the
// scheduler: two Philox draws and two pair updates interleave, so a warp has
// twice the instructions in flight between its loads and their uses.
//
// Same work units (of 2 x threads pairs), Philox counters (pair index
// row * hp + q, sweep, colour) and pair update (update_pair_draw) as k_march:
// the two agree bit for bit (the energy change fixes its roundings).
// Unmasked batches whose rows hold whole quads (nx a multiple of 8).
#include <cuda_runtime.h>

#include "mcx_march.cuh"

namespace mcx {

// Four opposite-colour sites of one row: 3 components.
struct OQuad {
  float4 v[3];
};

__device__ __forceinline__ void ldq(const float *p0, const float *p1, const float *p2, int off, OQuad &o) {
#ifdef MCX_OPP_L1
  o.v[0] = *reinterpret_cast<const float4 *>(p0 + off);
  o.v[1] = *reinterpret_cast<const float4 *>(p1 + off);
  o.v[2] = *reinterpret_cast<const float4 *>(p2 + off);
#else
  o.v[0] = __ldcg(reinterpret_cast<const float4 *>(p0 + off));
  o.v[1] = __ldcg(reinterpret_cast<const float4 *>(p1 + off));
  o.v[2] = __ldcg(reinterpret_cast<const float4 *>(p2 + off));
#endif
}

// The low (sites h0, h0+1) or high (h0+2, h0+3) pair of a quad as the pair
// update reads it.
__device__ __forceinline__ OPair lo_pair(const OQuad &q) {
  OPair o;
#pragma unroll
  for (int c = 0; c < 3; c++) o.v[c] = make_float2(q.v[c].x, q.v[c].y);
  o.pt = 0x0101;
  return o;
}
__device__ __forceinline__ OPair hi_pair(const OQuad &q) {
  OPair o;
#pragma unroll
  for (int c = 0; c < 3; c++) o.v[c] = make_float2(q.v[c].z, q.v[c].w);
  o.pt = 0x0101;
  return o;
}

// Resident CTAs per SM the compiler is asked for (register budget per thread:
// 65536 / (NT x blocks)).
#ifndef MCX_QMARCH_MIN_BLOCKS_64
#define MCX_QMARCH_MIN_BLOCKS_64 6
#endif
#ifndef MCX_QMARCH_MIN_BLOCKS_128
#define MCX_QMARCH_MIN_BLOCKS_128 3
#endif
#ifndef MCX_QMARCH_MIN_BLOCKS_256
#define MCX_QMARCH_MIN_BLOCKS_256 1
#endif
template <int NT>
constexpr int qmarch_min_blocks() {
  return NT == 64 ? MCX_QMARCH_MIN_BLOCKS_64 : (NT == 128 ? MCX_QMARCH_MIN_BLOCKS_128 : MCX_QMARCH_MIN_BLOCKS_256);
}

template <int POT, bool FIELD, int MODE, int NT, bool PER>
__global__ void __launch_bounds__(NT, qmarch_min_blocks<NT>()) k_qmarch(PassArgs a) {
  static_assert(MODE == MODE_SWEEP || MODE == MODE_SWEEP_MEASURE, "sweep modes only");
  const int4 u = a.units[blockIdx.x];
  const int r = u.x, c = a.colour;
  const RepDev &R = a.reps[r];
  const RepState *S = a.st + r;
  unsigned acc = 0;
  float qs[kQ];
#pragma unroll
  for (int q = 0; q < kQ; q++) qs[q] = 0.f;
  // the thread's pairs: p and p + 1 of the plane (row-major), the same row
  // because a row holds an even number of pairs
  const int p = u.y + 2 * (int)threadIdx.x;
  if (p < R.hp * R.ny) {
    const int hs = R.hs, ny = R.ny, nz = R.nz, hx = R.hx;
    const int j = (int)fastdiv((uint32_t)p, R.hp_m, R.hp_p);
    const int h0 = 2 * (p - j * R.hp);
    // the extra x neighbour: x- of site h0 when s = 0, x+ of site h0+3 when s = 1
    int ex0 = h0 - 1, ex1 = h0 + 4;
    float ee0 = 1.f, ee1 = 1.f;
    if (ex0 < 0) { if (R.xb == BOUND_PERIODIC) ex0 = hx - 1; else { ee0 = 0.f; ex0 = h0; } }
    if (ex1 == hx) { if (R.xb == BOUND_PERIODIC) ex1 = 0; else { ee1 = 0.f; ex1 = h0; } }
    const int dx0 = ex0 - h0, dx1 = ex1 - h0;  // relative to the quad's offset
    int jp = j + 1, jm = j - 1;
    float eyp = 1.f, eym = 1.f;
    if (jp == ny) { if (R.yb == BOUND_PERIODIC) jp = 0; else { eyp = 0.f; jp = j; } }
    if (jm < 0) { if (R.yb == BOUND_PERIODIC) jm = ny - 1; else { eym = 0.f; jm = j; } }
    const int dyp = (jp - j) * hs, dym = (jm - j) * hs, dz = ny * hs;
    const int P = R.plane;
    float *A0 = a.dir + R.dir_off + (long long)(c * 3) * P;
    float *A1 = A0 + P, *A2 = A1 + P;
    const float *O0 = a.dir + R.dir_off + (long long)((c ^ 1) * 3) * P;
    const float *O1 = O0 + P, *O2 = O1 + P;
    const int kb = u.z, ke = u.z + (u.w & kUnitPlanes);
    int off = (j + ny * kb) * hs + h0;
    uint32_t pid = (uint32_t)(j + ny * kb) * (uint32_t)R.hp + (uint32_t)(h0 >> 1);
    const uint32_t dpid = (uint32_t)ny * (uint32_t)R.hp;
    int s = (c + j + kb) & 1;
    const bool zper = R.zb == BOUND_PERIODIC;
    const uint32_t seed = R.seed, stream = R.stream;
    // the previous pass may still write directors and state until here; the
    // pointers pass through the wait so that no load is scheduled above it
    asm volatile("griddepcontrol.wait;" : "+l"(A0), "+l"(A1), "+l"(A2), "+l"(O0), "+l"(O1), "+l"(O2) : : "memory");
    const unsigned long long sw = S->sweep;
    const float ang = S->ang_var, invT = 1.0f / S->T;
    OQuad om, o0, op;
    const bool zm0 = kb > 0 || zper;
    if (zm0) {
      const int wrap = kb == 0 ? nz : 0;
      ldq(O0, O1, O2, off + (wrap - 1) * dz, om);
    } else {
#pragma unroll
      for (int q = 0; q < 3; q++) om.v[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    ldq(O0, O1, O2, off, o0);
    bool zm = zm0;
#pragma unroll 1
    for (int k = kb; k < ke; k++) {
      const bool zp = k + 1 < nz || zper;
      if (zp) {
        ldq(O0, O1, O2, off + (k + 1 < nz ? 1 : 1 - nz) * dz, op);
      } else {
#pragma unroll
        for (int q = 0; q < 3; q++) op.v[q] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      float4 ax = *reinterpret_cast<const float4 *>(A0 + off);
      float4 ay = *reinterpret_cast<const float4 *>(A1 + off);
      float4 az = *reinterpret_cast<const float4 *>(A2 + off);
      const int dx = s ? dx1 : dx0;
      const float xv[3] = {ldo1(O0 + off + dx), ldo1(O1 + off + dx), ldo1(O2 + off + dx)};
      OQuad yp, ym;
      ldq(O0, O1, O2, off + dyp, yp);
      ldq(O0, O1, O2, off + dym, ym);
      const uint4 rwA = pair_draw(pid, c, sw, seed, stream);
      const uint4 rwB = pair_draw(pid + 1, c, sw, seed, stream);
      // pair A (h0, h0+1): its extra x site is the quad's for s = 0 and the
      // opposite site h0+2 for s = 1; pair B (h0+2, h0+3): the opposite site
      // h0+1 for s = 0 and the quad's extra for s = 1
      const float xA[3] = {s ? o0.v[0].z : xv[0], s ? o0.v[1].z : xv[1], s ? o0.v[2].z : xv[2]};
      const float xB[3] = {s ? xv[0] : o0.v[0].y, s ? xv[1] : o0.v[1].y, s ? xv[2] : o0.v[2].y};
      float2 axA = make_float2(ax.x, ax.y), ayA = make_float2(ay.x, ay.y), azA = make_float2(az.x, az.y);
      float2 axB = make_float2(ax.z, ax.w), ayB = make_float2(ay.z, ay.w), azB = make_float2(az.z, az.w);
      update_pair_draw<POT, false, FIELD, MODE, PER>(a, R, c, s, true, ee0, 1.f, eyp, eym, lo_pair(o0), lo_pair(yp),
                                                     lo_pair(ym), lo_pair(op), lo_pair(om), xA, 0x0101, 1, zp, zm,
                                                     rwA, off, ang, invT, axA, ayA, azA, acc, qs);
      update_pair_draw<POT, false, FIELD, MODE, PER>(a, R, c, s, true, 1.f, ee1, eyp, eym, hi_pair(o0), hi_pair(yp),
                                                     hi_pair(ym), hi_pair(op), hi_pair(om), xB, 0x0101, 1, zp, zm,
                                                     rwB, off + 2, ang, invT, axB, ayB, azB, acc, qs);
      if (MODE == MODE_SWEEP_MEASURE && a.meas_both && c == 1) {  // the colour-0 quad of this row (PassArgs::meas_both)
        measure_opposite<FIELD>(R, o0.v[0].x, o0.v[1].x, o0.v[2].x, qs);
        measure_opposite<FIELD>(R, o0.v[0].y, o0.v[1].y, o0.v[2].y, qs);
        measure_opposite<FIELD>(R, o0.v[0].z, o0.v[1].z, o0.v[2].z, qs);
        measure_opposite<FIELD>(R, o0.v[0].w, o0.v[1].w, o0.v[2].w, qs);
      }
      *reinterpret_cast<float4 *>(A0 + off) = make_float4(axA.x, axA.y, axB.x, axB.y);
      *reinterpret_cast<float4 *>(A1 + off) = make_float4(ayA.x, ayA.y, ayB.x, ayB.y);
      *reinterpret_cast<float4 *>(A2 + off) = make_float4(azA.x, azA.y, azB.x, azB.y);
      om = o0;
      o0 = op;
      zm = true;
      off += dz;
      pid += dpid;
      s ^= 1;
    }
  }
  grid_dependency_wait();    // threads without pairs reach here without having waited
  grid_launch_dependents();  // the next pass may start its set-up now
  flush_replica<NT, MODE>(a, r, 1, (unsigned)R.mcta, acc, qs, false);
}

template <int POT, bool FIELD, int NT>
static const void *qmarch_fn(const Variant &v, int mode) {
  if (mode == MODE_SWEEP_MEASURE)
    return v.per ? (const void *)k_qmarch<POT, FIELD, MODE_SWEEP_MEASURE, NT, true>
                 : (const void *)k_qmarch<POT, FIELD, MODE_SWEEP_MEASURE, NT, false>;
  return v.per ? (const void *)k_qmarch<POT, FIELD, MODE_SWEEP, NT, true>
               : (const void *)k_qmarch<POT, FIELD, MODE_SWEEP, NT, false>;
}

template <int NT>
static const void *qmarch_fn_v(const Variant &v, int mode) {
  if (v.pot == POT_LL) return v.field ? qmarch_fn<POT_LL, true, NT>(v, mode) : qmarch_fn<POT_LL, false, NT>(v, mode);
  if (v.pot == POT_PEAR)
    return v.field ? qmarch_fn<POT_PEAR, true, NT>(v, mode) : qmarch_fn<POT_PEAR, false, NT>(v, mode);
  return v.field ? qmarch_fn<POT_GHRL, true, NT>(v, mode) : qmarch_fn<POT_GHRL, false, NT>(v, mode);
}

static const void *qmarch_kernel(const Variant &v, int mode, int nt) {
  switch (nt) {
    case 64: return qmarch_fn_v<64>(v, mode);
    case 256: return qmarch_fn_v<256>(v, mode);
    default: return qmarch_fn_v<128>(v, mode);
  }
}

bool qmarch_prepare(const Variant &v, int nt) {
  if (v.mask || !march_block_ok(nt)) return false;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, qmarch_kernel(v, MODE_SWEEP, nt), nt, 0) != cudaSuccess)
    return false;
  return n > 0;
}

int qmarch_blocks_per_sm(const Variant &v, int nt) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, qmarch_kernel(v, MODE_SWEEP, nt), nt, 0) != cudaSuccess)
    return 0;
  return n;
}

void launch_qmarch(const Variant &v, int mode, const PassArgs &a, int nt, bool pdl, cudaStream_t st) {
  if (v.mask) return;  // never selected there (qmarch_prepare is false)
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
  cudaLaunchKernelExC(&cfg, qmarch_kernel(v, mode, nt), params);
}

}  // namespace mcx
