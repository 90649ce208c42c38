// mcx_kernels.cu -- sm_103a kernels of the GB300 Metropolis engine.
//
//   k_sweep_pass   one red/black half-sweep of every replica in the batch
//                  (EvolveN::Monte_Carlo_Step, src/evolve.cpp:64-179 of the
//                  reference, 2 colours instead of 8): one thread updates 4
//                  consecutive same-colour sites of a row from float4 loads of
//                  its own colour and of the 5 neighbouring rows of the other
//                  colour; Philox4x32-10 per site; the acceptance count is
//                  warp-reduced into the replica's state.
//   k_measure      E and the Q-tensor sums of every replica in one pass over
//                  the lattice (energy_calculator, src/evolve.cpp:27-62, and
//                  Matrice_constructor, src/parameter_order.cpp:30-60):
//                  every bond has exactly one colour-1 end, so a colour-1
//                  thread sums its 6 bonds; warp shuffles + a block reduction
//                  in FP64, one FP64 atomic per block and quantity.
//   k_epilogue     per replica: the step-size rule (src/evolve.cpp:169-178),
//                  the RNG counter, and for measured sweeps S = largest
//                  eigenvalue of Q in FP64 and the running sums.
#include <cuda_runtime.h>

#include "mcx_device.cuh"
#include "mcx_kernels.cuh"

namespace mcx {

__device__ __forceinline__ float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void st4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }
__device__ __forceinline__ float comp(const float4 &v, int q) { return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w; }
__device__ __forceinline__ void setc(float4 &v, int q, float x) {
  if (q == 0) v.x = x;
  else if (q == 1) v.y = x;
  else if (q == 2) v.z = x;
  else v.w = x;
}
__device__ __forceinline__ uint8_t compb(uchar4 v, int q) { return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w; }

// The neighbourhood of one float4 group: own colour (a*), the other colour in
// the same row (o*), the four rows y+-1, z+-1 of the other colour, and the
// one extra other-colour site that the row's x neighbours need beyond the
// group (at h = 4*h4 - 1 when s = 0, at h = 4*h4 + 4 when s = 1, wrapped or
// absent at the row ends).
struct Group {
  int h4, j, k, s, q_ex;
  long long row, base;
  float4 ax, ay, az, ox, oy, oz;
  float4 n[4][3];  // y+, y-, z+, z- rows of the other colour
  bool e[4];       // row exists (boundary)
  float exx, exy, exz;
  bool ex_e;
  uchar4 pa, po, pn[4];
  uint8_t ex_pt;
};

template <bool MASK>
__device__ __forceinline__ void load_group(const RepDev &R, const float *__restrict__ dir, const uint8_t *__restrict__ pt,
                                           int c, long long g, Group &G) {
  const int g4 = R.g4, ny = R.ny, nz = R.nz, hx = R.hx, hs = R.hs;
  G.h4 = (int)(g % g4);
  G.row = g / g4;
  G.j = (int)(G.row % ny);
  G.k = (int)(G.row / ny);
  const int o = c ^ 1;
  G.s = (c + G.j + G.k) & 1;
  const long long plane = R.plane;
  const float *A = dir + R.dir_off + (long long)(c * 3) * plane;
  const float *O = dir + R.dir_off + (long long)(o * 3) * plane;
  G.base = G.row * hs + 4 * G.h4;
  G.ax = ld4(A + G.base);
  G.ay = ld4(A + plane + G.base);
  G.az = ld4(A + 2 * plane + G.base);
  G.ox = __ldg(reinterpret_cast<const float4 *>(O + G.base));
  G.oy = __ldg(reinterpret_cast<const float4 *>(O + plane + G.base));
  G.oz = __ldg(reinterpret_cast<const float4 *>(O + 2 * plane + G.base));
  int jj[4] = {G.j + 1, G.j - 1, G.j, G.j};
  int kk[4] = {G.k, G.k, G.k + 1, G.k - 1};
#pragma unroll
  for (int t = 0; t < 4; t++) {
    bool ex = true;
    if (t < 2) {
      if (jj[t] == ny) { if (R.yb == BOUND_PERIODIC) jj[t] = 0; else ex = false; }
      if (jj[t] < 0) { if (R.yb == BOUND_PERIODIC) jj[t] = ny - 1; else ex = false; }
    } else {
      if (kk[t] == nz) { if (R.zb == BOUND_PERIODIC) kk[t] = 0; else ex = false; }
      if (kk[t] < 0) { if (R.zb == BOUND_PERIODIC) kk[t] = nz - 1; else ex = false; }
    }
    G.e[t] = ex;
    const long long b = ((long long)jj[t] + (long long)ny * kk[t]) * hs + 4 * G.h4;
    if (ex) {
      G.n[t][0] = __ldg(reinterpret_cast<const float4 *>(O + b));
      G.n[t][1] = __ldg(reinterpret_cast<const float4 *>(O + plane + b));
      G.n[t][2] = __ldg(reinterpret_cast<const float4 *>(O + 2 * plane + b));
      if (MASK) G.pn[t] = __ldg(reinterpret_cast<const uchar4 *>(pt + R.pt_off + (long long)o * plane + b));
    } else {
      G.n[t][0] = G.n[t][1] = G.n[t][2] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (MASK) G.pn[t] = make_uchar4(0, 0, 0, 0);
    }
  }
  int exh;
  G.ex_e = true;
  if (G.s == 0) {
    exh = 4 * G.h4 - 1;
    if (exh < 0) { if (R.xb == BOUND_PERIODIC) exh = hx - 1; else G.ex_e = false; }
    G.q_ex = 0;
  } else {
    exh = 4 * G.h4 + 4;
    if (exh >= hx) { if (R.xb == BOUND_PERIODIC) exh = 0; else G.ex_e = false; }
    G.q_ex = min(3, hx - 1 - 4 * G.h4);
  }
  G.exx = G.exy = G.exz = 0.f;
  G.ex_pt = 0;
  if (G.ex_e) {
    const long long b = G.row * hs + exh;
    G.exx = __ldg(O + b);
    G.exy = __ldg(O + plane + b);
    G.exz = __ldg(O + 2 * plane + b);
    if (MASK) G.ex_pt = __ldg(pt + R.pt_off + (long long)o * plane + b);
  }
  if (MASK) {
    G.pa = __ldg(reinterpret_cast<const uchar4 *>(pt + R.pt_off + (long long)c * plane + G.base));
    G.po = __ldg(reinterpret_cast<const uchar4 *>(pt + R.pt_off + (long long)o * plane + G.base));
  }
}

// Neighbour directors and weights (1 = bond present and neighbour active) of
// site q of the group, in the reference slot order x+, x-, y+, y-, z+, z-.
template <bool MASK, int Q>
__device__ __forceinline__ void site_neighbours(const Group &G, float nb[6][3], float w[6]) {
  // x-
  float mx, my, mz, mw;
  float px, py, pz, pw;
  if (G.s == 0) {
    if (Q == 0) {
      mx = G.exx; my = G.exy; mz = G.exz;
      mw = G.ex_e ? (MASK ? (G.ex_pt != 0 ? 1.f : 0.f) : 1.f) : 0.f;
    } else {
      mx = comp(G.ox, Q - 1); my = comp(G.oy, Q - 1); mz = comp(G.oz, Q - 1);
      mw = MASK ? (compb(G.po, Q - 1) != 0 ? 1.f : 0.f) : 1.f;
    }
    px = comp(G.ox, Q); py = comp(G.oy, Q); pz = comp(G.oz, Q);
    pw = MASK ? (compb(G.po, Q) != 0 ? 1.f : 0.f) : 1.f;
  } else {
    mx = comp(G.ox, Q); my = comp(G.oy, Q); mz = comp(G.oz, Q);
    mw = MASK ? (compb(G.po, Q) != 0 ? 1.f : 0.f) : 1.f;
    if (Q == 3 || G.q_ex == Q) {
      px = G.exx; py = G.exy; pz = G.exz;
      pw = G.ex_e ? (MASK ? (G.ex_pt != 0 ? 1.f : 0.f) : 1.f) : 0.f;
    } else {
      const int q1 = Q < 3 ? Q + 1 : 3;
      px = comp(G.ox, q1); py = comp(G.oy, q1); pz = comp(G.oz, q1);
      pw = MASK ? (compb(G.po, q1) != 0 ? 1.f : 0.f) : 1.f;
    }
  }
  nb[0][0] = px; nb[0][1] = py; nb[0][2] = pz; w[0] = pw;
  nb[1][0] = mx; nb[1][1] = my; nb[1][2] = mz; w[1] = mw;
#pragma unroll
  for (int t = 0; t < 4; t++) {
    nb[2 + t][0] = comp(G.n[t][0], Q);
    nb[2 + t][1] = comp(G.n[t][1], Q);
    nb[2 + t][2] = comp(G.n[t][2], Q);
    w[2 + t] = G.e[t] ? (MASK ? (compb(G.pn[t], Q) != 0 ? 1.f : 0.f) : 1.f) : 0.f;
  }
}

// Bond energy of director a with neighbour b in slot d.
template <int POT, int D>
__device__ __forceinline__ float bond(const RepDev &R, float ax, float ay, float az, const float b[3]) {
  if (POT == POT_LL) {
    const float nij = ax * b[0] + ay * b[1] + az * b[2];
    return -1.5f * R.A * nij * nij;
  } else {
    return ghrl_bond<(D >> 1)>(R, ax, ay, az, b[0], b[1], b[2], (D & 1) ? -1.f : 1.f);
  }
}

// Energy change of replacing n0 by p at a site with neighbours nb / w.
template <int POT>
__device__ __forceinline__ float bonds_delta(const RepDev &R, float n0x, float n0y, float n0z, float px, float py,
                                             float pz, const float nb[6][3], const float w[6]) {
  if (POT == POT_LL) {
    float acc = 0.f;
#pragma unroll
    for (int d = 0; d < 6; d++) {
      const float dn = n0x * nb[d][0] + n0y * nb[d][1] + n0z * nb[d][2];
      const float dp = px * nb[d][0] + py * nb[d][1] + pz * nb[d][2];
      // the 0/1 weight multiplies one factor exactly, so masked and unmasked
      // specialisations round identically
      acc = fmaf((dp - dn) * w[d], dp + dn, acc);
    }
    return -1.5f * R.A * acc;
  } else {
    float acc = 0.f;
    acc = fmaf(w[0], bond<POT, 0>(R, px, py, pz, nb[0]) - bond<POT, 0>(R, n0x, n0y, n0z, nb[0]), acc);
    acc = fmaf(w[1], bond<POT, 1>(R, px, py, pz, nb[1]) - bond<POT, 1>(R, n0x, n0y, n0z, nb[1]), acc);
    acc = fmaf(w[2], bond<POT, 2>(R, px, py, pz, nb[2]) - bond<POT, 2>(R, n0x, n0y, n0z, nb[2]), acc);
    acc = fmaf(w[3], bond<POT, 3>(R, px, py, pz, nb[3]) - bond<POT, 3>(R, n0x, n0y, n0z, nb[3]), acc);
    acc = fmaf(w[4], bond<POT, 4>(R, px, py, pz, nb[4]) - bond<POT, 4>(R, n0x, n0y, n0z, nb[4]), acc);
    acc = fmaf(w[5], bond<POT, 5>(R, px, py, pz, nb[5]) - bond<POT, 5>(R, n0x, n0y, n0z, nb[5]), acc);
    return acc;
  }
}

template <int POT>
__device__ __forceinline__ float bonds_energy(const RepDev &R, float x, float y, float z, const float nb[6][3],
                                              const float w[6]) {
  return w[0] * bond<POT, 0>(R, x, y, z, nb[0]) + w[1] * bond<POT, 1>(R, x, y, z, nb[1]) +
         w[2] * bond<POT, 2>(R, x, y, z, nb[2]) + w[3] * bond<POT, 3>(R, x, y, z, nb[3]) +
         w[4] * bond<POT, 4>(R, x, y, z, nb[4]) + w[5] * bond<POT, 5>(R, x, y, z, nb[5]);
}

// Rotated proposal (src/evolve.cpp:136-152 / src/evolve.cu:143-163): rotate by
// pi*va about x (u1 < 0.333), y (u1 < 0.666) or z, then renormalise.  sin and
// cos are taken of |angle| and the sign restored, so the move and its reverse
// are exact mirror images (a symmetric proposal).
__device__ __forceinline__ void propose(float n0x, float n0y, float n0z, float u0, float u1, float ang, float &px,
                                        float &py, float &pz) {
  const float va = (2.f * u0 - 1.f) * ang;
  const float th = 3.14159265358979f * va;
  const float at = fabsf(th);
  float sn = __sinf(at);
  const float cs = __cosf(at);
  sn = copysignf(sn, th);
  if (u1 < 0.333f) {
    px = n0x;
    py = n0y * cs + n0z * sn;
    pz = n0z * cs - n0y * sn;
  } else if (u1 < 0.666f) {
    px = n0x * cs - n0z * sn;
    py = n0y;
    pz = n0z * cs + n0x * sn;
  } else {
    px = n0x * cs + n0y * sn;
    py = n0y * cs - n0x * sn;
    pz = n0z;
  }
  const float inv = rsqrtf(px * px + py * py + pz * pz);
  px *= inv;
  py *= inv;
  pz *= inv;
}

template <int POT, bool MASK, bool FIELD, bool TRACE, int Q>
__device__ __forceinline__ unsigned update_site(const RepDev &R, const PassArgs &a, Group &G, float ang, float invT,
                                                uint32_t sw_lo, uint32_t sw_hi) {
  const int h = 4 * G.h4 + Q;
  const int i = 2 * h + G.s;
  const uint32_t nat = (uint32_t)i + (uint32_t)R.nx * ((uint32_t)G.j + (uint32_t)R.ny * (uint32_t)G.k);
  bool act = h < R.hx;
  const uint8_t pself = MASK ? compb(G.pa, Q) : 1;
  if (MASK) act = act && pself != 0;
  if (!act) {
    if (TRACE && h < R.hx) {
      a.tr_dE[nat] = 0.f;
      a.tr_acc[nat] = 255;
    }
    return 0;
  }
  float nb[6][3], w[6];
  site_neighbours<MASK, Q>(G, nb, w);
  const float n0x = comp(G.ax, Q), n0y = comp(G.ay, Q), n0z = comp(G.az, Q);
  const uint4 r = philox4x32_10(make_uint4(nat, sw_lo, sw_hi, TAG_PLAIN), R.seed, R.stream);
  float px, py, pz;
  propose(n0x, n0y, n0z, u01(r.x), u01(r.y), ang, px, py, pz);
  float dE = bonds_delta<POT>(R, n0x, n0y, n0z, px, py, pz, nb, w);
  if (MASK && pself > 1) {
    const long long sb = R.ns_off + (long long)(a.colour * 3) * R.plane + G.base + Q;
    const float sx = __ldg(a.ns + sb), sy = __ldg(a.ns + sb + R.plane), sz = __ldg(a.ns + sb + 2 * R.plane);
    const int sid = pself - 2;
    if (sid < R.nsurf)
      dE += surface_energy(R, sid, px, py, pz, sx, sy, sz) - surface_energy(R, sid, n0x, n0y, n0z, sx, sy, sz);
  }
  if (FIELD) dE += field_energy(R, px, py, pz) - field_energy(R, n0x, n0y, n0z);
  // src/evolve.cpp:160: accept when u < exp(-(E_new - E_old)/T)
  const bool accept = u01(r.z) < __expf(-dE * invT);
  if (TRACE) {
    a.tr_dE[nat] = dE;
    a.tr_acc[nat] = accept ? 1 : 0;
    a.tr_prop[3 * (size_t)nat] = px;
    a.tr_prop[3 * (size_t)nat + 1] = py;
    a.tr_prop[3 * (size_t)nat + 2] = pz;
  }
  if (accept) {
    setc(G.ax, Q, px);
    setc(G.ay, Q, py);
    setc(G.az, Q, pz);
    return 1;
  }
  return 0;
}

template <int POT, bool MASK, bool FIELD, bool TRACE>
__global__ void __launch_bounds__(kBlock) k_sweep_pass(PassArgs a) {
  const int2 m = a.map[blockIdx.x];
  const RepDev &R = a.reps[m.x];
  RepState *S = a.st + m.x;
  const long long g = (long long)m.y + threadIdx.x;
  unsigned nacc = 0;
  if (g < R.ngroups) {
    const float ang = S->ang_var;
    const float invT = 1.0f / S->T;
    const unsigned long long sw = S->sweep;
    const uint32_t lo = (uint32_t)sw, hi = (uint32_t)(sw >> 32);
    Group G;
    load_group<MASK>(R, a.dir, a.pt, a.colour, g, G);
    nacc += update_site<POT, MASK, FIELD, TRACE, 0>(R, a, G, ang, invT, lo, hi);
    nacc += update_site<POT, MASK, FIELD, TRACE, 1>(R, a, G, ang, invT, lo, hi);
    nacc += update_site<POT, MASK, FIELD, TRACE, 2>(R, a, G, ang, invT, lo, hi);
    nacc += update_site<POT, MASK, FIELD, TRACE, 3>(R, a, G, ang, invT, lo, hi);
    float *A = a.dir + R.dir_off + (long long)(a.colour * 3) * R.plane + G.base;
    st4(A, G.ax);
    st4(A + R.plane, G.ay);
    st4(A + 2 * R.plane, G.az);
  }
  const unsigned wsum = __reduce_add_sync(0xffffffffu, nacc);
  if ((threadIdx.x & 31) == 0 && wsum) atomicAdd(&S->acc, wsum);
}

// ---------------------------------------------------------------------------
// Measurement.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int POT, bool MASK, bool FIELD, int Q>
__device__ __forceinline__ void measure_site(const RepDev &R, const MeasureArgs &a, const Group &G, float acc[kMacc]) {
  const int h = 4 * G.h4 + Q;
  if (h >= R.hx) return;
  // colour-1 site: all 6 of its bonds (every bond has one colour-1 end)
  {
    const uint8_t p1 = MASK ? compb(G.pa, Q) : 1;
    float nb[6][3], w[6];
    site_neighbours<MASK, Q>(G, nb, w);
    // w[d] = 1 when the bond exists and the neighbour is active; weight of a
    // bond in the all-site energy: [pt_j != 0] + [pt_i != 0] over existing
    // bonds (src/evolve.cpp:27-62 sums every site's local energy).
    float wc[6], wv[6];
    const float a1 = p1 != 0 ? 1.f : 0.f;
    float ex[6] = {1, 1, G.e[0] ? 1.f : 0.f, G.e[1] ? 1.f : 0.f, G.e[2] ? 1.f : 0.f, G.e[3] ? 1.f : 0.f};
    if (G.s == 0) { if (Q == 0) ex[1] = G.ex_e ? 1.f : 0.f; }
    else if (Q == 3 || G.q_ex == Q) ex[0] = G.ex_e ? 1.f : 0.f;
#pragma unroll
    for (int d = 0; d < 6; d++) {
      wc[d] = w[d] + ex[d] * a1;
      wv[d] = 2.f * w[d] * a1;
    }
    const float x = comp(G.ax, Q), y = comp(G.ay, Q), z = comp(G.az, Q);
    float eb[6];
    eb[0] = bond<POT, 0>(R, x, y, z, nb[0]);
    eb[1] = bond<POT, 1>(R, x, y, z, nb[1]);
    eb[2] = bond<POT, 2>(R, x, y, z, nb[2]);
    eb[3] = bond<POT, 3>(R, x, y, z, nb[3]);
    eb[4] = bond<POT, 4>(R, x, y, z, nb[4]);
    eb[5] = bond<POT, 5>(R, x, y, z, nb[5]);
#pragma unroll
    for (int d = 0; d < 6; d++) {
      acc[0] += wc[d] * eb[d];
      acc[1] += wv[d] * eb[d];
    }
    if (MASK && p1 > 1 && p1 - 2 < R.nsurf) {
      const long long sb = R.ns_off + 3LL * R.plane + G.base + Q;
      const float e = surface_energy(R, p1 - 2, x, y, z, __ldg(a.ns + sb), __ldg(a.ns + sb + R.plane),
                                     __ldg(a.ns + sb + 2 * R.plane));
      acc[0] += e;
      acc[1] += e;
    }
    if (FIELD) {
      const float e = field_energy(R, x, y, z);
      acc[0] += e;
      acc[1] += a1 * e;
    }
    if (a1 != 0.f) {
      acc[2] += x * x; acc[3] += x * y; acc[4] += x * z;
      acc[5] += y * y; acc[6] += y * z; acc[7] += z * z;
    }
  }
  // colour-0 site at the same (h, j, k): its non-bond terms and Q
  {
    const uint8_t p0 = MASK ? compb(G.po, Q) : 1;
    const float a0 = p0 != 0 ? 1.f : 0.f;
    const float x = comp(G.ox, Q), y = comp(G.oy, Q), z = comp(G.oz, Q);
    if (MASK && p0 > 1 && p0 - 2 < R.nsurf) {
      const long long sb = R.ns_off + G.base + Q;
      const float e = surface_energy(R, p0 - 2, x, y, z, __ldg(a.ns + sb), __ldg(a.ns + sb + R.plane),
                                     __ldg(a.ns + sb + 2 * R.plane));
      acc[0] += e;
      acc[1] += e;
    }
    if (FIELD) {
      const float e = field_energy(R, x, y, z);
      acc[0] += e;
      acc[1] += a0 * e;
    }
    if (a0 != 0.f) {
      acc[2] += x * x; acc[3] += x * y; acc[4] += x * z;
      acc[5] += y * y; acc[6] += y * z; acc[7] += z * z;
    }
  }
}

template <int POT, bool MASK, bool FIELD>
__global__ void __launch_bounds__(kBlock) k_measure(MeasureArgs a) {
  const int2 m = a.map[blockIdx.x];
  const RepDev &R = a.reps[m.x];
  const long long g = (long long)m.y + threadIdx.x;
  float acc[kMacc];
#pragma unroll
  for (int q = 0; q < kMacc; q++) acc[q] = 0.f;
  if (g < R.ngroups) {
    Group G;
    // "active" colour 1: its own rows plus the colour-0 neighbourhood; the
    // colour-0 row at the same position is G.o*.
    load_group<MASK>(R, a.dir, a.pt, 1, g, G);
    measure_site<POT, MASK, FIELD, 0>(R, a, G, acc);
    measure_site<POT, MASK, FIELD, 1>(R, a, G, acc);
    measure_site<POT, MASK, FIELD, 2>(R, a, G, acc);
    measure_site<POT, MASK, FIELD, 3>(R, a, G, acc);
  }
  __shared__ double red[kBlock / 32][kMacc];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kMacc; q++) {
    const double v = warp_sum((double)acc[q]);
    if (lane == 0) red[wid][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < kMacc) {
    double v = 0;
#pragma unroll
    for (int w = 0; w < kBlock / 32; w++) v += red[w][threadIdx.x];
    atomicAdd(a.macc + (size_t)m.x * kMacc + threadIdx.x, v);
  }
}

// ---------------------------------------------------------------------------
// Per-replica epilogue.
// ---------------------------------------------------------------------------

// Q-tensor from the accumulated sums (src/parameter_order.cpp:30-60):
// Q_ab = (3 sum n_a n_b - delta_ab * points) / (2 points), Q_zz = -Q_xx - Q_yy.
__device__ __forceinline__ void q_tensor(const double *m, double valid, double Q[9]) {
  const double d = 2.0 * valid;
  Q[0] = (3.0 * m[2] - valid) / d;
  Q[1] = 3.0 * m[3] / d;
  Q[2] = 3.0 * m[4] / d;
  Q[4] = (3.0 * m[5] - valid) / d;
  Q[5] = 3.0 * m[6] / d;
  Q[3] = Q[1];
  Q[6] = Q[2];
  Q[7] = Q[5];
  Q[8] = -Q[0] - Q[4];
}

// Largest eigenvalue of a symmetric 3x3 matrix in FP64: the root of the
// characteristic polynomial lambda^3 - tr lambda^2 + c1 lambda - det = 0
// bracketed from the trigonometric (Viete) estimate and polished by Newton
// steps.  Used per sweep, where a Jacobi solve's long FP64 dependency chain
// would dominate the sweep's latency.
__device__ double eig_max_sym3(const double Q[9]) {
  const double a = Q[0], b = Q[4], c = Q[8], d = Q[1], e = Q[5], f = Q[2];
  const double tr = a + b + c;
  const double m = tr / 3.0;
  const double a0 = a - m, b0 = b - m, c0 = c - m;
  // shifted matrix B = Q - m I: lambda_B^3 - p lambda_B - q = 0
  const double p = (a0 * a0 + b0 * b0 + c0 * c0 + 2.0 * (d * d + e * e + f * f)) / 2.0;
  const double q = a0 * (b0 * c0 - e * e) - d * (d * c0 - e * f) + f * (d * e - b0 * f);
  if (p <= 0.0) return m;
  const double r = sqrt(p / 3.0);
  double arg = q / (2.0 * r * r * r);
  arg = fmin(1.0, fmax(-1.0, arg));
  double x = 2.0 * r * cos(acos(arg) / 3.0);
#pragma unroll 1
  for (int it = 0; it < 4; it++) {
    const double fx = (x * x - p) * x - q;
    const double fp = 3.0 * x * x - p;
    if (fp <= 1e-300) break;
    const double nx = x - fx / fp;
    if (nx == x) break;
    x = nx;
  }
  return x + m;
}

template <bool MEASURE>
__global__ void k_epilogue(EpilogueArgs a) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.nrep) return;
  RepState &S = a.st[r];
  const RepDev &R = a.reps[r];
  const unsigned acc = S.acc;
  S.acc = 0;
  // src/evolve.cpp:169-178 with the reference's float/double rounding
  float av = S.ang_var;
  const double ratio = 1.0 * (double)acc / (double)R.valid;
  if (ratio < 0.5) {
    av = (float)((double)av * 0.99);
    if ((double)av < 0.01) av = (float)0.01;
  } else if (ratio > 0.5) {
    av = (float)((double)av / 0.99);
    if ((double)av > 1.0) av = (float)((double)av - 0.5);
  }
  S.ang_var = av;
  S.sweep += 1;
  double *st = a.stats + (size_t)r * kStats;
  st[7] += (double)acc;
  st[8] += 1.0;
  st[11] = (double)av;
  st[12] = (double)S.sweep;
  if (MEASURE) {
    double *mm = a.macc + (size_t)r * kMacc;
    const double E = mm[0] / (double)R.ntot;
    const double Ev = mm[1] / (double)R.valid;
    double Q[9];
    q_tensor(mm, (double)R.valid, Q);
    const double Sv = eig_max_sym3(Q);
    st[0] += 1.0;
    st[1] += Sv;
    st[2] += Sv * Sv;
    st[3] += E;
    st[4] += E * E;
    st[5] += Ev;
    st[6] += Ev * Ev;
    st[9] = E;
    st[10] = Sv;
    if (a.series_cap > 0) {
      const long long n = (long long)st[0] - 1;
      double *sr = a.series + ((size_t)r * a.series_cap + (size_t)(n % a.series_cap)) * 2;
      sr[0] = E;
      sr[1] = Sv;
    }
#pragma unroll
    for (int q = 0; q < kMacc; q++) mm[q] = 0.0;
  }
}

// Cyclic Jacobi (Golub & Van Loan, sec. 8.5) in FP64 for the on-demand
// measurement, which also reports the director (the eigenvector).
__device__ void jacobi_sym3(const double Qin[9], double &lam, double vec[3]) {
  double A[3][3], V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) A[i][j] = 0.5 * (Qin[3 * i + j] + Qin[3 * j + i]);
  for (int it = 0; it < 64; it++) {
    const double off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
    if (off <= 1e-300 || off <= 1e-17 * (fabs(A[0][0]) + fabs(A[1][1]) + fabs(A[2][2]) + off)) break;
    for (int pq = 0; pq < 3; pq++) {
      const int P = pq == 2 ? 1 : 0, Qi = pq == 0 ? 1 : 2;
      const double apq = A[P][Qi];
      if (apq == 0) continue;
      const double th = (A[Qi][Qi] - A[P][P]) / (2 * apq);
      const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1));
      const double c = 1 / sqrt(t * t + 1), s = t * c;
      for (int r = 0; r < 3; r++) {
        const double x = A[r][P], y = A[r][Qi];
        A[r][P] = c * x - s * y;
        A[r][Qi] = s * x + c * y;
      }
      for (int r = 0; r < 3; r++) {
        const double x = A[P][r], y = A[Qi][r];
        A[P][r] = c * x - s * y;
        A[Qi][r] = s * x + c * y;
      }
      for (int r = 0; r < 3; r++) {
        const double x = V[r][P], y = V[r][Qi];
        V[r][P] = c * x - s * y;
        V[r][Qi] = s * x + c * y;
      }
    }
  }
  int mi = 0;
  if (A[1][1] > A[mi][mi]) mi = 1;
  if (A[2][2] > A[mi][mi]) mi = 2;
  lam = A[mi][mi];
  vec[0] = V[0][mi];
  vec[1] = V[1][mi];
  vec[2] = V[2][mi];
}

__global__ void k_measure_out(EpilogueArgs a, double *out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.nrep) return;
  const RepDev &R = a.reps[r];
  double *mm = a.macc + (size_t)r * kMacc;
  double *o = out + (size_t)r * 16;
  o[0] = mm[0] / (double)R.ntot;
  o[1] = mm[1] / (double)R.valid;
  double Q[9];
  q_tensor(mm, (double)R.valid, Q);
  for (int q = 0; q < 9; q++) o[2 + q] = Q[q];
  double lam, v[3];
  jacobi_sym3(Q, lam, v);
  o[11] = lam;
  o[12] = v[0];
  o[13] = v[1];
  o[14] = v[2];
  o[15] = (double)R.valid;
  for (int q = 0; q < kMacc; q++) mm[q] = 0.0;
}

// ---------------------------------------------------------------------------
// Layout conversion and initial conditions (one replica, natural site order).
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long split_index(const RepDev &R, long long s, int &c) {
  const int i = (int)(s % R.nx);
  const long long t = s / R.nx;
  const int j = (int)(t % R.ny), k = (int)(t / R.ny);
  c = (i + j + k) & 1;
  return ((long long)j + (long long)R.ny * k) * R.hs + (i >> 1);
}

__global__ void k_aos_to_split(RepDev R, const float *__restrict__ aos, float *__restrict__ dir) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= R.ntot) return;
  int c;
  const long long p = split_index(R, s, c);
  float *d = dir + R.dir_off + (long long)(c * 3) * R.plane + p;
  d[0] = aos[3 * s];
  d[R.plane] = aos[3 * s + 1];
  d[2 * R.plane] = aos[3 * s + 2];
}

__global__ void k_split_to_aos(RepDev R, const float *__restrict__ dir, float *__restrict__ aos) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= R.ntot) return;
  int c;
  const long long p = split_index(R, s, c);
  const float *d = dir + R.dir_off + (long long)(c * 3) * R.plane + p;
  aos[3 * s] = d[0];
  aos[3 * s + 1] = d[R.plane];
  aos[3 * s + 2] = d[2 * R.plane];
}

__global__ void k_mask_to_split(RepDev R, const int *__restrict__ pt_aos, const float *__restrict__ ns_aos,
                                uint8_t *__restrict__ pt, float *__restrict__ ns) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= R.ntot) return;
  int c;
  const long long p = split_index(R, s, c);
  pt[R.pt_off + (long long)c * R.plane + p] = (uint8_t)pt_aos[s];
  if (ns != nullptr) {
    float *d = ns + R.ns_off + (long long)(c * 3) * R.plane + p;
    d[0] = ns_aos ? ns_aos[3 * s] : 0.f;
    d[R.plane] = ns_aos ? ns_aos[3 * s + 1] : 0.f;
    d[2 * R.plane] = ns_aos ? ns_aos[3 * s + 2] : 0.f;
  }
}

__global__ void k_split_to_mask(RepDev R, const uint8_t *__restrict__ pt, const float *__restrict__ ns,
                                int *__restrict__ pt_aos, float *__restrict__ ns_aos) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= R.ntot) return;
  int c;
  const long long p = split_index(R, s, c);
  pt_aos[s] = pt ? pt[R.pt_off + (long long)c * R.plane + p] : 1;
  const float *d = ns ? ns + R.ns_off + (long long)(c * 3) * R.plane + p : nullptr;
  ns_aos[3 * s] = d ? d[0] : 0.f;
  ns_aos[3 * s + 1] = d ? d[R.plane] : 0.f;
  ns_aos[3 * s + 2] = d ? d[2 * R.plane] : 0.f;
}

// mode 0: random on the sphere (z = 2u-1 uniform, azimuth 2 pi u') from
// Philox(site, 0, 0, TAG_IC); mode 1: the fixed director (hx, hy, hz).
// Inactive sites get (0, 0, 1) (src/ic.cpp:27-86).
__global__ void k_init(RepDev R, const uint8_t *__restrict__ pt, float *__restrict__ dir, int mode, uint32_t seed,
                       float fx, float fy, float fz) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= R.ntot) return;
  int c;
  const long long p = split_index(R, s, c);
  const bool active = pt == nullptr || pt[R.pt_off + (long long)c * R.plane + p] != 0;
  float x = 0.f, y = 0.f, z = 1.f;
  if (active) {
    if (mode == 0) {
      const uint4 r = philox4x32_10(make_uint4((uint32_t)s, 0u, 0u, TAG_IC), seed, R.stream);
      z = 2.f * u01(r.x) - 1.f;
      float sn, cs;
      sincospif(2.f * u01(r.y), &sn, &cs);
      const float rho = sqrtf(fmaxf(0.f, 1.f - z * z));
      x = rho * cs;
      y = rho * sn;
    } else {
      x = fx;
      y = fy;
      z = fz;
    }
  }
  float *d = dir + R.dir_off + (long long)(c * 3) * R.plane + p;
  d[0] = x;
  d[R.plane] = y;
  d[2 * R.plane] = z;
}

// ---------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------
template <int POT, bool MASK, bool FIELD, bool TRACE>
static void launch_pass_t(const PassArgs &a, int nblocks, cudaStream_t st) {
  k_sweep_pass<POT, MASK, FIELD, TRACE><<<nblocks, kBlock, 0, st>>>(a);
}

template <bool TRACE>
static void launch_pass_tr(const Variant &v, const PassArgs &a, int nblocks, cudaStream_t st) {
  if (v.pot == POT_LL) {
    if (v.mask) {
      if (v.field) launch_pass_t<POT_LL, true, true, TRACE>(a, nblocks, st);
      else launch_pass_t<POT_LL, true, false, TRACE>(a, nblocks, st);
    } else {
      if (v.field) launch_pass_t<POT_LL, false, true, TRACE>(a, nblocks, st);
      else launch_pass_t<POT_LL, false, false, TRACE>(a, nblocks, st);
    }
  } else {
    if (v.mask) {
      if (v.field) launch_pass_t<POT_GHRL, true, true, TRACE>(a, nblocks, st);
      else launch_pass_t<POT_GHRL, true, false, TRACE>(a, nblocks, st);
    } else {
      if (v.field) launch_pass_t<POT_GHRL, false, true, TRACE>(a, nblocks, st);
      else launch_pass_t<POT_GHRL, false, false, TRACE>(a, nblocks, st);
    }
  }
}

void launch_pass(const Variant &v, const PassArgs &a, int nblocks, bool trace, cudaStream_t st) {
  if (trace) launch_pass_tr<true>(v, a, nblocks, st);
  else launch_pass_tr<false>(v, a, nblocks, st);
}

void launch_measure(const Variant &v, const MeasureArgs &a, int nblocks, cudaStream_t st) {
#define MCX_M(P, M, F) k_measure<P, M, F><<<nblocks, kBlock, 0, st>>>(a)
  if (v.pot == POT_LL) {
    if (v.mask) { if (v.field) MCX_M(POT_LL, true, true); else MCX_M(POT_LL, true, false); }
    else { if (v.field) MCX_M(POT_LL, false, true); else MCX_M(POT_LL, false, false); }
  } else {
    if (v.mask) { if (v.field) MCX_M(POT_GHRL, true, true); else MCX_M(POT_GHRL, true, false); }
    else { if (v.field) MCX_M(POT_GHRL, false, true); else MCX_M(POT_GHRL, false, false); }
  }
#undef MCX_M
}

void launch_epilogue(const EpilogueArgs &a, bool measure, cudaStream_t st) {
  const int nb = (a.nrep + 127) / 128;
  if (measure) k_epilogue<true><<<nb, 128, 0, st>>>(a);
  else k_epilogue<false><<<nb, 128, 0, st>>>(a);
}

void launch_measure_out(const EpilogueArgs &a, double *out, cudaStream_t st) {
  k_measure_out<<<(a.nrep + 127) / 128, 128, 0, st>>>(a, out);
}

static int blocks_for(long long n) { return (int)((n + 255) / 256); }

void launch_aos_to_split(const RepDev &R, const float *aos, float *dir, cudaStream_t st) {
  k_aos_to_split<<<blocks_for(R.ntot), 256, 0, st>>>(R, aos, dir);
}
void launch_split_to_aos(const RepDev &R, const float *dir, float *aos, cudaStream_t st) {
  k_split_to_aos<<<blocks_for(R.ntot), 256, 0, st>>>(R, dir, aos);
}
void launch_mask_to_split(const RepDev &R, const int *pt_aos, const float *ns_aos, uint8_t *pt, float *ns,
                          cudaStream_t st) {
  k_mask_to_split<<<blocks_for(R.ntot), 256, 0, st>>>(R, pt_aos, ns_aos, pt, ns);
}
void launch_split_to_mask(const RepDev &R, const uint8_t *pt, const float *ns, int *pt_aos, float *ns_aos,
                          cudaStream_t st) {
  k_split_to_mask<<<blocks_for(R.ntot), 256, 0, st>>>(R, pt, ns, pt_aos, ns_aos);
}
void launch_init(const RepDev &R, const uint8_t *pt, float *dir, int mode, uint32_t seed, float fx, float fy, float fz,
                 cudaStream_t st) {
  k_init<<<blocks_for(R.ntot), 256, 0, st>>>(R, pt, dir, mode, seed, fx, fy, fz);
}

}  // namespace mcx
