// mcx_kernels.cu -- sm_103a kernels of the GB300 Metropolis engine.
//
//   k_pass       one red/black half-sweep of every replica in the batch
//                (EvolveN::Monte_Carlo_Step, src/evolve.cpp:64-179 of the
//                reference, with 2 colours instead of 8).  One thread per site
//                of the colour: coalesced loads of its director and of its 6
//                other-colour neighbours from the split SoA layout, a
//                Philox4x32-10 draw keyed by (seed, replica) and counted by
//                (site, sweep), the rotated proposal, the energy change, the
//                Metropolis test.  In measured sweeps the same pass also adds
//                the final state's energy and Q-tensor sums to the sweep's
//                ring slot (energy_calculator, src/evolve.cpp:27-62;
//                Matrice_constructor, src/parameter_order.cpp:30-60): every
//                bond has exactly one colour-1 end, and the colour-1 pass has
//                both ends final, so the bond energies come from the update's
//                own arithmetic.  The last CTA of a replica's colour-1 pass
//                applies the step-size rule (src/evolve.cpp:169-178) and
//                advances the sweep counters.
//   k_flush      per replica, for the measured sweeps since the last flush:
//                E, Q, S = largest eigenvalue of Q (FP64 Jacobi), the running
//                sums and the optional E/S series; off the sweep's path.
#include <cuda_runtime.h>

#include "mcx_device.cuh"
#include "mcx_kernels.cuh"

// Threads and CTAs per SM the direct pass kernel is compiled for.
constexpr int kPB = 128;
#ifndef MCX_PASS_MIN_BLOCKS
#define MCX_PASS_MIN_BLOCKS 5
#endif

namespace mcx {

// Bond energy of director a with neighbour b in slot d (x+, x-, y+, y-, z+, z-).
template <int POT, int D>
__device__ __forceinline__ float bond(const RepDev &R, float ax, float ay, float az, const float b[3]) {
  if (POT == POT_LL) {
    const float nij = ax * b[0] + ay * b[1] + az * b[2];
    return -1.5f * R.A * nij * nij;
  } else {
    return ghrl_bond<(D >> 1)>(R, ax, ay, az, b[0], b[1], b[2], (D & 1) ? -1.f : 1.f);
  }
}

// Weighted bond sum of director a over the six slots.  For LL the constant
// -1.5 A is applied by the caller so that old and new sums share it.
template <int POT>
__device__ __forceinline__ float bond_sum(const RepDev &R, float ax, float ay, float az, const float nb[6][3],
                                          const float w[6]) {
  if (POT == POT_LL) {
    float acc = 0.f;
#pragma unroll
    for (int d = 0; d < 6; d++) {
      const float nij = ax * nb[d][0] + ay * nb[d][1] + az * nb[d][2];
      acc = fmaf(nij * w[d], nij, acc);
    }
    return acc;
  } else {
    float acc = 0.f;
    acc = fmaf(w[0], bond<POT, 0>(R, ax, ay, az, nb[0]), acc);
    acc = fmaf(w[1], bond<POT, 1>(R, ax, ay, az, nb[1]), acc);
    acc = fmaf(w[2], bond<POT, 2>(R, ax, ay, az, nb[2]), acc);
    acc = fmaf(w[3], bond<POT, 3>(R, ax, ay, az, nb[3]), acc);
    acc = fmaf(w[4], bond<POT, 4>(R, ax, ay, az, nb[4]), acc);
    acc = fmaf(w[5], bond<POT, 5>(R, ax, ay, az, nb[5]), acc);
    return acc;
  }
}

template <int POT>
__device__ __forceinline__ float bond_scale(const RepDev &R) {
  return POT == POT_LL ? -1.5f * R.A : 1.f;
}

// Rotated proposal (src/evolve.cpp:136-152 / src/evolve.cu:143-163): rotate by
// pi*va about x (u1 < 0.333), y (u1 < 0.666) or z, then renormalise.  Written
// as one rotation of the component pair (u, v) = (y, z), (z, x) or (x, y):
// u' = u c + v s, v' = v c - u s, which is the reference's three formulas.
// sin and cos are taken of |angle| and the sign restored, so a move and its
// reverse are exact mirror images (a symmetric proposal).
__device__ __forceinline__ void propose(float x, float y, float z, float u0, float u1, float ang, float &px, float &py,
                                        float &pz) {
  const float va = (2.f * u0 - 1.f) * ang;
  const float th = 3.14159265358979f * va;
  const float at = fabsf(th);
  const float sn = copysignf(__sinf(at), th);
  const float cs = __cosf(at);
  const int axis = u1 < 0.333f ? 0 : (u1 < 0.666f ? 1 : 2);
  const float u = axis == 0 ? y : (axis == 1 ? z : x);
  const float v = axis == 0 ? z : (axis == 1 ? x : y);
  const float up = u * cs + v * sn;
  const float vp = v * cs - u * sn;
  px = axis == 0 ? x : (axis == 1 ? vp : up);
  py = axis == 0 ? up : (axis == 1 ? y : vp);
  pz = axis == 0 ? vp : (axis == 1 ? up : z);
  const float inv = rsqrtf(px * px + py * py + pz * pz);
  px *= inv;
  py *= inv;
  pz *= inv;
}

// One site update (and, in measured modes, its share of E and Q).  x, y, z
// hold the site's director and receive the final one; nb / w are the six
// neighbours and their update weights (bond present and neighbour active);
// e marks bonds present whatever the neighbour's type.
template <int POT, bool MASK, bool FIELD, int MODE>
__device__ __forceinline__ unsigned site_update(const RepDev &R, const PassArgs &a, int c, float &x, float &y,
                                                float &z, const float nb[6][3], const float w[6], const float e[6],
                                                int pself, float sx, float sy, float sz, const float u[3], float ang,
                                                float invT, uint32_t nat, float qs[kQ]) {
  constexpr bool MEAS = MODE == MODE_SWEEP_MEASURE || MODE == MODE_MEASURE_ONLY;
  constexpr bool UPD = MODE != MODE_MEASURE_ONLY;
  constexpr bool TRACE = MODE == MODE_TRACE;
  const int sid = pself - 2;
  const bool surf = MASK && pself > 1 && sid < R.nsurf;
  unsigned acc = 0;
  float eb = 0.f;  // final bond sum to active neighbours (unscaled for LL)
  if (pself != 0) {
    const float b_old = bond_sum<POT>(R, x, y, z, nb, w);
    eb = b_old;
    if (UPD) {
      float px, py, pz;
      propose(x, y, z, u[0], u[1], ang, px, py, pz);
      const float b_new = bond_sum<POT>(R, px, py, pz, nb, w);
      float dE = bond_scale<POT>(R) * (b_new - b_old);
      if (surf) dE += surface_energy(R, sid, px, py, pz, sx, sy, sz) - surface_energy(R, sid, x, y, z, sx, sy, sz);
      if (FIELD) dE += field_energy(R, px, py, pz) - field_energy(R, x, y, z);
      // src/evolve.cpp:160: accept when u < exp(-(E_new - E_old)/T)
      const bool accept = u[2] < __expf(-dE * invT);
      if (TRACE) {
        a.tr_dE[nat] = dE;
        a.tr_acc[nat] = accept ? 1 : 0;
        a.tr_prop[3 * (size_t)nat] = px;
        a.tr_prop[3 * (size_t)nat + 1] = py;
        a.tr_prop[3 * (size_t)nat + 2] = pz;
      }
      if (accept) {
        x = px;
        y = py;
        z = pz;
        eb = b_new;
        acc = 1;
      }
    }
  } else if (TRACE) {
    a.tr_dE[nat] = 0.f;
    a.tr_acc[nat] = 255;
  }
  if (MEAS) {
    const float act = pself != 0 ? 1.f : 0.f;
    if (pself != 0) {
      qs[2] += x * x;
      qs[3] += x * y;
      qs[4] += x * z;
      qs[5] += y * y;
      qs[6] += y * z;
    }
    if (surf) {
      const float es = surface_energy(R, sid, x, y, z, sx, sy, sz);
      qs[0] += es;
      qs[1] += es;
    }
    if (FIELD) {
      const float ef = field_energy(R, x, y, z);
      qs[0] += ef;
      qs[1] += act * ef;
    }
    if (c == 1) {
      // each bond counts in the local energy of each active end; the
      // all-site energy also counts inactive sites' bonds to active ones
      if (pself != 0) {
        const float ebs = bond_scale<POT>(R) * eb;
        qs[0] += 2.f * ebs;
        qs[1] += 2.f * ebs;
        if (MASK) {
          float wi[6];
#pragma unroll
          for (int d = 0; d < 6; d++) wi[d] = e[d] - w[d];
          qs[0] += bond_scale<POT>(R) * bond_sum<POT>(R, x, y, z, nb, wi);
        }
      } else {
        qs[0] += bond_scale<POT>(R) * bond_sum<POT>(R, x, y, z, nb, w);
      }
    }
  }
  return acc;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Block-wide, NT threads: adds this CTA's acceptance and measurement sums for
// replica r, counts `units` finished work units (map entries or tiles) out of
// the replica's `total`, and lets the CTA that finishes the replica's last
// unit of a colour-1 sweep pass apply the step-size rule and advance the sweep
// counters.  Sums stay FP32 inside the CTA; one FP64 atomic per quantity.
template <int NT, int MODE>
__device__ __forceinline__ void flush_replica(const PassArgs &a, int r, int units, unsigned total, unsigned acc,
                                              float qs[kQ], bool mask) {
  constexpr bool MEAS = MODE == MODE_SWEEP_MEASURE || MODE == MODE_MEASURE_ONLY;
  constexpr bool COUNT = MODE == MODE_SWEEP || MODE == MODE_SWEEP_MEASURE;
  __shared__ unsigned s_acc[NT / 32];
  __shared__ float s_q[NT / 32][kQ];
  __shared__ unsigned s_last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const RepDev &R = a.reps[r];
  RepState *S = a.st + r;
  if (COUNT) {
    const unsigned wa = __reduce_add_sync(0xffffffffu, acc);
    if (lane == 0) s_acc[wid] = wa;
  }
  if (MEAS) {
#pragma unroll
    for (int q = 0; q < kQ; q++) {
      float v = qs[q];
#pragma unroll
      for (int o2 = 16; o2 > 0; o2 >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o2);
      if (lane == 0) s_q[wid][q] = v;
    }
  }
  __syncthreads();
  const int lane_slot = blockIdx.x % kLanes;
  if (COUNT && threadIdx.x == 0) {
    unsigned tot = 0;
#pragma unroll
    for (int w2 = 0; w2 < NT / 32; w2++) tot += s_acc[w2];
    if (tot) atomicAdd(&S->acc[lane_slot], tot);
    __threadfence();
  }
  if (MEAS && threadIdx.x < kQ) {
    const int q = (!mask && threadIdx.x == 1) ? 0 : threadIdx.x;
    float v = 0.f;
#pragma unroll
    for (int w2 = 0; w2 < NT / 32; w2++) v += s_q[w2][q];
    const unsigned long long slot = MODE == MODE_MEASURE_ONLY ? (unsigned long long)a.ring_cap
                                                              : S->meas % (unsigned long long)a.ring_cap;
    double *ring = a.ring + (((size_t)r * (a.ring_cap + 1) + slot) * kLanes + lane_slot) * kQ;
    atomicAdd(ring + threadIdx.x, (double)v);
    __threadfence();
  }
  if (COUNT && a.colour == 1) {
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&S->done, (unsigned)units) + (unsigned)units == total;
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
      __threadfence();
      unsigned tot = 0;
#pragma unroll
      for (int l = 0; l < kLanes; l++) tot += atomicExch(&S->acc[l], 0u);
      // src/evolve.cpp:169-178 with the reference's float/double rounding
      float av = S->ang_var;
      const double ratio = 1.0 * (double)tot / (double)R.valid;
      if (ratio < 0.5) {
        av = (float)((double)av * 0.99);
        if ((double)av < 0.01) av = (float)0.01;
      } else if (ratio > 0.5) {
        av = (float)((double)av / 0.99);
        if ((double)av > 1.0) av = (float)((double)av - 0.5);
      }
      S->ang_var = av;
      S->sweep += 1;
      if (MODE == MODE_SWEEP_MEASURE) S->meas += 1;
      S->done = 0;
      double *st = a.stats + (size_t)r * kStats;
      st[7] += (double)tot;
      st[8] += 1.0;
      st[11] = (double)av;
      st[12] = (double)S->sweep;
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Direct pass: persistent CTAs walk the map (entries of kPB same-colour site
// pairs); each thread keeps a two-stage cp.async pipeline of its own pairs'
// neighbourhoods in shared memory, so the loads of its next pair fly while it
// updates the current one.  Slots are private to a thread: no block barrier
// between pairs.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async(void *dst, const void *src, int bytes, bool valid) {
  if (bytes == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(valid ? 8 : 0)
                 : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(valid ? 4 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Shared-memory slots of one stage, struct of arrays over the CTA's threads.
template <bool MASK>
struct PairStage {
  float2 v[18][kPB];  // own x y z, other colour same row x y z, rows y+ y- z+ z- (x y z each)
  float ex[3][kPB];   // the extra other-colour site (x y z)
  uint32_t pw[MASK ? 7 : 1][kPB];  // point-type words: own, other row, 4 rows, extra
};

// Where a thread's pair lives and who its neighbours are.
struct PairGeom {
  int row, h0, j, k, s, off, exh, offp;
  bool valid, hasB;
  float exe, er[4];
  int rr[4];
};

__device__ __forceinline__ void pair_geom(const RepDev &R, int c, int t, PairGeom &g) {
  g.valid = t < R.npair;
  const int tt = g.valid ? t : 0;
  g.row = (int)fastdiv((uint32_t)tt, R.hp_m, R.hp_p);
  g.h0 = 2 * (tt - g.row * R.hp);
  g.k = (int)fastdiv((uint32_t)g.row, R.ny_m, R.ny_p);
  g.j = g.row - g.k * R.ny;
  g.s = (c + g.j + g.k) & 1;
  g.hasB = g.h0 + 1 < R.hx;
  g.off = g.row * R.hs + g.h0;
  g.offp = g.row * R.hps + g.h0;
  g.exe = 1.f;
  if (g.s == 0) {
    g.exh = g.h0 - 1;
    if (g.exh < 0) { if (R.xb == BOUND_PERIODIC) g.exh = R.hx - 1; else { g.exe = 0.f; g.exh = g.h0; } }
  } else {
    g.exh = g.hasB ? g.h0 + 2 : g.h0 + 1;
    if (g.exh == R.hx) { if (R.xb == BOUND_PERIODIC) g.exh = 0; else { g.exe = 0.f; g.exh = g.h0; } }
  }
  const int ny = R.ny, nz = R.nz;
  g.rr[0] = g.row + 1; g.rr[1] = g.row - 1; g.rr[2] = g.row + ny; g.rr[3] = g.row - ny;
  g.er[0] = g.er[1] = g.er[2] = g.er[3] = 1.f;
  if (g.j + 1 == ny) { if (R.yb == BOUND_PERIODIC) g.rr[0] -= ny; else { g.er[0] = 0.f; g.rr[0] = g.row; } }
  if (g.j == 0) { if (R.yb == BOUND_PERIODIC) g.rr[1] += ny; else { g.er[1] = 0.f; g.rr[1] = g.row; } }
  if (g.k + 1 == nz) { if (R.zb == BOUND_PERIODIC) g.rr[2] -= ny * nz; else { g.er[2] = 0.f; g.rr[2] = g.row; } }
  if (g.k == 0) { if (R.zb == BOUND_PERIODIC) g.rr[3] += ny * nz; else { g.er[3] = 0.f; g.rr[3] = g.row; } }
}

template <bool MASK>
__device__ __forceinline__ void prefetch_pair(const PassArgs &a, int c, int2 m, PairStage<MASK> &st) {
  const RepDev &R = a.reps[m.x];
  PairGeom g;
  pair_geom(R, c, m.y + (int)threadIdx.x, g);
  const int P = R.plane, tid = threadIdx.x;
  const float *Ac = a.dir + R.dir_off + (long long)(c * 3) * P;
  const float *Oc = a.dir + R.dir_off + (long long)((c ^ 1) * 3) * P;
  const bool v = g.valid;
#pragma unroll
  for (int q = 0; q < 3; q++) {
    cp_async(&st.v[q][tid], Ac + (long long)q * P + g.off, 8, v);
    cp_async(&st.v[3 + q][tid], Oc + (long long)q * P + g.off, 8, v);
    cp_async(&st.ex[q][tid], Oc + (long long)q * P + (long long)g.row * R.hs + g.exh, 4, v && g.exe != 0.f);
#pragma unroll
    for (int d = 0; d < 4; d++)
      cp_async(&st.v[6 + 3 * d + q][tid], Oc + (long long)q * P + (long long)g.rr[d] * R.hs + g.h0, 8,
               v && g.er[d] != 0.f);
  }
  if (MASK) {
    // 4-byte words holding the needed point-type bytes (rows are 16-byte aligned)
    const uint8_t *pa = a.pt + R.pt_off + (long long)c * R.pplane;
    const uint8_t *po = a.pt + R.pt_off + (long long)(c ^ 1) * R.pplane;
    cp_async(&st.pw[0][tid], pa + (g.offp & ~3), 4, v);
    cp_async(&st.pw[1][tid], po + (g.offp & ~3), 4, v);
#pragma unroll
    for (int d = 0; d < 4; d++) cp_async(&st.pw[2 + d][tid], po + ((g.rr[d] * R.hps + g.h0) & ~3), 4, v && g.er[d] != 0.f);
    cp_async(&st.pw[6][tid], po + ((g.row * R.hps + g.exh) & ~3), 4, v && g.exe != 0.f);
  }
}

__device__ __forceinline__ uchar2 word_pair(uint32_t w, int byte) {
  const uint32_t x = w >> (8 * byte);
  return make_uchar2((uint8_t)(x & 0xFF), (uint8_t)((x >> 8) & 0xFF));
}

template <int POT, bool MASK, bool FIELD, int MODE>
__device__ __forceinline__ void compute_pair(const PassArgs &a, int c, int2 m, const PairStage<MASK> &st, unsigned &acc,
                                             float qs[kQ]) {
  constexpr bool UPD = MODE != MODE_MEASURE_ONLY;
  const RepDev &R = a.reps[m.x];
  RepState *S = a.st + m.x;
  PairGeom g;
  pair_geom(R, c, m.y + (int)threadIdx.x, g);
  if (!g.valid) return;
  const int tid = threadIdx.x, P = R.plane;
  float2 ax = st.v[0][tid], ay = st.v[1][tid], az = st.v[2][tid];
  const float2 ox = st.v[3][tid], oy = st.v[4][tid], oz = st.v[5][tid];
  const float ex = st.ex[0][tid], ey = st.ex[1][tid], ez = st.ex[2][tid];
  uchar2 pself2 = make_uchar2(1, 1), po2 = make_uchar2(1, 1), pr[4];
  uint8_t pex = 1;
  if (MASK) {
    const int b = g.offp & 3;
    pself2 = word_pair(st.pw[0][tid], b);
    po2 = word_pair(st.pw[1][tid], b);
#pragma unroll
    for (int d = 0; d < 4; d++) pr[d] = word_pair(st.pw[2 + d][tid], (g.rr[d] * R.hps + g.h0) & 3);
    pex = (uint8_t)((st.pw[6][tid] >> (8 * ((g.row * R.hps + g.exh) & 3))) & 0xFF);
  }
  float uA[3] = {0.f, 0.f, 0.f}, uB[3] = {0.f, 0.f, 0.f};
  float ang = 0.f, invT = 0.f;
  if (UPD) {
    const unsigned long long sw = S->sweep;
    const uint32_t pid = (uint32_t)(m.y + tid);
    const uint4 rw = philox4x32_10(make_uint4(pid, (uint32_t)sw, (uint32_t)(sw >> 32), TAG_PLAIN | (uint32_t)c),
                                   R.seed, R.stream);
    pair_uniforms(rw, uA, uB);
    ang = S->ang_var;
    invT = 1.0f / S->T;
  }
  auto wt = [&](float ee, uint8_t pp) { return MASK ? (ee != 0.f && pp != 0 ? 1.f : 0.f) : ee; };
  float nb[6][3], w[6], e[6];
  {
    if (g.s == 0) {
      nb[0][0] = ox.x; nb[0][1] = oy.x; nb[0][2] = oz.x; e[0] = 1.f; w[0] = wt(1.f, po2.x);
      nb[1][0] = ex; nb[1][1] = ey; nb[1][2] = ez; e[1] = g.exe; w[1] = wt(g.exe, pex);
    } else {
      if (g.hasB) {
        nb[0][0] = ox.y; nb[0][1] = oy.y; nb[0][2] = oz.y; e[0] = 1.f; w[0] = wt(1.f, po2.y);
      } else {
        nb[0][0] = ex; nb[0][1] = ey; nb[0][2] = ez; e[0] = g.exe; w[0] = wt(g.exe, pex);
      }
      nb[1][0] = ox.x; nb[1][1] = oy.x; nb[1][2] = oz.x; e[1] = 1.f; w[1] = wt(1.f, po2.x);
    }
#pragma unroll
    for (int d = 0; d < 4; d++) {
      const float2 X = st.v[6 + 3 * d][tid], Y = st.v[7 + 3 * d][tid], Z = st.v[8 + 3 * d][tid];
      nb[2 + d][0] = X.x; nb[2 + d][1] = Y.x; nb[2 + d][2] = Z.x;
      e[2 + d] = g.er[d];
      w[2 + d] = wt(g.er[d], MASK ? pr[d].x : 1);
    }
    const int ps = MASK ? pself2.x : 1;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    if (MASK && ps > 1) {
      const float *nsb = a.ns + R.ns_off + (long long)(c * 3) * P + g.off;
      sx = __ldg(nsb);
      sy = __ldg(nsb + P);
      sz = __ldg(nsb + 2 * P);
    }
    const uint32_t nat = (uint32_t)(2 * g.h0 + g.s) + (uint32_t)R.nx * (uint32_t)g.row;
    acc += site_update<POT, MASK, FIELD, MODE>(R, a, c, ax.x, ay.x, az.x, nb, w, e, ps, sx, sy, sz, uA, ang, invT,
                                               nat, qs);
  }
  if (g.hasB) {
    if (g.s == 0) {
      nb[0][0] = ox.y; nb[0][1] = oy.y; nb[0][2] = oz.y; e[0] = 1.f; w[0] = wt(1.f, po2.y);
      nb[1][0] = ox.x; nb[1][1] = oy.x; nb[1][2] = oz.x; e[1] = 1.f; w[1] = wt(1.f, po2.x);
    } else {
      nb[0][0] = ex; nb[0][1] = ey; nb[0][2] = ez; e[0] = g.exe; w[0] = wt(g.exe, pex);
      nb[1][0] = ox.y; nb[1][1] = oy.y; nb[1][2] = oz.y; e[1] = 1.f; w[1] = wt(1.f, po2.y);
    }
#pragma unroll
    for (int d = 0; d < 4; d++) {
      const float2 X = st.v[6 + 3 * d][tid], Y = st.v[7 + 3 * d][tid], Z = st.v[8 + 3 * d][tid];
      nb[2 + d][0] = X.y; nb[2 + d][1] = Y.y; nb[2 + d][2] = Z.y;
      e[2 + d] = g.er[d];
      w[2 + d] = wt(g.er[d], MASK ? pr[d].y : 1);
    }
    const int ps = MASK ? pself2.y : 1;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    if (MASK && ps > 1) {
      const float *nsb = a.ns + R.ns_off + (long long)(c * 3) * P + g.off + 1;
      sx = __ldg(nsb);
      sy = __ldg(nsb + P);
      sz = __ldg(nsb + 2 * P);
    }
    const uint32_t nat = (uint32_t)(2 * g.h0 + 2 + g.s) + (uint32_t)R.nx * (uint32_t)g.row;
    acc += site_update<POT, MASK, FIELD, MODE>(R, a, c, ax.y, ay.y, az.y, nb, w, e, ps, sx, sy, sz, uB, ang, invT,
                                               nat, qs);
  }
  if (UPD) {
    float *gA = a.dir + R.dir_off + (long long)(c * 3) * P + g.off;
    *reinterpret_cast<float2 *>(gA) = ax;
    *reinterpret_cast<float2 *>(gA + P) = ay;
    *reinterpret_cast<float2 *>(gA + 2 * P) = az;
  }
}

template <int POT, bool MASK, bool FIELD, int MODE>
__global__ void __launch_bounds__(kPB, MCX_PASS_MIN_BLOCKS) k_pass(PassArgs a) {
  __shared__ PairStage<MASK> stages[2];
  const int c = a.colour;
  const int G = gridDim.x, n = a.nmap;
  int e = blockIdx.x;
  if (e < n) prefetch_pair<MASK>(a, c, a.map[e], stages[0]);
  cp_async_commit();
  int cur = -1, units = 0;
  unsigned acc = 0;
  float qs[kQ];
#pragma unroll
  for (int q = 0; q < kQ; q++) qs[q] = 0.f;
  for (int it = 0; e < n; it++, e += G) {
    const int2 m = a.map[e];
    if (e + G < n) prefetch_pair<MASK>(a, c, a.map[e + G], stages[(it + 1) & 1]);
    cp_async_commit();
    if (m.x != cur) {
      if (cur >= 0) {
        flush_replica<kPB, MODE>(a, cur, units, (unsigned)a.reps[cur].ncta, acc, qs, MASK);
        acc = 0;
#pragma unroll
        for (int q = 0; q < kQ; q++) qs[q] = 0.f;
      }
      cur = m.x;
      units = 0;
    }
    cp_async_wait1();
    compute_pair<POT, MASK, FIELD, MODE>(a, c, m, stages[it & 1], acc, qs);
    units++;
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  if (cur >= 0) flush_replica<kPB, MODE>(a, cur, units, (unsigned)a.reps[cur].ncta, acc, qs, MASK);
}

// ---------------------------------------------------------------------------
// Staged pass: tiles of rows brought into shared memory by TMA bulk copies.
//
// A tile is tj x tk rows (tj | ny, tk | nz) of one replica.  For colour c it
// needs the tile's own rows (A) and the other colour's rows with a one-row
// halo in j and k (O): every row is a contiguous hs-float run in the split
// layout, so each is one cp.async.bulk (rows of a plane merge into one copy).
// Stage layout: A [3][tj*tk][hs] floats, O [3][(tk+2)*(tj+2)][hs] floats,
// then the point types Ap [tj*tk][hps], Op [(tk+2)*(tj+2)][hps] bytes.  O slot
// of row (jl, kl) relative to the tile is (kl+1)*(tj+2) + jl+1; corner slots
// are never filled or read.  Absent rows (free boundaries) are not copied and
// are read with weight 0 (shared memory is zeroed once, so stale values are
// finite).  Each persistent CTA double-buffers: the next tile's copies fly
// while the current tile is updated; completion is tracked by one mbarrier
// per stage (arrive.expect_tx + complete_tx), and every wait is bounded.
// ---------------------------------------------------------------------------
#ifndef MCX_TPASS_MIN_BLOCKS
#define MCX_TPASS_MIN_BLOCKS 3
#endif
#ifndef MCX_TPASS_STAGES
#define MCX_TPASS_STAGES 3
#endif
constexpr int kStages = MCX_TPASS_STAGES;
constexpr long long kWaitLimit = 1LL << 26;  // try_wait polls before giving up


__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for a stage's copies; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  for (long long i = 0; i < kWaitLimit; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

struct StageView {
  float *A, *O;
  uint8_t *Ap, *Op;
  int SA, SO;
};

__device__ __forceinline__ StageView stage_view(char *base, const RepDev &R) {
  StageView v;
  v.SA = R.tj * R.tk;
  v.SO = (R.tk + 2) * (R.tj + 2);
  v.A = reinterpret_cast<float *>(base);
  v.O = v.A + 3 * v.SA * R.hs;
  v.Ap = reinterpret_cast<uint8_t *>(v.O + 3 * v.SO * R.hs);
  v.Op = v.Ap + v.SA * R.hps;
  return v;
}

// Copy i of a tile (i < (4 tk + 2) * (3 + MASK)): component q = i / nseg
// (q = 3: point types), segment g = i % nseg.  Segments 0 .. tk-1 are the
// tile's own rows of plane k0 + g; then the other colour's planes k0-1 (one
// run), k0 .. k0+tk-1 (three runs each: the tj tile rows, the row below, the
// row above) and k0+tk (one run).  Returns the byte count, 0 when the rows
// are absent (free boundary).
template <bool MASK>
__device__ __forceinline__ uint32_t tile_copy(const PassArgs &a, const RepDev &R, int c, int j0, int k0,
                                              const StageView &v, int i, void *&dst, const void *&src) {
  const int hs = R.hs, tj = R.tj, tk = R.tk, ny = R.ny, nz = R.nz, P = R.plane, hps = R.hps;
  const int nseg = 4 * tk + 2;
  const int q = i / nseg, g = i - q * nseg;
  const bool ptq = MASK && q == 3;
  if (g < tk) {
    const int row = j0 + ny * (k0 + g);
    if (ptq) {
      dst = v.Ap + (size_t)g * tj * hps;
      src = a.pt + R.pt_off + (long long)c * R.pplane + (long long)row * hps;
      return (uint32_t)(tj * hps);
    }
    dst = v.A + ((size_t)q * v.SA + g * tj) * hs;
    src = a.dir + R.dir_off + (long long)(c * 3 + q) * P + (long long)row * hs;
    return (uint32_t)(tj * hs * 4);
  }
  const int o = g - tk;
  int kl, jl, nrows;
  if (o == 0) {
    kl = -1; jl = 0; nrows = tj;
  } else if (o == 3 * tk + 1) {
    kl = tk; jl = 0; nrows = tj;
  } else {
    kl = (o - 1) / 3;
    const int run = (o - 1) - 3 * kl;
    jl = run == 0 ? 0 : (run == 1 ? -1 : tj);
    nrows = run == 0 ? tj : 1;
  }
  int k = k0 + kl;
  if (k < 0 || k >= nz) {
    if (R.zb != BOUND_PERIODIC) return 0;
    k = (k + nz) % nz;
  }
  int j = j0 + jl;
  if (j < 0 || j >= ny) {
    if (R.yb != BOUND_PERIODIC) return 0;
    j = (j + ny) % ny;
  }
  const int slot = (kl + 1) * (tj + 2) + jl + 1;
  const int row = j + ny * k;
  if (ptq) {
    dst = v.Op + (size_t)slot * hps;
    src = a.pt + R.pt_off + (long long)(c ^ 1) * R.pplane + (long long)row * hps;
    return (uint32_t)(nrows * hps);
  }
  dst = v.O + ((size_t)q * v.SO + slot) * hs;
  src = a.dir + R.dir_off + (long long)((c ^ 1) * 3 + q) * P + (long long)row * hs;
  return (uint32_t)(nrows * hs * 4);
}

// Issued by the 32 lanes of warp 0 together: the byte total is warp-reduced
// and registered on the stage's mbarrier by lane 0 before any copy starts.
template <bool MASK>
__device__ __forceinline__ void issue_tile(const PassArgs &a, int c, int t, char *stage, uint64_t *bar) {
  const int4 td = a.tiles[t];
  const RepDev &R = a.reps[td.x];
  const StageView v = stage_view(stage, R);
  const int lane = threadIdx.x & 31;
  const int ncopy = (4 * R.tk + 2) * (MASK ? 4 : 3);
  uint32_t bytes = 0;
  for (int i = lane; i < ncopy; i += 32) {
    void *d;
    const void *sp;
    bytes += tile_copy<MASK>(a, R, c, td.y, td.z, v, i, d, sp);
  }
  bytes = __reduce_add_sync(0xffffffffu, bytes);
  if (lane == 0) mbar_arrive_expect_tx(bar, bytes);
  __syncwarp();
  for (int i = lane; i < ncopy; i += 32) {
    void *d;
    const void *sp;
    const uint32_t b = tile_copy<MASK>(a, R, c, td.y, td.z, v, i, d, sp);
    if (b) bulk_copy_g2s(d, sp, b, bar);
  }
}

template <int POT, bool MASK, bool FIELD, int MODE>
__device__ __forceinline__ void compute_tile(const PassArgs &a, const RepDev &R, RepState *S, int c, int j0, int k0,
                                             const StageView &v, unsigned &acc, float qs[kQ]) {
  constexpr bool UPD = MODE != MODE_MEASURE_ONLY;
  const int hx = R.hx, ny = R.ny, nz = R.nz, hs = R.hs, hps = R.hps, tj = R.tj, P = R.plane;
  const int SA = v.SA, SO = v.SO, tjs = tj + 2;
  const int npairs = tj * R.tk * R.hp;
  float *gA = a.dir + R.dir_off + (long long)(c * 3) * P;
  const unsigned long long sw = S->sweep;
  const float ang = S->ang_var;
  const float invT = 1.0f / S->T;
  for (int p = threadIdx.x; p < npairs; p += kBlock) {
    const int rl = (int)fastdiv((uint32_t)p, R.hp_m, R.hp_p);
    const int h0 = 2 * (p - rl * R.hp);
    const int kl = (int)fastdiv((uint32_t)rl, R.tj_m, R.tj_p);
    const int jl = rl - kl * tj;
    const int j = j0 + jl, k = k0 + kl;
    const int row = j + ny * k;
    const int s = (c + j + k) & 1;
    const bool hasB = h0 + 1 < hx;
    const int aslot = kl * tj + jl;
    const int oslot = (kl + 1) * tjs + jl + 1;
    const float *As = v.A + (size_t)aslot * hs + h0;
    const float *Os = v.O + (size_t)oslot * hs;
    float2 ax = *reinterpret_cast<const float2 *>(As);
    float2 ay = *reinterpret_cast<const float2 *>(As + (size_t)SA * hs);
    float2 az = *reinterpret_cast<const float2 *>(As + (size_t)2 * SA * hs);
    const float2 ox = *reinterpret_cast<const float2 *>(Os + h0);
    const float2 oy = *reinterpret_cast<const float2 *>(Os + (size_t)SO * hs + h0);
    const float2 oz = *reinterpret_cast<const float2 *>(Os + (size_t)2 * SO * hs + h0);
    int exh;
    float exe = 1.f;
    if (s == 0) {
      exh = h0 - 1;
      if (exh < 0) { if (R.xb == BOUND_PERIODIC) exh = hx - 1; else { exe = 0.f; exh = h0; } }
    } else {
      exh = hasB ? h0 + 2 : h0 + 1;
      if (exh == hx) { if (R.xb == BOUND_PERIODIC) exh = 0; else { exe = 0.f; exh = h0; } }
    }
    const float ex = Os[exh], ey = Os[(size_t)SO * hs + exh], ez = Os[(size_t)2 * SO * hs + exh];
    float er[4] = {1.f, 1.f, 1.f, 1.f};
    if (j + 1 == ny && R.yb != BOUND_PERIODIC) er[0] = 0.f;
    if (j == 0 && R.yb != BOUND_PERIODIC) er[1] = 0.f;
    if (k + 1 == nz && R.zb != BOUND_PERIODIC) er[2] = 0.f;
    if (k == 0 && R.zb != BOUND_PERIODIC) er[3] = 0.f;
    const int rslot[4] = {oslot + 1, oslot - 1, oslot + tjs, oslot - tjs};
    float2 nr[4][3];
    uchar2 pr[4];
#pragma unroll
    for (int d = 0; d < 4; d++) {
      const float *Ro = v.O + (size_t)rslot[d] * hs + h0;
      nr[d][0] = *reinterpret_cast<const float2 *>(Ro);
      nr[d][1] = *reinterpret_cast<const float2 *>(Ro + (size_t)SO * hs);
      nr[d][2] = *reinterpret_cast<const float2 *>(Ro + (size_t)2 * SO * hs);
      if (MASK) pr[d] = *reinterpret_cast<const uchar2 *>(v.Op + (size_t)rslot[d] * hps + h0);
    }
    uchar2 pself2 = make_uchar2(1, 1), po2 = make_uchar2(1, 1);
    uint8_t pex = 1;
    if (MASK) {
      pself2 = *reinterpret_cast<const uchar2 *>(v.Ap + (size_t)aslot * hps + h0);
      po2 = *reinterpret_cast<const uchar2 *>(v.Op + (size_t)oslot * hps + h0);
      pex = v.Op[(size_t)oslot * hps + exh];
    }
    float uA[3] = {0.f, 0.f, 0.f}, uB[3] = {0.f, 0.f, 0.f};
    if (UPD) {
      const uint32_t pid = (uint32_t)row * (uint32_t)R.hp + (uint32_t)(h0 >> 1);
      const uint4 rw = philox4x32_10(make_uint4(pid, (uint32_t)sw, (uint32_t)(sw >> 32), TAG_PLAIN | (uint32_t)c),
                                     R.seed, R.stream);
      pair_uniforms(rw, uA, uB);
    }
    auto wt = [&](float ee, uint8_t pp) { return MASK ? (ee != 0.f && pp != 0 ? 1.f : 0.f) : ee; };
    float nb[6][3], w[6], e[6];
    {
      if (s == 0) {
        nb[0][0] = ox.x; nb[0][1] = oy.x; nb[0][2] = oz.x; e[0] = 1.f; w[0] = wt(1.f, po2.x);
        nb[1][0] = ex; nb[1][1] = ey; nb[1][2] = ez; e[1] = exe; w[1] = wt(exe, pex);
      } else {
        if (hasB) {
          nb[0][0] = ox.y; nb[0][1] = oy.y; nb[0][2] = oz.y; e[0] = 1.f; w[0] = wt(1.f, po2.y);
        } else {
          nb[0][0] = ex; nb[0][1] = ey; nb[0][2] = ez; e[0] = exe; w[0] = wt(exe, pex);
        }
        nb[1][0] = ox.x; nb[1][1] = oy.x; nb[1][2] = oz.x; e[1] = 1.f; w[1] = wt(1.f, po2.x);
      }
#pragma unroll
      for (int d = 0; d < 4; d++) {
        nb[2 + d][0] = nr[d][0].x; nb[2 + d][1] = nr[d][1].x; nb[2 + d][2] = nr[d][2].x;
        e[2 + d] = er[d];
        w[2 + d] = wt(er[d], MASK ? pr[d].x : 1);
      }
      const int ps = MASK ? pself2.x : 1;
      float sx = 0.f, sy = 0.f, sz = 0.f;
      if (MASK && ps > 1) {
        const float *nsb = a.ns + R.ns_off + (long long)(c * 3) * P + (long long)row * hs + h0;
        sx = __ldg(nsb);
        sy = __ldg(nsb + P);
        sz = __ldg(nsb + 2 * P);
      }
      const uint32_t nat = (uint32_t)(2 * h0 + s) + (uint32_t)R.nx * (uint32_t)row;
      acc += site_update<POT, MASK, FIELD, MODE>(R, a, c, ax.x, ay.x, az.x, nb, w, e, ps, sx, sy, sz, uA, ang, invT,
                                                 nat, qs);
    }
    if (hasB) {
      if (s == 0) {
        nb[0][0] = ox.y; nb[0][1] = oy.y; nb[0][2] = oz.y; e[0] = 1.f; w[0] = wt(1.f, po2.y);
        nb[1][0] = ox.x; nb[1][1] = oy.x; nb[1][2] = oz.x; e[1] = 1.f; w[1] = wt(1.f, po2.x);
      } else {
        nb[0][0] = ex; nb[0][1] = ey; nb[0][2] = ez; e[0] = exe; w[0] = wt(exe, pex);
        nb[1][0] = ox.y; nb[1][1] = oy.y; nb[1][2] = oz.y; e[1] = 1.f; w[1] = wt(1.f, po2.y);
      }
#pragma unroll
      for (int d = 0; d < 4; d++) {
        nb[2 + d][0] = nr[d][0].y; nb[2 + d][1] = nr[d][1].y; nb[2 + d][2] = nr[d][2].y;
        e[2 + d] = er[d];
        w[2 + d] = wt(er[d], MASK ? pr[d].y : 1);
      }
      const int ps = MASK ? pself2.y : 1;
      float sx = 0.f, sy = 0.f, sz = 0.f;
      if (MASK && ps > 1) {
        const float *nsb = a.ns + R.ns_off + (long long)(c * 3) * P + (long long)row * hs + h0 + 1;
        sx = __ldg(nsb);
        sy = __ldg(nsb + P);
        sz = __ldg(nsb + 2 * P);
      }
      const uint32_t nat = (uint32_t)(2 * h0 + 2 + s) + (uint32_t)R.nx * (uint32_t)row;
      acc += site_update<POT, MASK, FIELD, MODE>(R, a, c, ax.y, ay.y, az.y, nb, w, e, ps, sx, sy, sz, uB, ang, invT,
                                                 nat, qs);
    }
    if (UPD) {
      float *g = gA + (long long)row * hs + h0;
      *reinterpret_cast<float2 *>(g) = ax;
      *reinterpret_cast<float2 *>(g + P) = ay;
      *reinterpret_cast<float2 *>(g + 2 * P) = az;
    }
  }
}

template <int POT, bool MASK, bool FIELD, int MODE>
__global__ void __launch_bounds__(kBlock, MCX_TPASS_MIN_BLOCKS) k_tpass(PassArgs a) {
  extern __shared__ __align__(128) char smem[];
  __shared__ __align__(8) uint64_t bars[kStages];
  __shared__ int s_ok;
  const int c = a.colour;
  // zero the stages once: rows that are never copied (absent halos, corner
  // slots) must hold finite values
  for (int i = threadIdx.x; i < kStages * a.stage_bytes / 16; i += kBlock)
    reinterpret_cast<float4 *>(smem)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (threadIdx.x == 0) {
    for (int q = 0; q < kStages; q++) mbar_init(&bars[q], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int G = gridDim.x;
  const bool producer = threadIdx.x < 32;
  // prologue: the first kStages-1 tiles
  if (producer) {
    fence_proxy_async();
    for (int q = 0; q < kStages - 1; q++) {
      const int tq = blockIdx.x + q * G;
      if (tq < a.ntiles) issue_tile<MASK>(a, c, tq, smem + q * a.stage_bytes, &bars[q]);
    }
  }
  int cur = -1, ntl = 0;
  unsigned acc = 0;
  float qs[kQ];
#pragma unroll
  for (int q = 0; q < kQ; q++) qs[q] = 0.f;
  int it = 0;
  for (int t = blockIdx.x; t < a.ntiles; it++, t += G) {
    const int sidx = it % kStages;
    const int4 td = a.tiles[t];
    if (td.x != cur) {
      if (cur >= 0) {
        flush_replica<kBlock, MODE>(a, cur, ntl, (unsigned)a.reps[cur].ntile, acc, qs, MASK);
        acc = 0;
#pragma unroll
        for (int q = 0; q < kQ; q++) qs[q] = 0.f;
      }
      cur = td.x;
      ntl = 0;
    }
    if (producer) {
      // refill the stage the previous iteration released
      const int tn = t + (kStages - 1) * G;
      if (tn < a.ntiles) {
        const int sn = (it + kStages - 1) % kStages;
        fence_proxy_async();
        issue_tile<MASK>(a, c, tn, smem + sn * a.stage_bytes, &bars[sn]);
      }
      if (threadIdx.x == 0) s_ok = mbar_wait(&bars[sidx], (uint32_t)((it / kStages) & 1)) ? 1 : 0;
    }
    __syncthreads();
    if (!s_ok) {
      // a stage never completed: report it, let the copies still in flight
      // land (bounded), and leave without touching the sums
      if (threadIdx.x == 0) {
        atomicExch(a.err, 1u);
        for (int q = 0; q < kStages; q++) {
          const int last = it + q;  // iterations whose copies may be in flight
          const int tq = blockIdx.x + last * G;
          if (tq < a.ntiles) mbar_wait(&bars[last % kStages], (uint32_t)((last / kStages) & 1));
        }
      }
      return;
    }
    const RepDev &R = a.reps[td.x];
    compute_tile<POT, MASK, FIELD, MODE>(a, R, a.st + td.x, c, td.y, td.z,
                                         stage_view(smem + sidx * a.stage_bytes, R), acc, qs);
    ntl++;
    __syncthreads();
  }
  if (cur >= 0) flush_replica<kBlock, MODE>(a, cur, ntl, (unsigned)a.reps[cur].ntile, acc, qs, MASK);
}

// ---------------------------------------------------------------------------
// Statistics off the sweep path.
// ---------------------------------------------------------------------------

// Q-tensor from the sums (src/parameter_order.cpp:30-60):
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

// Cyclic Jacobi (Golub & Van Loan, sec. 8.5) in FP64: largest eigenvalue of a
// symmetric 3x3 matrix and its unit eigenvector.
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

// Sums a ring slot's lanes and clears it.
__device__ __forceinline__ void take_slot(double *slot, double m[kQ]) {
  for (int q = 0; q < kQ; q++) m[q] = 0.0;
  for (int l = 0; l < kLanes; l++)
    for (int q = 0; q < kQ; q++) {
      m[q] += slot[l * kQ + q];
      slot[l * kQ + q] = 0.0;
    }
}

constexpr int kFlushThreads = 128;

// One CTA per replica.  Thread t handles pending sweeps t, t+128, ... in
// order, then a fixed tree adds the per-thread sums: the result does not
// depend on scheduling.
__global__ void __launch_bounds__(kFlushThreads) k_flush(FlushArgs f) {
  const int r = blockIdx.x;
  const RepDev &R = f.reps[r];
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};  // S, S^2, E, E^2, Ev, Ev^2, n
  double lastE = 0, lastS = 0;
  for (int q = threadIdx.x; q < f.count; q += kFlushThreads) {
    const unsigned long long n = f.first + (unsigned long long)q;
    double *slot = f.ring + ((size_t)r * (f.ring_cap + 1) + (size_t)(n % f.ring_cap)) * kLanes * kQ;
    double mm[kQ];
    take_slot(slot, mm);
    const double E = mm[0] / (double)R.ntot;
    const double Ev = mm[1] / (double)R.valid;
    double Q[9], lam, v[3];
    q_tensor(mm, (double)R.valid, Q);
    jacobi_sym3(Q, lam, v);
    acc[0] += lam;
    acc[1] += lam * lam;
    acc[2] += E;
    acc[3] += E * E;
    acc[4] += Ev;
    acc[5] += Ev * Ev;
    acc[6] += 1.0;
    if (q == f.count - 1) {
      lastE = E;
      lastS = lam;
    }
    if (f.series_cap > 0) {
      double *sr = f.series + ((size_t)r * f.series_cap + (size_t)(n % f.series_cap)) * 2;
      sr[0] = E;
      sr[1] = lam;
    }
  }
  __shared__ double red[kFlushThreads][7];
  for (int q = 0; q < 7; q++) red[threadIdx.x][q] = acc[q];
  __syncthreads();
  for (int stride = kFlushThreads / 2; stride > 0; stride >>= 1) {
    if ((int)threadIdx.x < stride)
      for (int q = 0; q < 7; q++) red[threadIdx.x][q] += red[threadIdx.x + stride][q];
    __syncthreads();
  }
  if ((int)threadIdx.x == (f.count - 1) % kFlushThreads) {
    double *st = f.stats + (size_t)r * kStats;
    st[9] = lastE;
    st[10] = lastS;
  }
  if (threadIdx.x == 0) {
    double *st = f.stats + (size_t)r * kStats;
    st[0] += red[0][6];
    st[1] += red[0][0];
    st[2] += red[0][1];
    st[3] += red[0][2];
    st[4] += red[0][3];
    st[5] += red[0][4];
    st[6] += red[0][5];
  }
}

// The on-demand measurement slot (index ring_cap) -> E, E_valid, Q, S,
// director, valid (the mcx_measure layout).
__global__ void k_measure_out(const RepDev *reps, double *ring, int ring_cap, int nrep, double *out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrep) return;
  const RepDev &R = reps[r];
  double mm[kQ];
  take_slot(ring + ((size_t)r * (ring_cap + 1) + (size_t)ring_cap) * kLanes * kQ, mm);
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
}

// ---------------------------------------------------------------------------
// Layout conversion and initial conditions (one replica, natural site order).
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long split_index(const RepDev &R, long long s, int &c, long long &row, int &h) {
  const int i = (int)(s % R.nx);
  row = s / R.nx;
  const int j = (int)(row % R.ny), k = (int)(row / R.ny);
  c = (i + j + k) & 1;
  h = i >> 1;
  return row * R.hs + h;
}

__global__ void k_aos_to_split(RepDev R, const float *__restrict__ aos, float *__restrict__ dir) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= R.ntot) return;
  int c, h;
  long long row;
  const long long p = split_index(R, s, c, row, h);
  const long long pp = row * R.hps + h;
  float *d = dir + R.dir_off + (long long)(c * 3) * R.plane + p;
  d[0] = aos[3 * s];
  d[R.plane] = aos[3 * s + 1];
  d[2 * R.plane] = aos[3 * s + 2];
}

__global__ void k_split_to_aos(RepDev R, const float *__restrict__ dir, float *__restrict__ aos) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= R.ntot) return;
  int c, h;
  long long row;
  const long long p = split_index(R, s, c, row, h);
  const long long pp = row * R.hps + h;
  const float *d = dir + R.dir_off + (long long)(c * 3) * R.plane + p;
  aos[3 * s] = d[0];
  aos[3 * s + 1] = d[R.plane];
  aos[3 * s + 2] = d[2 * R.plane];
}

__global__ void k_mask_to_split(RepDev R, const int *__restrict__ pt_aos, const float *__restrict__ ns_aos,
                                uint8_t *__restrict__ pt, float *__restrict__ ns) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= R.ntot) return;
  int c, h;
  long long row;
  const long long p = split_index(R, s, c, row, h);
  const long long pp = row * R.hps + h;
  pt[R.pt_off + (long long)c * R.pplane + pp] = (uint8_t)pt_aos[s];
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
  int c, h;
  long long row;
  const long long p = split_index(R, s, c, row, h);
  const long long pp = row * R.hps + h;
  pt_aos[s] = pt ? pt[R.pt_off + (long long)c * R.pplane + pp] : 1;
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
  int c, h;
  long long row;
  const long long p = split_index(R, s, c, row, h);
  const long long pp = row * R.hps + h;
  const bool active = pt == nullptr || pt[R.pt_off + (long long)c * R.pplane + pp] != 0;
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
template <int POT, bool MASK, bool FIELD>
static void launch_pass_pmf(int mode, const PassArgs &a, int nblocks, cudaStream_t st) {
  switch (mode) {
    case MODE_SWEEP: k_pass<POT, MASK, FIELD, MODE_SWEEP><<<nblocks, kPB, 0, st>>>(a); break;
    case MODE_SWEEP_MEASURE: k_pass<POT, MASK, FIELD, MODE_SWEEP_MEASURE><<<nblocks, kPB, 0, st>>>(a); break;
    case MODE_MEASURE_ONLY: k_pass<POT, MASK, FIELD, MODE_MEASURE_ONLY><<<nblocks, kPB, 0, st>>>(a); break;
    default: k_pass<POT, MASK, FIELD, MODE_TRACE><<<nblocks, kPB, 0, st>>>(a); break;
  }
}

template <int POT>
static void launch_pass_p(const Variant &v, int mode, const PassArgs &a, int nblocks, cudaStream_t st) {
  if (v.mask) {
    if (v.field) launch_pass_pmf<POT, true, true>(mode, a, nblocks, st);
    else launch_pass_pmf<POT, true, false>(mode, a, nblocks, st);
  } else {
    if (v.field) launch_pass_pmf<POT, false, true>(mode, a, nblocks, st);
    else launch_pass_pmf<POT, false, false>(mode, a, nblocks, st);
  }
}

template <int POT, bool MASK, bool FIELD>
static const void *pass_fn(int mode) {
  switch (mode) {
    case MODE_SWEEP: return (const void *)k_pass<POT, MASK, FIELD, MODE_SWEEP>;
    case MODE_SWEEP_MEASURE: return (const void *)k_pass<POT, MASK, FIELD, MODE_SWEEP_MEASURE>;
    case MODE_MEASURE_ONLY: return (const void *)k_pass<POT, MASK, FIELD, MODE_MEASURE_ONLY>;
    default: return (const void *)k_pass<POT, MASK, FIELD, MODE_TRACE>;
  }
}

int pass_block_threads() { return kPB; }

int pass_blocks_per_sm(const Variant &v, int mode) {
  const void *fn;
  if (v.pot == POT_LL) {
    if (v.mask) fn = v.field ? pass_fn<POT_LL, true, true>(mode) : pass_fn<POT_LL, true, false>(mode);
    else fn = v.field ? pass_fn<POT_LL, false, true>(mode) : pass_fn<POT_LL, false, false>(mode);
  } else {
    if (v.mask) fn = v.field ? pass_fn<POT_GHRL, true, true>(mode) : pass_fn<POT_GHRL, true, false>(mode);
    else fn = v.field ? pass_fn<POT_GHRL, false, true>(mode) : pass_fn<POT_GHRL, false, false>(mode);
  }
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kPB, 0) != cudaSuccess) return 0;
  return n;
}

void launch_pass(const Variant &v, int mode, const PassArgs &a, int nblocks, cudaStream_t st) {
  if (v.pot == POT_LL) launch_pass_p<POT_LL>(v, mode, a, nblocks, st);
  else launch_pass_p<POT_GHRL>(v, mode, a, nblocks, st);
}

template <int POT, bool MASK, bool FIELD>
static void tpass_pmf(int mode, const PassArgs &a, int grid, int smem, cudaStream_t st) {
  switch (mode) {
    case MODE_SWEEP: k_tpass<POT, MASK, FIELD, MODE_SWEEP><<<grid, kBlock, smem, st>>>(a); break;
    case MODE_SWEEP_MEASURE: k_tpass<POT, MASK, FIELD, MODE_SWEEP_MEASURE><<<grid, kBlock, smem, st>>>(a); break;
    default: k_tpass<POT, MASK, FIELD, MODE_TRACE><<<grid, kBlock, smem, st>>>(a); break;
  }
}

template <int POT, bool MASK, bool FIELD>
static const void *tpass_fn(int mode) {
  switch (mode) {
    case MODE_SWEEP: return (const void *)k_tpass<POT, MASK, FIELD, MODE_SWEEP>;
    case MODE_SWEEP_MEASURE: return (const void *)k_tpass<POT, MASK, FIELD, MODE_SWEEP_MEASURE>;
    default: return (const void *)k_tpass<POT, MASK, FIELD, MODE_TRACE>;
  }
}

static const void *tpass_select(const Variant &v, int mode) {
  if (v.pot == POT_LL) {
    if (v.mask) return v.field ? tpass_fn<POT_LL, true, true>(mode) : tpass_fn<POT_LL, true, false>(mode);
    return v.field ? tpass_fn<POT_LL, false, true>(mode) : tpass_fn<POT_LL, false, false>(mode);
  }
  if (v.mask) return v.field ? tpass_fn<POT_GHRL, true, true>(mode) : tpass_fn<POT_GHRL, true, false>(mode);
  return v.field ? tpass_fn<POT_GHRL, false, true>(mode) : tpass_fn<POT_GHRL, false, false>(mode);
}

int tpass_smem_bytes(int stage_bytes) { return kStages * stage_bytes; }

int tpass_blocks_per_sm(const Variant &v, int mode, int stage_bytes) {
  const void *fn = tpass_select(v, mode);
  const int smem = tpass_smem_bytes(stage_bytes);
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kBlock, smem) != cudaSuccess) return 0;
  return n;
}

void launch_tpass(const Variant &v, int mode, const PassArgs &a, int grid, cudaStream_t st) {
  const int smem = tpass_smem_bytes(a.stage_bytes);
  if (v.pot == POT_LL) {
    if (v.mask) {
      if (v.field) tpass_pmf<POT_LL, true, true>(mode, a, grid, smem, st);
      else tpass_pmf<POT_LL, true, false>(mode, a, grid, smem, st);
    } else {
      if (v.field) tpass_pmf<POT_LL, false, true>(mode, a, grid, smem, st);
      else tpass_pmf<POT_LL, false, false>(mode, a, grid, smem, st);
    }
  } else {
    if (v.mask) {
      if (v.field) tpass_pmf<POT_GHRL, true, true>(mode, a, grid, smem, st);
      else tpass_pmf<POT_GHRL, true, false>(mode, a, grid, smem, st);
    } else {
      if (v.field) tpass_pmf<POT_GHRL, false, true>(mode, a, grid, smem, st);
      else tpass_pmf<POT_GHRL, false, false>(mode, a, grid, smem, st);
    }
  }
}

void launch_flush(const FlushArgs &f, int nrep, cudaStream_t st) {
  k_flush<<<nrep, kFlushThreads, 0, st>>>(f);
}

void launch_measure_out(const RepDev *reps, double *ring, int ring_cap, int nrep, double *out, cudaStream_t st) {
  k_measure_out<<<(nrep + 127) / 128, 128, 0, st>>>(reps, ring, ring_cap, nrep, out);
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
