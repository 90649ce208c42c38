// mcx_pass.cuh -- the direct red/black pass, shared by the translation units
// that instantiate it (plain proposal: mcx_kernels.cu; learned proposal:
// mcx_learned.cu).
//
//   k_pass  one red/black half-sweep of every replica in the batch
//           (EvolveN::Monte_Carlo_Step, src/evolve.cpp:64-179 of the
//           reference, with 2 colours instead of 8).  Persistent CTAs walk the
//           map of work units (kPB same-colour site pairs each); each thread
//           keeps a two-stage cp.async pipeline of its pairs' neighbourhoods
//           in shared memory; a Philox4x32-10 draw per pair (plain proposal)
//           or per site (learned proposal) drives the proposal and the
//           Metropolis(-Hastings) test.  In measured sweeps the same pass adds
//           the final state's energy and Q-tensor sums to the sweep's ring
//           slot (energy_calculator, src/evolve.cpp:27-62; Matrice_constructor,
//           src/parameter_order.cpp:30-60).  The CTA that finishes a
//           replica's last work unit of a colour-1 pass applies the step-size
//           rule (src/evolve.cpp:169-178) and advances the sweep counters.
#pragma once
#include <cuda_runtime.h>

#include "mcx_device.cuh"
#include "mcx_kernels.cuh"
#include "mcx_mlp.cuh"

// Threads and CTAs per SM the direct pass kernel is compiled for.
constexpr int kPB = 128;
#ifndef MCX_PASS_MIN_BLOCKS
#define MCX_PASS_MIN_BLOCKS 5
#endif

namespace mcx {

// Bond energy of director a with neighbour b in slot d (x+, x-, y+, y-, z+, z-).
//
// The energy change of a move fixes every rounding: a product that feeds a
// sum is either an fmaf or an explicit __fmul_rn, which the compiler cannot
// fuse with what follows, and sums keep their written order.  Every kernel
// that inlines the update (each pass form) therefore computes the same bits
// and takes the same Metropolis decisions; left to the compiler, two forms'
// multiply-add fusions could differ and a decision within an ulp of its
// threshold could go either way.  Products by 0/1 weights or by +-1 are
// exact and stay plain, so the compiler can still fold them.
template <int POT, int D>
__device__ __forceinline__ float bond(const RepDev &R, float ax, float ay, float az, const float b[3]) {
  const float nij = dot3_rn(ax, ay, az, b[0], b[1], b[2]);
  if (POT == POT_LL) {
    return __fmul_rn(__fmul_rn(-1.5f, R.A), __fmul_rn(nij, nij));
  } else if (POT == POT_PEAR) {
    // src/potential.cpp:10-15: -A nij^2 - B1 nij - (C/4)(1 + 2 nij + nij^2)((nj - ni) . rij),
    // rij = +-(unit vector of the slot's axis)
    constexpr int X = D >> 1;
    const float ai = X == 0 ? ax : (X == 1 ? ay : az);
    const float aj = X == 0 ? b[0] : (X == 1 ? b[1] : b[2]);
    const float d = (D & 1) ? __fsub_rn(ai, aj) : __fsub_rn(aj, ai);
    const float splay = __fmul_rn(fmaf(nij, __fadd_rn(nij, 2.f), 1.f), d);
    return fmaf(-R.A, __fmul_rn(nij, nij), fmaf(-R.B1, nij, __fmul_rn(-0.25f * R.C, splay)));
  } else {
    return ghrl_bond_var<(D >> 1)>(R, ax, ay, az, b[0], b[1], b[2], (D & 1) ? -1.f : 1.f);
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
      const float nij = dot3_rn(ax, ay, az, nb[d][0], nb[d][1], nb[d][2]);
      acc = fmaf(nij * w[d], nij, acc);  // w is 0 or 1: nij * w is exact
    }
    return acc;
  } else {
    float acc = w[0] * bond<POT, 0>(R, ax, ay, az, nb[0]);  // w is 0 or 1: exact
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

// The part of a weighted bond sum that bond() leaves out (the GHRL bond's
// constant per bond); measurements add it, energy differences do not need it.
template <int POT>
__device__ __forceinline__ float bond_const(const RepDev &R, const float w[6]) {
  if (POT != POT_GHRL) return 0.f;
  return R.gconst * (((w[0] + w[1]) + (w[2] + w[3])) + (w[4] + w[5]));
}

// Rotated proposal (src/evolve.cpp:136-152 / src/evolve.cu:143-163): rotate by
// pi*va about x (u1 < 0.333), y (u1 < 0.666) or z, then renormalise.  Written
// as one rotation of the component pair (u, v) = (y, z), (z, x) or (x, y):
// u' = u c + v s, v' = v c - u s, which is the reference's three formulas.
// sin and cos are taken of |angle| and the sign restored, so a move and its
// reverse are exact mirror images (a symmetric proposal).  The rotation is
// left to the compiler's multiply-add fusion (written with explicit fmaf it
// costs 8% more instructions per pass); unlike the energy change, where a
// difference only shows at a near tie, a form whose fusion differed here
// would move every accepted site by an ulp, which the bit-for-bit tests
// across forms see at once.
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
      // every rounding of dE is explicit (see bond()): all pass forms take
      // the same decisions
      float dE = __fmul_rn(bond_scale<POT>(R), __fsub_rn(b_new, b_old));
      if (surf)
        dE = __fadd_rn(dE, __fsub_rn(surface_energy(R, sid, px, py, pz, sx, sy, sz),
                                     surface_energy(R, sid, x, y, z, sx, sy, sz)));
      if (FIELD) dE = __fadd_rn(dE, __fsub_rn(field_energy(R, px, py, pz), field_energy(R, x, y, z)));
      // src/evolve.cpp:160: accept when u < exp(-(E_new - E_old)/T)
      const bool accept = u[2] < __expf(__fmul_rn(-dE, invT));
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
        const float ebs = bond_scale<POT>(R) * eb + bond_const<POT>(R, w);
        qs[0] += 2.f * ebs;
        qs[1] += 2.f * ebs;
        if (MASK) {
          float wi[6];
#pragma unroll
          for (int d = 0; d < 6; d++) wi[d] = e[d] - w[d];
          qs[0] += bond_scale<POT>(R) * bond_sum<POT>(R, x, y, z, nb, wi) + bond_const<POT>(R, wi);
        }
      } else {
        qs[0] += bond_scale<POT>(R) * bond_sum<POT>(R, x, y, z, nb, w) + bond_const<POT>(R, w);
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
// Acceptances and finished units share one 64-bit counter, so a colour-0 CTA
// leaves with a fire-and-forget atomic and a colour-1 CTA learns whether it
// is the last (and the sweep's acceptance total) from a single atomic, with
// no fences: the measurement ring is read by later kernels only.
// colour: the pass's colour when the kernel runs several passes (a.colour
// otherwise).  Replica state and running sums are read past L1 (__ldcg): a
// kernel that runs several passes reads what other CTAs wrote in this launch.
// The ring slot of the sweep a measured pass adds to.  Only the CTA that
// ends a replica's colour-1 pass advances S->meas, after every CTA of that
// pass has added to the slot, so a pass may read it once the previous pass
// is done (after griddepcontrol.wait).
__device__ __forceinline__ int ring_slot(const PassArgs &a, const RepState *S) {
  return (int)(__ldcg(&S->meas) % (unsigned long long)a.ring_cap);
}

// slot_pre: the ring slot if the caller read it early (ring_slot; -1: read
// it here, at the end of the CTA, where its latency is exposed).
template <int NT, int MODE>
__device__ __forceinline__ void flush_replica(const PassArgs &a, int r, int units, unsigned total, unsigned acc,
                                              float qs[kQ], bool mask, int colour = -1, int slot_pre = -1) {
  constexpr bool MEAS = MODE == MODE_SWEEP_MEASURE || MODE == MODE_MEASURE_ONLY;
  constexpr bool COUNT = MODE == MODE_SWEEP || MODE == MODE_SWEEP_MEASURE;
  __shared__ unsigned s_acc[NT / 32];
  __shared__ float s_q[NT / 32][kQ];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const RepDev &R = a.reps[r];
  RepState *S = a.st + r;
  // what the step-size rule needs, loaded before the reductions so that the
  // load latency overlaps them (only the last CTA of the sweep, which
  // changes these, uses them, and it reads them before its own update)
  float av0 = 0.f;
  unsigned long long sweep0 = 0, meas0 = 0;
  unsigned frozen0 = 0;
  if (COUNT && threadIdx.x == 0) {
    av0 = __ldcg(&S->ang_var);
    sweep0 = __ldcg(&S->sweep);
    meas0 = __ldcg(&S->meas);
    frozen0 = __ldcg(&S->frozen);
  }
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
  if (MEAS && threadIdx.x < kQ) {
    const int lane_slot = blockIdx.x % kLanes;
    const int q = (!mask && threadIdx.x == 1) ? 0 : threadIdx.x;
    float v = 0.f;
#pragma unroll
    for (int w2 = 0; w2 < NT / 32; w2++) v += s_q[w2][q];
    const unsigned long long slot = MODE == MODE_MEASURE_ONLY ? (unsigned long long)a.ring_cap
                                    : slot_pre >= 0           ? (unsigned long long)slot_pre
                                                              : __ldcg(&S->meas) % (unsigned long long)a.ring_cap;
    double *ring = a.ring + (((size_t)r * (a.ring_cap + 1) + slot) * kLanes + lane_slot) * kQ;
    atomicAdd(ring + threadIdx.x, (double)v);
  }
  __syncwarp();  // warp 0's reads of the ring slot come before its thread 0 can end the sweep
  if (COUNT && threadIdx.x == 0) {
    unsigned tot = 0;
#pragma unroll
    for (int w2 = 0; w2 < NT / 32; w2++) tot += s_acc[w2];
    if ((colour < 0 ? a.colour : colour) != 1) {
      if (tot) atomicAdd(&S->cnt, (unsigned long long)tot);
    } else {
      const unsigned long long add = ((unsigned long long)(unsigned)units << 32) | tot;
      const unsigned long long old = atomicAdd(&S->cnt, add);
      if ((unsigned)(old >> 32) + (unsigned)units == total) {  // the replica's last unit of the sweep
        const unsigned sweep_acc = (unsigned)old + tot;
        S->cnt = 0ull;
        // src/evolve.cpp:169-178 with the reference's float/double rounding
        float av = av0;
        const double ratio = 1.0 * (double)sweep_acc / (double)R.valid;
        if (frozen0) {
        } else if (ratio < 0.5) {
          av = (float)((double)av * 0.99);
          if ((double)av < 0.01) av = (float)0.01;
        } else if (ratio > 0.5) {
          av = (float)((double)av / 0.99);
          if ((double)av > 1.0) av = (float)((double)av - 0.5);
        }
        S->ang_var = av;
        const unsigned long long sweep = sweep0 + 1;
        S->sweep = sweep;
        if (MODE == MODE_SWEEP_MEASURE) S->meas = meas0 + 1;
        double *st = a.stats + (size_t)r * kStats;
        atomicAdd(st + 7, (double)sweep_acc);
        atomicAdd(st + 8, 1.0);
        st[11] = (double)av;
        st[12] = (double)sweep;
      }
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

// Odd nx (free x bound only): a colour's sites of a row are i = 2h + s
// (s = (c + j + k) & 1), h < hx = (nx + 1) / 2, so the row's last storage
// slot h = hx - 1 holds the real site nx - 1 when s = 0 -- its x+ slot is the
// other colour's phantom, so it has no x+ bond -- and a phantom (i = nx) when
// s = 1.  Phantoms have point type 0, never move and add nothing to a
// measurement.  Returns 1 / 2 when site A / B of the pair at h0 is in that
// slot, else 0 (always 0 in unmasked kernels: an odd-nx replica has a mask;
// and in kernels built with ODD false, for batches without an odd nx).
template <bool MASK, bool ODD = true>
__device__ __forceinline__ uint8_t odd_tail(const RepDev &R, int h0) {
  if (!MASK || !ODD || !(R.nx & 1)) return 0;
  return h0 == R.hx - 1 ? 1 : (h0 + 1 == R.hx - 1 ? 2 : 0);
}

// Where a thread's pair lives and who its neighbours are.
struct PairGeom {
  int row, h0, j, k, s, off, exh, offp;
  bool valid, hasB;
  uint8_t tail;  // odd_tail
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
  g.tail = odd_tail<true>(R, g.h0);
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
  // odd nx: the phantom of an s = 1 row is skipped, the last site of an
  // s = 0 row has no x+ bond (odd_tail)
  const bool skipA = MASK && g.s == 1 && g.tail == 1, skipB = MASK && g.s == 1 && g.tail == 2;
  if (!skipA) {
    if (g.s == 0) {
      nb[0][0] = ox.x; nb[0][1] = oy.x; nb[0][2] = oz.x; e[0] = 1.f; w[0] = wt(1.f, po2.x);
      nb[1][0] = ex; nb[1][1] = ey; nb[1][2] = ez; e[1] = g.exe; w[1] = wt(g.exe, pex);
      if (MASK && g.tail == 1) e[0] = w[0] = 0.f;
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
  if (g.hasB && !skipB) {
    if (g.s == 0) {
      nb[0][0] = ox.y; nb[0][1] = oy.y; nb[0][2] = oz.y; e[0] = 1.f; w[0] = wt(1.f, po2.y);
      nb[1][0] = ox.x; nb[1][1] = oy.x; nb[1][2] = oz.x; e[1] = 1.f; w[1] = wt(1.f, po2.x);
      if (MASK && g.tail == 2) e[0] = w[0] = 0.f;
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

// One site update with the learned proposal: n' drawn from the network's
// antipodal vMF mixture (mcx_mlp.cuh), accepted with the Metropolis-Hastings
// probability min(1, exp(-dE/T) cosh(kappa mu.n)/cosh(kappa mu.n')); the
// network outputs depend only on the neighbours, so they are the same for the
// move and its reverse.  Four uniforms per site from Philox4x32-10 with
// counter (site, sweep, TAG_VMF).
template <int POT, bool MASK, bool FIELD, int MODE>
__device__ __forceinline__ unsigned site_update_learned(const RepDev &R, const PassArgs &a, int c, float &x, float &y,
                                                        float &z, const float nb[6][3], const float w[6],
                                                        const float e[6], int pself, float sx, float sy, float sz,
                                                        const float yo[4], float invT, uint32_t nat,
                                                        unsigned long long sw, float qs[kQ]) {
  constexpr bool MEAS = MODE == MODE_SWEEP_MEASURE || MODE == MODE_MEASURE_ONLY;
  constexpr bool UPD = MODE != MODE_MEASURE_ONLY;
  constexpr bool TRACE = MODE == MODE_TRACE;
  const int sid = pself - 2;
  const bool surf = MASK && pself > 1 && sid < R.nsurf;
  unsigned acc = 0;
  float eb = 0.f;
  if (pself != 0) {
    const float b_old = bond_sum<POT>(R, x, y, z, nb, w);
    eb = b_old;
    if (UPD) {
      const uint4 r = philox4x32_10(make_uint4(nat, (uint32_t)sw, (uint32_t)(sw >> 32), TAG_VMF), R.seed, R.stream);
      float mu[3], kappa, v[3];
      vmf_params(yo, mu, kappa);
      vmf_sample(mu, kappa, u01(r.x), u01(r.y), u01(r.z), v);
      const float b_new = bond_sum<POT>(R, v[0], v[1], v[2], nb, w);
      // every rounding of the log ratio fixed, as for the plain move's dE:
      // the learned forms with the same network take the same decisions
      float dE = __fmul_rn(bond_scale<POT>(R), __fsub_rn(b_new, b_old));
      if (surf)
        dE = __fadd_rn(dE, __fsub_rn(surface_energy(R, sid, v[0], v[1], v[2], sx, sy, sz),
                                     surface_energy(R, sid, x, y, z, sx, sy, sz)));
      if (FIELD) dE = __fadd_rn(dE, __fsub_rn(field_energy(R, v[0], v[1], v[2]), field_energy(R, x, y, z)));
      const float lo = log_cosh_shift(__fmul_rn(kappa, dot3_rn(mu[0], mu[1], mu[2], x, y, z)));
      const float ln = log_cosh_shift(__fmul_rn(kappa, dot3_rn(mu[0], mu[1], mu[2], v[0], v[1], v[2])));
      const float lr = __fsub_rn(fmaf(-dE, invT, lo), ln);
      const bool accept = u01(r.w) < __expf(lr);
      if (TRACE) {
        a.tr_dE[nat] = dE;
        a.tr_acc[nat] = accept ? 1 : 0;
        a.tr_prop[3 * (size_t)nat] = v[0];
        a.tr_prop[3 * (size_t)nat + 1] = v[1];
        a.tr_prop[3 * (size_t)nat + 2] = v[2];
        if (a.tr_y)
          for (int q = 0; q < 4; q++) a.tr_y[4 * (size_t)nat + q] = yo[q];
      }
      if (accept) {
        x = v[0];
        y = v[1];
        z = v[2];
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
      if (pself != 0) {
        const float ebs = bond_scale<POT>(R) * eb + bond_const<POT>(R, w);
        qs[0] += 2.f * ebs;
        qs[1] += 2.f * ebs;
        if (MASK) {
          float wi[6];
#pragma unroll
          for (int d = 0; d < 6; d++) wi[d] = e[d] - w[d];
          qs[0] += bond_scale<POT>(R) * bond_sum<POT>(R, x, y, z, nb, wi) + bond_const<POT>(R, wi);
        }
      } else {
        qs[0] += bond_scale<POT>(R) * bond_sum<POT>(R, x, y, z, nb, w) + bond_const<POT>(R, w);
      }
    }
  }
  return acc;
}

// Network input row of one site: its six neighbours (absent or inactive ones
// as zero vectors) in slot order, then T, then zeros to 32 columns; BF16,
// packed in pairs.
__device__ __forceinline__ void feature_words(const float nb[6][3], const float w[6], float T, bool live,
                                              uint32_t r[16]) {
  float f[20];
#pragma unroll
  for (int d = 0; d < 6; d++) {
    const float wd = live ? w[d] : 0.f;
    f[3 * d] = nb[d][0] * wd;
    f[3 * d + 1] = nb[d][1] * wd;
    f[3 * d + 2] = nb[d][2] * wd;
  }
  f[18] = live ? T : 0.f;
  f[19] = 0.f;
#pragma unroll
  for (int q = 0; q < 10; q++) r[q] = pack_bf16(f[2 * q], f[2 * q + 1]);
#pragma unroll
  for (int q = 10; q < 16; q++) r[q] = 0u;
}

__device__ __forceinline__ void write_features(__nv_bfloat16 *row, const float nb[6][3], const float w[6], float T,
                                               bool live) {
  uint32_t r[16];
  feature_words(nb, w, T, live, r);
  uint32_t *d = reinterpret_cast<uint32_t *>(row);
#pragma unroll
  for (int q = 0; q < 16; q++) d[q] = r[q];
}

template <int POT, bool MASK, bool FIELD, int MODE>
__device__ __forceinline__ void compute_pair_learned(const PassArgs &a, int c, int2 m, const PairStage<MASK> &st,
                                                     const uint8_t *W, __nv_bfloat16 *X, float *Y, unsigned &acc,
                                                     float qs[kQ]) {
  constexpr bool UPD = MODE != MODE_MEASURE_ONLY;
  const RepDev &R = a.reps[m.x];
  RepState *S = a.st + m.x;
  const int lane = threadIdx.x & 31, tid = threadIdx.x, P = R.plane;
  PairGeom g;
  pair_geom(R, c, m.y + tid, g);
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
  auto wt = [&](float ee, uint8_t pp) { return MASK ? (ee != 0.f && pp != 0 ? 1.f : 0.f) : ee; };
  float nbA[6][3], wA[6], eA[6], nbB[6][3], wB[6], eB[6];
  if (g.s == 0) {
    nbA[0][0] = ox.x; nbA[0][1] = oy.x; nbA[0][2] = oz.x; eA[0] = 1.f; wA[0] = wt(1.f, po2.x);
    nbA[1][0] = ex; nbA[1][1] = ey; nbA[1][2] = ez; eA[1] = g.exe; wA[1] = wt(g.exe, pex);
    nbB[0][0] = ox.y; nbB[0][1] = oy.y; nbB[0][2] = oz.y; eB[0] = 1.f; wB[0] = wt(1.f, po2.y);
    nbB[1][0] = ox.x; nbB[1][1] = oy.x; nbB[1][2] = oz.x; eB[1] = 1.f; wB[1] = wt(1.f, po2.x);
    if (MASK && g.tail == 1) eA[0] = wA[0] = 0.f;
    if (MASK && g.tail == 2) eB[0] = wB[0] = 0.f;
  } else {
    if (g.hasB) {
      nbA[0][0] = ox.y; nbA[0][1] = oy.y; nbA[0][2] = oz.y; eA[0] = 1.f; wA[0] = wt(1.f, po2.y);
    } else {
      nbA[0][0] = ex; nbA[0][1] = ey; nbA[0][2] = ez; eA[0] = g.exe; wA[0] = wt(g.exe, pex);
    }
    nbA[1][0] = ox.x; nbA[1][1] = oy.x; nbA[1][2] = oz.x; eA[1] = 1.f; wA[1] = wt(1.f, po2.x);
    nbB[0][0] = ex; nbB[0][1] = ey; nbB[0][2] = ez; eB[0] = g.exe; wB[0] = wt(g.exe, pex);
    nbB[1][0] = ox.y; nbB[1][1] = oy.y; nbB[1][2] = oz.y; eB[1] = 1.f; wB[1] = wt(1.f, po2.y);
  }
#pragma unroll
  for (int d = 0; d < 4; d++) {
    const float2 Xv = st.v[6 + 3 * d][tid], Yv = st.v[7 + 3 * d][tid], Zv = st.v[8 + 3 * d][tid];
    nbA[2 + d][0] = Xv.x; nbA[2 + d][1] = Yv.x; nbA[2 + d][2] = Zv.x;
    nbB[2 + d][0] = Xv.y; nbB[2 + d][1] = Yv.y; nbB[2 + d][2] = Zv.y;
    eA[2 + d] = eB[2 + d] = g.er[d];
    wA[2 + d] = wt(g.er[d], MASK ? pr[d].x : 1);
    wB[2 + d] = wt(g.er[d], MASK ? pr[d].y : 1);
  }
  const int psA = MASK ? pself2.x : 1, psB = MASK ? pself2.y : 1;
  const float T = g.valid ? S->T : 0.f;
  __syncwarp();
  write_features(X + (size_t)(2 * lane) * kXs, nbA, wA, T, g.valid);
  write_features(X + (size_t)(2 * lane + 1) * kXs, nbB, wB, T, g.valid && g.hasB);
  __syncwarp();
  mlp_warp(W, X, Y);
  __syncwarp();
  if (!g.valid) return;
  float yA[4], yB[4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    yA[q] = Y[(2 * lane) * 4 + q];
    yB[q] = Y[(2 * lane + 1) * 4 + q];
  }
  float2 ax = st.v[0][tid], ay = st.v[1][tid], az = st.v[2][tid];
  const unsigned long long sw = UPD ? S->sweep : 0ull;
  const float invT = UPD ? 1.0f / S->T : 0.f;
  const bool skipA = MASK && g.s == 1 && g.tail == 1, skipB = MASK && g.s == 1 && g.tail == 2;
  if (!skipA) {
    float sx = 0.f, sy = 0.f, sz = 0.f;
    if (MASK && psA > 1) {
      const float *nsb = a.ns + R.ns_off + (long long)(c * 3) * P + g.off;
      sx = __ldg(nsb);
      sy = __ldg(nsb + P);
      sz = __ldg(nsb + 2 * P);
    }
    const uint32_t nat = (uint32_t)(2 * g.h0 + g.s) + (uint32_t)R.nx * (uint32_t)g.row;
    acc += site_update_learned<POT, MASK, FIELD, MODE>(R, a, c, ax.x, ay.x, az.x, nbA, wA, eA, psA, sx, sy, sz, yA,
                                                       invT, nat, sw, qs);
  }
  if (g.hasB && !skipB) {
    float sx = 0.f, sy = 0.f, sz = 0.f;
    if (MASK && psB > 1) {
      const float *nsb = a.ns + R.ns_off + (long long)(c * 3) * P + g.off + 1;
      sx = __ldg(nsb);
      sy = __ldg(nsb + P);
      sz = __ldg(nsb + 2 * P);
    }
    const uint32_t nat = (uint32_t)(2 * g.h0 + 2 + g.s) + (uint32_t)R.nx * (uint32_t)g.row;
    acc += site_update_learned<POT, MASK, FIELD, MODE>(R, a, c, ax.y, ay.y, az.y, nbB, wB, eB, psB, sx, sy, sz, yB,
                                                       invT, nat, sw, qs);
  }
  if (UPD) {
    float *gA = a.dir + R.dir_off + (long long)(c * 3) * P + g.off;
    *reinterpret_cast<float2 *>(gA) = ax;
    *reinterpret_cast<float2 *>(gA + P) = ay;
    *reinterpret_cast<float2 *>(gA + 2 * P) = az;
  }
}

// Dynamic shared memory of the learned pass: weights, then per warp its 64
// input rows and 64 output rows.
constexpr int kLearnSmem = kMlpBytes + (kPB / 32) * (64 * kXs * 2 + 64 * 4 * 4);

// The learned pass is bound by arithmetic, not by loads: it keeps one stage
// (no prefetch of the next pair) so that three CTAs fit on an SM.
template <int POT, bool MASK, bool FIELD, int MODE, bool LEARN>
#ifndef MCX_LEARN_MIN_BLOCKS
#define MCX_LEARN_MIN_BLOCKS 3
#endif
__global__ void __launch_bounds__(kPB, LEARN ? MCX_LEARN_MIN_BLOCKS : MCX_PASS_MIN_BLOCKS) k_pass(PassArgs a) {
  __shared__ PairStage<MASK> stages[LEARN ? 1 : 2];
  extern __shared__ __align__(16) uint8_t dyn_smem[];
  const int c = a.colour;
  uint8_t *mlpW = dyn_smem;
  __nv_bfloat16 *mlpX = reinterpret_cast<__nv_bfloat16 *>(dyn_smem + kMlpBytes) + (size_t)(threadIdx.x >> 5) * 64 * kXs;
  float *mlpY = reinterpret_cast<float *>(dyn_smem + kMlpBytes + (kPB / 32) * 64 * kXs * 2) +
                (size_t)(threadIdx.x >> 5) * 64 * 4;
  if (LEARN) {
    for (int i = threadIdx.x; i < kMlpBytes / 16; i += kPB)
      reinterpret_cast<int4 *>(mlpW)[i] = reinterpret_cast<const int4 *>(a.mlp)[i];
    __syncthreads();
  }
  const int G = gridDim.x, n = a.nmap;
  int e = blockIdx.x;
  if (!LEARN && e < n) prefetch_pair<MASK>(a, c, a.map[e], stages[0]);
  cp_async_commit();
  int cur = -1, units = 0;
  unsigned acc = 0;
  float qs[kQ];
#pragma unroll
  for (int q = 0; q < kQ; q++) qs[q] = 0.f;
  for (int it = 0; e < n; it++, e += G) {
    const int2 m = a.map[e];
    if (LEARN) {
      prefetch_pair<MASK>(a, c, m, stages[0]);
    } else if (e + G < n) {
      prefetch_pair<MASK>(a, c, a.map[e + G], stages[(it + 1) & 1]);
    }
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
    if (LEARN) {
      asm volatile("cp.async.wait_all;" ::: "memory");
      compute_pair_learned<POT, MASK, FIELD, MODE>(a, c, m, stages[0], mlpW, mlpX, mlpY, acc, qs);
      __syncwarp();  // every lane done with its stage slots before they are refilled
    } else {
      cp_async_wait1();
      compute_pair<POT, MASK, FIELD, MODE>(a, c, m, stages[it & 1], acc, qs);
    }
    units++;
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  if (cur >= 0) flush_replica<kPB, MODE>(a, cur, units, (unsigned)a.reps[cur].ncta, acc, qs, MASK);
}


}  // namespace mcx
