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
#include "mcx_pass.cuh"
#include "mcx_tma.cuh"

namespace mcx {

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

// Local order parameter of every site (lattice_order_parameter,
// src/parameter_order.cpp:62-113): Q over the site and its existing active
// neighbours, accumulated in FP32 in the reference's order (x-, y-, z-, the
// site, z+, y+, x+; upper triangle, 3 n_l n_m per point and -1 on the
// diagonal, over 2 points), its largest eigenvalue by Jacobi in FP64.  NaN at
// inactive sites (src/io.cpp:66-71).  Natural site order.
__device__ __forceinline__ bool bound_ok(int &x, int n, int b) {
  if (x >= 0 && x < n) return true;
  if (b != BOUND_PERIODIC) return false;
  x = x < 0 ? x + n : x - n;
  return true;
}

__device__ __forceinline__ void site_dir(const RepDev &R, const float *dir, int i, int j, int k, float v[3]) {
  const int c = (i + j + k) & 1;
  const long long off = (long long)(j + R.ny * k) * R.hs + (i >> 1);
  const float *d = dir + R.dir_off + (long long)(c * 3) * R.plane + off;
  v[0] = d[0];
  v[1] = d[R.plane];
  v[2] = d[2 * R.plane];
}

__device__ __forceinline__ int site_type(const RepDev &R, const uint8_t *pt, int i, int j, int k) {
  if (pt == nullptr) return 1;
  const int c = (i + j + k) & 1;
  return pt[R.pt_off + (long long)c * R.pplane + (long long)(j + R.ny * k) * R.hps + (i >> 1)];
}

__global__ void k_local_order(RepDev R, const float *__restrict__ dir, const uint8_t *__restrict__ pt,
                              float *__restrict__ out) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= R.ntot) return;
  const int i = (int)(s % R.nx), j = (int)((s / R.nx) % R.ny), k = (int)(s / ((long long)R.nx * R.ny));
  if (site_type(R, pt, i, j, k) == 0) {
    out[s] = __int_as_float(0x7fc00000);
    return;
  }
  const int d[7][3] = {{-1, 0, 0}, {0, -1, 0}, {0, 0, -1}, {0, 0, 0}, {0, 0, 1}, {0, 1, 0}, {1, 0, 0}};
  float Q[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  int points = 0;
  for (int q = 0; q < 7; q++) {
    int ii = i + d[q][0], jj = j + d[q][1], kk = k + d[q][2];
    if (!bound_ok(ii, R.nx, R.xb) || !bound_ok(jj, R.ny, R.yb) || !bound_ok(kk, R.nz, R.zb)) continue;
    if (site_type(R, pt, ii, jj, kk) == 0) continue;
    float v[3];
    site_dir(R, dir, ii, jj, kk, v);
    for (int l = 0; l < 3; l++) {
      for (int m = 0; m <= l; m++) Q[3 * m + l] += 3.0f * (v[l] * v[m]);
      Q[4 * l] -= 1.f;
    }
    points++;
  }
  const float den = 2.0f * (float)points;
  double Qd[9];
  Qd[0] = Q[0] / den;
  Qd[1] = Q[1] / den;
  Qd[2] = Q[2] / den;
  Qd[4] = Q[4] / den;
  Qd[5] = Q[5] / den;
  Qd[8] = Q[8] / den;
  Qd[3] = Qd[1];
  Qd[6] = Qd[2];
  Qd[7] = Qd[5];
  double lam, vec[3];
  jacobi_sym3(Qd, lam, vec);
  out[s] = (float)lam;
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
    case MODE_SWEEP: k_pass<POT, MASK, FIELD, MODE_SWEEP, false><<<nblocks, kPB, 0, st>>>(a); break;
    case MODE_SWEEP_MEASURE: k_pass<POT, MASK, FIELD, MODE_SWEEP_MEASURE, false><<<nblocks, kPB, 0, st>>>(a); break;
    case MODE_MEASURE_ONLY: k_pass<POT, MASK, FIELD, MODE_MEASURE_ONLY, false><<<nblocks, kPB, 0, st>>>(a); break;
    default: k_pass<POT, MASK, FIELD, MODE_TRACE, false><<<nblocks, kPB, 0, st>>>(a); break;
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
    case MODE_SWEEP: return (const void *)k_pass<POT, MASK, FIELD, MODE_SWEEP, false>;
    case MODE_SWEEP_MEASURE: return (const void *)k_pass<POT, MASK, FIELD, MODE_SWEEP_MEASURE, false>;
    case MODE_MEASURE_ONLY: return (const void *)k_pass<POT, MASK, FIELD, MODE_MEASURE_ONLY, false>;
    default: return (const void *)k_pass<POT, MASK, FIELD, MODE_TRACE, false>;
  }
}

int pass_block_threads() { return kPB; }

int pass_blocks_per_sm(const Variant &v, int mode) {
  const void *fn;
  if (v.pot == POT_LL) {
    if (v.mask) fn = v.field ? pass_fn<POT_LL, true, true>(mode) : pass_fn<POT_LL, true, false>(mode);
    else fn = v.field ? pass_fn<POT_LL, false, true>(mode) : pass_fn<POT_LL, false, false>(mode);
  } else if (v.pot == POT_PEAR) {
    if (v.mask) fn = v.field ? pass_fn<POT_PEAR, true, true>(mode) : pass_fn<POT_PEAR, true, false>(mode);
    else fn = v.field ? pass_fn<POT_PEAR, false, true>(mode) : pass_fn<POT_PEAR, false, false>(mode);
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
  else if (v.pot == POT_PEAR) launch_pass_p<POT_PEAR>(v, mode, a, nblocks, st);
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
  if (v.pot == POT_PEAR) return 0;  // the staged pass is built for LL and GHRL only
  const void *fn = tpass_select(v, mode);
  const int smem = tpass_smem_bytes(stage_bytes);
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kBlock, smem) != cudaSuccess) return 0;
  return n;
}

void launch_tpass(const Variant &v, int mode, const PassArgs &a, int grid, cudaStream_t st) {
  if (v.pot == POT_PEAR) return;  // never selected for Pear (tpass_blocks_per_sm is 0)
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
// Sum of the directors of every site (the polarization's numerator), FP64.
__global__ void k_polarization(RepDev R, const float *__restrict__ dir, double *out) {
  __shared__ double red[3][8];
  double v[3] = {0, 0, 0};
  for (long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x; s < 2LL * R.plane; s += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(s / R.plane);
    const long long o = s - (long long)c * R.plane;
    const long long row = o / R.hs;
    const int h = (int)(o - row * R.hs);
    const int j = (int)(row % R.ny), k = (int)(row / R.ny);
    const int i = 2 * h + ((c + j + k) & 1);
    if (h >= R.hx || i >= R.nx) continue;  // row padding
    const float *d = dir + R.dir_off + (long long)(c * 3) * R.plane + o;
    v[0] += d[0];
    v[1] += d[R.plane];
    v[2] += d[2 * R.plane];
  }
  for (int q = 0; q < 3; q++) {
    for (int off = 16; off > 0; off >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], off);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = v[q];
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0;
    for (int w = 0; w < 8; w++) t += red[threadIdx.x][w];
    atomicAdd(out + threadIdx.x, t);
  }
}

void launch_polarization(const RepDev &R, const float *dir, double *out, cudaStream_t st) {
  cudaMemsetAsync(out, 0, 3 * sizeof(double), st);
  k_polarization<<<256, 256, 0, st>>>(R, dir, out);
}

// Replica combination (average_replicas.py:74-103).  One CTA; every thread
// walks the index list with a fixed stride and the partial sums meet in a
// fixed-order tree, so the result does not depend on timing.  Pass 1 sums T,
// S, varS, E, varE and P and finds the T range; pass 2 sums the squared
// deviations of S and E from their means (numpy's var with ddof 0).
// pol: three FP64 director sums per listed replica, or null.
constexpr int kCombineThreads = 256;

struct CombineRow {
  double S, vS, E, vE;
};

__device__ __forceinline__ CombineRow combine_row(const double *st) {
  const double n = st[0];
  const double S = st[1] / n, E = st[3] / n;
  return {S, st[2] / n - S * S, E, st[4] / n - E * E};
}

template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double (*red)[kCombineThreads]) {
  for (int q = 0; q < K; q++) red[q][threadIdx.x] = v[q];
  __syncthreads();
  for (int w = kCombineThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int q = 0; q < K; q++) red[q][threadIdx.x] += red[q][threadIdx.x + w];
    __syncthreads();
  }
  for (int q = 0; q < K; q++) v[q] = red[q][0];
  __syncthreads();
}

__global__ void __launch_bounds__(kCombineThreads) k_combine(const RepDev *rep, const RepState *rst,
                                                             const double *stats, const double *pol,
                                                             const int *idx, int n, double *out) {
  __shared__ double red[6][kCombineThreads];
  __shared__ float tmin[kCombineThreads], tmax[kCombineThreads];
  __shared__ int empty[kCombineThreads];
  double v[6] = {0, 0, 0, 0, 0, 0};  // T, S, varS, E, varE, P
  float lo = INFINITY, hi = -INFINITY;
  int ne = 0;
  for (int i = threadIdx.x; i < n; i += kCombineThreads) {
    const int r = idx[i];
    const double *st = stats + (size_t)r * kStats;
    const float T = rst[r].T;
    lo = fminf(lo, T);
    hi = fmaxf(hi, T);
    v[0] += (double)T;
    if (st[0] <= 0) {
      ne++;
      continue;
    }
    const CombineRow c = combine_row(st);
    v[1] += c.S;
    v[2] += c.vS;
    v[3] += c.E;
    v[4] += c.vE;
    if (pol) {
      const double *p = pol + 3 * (size_t)i;
      v[5] += sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]) / (double)rep[r].ntot;
    }
  }
  tmin[threadIdx.x] = lo;
  tmax[threadIdx.x] = hi;
  empty[threadIdx.x] = ne;
  block_sum(v, red);  // its barriers also publish tmin/tmax/empty
  if (threadIdx.x == 0)
    for (int t = 1; t < kCombineThreads; t++) {
      lo = fminf(lo, tmin[t]);
      hi = fmaxf(hi, tmax[t]);
      ne += empty[t];
    }
  const double inv = 1.0 / (double)n;
  const double mS = v[1] * inv, mE = v[3] * inv;
  double d[2] = {0, 0};
  for (int i = threadIdx.x; i < n; i += kCombineThreads) {
    const double *st = stats + (size_t)idx[i] * kStats;
    if (st[0] <= 0) continue;
    const CombineRow c = combine_row(st);
    d[0] += (c.S - mS) * (c.S - mS);
    d[1] += (c.E - mE) * (c.E - mE);
  }
  block_sum(d, red);
  if (threadIdx.x == 0) {
    out[0] = v[0] * inv;
    out[1] = mS;
    out[2] = v[2] * inv + d[0] * inv;
    out[3] = mE;
    out[4] = v[4] * inv + d[1] * inv;
    out[5] = pol ? v[5] * inv : __longlong_as_double(0x7ff8000000000000LL);
    out[6] = (double)n;
    out[7] = (double)hi - (double)lo;
    out[8] = (double)ne;
  }
}

void launch_combine(const RepDev *rep, const RepState *st, const double *stats, const double *pol, const int *idx,
                    int n, double *out, cudaStream_t s) {
  k_combine<<<1, kCombineThreads, 0, s>>>(rep, st, stats, pol, idx, n, out);
}

void launch_local_order(const RepDev &R, const float *dir, const uint8_t *pt, float *out, cudaStream_t st) {
  k_local_order<<<(unsigned)((R.ntot + 255) / 256), 256, 0, st>>>(R, dir, pt, out);
}

void launch_init(const RepDev &R, const uint8_t *pt, float *dir, int mode, uint32_t seed, float fx, float fy, float fz,
                 cudaStream_t st) {
  k_init<<<blocks_for(R.ntot), 256, 0, st>>>(R, pt, dir, mode, seed, fx, fy, fz);
}

}  // namespace mcx
