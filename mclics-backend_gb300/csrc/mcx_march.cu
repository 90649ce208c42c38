// mcx_march.cu -- the plain-proposal red/black pass as a z-march (the sweep
// kernel of mcx_sweep for the reference's rotation move).
//
//   k_march  one red/black half-sweep of every replica (EvolveN::
//            Monte_Carlo_Step, src/evolve.cpp:64-179 of the reference, with 2
//            colours instead of 8).  A CTA owns NT consecutive same-colour
//            site pairs of one z-plane (pairs numbered row-major within the
//            plane; in masked replicas whose rows cross the mask's edge, a
//            tile of kTileW pairs x NT / kTileW rows) and marches them
//            through a chunk of K planes.  Per plane
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
// It computes what the other passes compute (same site_update, same Philox
// counter: pair index row * hp + q, sweep, colour), and as the energy change
// fixes every rounding (bond_sum in mcx_pass.cuh), it runs the same chain bit
// for bit.  The kernel template is in mcx_march_kernel.cuh; the variant for
// masked batches with an odd nx is built in mcx_march_odd.cu.
#include <cuda_runtime.h>

#include "mcx_march.cuh"
#include "mcx_march_kernel.cuh"
#include "mcx_tma.cuh"

namespace mcx {

// ---------------------------------------------------------------------------
// The z-march with its rows staged in shared memory by bulk copies (TMA).
//
// A CTA's block of NT pairs spans rows jA0..jA1 of a plane.  Per plane it
// needs its own rows (A) and the opposite colour's rows jA0-1..jA1+1 (O);
// rows of a plane are contiguous in the split layout, so each is one
// cp.async.bulk per component (plus one row for each y edge that wraps).
// Shared memory holds a ring of four O planes (k-1, k, k+1 and k+2 in
// flight) and two A planes (k and k+1 in flight).  Thread 0 issues the next
// plane's copies before the block computes the current one, so the copies
// overlap the arithmetic; an mbarrier per step parity counts the bytes, and
// every wait is bounded (on timeout: error flag, drain, exit).  Rows that do
// not exist (free y or z boundaries) are filled with a copy of a real row, so
// shared memory never holds undefined values; their bonds have weight 0.
// Unmasked lattices only.
// ---------------------------------------------------------------------------
struct TSlots {
  float *base;
  int so, sa;    // floats per O slot and per A slot
  int nrO, nrA;  // rows per O / A slot
  __device__ __forceinline__ float *O(int kk) const { return base + (size_t)((kk + 4) & 3) * so; }
  __device__ __forceinline__ float *A(int kk) const { return base + (size_t)4 * so + (size_t)(kk & 1) * sa; }
};

// The plane index a z neighbour kk of the march reads (wrapped when z is
// periodic; a plane that does not exist reads plane `fallback`).
__device__ __forceinline__ int tm_plane(const RepDev &R, int kk, int fallback) {
  if (kk < 0) return R.zb == BOUND_PERIODIC ? kk + R.nz : fallback;
  if (kk >= R.nz) return R.zb == BOUND_PERIODIC ? kk - R.nz : fallback;
  return kk;
}

// Issues the copies of opposite plane kk (already wrapped; on = false: the
// plane does not exist, copy plane `self` instead) into slot `dst`; returns
// the bytes.
__device__ __forceinline__ uint32_t tm_copy_O(const RepDev &R, const float *Ob, int kk, int jA0, int jA1, float *dst,
                                              int nrO, uint64_t *bar, bool issue) {
  const int hs = R.hs, ny = R.ny, P = R.plane;
  const int base = ny * kk;
  const int j_lo = max(jA0 - 1, 0), j_hi = min(jA1 + 1, ny - 1);
  uint32_t bytes = 0;
#pragma unroll
  for (int q = 0; q < 3; q++) {
    float *d = dst + (size_t)q * nrO * hs;
    const float *src = Ob + (size_t)q * P;
    const uint32_t nb = (uint32_t)(j_hi - j_lo + 1) * hs * 4;
    if (issue) bulk_copy_g2s(d + (size_t)(j_lo - (jA0 - 1)) * hs, src + (size_t)(base + j_lo) * hs, nb, bar);
    bytes += nb;
    if (jA0 == 0) {  // slot 0 is row -1: row ny-1 when y is periodic, else row 0 (weight 0)
      const int jr = R.yb == BOUND_PERIODIC ? ny - 1 : 0;
      if (issue) bulk_copy_g2s(d, src + (size_t)(base + jr) * hs, hs * 4, bar);
      bytes += hs * 4;
    }
    if (jA1 == ny - 1) {  // the last slot is row ny: row 0 when periodic, else row ny-1
      const int jr = R.yb == BOUND_PERIODIC ? 0 : ny - 1;
      if (issue) bulk_copy_g2s(d + (size_t)(nrO - 1) * hs, src + (size_t)(base + jr) * hs, hs * 4, bar);
      bytes += hs * 4;
    }
  }
  return bytes;
}

__device__ __forceinline__ uint32_t tm_copy_A(const RepDev &R, const float *Ab, int kk, int jA0, int nrA, float *dst,
                                              uint64_t *bar, bool issue) {
  const int hs = R.hs, P = R.plane;
  const uint32_t nb = (uint32_t)nrA * hs * 4;
  if (issue)
#pragma unroll
    for (int q = 0; q < 3; q++)
      bulk_copy_g2s(dst + (size_t)q * nrA * hs, Ab + (size_t)q * P + (size_t)(R.ny * kk + jA0) * hs, nb, bar);
  return 3 * nb;
}

// Registers the bytes of a step's copies on its mbarrier, then issues them
// (O planes kk0..kk1 of the march, fallback plane for absent ones, and A
// plane ka when ka >= 0).
__device__ __forceinline__ void tm_issue(const RepDev &R, const float *Ob, const float *Ab, int kk0, int kk1,
                                         int fallback, int ka, int jA0, int jA1, const TSlots &sl, uint64_t *bar) {
  uint32_t bytes = 0;
  for (int kk = kk0; kk <= kk1; kk++)
    bytes += tm_copy_O(R, Ob, tm_plane(R, kk, fallback), jA0, jA1, sl.O(kk), sl.nrO, bar, false);
  if (ka >= 0) bytes += tm_copy_A(R, Ab, ka, jA0, sl.nrA, sl.A(ka), bar, false);
  mbar_arrive_expect_tx(bar, bytes);
  for (int kk = kk0; kk <= kk1; kk++)
    tm_copy_O(R, Ob, tm_plane(R, kk, fallback), jA0, jA1, sl.O(kk), sl.nrO, bar, true);
  if (ka >= 0) tm_copy_A(R, Ab, ka, jA0, sl.nrA, sl.A(ka), bar, true);
}

__device__ __forceinline__ void lds_opair(const float *slot, int nrO, int hs, int row, int h, OPair &o) {
  const int base = row * hs + h;
  o.v[0] = *reinterpret_cast<const float2 *>(slot + base);
  o.v[1] = *reinterpret_cast<const float2 *>(slot + (size_t)nrO * hs + base);
  o.v[2] = *reinterpret_cast<const float2 *>(slot + (size_t)2 * nrO * hs + base);
  o.pt = 0x0101;
}

template <int POT, bool FIELD, int MODE, int NT, bool PER>
__global__ void __launch_bounds__(NT, march_min_blocks<POT, false, NT>()) k_tmarch(PassArgs a) {
  static_assert(MODE == MODE_SWEEP || MODE == MODE_SWEEP_MEASURE, "sweep modes only");
  extern __shared__ __align__(128) char smem[];
  __shared__ __align__(8) uint64_t bars[2];
  const int4 u = a.units[blockIdx.x];
  const int r = u.x, c = a.colour;
  const RepDev &R = a.reps[r];
  const RepState *S = a.st + r;
  const int hp = R.hp, hs = R.hs, ny = R.ny, nz = R.nz, hx = R.hx;
  const int p0 = u.y, pend = min(p0 + NT, hp * ny);
  const int jA0 = (int)fastdiv((uint32_t)p0, R.hp_m, R.hp_p), jA1 = (int)fastdiv((uint32_t)(pend - 1), R.hp_m, R.hp_p);
  TSlots sl;
  sl.nrA = jA1 - jA0 + 1;
  sl.nrO = sl.nrA + 2;
  sl.base = reinterpret_cast<float *>(smem);
  sl.so = a.tm_o;
  sl.sa = a.tm_a;
  const float *Ob = a.dir + R.dir_off + (long long)((c ^ 1) * 3) * R.plane;
  float *Ag = a.dir + R.dir_off + (long long)(c * 3) * R.plane;
  const int kb = u.z, L = u.w;
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // geometry of this thread's pair (constants only)
  const int p = p0 + (int)threadIdx.x;
  const bool valid = p < pend;
  const int j = valid ? (int)fastdiv((uint32_t)p, R.hp_m, R.hp_p) : jA0;
  const int h0 = valid ? 2 * (p - j * hp) : 0;
  const bool hasB = h0 + 1 < hx;
  int ex0 = h0 - 1, ex1 = hasB ? h0 + 2 : h0 + 1;
  float ee0 = 1.f, ee1 = 1.f;
  if (ex0 < 0) { if (R.xb == BOUND_PERIODIC) ex0 = hx - 1; else { ee0 = 0.f; ex0 = h0; } }
  if (ex1 == hx) { if (R.xb == BOUND_PERIODIC) ex1 = 0; else { ee1 = 0.f; ex1 = h0; } }
  const float eyp = (j + 1 < ny || R.yb == BOUND_PERIODIC) ? 1.f : 0.f;
  const float eym = (j > 0 || R.yb == BOUND_PERIODIC) ? 1.f : 0.f;
  const int rA = j - jA0, rO = j - jA0 + 1;  // rows of the pair in the A and O slots
  const uint32_t seed = R.seed, stream = R.stream;
  grid_dependency_wait();  // the directors and the state may still be written by the previous pass
  const unsigned long long sw = S->sweep;
  const float ang = S->ang_var, invT = 1.0f / S->T;
  // prologue: O planes kb-1, kb, kb+1 and A plane kb on bars[0]
  if (threadIdx.x == 0) {
    fence_proxy_async();
    tm_issue(R, Ob, Ag, kb - 1, kb + 1, kb, kb, jA0, jA1, sl, &bars[0]);
  }
  unsigned acc = 0;
  float qs[kQ];
#pragma unroll
  for (int q = 0; q < kQ; q++) qs[q] = 0.f;
  for (int t = 0; t < L; t++) {
    const int k = kb + t;
    // copies for the next step: A plane k+1, O plane k+2
    if (threadIdx.x == 0 && t + 1 < L) {
      fence_proxy_async();
      tm_issue(R, Ob, Ag, k + 2, k + 2, k + 1, k + 1, jA0, jA1, sl, &bars[(t + 1) & 1]);
    }
    const bool ok = mbar_wait(&bars[t & 1], (uint32_t)((t >> 1) & 1));
    if (__syncthreads_or(!ok)) {
      // a step's copies never completed: report, let the copies in flight
      // land (bounded: this step's, and the next step's when they were
      // issued), leave without touching the sums
      if (threadIdx.x == 0) {
        atomicExch(a.err, 1u);
        mbar_wait(&bars[t & 1], (uint32_t)((t >> 1) & 1));
        if (t + 1 < L) mbar_wait(&bars[(t + 1) & 1], (uint32_t)(((t + 1) >> 1) & 1));
      }
      return;
    }
    if (valid) {
      const int s = (c + j + k) & 1;
      const float *OK = sl.O(k), *OP = sl.O(k + 1), *OM = sl.O(k - 1);
      const float *AK = sl.A(k);
      float2 ax = *reinterpret_cast<const float2 *>(AK + rA * hs + h0);
      float2 ay = *reinterpret_cast<const float2 *>(AK + (size_t)sl.nrA * hs + rA * hs + h0);
      float2 az = *reinterpret_cast<const float2 *>(AK + (size_t)2 * sl.nrA * hs + rA * hs + h0);
      const int exh = s ? ex1 : ex0;
      const float exv[3] = {OK[rO * hs + exh], OK[(size_t)sl.nrO * hs + rO * hs + exh],
                            OK[(size_t)2 * sl.nrO * hs + rO * hs + exh]};
      OPair o0, yp, ym, op, om;
      lds_opair(OK, sl.nrO, hs, rO, h0, o0);
      lds_opair(OK, sl.nrO, hs, rO + 1, h0, yp);
      lds_opair(OK, sl.nrO, hs, rO - 1, h0, ym);
      lds_opair(OP, sl.nrO, hs, rO, h0, op);
      lds_opair(OM, sl.nrO, hs, rO, h0, om);
      const bool zp = k + 1 < nz || R.zb == BOUND_PERIODIC, zm = k > 0 || R.zb == BOUND_PERIODIC;
      const int row = j + ny * k;
      update_pair<POT, false, FIELD, MODE, PER>(a, R, c, s, hasB, ee0, ee1, eyp, eym, o0, yp, ym, op, om, exv, 0x0101,
                                                1, zp, zm, (uint32_t)row * (uint32_t)hp + (uint32_t)(h0 >> 1),
                                                (long long)row * hs + h0, seed, stream, sw, ang, invT, ax, ay, az,
                                                acc, qs);
      float *g = Ag + (size_t)row * hs + h0;
      *reinterpret_cast<float2 *>(g) = ax;
      *reinterpret_cast<float2 *>(g + R.plane) = ay;
      *reinterpret_cast<float2 *>(g + 2 * R.plane) = az;
    }
    __syncthreads();  // the slots of this step may be refilled from here on
  }
  grid_launch_dependents();
  flush_replica<NT, MODE>(a, r, 1, (unsigned)R.mcta, acc, qs, false);
}

// ---------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------
template <int POT, bool MASK, bool FIELD, int NT, bool PER>
static const void *march_fn(int mode) {
  return mode == MODE_SWEEP_MEASURE ? (const void *)k_march<POT, MASK, FIELD, MODE_SWEEP_MEASURE, NT, PER, false>
                                    : (const void *)k_march<POT, MASK, FIELD, MODE_SWEEP, NT, PER, false>;
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
  if (v.pot == POT_PEAR) {
    if (v.mask)
      return v.field ? march_fn<POT_PEAR, true, true, NT, false>(mode) : march_fn<POT_PEAR, true, false, NT, false>(mode);
    return v.field ? march_fn_unmasked<POT_PEAR, true, NT>(v, mode) : march_fn_unmasked<POT_PEAR, false, NT>(v, mode);
  }
  if (v.mask)
    return v.field ? march_fn<POT_GHRL, true, true, NT, false>(mode) : march_fn<POT_GHRL, true, false, NT, false>(mode);
  return v.field ? march_fn_unmasked<POT_GHRL, true, NT>(v, mode) : march_fn_unmasked<POT_GHRL, false, NT>(v, mode);
}

static const void *march_kernel(const Variant &v, int mode, int nt) {
  if (v.mask && v.odd) return march_kernel_odd(v, mode, nt);
  switch (nt) {
    case 64: return march_fn_v<64>(v, mode);
    case 256: return march_fn_v<256>(v, mode);
    default: return march_fn_v<128>(v, mode);
  }
}

bool march_block_ok(int nt) { return nt == 64 || nt == 128 || nt == 256; }

template <int POT, bool FIELD, int NT>
static const void *tmarch_fn(const Variant &v, int mode) {
  if (mode == MODE_SWEEP_MEASURE)
    return v.per ? (const void *)k_tmarch<POT, FIELD, MODE_SWEEP_MEASURE, NT, true>
                 : (const void *)k_tmarch<POT, FIELD, MODE_SWEEP_MEASURE, NT, false>;
  return v.per ? (const void *)k_tmarch<POT, FIELD, MODE_SWEEP, NT, true>
               : (const void *)k_tmarch<POT, FIELD, MODE_SWEEP, NT, false>;
}

template <int NT>
static const void *tmarch_fn_v(const Variant &v, int mode) {
  if (v.pot == POT_LL) return v.field ? tmarch_fn<POT_LL, true, NT>(v, mode) : tmarch_fn<POT_LL, false, NT>(v, mode);
  return v.field ? tmarch_fn<POT_GHRL, true, NT>(v, mode) : tmarch_fn<POT_GHRL, false, NT>(v, mode);
}

static const void *tmarch_kernel(const Variant &v, int mode, int nt) {
  switch (nt) {
    case 64: return tmarch_fn_v<64>(v, mode);
    case 256: return tmarch_fn_v<256>(v, mode);
    default: return tmarch_fn_v<128>(v, mode);
  }
}

int tmarch_smem_bytes(const PassArgs &a) { return (4 * a.tm_o + 2 * a.tm_a) * 4; }

bool tmarch_prepare(const Variant &v, int nt, int smem_bytes) {
  if (v.mask || v.pot == POT_PEAR) return false;  // built for unmasked LL and GHRL
  for (int mode : {MODE_SWEEP, MODE_SWEEP_MEASURE})
    if (cudaFuncSetAttribute(tmarch_kernel(v, mode, nt), cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes) !=
        cudaSuccess)
      return false;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, tmarch_kernel(v, MODE_SWEEP, nt), nt, smem_bytes) !=
      cudaSuccess)
    return false;
  return n > 0;
}

void launch_tmarch(const Variant &v, int mode, const PassArgs &a, int nt, bool pdl, cudaStream_t st) {
  if (v.mask || v.pot == POT_PEAR) return;  // never selected there (tmarch_prepare is false)
  PassArgs args = a;
  void *params[] = {&args};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(a.nunits);
  cfg.blockDim = dim3(nt);
  cfg.dynamicSmemBytes = tmarch_smem_bytes(a);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelExC(&cfg, tmarch_kernel(v, mode, nt), params);
}

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
