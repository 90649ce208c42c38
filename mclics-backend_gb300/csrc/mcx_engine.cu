// mcx_engine.cu -- the C ABI of include/mcx.h: a batch of replicas resident
// on one GB300, swept by the red/black kernels of mcx_kernels.cu, with the
// per-sweep sequence (pass 0, pass 1, [measure], epilogue) captured once into
// CUDA graphs of kChunk sweeps and replayed.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/mcx.h"
#include "mcx_device.cuh"
#include "mcx_host.h"
#include "mcx_kernels.cuh"

using namespace mcx;

namespace {
constexpr int kChunk = 16;     // sweeps per captured graph
constexpr int kRingCap = 512;  // measured sweeps buffered before the statistics are folded
std::string g_last_error;
}  // namespace

void mcx::set_last_error(const char *msg) { g_last_error = msg ? msg : ""; }

struct mcx_engine {
  int nrep = 0;
  std::vector<mcx_replica_desc> desc;
  std::vector<RepDev> rep;
  std::vector<int2> map;
  Variant var{};
  cudaStream_t stream = nullptr;
  RepDev *d_rep = nullptr;
  int2 *d_map = nullptr;
  float *d_dir = nullptr;
  uint8_t *d_pt = nullptr;
  float *d_ns = nullptr;
  RepState *d_st = nullptr;
  double *d_stats = nullptr;
  double *d_ring = nullptr;  // [nrep][ring_cap + 1][kLanes][kQ]
  int ring_cap = kRingCap;
  unsigned long long meas_flushed = 0;  // measured sweeps already folded into the stats
  int pending = 0;                      // measured sweeps waiting in the ring
  double *d_series = nullptr;
  int series_cap = 0;
  double *d_mout = nullptr;
  float *d_stage = nullptr;  // AoS staging, 3 * max sites floats
  int *d_stage_pt = nullptr;
  long long max_sites = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // [measure]
  long long launches = 0;
  std::string err;
  // staged (TMA) pass
  bool staged = false;      // sweeps use k_tpass
  bool can_stage = false;   // every replica fits a stage
  std::vector<int4> tiles;  // (replica, j0, k0, 0)
  int4 *d_tiles = nullptr;
  int stage_bytes = 0;
  int grid[2] = {0, 0};     // persistent CTAs of the staged pass for [measure]
  int pgrid[4] = {0, 0, 0, 0};  // persistent CTAs of the direct pass per PassMode
  unsigned *d_err = nullptr;
  // learned proposal
  int proposal = MCX_PROPOSAL_PLAIN;
  uint8_t *d_mlp = nullptr;
  std::vector<float> mlp;  // FP32 weights as last set or trained
  int lgrid[4] = {0, 0, 0, 0};
  // z-march pass (the default sweep pass of the plain proposal)
  bool march = true;
  int march_nt = 128, march_k = 8;
  bool pdl = true;  // programmatic dependent launch of the z-march passes
  bool tmarch = false;  // the z-march with rows staged by bulk copies (unmasked lattices)
  bool amarch = false;  // the z-march with a per-thread cp.async prefetch (unmasked LL / GHRL)
  bool pmarch = false;  // the z-march as one cooperative launch per run of sweeps (grid barriers)
  bool qmarch = false;  // the z-march with four sites per thread (unmasked, nx a multiple of 8)
  // per replica of a masked batch, row j + ny * k: 0 no active site, 1 only
  // bulk sites (point type 1), 2 anything else (empty: unknown)
  std::vector<std::vector<uint8_t>> rowact;
  // per replica of a masked batch cut into tiles (tiled[r]): the class (as
  // rowact) of row j + ny * k over the x range of tile column s, with the x
  // neighbours on either side: segact[r][(j + ny * k) * nseg + s]
  std::vector<std::vector<uint8_t>> segact;
  std::vector<char> tiled;
  bool defer_plan = false;  // mcx_create / mcx_load: masks uploaded first, units planned once after
  // learned-proposal z-march: its own units (128 pairs x kLearnPlanes planes)
  std::vector<int4> lunits;
  int4 *d_lunits = nullptr;
  bool lmarch_ok = false;
  bool ltc = false;  // the learned z-march's network on the tcgen05 tensor cores (else warp-level mma.sync)
  int tm_o = 0, tm_a = 0;  // its shared-memory slot sizes (floats)
  std::vector<int4> units;
  int4 *d_units = nullptr;
  long long dir_total = 0;  // floats of d_dir
  // training of the network: FP32 master weights, Adam moments, gradient
  float *d_w = nullptr, *d_am = nullptr, *d_av = nullptr, *d_g = nullptr, *d_loss = nullptr;
  bool w_stale = true;  // d_w does not hold e->mlp yet (Adam restarts)
  int adam_step = 0;
  float *d_samples = nullptr;
  long long sample_cap = 0;
  int *d_idx = nullptr, *d_repof = nullptr;
  long long idx_cap = 0, repof_cap = 0, loss_bytes = 0;
  int held_samples = 0;  // samples in d_samples (last collection or mcx_mlp_grad upload)
};

static void drop_graphs(mcx_engine *e);
static PassArgs pass_args(mcx_engine *e);
static bool use_tmarch(mcx_engine *e, bool on);
static bool qmarch_ok(const mcx_engine *e);
static mcx_status apply_march_shape(mcx_engine *e, int nt, int k);

static mcx_status fail(mcx_engine *e, mcx_status st, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (e) e->err = buf;
  else g_last_error = buf;
  return st;
}

#define CK(e, call)                                                                                   \
  do {                                                                                                \
    cudaError_t _r = (call);                                                                          \
    if (_r != cudaSuccess) return fail(e, MCX_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(_r));      \
  } while (0)

#define CKL(e)                                                                                        \
  do {                                                                                                \
    cudaError_t _r = cudaGetLastError();                                                              \
    if (_r != cudaSuccess) return fail(e, MCX_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(_r)); \
  } while (0)

static long long align_up(long long x, long long a) { return (x + a - 1) / a * a; }

// n / d == (n * m) >> p for every n < 2^31 with p = 31 + ceil(log2 d) and
// m = ceil(2^p / d), which fits in 32 bits (Granlund & Montgomery, PLDI'94).
static void div_magic(uint32_t d, uint32_t &m, int &p) {
  int L = 0;
  while ((1ull << L) < d) L++;
  p = 31 + L;
  m = (uint32_t)(((1ull << p) + d - 1) / d);
}

// Shared-memory bytes of one stage of the staged pass for a tj x tk tile.
static long long stage_bytes_for(const RepDev &R, int tj, int tk, bool mask) {
  const long long SA = (long long)tj * tk, SO = (long long)(tk + 2) * (tj + 2);
  long long b = 12LL * R.hs * (SA + SO);
  if (mask) b += (long long)R.hps * (SA + SO);
  return align_up(b, 128);
}

// Chooses the staged pass's tile (tj | ny, tk | nz): as many site pairs as a
// CTA's 256 threads can take twice over, weighted by the fraction of the
// stage that is the tile itself rather than its halo, within the budget.
static bool plan_tiles(RepDev &R, bool mask, long long budget) {
  double best = -1;
  int btj = 0, btk = 0;
  for (int tk = 1; tk <= R.nz; tk++) {
    if (R.nz % tk) continue;
    for (int tj = 1; tj <= R.ny; tj++) {
      if (R.ny % tj) continue;
      const long long pairs = (long long)tj * tk * R.hp;
      if (pairs > 1024) continue;
      if (stage_bytes_for(R, tj, tk, mask) > budget) continue;
      const double SA = (double)tj * tk, SO = (double)(tk + 2) * (tj + 2);
      const double score = (double)std::min<long long>(pairs, 2 * kBlock) * SA / (SA + SO);
      if (score > best) {
        best = score;
        btj = tj;
        btk = tk;
      }
    }
  }
  if (btj == 0) return false;
  R.tj = btj;
  R.tk = btk;
  R.ntj = R.ny / btj;
  R.ntile = R.ntj * (R.nz / btk);
  div_magic((uint32_t)btj, R.tj_m, R.tj_p);
  div_magic((uint32_t)R.ntj, R.ntj_m, R.ntj_p);
  return true;
}

extern "C" int mcx_version(void) { return 1; }

extern "C" const char *mcx_last_error(const mcx_engine *e) { return e ? e->err.c_str() : g_last_error.c_str(); }

void mcx::set_engine_error(mcx_engine *e, const char *msg) { e->err = msg ? msg : ""; }

extern "C" int mcx_num_replicas(const mcx_engine *e) { return e ? e->nrep : 0; }

extern "C" long long mcx_kernel_launches(const mcx_engine *e) { return e ? e->launches : 0; }

static void free_engine(mcx_engine *e) {
  if (!e) return;
  for (int m = 0; m < 2; m++)
    if (e->graph[m]) cudaGraphExecDestroy(e->graph[m]);
  cudaFree(e->d_rep);
  cudaFree(e->d_map);
  cudaFree(e->d_dir);
  cudaFree(e->d_pt);
  cudaFree(e->d_ns);
  cudaFree(e->d_st);
  cudaFree(e->d_ring);
  cudaFree(e->d_stats);
  cudaFree(e->d_series);
  cudaFree(e->d_mout);
  cudaFree(e->d_stage);
  cudaFree(e->d_stage_pt);
  cudaFree(e->d_tiles);
  cudaFree(e->d_err);
  cudaFree(e->d_mlp);
  cudaFree(e->d_units);
  cudaFree(e->d_lunits);
  cudaFree(e->d_w);
  cudaFree(e->d_am);
  cudaFree(e->d_av);
  cudaFree(e->d_g);
  cudaFree(e->d_loss);
  cudaFree(e->d_samples);
  cudaFree(e->d_idx);
  cudaFree(e->d_repof);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
}

extern "C" void mcx_destroy(mcx_engine *e) { free_engine(e); }

static mcx_status check_desc(const mcx_replica_desc &d, int r) {
  if (d.nx < 2 || d.ny < 1 || d.nz < 1) return fail(nullptr, MCX_ERR_INVALID, "replica %d: lattice %dx%dx%d too small", r, d.nx, d.ny, d.nz);
  if ((long long)d.nx * d.ny * d.nz >= (1LL << 31)) return fail(nullptr, MCX_ERR_INVALID, "replica %d: more than 2^31 sites", r);
  if (d.geometry < 0 || d.geometry > 3) return fail(nullptr, MCX_ERR_INVALID, "replica %d: bad geometry %d", r, d.geometry);
  if (d.potential < 0 || d.potential > 2) return fail(nullptr, MCX_ERR_INVALID, "replica %d: bad potential %d", r, d.potential);
  if (d.n_surfaces < 0 || d.n_surfaces > MCX_MAX_SURFACES) return fail(nullptr, MCX_ERR_INVALID, "replica %d: bad surface count %d", r, d.n_surfaces);
  for (int s = 0; s < d.n_surfaces; s++)
    if (d.anchoring[s] < 0 || d.anchoring[s] > 7) return fail(nullptr, MCX_ERR_INVALID, "replica %d: bad anchoring %d on surface %d", r, d.anchoring[s], s);
  if (d.geometry == MCX_GEO_SLAB && d.n_surfaces < 2) return fail(nullptr, MCX_ERR_INVALID, "replica %d: slab geometry needs 2 surfaces", r);
  if (d.geometry == MCX_GEO_SPHERE && d.n_surfaces < 1) return fail(nullptr, MCX_ERR_INVALID, "replica %d: sphere geometry needs 1 surface", r);
  return MCX_OK;
}

// Bounds as the geometry forces them (src/geometry_slab.cpp:23,
// src/geometry_sphere.cpp:19-21).  A periodic axis of odd length would make a
// site its own-colour neighbour, so red/black sweeps need even lengths on
// periodic axes; free axes may have any length (an odd nx is stored padded:
// odd_tail in mcx_pass.cuh).
static void effective_bounds(mcx_replica_desc &d) {
  if (d.geometry == MCX_GEO_SLAB) d.zbound = MCX_BOUND_FREE;
  if (d.geometry == MCX_GEO_SPHERE) d.xbound = d.ybound = d.zbound = MCX_BOUND_FREE;
}

// Work units of the z-march pass: per replica, blocks of march_nt pairs of a
// plane times chunks of march_k planes, chunk-major so that the CTAs resident
// together work on neighbouring planes.
//
// march_k > 0 fixes the chunk depth.  march_k <= 0 balances the chunks
// against the CTAs the GPU holds at once (SMs x resident CTAs of the kernel):
// the column blocks of all replicas are cut into chunks of near-equal depth
// (sizes differ by at most one plane) so that the units fill max(1, -march_k)
// waves, which keeps the last wave from running mostly idle.
// The class of a unit of a masked replica from its rows and planes and the
// rows and planes next to them: kUnitDead when none holds an active site,
// kUnitBulk when all hold bulk sites only, 0 otherwise.
static int unit_class(const mcx_engine *e, const int4 &u, int nt) {
  const std::vector<uint8_t> &act = e->rowact[u.x];
  if (act.empty()) return 0;
  const RepDev &R = e->rep[u.x];
  if (u.w & kUnitTiled) {  // the tile's rows, over its x range (segact), and the rows and planes next to them
    const std::vector<uint8_t> &seg = e->segact[u.x];
    const int nseg = (R.hp + kTileW - 1) / kTileW;
    const int j0 = u.y >> kTileQBits, sc = (u.y & ((1 << kTileQBits) - 1)) / kTileW;
    const int j1 = std::min(j0 + nt / kTileW, R.ny) - 1, nk = u.w & kUnitPlanes;
    unsigned seen = 0;
    for (int k = u.z - 1; k <= u.z + nk; k++) {
      int kk = k;
      if (kk < 0 || kk >= R.nz) {
        if (R.zb != BOUND_PERIODIC) continue;
        kk = (kk + R.nz) % R.nz;
      }
      for (int j = j0 - 1; j <= j1 + 1; j++) {
        int jj = j;
        if (jj < 0 || jj >= R.ny) {
          if (R.yb != BOUND_PERIODIC) continue;
          jj = (jj + R.ny) % R.ny;
        }
        seen |= 1u << seg[((size_t)jj + (size_t)R.ny * kk) * nseg + sc];
      }
    }
    return seen == 1u ? kUnitDead : (seen == 2u ? kUnitBulk : 0);
  }
  const int pend = std::min(u.y + nt, R.hp * R.ny);
  const int j0 = u.y / R.hp, j1 = (pend - 1) / R.hp, nk = u.w & kUnitPlanes;
  unsigned seen = 0;  // bit c: a row of class c
  for (int k = u.z - 1; k <= u.z + nk; k++) {
    int kk = k;
    if (kk < 0 || kk >= R.nz) {
      if (R.zb != BOUND_PERIODIC) continue;
      kk = (kk + R.nz) % R.nz;
    }
    for (int j = j0 - 1; j <= j1 + 1; j++) {
      int jj = j;
      if (jj < 0 || jj >= R.ny) {
        if (R.yb != BOUND_PERIODIC) continue;
        jj = (jj + R.ny) % R.ny;
      }
      seen |= 1u << act[(size_t)jj + (size_t)R.ny * kk];
    }
  }
  return seen == 1u ? kUnitDead : (seen == 2u ? kUnitBulk : 0);
}

// Site pairs of a plane per z-march work unit: one per thread, two per thread
// in the four-site form.
static int unit_pairs(const mcx_engine *e) { return e->qmarch ? 2 * e->march_nt : e->march_nt; }

static bool unit_dead(const mcx_engine *e, const int4 &u) { return unit_class(e, u, unit_pairs(e)) == kUnitDead; }

// Flags of the z-march units and of the learned z-march's units (which only
// use kUnitDead).
static void mark_dead_units(mcx_engine *e) {
  for (int4 &u : e->units) u.w = (u.w & (kUnitPlanes | kUnitTiled)) | unit_class(e, u, unit_pairs(e));
  for (int4 &u : e->lunits) {
    const int cls = unit_class(e, u, lmarch_block_threads());
    u.w = (u.w & kUnitPlanes) | (cls == kUnitDead ? kUnitDead : 0);
  }
}

// Plane runs of a replica for the z-march's chunks: maximal runs of planes k
// whose units can all be bulk units (every row of planes k-1..k+1 that exist
// holds bulk sites only) and runs of the other planes.  Chunks never straddle
// two runs, so the planes at a slab's surfaces get short chunks of their own
// and the rest of the replica runs the unmasked update.  One run for
// unmasked replicas and for the persistent form (all units in one wave).
static std::vector<int2> plane_runs(const mcx_engine *e, int r) {
  const RepDev &R = e->rep[r];
  const std::vector<uint8_t> &act = e->rowact[r];
  std::vector<int2> runs;
  if (act.empty() || e->pmarch) {
    runs.push_back(make_int2(0, R.nz));
    return runs;
  }
  std::vector<char> bulk(R.nz);
  for (int k = 0; k < R.nz; k++) {
    bool b = true;
    for (int j = 0; j < R.ny && b; j++) b = act[(size_t)j + (size_t)R.ny * k] == 1;
    bulk[k] = b;
  }
  auto eligible = [&](int k) {
    for (int d = -1; d <= 1; d++) {
      int kk = k + d;
      if (kk < 0 || kk >= R.nz) {
        if (R.zb != BOUND_PERIODIC) continue;
        kk = (kk + R.nz) % R.nz;
      }
      if (!bulk[kk]) return false;
    }
    return true;
  };
  int k0 = 0;
  for (int k = 1; k <= R.nz; k++)
    if (k == R.nz || eligible(k) != eligible(k0)) {
      runs.push_back(make_int2(k0, k));
      k0 = k;
    }
  return runs;
}

// Whether the z-march cuts replica r into tiles (kUnitTiled): a masked
// replica, some of whose rows cross the mask's edge, with rows at least two
// tiles wide; not for the persistent form (whose units must fit one wave) nor
// the four-site form (unmasked), nor an odd nx (phantom slots sit at the row
// ends).
static bool use_tiles(const mcx_engine *e, int r) {
  const RepDev &R = e->rep[r];
  return e->var.mask && !e->var.odd && !e->pmarch && !e->qmarch && r < (int)e->tiled.size() && e->tiled[r] &&
         R.hp >= 2 * kTileW && R.hp < (1 << kTileQBits) && R.ny < (1 << (30 - kTileQBits));  // (j0 << 12) | q0 fits
}

static void plan_march(mcx_engine *e) {
  e->units.clear();
  const int nt = e->march_nt, np = unit_pairs(e);
  double avg = 0.0;  // balanced: planes per unit
  const int march_k = e->pmarch ? 0 : e->march_k;
  if (march_k <= 0) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int per_sm = e->pmarch   ? pmarch_blocks_per_sm(e->var, nt)
                       : e->amarch ? amarch_blocks_per_sm(e->var, nt)
                       : e->qmarch ? qmarch_blocks_per_sm(e->var, nt)
                                   : march_blocks_per_sm(e->var, MODE_SWEEP, nt);
    // the persistent form needs every unit resident at once: one wave
    const long long slots = (long long)std::max(1, nsm) * std::max(1, per_sm) * (e->pmarch ? 1 : std::max(1, -e->march_k));
    // work: column blocks x planes, without the dead ones (no active site in or next to them),
    // which cost next to nothing; the persistent form counts every unit, all resident at once
    long long work = 0;
    for (int r = 0; r < e->nrep; r++) {
      const RepDev &R = e->rep[r];
      const int npp = R.hp * R.ny;
      if (use_tiles(e, r)) {
        for (int j0 = 0; j0 < R.ny; j0 += nt / kTileW)
          for (int q0 = 0; q0 < R.hp; q0 += kTileW)
            for (int k = 0; k < R.nz; k++)
              work += !unit_dead(e, make_int4(r, (j0 << kTileQBits) | q0, k, 1 | kUnitTiled)) ? 1 : 0;
        continue;
      }
      for (int p0 = 0; p0 < npp; p0 += np)
        for (int k = 0; k < R.nz; k++)
          work += e->pmarch || !unit_dead(e, make_int4(r, p0, k, 1)) ? 1 : 0;
    }
    avg = std::max(1.0, (double)work / (double)slots);
  }
  for (int r = 0; r < e->nrep; r++) {
    RepDev &R = e->rep[r];
    const int npp = R.hp * R.ny;
    R.mcta = 0;
    const bool tiles = use_tiles(e, r);
    // the units of one chunk of planes k0 .. k0 + nk - 1: NT consecutive pairs
    // of the plane, or tiles
    auto chunk = [&](int k0, int nk) {
      if (tiles) {
        for (int j0 = 0; j0 < R.ny; j0 += nt / kTileW)
          for (int q0 = 0; q0 < R.hp; q0 += kTileW) {
            e->units.push_back(make_int4(r, (j0 << kTileQBits) | q0, k0, nk | kUnitTiled));
            R.mcta++;
          }
        return;
      }
      for (int p0 = 0; p0 < npp; p0 += np) {
        e->units.push_back(make_int4(r, p0, k0, nk));
        R.mcta++;
      }
    };
    for (const int2 run : plane_runs(e, r)) {
      const int len = run.y - run.x;
      if (march_k > 0) {
        const int K = std::min(march_k, len);
        for (int k0 = run.x; k0 < run.y; k0 += K) chunk(k0, std::min(K, run.y - k0));
      } else {
        // rounded down, so that the units never exceed the waves asked for
        const int chunks = std::max(1, std::min(len, (int)std::floor(len / avg)));
        for (int q = 0; q < chunks; q++) {
          const int k0 = run.x + (int)((long long)q * len / chunks), k1 = run.x + (int)((long long)(q + 1) * len / chunks);
          chunk(k0, k1 - k0);
        }
      }
    }
  }
  mark_dead_units(e);
}

extern "C" mcx_status mcx_create(int n, const mcx_replica_desc *descs, mcx_engine **out) {
  if (!out || !descs || n <= 0) return fail(nullptr, MCX_ERR_INVALID, "mcx_create: need n > 0 descriptors and an output pointer");
  *out = nullptr;
  for (int r = 0; r < n; r++) {
    mcx_status st = check_desc(descs[r], r);
    if (st) return st;
    if (descs[r].potential != descs[0].potential)
      return fail(nullptr, MCX_ERR_UNSUPPORTED, "all replicas of one engine must use the same pair potential");
    mcx_replica_desc d = descs[r];
    effective_bounds(d);
    if ((d.xbound == MCX_BOUND_PERIODIC && d.nx % 2) || (d.ybound == MCX_BOUND_PERIODIC && d.ny % 2) ||
        (d.zbound == MCX_BOUND_PERIODIC && d.nz % 2))
      return fail(nullptr, MCX_ERR_UNSUPPORTED,
                  "replica %d: lattice %dx%dx%d has an odd periodic axis; red/black sweeps need even lengths on "
                  "periodic axes (odd lengths are supported on free axes)",
                  r, d.nx, d.ny, d.nz);
  }
  mcx_engine *e = new mcx_engine();
  e->nrep = n;
  e->desc.assign(descs, descs + n);
  e->var.pot = descs[0].potential;
  e->var.mask = false;
  e->var.field = false;
  e->var.per = true;
  long long dir_total = 0, pt_total = 0;
  e->rep.resize(n);
  e->rowact.resize(n);
  e->segact.resize(n);
  e->tiled.assign(n, 0);
  for (int r = 0; r < n; r++) {
    mcx_replica_desc &d = e->desc[r];
    effective_bounds(d);
    RepDev &R = e->rep[r];
    memset(&R, 0, sizeof R);
    R.nx = d.nx;
    R.ny = d.ny;
    R.nz = d.nz;
    R.hx = (d.nx + 1) / 2;  // odd nx: one padding slot per row (odd_tail)
    R.hs = (int)align_up(R.hx, 4);
    R.xb = d.xbound;
    R.yb = d.ybound;
    R.zb = d.zbound;
    R.nsurf = d.n_surfaces;
    R.ntot = d.nx * d.ny * d.nz;
    R.plane = R.hs * d.ny * d.nz;
    R.hp = (R.hx + 1) / 2;
    R.npair = R.hp * d.ny * d.nz;
    div_magic((uint32_t)R.hp, R.hp_m, R.hp_p);
    div_magic((uint32_t)d.ny, R.ny_m, R.ny_p);
    R.dir_off = dir_total;
    dir_total += align_up(6LL * R.plane, 64);
    R.hps = (int)align_up(R.hs, 16);
    R.pplane = R.hps * d.ny * d.nz;
    R.pt_off = pt_total;
    pt_total += align_up(2LL * R.pplane, 256);
    R.A = d.A;
    R.elecA = d.elecA;
    R.elecE = d.elecE;
    R.ex = d.elecX;
    R.ey = d.elecY;
    R.ez = d.elecZ;
    float g[5] = {0, 0, 1, 0, 0};
    if (d.potential == MCX_POT_GHRL) ghrl_constants(d.k11, d.k22, d.k33, d.p0, g);
    R.B1 = d.B1;
    R.C = d.C;
    R.lam = g[0];
    R.mu = g[1];
    R.nu = g[2];
    R.rho = g[3];
    R.sigma = g[4];
    R.ga = 1.5f * R.rho;
    R.gb = R.lam - 0.5f * R.rho;
    R.gc = 1.5f * R.nu;
    R.gconst = d.potential == MCX_POT_GHRL ? -0.5f * R.nu - R.mu / 9.0f : 0.0f;
    R.seed = d.seed;
    R.stream = d.stream;
    for (int s = 0; s < d.n_surfaces; s++) {
      R.anch[s] = d.anchoring[s];
      R.W[s] = d.W[s];
      float ax[3];
      anchoring_axis(d.theta_s[s], d.phi_s[s], ax);
      R.dx[s] = ax[0];
      R.dy[s] = ax[1];
      R.dz[s] = ax[2];
    }
    // an odd nx needs the mask: its padding slots are inactive sites
    if (d.geometry != MCX_GEO_BULK || d.nx % 2) e->var.mask = true;
    if (d.nx % 2) e->var.odd = true;
    if (d.xbound != MCX_BOUND_PERIODIC || d.ybound != MCX_BOUND_PERIODIC || d.zbound != MCX_BOUND_PERIODIC ||
        d.nx % 4 != 0)
      e->var.per = false;
    if (d.elecA != 0.f) e->var.field = true;
    e->max_sites = std::max(e->max_sites, (long long)R.ntot);
    R.ncta = 0;
    for (long long b = 0; b < R.npair; b += pass_block_threads()) {
      e->map.push_back(make_int2(r, (int)b));
      R.ncta++;
    }
  }
  if (e->var.mask) e->var.per = false;
  for (int r = 0; r < n; r++) e->rep[r].ns_off = e->var.mask ? e->rep[r].dir_off : -1;
  {
    const char *nt = getenv("MCX_MARCH_NT"), *kk = getenv("MCX_MARCH_K"), *mo = getenv("MCX_MARCH");
    if (nt && march_block_ok(atoi(nt))) e->march_nt = atoi(nt);
    if (kk && atoi(kk) > 0) e->march_k = atoi(kk);
    if (mo && atoi(mo) == 0) e->march = false;
    const char *pd = getenv("MCX_PDL");
    if (pd && atoi(pd) == 0) e->pdl = false;
    plan_march(e);
  }
  {
    const char *kb = getenv("MCX_STAGE_KB");
    const long long budget = (kb ? atoll(kb) : 40) * 1024;
    e->can_stage = true;
    // the staged pass does not handle the padding slots of an odd nx
    for (int r = 0; r < n; r++)
      if (e->rep[r].nx % 2) e->can_stage = false;
    for (int r = 0; r < n && e->can_stage; r++) {
      RepDev &R = e->rep[r];
      if (!plan_tiles(R, e->var.mask, budget)) {
        e->can_stage = false;
        break;
      }
      R.tile0 = (int)e->tiles.size();
      for (int kb2 = 0; kb2 < R.nz / R.tk; kb2++)
        for (int jb = 0; jb < R.ntj; jb++) e->tiles.push_back(make_int4(r, jb * R.tj, kb2 * R.tk, 0));
      e->stage_bytes = (int)std::max<long long>(e->stage_bytes, stage_bytes_for(R, R.tj, R.tk, e->var.mask));
    }
    // the direct pass measures faster on every lattice tried so far; the
    // staged pass is opt-in (mcx_set_staged or MCX_STAGED=1)
    const char *st = getenv("MCX_STAGED");
    e->staged = e->can_stage && st && atoi(st) == 1;
  }
  mcx_status st = MCX_OK;
#define CKC(call)                                                                                  \
  do {                                                                                             \
    cudaError_t _r = (call);                                                                       \
    if (_r != cudaSuccess) {                                                                       \
      st = fail(nullptr, _r == cudaErrorMemoryAllocation ? MCX_ERR_NOMEM : MCX_ERR_CUDA, "%s: %s", #call, \
                cudaGetErrorString(_r));                                                           \
      free_engine(e);                                                                              \
      return st;                                                                                   \
    }                                                                                              \
  } while (0)
  CKC(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
  e->dir_total = dir_total;
  CKC(cudaMalloc(&e->d_dir, sizeof(float) * dir_total));
  CKC(cudaMemsetAsync(e->d_dir, 0, sizeof(float) * dir_total, e->stream));
  if (e->var.mask) {
    CKC(cudaMalloc(&e->d_pt, pt_total));
    CKC(cudaMemsetAsync(e->d_pt, 0, pt_total, e->stream));
    CKC(cudaMalloc(&e->d_ns, sizeof(float) * dir_total));
    CKC(cudaMemsetAsync(e->d_ns, 0, sizeof(float) * dir_total, e->stream));
  }
  CKC(cudaMalloc(&e->d_units, sizeof(int4) * e->units.size()));
  CKC(cudaMemcpyAsync(e->d_units, e->units.data(), sizeof(int4) * e->units.size(), cudaMemcpyHostToDevice, e->stream));
  CKC(cudaMalloc(&e->d_rep, sizeof(RepDev) * n));
  CKC(cudaMalloc(&e->d_map, sizeof(int2) * e->map.size()));
  CKC(cudaMalloc(&e->d_st, sizeof(RepState) * n));
  const size_t ring_n = (size_t)n * (e->ring_cap + 1) * kLanes * kQ;
  CKC(cudaMalloc(&e->d_ring, sizeof(double) * ring_n));
  CKC(cudaMemsetAsync(e->d_ring, 0, sizeof(double) * ring_n, e->stream));
  CKC(cudaMalloc(&e->d_stats, sizeof(double) * kStats * n));
  CKC(cudaMemsetAsync(e->d_stats, 0, sizeof(double) * kStats * n, e->stream));
  CKC(cudaMalloc(&e->d_mout, sizeof(double) * 16 * n));
  CKC(cudaMalloc(&e->d_err, 2 * sizeof(unsigned)));  // the error flag, then the grid-barrier counter
  CKC(cudaMemsetAsync(e->d_err, 0, 2 * sizeof(unsigned), e->stream));
  {
    int dev = 0, nsm = 0;
    CKC(cudaGetDevice(&dev));
    CKC(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    for (int m = 0; m < 4; m++) {
      const int per = pass_blocks_per_sm(e->var, m);
      if (per <= 0) {
        st = fail(nullptr, MCX_ERR_CUDA, "direct pass kernel cannot be resident (occupancy 0)");
        free_engine(e);
        return st;
      }
      e->pgrid[m] = (int)std::min<long long>((long long)per * nsm, (long long)e->map.size());
    }
  }
  if (e->can_stage) {
    CKC(cudaMalloc(&e->d_tiles, sizeof(int4) * e->tiles.size()));
    CKC(cudaMemcpyAsync(e->d_tiles, e->tiles.data(), sizeof(int4) * e->tiles.size(), cudaMemcpyHostToDevice, e->stream));
    int dev = 0, nsm = 0;
    CKC(cudaGetDevice(&dev));
    CKC(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    for (int m = 0; m < 2; m++) {
      const int per = tpass_blocks_per_sm(e->var, m ? MODE_SWEEP_MEASURE : MODE_SWEEP, e->stage_bytes);
      e->grid[m] = std::min<long long>((long long)per * nsm, (long long)e->tiles.size());
      if (per <= 0) e->can_stage = e->staged = false;
    }
    // the trace specialisation (parity checks) needs the same shared-memory opt-in
    if (e->can_stage && tpass_blocks_per_sm(e->var, MODE_TRACE, e->stage_bytes) <= 0) e->can_stage = e->staged = false;
  }
  CKC(cudaMalloc(&e->d_stage, sizeof(float) * 3 * e->max_sites));
  CKC(cudaMalloc(&e->d_stage_pt, sizeof(int) * e->max_sites));
  CKC(cudaMemcpyAsync(e->d_map, e->map.data(), sizeof(int2) * e->map.size(), cudaMemcpyHostToDevice, e->stream));
  // masks: valid counts first (they go into RepDev)
  std::vector<int> pt;
  std::vector<float> ns;
  for (int r = 0; r < n; r++) {
    RepDev &R = e->rep[r];
    build_mask(e->desc[r], pt, ns);  // custom geometry starts as all-bulk until mcx_set_mask
    long v = 0;
    for (int x : pt) v += x != 0;
    R.valid = (int)v;
  }
  CKC(cudaMemcpyAsync(e->d_rep, e->rep.data(), sizeof(RepDev) * n, cudaMemcpyHostToDevice, e->stream));
  std::vector<RepState> hs(n);
  for (int r = 0; r < n; r++) {
    memset(&hs[r], 0, sizeof(RepState));
    hs[r].T = e->desc[r].T;
    hs[r].ang_var = e->desc[r].ang_var > 0 ? e->desc[r].ang_var : 0.5f;
  }
  CKC(cudaMemcpyAsync(e->d_st, hs.data(), sizeof(RepState) * n, cudaMemcpyHostToDevice, e->stream));
  CKC(cudaStreamSynchronize(e->stream));
  e->defer_plan = true;
  for (int r = 0; r < n; r++) {
    if (e->var.mask) {
      build_mask(e->desc[r], pt, ns);
      st = mcx_set_mask(e, r, pt.data(), ns.data());
      if (st) {
        g_last_error = e->err;
        free_engine(e);
        return st;
      }
    }
    st = mcx_init_homogeneous(e, r, 0.f, 0.f);
    if (st) {
      g_last_error = e->err;
      free_engine(e);
      return st;
    }
  }
  e->defer_plan = false;
  if (e->var.mask) {
    st = apply_march_shape(e, e->march_nt, e->march_k);
    if (st) {
      g_last_error = e->err;
      free_engine(e);
      return st;
    }
  }
  CKC(cudaStreamSynchronize(e->stream));
#undef CKC
  *out = e;
  return MCX_OK;
}

static mcx_status check_rep(mcx_engine *e, int r) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (r < 0 || r >= e->nrep) return fail(e, MCX_ERR_INVALID, "replica %d out of range [0, %d)", r, e->nrep);
  return MCX_OK;
}

extern "C" mcx_status mcx_get_desc(const mcx_engine *ce, int r, mcx_replica_desc *d, float *ghrl) {
  mcx_engine *e = const_cast<mcx_engine *>(ce);
  if (mcx_status st = check_rep(e, r)) return st;
  if (d) *d = e->desc[r];
  if (ghrl) {
    const RepDev &R = e->rep[r];
    ghrl[0] = R.lam;
    ghrl[1] = R.mu;
    ghrl[2] = R.nu;
    ghrl[3] = R.rho;
    ghrl[4] = R.sigma;
  }
  return MCX_OK;
}

extern "C" mcx_status mcx_set_state(mcx_engine *e, int r, const float *ni) {
  if (mcx_status st = check_rep(e, r)) return st;
  if (!ni) return fail(e, MCX_ERR_INVALID, "null director array");
  const RepDev &R = e->rep[r];
  CK(e, cudaMemcpyAsync(e->d_stage, ni, sizeof(float) * 3 * R.ntot, cudaMemcpyHostToDevice, e->stream));
  launch_aos_to_split(R, e->d_stage, e->d_dir, e->stream);
  CKL(e);
  CK(e, cudaStreamSynchronize(e->stream));
  return MCX_OK;
}

extern "C" mcx_status mcx_get_state(mcx_engine *e, int r, float *ni) {
  if (mcx_status st = check_rep(e, r)) return st;
  if (!ni) return fail(e, MCX_ERR_INVALID, "null director array");
  const RepDev &R = e->rep[r];
  launch_split_to_aos(R, e->d_dir, e->d_stage, e->stream);
  CKL(e);
  CK(e, cudaMemcpyAsync(ni, e->d_stage, sizeof(float) * 3 * R.ntot, cudaMemcpyDeviceToHost, e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  return MCX_OK;
}

extern "C" mcx_status mcx_init_random(mcx_engine *e, int r, unsigned int seed) {
  if (mcx_status st = check_rep(e, r)) return st;
  launch_init(e->rep[r], e->d_pt, e->d_dir, 0, seed, 0.f, 0.f, 1.f, e->stream);
  CKL(e);
  CK(e, cudaStreamSynchronize(e->stream));
  return MCX_OK;
}

extern "C" mcx_status mcx_init_homogeneous(mcx_engine *e, int r, float theta_0, float phi_0) {
  if (mcx_status st = check_rep(e, r)) return st;
  // src/ic.cpp:77-79 (double math, stored as float)
  const float fx = (float)(sin(theta_0 * M_PI / 180) * cos(phi_0 * M_PI / 180));
  const float fy = (float)(sin(theta_0 * M_PI / 180) * sin(phi_0 * M_PI / 180));
  const float fz = (float)cos(theta_0 * M_PI / 180);
  launch_init(e->rep[r], e->d_pt, e->d_dir, 1, 0, fx, fy, fz, e->stream);
  CKL(e);
  CK(e, cudaStreamSynchronize(e->stream));
  return MCX_OK;
}

extern "C" mcx_status mcx_set_mask(mcx_engine *e, int r, const int *pt, const float *ns) {
  if (mcx_status st = check_rep(e, r)) return st;
  if (!pt) return fail(e, MCX_ERR_INVALID, "null point-type array");
  RepDev &R = e->rep[r];
  long v = 0;
  for (long s = 0; s < R.ntot; s++) {
    if (pt[s] < 0 || pt[s] > 255) return fail(e, MCX_ERR_INVALID, "point type %d at site %ld out of [0, 255]", pt[s], s);
    if (pt[s] > 1 && pt[s] - 2 >= R.nsurf)
      return fail(e, MCX_ERR_INVALID, "point type %d at site %ld names surface %d but the replica has %d", pt[s], s, pt[s] - 2, R.nsurf);
    v += pt[s] != 0;
  }
  if (!e->var.mask) {
    bool all_bulk = true;
    for (long s = 0; s < R.ntot && all_bulk; s++) all_bulk = pt[s] == 1;
    if (all_bulk) return MCX_OK;
    return fail(e, MCX_ERR_UNSUPPORTED, "engine was created without masks (all replicas bulk); create it with a non-bulk geometry");
  }
  if (v == 0) return fail(e, MCX_ERR_INVALID, "mask has no active site");
  CK(e, cudaMemcpyAsync(e->d_stage_pt, pt, sizeof(int) * R.ntot, cudaMemcpyHostToDevice, e->stream));
  if (ns) CK(e, cudaMemcpyAsync(e->d_stage, ns, sizeof(float) * 3 * R.ntot, cudaMemcpyHostToDevice, e->stream));
  launch_mask_to_split(R, e->d_stage_pt, ns ? e->d_stage : nullptr, e->d_pt, e->d_ns, e->stream);
  CKL(e);
  R.valid = (int)v;
  CK(e, cudaMemcpyAsync(&e->d_rep[r].valid, &R.valid, sizeof(int), cudaMemcpyHostToDevice, e->stream));
  // which rows hold an active site: z-march units far from every one skip their updates
  std::vector<uint8_t> &act = e->rowact[r];
  act.assign((size_t)R.ny * R.nz, 0);
  for (long row = 0; row < (long)R.ny * R.nz; row++) {
    bool any = false, bulk = true;
    for (int i = 0; i < R.nx; i++) {
      any |= pt[row * R.nx + i] != 0;
      bulk &= pt[row * R.nx + i] == 1;
    }
    // an odd-nx row also holds a padding slot (inactive): never a bulk row
    act[row] = bulk && R.nx % 2 == 0 ? 1 : (any ? 2 : 0);
  }
  // rows that cross the mask's edge (active and inactive sites): cut the
  // replica into tiles, classed over each tile column's x range (with the x
  // neighbours on either side)
  {
    bool mixed = false;
    for (long row = 0; row < (long)R.ny * R.nz && !mixed; row++) {
      bool any = false, none = false;
      for (int i = 0; i < R.nx; i++) (pt[row * R.nx + i] != 0 ? any : none) = true;
      mixed = any && none;
    }
    e->tiled[r] = mixed;
    std::vector<uint8_t> &seg = e->segact[r];
    seg.clear();
    if (mixed) {
      const int nseg = (R.hp + kTileW - 1) / kTileW, w = 4 * kTileW;  // x sites per tile column
      seg.assign((size_t)R.ny * R.nz * nseg, 0);
      for (long row = 0; row < (long)R.ny * R.nz; row++)
        for (int sc = 0; sc < nseg; sc++) {
          bool any = false, bulk = true;
          for (int x = sc * w - 1; x <= (sc + 1) * w; x++) {
            int xx = x;
            if (xx < 0 || xx >= R.nx) {
              if (R.xb != BOUND_PERIODIC) continue;
              xx = (xx + R.nx) % R.nx;
            }
            any |= pt[row * R.nx + xx] != 0;
            bulk &= pt[row * R.nx + xx] == 1;
          }
          seg[(size_t)row * nseg + sc] = bulk && R.nx % 2 == 0 ? 1 : (any ? 2 : 0);
        }
    }
  }
  // the z-march's chunks follow the mask's plane runs: plan them again (in
  // mcx_create and mcx_load once, after every replica's mask)
  if (e->defer_plan) {
    mark_dead_units(e);
  } else if (mcx_status st = apply_march_shape(e, e->march_nt, e->march_k)) {
    return st;
  }
  if (e->d_lunits && !e->lunits.empty())
    CK(e, cudaMemcpyAsync(e->d_lunits, e->lunits.data(), sizeof(int4) * e->lunits.size(), cudaMemcpyHostToDevice,
                          e->stream));
  drop_graphs(e);
  CK(e, cudaStreamSynchronize(e->stream));
  return MCX_OK;
}

extern "C" mcx_status mcx_get_mask(mcx_engine *e, int r, int *pt, float *ns) {
  if (mcx_status st = check_rep(e, r)) return st;
  const RepDev &R = e->rep[r];
  float *dns = e->d_stage;
  launch_split_to_mask(R, e->d_pt, e->d_ns, e->d_stage_pt, dns, e->stream);
  CKL(e);
  if (pt) CK(e, cudaMemcpyAsync(pt, e->d_stage_pt, sizeof(int) * R.ntot, cudaMemcpyDeviceToHost, e->stream));
  if (ns) CK(e, cudaMemcpyAsync(ns, dns, sizeof(float) * 3 * R.ntot, cudaMemcpyDeviceToHost, e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  return MCX_OK;
}

template <typename T>
static mcx_status set_scalar(mcx_engine *e, int r, size_t off, T v, bool in_rep) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  const int r0 = r < 0 ? 0 : r, r1 = r < 0 ? e->nrep : r + 1;
  if (r >= e->nrep) return fail(e, MCX_ERR_INVALID, "replica %d out of range", r);
  for (int q = r0; q < r1; q++) {
    char *base = in_rep ? (char *)(e->d_rep + q) : (char *)(e->d_st + q);
    CK(e, cudaMemcpyAsync(base + off, &v, sizeof(T), cudaMemcpyHostToDevice, e->stream));
  }
  CK(e, cudaStreamSynchronize(e->stream));
  return MCX_OK;
}

extern "C" mcx_status mcx_set_temperature(mcx_engine *e, int r, float T) {
  mcx_status st = set_scalar(e, r, offsetof(RepState, T), T, false);
  if (!st && e)
    for (int q = (r < 0 ? 0 : r); q < (r < 0 ? e->nrep : r + 1); q++) e->desc[q].T = T;
  return st;
}

extern "C" mcx_status mcx_set_field(mcx_engine *e, int r, float E) {
  if (e && !e->var.field) {
    bool any = false;
    for (int q = 0; q < e->nrep; q++) any |= e->desc[q].elecA != 0.f;
    if (!any) return fail(e, MCX_ERR_UNSUPPORTED, "engine has no field term (elecA = 0 on every replica)");
  }
  mcx_status st = set_scalar(e, r, offsetof(RepDev, elecE), E, true);
  if (!st && e)
    for (int q = (r < 0 ? 0 : r); q < (r < 0 ? e->nrep : r + 1); q++) {
      e->desc[q].elecE = E;
      e->rep[q].elecE = E;
    }
  return st;
}

extern "C" mcx_status mcx_set_step(mcx_engine *e, int r, float a) {
  return set_scalar(e, r, offsetof(RepState, ang_var), a, false);
}

extern "C" mcx_status mcx_set_adapt(mcx_engine *e, int r, int on) {
  return set_scalar(e, r, offsetof(RepState, frozen), on ? 0u : 1u, false);
}

static PassArgs pass_args(mcx_engine *e) {
  PassArgs pa{};
  pa.reps = e->d_rep;
  pa.map = e->d_map;
  pa.dir = e->d_dir;
  pa.pt = e->d_pt;
  pa.ns = e->d_ns;
  pa.st = e->d_st;
  pa.stats = e->d_stats;
  pa.ring = e->d_ring;
  pa.ring_cap = e->ring_cap;
  pa.nmap = (int)e->map.size();
  pa.mlp = e->d_mlp;
  pa.tiles = e->d_tiles;
  pa.ntiles = (int)e->tiles.size();
  pa.stage_bytes = e->stage_bytes;
  pa.err = e->d_err;
  pa.units = e->d_units;
  pa.nunits = (int)e->units.size();
  pa.tm_o = e->tm_o;
  pa.tm_a = e->tm_a;
  return pa;
}

// One red/black pass of every replica, staged or direct.
static void launch_sweep_pass(mcx_engine *e, PassArgs &pa, int colour, bool measure) {
  pa.colour = colour;
  int mode = measure ? MODE_SWEEP_MEASURE : MODE_SWEEP;
  // the plain z-march of an unmasked batch (register, prefetching and
  // four-site forms) measures both colours in its colour-1 pass
  // (PassArgs::meas_both)
  const bool both = e->proposal == MCX_PROPOSAL_PLAIN && !e->staged && e->march && !e->tmarch && !e->var.mask;
  pa.meas_both = measure && both ? 1 : 0;
  if (measure && both && colour == 0) mode = MODE_SWEEP;
  if (e->proposal == MCX_PROPOSAL_VMF_MLP) {
    if (e->march && e->lmarch_ok) {
      pa.units = e->d_lunits;
      pa.nunits = (int)e->lunits.size();
      launch_lmarch(e->var, mode, pa, e->pdl, e->ltc, e->stream);
    } else {
      launch_pass_learned(e->var, mode, pa, e->lgrid[mode], e->stream);
    }
  } else if (e->staged) launch_tpass(e->var, mode, pa, e->grid[measure ? 1 : 0], e->stream);
  else if (e->march && e->tmarch) launch_tmarch(e->var, mode, pa, e->march_nt, e->pdl, e->stream);
  else if (e->march && e->amarch) launch_amarch(e->var, mode, pa, e->march_nt, e->pdl, e->stream);
  else if (e->march && e->qmarch) launch_qmarch(e->var, mode, pa, e->march_nt, e->pdl, e->stream);
  else if (e->march) launch_march(e->var, mode, pa, e->march_nt, e->pdl, e->stream);
  else launch_pass(e->var, mode, pa, e->pgrid[mode], e->stream);
}

// One sweep's kernels on e->stream: the two colours.
static void enqueue_sweep(mcx_engine *e, bool measure) {
  PassArgs pa = pass_args(e);
  for (int c = 0; c < 2; c++) launch_sweep_pass(e, pa, c, measure);
}

static mcx_status build_graph(mcx_engine *e, int measure) {
  cudaGraph_t g;
  CK(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
  for (int s = 0; s < kChunk; s++) enqueue_sweep(e, measure != 0);
  cudaError_t lr = cudaGetLastError();
  cudaError_t r = cudaStreamEndCapture(e->stream, &g);
  if (lr != cudaSuccess) return fail(e, MCX_ERR_CUDA, "capture: %s", cudaGetErrorString(lr));
  if (r != cudaSuccess) return fail(e, MCX_ERR_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(r));
  r = cudaGraphInstantiate(&e->graph[measure], g, 0);
  cudaGraphDestroy(g);
  if (r != cudaSuccess) return fail(e, MCX_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(r));
  return MCX_OK;
}

// Folds the measured sweeps waiting in the ring into the running sums.
static mcx_status flush(mcx_engine *e) {
  if (e->pending == 0) return MCX_OK;
  FlushArgs f{e->d_rep, e->d_ring, e->ring_cap, e->d_stats, e->d_series, e->series_cap, e->meas_flushed, e->pending};
  launch_flush(f, e->nrep, e->stream);
  e->launches += 1;
  CKL(e);
  e->meas_flushed += (unsigned long long)e->pending;
  e->pending = 0;
  return MCX_OK;
}

// Sweeps per cooperative launch of the persistent z-march (keeps its barrier
// counter, 2 x sweeps x CTAs, far from 32-bit overflow).
constexpr int kPersistentSweeps = 4096;

// The persistent form's units must all be resident at once (a cooperative
// launch of more CTAs than the GPU holds fails).
static bool pmarch_fits(const mcx_engine *e) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return (long long)e->units.size() <= (long long)nsm * pmarch_blocks_per_sm(e->var, e->march_nt);
}

static bool persistent(const mcx_engine *e) {
  return e->pmarch && e->march && !e->staged && e->proposal == MCX_PROPOSAL_PLAIN;
}

static mcx_status run_sweeps(mcx_engine *e, int n, int m) {
  if (persistent(e) && pmarch_fits(e)) {  // otherwise the register march below (the same update)
    PassArgs pa = pass_args(e);
    for (int done = 0; done < n;) {
      const int k = std::min(n - done, kPersistentSweeps);
      CK(e, launch_pmarch(e->var, m ? MODE_SWEEP_MEASURE : MODE_SWEEP, pa, e->march_nt, k, e->d_err + 1, e->stream));
      e->launches += 1;
      done += k;
    }
    return MCX_OK;
  }
  if (n >= kChunk && !e->graph[m]) {
    if (mcx_status st = build_graph(e, m)) return st;
  }
  int done = 0;
  while (n - done >= kChunk) {
    CK(e, cudaGraphLaunch(e->graph[m], e->stream));
    e->launches += 2 * kChunk;
    done += kChunk;
  }
  for (; done < n; done++) {
    enqueue_sweep(e, m != 0);
    e->launches += 2;
  }
  CKL(e);
  return MCX_OK;
}

extern "C" mcx_status mcx_sweep(mcx_engine *e, int n, int measure) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (n < 0) return fail(e, MCX_ERR_INVALID, "negative sweep count");
  if (!measure) return run_sweeps(e, n, 0);
  while (n > 0) {
    const int chunk = std::min(n, e->ring_cap - e->pending);
    if (mcx_status st = run_sweeps(e, chunk, 1)) return st;
    e->pending += chunk;
    n -= chunk;
    if (e->pending == e->ring_cap)
      if (mcx_status st = flush(e)) return st;
  }
  return MCX_OK;
}

// Reads (and clears) the staged pass's timeout flag after a synchronisation.
static mcx_status check_err_flag(mcx_engine *e) {
  unsigned f = 0;
  CK(e, cudaMemcpy(&f, e->d_err, sizeof f, cudaMemcpyDeviceToHost));
  if (f) {
    CK(e, cudaMemset(e->d_err, 0, sizeof f));
    if (f & 2u)
      return fail(e, MCX_ERR_CUDA, "persistent z-march: a grid barrier was not reached in time; results are invalid");
    if (f & 4u)
      return fail(e, MCX_ERR_CUDA, "tensor-core network: an MMA did not complete in time; results are invalid");
    return fail(e, MCX_ERR_CUDA, "staged pass: a shared-memory tile copy did not complete in time; results are invalid");
  }
  return MCX_OK;
}

extern "C" mcx_status mcx_sync(mcx_engine *e) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  CK(e, cudaStreamSynchronize(e->stream));
  return check_err_flag(e);
}

extern "C" mcx_status mcx_set_pass(mcx_engine *e, int kind) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (kind < MCX_PASS_MARCH || kind > MCX_PASS_MARCH_QUAD)
    return fail(e, MCX_ERR_INVALID, "unknown pass kernel %d", kind);
  if (kind == MCX_PASS_STAGED && !e->can_stage)
    return fail(e, MCX_ERR_UNSUPPORTED, "a replica's rows do not fit the staged pass's shared memory");
  CK(e, cudaStreamSynchronize(e->stream));
  if (kind == MCX_PASS_MARCH_TMA && !use_tmarch(e, true))
    return fail(e, MCX_ERR_UNSUPPORTED, "the TMA-staged z-march needs an unmasked batch whose rows fit in shared memory");
  if (kind == MCX_PASS_MARCH_ASYNC && !amarch_prepare(e->var, e->march_nt))
    return fail(e, MCX_ERR_UNSUPPORTED, "the prefetching z-march needs an unmasked LL or GHRL batch");
  if (kind == MCX_PASS_MARCH_PERSISTENT && !pmarch_block_ok(e->march_nt))
    return fail(e, MCX_ERR_UNSUPPORTED, "the persistent z-march runs blocks of 128 or 256 threads");
  if (kind == MCX_PASS_MARCH_QUAD && !qmarch_ok(e))
    return fail(e, MCX_ERR_UNSUPPORTED, "the four-site z-march needs an unmasked batch with nx a multiple of 8");
  if (kind != MCX_PASS_MARCH_TMA) e->tmarch = false;
  e->amarch = kind == MCX_PASS_MARCH_ASYNC;
  e->qmarch = kind == MCX_PASS_MARCH_QUAD;
  e->pmarch = kind == MCX_PASS_MARCH_PERSISTENT;
  e->staged = kind == MCX_PASS_STAGED;
  e->march = kind == MCX_PASS_MARCH || kind == MCX_PASS_MARCH_TMA || kind == MCX_PASS_MARCH_ASYNC ||
             kind == MCX_PASS_MARCH_PERSISTENT || kind == MCX_PASS_MARCH_QUAD;
  if (e->march) {
    if (mcx_status st = apply_march_shape(e, e->march_nt, e->march_k)) return st;  // chunks follow the form's residency
    if (e->pmarch && !pmarch_fits(e)) {
      e->pmarch = false;
      apply_march_shape(e, e->march_nt, e->march_k);
      return fail(e, MCX_ERR_UNSUPPORTED, "the persistent z-march needs every work unit resident at once; this batch has more column blocks than the GPU holds CTAs");
    }
    return MCX_OK;
  }
  drop_graphs(e);
  return MCX_OK;
}

extern "C" int mcx_get_pass(const mcx_engine *e) {
  if (!e) return -1;
  if (e->staged) return MCX_PASS_STAGED;
  if (!e->march) return MCX_PASS_DIRECT;
  if (e->pmarch) return MCX_PASS_MARCH_PERSISTENT;
  if (e->qmarch) return MCX_PASS_MARCH_QUAD;
  return e->tmarch ? MCX_PASS_MARCH_TMA : (e->amarch ? MCX_PASS_MARCH_ASYNC : MCX_PASS_MARCH);
}

extern "C" mcx_status mcx_set_staged(mcx_engine *e, int on) {
  return mcx_set_pass(e, on ? MCX_PASS_STAGED : MCX_PASS_MARCH);
}

extern "C" int mcx_get_staged(const mcx_engine *e) { return e && e->staged ? 1 : 0; }

// Re-plans the z-march units for a block size and chunk depth and uploads
// them with the replicas' CTA counts.
// Units of the learned-proposal z-march: per replica, blocks of its CTA size
// of a plane's pairs times chunks of kLearnPlanes planes; uploads them and the
// replicas' CTA counts.
constexpr int kLearnPlanes = 8;
static mcx_status plan_lmarch(mcx_engine *e) {
  e->lunits.clear();
  const int nt = lmarch_block_threads();
  for (int r = 0; r < e->nrep; r++) {
    RepDev &R = e->rep[r];
    const int npp = R.hp * R.ny, K = std::min(kLearnPlanes, R.nz);
    R.lcta = 0;
    for (int k0 = 0; k0 < R.nz; k0 += K)
      for (int p0 = 0; p0 < npp; p0 += nt) {
        e->lunits.push_back(make_int4(r, p0, k0, std::min(K, R.nz - k0)));
        R.lcta++;
      }
  }
  for (int4 &u : e->lunits) u.w |= unit_class(e, u, nt) == kUnitDead ? kUnitDead : 0;
  cudaFree(e->d_lunits);
  e->d_lunits = nullptr;
  CK(e, cudaMalloc(&e->d_lunits, sizeof(int4) * e->lunits.size()));
  CK(e, cudaMemcpyAsync(e->d_lunits, e->lunits.data(), sizeof(int4) * e->lunits.size(), cudaMemcpyHostToDevice,
                        e->stream));
  CK(e, cudaMemcpyAsync(e->d_rep, e->rep.data(), sizeof(RepDev) * e->nrep, cudaMemcpyHostToDevice, e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  return MCX_OK;
}

// Shared-memory slots of the TMA-staged z-march for the current units: an O
// slot holds 3 components x (rows spanned + 2) rows, an A slot 3 x rows.
static void plan_tmarch_slots(mcx_engine *e) {
  long long o = 0, a = 0;
  for (const int4 &u : e->units) {
    const RepDev &R = e->rep[u.x];
    const int pend = std::min(u.y + e->march_nt, R.hp * R.ny);
    const int nrA = (pend - 1) / R.hp - u.y / R.hp + 1;
    o = std::max(o, 3LL * (nrA + 2) * R.hs);
    a = std::max(a, 3LL * nrA * R.hs);
  }
  e->tm_o = (int)align_up(o, 32);
  e->tm_a = (int)align_up(a, 32);
}

// The four-site z-march runs unmasked batches whose rows hold whole quads
// of same-colour sites (nx a multiple of 8).
static bool qmarch_ok(const mcx_engine *e) {
  if (e->var.mask) return false;
  for (const RepDev &R : e->rep)
    if (R.nx % 8) return false;
  return qmarch_prepare(e->var, e->march_nt);
}

// Selects the TMA-staged form of the z-march when it can run (unmasked
// lattices whose slots fit in shared memory).
static bool use_tmarch(mcx_engine *e, bool on) {
  e->tmarch = false;
  if (!on || e->var.mask) return false;
  plan_tmarch_slots(e);
  const long long bytes = (4LL * e->tm_o + 2LL * e->tm_a) * 4;
  if (bytes > 200 * 1024) return false;
  e->tmarch = tmarch_prepare(e->var, e->march_nt, (int)bytes);
  return e->tmarch;
}

static mcx_status apply_march_shape(mcx_engine *e, int nt, int k) {
  e->march_nt = nt;
  e->march_k = k;
  const size_t before = e->units.size();
  if (e->amarch) e->amarch = amarch_prepare(e->var, nt);  // before planning: its residency sets the waves
  if (e->qmarch) e->qmarch = qmarch_ok(e);
  plan_march(e);
  if (e->tmarch) use_tmarch(e, true);
  if (e->units.size() > before || !e->d_units) {
    cudaFree(e->d_units);
    e->d_units = nullptr;
    CK(e, cudaMalloc(&e->d_units, sizeof(int4) * e->units.size()));
  }
  CK(e, cudaMemcpyAsync(e->d_units, e->units.data(), sizeof(int4) * e->units.size(), cudaMemcpyHostToDevice, e->stream));
  CK(e, cudaMemcpyAsync(e->d_rep, e->rep.data(), sizeof(RepDev) * e->nrep, cudaMemcpyHostToDevice, e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  drop_graphs(e);
  return MCX_OK;
}

extern "C" mcx_status mcx_set_march_shape(mcx_engine *e, int block, int planes) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (!march_block_ok(block) || planes < -8) return fail(e, MCX_ERR_INVALID, "z-march shape %d threads x %d planes", block, planes);
  if (e->pmarch && !pmarch_block_ok(block))
    return fail(e, MCX_ERR_UNSUPPORTED, "the persistent z-march runs blocks of 128 or 256 threads");
  CK(e, cudaStreamSynchronize(e->stream));
  return apply_march_shape(e, block, planes);
}

static void launch_march_form(mcx_engine *e, int form, const PassArgs &pa, int nt) {
  if (form == 1) launch_tmarch(e->var, MODE_SWEEP, pa, nt, e->pdl, e->stream);
  else if (form == 2) launch_amarch(e->var, MODE_SWEEP, pa, nt, e->pdl, e->stream);
  else if (form == 4) launch_qmarch(e->var, MODE_SWEEP, pa, nt, e->pdl, e->stream);
  else launch_march(e->var, MODE_SWEEP, pa, nt, e->pdl, e->stream);
}

// Times the z-march pass for every candidate shape on a scratch copy of the
// directors and per-replica state (the engine's own state is untouched) and
// keeps the fastest.
extern "C" mcx_status mcx_autotune(mcx_engine *e, int *block, int *planes, float *pass_us) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  CK(e, cudaStreamSynchronize(e->stream));
  int maxnz = 1;
  for (const RepDev &R : e->rep) maxnz = std::max(maxnz, R.nz);
  float *d_dir = nullptr;
  RepState *d_st = nullptr;
  double *d_stats = nullptr, *d_ring = nullptr;
  const size_t ring_n = (size_t)e->nrep * (e->ring_cap + 1) * kLanes * kQ;
  cudaEvent_t t0, t1;
  mcx_status st = MCX_OK;
  int best_nt = e->march_nt, best_k = e->march_k,
      best_form = e->pmarch ? 3 : (e->tmarch ? 1 : (e->amarch ? 2 : (e->qmarch ? 4 : 0)));
  float best = 1e30f;
#define CKA(call)                                                                                    \
  do {                                                                                               \
    cudaError_t _r = (call);                                                                         \
    if (_r != cudaSuccess) {                                                                         \
      st = fail(e, MCX_ERR_CUDA, "autotune: %s: %s", #call, cudaGetErrorString(_r));                 \
      goto done;                                                                                     \
    }                                                                                                \
  } while (0)
  CKA(cudaEventCreate(&t0));
  CKA(cudaEventCreate(&t1));
  CKA(cudaMalloc(&d_dir, sizeof(float) * e->dir_total));
  CKA(cudaMalloc(&d_st, sizeof(RepState) * e->nrep));
  CKA(cudaMalloc(&d_stats, sizeof(double) * kStats * e->nrep));
  CKA(cudaMalloc(&d_ring, sizeof(double) * ring_n));
  CKA(cudaMemcpyAsync(d_dir, e->d_dir, sizeof(float) * e->dir_total, cudaMemcpyDeviceToDevice, e->stream));
  CKA(cudaMemcpyAsync(d_st, e->d_st, sizeof(RepState) * e->nrep, cudaMemcpyDeviceToDevice, e->stream));
  {
    const int nts[3] = {64, 128, 256};
    const int ks[10] = {1, 2, 4, 8, 16, 32, 0, -2, -3, -4};  // fixed depths, then balanced over 1..4 waves
    // forms: 0 the register march, 1 rows staged by bulk copies, 2 the per-thread prefetch,
    // 3 one cooperative launch per run of sweeps (one wave of units: a single shape per block size),
    // 4 four sites per thread
    for (int form = 0; form < 5; form++)
    for (int a = 0; a < 3; a++)
      for (int ki = 0; ki < 10; ki++) {
        const int k = ks[ki];
        if (k > maxnz && k > 1) continue;
        if (form == 3 && (k != 0 || !pmarch_block_ok(nts[a]) || pmarch_blocks_per_sm(e->var, nts[a]) == 0)) continue;
        e->tmarch = form == 1;
        e->amarch = form == 2;
        e->pmarch = form == 3;
        e->qmarch = form == 4;
        if ((st = apply_march_shape(e, nts[a], k))) goto done;
        if ((form == 1 && !e->tmarch) || (form == 2 && !e->amarch) || (form == 3 && !pmarch_fits(e)) ||
            (form == 4 && !e->qmarch))
          continue;  // the form cannot run this batch
        PassArgs pa = pass_args(e);
        pa.dir = d_dir;
        pa.st = d_st;
        pa.stats = d_stats;
        pa.ring = d_ring;
        const int reps = 8;
        if (form == 3) {
          CKA(launch_pmarch(e->var, MODE_SWEEP, pa, nts[a], 2, e->d_err + 1, e->stream));
          CKA(cudaEventRecord(t0, e->stream));
          CKA(launch_pmarch(e->var, MODE_SWEEP, pa, nts[a], reps, e->d_err + 1, e->stream));
        } else {
          for (int w = 0; w < 2; w++)
            for (int c = 0; c < 2; c++) {
              pa.colour = c;
              launch_march_form(e, form, pa, nts[a]);
            }
          CKA(cudaEventRecord(t0, e->stream));
          for (int q = 0; q < reps; q++)
            for (int c = 0; c < 2; c++) {
              pa.colour = c;
              launch_march_form(e, form, pa, nts[a]);
            }
        }
        CKA(cudaEventRecord(t1, e->stream));
        CKA(cudaGetLastError());
        CKA(cudaEventSynchronize(t1));
        e->launches += 4 + 2 * reps;
        float ms = 0.f;
        CKA(cudaEventElapsedTime(&ms, t0, t1));
        const float us = ms * 1e3f / (2 * reps);
        if (us < best) {
          best = us;
          best_nt = nts[a];
          best_k = k;
          best_form = form;
        }
      }
  }
  e->tmarch = best_form == 1;
  e->amarch = best_form == 2;
  e->pmarch = best_form == 3;
  e->qmarch = best_form == 4;
  st = apply_march_shape(e, best_nt, best_k);
  if (st == MCX_OK) st = check_err_flag(e);
done:
#undef CKA
  cudaStreamSynchronize(e->stream);
  cudaFree(d_dir);
  cudaFree(d_st);
  cudaFree(d_stats);
  cudaFree(d_ring);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (st == MCX_OK) {
    if (block) *block = best_nt;
    if (planes) *planes = best_k;
    if (pass_us) *pass_us = best;
  }
  return st;
}

static void drop_graphs(mcx_engine *e) {
  for (int m = 0; m < 2; m++)
    if (e->graph[m]) {
      cudaGraphExecDestroy(e->graph[m]);
      e->graph[m] = nullptr;
    }
}

extern "C" int mcx_mlp_params(void) { return MCX_MLP_PARAMS; }

static mcx_status upload_mlp(mcx_engine *e, const float *w);

extern "C" mcx_status mcx_set_mlp(mcx_engine *e, const float *w, int n) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (e->var.pot == POT_PEAR)
    return fail(e, MCX_ERR_UNSUPPORTED,
                "the learned proposal's head-tail symmetric mixture is built for LL and GHRL; the Pear potential is polar");
  if (!w || n != MCX_MLP_PARAMS) return fail(e, MCX_ERR_INVALID, "mcx_set_mlp: expected %d weights, got %d", MCX_MLP_PARAMS, n);
  for (int i = 0; i < n; i++)
    if (!(w[i] == w[i]) || w[i] > 1e30f || w[i] < -1e30f) return fail(e, MCX_ERR_INVALID, "mcx_set_mlp: weight %d is not finite", i);
  if (mcx_status st = upload_mlp(e, w)) return st;
  e->mlp.assign(w, w + n);
  e->w_stale = true;
  drop_graphs(e);  // captured launches hold the weight pointer only, but keep it simple
  return MCX_OK;
}

// Packs FP32 weights into the inference layout on the device (allocating it
// and sizing the learned pass's grid on first use).
static mcx_status upload_mlp(mcx_engine *e, const float *w) {
  std::vector<uint8_t> packed(mlp_device_bytes());
  pack_mlp_weights(w, packed.data());
  CK(e, cudaStreamSynchronize(e->stream));
  if (!e->d_mlp) {
    cudaError_t r = cudaMalloc(&e->d_mlp, packed.size());
    if (r != cudaSuccess) return fail(e, MCX_ERR_NOMEM, "mcx_set_mlp: %s", cudaGetErrorString(r));
    int dev = 0, nsm = 0;
    CK(e, cudaGetDevice(&dev));
    CK(e, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    for (int m = 0; m < 4; m++) {
      if (m == MODE_MEASURE_ONLY) continue;
      const int per = pass_learned_blocks_per_sm(e->var, m);
      if (per <= 0) return fail(e, MCX_ERR_CUDA, "learned pass kernel cannot be resident");
      e->lgrid[m] = (int)std::min<long long>((long long)per * nsm, (long long)e->map.size());
    }
    const char *lm = getenv("MCX_LMARCH");
    const char *lp = getenv("MCX_MLP_PATH");
    // the warp-level network is the default: measured faster inside the
    // learned z-march (LL 96^3 x 128: 3.43 against 3.87 ms per pass)
    e->ltc = lp && atoi(lp) == MCX_MLP_TCGEN05 && lmarch_prepare(e->var, true);
    e->lmarch_ok = !(lm && atoi(lm) == 0) && lmarch_prepare(e->var, e->ltc);
    if (e->lmarch_ok)
      if (mcx_status st = plan_lmarch(e)) return st;
  }
  CK(e, cudaMemcpy(e->d_mlp, packed.data(), packed.size(), cudaMemcpyHostToDevice));
  return MCX_OK;
}

extern "C" mcx_status mcx_get_mlp(mcx_engine *e, float *w) {
  if (!e || !w) return fail(e, MCX_ERR_INVALID, "mcx_get_mlp: null argument");
  if (e->mlp.empty()) return fail(e, MCX_ERR_INVALID, "no network weights set");
  memcpy(w, e->mlp.data(), sizeof(float) * e->mlp.size());
  return MCX_OK;
}

extern "C" mcx_status mcx_set_proposal(mcx_engine *e, int kind) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (kind != MCX_PROPOSAL_PLAIN && kind != MCX_PROPOSAL_VMF_MLP) return fail(e, MCX_ERR_INVALID, "unknown proposal %d", kind);
  if (kind == MCX_PROPOSAL_VMF_MLP && !e->d_mlp) return fail(e, MCX_ERR_INVALID, "set the network weights (mcx_set_mlp) first");
  CK(e, cudaStreamSynchronize(e->stream));
  e->proposal = kind;
  drop_graphs(e);
  return MCX_OK;
}

// ---------------------------------------------------------------------------
// Training of the learned proposal (kernels in mcx_train.cu).
// ---------------------------------------------------------------------------
static cudaError_t ensure_bytes(void **p, long long *cap, long long bytes) {
  if (*cap >= bytes) return cudaSuccess;
  cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  cudaError_t r = cudaMalloc(p, (size_t)bytes);
  if (r == cudaSuccess) *cap = bytes;
  return r;
}

// The FP32 master weights and Adam moments on the device, current with e->mlp.
static mcx_status train_prepare(mcx_engine *e) {
  if (e->mlp.empty()) return fail(e, MCX_ERR_INVALID, "set the network weights (mcx_set_mlp) first");
  const size_t wb = sizeof(float) * MCX_MLP_PARAMS;
  if (!e->d_w) {
    float **bufs[4] = {&e->d_w, &e->d_am, &e->d_av, &e->d_g};
    for (float **b : bufs) {
      cudaError_t r = cudaMalloc(b, wb);
      if (r != cudaSuccess) return fail(e, MCX_ERR_NOMEM, "training buffers: %s", cudaGetErrorString(r));
    }
  }
  if (e->w_stale) {
    CK(e, cudaMemcpyAsync(e->d_w, e->mlp.data(), wb, cudaMemcpyHostToDevice, e->stream));
    CK(e, cudaMemsetAsync(e->d_am, 0, wb, e->stream));
    CK(e, cudaMemsetAsync(e->d_av, 0, wb, e->stream));
    CK(e, cudaStreamSynchronize(e->stream));
    e->adam_step = 0;
    e->w_stale = false;
  }
  return MCX_OK;
}

static mcx_status check_augment(mcx_engine *e, int augment) {
  if (augment & ~(MCX_AUG_FLIP | MCX_AUG_ROTATE)) return fail(e, MCX_ERR_INVALID, "unknown augmentation bits %d", augment);
  if (augment & MCX_AUG_ROTATE) {
    bool ok = e->var.pot == POT_LL && !e->var.field;
    for (const auto &d : e->desc) ok = ok && d.n_surfaces == 0;
    if (!ok)
      return fail(e, MCX_ERR_INVALID,
                  "MCX_AUG_ROTATE needs Lebwohl-Lasher replicas without field or surfaces (a rotation is not a symmetry otherwise)");
  }
  return MCX_OK;
}

// Draws n samples into e->d_samples (queued on the engine stream).
static mcx_status collect(mcx_engine *e, int n, unsigned seed, int augment) {
  const int F = sample_floats();
  CK(e, ensure_bytes((void **)&e->d_samples, &e->sample_cap, (long long)n * F * sizeof(float)));
  const int nb = (n + 255) / 256;
  std::vector<int> rep_of(nb);
  for (int b = 0; b < nb; b++) rep_of[b] = b % e->nrep;
  CK(e, ensure_bytes((void **)&e->d_repof, &e->repof_cap, (long long)nb * sizeof(int)));
  CK(e, cudaMemcpyAsync(e->d_repof, rep_of.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, e->stream));
  CK(e, launch_collect(e->d_rep, e->d_st, e->d_dir, e->d_pt, e->d_samples, e->d_repof, n, seed, augment, e->stream));
  e->launches++;
  e->held_samples = n;
  // rep_of is a local vector: the copy must finish before it goes
  CK(e, cudaStreamSynchronize(e->stream));
  return MCX_OK;
}

static int grad_grid(int n) {
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return std::max(1, std::min((n + 63) / 64, 2 * nsm));
}

extern "C" mcx_status mcx_collect_samples(mcx_engine *e, int n, unsigned int seed, int augment, float *out) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (n < 1) return fail(e, MCX_ERR_INVALID, "mcx_collect_samples: n = %d", n);
  if (mcx_status st = check_augment(e, augment)) return st;
  if (mcx_status st = collect(e, n, seed, augment)) return st;
  if (out) {
    CK(e, cudaMemcpyAsync(out, e->d_samples, sizeof(float) * (size_t)n * sample_floats(), cudaMemcpyDeviceToHost, e->stream));
    CK(e, cudaStreamSynchronize(e->stream));
  }
  return MCX_OK;
}

extern "C" mcx_status mcx_mlp_grad(mcx_engine *e, const float *samples, int n, float *grad, float *loss) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (!samples || !grad || n < 1) return fail(e, MCX_ERR_INVALID, "mcx_mlp_grad: bad arguments");
  if (mcx_status st = train_prepare(e)) return st;
  const size_t sb = sizeof(float) * (size_t)n * sample_floats();
  CK(e, ensure_bytes((void **)&e->d_samples, &e->sample_cap, (long long)sb));
  CK(e, ensure_bytes((void **)&e->d_loss, &e->loss_bytes, sizeof(float)));
  CK(e, cudaMemcpyAsync(e->d_samples, samples, sb, cudaMemcpyHostToDevice, e->stream));
  e->held_samples = n;
  CK(e, cudaMemsetAsync(e->d_g, 0, sizeof(float) * MCX_MLP_PARAMS, e->stream));
  CK(e, cudaMemsetAsync(e->d_loss, 0, sizeof(float), e->stream));
  CK(e, launch_mlp_grad(e->d_w, e->d_samples, nullptr, n, e->d_g, e->d_loss, grad_grid(n), e->stream));
  e->launches++;
  CK(e, cudaMemcpyAsync(grad, e->d_g, sizeof(float) * MCX_MLP_PARAMS, cudaMemcpyDeviceToHost, e->stream));
  float l = 0.f;
  CK(e, cudaMemcpyAsync(&l, e->d_loss, sizeof(float), cudaMemcpyDeviceToHost, e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  if (loss) *loss = l;
  return MCX_OK;
}

extern "C" mcx_status mcx_set_mlp_path(mcx_engine *e, int path) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (path != MCX_MLP_WARP_MMA && path != MCX_MLP_TCGEN05)
    return fail(e, MCX_ERR_INVALID, "mcx_set_mlp_path: unknown path %d", path);
  if (!e->d_mlp) return fail(e, MCX_ERR_INVALID, "mcx_set_mlp_path: set the network weights (mcx_set_mlp) first");
  if (!e->lmarch_ok) return fail(e, MCX_ERR_UNSUPPORTED, "mcx_set_mlp_path: the learned z-march does not run this batch");
  CK(e, cudaStreamSynchronize(e->stream));
  if (path == MCX_MLP_TCGEN05 && !lmarch_prepare(e->var, true))
    return fail(e, MCX_ERR_UNSUPPORTED, "mcx_set_mlp_path: the tensor-core form cannot be resident");
  e->ltc = path == MCX_MLP_TCGEN05;
  if (!lmarch_prepare(e->var, e->ltc)) return fail(e, MCX_ERR_CUDA, "mcx_set_mlp_path: learned z-march set-up failed");
  drop_graphs(e);
  return MCX_OK;
}

extern "C" int mcx_get_mlp_path(const mcx_engine *e) { return e && e->ltc ? MCX_MLP_TCGEN05 : MCX_MLP_WARP_MMA; }

extern "C" mcx_status mcx_mlp_forward(mcx_engine *e, const float *inputs, int n, float *outputs, int path) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (!inputs || !outputs || n < 1) return fail(e, MCX_ERR_INVALID, "mcx_mlp_forward: bad arguments");
  if (path != MCX_MLP_WARP_MMA && path != MCX_MLP_TCGEN05)
    return fail(e, MCX_ERR_INVALID, "mcx_mlp_forward: unknown path %d", path);
  if (!e->d_mlp || e->mlp.empty()) return fail(e, MCX_ERR_INVALID, "mcx_mlp_forward: no network set (mcx_set_mlp)");
  float *d_in = nullptr, *d_out = nullptr;
  struct Bufs {
    float **a, **b;
    ~Bufs() {
      cudaFree(*a);
      cudaFree(*b);
    }
  } bufs{&d_in, &d_out};
  CK(e, cudaMalloc(&d_in, sizeof(float) * 19 * (size_t)n));
  CK(e, cudaMalloc(&d_out, sizeof(float) * 4 * (size_t)n));
  CK(e, cudaMemcpyAsync(d_in, inputs, sizeof(float) * 19 * (size_t)n, cudaMemcpyHostToDevice, e->stream));
  CK(e, launch_mlp_forward(e->d_mlp, d_in, n, d_out, path == MCX_MLP_TCGEN05, e->d_err, e->stream));
  e->launches++;
  CK(e, cudaMemcpyAsync(outputs, d_out, sizeof(float) * 4 * (size_t)n, cudaMemcpyDeviceToHost, e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  return check_err_flag(e);
}

extern "C" mcx_status mcx_train_mlp(mcx_engine *e, const mcx_train_config *cfg, float *loss) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (!cfg) return fail(e, MCX_ERR_INVALID, "mcx_train_mlp: null config");
  if (cfg->samples < 0 || cfg->batch < 1 || cfg->steps < 0)
    return fail(e, MCX_ERR_INVALID, "mcx_train_mlp: samples %d, batch %d, steps %d", cfg->samples, cfg->batch, cfg->steps);
  if (cfg->samples == 0 && e->held_samples == 0)
    return fail(e, MCX_ERR_INVALID, "mcx_train_mlp: samples = 0 reuses the last collection, but there is none");
  if (!(cfg->lr > 0.f) || cfg->lr > 1.f) return fail(e, MCX_ERR_INVALID, "mcx_train_mlp: learning rate %g", (double)cfg->lr);
  if (mcx_status st = check_augment(e, cfg->augment)) return st;
  if (mcx_status st = train_prepare(e)) return st;
  if (cfg->samples > 0)
    if (mcx_status st = collect(e, cfg->samples, cfg->seed, cfg->augment)) return st;
  const int nsamp = e->held_samples;
  CK(e, ensure_bytes((void **)&e->d_idx, &e->idx_cap, (long long)cfg->batch * sizeof(int)));
  CK(e, ensure_bytes((void **)&e->d_loss, &e->loss_bytes, (long long)std::max(1, cfg->steps) * sizeof(float)));
  CK(e, cudaMemsetAsync(e->d_loss, 0, sizeof(float) * std::max(1, cfg->steps), e->stream));
  const int grid = grad_grid(cfg->batch);
  for (int s = 0; s < cfg->steps; s++) {
    e->adam_step++;
    CK(e, launch_batch_index(e->d_idx, cfg->batch, nsamp, cfg->seed, (uint32_t)e->adam_step, e->stream));
    CK(e, cudaMemsetAsync(e->d_g, 0, sizeof(float) * MCX_MLP_PARAMS, e->stream));
    CK(e, launch_mlp_grad(e->d_w, e->d_samples, e->d_idx, cfg->batch, e->d_g, e->d_loss + s, grid, e->stream));
    CK(e, launch_adam(e->d_w, e->d_am, e->d_av, e->d_g, e->adam_step, cfg->lr, e->stream));
    e->launches += 3;
  }
  std::vector<float> w(MCX_MLP_PARAMS);
  CK(e, cudaMemcpyAsync(w.data(), e->d_w, sizeof(float) * MCX_MLP_PARAMS, cudaMemcpyDeviceToHost, e->stream));
  if (loss && cfg->steps > 0)
    CK(e, cudaMemcpyAsync(loss, e->d_loss, sizeof(float) * cfg->steps, cudaMemcpyDeviceToHost, e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  for (int i = 0; i < MCX_MLP_PARAMS; i++)
    if (!(w[i] == w[i])) return fail(e, MCX_ERR_CUDA, "mcx_train_mlp: weight %d diverged (NaN); lower the learning rate", i);
  if (mcx_status st = upload_mlp(e, w.data())) return st;
  e->mlp = w;
  return MCX_OK;
}

// ---------------------------------------------------------------------------
// Snapshots, checkpoints, replica exchange.
// ---------------------------------------------------------------------------
extern "C" mcx_status mcx_polarization(mcx_engine *e, int r, double *P) {
  if (mcx_status st = check_rep(e, r)) return st;
  if (!P) return fail(e, MCX_ERR_INVALID, "mcx_polarization: null output");
  launch_polarization(e->rep[r], e->d_dir, e->d_mout, e->stream);
  e->launches++;
  CKL(e);
  double sum[3];
  CK(e, cudaMemcpyAsync(sum, e->d_mout, sizeof sum, cudaMemcpyDeviceToHost, e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  const double N = (double)e->rep[r].ntot;
  *P = sqrt(sum[0] * sum[0] + sum[1] * sum[1] + sum[2] * sum[2]) / N;
  return MCX_OK;
}

extern "C" mcx_status mcx_local_order(mcx_engine *e, int r, float *S) {
  if (mcx_status st = check_rep(e, r)) return st;
  if (!S) return fail(e, MCX_ERR_INVALID, "mcx_local_order: null output");
  const RepDev &R = e->rep[r];
  launch_local_order(R, e->d_dir, e->d_pt, e->d_stage, e->stream);
  e->launches++;
  CKL(e);
  CK(e, cudaMemcpyAsync(S, e->d_stage, sizeof(float) * R.ntot, cudaMemcpyDeviceToHost, e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  return MCX_OK;
}

namespace {
const char kCkptMagic[8] = {'M', 'C', 'X', 'C', 'K', 'P', 'T', '1'};
struct CkptState {
  float T, ang_var;
  unsigned long long sweep, meas;
  unsigned int frozen, pad;
};
struct FileCloser {
  FILE *f;
  ~FileCloser() {
    if (f) fclose(f);
  }
};
}  // namespace

extern "C" mcx_status mcx_save(mcx_engine *e, const char *path) {
  if (!e || !path) return fail(e, MCX_ERR_INVALID, "mcx_save: null argument");
  if (mcx_status st = flush(e)) return st;
  CK(e, cudaStreamSynchronize(e->stream));
  FileCloser fc{fopen(path, "wb")};
  if (!fc.f) return fail(e, MCX_ERR_IO, "mcx_save: cannot open %s", path);
  std::vector<RepState> st(e->nrep);
  std::vector<double> stats((size_t)kStats * e->nrep);
  CK(e, cudaMemcpy(st.data(), e->d_st, sizeof(RepState) * e->nrep, cudaMemcpyDeviceToHost));
  CK(e, cudaMemcpy(stats.data(), e->d_stats, sizeof(double) * stats.size(), cudaMemcpyDeviceToHost));
  const uint32_t hdr[4] = {1u, (uint32_t)e->nrep, (uint32_t)sizeof(mcx_replica_desc), e->mlp.empty() ? 0u : 1u};
  bool ok = fwrite(kCkptMagic, 1, 8, fc.f) == 8 && fwrite(hdr, sizeof hdr, 1, fc.f) == 1;
  for (int r = 0; r < e->nrep && ok; r++) {
    const RepDev &R = e->rep[r];
    CkptState cs{st[r].T, st[r].ang_var, st[r].sweep, st[r].meas, st[r].frozen, 0u};
    std::vector<float> ni(3 * (size_t)R.ntot);
    if (mcx_status s2 = mcx_get_state(e, r, ni.data())) return s2;
    ok = fwrite(&e->desc[r], sizeof(mcx_replica_desc), 1, fc.f) == 1 && fwrite(&cs, sizeof cs, 1, fc.f) == 1 &&
         fwrite(stats.data() + (size_t)kStats * r, sizeof(double), kStats, fc.f) == (size_t)kStats &&
         fwrite(ni.data(), sizeof(float), ni.size(), fc.f) == ni.size();
    if (ok && e->var.mask) {
      std::vector<int> pt(R.ntot);
      std::vector<float> ns(3 * (size_t)R.ntot);
      if (mcx_status s2 = mcx_get_mask(e, r, pt.data(), ns.data())) return s2;
      ok = fwrite(pt.data(), sizeof(int), pt.size(), fc.f) == pt.size() &&
           fwrite(ns.data(), sizeof(float), ns.size(), fc.f) == ns.size();
    }
  }
  if (ok && !e->mlp.empty()) {
    const int32_t prop = e->proposal;
    ok = fwrite(&prop, sizeof prop, 1, fc.f) == 1 && fwrite(e->mlp.data(), sizeof(float), e->mlp.size(), fc.f) == e->mlp.size();
  }
  if (!ok) return fail(e, MCX_ERR_IO, "mcx_save: write to %s failed", path);
  return MCX_OK;
}

// Reads and checks the whole checkpoint into host buffers before it touches
// the engine, so a file that is truncated, made for other replicas or holding
// an invalid mask or network leaves the engine as it was.
extern "C" mcx_status mcx_load(mcx_engine *e, const char *path) {
  if (!e || !path) return fail(e, MCX_ERR_INVALID, "mcx_load: null argument");
  FileCloser fc{fopen(path, "rb")};
  if (!fc.f) return fail(e, MCX_ERR_IO, "mcx_load: cannot open %s", path);
  char magic[8];
  uint32_t hdr[4];
  if (fread(magic, 1, 8, fc.f) != 8 || memcmp(magic, kCkptMagic, 8) != 0 || fread(hdr, sizeof hdr, 1, fc.f) != 1)
    return fail(e, MCX_ERR_PARSE, "mcx_load: %s is not an engine checkpoint", path);
  if (hdr[0] != 1u || hdr[2] != sizeof(mcx_replica_desc))
    return fail(e, MCX_ERR_PARSE, "mcx_load: checkpoint version %u / descriptor size %u not supported", hdr[0], hdr[2]);
  if ((int)hdr[1] != e->nrep)
    return fail(e, MCX_ERR_INVALID, "mcx_load: checkpoint holds %u replicas, the engine %d", hdr[1], e->nrep);
  const int n = e->nrep;
  std::vector<CkptState> cs(n);
  std::vector<double> stats((size_t)kStats * n);
  std::vector<std::vector<float>> ni(n), ns(n);
  std::vector<std::vector<int>> pt(n);
  for (int r = 0; r < n; r++) {
    const RepDev &R = e->rep[r];
    mcx_replica_desc d;
    if (fread(&d, sizeof d, 1, fc.f) != 1 || fread(&cs[r], sizeof cs[r], 1, fc.f) != 1 ||
        fread(stats.data() + (size_t)kStats * r, sizeof(double), kStats, fc.f) != (size_t)kStats)
      return fail(e, MCX_ERR_PARSE, "mcx_load: %s is truncated", path);
    // the whole descriptor must be the engine's (temperature and step size
    // are state and come from the checkpoint): another seed or stream would
    // not continue the saved trajectory, other physics not the saved model
    mcx_replica_desc a = d, b = e->desc[r];
    a.T = b.T = 0.f;
    a.ang_var = b.ang_var = 0.f;
    if (memcmp(&a, &b, sizeof a) != 0) {
      const char *what = d.nx != b.nx || d.ny != b.ny || d.nz != b.nz ? "lattice size"
                         : d.geometry != b.geometry || d.xbound != b.xbound || d.ybound != b.ybound ||
                                   d.zbound != b.zbound
                             ? "geometry or bounds"
                         : d.potential != b.potential ? "pair potential"
                         : d.seed != b.seed || d.stream != b.stream ? "RNG seed or stream"
                                                                    : "physical parameters (couplings, field, anchoring)";
      return fail(e, MCX_ERR_INVALID, "mcx_load: replica %d of the checkpoint differs from the engine's in its %s",
                  r, what);
    }
    ni[r].resize(3 * (size_t)R.ntot);
    if (fread(ni[r].data(), sizeof(float), ni[r].size(), fc.f) != ni[r].size())
      return fail(e, MCX_ERR_PARSE, "mcx_load: %s is truncated", path);
    if (e->var.mask) {
      pt[r].resize(R.ntot);
      ns[r].resize(3 * (size_t)R.ntot);
      if (fread(pt[r].data(), sizeof(int), pt[r].size(), fc.f) != pt[r].size() ||
          fread(ns[r].data(), sizeof(float), ns[r].size(), fc.f) != ns[r].size())
        return fail(e, MCX_ERR_PARSE, "mcx_load: %s is truncated", path);
      long active = 0;
      for (long q = 0; q < R.ntot; q++) {
        const int v = pt[r][q];
        if (v < 0 || v > 255 || (v > 1 && v - 2 >= R.nsurf))
          return fail(e, MCX_ERR_PARSE, "mcx_load: replica %d: point type %d at site %ld is invalid", r, v, q);
        active += v != 0;
      }
      if (active == 0) return fail(e, MCX_ERR_PARSE, "mcx_load: replica %d: mask has no active site", r);
    }
  }
  int32_t prop = 0;
  std::vector<float> w;
  if (hdr[3] & 1u) {
    w.resize(MCX_MLP_PARAMS);
    if (fread(&prop, sizeof prop, 1, fc.f) != 1 || fread(w.data(), sizeof(float), w.size(), fc.f) != w.size())
      return fail(e, MCX_ERR_PARSE, "mcx_load: %s is truncated", path);
    if (prop != MCX_PROPOSAL_PLAIN && prop != MCX_PROPOSAL_VMF_MLP)
      return fail(e, MCX_ERR_PARSE, "mcx_load: unknown proposal %d", prop);
    if (e->var.pot == POT_PEAR)
      return fail(e, MCX_ERR_UNSUPPORTED, "mcx_load: the checkpoint holds a network; Pear runs the plain proposal only");
  }
  // everything read and checked: apply
  if (mcx_status st = flush(e)) return st;
  CK(e, cudaStreamSynchronize(e->stream));
  std::vector<RepState> st(n);
  CK(e, cudaMemcpy(st.data(), e->d_st, sizeof(RepState) * n, cudaMemcpyDeviceToHost));
  e->defer_plan = true;
  for (int r = 0; r < n && e->var.mask; r++)
    if (mcx_status s2 = mcx_set_mask(e, r, pt[r].data(), ns[r].data())) {
      e->defer_plan = false;
      return s2;
    }
  e->defer_plan = false;
  if (e->var.mask)
    if (mcx_status s2 = apply_march_shape(e, e->march_nt, e->march_k)) return s2;
  for (int r = 0; r < n; r++) {
    if (mcx_status s2 = mcx_set_state(e, r, ni[r].data())) return s2;
    st[r].T = cs[r].T;
    st[r].ang_var = cs[r].ang_var;
    st[r].sweep = cs[r].sweep;
    st[r].meas = cs[r].meas;
    st[r].frozen = cs[r].frozen;
    st[r].cnt = 0;
    e->desc[r].T = cs[r].T;
  }
  if (!w.empty()) {
    if (mcx_status s2 = mcx_set_mlp(e, w.data(), MCX_MLP_PARAMS)) return s2;
    if (mcx_status s2 = mcx_set_proposal(e, prop)) return s2;
  }
  CK(e, cudaMemcpyAsync(e->d_st, st.data(), sizeof(RepState) * n, cudaMemcpyHostToDevice, e->stream));
  CK(e, cudaMemcpyAsync(e->d_stats, stats.data(), sizeof(double) * stats.size(), cudaMemcpyHostToDevice, e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  e->meas_flushed = st[0].meas;
  e->pending = 0;
  return MCX_OK;
}

// Replica exchange between replicas of the same Hamiltonian at different
// temperatures: pair (a, b) swaps its temperatures (and step sizes) with
// probability min(1, exp((1/Ta - 1/Tb)(Ha - Hb))), H the total energy of the
// current state, u from Philox4x32-10 counter (pair, round_lo, round_hi,
// TAG_PT), key (seed, 0).
extern "C" mcx_status mcx_exchange(mcx_engine *e, int n, const int *pairs, unsigned int seed,
                                   unsigned long long round, int *accepted) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (n < 0 || (n > 0 && !pairs)) return fail(e, MCX_ERR_INVALID, "mcx_exchange: bad pair list");
  auto same = [](const mcx_replica_desc &x, const mcx_replica_desc &y) {
    mcx_replica_desc a = x, b = y;
    a.T = b.T = 0.f;
    a.ang_var = b.ang_var = 0.f;
    a.seed = b.seed = 0;
    a.stream = b.stream = 0;
    return memcmp(&a, &b, sizeof a) == 0;
  };
  std::vector<char> used(e->nrep, 0);
  for (int i = 0; i < n; i++) {
    const int a = pairs[2 * i], b = pairs[2 * i + 1];
    if (a < 0 || b < 0 || a >= e->nrep || b >= e->nrep || a == b || used[a] || used[b])
      return fail(e, MCX_ERR_INVALID, "mcx_exchange: pair %d (%d, %d) is not two distinct unused replicas", i, a, b);
    used[a] = used[b] = 1;
    if (!same(e->desc[a], e->desc[b]))
      return fail(e, MCX_ERR_INVALID, "mcx_exchange: replicas %d and %d differ in more than T (not one Hamiltonian)", a, b);
  }
  std::vector<RepState> st(e->nrep);
  CK(e, cudaStreamSynchronize(e->stream));
  CK(e, cudaMemcpy(st.data(), e->d_st, sizeof(RepState) * e->nrep, cudaMemcpyDeviceToHost));
  for (int i = 0; i < n; i++) {
    const int a = pairs[2 * i], b = pairs[2 * i + 1];
    double ma[MCX_MEASURE_LEN], mb[MCX_MEASURE_LEN];
    if (mcx_status s2 = mcx_measure(e, a, ma)) return s2;
    if (mcx_status s2 = mcx_measure(e, b, mb)) return s2;
    const double N = (double)e->rep[a].ntot;
    const double Ha = ma[MCX_M_E] * N, Hb = mb[MCX_M_E] * N;
    const double Ta = st[a].T, Tb = st[b].T;
    const uint4 w = philox4x32_10(make_uint4((uint32_t)i, (uint32_t)round, (uint32_t)(round >> 32), TAG_PT), seed, 0u);
    const double u = (double)u01(w.x);
    const double lr = (1.0 / Ta - 1.0 / Tb) * (Ha - Hb);
    const bool acc = lr >= 0.0 || u < exp(lr);
    if (accepted) accepted[i] = acc ? 1 : 0;
    if (acc) {
      std::swap(st[a].T, st[b].T);
      std::swap(st[a].ang_var, st[b].ang_var);
      std::swap(e->desc[a].T, e->desc[b].T);
    }
  }
  for (int q = 0; q < e->nrep; q++) {
    CK(e, cudaMemcpyAsync((char *)(e->d_st + q) + offsetof(RepState, T), &st[q].T, sizeof(float),
                          cudaMemcpyHostToDevice, e->stream));
    CK(e, cudaMemcpyAsync((char *)(e->d_st + q) + offsetof(RepState, ang_var), &st[q].ang_var, sizeof(float),
                          cudaMemcpyHostToDevice, e->stream));
  }
  CK(e, cudaStreamSynchronize(e->stream));
  return MCX_OK;
}

extern "C" mcx_status mcx_combine_stats(mcx_engine *e, int n, const int *replicas, double *out) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (!out) return fail(e, MCX_ERR_INVALID, "mcx_combine_stats: null output");
  std::vector<int> idx;
  if (n <= 0 || !replicas) {
    if (n > 0) return fail(e, MCX_ERR_INVALID, "mcx_combine_stats: null replica list");
    for (int q = 0; q < e->nrep; q++) idx.push_back(q);
  } else {
    idx.assign(replicas, replicas + n);
  }
  int pear = 0;
  for (int r : idx) {
    if (mcx_status st = check_rep(e, r)) return st;
    pear += e->desc[r].potential == MCX_POT_PEAR;
  }
  const int m = (int)idx.size();
  if (pear != 0 && pear != m)
    return fail(e, MCX_ERR_INVALID, "mcx_combine_stats: Pear replicas mixed with other potentials");
  if (mcx_status st = flush(e)) return st;
  // scratch: the index list, then 3 director sums per replica (Pear), then the output
  const size_t pol_off = ((size_t)m * sizeof(int) + 15) / 16 * 16;
  const size_t out_off = pol_off + (pear ? (size_t)m * 3 * sizeof(double) : 0);
  char *scratch = nullptr;
  CK(e, cudaMallocAsync((void **)&scratch, out_off + 16 * sizeof(double), e->stream));
  struct Free {
    mcx_engine *e;
    char *p;
    ~Free() { cudaFreeAsync(p, e->stream); }
  } guard{e, scratch};
  int *d_idx = (int *)scratch;
  double *d_pol = pear ? (double *)(scratch + pol_off) : nullptr;
  double *d_out = (double *)(scratch + out_off);
  CK(e, cudaMemcpyAsync(d_idx, idx.data(), (size_t)m * sizeof(int), cudaMemcpyHostToDevice, e->stream));
  for (int i = 0; pear && i < m; i++) {
    launch_polarization(e->rep[idx[i]], e->d_dir, d_pol + 3 * (size_t)i, e->stream);
    e->launches++;
  }
  launch_combine(e->d_rep, e->d_st, e->d_stats, d_pol, d_idx, m, d_out, e->stream);
  e->launches++;
  CKL(e);
  double h[MCX_COMBINED_LEN + 1];
  CK(e, cudaMemcpyAsync(h, d_out, sizeof h, cudaMemcpyDeviceToHost, e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  if (h[MCX_COMBINED_LEN] > 0)
    return fail(e, MCX_ERR_INVALID, "mcx_combine_stats: %d replica(s) without measured sweeps",
                (int)h[MCX_COMBINED_LEN]);
  memcpy(out, h, sizeof(double) * MCX_COMBINED_LEN);
  if (h[MCX_CB_T_SPREAD] > 1e-3)
    return fail(e, MCX_ERR_INVALID, "mcx_combine_stats: temperatures differ by %g (> 1e-3)", h[MCX_CB_T_SPREAD]);
  return MCX_OK;
}

extern "C" mcx_status mcx_debug_barrier_timeout(mcx_engine *e) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (!persistent(e)) return fail(e, MCX_ERR_INVALID, "the persistent z-march is not selected");
  PassArgs pa = pass_args(e);
  CK(e, launch_pmarch(e->var, MODE_SWEEP, pa, e->march_nt, 1, e->d_err + 1, e->stream, 1u));
  e->launches += 1;
  CK(e, cudaStreamSynchronize(e->stream));
  return check_err_flag(e);
}

extern "C" mcx_status mcx_measure(mcx_engine *e, int r, double *out) {
  if (mcx_status st = check_rep(e, r)) return st;
  if (!out) return fail(e, MCX_ERR_INVALID, "null output");
  PassArgs pa = pass_args(e);
  for (int c = 0; c < 2; c++) {
    pa.colour = c;
    launch_pass(e->var, MODE_MEASURE_ONLY, pa, e->pgrid[MODE_MEASURE_ONLY], e->stream);
  }
  launch_measure_out(e->d_rep, e->d_ring, e->ring_cap, e->nrep, e->d_mout, e->stream);
  e->launches += 3;
  CKL(e);
  CK(e, cudaMemcpyAsync(out, e->d_mout + (size_t)r * 16, sizeof(double) * 16, cudaMemcpyDeviceToHost, e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  return MCX_OK;
}

extern "C" mcx_status mcx_get_stats(mcx_engine *e, int r, double *out) {
  if (mcx_status st = check_rep(e, r)) return st;
  if (!out) return fail(e, MCX_ERR_INVALID, "null output");
  if (mcx_status st = flush(e)) return st;
  CK(e, cudaMemcpyAsync(out, e->d_stats + (size_t)r * kStats, sizeof(double) * kStats, cudaMemcpyDeviceToHost,
                        e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  return check_err_flag(e);
}

extern "C" mcx_status mcx_reset_stats(mcx_engine *e, int r) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  const int r0 = r < 0 ? 0 : r, r1 = r < 0 ? e->nrep : r + 1;
  if (r >= e->nrep) return fail(e, MCX_ERR_INVALID, "replica %d out of range", r);
  if (mcx_status st = flush(e)) return st;
  // keep the step size and sweep index entries (11, 12), clear the sums
  for (int q = r0; q < r1; q++)
    CK(e, cudaMemsetAsync(e->d_stats + (size_t)q * kStats, 0, sizeof(double) * 11, e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  return MCX_OK;
}

extern "C" mcx_status mcx_set_series(mcx_engine *e, int cap) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (cap < 0) return fail(e, MCX_ERR_INVALID, "negative series capacity");
  if (mcx_status st = flush(e)) return st;
  CK(e, cudaStreamSynchronize(e->stream));
  cudaFree(e->d_series);
  e->d_series = nullptr;
  e->series_cap = 0;
  if (cap > 0) {
    cudaError_t r = cudaMalloc(&e->d_series, sizeof(double) * 2 * (size_t)cap * e->nrep);
    if (r != cudaSuccess) return fail(e, MCX_ERR_NOMEM, "series buffer: %s", cudaGetErrorString(r));
    CK(e, cudaMemset(e->d_series, 0, sizeof(double) * 2 * (size_t)cap * e->nrep));
    e->series_cap = cap;
  }
  return MCX_OK;
}

extern "C" mcx_status mcx_get_series(mcx_engine *e, int r, int count, double *out) {
  if (mcx_status st = check_rep(e, r)) return st;
  if (!out || count < 0) return fail(e, MCX_ERR_INVALID, "bad series request");
  if (count > e->series_cap) return fail(e, MCX_ERR_INVALID, "count %d exceeds series capacity %d", count, e->series_cap);
  if (mcx_status st = flush(e)) return st;
  const long long n = (long long)e->meas_flushed;
  if (count > n) return fail(e, MCX_ERR_INVALID, "only %lld measured sweeps recorded", n);
  std::vector<double> ring(2 * (size_t)e->series_cap);
  CK(e, cudaMemcpyAsync(ring.data(), e->d_series + (size_t)r * e->series_cap * 2, sizeof(double) * ring.size(),
                        cudaMemcpyDeviceToHost, e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  for (int q = 0; q < count; q++) {
    const long long idx = (n - count + q) % e->series_cap;
    out[2 * q] = ring[2 * idx];
    out[2 * q + 1] = ring[2 * idx + 1];
  }
  return MCX_OK;
}

extern "C" void *mcx_stream(mcx_engine *e) { return e ? (void *)e->stream : nullptr; }

extern "C" mcx_status mcx_sweep_timing(mcx_engine *e, int n, float *ms) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (n <= 0 || !ms) return fail(e, MCX_ERR_INVALID, "need n_sweeps > 0 and an output");
  cudaEvent_t a, b;
  CK(e, cudaEventCreate(&a));
  CK(e, cudaEventCreate(&b));
  mcx_status st = MCX_OK;
  {
    cudaError_t r = cudaEventRecord(a, e->stream);
    if (r == cudaSuccess) st = run_sweeps(e, n, 0);
    if (r == cudaSuccess && !st) r = cudaEventRecord(b, e->stream);
    if (r == cudaSuccess && !st) r = cudaEventSynchronize(b);
    if (r == cudaSuccess && !st) r = cudaEventElapsedTime(ms, a, b);
    if (r != cudaSuccess && !st) st = fail(e, MCX_ERR_CUDA, "mcx_sweep_timing: %s", cudaGetErrorString(r));
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return st;
}

extern "C" mcx_status mcx_pass_timing(mcx_engine *e, int n, float *pass_ms, float *total_ms) {
  if (!e) return fail(nullptr, MCX_ERR_INVALID, "null engine");
  if (n <= 0) return fail(e, MCX_ERR_INVALID, "need n_sweeps > 0");
  std::vector<cudaEvent_t> ev(4 * (size_t)n);
  for (auto &x : ev) CK(e, cudaEventCreate(&x));
  PassArgs pa = pass_args(e);
  for (int s = 0; s < n; s++)
    for (int c = 0; c < 2; c++) {
      CK(e, cudaEventRecord(ev[4 * s + 2 * c], e->stream));
      launch_sweep_pass(e, pa, c, false);
      CK(e, cudaEventRecord(ev[4 * s + 2 * c + 1], e->stream));
    }
  e->launches += 2LL * n;
  CKL(e);
  CK(e, cudaStreamSynchronize(e->stream));
  float sum = 0.f, t;
  for (int q = 0; q < 2 * n; q++) {
    CK(e, cudaEventElapsedTime(&t, ev[2 * q], ev[2 * q + 1]));
    sum += t;
  }
  CK(e, cudaEventElapsedTime(&t, ev[0], ev.back()));
  if (pass_ms) *pass_ms = sum;
  if (total_ms) *total_ms = t;
  for (auto &x : ev) cudaEventDestroy(x);
  return MCX_OK;
}

extern "C" void mcx_ghrl_constants(float k11, float k22, float k33, float p0, float *out) {
  ghrl_constants(k11, k22, k33, p0, out);
}

extern "C" mcx_status mcx_build_mask(const mcx_replica_desc *d, int *pt, float *ns) {
  if (!d || !pt || !ns) return fail(nullptr, MCX_ERR_INVALID, "mcx_build_mask: null argument");
  if (d->geometry == MCX_GEO_CUSTOM) return fail(nullptr, MCX_ERR_INVALID, "custom geometry comes from a file");
  if (mcx_status st = check_desc(*d, 0)) return st;
  std::vector<int> p;
  std::vector<float> n;
  build_mask(*d, p, n);
  memcpy(pt, p.data(), sizeof(int) * p.size());
  memcpy(ns, n.data(), sizeof(float) * n.size());
  return MCX_OK;
}

extern "C" mcx_status mcx_read_geometry(const char *path, int nx, int ny, int nz, int *pt, float *ns, int *nsurf) {
  if (!path || !pt || !ns || nx <= 0 || ny <= 0 || nz <= 0) return fail(nullptr, MCX_ERR_INVALID, "mcx_read_geometry: bad argument");
  std::vector<int> p;
  std::vector<float> n;
  std::string err;
  int k = read_custom_geometry(path, nx, ny, nz, p, n, err);
  if (k < 0) return fail(nullptr, MCX_ERR_PARSE, "%s", err.c_str());
  memcpy(pt, p.data(), sizeof(int) * p.size());
  memcpy(ns, n.data(), sizeof(float) * n.size());
  if (nsurf) *nsurf = k;
  return MCX_OK;
}

extern "C" mcx_status mcx_debug_pass(mcx_engine *e, int r, int colour, float *dE, unsigned char *acc, float *prop) {
  return mcx_debug_pass_mlp(e, r, colour, dE, acc, prop, nullptr);
}

extern "C" mcx_status mcx_debug_pass_mlp(mcx_engine *e, int r, int colour, float *dE, unsigned char *acc, float *prop,
                                         float *mlp_out) {
  if (mcx_status st = check_rep(e, r)) return st;
  if (colour != 0 && colour != 1) return fail(e, MCX_ERR_INVALID, "colour must be 0 or 1");
  const RepDev &R = e->rep[r];
  float *d_dE = nullptr, *d_prop = nullptr;
  uint8_t *d_acc = nullptr;
  int2 *d_map = nullptr;
  std::vector<int2> sub;
  for (const int2 &m : e->map)
    if (m.x == r) sub.push_back(m);
  CK(e, cudaMalloc(&d_dE, sizeof(float) * R.ntot));
  CK(e, cudaMalloc(&d_prop, sizeof(float) * 3 * R.ntot));
  CK(e, cudaMalloc(&d_acc, R.ntot));
  CK(e, cudaMalloc(&d_map, sizeof(int2) * sub.size()));
  float *d_y = nullptr;
  if (mlp_out) {
    CK(e, cudaMalloc(&d_y, sizeof(float) * 4 * R.ntot));
    CK(e, cudaMemsetAsync(d_y, 0, sizeof(float) * 4 * R.ntot, e->stream));
  }
  CK(e, cudaMemsetAsync(d_dE, 0, sizeof(float) * R.ntot, e->stream));
  CK(e, cudaMemsetAsync(d_prop, 0, sizeof(float) * 3 * R.ntot, e->stream));
  CK(e, cudaMemsetAsync(d_acc, 0xFF, R.ntot, e->stream));
  CK(e, cudaMemcpyAsync(d_map, sub.data(), sizeof(int2) * sub.size(), cudaMemcpyHostToDevice, e->stream));
  PassArgs pa = pass_args(e);
  pa.map = d_map;
  pa.colour = colour;
  pa.tr_dE = d_dE;
  pa.tr_acc = d_acc;
  pa.tr_prop = d_prop;
  pa.tr_y = d_y;
  int4 *d_sub_tiles = nullptr;
  if (e->proposal == MCX_PROPOSAL_VMF_MLP) {
    pa.nmap = (int)sub.size();
    launch_pass_learned(e->var, MODE_TRACE, pa, std::min(e->lgrid[MODE_TRACE], (int)sub.size()), e->stream);
  } else if (e->staged) {
    const RepDev &Rr = e->rep[r];
    CK(e, cudaMalloc(&d_sub_tiles, sizeof(int4) * Rr.ntile));
    CK(e, cudaMemcpyAsync(d_sub_tiles, e->tiles.data() + Rr.tile0, sizeof(int4) * Rr.ntile, cudaMemcpyHostToDevice,
                          e->stream));
    pa.tiles = d_sub_tiles;
    pa.ntiles = Rr.ntile;
    launch_tpass(e->var, MODE_TRACE, pa, std::min(e->grid[0], Rr.ntile), e->stream);
  } else {
    pa.nmap = (int)sub.size();
    launch_pass(e->var, MODE_TRACE, pa, std::min(e->pgrid[MODE_TRACE], (int)sub.size()), e->stream);
  }
  e->launches += 1;
  CKL(e);
  if (dE) CK(e, cudaMemcpyAsync(dE, d_dE, sizeof(float) * R.ntot, cudaMemcpyDeviceToHost, e->stream));
  if (acc) CK(e, cudaMemcpyAsync(acc, d_acc, R.ntot, cudaMemcpyDeviceToHost, e->stream));
  if (prop) CK(e, cudaMemcpyAsync(prop, d_prop, sizeof(float) * 3 * R.ntot, cudaMemcpyDeviceToHost, e->stream));
  if (mlp_out) CK(e, cudaMemcpyAsync(mlp_out, d_y, sizeof(float) * 4 * R.ntot, cudaMemcpyDeviceToHost, e->stream));
  CK(e, cudaStreamSynchronize(e->stream));
  cudaFree(d_dE);
  cudaFree(d_prop);
  cudaFree(d_acc);
  cudaFree(d_map);
  cudaFree(d_sub_tiles);
  cudaFree(d_y);
  return check_err_flag(e);
}
