// mcx_kernels.cuh -- launch interface between the engine (mcx_engine.cu) and
// the kernels (mcx_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "mcx_device.cuh"

namespace mcx {

// Which specialisation of the pass kernel a batch runs: the pair potential,
// whether any replica has a mask (inactive or surface sites), and whether any
// replica has a field term.  Fixed per engine.
struct Variant {
  int pot;
  bool mask;
  bool field;
  bool per;  // every replica periodic in x, y and z with nx a multiple of 4 (no mask)
  bool odd = false;  // some replica has an odd nx (then the batch has a mask)
};

// What a pass launch does.
enum PassMode : int {
  MODE_SWEEP = 0,         // update one colour; colour 1 ends the sweep
  MODE_SWEEP_MEASURE = 1, // the same, and add E / Q of the final state to the sweep's ring slot
  MODE_MEASURE_ONLY = 2,  // no update: E / Q of the current state into the extra ring slot
  MODE_TRACE = 3          // update one colour of one replica and record every site
};

// z-march work units are int4 (replica, first pair, first plane, planes |
// flags).  kUnitDead marks a unit of a masked replica whose rows and planes,
// and the rows and planes next to them, hold no active site: its sites never
// move and have no bond to an active site, so its only work is the field
// energy of its sites in measured sweeps (what the full update adds for an
// inactive site).
constexpr int kUnitDead = 1 << 30;
// kUnitBulk marks a unit of a masked replica whose rows and planes, and the
// rows and planes next to them, hold only bulk sites (point type 1): it runs
// the unmasked update, which gives the same result there without the mask's
// loads and weights.
constexpr int kUnitBulk = 1 << 29;
// kUnitTiled marks a unit of the z-march that is a tile of kTileW pairs of a
// row times NT / kTileW rows (its second field (j0 << 12) | q0: first row,
// first pair of the row) rather than NT consecutive pairs of the plane.
// Masked replicas whose rows cross the mask's edge (droplets) are cut into
// tiles, so that the units inside the droplet hold only bulk sites and run
// the unmasked update.
constexpr int kUnitTiled = 1 << 28;
constexpr int kUnitPlanes = kUnitTiled - 1;
constexpr int kTileLg = 2, kTileW = 1 << kTileLg;  // pairs per tile row (one 32-byte sector)
constexpr int kTileQBits = 12;                      // q0 field: hp < 4096

struct PassArgs {
  const RepDev *reps;
  const int2 *map;  // work units of the direct pass: (replica, first same-colour pair)
  int nmap;
  float *dir;
  const uint8_t *pt;
  const float *ns;
  RepState *st;
  double *stats;  // [nrep][kStats]
  double *ring;   // [nrep][ring_cap + 1][kLanes][kQ]
  int ring_cap;
  int colour;
  // trace outputs (natural site order of one replica)
  float *tr_dE;
  uint8_t *tr_acc;
  float *tr_prop;
  float *tr_y;  // learned proposal: the network's 4 outputs per site (may be null)
  // learned proposal: the network's weights in the mcx_mlp.cuh layout
  const uint8_t *mlp;
  // staged pass: the flat tile list and the shared-memory stage size
  const int4 *tiles;  // (replica, j0, k0, 0)
  int ntiles;
  int stage_bytes;
  unsigned *err;  // set to 1 when a shared-memory copy did not arrive in time
  // z-march pass: (replica, first pair of the plane, first plane, planes)
  const int4 *units;
  int nunits;
  // TMA-staged z-march: floats per O slot and per A slot of shared memory
  int tm_o, tm_a;
  // measured sweeps of an unmasked batch on the z-march (register, prefetching
  // and four-site forms): the colour-0
  // pass runs unmeasured and the colour-1 pass (MODE_SWEEP_MEASURE) also adds
  // the Q-tensor and field terms of the colour-0 sites, read from the opposite
  // pairs it loads anyway (one reduction per sweep instead of two)
  int meas_both;
};

struct FlushArgs {
  const RepDev *reps;
  double *ring;
  int ring_cap;
  double *stats;
  double *series;  // [nrep][series_cap][2] or null
  int series_cap;
  unsigned long long first;  // measured-sweep index of the first pending slot
  int count;                 // pending slots
};

// The direct pass over a.map with `nblocks` persistent CTAs.
void launch_pass(const Variant &v, int mode, const PassArgs &a, int nblocks, cudaStream_t st);
int pass_blocks_per_sm(const Variant &v, int mode);
// The z-march pass (mcx_march.cu): one CTA of nt threads per unit of a.units;
// pdl lets the launch overlap the previous grid's tail (programmatic
// dependent launch; the kernel waits for it before touching shared state).
void launch_march(const Variant &v, int mode, const PassArgs &a, int nt, bool pdl, cudaStream_t st);
bool march_block_ok(int nt);
// the z-march kernel of a masked batch with an odd nx (mcx_march_odd.cu)
const void *march_kernel_odd(const Variant &v, int mode, int nt);
// The z-march with its rows staged in shared memory by bulk copies (unmasked
// lattices): prepare (shared-memory attribute, residency) once per shape.
bool tmarch_prepare(const Variant &v, int nt, int smem_bytes);
int tmarch_smem_bytes(const PassArgs &a);
void launch_tmarch(const Variant &v, int mode, const PassArgs &a, int nt, bool pdl, cudaStream_t st);
int march_blocks_per_sm(const Variant &v, int mode, int nt);
// The z-march with a per-thread cp.async prefetch of the next plane
// (mcx_amarch.cu; unmasked LL and GHRL): prepare once per block size.
bool amarch_prepare(const Variant &v, int nt);
int amarch_smem_bytes(int nt);
int amarch_blocks_per_sm(const Variant &v, int nt);
void launch_amarch(const Variant &v, int mode, const PassArgs &a, int nt, bool pdl, cudaStream_t st);
// The z-march with four same-colour sites per thread (mcx_qmarch.cu;
// unmasked batches, nx a multiple of 8): units of 2 x nt pairs.
bool qmarch_prepare(const Variant &v, int nt);
int qmarch_blocks_per_sm(const Variant &v, int nt);
void launch_qmarch(const Variant &v, int mode, const PassArgs &a, int nt, bool pdl, cudaStream_t st);
// The z-march as one cooperative launch for nsweeps sweeps (mcx_pmarch.cu):
// a.units must fit one wave (pmarch_blocks_per_sm per SM); bar is a counter
// the launch zeroes first; extra > 0 makes every grid barrier unreachable
// (a test of the bounded wait and its error flag).
bool pmarch_block_ok(int nt);
int pmarch_blocks_per_sm(const Variant &v, int nt);
cudaError_t launch_pmarch(const Variant &v, int mode, const PassArgs &a, int nt, int nsweeps, unsigned *bar,
                          cudaStream_t st, unsigned extra = 0);
// The learned-proposal z-march (mcx_lmarch.cu): units of lmarch_block_threads()
// pairs; lmarch_prepare sets its shared memory and checks residency.  tc: the
// network on the tcgen05 tensor cores (else the warp-level mma.sync code).
int lmarch_block_threads();
bool lmarch_prepare(const Variant &v, bool tc);
void launch_lmarch(const Variant &v, int mode, const PassArgs &a, bool pdl, bool tc, cudaStream_t st);
// The direct pass with the learned proposal (mcx_learned.cu).
void launch_pass_learned(const Variant &v, int mode, const PassArgs &a, int nblocks, cudaStream_t st);
int pass_learned_blocks_per_sm(const Variant &v, int mode);
// Packs FP32 weights (the flat layout of mcx_set_mlp) into the device layout.
void pack_mlp_weights(const float *flat, uint8_t *out);
int mlp_device_bytes();
int pass_block_threads();
// The staged (TMA) pass over a.tiles with `grid` persistent CTAs.
void launch_tpass(const Variant &v, int mode, const PassArgs &a, int grid, cudaStream_t st);
// Dynamic shared memory of the staged pass for a stage size, and the CTAs
// per SM it reaches (0 if it cannot run).
int tpass_smem_bytes(int stage_bytes);
int tpass_blocks_per_sm(const Variant &v, int mode, int stage_bytes);
void launch_flush(const FlushArgs &f, int nrep, cudaStream_t st);
void launch_measure_out(const RepDev *reps, double *ring, int ring_cap, int nrep, double *out, cudaStream_t st);
void launch_aos_to_split(const RepDev &R, const float *aos, float *dir, cudaStream_t st);
void launch_split_to_aos(const RepDev &R, const float *dir, float *aos, cudaStream_t st);
void launch_mask_to_split(const RepDev &R, const int *pt_aos, const float *ns_aos, uint8_t *pt, float *ns,
                          cudaStream_t st);
void launch_split_to_mask(const RepDev &R, const uint8_t *pt, const float *ns, int *pt_aos, float *ns_aos,
                          cudaStream_t st);
void launch_init(const RepDev &R, const uint8_t *pt, float *dir, int mode, uint32_t seed, float fx, float fy, float fz,
                 cudaStream_t st);
// Sum of every site's director (3 doubles at out).
void launch_polarization(const RepDev &R, const float *dir, double *out, cudaStream_t st);
// out: the MCX_COMBINED_LEN doubles of mcx_combine_stats, then the count of
// listed replicas without measured sweeps.
void launch_combine(const RepDev *rep, const RepState *st, const double *stats, const double *pol, const int *idx,
                    int n, double *out, cudaStream_t s);
// Per-site local order parameter (natural order; NaN at inactive sites).
void launch_local_order(const RepDev &R, const float *dir, const uint8_t *pt, float *out, cudaStream_t st);

// The network on n rows of 19 inputs -> n x 4 outputs (mcx_tcmlp.cu): on the
// tcgen05 tensor cores (accumulators in TMEM) or with the learned passes'
// warp-level mma.sync code; err receives bit 4 when an MMA wait ran out.
cudaError_t launch_mlp_forward(const uint8_t *mlp, const float *in, int n, float *out, int tensor_cores,
                               unsigned *err, cudaStream_t st);

// Training of the learned proposal's network (mcx_train.cu).
int train_smem_bytes();
int sample_floats();
cudaError_t launch_collect(const RepDev *reps, const RepState *st, const float *dir, const uint8_t *pt, float *out,
                           const int *rep_of, int n, uint32_t seed, int augment, cudaStream_t s);
cudaError_t launch_mlp_grad(const float *w, const float *samples, const int *index, int n, float *grad, float *loss,
                            int grid, cudaStream_t s);
cudaError_t launch_adam(float *w, float *m, float *v, const float *g, int step, float lr, cudaStream_t s);
cudaError_t launch_batch_index(int *idx, int n, int nsamples, uint32_t seed, uint32_t step, cudaStream_t s);

}  // namespace mcx
