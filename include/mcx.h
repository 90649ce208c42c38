/*
 * mcx.h -- C ABI of the GB300 Metropolis engine for the McLiCS nematic
 * lattice model (Lebwohl-Lasher / GHRL pair energies, electric field,
 * bulk / slab / sphere / custom geometries with surface anchoring).
 *
 * Plain C types only: pointers, sizes, enums.  Directors cross the boundary
 * in the reference's AoS layout ni[(i + Nx*(j + Ny*k))*3 + c]
 * (include/define.h:10-12 of the reference); the engine keeps them on the
 * GPU in a split red/black SoA layout and converts at the boundary.
 *
 * What each entry point replaces in the reference (paths relative to the
 * McLiCS project root):
 *
 *   mcx_create        EvolveNGPU construction + one-time device setup:
 *                     simulator::Setup_simmulation (src/simulatorGPU.cpp:24-108),
 *                     thermalEvolveNGPU::run device allocation/copies and
 *                     initRNG (src/evolve_thermal.cu:44-64), setGPUup/
 *                     setSurfaces/passGPUns (src/evolve.cu:205-263,275-341),
 *                     setGHRL (src/io.cpp:277-302).  Replaces the
 *                     one-lattice-per-process statics with a batch of
 *                     replicas of any sizes.
 *   mcx_set_state     cudaMemcpy(d_ni, ni, ...) (src/evolve_thermal.cu:58)
 *   mcx_get_state     cudaMemcpy(ni, d_ni, ...) (src/evolve_thermal.cu:90,96)
 *   mcx_set_mask      Geometry::set_point_type_normals for custom geometry
 *                     (src/geometry_custom.cpp:57-128) and the pt/ns uploads
 *                     (src/evolve_thermal.cu:59, src/evolve.cu:321-325)
 *   mcx_set_temperature  cudaMemcpy(d_T, &params->T, ...) (src/evolve_thermal.cu:80)
 *   mcx_set_field     params->elecE stepping (src/evolve_electric.cpp:59)
 *   mcx_sweep         EvolveNGPU::Monte_Carlo_Step_GPU (src/evolve.cu:265-388)
 *                     / EvolveN::Monte_Carlo_Step (src/evolve.cpp:64-179),
 *                     n times, with the step-size rule applied on the GPU;
 *                     with measure != 0 also energy_calculator_GPU
 *                     (src/evolve.cu:390-436) + Matrice_constructor +
 *                     Eigen_value_evaluation (src/parameter_order.cpp:11-60)
 *                     after every sweep, accumulated as the run loops do
 *                     (src/evolve_thermal.cpp:66-79).
 *   mcx_measure       one energy_calculator + Matrice_constructor +
 *                     Eigen_value_evaluation on the current state.
 *   mcx_get_stats     the S1/S2/E/E2 means written to po.dat
 *                     (src/evolve_thermal.cpp:80-87).
 *   mcx_run_file      ./mc_sim <paramfile> (src/main.cpp:63-83) with
 *                     evol thermalGPU / electricGPU / stepGPU / quenchGPU
 *                     (also accepted: thermalGB300 etc.).
 *
 * Errors are returned as status codes (the reference calls exit(n)); the
 * message of the last failure is available from mcx_last_error().  An engine
 * handle is single-threaded and owns one CUDA stream; every call that returns
 * host data synchronises that stream.
 */
#ifndef MCX_H_
#define MCX_H_

#ifdef __cplusplus
extern "C" {
#endif

#define MCX_MAX_SURFACES 16
#define MCX_MEASURE_LEN 16
#define MCX_STATS_LEN 16

typedef enum {
  MCX_OK = 0,
  MCX_ERR_INVALID = 1,     /* bad argument (sizes, enums, replica index) */
  MCX_ERR_CUDA = 2,        /* a CUDA call failed; see mcx_last_error */
  MCX_ERR_NOMEM = 3,       /* device or host allocation failed */
  MCX_ERR_UNSUPPORTED = 4, /* a configuration the engine does not run */
  MCX_ERR_IO = 5,          /* file could not be read or written */
  MCX_ERR_PARSE = 6        /* parameter or geometry file is malformed */
} mcx_status;

typedef enum { MCX_POT_LL = 0, MCX_POT_GHRL = 1, MCX_POT_PEAR = 2 } mcx_potential;
typedef enum { MCX_GEO_BULK = 0, MCX_GEO_SLAB = 1, MCX_GEO_SPHERE = 2, MCX_GEO_CUSTOM = 3 } mcx_geometry;
typedef enum { MCX_BOUND_FREE = 0, MCX_BOUND_PERIODIC = 1 } mcx_bound;
typedef enum {
  MCX_ANCH_HOMEOTROPIC = 0,      /* -W (n.s)^2, s = surface normal */
  MCX_ANCH_FG = 1,               /* +W (n.s)^2 (planar) */
  MCX_ANCH_RP = 2,               /* -W (n.d)^2, d from (theta_s, phi_s) */
  MCX_ANCH_STRONG = 3,           /* -W (n.d)^2 */
  MCX_ANCH_HOMEOTROPIC_GHRL = 4, /* W * GHRL bond form against s */
  MCX_ANCH_FG_GHRL = 5,
  MCX_ANCH_RP_GHRL = 6,
  MCX_ANCH_STRONG_GHRL = 7
} mcx_anchoring;

/* One replica: a lattice, its physics and its Monte Carlo state.  Field
 * names follow the reference's parameter keys (include/parameters.h:11-83). */
typedef struct {
  int nx, ny, nz;
  int geometry;                /* mcx_geometry */
  int xbound, ybound, zbound;  /* mcx_bound; slab forces z free, sphere all free */
  int potential;               /* mcx_potential */
  float A;                     /* LL coupling */
  float k11, k22, k33, p0;     /* GHRL elastic constants and pitch (0 = achiral) */
  float elecA;                 /* dielectric anisotropy; 0 disables the field term */
  float elecX, elecY, elecZ;   /* field direction (not normalised, as in the reference) */
  float elecE;                 /* field strength */
  float T;                     /* temperature */
  float ang_var;               /* initial step size (the reference starts at 0.5) */
  unsigned int seed;           /* Philox key word 0 */
  unsigned int stream;         /* Philox key word 1; distinct per replica */
  int n_surfaces;
  int anchoring[MCX_MAX_SURFACES]; /* mcx_anchoring, per surface id (pt - 2) */
  float W[MCX_MAX_SURFACES];
  float theta_s[MCX_MAX_SURFACES]; /* degrees */
  float phi_s[MCX_MAX_SURFACES];   /* degrees */
  float radius;                /* sphere: droplet radius; 0 = Nz/2 as the reference */
  float B1, C;                 /* Pear (splay-bend) potential: polar and splay couplings */
} mcx_replica_desc;

typedef struct mcx_engine mcx_engine;

/* mcx_measure() output layout (MCX_MEASURE_LEN doubles). */
enum {
  MCX_M_E = 0,        /* energy per site over all sites, the CPU path's E (src/evolve.cpp:27-62) */
  MCX_M_E_VALID = 1,  /* energy per active site (the GPU path's normalisation) */
  MCX_M_Q = 2,        /* 9 entries, row-major Q-tensor */
  MCX_M_S = 11,       /* largest eigenvalue of Q */
  MCX_M_DIRECTOR = 12,/* 3 entries: its unit eigenvector */
  MCX_M_VALID = 15    /* number of active sites */
};

/* mcx_get_stats() output layout (MCX_STATS_LEN doubles), sums over measured
 * sweeps since the last reset. */
enum {
  MCX_ST_N = 0,        /* measured sweeps */
  MCX_ST_S1 = 1,       /* sum S */
  MCX_ST_S2 = 2,       /* sum S^2 */
  MCX_ST_E1 = 3,       /* sum E (all-site normalisation) */
  MCX_ST_E2 = 4,       /* sum E^2 */
  MCX_ST_EV1 = 5,      /* sum E_valid */
  MCX_ST_EV2 = 6,      /* sum E_valid^2 */
  MCX_ST_ACC = 7,      /* accepted moves, all sweeps since reset */
  MCX_ST_SWEEPS = 8,   /* sweeps since reset */
  MCX_ST_LAST_E = 9,   /* last measured E */
  MCX_ST_LAST_S = 10,  /* last measured S */
  MCX_ST_ANG_VAR = 11, /* current step size */
  MCX_ST_SWEEP_INDEX = 12 /* total sweeps done (the RNG counter) */
};

int mcx_version(void);

/* Allocates the device state for n_replicas replicas (any sizes; an axis that
 * is periodic after the geometry forces the bounds must have even length, as
 * red/black sweeps need -- MCX_ERR_UNSUPPORTED otherwise) and fills the
 * geometry masks of bulk/slab/sphere replicas.  Directors start along +z; use mcx_set_state or
 * mcx_init_random / mcx_init_homogeneous to set them. */
mcx_status mcx_create(int n_replicas, const mcx_replica_desc *descs, mcx_engine **out);
void mcx_destroy(mcx_engine *eng);
/* Message of the last failure on this engine (eng == NULL: of the last
 * failed mcx_create / mcx_run_file). */
const char *mcx_last_error(const mcx_engine *eng);

int mcx_num_replicas(const mcx_engine *eng);
/* Copies a replica's descriptor as the engine uses it (bounds forced by the
 * geometry, GHRL constants derived). ghrl_out (5 floats: lambda, mu, nu, rho,
 * sigma) may be NULL. */
mcx_status mcx_get_desc(const mcx_engine *eng, int replica, mcx_replica_desc *desc, float *ghrl_out);

mcx_status mcx_set_state(mcx_engine *eng, int replica, const float *ni_aos);
mcx_status mcx_get_state(mcx_engine *eng, int replica, float *ni_aos);
/* Random directors uniform on the sphere (Philox keyed by seed, replica) and
 * (0,0,1) on inactive sites (src/ic.cpp:27-59); homogeneous along
 * (theta_0, phi_0) in degrees (src/ic.cpp:61-86). */
mcx_status mcx_init_random(mcx_engine *eng, int replica, unsigned int seed);
mcx_status mcx_init_homogeneous(mcx_engine *eng, int replica, float theta_0, float phi_0);

/* pt: int per site (0 inactive, 1 bulk, >= 2 surface id + 2); ns_aos: surface
 * normal per site (may be NULL: zeros). */
mcx_status mcx_set_mask(mcx_engine *eng, int replica, const int *pt, const float *ns_aos);
mcx_status mcx_get_mask(mcx_engine *eng, int replica, int *pt, float *ns_aos);

/* replica = -1 applies to every replica. */
mcx_status mcx_set_temperature(mcx_engine *eng, int replica, float T);
mcx_status mcx_set_field(mcx_engine *eng, int replica, float elecE);
mcx_status mcx_set_step(mcx_engine *eng, int replica, float ang_var);
/* on = 0 freezes the step size (the reference adapts it after every sweep
 * towards 50% acceptance, src/evolve.cpp:169-178; a frozen step keeps the
 * chain time-homogeneous for autocorrelation measurements); 1 restores the
 * reference's rule (the default).  No counterpart in the reference. */
mcx_status mcx_set_adapt(mcx_engine *eng, int replica, int on);

/* n_sweeps red/black Metropolis sweeps of every replica, on the engine's
 * stream (asynchronous).  measure != 0 measures E, Q and S after every sweep
 * and adds them to the running sums read by mcx_get_stats. */
mcx_status mcx_sweep(mcx_engine *eng, int n_sweeps, int measure);
mcx_status mcx_sync(mcx_engine *eng);
mcx_status mcx_measure(mcx_engine *eng, int replica, double *out /* MCX_MEASURE_LEN */);
mcx_status mcx_get_stats(mcx_engine *eng, int replica, double *out /* MCX_STATS_LEN */);
mcx_status mcx_reset_stats(mcx_engine *eng, int replica);

/* Records E and S of every measured sweep of every replica in a device ring
 * of `capacity` sweeps (0 disables); mcx_get_series copies the last `count`
 * values (E then S interleaved per sweep) of one replica. */
mcx_status mcx_set_series(mcx_engine *eng, int capacity);
mcx_status mcx_get_series(mcx_engine *eng, int replica, int count, double *es_out);

/* One red/black pass (colour 0 or 1) of one replica with a trace: per site
 * (AoS order) the float energy change, the decision and the proposed
 * director.  Sites not updated in the pass get dE = 0, acc = 255.  Used by
 * the parity tests; does not advance the RNG counter or the step size. */
mcx_status mcx_debug_pass(mcx_engine *eng, int replica, int colour, float *dE, unsigned char *acc,
                          float *proposal_aos);

/* Kernel launches issued by this engine since creation (sweep, measure and
 * epilogue kernels; graph launches count each kernel node). */
long long mcx_kernel_launches(const mcx_engine *eng);

/* Chooses the sweep kernel: on != 0 the staged pass (tiles of rows brought
 * into shared memory by TMA bulk copies, double-buffered, persistent CTAs),
 * 0 the direct pass (each thread loads its neighbours from global memory).
 * The direct pass is the default (it measures faster on the lattices
 * benchmarked so far); the staged pass needs every replica's tile to fit in
 * shared memory.  Both compute the same update (see mcx_set_pass). */
mcx_status mcx_set_staged(mcx_engine *eng, int on);
int mcx_get_staged(const mcx_engine *eng);

/* The kernel that runs the plain proposal's sweeps.  All compute the same
 * update from the same Philox counters with every rounding of the energy
 * change fixed, so every form and shape runs the same chain bit for bit
 * (states, step sizes, acceptance counts; the measured sums agree to FP32
 * summation order): the autotuner's choice changes the speed, never the
 * trajectory.
 *
 *   MCX_PASS_MARCH   the default: a CTA marches a block of same-colour site
 *                    pairs of one z-plane through a chunk of planes, keeping
 *                    the z neighbours in registers;
 *   MCX_PASS_DIRECT  persistent CTAs, each pair's neighbourhood loaded by
 *                    cp.async into shared memory;
 *   MCX_PASS_STAGED  the staged TMA pass above (mcx_set_staged);
 *   MCX_PASS_MARCH_TMA  the z-march with each plane's rows brought into
 *                    shared memory by bulk copies one plane ahead (unmasked
 *                    batches only);
 *   MCX_PASS_MARCH_ASYNC  the z-march with every thread copying its next
 *                    plane's neighbourhood into shared memory by cp.async
 *                    while it updates the current plane (unmasked LL and GHRL
 *                    batches only);
 *   MCX_PASS_MARCH_PERSISTENT  the z-march as one cooperative launch per run
 *                    of sweeps, its passes separated by grid barriers (blocks
 *                    of 128 or 256 threads; one wave of units);
 *   MCX_PASS_MARCH_QUAD  the z-march with four same-colour sites (two pairs)
 *                    per thread and 16-byte loads (unmasked batches with nx a
 *                    multiple of 8).
 * No counterpart in the reference. */
typedef enum {
  MCX_PASS_MARCH = 0,
  MCX_PASS_DIRECT = 1,
  MCX_PASS_STAGED = 2,
  MCX_PASS_MARCH_TMA = 3,
  MCX_PASS_MARCH_ASYNC = 4,
  MCX_PASS_MARCH_PERSISTENT = 5,
  MCX_PASS_MARCH_QUAD = 6
} mcx_pass_kind;
mcx_status mcx_set_pass(mcx_engine *eng, int kind);
int mcx_get_pass(const mcx_engine *eng);
/* The z-march pass's shape: CTA size (64, 128 or 256 threads, one site pair
 * each) and chunk depth (planes per CTA; planes <= 0 cuts near-equal chunks
 * so that the work units fill max(1, -planes) waves of the CTAs the GPU holds
 * at once).  Default 128 x 8. */
mcx_status mcx_set_march_shape(mcx_engine *eng, int block, int planes);
/* Autotuner: times the z-march pass (register and, for unmasked batches,
 * TMA-staged forms) for block sizes {64, 128, 256} and chunk
 * depths {1, 2, 4, ..., 32} (up to the deepest lattice) and balanced chunks
 * over 1 to 4 waves (planes 0, -2, -3, -4) on a scratch copy of
 * the engine's state (the state itself is untouched), keeps the fastest and
 * reports it (any output may be NULL).  Synchronous. */
mcx_status mcx_autotune(mcx_engine *eng, int *block, int *planes, float *pass_us);

/* Learned proposal (no counterpart in the reference).  A small network reads
 * a site's six neighbour directors and T (19 inputs) and gives the mean axis
 * and log-concentration of an antipodal von Mises-Fisher mixture,
 * q(n') = kappa/(4 pi sinh kappa) cosh(kappa mu.n'); sweeps with
 * MCX_PROPOSAL_VMF_MLP draw n' from it and accept with the exact
 * Metropolis-Hastings ratio exp(-dE/T) cosh(kappa mu.n)/cosh(kappa mu.n'),
 * so the stationary distribution is the same as with the plain rotation
 * (MCX_PROPOSAL_PLAIN, the default and the reference's move).
 * Weights (MCX_MLP_PARAMS floats, row index = input):
 *   W1 [32][64] (input rows 19..31 zero), b1 [64], W2 [64][64], b2 [64],
 *   W3 [64][8] (output columns 4..7 zero), b3 [8];
 * inputs are the neighbours x+ x- y+ y- z+ z- (3 each, zero when absent or
 * inactive) then T; outputs mu (3) and log kappa (clamped to [-4, 6]).
 * The network runs in BF16 with FP32 accumulation on the tensor cores. */
typedef enum { MCX_PROPOSAL_PLAIN = 0, MCX_PROPOSAL_VMF_MLP = 1 } mcx_proposal;
#define MCX_MLP_PARAMS 6792
int mcx_mlp_params(void);
mcx_status mcx_set_mlp(mcx_engine *eng, const float *weights, int n);
mcx_status mcx_get_mlp(mcx_engine *eng, float *weights);
mcx_status mcx_set_proposal(mcx_engine *eng, int kind);
/* mcx_debug_pass plus, per site, the network's 4 outputs (learned proposal;
 * mlp_out may be NULL). */
mcx_status mcx_debug_pass_mlp(mcx_engine *eng, int replica, int colour, float *dE, unsigned char *acc,
                              float *proposal_aos, float *mlp_out);

/* Training of the learned proposal on the GPU (no counterpart in the
 * reference).  A training sample is MCX_SAMPLE_FLOATS floats: the 19 network
 * inputs of one active site, its director (3), then the replica and the
 * site's natural index (x + nx (y + ny z)) as int32 bit patterns.  The loss is
 * the mean negative log-density of the directors under the mixture, i.e.
 * maximum likelihood of the conditional distribution of a site given its
 * neighbours when the states are in equilibrium.
 *
 * mcx_collect_samples draws n sites (uniformly among each replica's active
 * sites; replicas in turn by blocks of 256 samples) from the current states
 * and copies the samples to `out` (host, may be NULL to keep them on the
 * device only).  augment: MCX_AUG_FLIP flips each director's sign at random
 * (always a symmetry); MCX_AUG_ROTATE applies one uniform random rotation to
 * all 7 directors of a sample (a symmetry only of field-free Lebwohl-Lasher
 * replicas without surfaces, rejected otherwise).
 *
 * mcx_train_mlp collects cfg->samples samples (as above; 0 reuses the samples
 * the engine holds: its last collection or mcx_mlp_grad input) and runs cfg->steps
 * Adam steps (beta1 0.9, beta2 0.999, eps 1e-8) on minibatches of cfg->batch
 * drawn with replacement, starting from the current weights (mcx_set_mlp
 * first); the Adam moments persist across calls until mcx_set_mlp.  The
 * trained weights become the proposal's; loss (steps floats, may be NULL)
 * receives each step's minibatch loss.
 *
 * mcx_mlp_grad evaluates the loss and its gradient (MCX_MLP_PARAMS floats,
 * the weight layout) at the current weights over n host samples (only the
 * first 22 floats of each are read), with the training kernel. */
#define MCX_SAMPLE_FLOATS 24
enum { MCX_AUG_FLIP = 1, MCX_AUG_ROTATE = 2 };
typedef struct {
  int samples;
  int batch;
  int steps;
  float lr;
  unsigned int seed;
  int augment;
} mcx_train_config;
mcx_status mcx_collect_samples(mcx_engine *eng, int n, unsigned int seed, int augment, float *out);
mcx_status mcx_train_mlp(mcx_engine *eng, const mcx_train_config *cfg, float *loss);
mcx_status mcx_mlp_grad(mcx_engine *eng, const float *samples, int n, float *grad, float *loss);

/* The network set by mcx_set_mlp on n rows of its 19 inputs (host, n x 19
 * floats: the six neighbours x+ x- y+ y- z+ z- then T) -> outputs (host,
 * n x 4: mu, log kappa before its clamp), on the GPU; no counterpart in the
 * reference.  path MCX_MLP_TCGEN05 runs it on the 5th-generation tensor cores
 * (tcgen05.mma, FP32 accumulators in tensor memory, 128 rows per MMA tile);
 * MCX_MLP_WARP_MMA with the warp-level mma.sync code of the learned passes.
 * Both take BF16 inputs, weights and activations with FP32 accumulation and
 * the same GELU arithmetic; they differ only in the order of the FP32 sums. */
enum { MCX_MLP_WARP_MMA = 0, MCX_MLP_TCGEN05 = 1 };
mcx_status mcx_mlp_forward(mcx_engine *eng, const float *inputs, int n, float *outputs, int path);
/* Which code evaluates the network inside the learned z-march (the learned
 * proposal's sweep kernel): MCX_MLP_TCGEN05 evaluates each plane's 256 sites
 * of a CTA as two M = 128 tcgen05 tiles with the accumulators in tensor
 * memory; MCX_MLP_WARP_MMA, the default (measured faster), the warp-level
 * mma.sync code.  Call after mcx_set_mlp.  The two give the same outputs up
 * to the order of FP32 sums, so their chains part after a few sweeps but
 * sample the same law.  No counterpart in the reference. */
mcx_status mcx_set_mlp_path(mcx_engine *eng, int path);
int mcx_get_mlp_path(const mcx_engine *eng);

/* The engine's CUDA stream (a cudaStream_t), for callers that record events
 * or order their own work against the engine's. */
void *mcx_stream(mcx_engine *eng);

/* n_sweeps unmeasured sweeps launched one kernel at a time with CUDA events
 * around every red/black pass kernel; pass_ms receives the summed duration of
 * the 2*n_sweeps pass kernels, total_ms the whole sequence.  For profiling:
 * the sweeps are real (state, RNG counter and step size advance). */
mcx_status mcx_pass_timing(mcx_engine *eng, int n_sweeps, float *pass_ms, float *total_ms);
/* n_sweeps unmeasured sweeps through mcx_sweep's own path (captured graphs of
 * 16 sweeps) between two CUDA events on the engine's stream; ms receives the
 * elapsed time.  Divided by 2*n_sweeps it is the pass kernel's average
 * duration in the production launch sequence, launch gaps included.  The
 * sweeps are real (state, RNG counter and step size advance). */
mcx_status mcx_sweep_timing(mcx_engine *eng, int n_sweeps, float *ms);
/* Test of the persistent z-march's bounded grid-barrier wait: one launch
 * whose barriers cannot complete.  Every CTA gives up after its poll limit
 * (about a second), sets the error flag and leaves; returns MCX_ERR_CUDA with
 * the barrier message (MCX_ERR_INVALID when that pass kind is not selected).
 * The engine's directors are left mid-sweep. */
mcx_status mcx_debug_barrier_timeout(mcx_engine *eng);

/* Host-only helpers (no GPU needed). */
/* setGHRL (src/io.cpp:277-302): out = lambda, mu, nu, rho, sigma. */
void mcx_ghrl_constants(float k11, float k22, float k33, float p0, float *out5);
/* Geometry::set_point_type_normals of bulk / slab / sphere
 * (src/geometry_bulk.cpp:57-61, src/geometry_slab.cpp:47-67,
 * src/geometry_sphere.cpp:28-54) in AoS order; MCX_ERR_INVALID for custom. */
mcx_status mcx_build_mask(const mcx_replica_desc *desc, int *pt, float *ns_aos);
/* Custom geometry file (src/geometry_custom.cpp:57-128) for an nx*ny*nz
 * lattice; *n_surfaces receives max(pt) - 1. */
mcx_status mcx_read_geometry(const char *path, int nx, int ny, int nz, int *pt, float *ns_aos, int *n_surfaces);
/* Parses and validates a parameter file (src/io.cpp:81-253) without running
 * it; desc (may be NULL) receives replica 0's descriptor. */
mcx_status mcx_check_file(const char *param_file, mcx_replica_desc *desc);

/* Allocation-free measurement (no counterpart in the reference: a GB300
 * addition).  Some callers cannot allocate device memory when they need a
 * measurement -- a framework that owns every device allocation through its
 * own pool, or a latency-critical loop where cudaMalloc would synchronise the
 * device.  This computes the mcx_measure layout (MCX_MEASURE_LEN doubles, in
 * device memory at d_out) for a director field the caller already holds on
 * the device: d_ni_aos is 3 floats per site in the reference's AoS order;
 * d_pt (ints, NULL = every site active bulk) and d_ns_aos (NULL = zero
 * normals) likewise.  Boundaries are desc's, forced by its geometry as
 * mcx_create does.  It calls no cudaMalloc, cudaFree or allocating library
 * routine: its only working memory is a fixed file-scope device array of
 * MCX_NOALLOC_MAX_BLOCKS x 8 doubles plus a counter (68 KB), present on every
 * GPU that loads the library until the process exits.  The first call on a
 * device (made with that device current) looks up the array's device address
 * with cudaGetSymbolAddress; make that first call before any stream capture.
 * Every call shares the array: calls whose kernels overlap on the GPU (for
 * example on two streams at once) race and give wrong results; calls ordered
 * on one stream are safe.  Lattices above MCX_NOALLOC_MAX_SITES sites, and
 * descriptors with an unknown potential (LL, GHRL and Pear are measured) or
 * anchoring, are rejected with MCX_ERR_INVALID.  Asynchronous on `stream` (a
 * cudaStream_t, NULL = the default stream). */
#define MCX_NOALLOC_MAX_BLOCKS 1024
#define MCX_NOALLOC_MAX_SITES (1 << 27)
mcx_status mcx_measure_noalloc(const mcx_replica_desc *desc, const float *d_ni_aos, const int *d_pt,
                               const float *d_ns_aos, double *d_out, void *stream);

/* Polarization of a replica's current state, |sum of directors| / sites over
 * all sites (Polarization, src/parameter_order.cpp:142-155; the sixth po.dat
 * column of Pear runs). */
mcx_status mcx_polarization(mcx_engine *eng, int replica, double *P);

/* Local order parameter of every site of a replica (lattice_order_parameter,
 * src/parameter_order.cpp:62-113, as the snapshot writer print_n,
 * src/io.cpp:50-80, reports it): the largest eigenvalue of Q over the site and
 * its existing active neighbours; NaN at inactive sites.  S: one float per
 * site, natural order.  Computed on the GPU. */
mcx_status mcx_local_order(mcx_engine *eng, int replica, float *S);

/* print_n (src/io.cpp:50-80): writes a replica's current state as the
 * reference's snapshot file, header "x,y,z,nx,ny,nz,S,pt" and one
 * "%d,%d,%d,%g,%g,%g,%g,%d" line per site in natural order, S the local
 * order parameter (mcx_local_order; nan at inactive sites).  MCX_ERR_IO when
 * the file cannot be written. */
mcx_status mcx_print_n(mcx_engine *eng, int replica, const char *path);

/* Checkpoint (no counterpart in the reference): every replica's descriptor,
 * directors, mask, temperature, step size, sweep and measured-sweep counters
 * (the Philox counters: a loaded engine continues the saved trajectory bit
 * for bit), running sums, and the network weights and proposal when set.  The
 * measured-sweep series and the training optimiser state are not saved.
 * mcx_load needs an engine whose replicas have the saved descriptors
 * (everything but temperature and step size, which are restored: sizes,
 * geometry, bounds, potential, couplings, field, anchoring, RNG seed and
 * stream); otherwise MCX_ERR_INVALID.  It reads and checks the whole file
 * before changing anything, so a failed load leaves the engine as it was. */
mcx_status mcx_save(mcx_engine *eng, const char *path);
mcx_status mcx_load(mcx_engine *eng, const char *path);

/* Replica exchange (parallel tempering; no counterpart in the reference):
 * for each pair (pairs[2i], pairs[2i+1]) of replicas with the same
 * Hamiltonian (descriptors equal except T, step size and RNG keys), swap
 * their temperatures and step sizes with probability
 * min(1, exp((1/Ta - 1/Tb)(Ha - Hb))), H = E * sites the total energy of the
 * current states; the uniform is Philox4x32-10 of (i, round, TAG 4) with key
 * (seed, 0).  accepted (n ints, may be NULL) receives the decisions.  The
 * running sums stay with the replica (reset them after an exchange to gather
 * statistics per temperature). */
mcx_status mcx_exchange(mcx_engine *eng, int n_pairs, const int *pairs, unsigned int seed, unsigned long long round,
                        int *accepted);

/* mcx_combine_stats() output layout (MCX_COMBINED_LEN doubles). */
enum {
  MCX_CB_T = 0,        /* mean temperature of the combined replicas */
  MCX_CB_S = 1,        /* mean over replicas of their po.dat S */
  MCX_CB_VAR_S = 2,    /* mean of their varS + variance (ddof 0) of their S */
  MCX_CB_E = 3,        /* the same for E */
  MCX_CB_VAR_E = 4,
  MCX_CB_P = 5,        /* mean polarization of the current states (Pear), else NaN */
  MCX_CB_N = 6,        /* replicas combined */
  MCX_CB_T_SPREAD = 7  /* largest minus smallest temperature */
};
#define MCX_COMBINED_LEN 8

/* Combines independent replicas into one po.dat row on the GPU, the way
 * average_replicas.py:74-103 combines po.dat files of runs that differ only in
 * their seed: each replica's row is S = S1/N, varS = S2/N - S^2, E and varE
 * likewise (the columns of src/evolve_thermal.cpp:78-86 over its measured
 * sweeps); the combined row is the mean S, the law-of-total-variance
 * mean(varS) + var(S) and the same for E, and for Pear replicas the mean
 * polarization.  replicas: n indices (NULL with n <= 0: every replica).
 * Errors (MCX_ERR_INVALID): a replica without measured sweeps; Pear mixed
 * with other potentials (the script's differing column counts); temperatures
 * more than 1e-3 apart (a point the script skips) -- out is filled in that
 * last case, so the caller can see the spread. */
mcx_status mcx_combine_stats(mcx_engine *eng, int n, const int *replicas, double *out /* MCX_COMBINED_LEN */);

/* ./mc_sim <param_file> (src/main.cpp:63-83): reads the reference's parameter
 * file (src/io.cpp:81-253), runs the selected mode on the GPU and writes
 * po.dat and director_field_*.csv into out_dir (NULL: current directory). */
mcx_status mcx_run_file(const char *param_file, const char *out_dir);

#ifdef __cplusplus
}
#endif
#endif
