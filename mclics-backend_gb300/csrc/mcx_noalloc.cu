// mcx_noalloc.cu -- mcx_measure_noalloc: E, Q and S of a director field that
// the caller already holds in device memory, computed without allocating.
//
// Some callers cannot allocate device memory when they need a measurement: a
// host framework that owns every device allocation through its own pool and
// forbids others, or a caller inside a latency-critical loop where a
// cudaMalloc would synchronise the device.  This entry point takes the
// caller's buffers (directors, optional point types and normals, an output of
// 16 doubles) and keeps its only working memory -- the per-block partial sums
// of the reduction -- in a fixed file-scope device array.  That array lives on
// every GPU that loads the library until the process exits.
//
// It is the allocation-free variant of the engine's measurement (the E/Q sums
// of mcx_measure): every site adds its local energy (the reference's
// energy_calculator, src/evolve.cpp:27-62) and its Q-tensor terms
// (Matrice_constructor, src/parameter_order.cpp:30-60); the last block folds
// the partial sums in a fixed order and solves the 3x3 eigenproblem in FP64.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "../../include/mcx.h"
#include "mcx_device.cuh"
#include "mcx_host.h"

namespace mcx {
namespace {

constexpr int kNaThreads = 256;
constexpr int kNaBlocks = MCX_NOALLOC_MAX_BLOCKS;
constexpr int kNaQ = 8;  // E_all, E_valid, xx, xy, xz, yy, yz, active count
constexpr int kMaxDevices = 64;

// The shared working memory of every call: one row of partial sums per
// block, and the count of blocks that have finished.  Host code must not use
// these names as device addresses; it asks cudaGetSymbolAddress once per
// device.
static __device__ __align__(256) double g_na_partial[kNaBlocks][kNaQ];
static __device__ __align__(256) unsigned int g_na_done;

struct NaParams {
  int nx, ny, nz;
  int xb, yb, zb;
  int pot;
  float A, lam, mu, nu, rho, sigma;
  float B1, C;  // Pear
  float elecA, elecE, ex, ey, ez;
  int nsurf;
  int anch[kMaxSurf];
  float W[kMaxSurf];
  float dx[kMaxSurf], dy[kMaxSurf], dz[kMaxSurf];
};

// The replica view the shared energy functions expect.
__device__ __forceinline__ RepDev as_rep(const NaParams &p) {
  RepDev R;
  R.A = p.A;
  R.B1 = p.B1;
  R.C = p.C;
  R.lam = p.lam;
  R.mu = p.mu;
  R.nu = p.nu;
  R.rho = p.rho;
  R.sigma = p.sigma;
  R.elecA = p.elecA;
  R.elecE = p.elecE;
  R.ex = p.ex;
  R.ey = p.ey;
  R.ez = p.ez;
  R.nsurf = p.nsurf;
  for (int s = 0; s < kMaxSurf; s++) {
    R.anch[s] = p.anch[s];
    R.W[s] = p.W[s];
    R.dx[s] = p.dx[s];
    R.dy[s] = p.dy[s];
    R.dz[s] = p.dz[s];
  }
  return R;
}

// Bond energy of director a with its neighbour b in slot d (x+, x-, y+, y-,
// z+, z-; r = +-e_axis): Lebwohl-Lasher, Pear and GHRL (src/potential.cpp:10-38).
__device__ __forceinline__ float pair_energy(const RepDev &R, int pot, int d, float ax, float ay, float az, float bx,
                                             float by, float bz) {
  if (pot == POT_LL) {
    const float nij = ax * bx + ay * by + az * bz;
    return -1.5f * R.A * nij * nij;
  }
  if (pot == POT_PEAR) {
    // -A nij^2 - B1 nij - (C/4)(1 + 2 nij + nij^2)((b - a) . r)
    const float nij = ax * bx + ay * by + az * bz;
    const int x = d >> 1;
    const float dr = (x == 0 ? bx - ax : (x == 1 ? by - ay : bz - az)) * ((d & 1) ? -1.f : 1.f);
    return -R.A * nij * nij - R.B1 * nij - (R.C * 0.25f) * ((1.f + 2.f * nij + nij * nij) * dr);
  }
  const float sg = (d & 1) ? -1.f : 1.f;
  switch (d >> 1) {
    case 0: return ghrl_bond<0>(R, ax, ay, az, bx, by, bz, sg);
    case 1: return ghrl_bond<1>(R, ax, ay, az, bx, by, bz, sg);
    default: return ghrl_bond<2>(R, ax, ay, az, bx, by, bz, sg);
  }
}

// Largest eigenvalue and unit eigenvector of a symmetric 3x3 matrix, cyclic
// Jacobi in FP64 (Golub & Van Loan, sec. 8.5).
__device__ void na_jacobi(const double Qin[9], double &lam, double vec[3]) {
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

__global__ void __launch_bounds__(kNaThreads) k_measure_noalloc(NaParams p, const float *__restrict__ ni,
                                                                const int *__restrict__ pt,
                                                                const float *__restrict__ ns, double *out,
                                                                double (*partial)[kNaQ], unsigned *done) {
  const RepDev R = as_rep(p);
  const long long n = (long long)p.nx * p.ny * p.nz;
  double acc[kNaQ] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (long long s = (long long)blockIdx.x * kNaThreads + threadIdx.x; s < n; s += (long long)gridDim.x * kNaThreads) {
    const int i = (int)(s % p.nx);
    const long long row = s / p.nx;
    const int j = (int)(row % p.ny), k = (int)(row / p.ny);
    const int ps = pt ? pt[s] : 1;
    const float x = ni[3 * s], y = ni[3 * s + 1], z = ni[3 * s + 2];
    float e = 0.f;
    const int ci[6] = {i + 1, i - 1, j + 1, j - 1, k + 1, k - 1};
    for (int d = 0; d < 6; d++) {
      const int ax = d >> 1;
      const int N = ax == 0 ? p.nx : (ax == 1 ? p.ny : p.nz);
      const int b = ax == 0 ? p.xb : (ax == 1 ? p.yb : p.zb);
      int q = ci[d];
      if (q < 0 || q >= N) {
        if (b != BOUND_PERIODIC) continue;
        q = (q + N) % N;
      }
      const long long t = ax == 0 ? (long long)q + (long long)p.nx * row
                                  : (ax == 1 ? (long long)i + (long long)p.nx * ((long long)q + (long long)p.ny * k)
                                             : (long long)i + (long long)p.nx * ((long long)j + (long long)p.ny * q));
      if (pt && pt[t] == 0) continue;
      e += pair_energy(R, p.pot, d, x, y, z, ni[3 * t], ni[3 * t + 1], ni[3 * t + 2]);
    }
    if (ps > 1 && ps - 2 < p.nsurf) {
      const float sx = ns ? ns[3 * s] : 0.f, sy = ns ? ns[3 * s + 1] : 0.f, sz = ns ? ns[3 * s + 2] : 0.f;
      e += surface_energy(R, ps - 2, x, y, z, sx, sy, sz);
    }
    if (p.elecA != 0.f) e += field_energy(R, x, y, z);
    acc[0] += e;
    if (ps != 0) {
      acc[1] += e;
      acc[2] += (double)(x * x);
      acc[3] += (double)(x * y);
      acc[4] += (double)(x * z);
      acc[5] += (double)(y * y);
      acc[6] += (double)(y * z);
      acc[7] += 1.0;
    }
  }
  __shared__ double red[kNaThreads / 32][kNaQ];
  __shared__ unsigned s_last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int q = 0; q < kNaQ; q++) {
    double v = acc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < kNaQ) {
    double v = 0;
    for (int w = 0; w < kNaThreads / 32; w++) v += red[w][threadIdx.x];
    partial[blockIdx.x][threadIdx.x] = v;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last || threadIdx.x != 0) return;
  __threadfence();
  double m[kNaQ] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (unsigned b = 0; b < gridDim.x; b++)
    for (int q = 0; q < kNaQ; q++) m[q] += partial[b][q];
  const double valid = m[7];
  const double dd = 2.0 * valid;
  double Q[9];
  Q[0] = (3.0 * m[2] - valid) / dd;
  Q[1] = 3.0 * m[3] / dd;
  Q[2] = 3.0 * m[4] / dd;
  Q[4] = (3.0 * m[5] - valid) / dd;
  Q[5] = 3.0 * m[6] / dd;
  Q[3] = Q[1];
  Q[6] = Q[2];
  Q[7] = Q[5];
  Q[8] = -Q[0] - Q[4];
  out[0] = m[0] / (double)n;
  out[1] = valid > 0 ? m[1] / valid : 0.0;
  for (int q = 0; q < 9; q++) out[2 + q] = Q[q];
  double lam, v[3];
  na_jacobi(Q, lam, v);
  out[11] = lam;
  out[12] = v[0];
  out[13] = v[1];
  out[14] = v[2];
  out[15] = valid;
  *done = 0;  // leave the counter at zero for the next call
}

// Device addresses of the shared scratch, looked up once per device.
std::mutex g_na_mutex;
double (*g_na_partial_ptr[kMaxDevices])[kNaQ];
unsigned *g_na_done_ptr[kMaxDevices];

}  // namespace
}  // namespace mcx

using namespace mcx;

extern "C" mcx_status mcx_measure_noalloc(const mcx_replica_desc *desc, const float *d_ni, const int *d_pt,
                                          const float *d_ns, double *d_out, void *stream) {
  if (!desc || !d_ni || !d_out) {
    set_last_error("mcx_measure_noalloc: desc, directors and output are required");
    return MCX_ERR_INVALID;
  }
  if (desc->nx < 1 || desc->ny < 1 || desc->nz < 1) {
    set_last_error("mcx_measure_noalloc: lattice dimensions must be positive");
    return MCX_ERR_INVALID;
  }
  const long long n = (long long)desc->nx * desc->ny * desc->nz;
  if (n > MCX_NOALLOC_MAX_SITES) {
    char buf[160];
    snprintf(buf, sizeof buf, "mcx_measure_noalloc: %lld sites exceed the maximum of %d", n, MCX_NOALLOC_MAX_SITES);
    set_last_error(buf);
    return MCX_ERR_INVALID;
  }
  if (desc->potential < MCX_POT_LL || desc->potential > MCX_POT_PEAR) {
    char buf[120];
    snprintf(buf, sizeof buf, "mcx_measure_noalloc: unknown potential %d (0 LL, 1 GHRL, 2 Pear)", desc->potential);
    set_last_error(buf);
    return MCX_ERR_INVALID;
  }
  if (desc->n_surfaces < 0 || desc->n_surfaces > MCX_MAX_SURFACES) {
    char buf[120];
    snprintf(buf, sizeof buf, "mcx_measure_noalloc: surface count %d outside [0, %d]", desc->n_surfaces,
             MCX_MAX_SURFACES);
    set_last_error(buf);
    return MCX_ERR_INVALID;
  }
  for (int s = 0; s < desc->n_surfaces; s++)
    if (desc->anchoring[s] < MCX_ANCH_HOMEOTROPIC || desc->anchoring[s] > MCX_ANCH_STRONG_GHRL) {
      char buf[120];
      snprintf(buf, sizeof buf, "mcx_measure_noalloc: unknown anchoring %d on surface %d", desc->anchoring[s], s);
      set_last_error(buf);
      return MCX_ERR_INVALID;
    }
  int dev = 0;
  cudaError_t rc = cudaGetDevice(&dev);
  if (rc != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_last_error("mcx_measure_noalloc: no usable current device");
    return MCX_ERR_CUDA;
  }
  {
    // first call on this device (with it current): find the scratch's device
    // addresses; later calls reuse them
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_partial_ptr[dev]) {
      void *pp = nullptr, *pd = nullptr;
      rc = cudaGetSymbolAddress(&pp, g_na_partial);
      if (rc == cudaSuccess) rc = cudaGetSymbolAddress(&pd, g_na_done);
      if (rc != cudaSuccess) {
        char buf[200];
        snprintf(buf, sizeof buf, "mcx_measure_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(rc));
        set_last_error(buf);
        return MCX_ERR_CUDA;
      }
      g_na_partial_ptr[dev] = reinterpret_cast<double (*)[kNaQ]>(pp);
      g_na_done_ptr[dev] = reinterpret_cast<unsigned *>(pd);
    }
  }
  NaParams p;
  memset(&p, 0, sizeof p);
  p.nx = desc->nx;
  p.ny = desc->ny;
  p.nz = desc->nz;
  p.xb = desc->xbound;
  p.yb = desc->ybound;
  p.zb = desc->zbound;
  if (desc->geometry == MCX_GEO_SLAB) p.zb = MCX_BOUND_FREE;
  if (desc->geometry == MCX_GEO_SPHERE) p.xb = p.yb = p.zb = MCX_BOUND_FREE;
  p.pot = desc->potential;
  p.A = desc->A;
  p.B1 = desc->B1;
  p.C = desc->C;
  float g[5] = {0, 0, 1, 0, 0};
  if (desc->potential == MCX_POT_GHRL) ghrl_constants(desc->k11, desc->k22, desc->k33, desc->p0, g);
  p.lam = g[0];
  p.mu = g[1];
  p.nu = g[2];
  p.rho = g[3];
  p.sigma = g[4];
  p.elecA = desc->elecA;
  p.elecE = desc->elecE;
  p.ex = desc->elecX;
  p.ey = desc->elecY;
  p.ez = desc->elecZ;
  p.nsurf = desc->n_surfaces;
  for (int s = 0; s < desc->n_surfaces; s++) {
    p.anch[s] = desc->anchoring[s];
    p.W[s] = desc->W[s];
    float ax[3];
    anchoring_axis(desc->theta_s[s], desc->phi_s[s], ax);
    p.dx[s] = ax[0];
    p.dy[s] = ax[1];
    p.dz[s] = ax[2];
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const long long want = (n + kNaThreads - 1) / kNaThreads;
  const int grid = (int)(want < kNaBlocks ? want : kNaBlocks);
  // the block counter must start at zero: a call that stopped part way would
  // have left it elsewhere
  rc = cudaMemsetAsync(g_na_done_ptr[dev], 0, sizeof(unsigned), st);
  if (rc == cudaSuccess) {
    k_measure_noalloc<<<grid, kNaThreads, 0, st>>>(p, d_ni, d_pt, d_ns, d_out, g_na_partial_ptr[dev],
                                                    g_na_done_ptr[dev]);
    rc = cudaGetLastError();
  }
  if (rc != cudaSuccess) {
    char buf[200];
    snprintf(buf, sizeof buf, "mcx_measure_noalloc: %s", cudaGetErrorString(rc));
    set_last_error(buf);
    return MCX_ERR_CUDA;
  }
  return MCX_OK;
}
