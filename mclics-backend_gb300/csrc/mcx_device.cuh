// mcx_device.cuh -- device-side building blocks of the GB300 Metropolis
// engine: replica table, Philox4x32-10, pair / anchoring / field energies.
//
// Director layout in HBM (per replica): a split red/black SoA.  Colour
// c = (i + j + k) & 1; colour c of row (j, k) holds the sites
// i = 2h + ((c + j + k) & 1), h = 0 .. hx-1 (hx = nx/2), stored at
//   dir[dir_off + (c*3 + comp)*plane + (j + ny*k)*hs + h],
// hs = hx rounded up to a multiple of 4 (16-byte rows), plane = hs*ny*nz.
// A red/black pass reads the whole other colour and reads + writes its own,
// each as coalesced float4 rows.  Point types (pt) use the same split layout
// as bytes; surface normals (ns) as floats.
#pragma once
#include <cstdint>

namespace mcx {

constexpr int kMaxSurf = 16;
constexpr int kBlock = 256;  // threads per CTA of the pass kernels: one site each
constexpr int kLanes = 8;    // atomic lanes per replica (spreads same-address atomics)
constexpr int kQ = 7;        // measured sums: E_all, E_valid, n_a n_b for xx xy xz yy yz

enum : int { POT_LL = 0, POT_GHRL = 1, POT_PEAR = 2 };
enum : int { BOUND_FREE = 0, BOUND_PERIODIC = 1 };
enum : int {
  ANCH_HOMEOTROPIC = 0,
  ANCH_FG = 1,
  ANCH_RP = 2,
  ANCH_STRONG = 3,
  ANCH_HOMEOTROPIC_GHRL = 4,
  ANCH_FG_GHRL = 5,
  ANCH_RP_GHRL = 6,
  ANCH_STRONG_GHRL = 7
};
// Philox counter word 3: which stream of uniforms.
// The pass colour is or-ed into the low bit.
enum : uint32_t { TAG_PLAIN = 0u, TAG_VMF = 2u, TAG_PT = 4u, TAG_IC = 0x1C000000u };

// Per-replica constants, resident in device memory (read-only in kernels).
struct RepDev {
  int nx, ny, nz;
  int hx, hs;  // half-row length, padded row stride (a multiple of 4)
  int xb, yb, zb;
  int nsurf;
  int valid;  // active sites
  int ntot;   // nx*ny*nz
  int hp;     // same-colour site pairs per row, (hx + 1) / 2
  int npair;  // pairs per colour, hp*ny*nz: one thread each
  int plane;  // elements per (colour, component) plane, hs*ny*nz
  int hps;    // point-type row stride in bytes (a multiple of 16)
  int pplane; // point-type bytes per colour, hps*ny*nz
  int ncta;   // CTAs of this replica in one direct pass launch
  int mcta;   // CTAs of this replica in one z-march pass launch
  int lcta;   // CTAs of this replica in one learned z-march pass launch
  uint32_t hp_m, ny_m;  // n / hp == (n * hp_m) >> hp_p for n < 2^31
  int hp_p, ny_p;
  // tiles of the staged pass: tj x tk rows (tj | ny, tk | nz), ntile per colour
  int tj, tk, ntj, ntile, tile0;  // tile0: index of the replica's first tile
  uint32_t tj_m, ntj_m;
  int tj_p, ntj_p;
  long long dir_off;  // float offset of this replica's [2][3][plane] block
  long long pt_off;   // byte offset of its [2][plane] point types
  long long ns_off;   // float offset of its [2][3][plane] normals
  float A, elecA, elecE, ex, ey, ez;
  float lam, mu, nu, rho, sigma;
  // the GHRL bond regrouped for the pass (ghrl_bond_var): ga = 1.5 rho,
  // gb = lambda - rho / 2, gc = 1.5 nu; gconst = -nu / 2 - mu / 9 the part
  // every bond shares
  float ga, gb, gc, gconst;
  float B1, C;  // Pear potential
  uint32_t seed, stream;
  int anch[kMaxSurf];
  float W[kMaxSurf];
  float dx[kMaxSurf], dy[kMaxSurf], dz[kMaxSurf];  // anchoring easy axis
};

// Mutable per-replica scalars, one struct per replica in device memory.
struct RepState {
  float T;
  float ang_var;
  unsigned long long sweep;  // sweeps done: the RNG counter
  unsigned long long meas;   // measured sweeps done: the ring-slot counter
  // the sweep in progress: accepted moves (low 32 bits; a replica has fewer
  // than 2^31 sites) and work units of its colour-1 pass finished (high 32)
  unsigned long long cnt;
  unsigned int frozen;  // nonzero: the step size stays fixed (no adaptation)
};

// Running sums (doubles), indexed by the MCX_ST_* layout of mcx.h.
constexpr int kStats = 16;

__host__ __device__ __forceinline__ uint32_t fastdiv(uint32_t n, uint32_t m, int p) {
  return (uint32_t)(((unsigned long long)n * m) >> p);
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
// ---------------------------------------------------------------------------
// One widening multiply gives both halves (on the GPU a single 32x32->64
// multiply-add instead of separate low and high multiplies).
__host__ __device__ __forceinline__ void mulhilo32(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
  const unsigned long long p = (unsigned long long)a * b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}

__host__ __device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(0xD2511F53u, c.x, hi0, lo0);
    mulhilo32(0xCD9E8D57u, c.z, hi1, lo1);
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// 24-bit uniform on [0, 1), exact in float.
__host__ __device__ __forceinline__ float u01(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-8f; }

// The six 21-bit uniforms of one Philox draw, for the even (A) and odd (B)
// site of a same-colour pair: A takes the top 21 bits of words 0, 1, 2; B the
// top 21 bits of word 3 and the low bits of words 0|1 and 2|3.
__host__ __device__ __forceinline__ void pair_uniforms(uint4 w, float uA[3], float uB[3]) {
  const float sc = 4.76837158203125e-7f;  // 2^-21
  uA[0] = (float)(w.x >> 11) * sc;
  uA[1] = (float)(w.y >> 11) * sc;
  uA[2] = (float)(w.z >> 11) * sc;
  uB[0] = (float)(w.w >> 11) * sc;
  uB[1] = (float)(((w.x & 0x7FFu) << 10) | (w.y & 0x3FFu)) * sc;
  uB[2] = (float)(((w.z & 0x7FFu) << 10) | (w.w & 0x3FFu)) * sc;
}

// ---------------------------------------------------------------------------
// Energies.  Neighbour slots follow the reference order x+, x-, y+, y-, z+,
// z- (src/geometry.cpp:19-72); slot d has axis d >> 1 and sign +1 for even d.
// ---------------------------------------------------------------------------

// Chiral term component as the reference writes it (src/potential.cpp:30-32)
// for r = +e_axis: (a x b) with the reference's sign convention.
// a . b with its roundings fixed (this order; fmaf is always fused)
__device__ __forceinline__ float dot3_rn(float ax, float ay, float az, float bx, float by, float bz) {
  return fmaf(az, bz, fmaf(ay, by, __fmul_rn(ax, bx)));
}

// cross_ref with its roundings fixed
template <int AXIS>
__device__ __forceinline__ float cross_ref_rn(float ax, float ay, float az, float bx, float by, float bz) {
  if (AXIS == 0) return fmaf(az, by, -__fmul_rn(ay, bz));
  if (AXIS == 1) return fmaf(ax, bz, -__fmul_rn(az, bx));
  return fmaf(ay, bx, -__fmul_rn(ax, by));
}

template <int AXIS>
__device__ __forceinline__ float cross_ref(float ax, float ay, float az, float bx, float by, float bz) {
  if (AXIS == 0) return az * by - ay * bz;
  if (AXIS == 1) return ax * bz - az * bx;
  return ay * bx - ax * by;
}

// GHRL bond energy (src/potential.cpp:22-38) for r = sign * e_axis.
template <int AXIS>
__device__ __forceinline__ float ghrl_bond(const RepDev &R, float ax, float ay, float az, float bx, float by, float bz,
                                           float sign) {
  const float ai = AXIS == 0 ? ax : (AXIS == 1 ? ay : az);
  const float aj = AXIS == 0 ? bx : (AXIS == 1 ? by : bz);
  const float nij = ax * bx + ay * by + az * bz;
  const float P2 = 1.5f * nij * nij - 0.5f;
  const float E1 = 1.5f * ai * ai + 1.5f * aj * aj - 1.0f;
  const float cr = sign * cross_ref<AXIS>(ax, ay, az, bx, by, bz);
  const float sg = nij > 0.f ? 1.f : -1.f;
  return E1 * (R.rho * P2 + R.lam) + R.mu * (ai * aj * nij - (1.0f / 9.0f)) + R.nu * P2 + R.sigma * sg * cr;
}

// The GHRL bond without its constant part, as the pass evaluates it:
// ghrl_bond = ghrl_bond_var + gconst.  Regrouped as
// E1 (ga q + gb) + gc q + mu aj ai nij + sigma sgn(nij) cr, q = nij^2,
// E1 = 1.5 ai^2 + (1.5 aj^2 - 1): the neighbour-only terms (1.5 aj^2 - 1,
// mu aj) are shared by the old and the new director's evaluation, and the
// constant drops out of every energy difference (measurements add
// gconst per bond).
template <int AXIS>
__device__ __forceinline__ float ghrl_bond_var(const RepDev &R, float ax, float ay, float az, float bx, float by,
                                               float bz, float sign) {
  const float ai = AXIS == 0 ? ax : (AXIS == 1 ? ay : az);
  const float aj = AXIS == 0 ? bx : (AXIS == 1 ? by : bz);
  // roundings fixed (explicit intrinsics): the pass's energy changes are
  // the same bits in every kernel
  const float nij = dot3_rn(ax, ay, az, bx, by, bz);
  const float q = __fmul_rn(nij, nij);
  const float E1 = fmaf(__fmul_rn(1.5f, ai), ai, fmaf(__fmul_rn(1.5f, aj), aj, -1.0f));
  float v = fmaf(E1, fmaf(R.ga, q, R.gb), fmaf(R.gc, q, __fmul_rn(__fmul_rn(R.mu, aj), __fmul_rn(ai, nij))));
  if (R.sigma != 0.f) {  // the chiral term (p0 != 0); the branch is uniform: a CTA serves one replica
    const float cr = sign * cross_ref_rn<AXIS>(ax, ay, az, bx, by, bz);  // sign is +-1: exact
    v = fmaf(R.sigma, nij > 0.f ? cr : -cr, v);
  }
  return v;
}

// Anchoring energy of surface `sid` (src/anchoring_*.cpp, CPU semantics).
__device__ __forceinline__ float ghrl_form(const RepDev &R, float ai, float aj, float nij, float cross) {
  const float P2 = 1.5f * nij * nij - 0.5f;
  const float E1 = 1.5f * ai * ai + 1.5f * aj * aj - 1.0f;
  const float sg = nij > 0.f ? 1.f : -1.f;
  return E1 * (R.rho * P2 + R.lam) + R.mu * (ai * aj * nij) + R.nu * P2 + R.sigma * sg * cross;
}

__device__ __forceinline__ float cross3(float ax, float ay, float az, float bx, float by, float bz, float rx, float ry,
                                        float rz) {
  return (az * by - ay * bz) * rx + (ax * bz - az * bx) * ry + (ay * bx - ax * by) * rz;
}

static __device__ __noinline__ float surface_energy(const RepDev &R, int sid, float nx, float ny, float nz, float sx, float sy,
                                             float sz) {
  const float W = R.W[sid];
  const float dx = R.dx[sid], dy = R.dy[sid], dz = R.dz[sid];
  switch (R.anch[sid]) {
    case ANCH_HOMEOTROPIC: {
      const float c = nx * sx + ny * sy + nz * sz;
      return -W * c * c;
    }
    case ANCH_FG: {
      const float c = nx * sx + ny * sy + nz * sz;
      return W * c * c;
    }
    case ANCH_RP:
    case ANCH_STRONG:
    case ANCH_STRONG_GHRL: {
      const float c = nx * dx + ny * dy + nz * dz;
      return -W * c * c;
    }
    case ANCH_HOMEOTROPIC_GHRL: {
      const float a = nx * sx + ny * sy + nz * sz;
      return W * ghrl_form(R, a, 1.0f, a, cross3(nx, ny, nz, sx, sy, sz, sx, sy, sz));
    }
    case ANCH_FG_GHRL: {
      const float m = sqrtf(fabsf(nx * sx + ny * sy + nz * sz));
      float vx = nx - sx * m, vy = ny - sy * m, vz = nz - sz * m;
      const float L = sqrtf(fabsf(vx * vx + vy * vy + vz * vz));
      const float d = L > 0.f ? L : 1.f;
      vx /= d;
      vy /= d;
      vz /= d;
      return W * ghrl_form(R, nx * sx + ny * sy + nz * sz, vx * sx + vy * sy + vz * sz, nx * vx + ny * vy + nz * vz,
                           cross3(nx, ny, nz, vx, vy, vz, sx, sy, sz));
    }
    case ANCH_RP_GHRL:
      return W * ghrl_form(R, nx * sx + ny * sy + nz * sz, dx * sx + dy * sy + dz * sz, nx * dx + ny * dy + nz * dz,
                           cross3(nx, ny, nz, dx, dy, dz, sx, sy, sz));
    default:
      return 0.f;
  }
}

// Electric term (src/potential.cpp:39-43).
__device__ __forceinline__ float field_energy(const RepDev &R, float nx, float ny, float nz) {
  const float d = __fmul_rn(R.elecE, dot3_rn(nx, ny, nz, R.ex, R.ey, R.ez));
  return __fmul_rn(__fmul_rn(-R.elecA, d), d);
}

}  // namespace mcx
