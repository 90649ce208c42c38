/*
 * mcx_port.c -- a C port of the reference's CPU sweep for timing
 * (TEST INFRASTRUCTURE: the benchmark's CPU baseline and reference arm where
 * the reference's own build is absent; never part of the product).
 *
 * orc_port_sweep follows EvolveN::Monte_Carlo_Step (src/evolve.cpp:64-179)
 * operation for operation, so that it costs what the reference costs on the
 * same cores:
 *   - the copy of the whole director field into a scratch array at the start
 *     of every sweep (src/evolve.cpp:87-88; the reference never reads it);
 *   - 8 colours of 2x2x2 boxes, each colour an OpenMP loop over the boxes
 *     with a static schedule (src/evolve.cpp:89-91), every site reading its
 *     7 neighbours with the boundary rule of the axis (setNni,
 *     src/evolve.cpp:11-25; src/potential.cpp:44-54);
 *   - the proposal in float with cosf/sinf of (float)(M_PI * va), not
 *     renormalised (src/evolve.cpp:136-152);
 *   - the local energy twice per site, as latice_Potential does it: bond
 *     energies in float with the reference's double literals
 *     (src/potential.cpp:10-43), summed over active neighbours in a double
 *     (src/geometry.cpp:19-72), then the surface and field terms in float
 *     (src/geometry_bulk.cpp:63-72, src/geometry_sphere.cpp:56-69);
 *   - acceptance u < exp(-(E_new - E_old) / T) in double (src/evolve.cpp:160);
 *   - the step-size rule with its float / double rounding
 *     (src/evolve.cpp:169-178).
 * The uniforms come from one generator per OpenMP thread seeded
 * seed * 104729 + thread (src/evolve_thermal.cpp:40-45), each the splitmix64
 * generator of the test-only GSL shim the reference is built with here, so
 * both pay the same per-draw cost.  Surface anchoring uses the oracle's FP64
 * expressions, rounded to float.
 */
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "mcx_oracle.h"

typedef struct {
  unsigned long long s;
  char pad[56]; /* one generator per cache line */
} port_rng;

static double port_uniform(port_rng *r) {
  unsigned long long z = (r->s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

/* One neighbour as setNni leaves it: the director and the point type (0 when
 * the bond does not exist). */
typedef struct {
  float x, y, z;
  int pt;
} port_nni;

/* Periodic_Boundary and Free_Boundary (src/potential.cpp:44-54). */
static int port_periodic(int *ii, int n) {
  *ii = (*ii + n) % n;
  return 1;
}

static int port_free(int *ii, int n) { return !(*ii == -1 || *ii == n); }

static void port_set(const float *ni, const int *pt, long pos, int exists, port_nni *o) {
  if (exists) {
    o->x = ni[pos * 3];
    o->y = ni[pos * 3 + 1];
    o->z = ni[pos * 3 + 2];
    o->pt = pt[pos];
  } else {
    o->pt = 0;
  }
}

/* The bond energies of src/potential.cpp:10-38 in the reference's types. */
static float port_bond_ll(const orc_params *p, const float a[3], const float b[3], const float r[3]) {
  (void)r;
  const float nij = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
  return (float)(-(float)p->A * 1.5 * nij * nij);
}

static float port_bond_pear(const orc_params *p, const float a[3], const float b[3], const float r[3]) {
  const float nij = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
  const float ps = +(1 + 2 * nij + nij * nij) * ((b[0] - a[0]) * r[0] + (b[1] - a[1]) * r[1] + (b[2] - a[2]) * r[2]);
  return (float)(-(float)p->A * nij * nij - (float)p->B1 * nij - ((float)p->C * 0.25) * ps);
}

static float port_bond_ghrl(const orc_params *p, const float a[3], const float b[3], const float r[3]) {
  const float nij = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
  const float el = (float)p->lam, em = (float)p->mu, en = (float)p->nu, er = (float)p->rho, es = (float)p->sigma;
  const float ai = a[0] * r[0] + a[1] * r[1] + a[2] * r[2];
  const float aj = b[0] * r[0] + b[1] * r[1] + b[2] * r[2];
  const float pij = ((float)1.5) * nij * nij - ((float)0.5);
  const float cr = (a[2] * b[1] - a[1] * b[2]) * r[0] + (a[0] * b[2] - a[2] * b[0]) * r[1] +
                   (a[1] * b[0] - a[0] * b[1]) * r[2];
  const float E1 = (float)((1.5 * ai * ai) + (1.5 * aj * aj) - 1);
  return (float)((E1 * (er * pij + el) + em * (ai * aj * nij - 1.0 / 9)) + en * pij + es * (nij > 0 ? 1 : -1) * cr);
}

static const float PORT_R[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};

/* The reference reaches the bond energy, the boundary rules and the local
 * energy through pointers chosen at set-up (params->bulk_potential,
 * params->XBound..ZBound, the virtual latice_Potential); the port calls them
 * through pointers too, so neither is inlined. */
typedef float (*port_bond_fn)(const orc_params *, const float *, const float *, const float *);
typedef int (*port_bound_fn)(int *, int);
typedef float (*port_local_fn)(const orc_params *, const port_nni *, const float *);
static port_bond_fn g_bond;
static port_bound_fn g_bound[3];
static port_local_fn g_local;

/* Geometry::newman_neighbours (src/geometry.cpp:19-72). */
static __attribute__((noinline)) float port_neighbours(const orc_params *p, const port_nni nb[8], const float n[3]) {
  double E = 0;
  for (int d = 0; d < 6; d++)
    if (nb[1 + d].pt) {
      const float b[3] = {nb[1 + d].x, nb[1 + d].y, nb[1 + d].z};
      E += g_bond(p, n, b, PORT_R[d]);
    }
  return (float)E;
}

/* latice_Potential of the bulk / slab / sphere / custom geometries (a
 * virtual call in the reference: reached through g_local). */
static float port_local_impl(const orc_params *p, const port_nni nb[8], const float n[3]) {
  float e = port_neighbours(p, nb, n);
  if (nb[0].pt > 1) {
    const double nd[3] = {n[0], n[1], n[2]}, sd[3] = {nb[7].x, nb[7].y, nb[7].z};
    e += (float)orc_surface(p, nb[0].pt - 2, nd, sd, NULL);
  }
  if (p->elecA != 0) {
    const float d = (float)p->elecE * (n[0] * (float)p->ex + n[1] * (float)p->ey + n[2] * (float)p->ez);
    e += -(float)p->elecA * (d * d);
  }
  return e;
}

/* Generators for `threads` OpenMP threads, seeded as the reference seeds its
 * ranlxs0 generators; pass the result to orc_port_sweep, free with free(). */
void *orc_port_rngs(unsigned long seed, int threads) {
  port_rng *r = (port_rng *)calloc((size_t)threads, sizeof(port_rng));
  for (int t = 0; t < threads; t++) r[t].s = 0x9E3779B97F4A7C15ULL * (seed * 104729 + (unsigned long)t + 1);
  return r;
}

/* One sweep on `threads` OpenMP threads (at most as many as generators were
 * made); returns the accepted moves and updates *ang_var.  vallid: the active
 * sites (orc_count_valid; the reference counts them once, in a function
 * static).  scratch: 3 floats per site (the reference's unused copy of the
 * field). */
long orc_port_sweep(const orc_params *p, float *ni, const int *pt, const float *ns, float T, float *ang_var,
                    long vallid, void *rngs, int threads, float *scratch) {
  const int Nx = p->nx, Ny = p->ny, Nz = p->nz;
  const long Nt = (long)Nx * Ny * Nz;
  port_rng *rng = (port_rng *)rngs;
  g_bond = p->potential == ORC_POT_LL ? port_bond_ll : (p->potential == ORC_POT_PEAR ? port_bond_pear : port_bond_ghrl);
  g_bound[0] = p->xb == ORC_BOUND_PERIODIC ? port_periodic : port_free;
  g_bound[1] = p->yb == ORC_BOUND_PERIODIC ? port_periodic : port_free;
  g_bound[2] = p->zb == ORC_BOUND_PERIODIC ? port_periodic : port_free;
  g_local = port_local_impl;
  for (long q = 0; q < Nt * 3; q++) scratch[q] = ni[q];
  const int Ni = Nx / 2 + Nx % 2, Nj = Ny / 2 + Ny % 2, Nk = Nz / 2 + Nz % 2;
  const long Ntt = (long)Ni * Nj * Nk;
  const float av = *ang_var;
  long acceptance = 0;
#pragma omp parallel num_threads(threads) reduction(+ : acceptance)
  for (int tick = 0; tick < 8; tick++) {
    port_rng *r = &rng[omp_get_thread_num()];
#pragma omp for schedule(static)
    for (long nt = 0; nt < Ntt; nt++) {
      const int iBox = (int)(nt % Ni), jBox = (int)((nt / Ni) % Nj), kBox = (int)(nt / Ni / Nj);
      const int i = tick % 2 + iBox * 2, j = (tick / 2) % 2 + jBox * 2, k = tick / 4 + kBox * 2;
      if (i >= Nx || j >= Ny || k >= Nz) continue;
      const long s = i + (long)Nx * (j + (long)Ny * k);
      if (pt[s] == 0) continue;
      int ip = i + 1, im = i - 1, jp = j + 1, jm = j - 1, kp = k + 1, km = k - 1;
      const int ex[6] = {g_bound[0](&ip, Nx), g_bound[0](&im, Nx), g_bound[1](&jp, Ny),
                         g_bound[1](&jm, Ny), g_bound[2](&kp, Nz), g_bound[2](&km, Nz)};
      port_nni nb[8];
      port_set(ni, pt, s, 1, &nb[0]);
      port_set(ni, pt, ip + (long)Nx * (j + (long)Ny * k), ex[0], &nb[1]);
      port_set(ni, pt, im + (long)Nx * (j + (long)Ny * k), ex[1], &nb[2]);
      port_set(ni, pt, i + (long)Nx * (jp + (long)Ny * k), ex[2], &nb[3]);
      port_set(ni, pt, i + (long)Nx * (jm + (long)Ny * k), ex[3], &nb[4]);
      port_set(ni, pt, i + (long)Nx * (j + (long)Ny * kp), ex[4], &nb[5]);
      port_set(ni, pt, i + (long)Nx * (j + (long)Ny * km), ex[5], &nb[6]);
      if (nb[0].pt > 1) {
        nb[7].x = ns[s * 3];
        nb[7].y = ns[s * 3 + 1];
        nb[7].z = ns[s * 3 + 2];
        nb[7].pt = 1;
      }
      const float va = (float)((2 * port_uniform(r) - 1) * av);
      const float rt = (float)port_uniform(r);
      const float x = ni[s * 3], y = ni[s * 3 + 1], z = ni[s * 3 + 2];
      float nn[3];
      if (rt < 0.333) {
        nn[0] = x;
        nn[1] = y * cosf(M_PI * va) + z * sinf(M_PI * va);
        nn[2] = z * cosf(M_PI * va) - y * sinf(M_PI * va);
      } else if (rt < 0.666) {
        nn[0] = x * cosf(M_PI * va) - z * sinf(M_PI * va);
        nn[1] = y;
        nn[2] = z * cosf(M_PI * va) + x * sinf(M_PI * va);
      } else {
        nn[0] = x * cosf(M_PI * va) + y * sinf(M_PI * va);
        nn[1] = y * cosf(M_PI * va) - x * sinf(M_PI * va);
        nn[2] = z;
      }
      const float n0[3] = {x, y, z};
      const float E_old = g_local(p, nb, n0);
      const float E_new = g_local(p, nb, nn);
      if (port_uniform(r) < exp(-(E_new - E_old) / T)) {
        ni[s * 3] = nn[0];
        ni[s * 3 + 1] = nn[1];
        ni[s * 3 + 2] = nn[2];
        acceptance++;
      }
    }
  }
  float a = *ang_var;
  if (1.0 * acceptance / vallid < 0.5) {
    a *= 0.99;
    if (a < 0.01) a = 0.01;
  } else if (1.0 * acceptance / vallid > 0.5) {
    a /= 0.99;
    if (a > 1.0) a -= 0.5;
  }
  *ang_var = a;
  return acceptance;
}
