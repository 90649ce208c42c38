/*
 * ref_harness.cpp -- extern "C" entry points over the McLiCS reference's own
 * C++ (TEST INFRASTRUCTURE ONLY).
 *
 * Built by oracle/Makefile together with the unmodified reference sources
 * (read in place from the reference tree, never copied) and the test-only GSL
 * shim into oracle/_ref/libref_mcx.so.  The tests use it to pin the oracle's
 * restatement to the reference's arithmetic, and the benchmark's reference
 * arm uses it to time EvolveN::Monte_Carlo_Step on the host cores.
 *
 * The reference keeps lattice-sized state in function-local statics
 * (src/evolve.cpp:28,66-68, src/parameter_order.cpp:31-33), so one process
 * supports one lattice: callers load this library in a fresh process per
 * configuration.
 */
#include <math.h>
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include <string>
#include <vector>

#include "../include/anchoring.h"
#include "../include/define.h"
#include "../include/evolve.h"
#include "../include/geometry.h"
#include "../include/io.h"
#include "../include/parameter_order.h"
#include "../include/parameters.h"
#include "../include/potential.h"

static Parameters *P = nullptr;
static Geometry *G = nullptr;
static EvolveN *EV = nullptr;
static int *PT = nullptr;
static float *NI = nullptr;
static long NT = 0;
static std::vector<gsl_rng *> RNG;

static int (*bound_fn(const char *s))(int &, int) {
  return strcasecmp(s, "periodic") == 0 ? &Periodic_Boundary : &Free_Boundary;
}

/* Mirrors simulator::Setup_simmulation (src/simulator.cpp:24-103) for one
 * lattice, without the initial condition and without printing snapshots. */
extern "C" int ref_setup(int nx, int ny, int nz, const char *geometry, const char *xb, const char *yb, const char *zb,
                         const char *potential, float A, float k11, float k22, float k33, float p0, float elecA,
                         float ex, float ey, float ez, float elecE, int nsurf, const char *const *anch, const float *W,
                         const float *theta_s, const float *phi_s, const char *bound_file) {
  P = new Parameters();
  P->Nx = nx;
  P->Ny = ny;
  P->Nz = nz;
  snprintf(P->geometry, sizeof(P->geometry), "%s", geometry);
  snprintf(P->XBoundtype, sizeof(P->XBoundtype), "%s", xb);
  snprintf(P->YBoundtype, sizeof(P->YBoundtype), "%s", yb);
  snprintf(P->ZBoundtype, sizeof(P->ZBoundtype), "%s", zb);
  snprintf(P->potential, sizeof(P->potential), "%s", potential);
  if (bound_file) snprintf(P->bound_file_name, sizeof(P->bound_file_name), "%s", bound_file);
  P->A = A;
  P->k11 = k11;
  P->k22 = k22;
  P->k33 = k33;
  P->p0 = p0;
  P->elecA = elecA;
  P->elecX = ex;
  P->elecY = ey;
  P->elecZ = ez;
  P->elecE = elecE;
  for (int s = 0; s < nsurf; s++) {
    P->anchoring_type[s] = anch[s];
    P->W[s] = W[s];
    P->theta_s[s] = theta_s[s];
    P->phi_s[s] = phi_s[s];
  }
  NT = (long)nx * ny * nz;
  PT = (int *)calloc(3 * NT, sizeof(int));
  NI = (float *)calloc(3 * NT, sizeof(float));
  EV = new EvolveN(NI, PT, P);
  if (strcasecmp(geometry, "bulk") == 0)
    G = new Bulk_Geometry(PT, P);
  else if (strcasecmp(geometry, "slab") == 0)
    G = new Slab_Geometry(PT, P);
  else if (strcasecmp(geometry, "sphere") == 0)
    G = new Sphere_Geometry(PT, P);
  else if (strcasecmp(geometry, "custom") == 0)
    G = new Custom_Geometry(PT, P);
  else
    return -1;
  EV->geometry = G;
  P->XBound = bound_fn(P->XBoundtype);
  P->YBound = bound_fn(P->YBoundtype);
  P->ZBound = bound_fn(P->ZBoundtype);
  /* Tests of the anchoring energies on their own configure more surfaces
   * than the geometry has; the extra ones are never reached by
   * latice_Potential. */
  if (nsurf > G->nSurfaces) {
    G->nSurfaces = nsurf;
    G->surfaces.resize(nsurf);
  }
  G->Boundary_Init(P);
  if (strcasecmp(potential, "ghrl") == 0) {
    G->bulk_potential = &Bulk_Energy_GHRL;
    setGHRL(*P);
  } else {
    G->bulk_potential = &Bulk_Energy_Lebwohl_Lasher;
  }
  int nth = omp_get_max_threads();
  for (int t = 0; t < nth; t++) {
    gsl_rng *r = gsl_rng_alloc(gsl_rng_ranlxs0);
    gsl_rng_set(r, 104729 + t);
    RNG.push_back(r);
  }
  fflush(stdout);
  return 0;
}

extern "C" void ref_get_mask(int *pt, float *ns) {
  memcpy(pt, PT, sizeof(int) * NT);
  memcpy(ns, G->ns, sizeof(float) * 3 * NT);
}

extern "C" void ref_get_ghrl(float out[5]) {
  out[0] = P->ghrl_lambda;
  out[1] = P->ghrl_mu;
  out[2] = P->ghrl_nu;
  out[3] = P->ghrl_rho;
  out[4] = P->ghrl_sigma;
}

extern "C" float ref_pair(const float ni[3], const float nj[3], const float rij[3]) {
  float a[3] = {ni[0], ni[1], ni[2]}, b[3] = {nj[0], nj[1], nj[2]}, r[3] = {rij[0], rij[1], rij[2]};
  return G->bulk_potential(a, b, P, r, 1);
}

extern "C" float ref_surface(int sid, const float n[3], const float s[3]) {
  float a[3] = {n[0], n[1], n[2]}, b[3] = {s[0], s[1], s[2]};
  return G->surfaces[sid]->surface_potential(a, b);
}

extern "C" float ref_field(const float n[3]) {
  float a[3] = {n[0], n[1], n[2]};
  return Electric_Potential(a, P);
}

/* Local energy of `site` with director n, the neighbourhood gathered the way
 * src/evolve.cpp:116-135 gathers it. */
extern "C" float ref_local_energy(const float *field, long site, const float n[3]) {
  int Nx = P->Nx, Ny = P->Ny;
  int i = site % Nx, j = (site / Nx) % Ny, k = site / ((long)Nx * Ny);
  int ip = i + 1, im = i - 1, jp = j + 1, jm = j - 1, kp = k + 1, km = k - 1;
  int ex[6] = {P->XBound(ip, Nx), P->XBound(im, Nx), P->YBound(jp, Ny),
               P->YBound(jm, Ny), P->ZBound(kp, P->Nz), P->ZBound(km, P->Nz)};
  long pos[7] = {site,
                 ip + (long)Nx * (j + (long)Ny * k),
                 im + (long)Nx * (j + (long)Ny * k),
                 i + (long)Nx * (jp + (long)Ny * k),
                 i + (long)Nx * (jm + (long)Ny * k),
                 i + (long)Nx * (j + (long)Ny * kp),
                 i + (long)Nx * (j + (long)Ny * km)};
  nni loc[8];
  memset(loc, 0, sizeof(loc));
  for (int q = 0; q < 7; q++) {
    if (q == 0 || ex[q - 1] == 1) {
      loc[q].x = field[pos[q] * 3];
      loc[q].y = field[pos[q] * 3 + 1];
      loc[q].z = field[pos[q] * 3 + 2];
      loc[q].pt = PT[pos[q]];
    } else {
      loc[q].pt = 0;
    }
  }
  loc[0].x = n[0];
  loc[0].y = n[1];
  loc[0].z = n[2];
  if (loc[0].pt > 1) {
    loc[7].x = G->ns[site * 3];
    loc[7].y = G->ns[site * 3 + 1];
    loc[7].z = G->ns[site * 3 + 2];
    loc[7].pt = 1;
  }
  return G->latice_Potential(loc);
}

/* Threads for a sweep: the request, but never more than the generators made
 * at setup (one per thread that OpenMP offered then), since each sweep thread
 * draws from its own. */
static int sweep_threads(int nthreads) {
  const int made = (int)RNG.size();
  return nthreads > 0 && nthreads < made ? nthreads : made;
}

/* One EvolveN::Monte_Carlo_Step (src/evolve.cpp:64-179).  With feed != NULL
 * the sweep runs on one thread and draws its uniforms from feed in order;
 * returns the number of uniforms consumed. */
extern "C" long ref_sweep(float *ni, float T, float *ang_var, const double *feed, long nfeed, int nthreads) {
  memcpy(NI, ni, sizeof(float) * 3 * NT);
  P->T = T;
  omp_set_num_threads(feed ? 1 : sweep_threads(nthreads));
  mcx_shim_feed(feed, nfeed);
  EV->Monte_Carlo_Step(*ang_var, RNG.data());
  long used = mcx_shim_feed_used();
  mcx_shim_feed(nullptr, 0);
  memcpy(ni, NI, sizeof(float) * 3 * NT);
  return used;
}

/* Sweeps in place on the library's own copy (for timing: no copies). */
extern "C" void ref_set_state(const float *ni) { memcpy(NI, ni, sizeof(float) * 3 * NT); }
extern "C" void ref_get_state(float *ni) { memcpy(ni, NI, sizeof(float) * 3 * NT); }
extern "C" float ref_sweeps_inplace(int n, float T, float ang_var, int nthreads) {
  P->T = T;
  omp_set_num_threads(sweep_threads(nthreads));
  for (int s = 0; s < n; s++) EV->Monte_Carlo_Step(ang_var, RNG.data());
  return ang_var;
}

/* EvolveN::energy_calculator (src/evolve.cpp:27-62). */
extern "C" float ref_energy(const float *ni) {
  memcpy(NI, ni, sizeof(float) * 3 * NT);
  return EV->energy_calculator();
}

/* Matrice_constructor + Eigen_value_evaluation (src/parameter_order.cpp). */
extern "C" float ref_order(const float *ni, float Q[9], float vec[3]) {
  Matrice_constructor((float *)ni, Q, PT, *P);
  return Eigen_value_evaluation(Q, vec);
}

/* lattice_order_parameter (src/parameter_order.cpp:62-113) at every active
 * site, the local S of the reference's snapshots; NaN at inactive sites. */
extern "C" void ref_local_order(const float *ni, float *out) {
  const int nx = P->Nx, ny = P->Ny, nz = P->Nz;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const long s = i + (long)nx * (j + (long)ny * k);
        out[s] = PT[s] != 0 ? lattice_order_parameter((float *)ni, PT, i, j, k, *P) : NAN;
      }
}

/* print_n (src/io.cpp:50-80): the reference's snapshot file of state ni. */
extern "C" int ref_print_n(const float *ni, const char *path) {
  memcpy(NI, ni, sizeof(float) * 3 * NT);
  return print_n((char *)path, NI, *P, PT);
}

extern "C" int ref_max_threads(void) { return (int)RNG.size(); }

/* The Pear potential (src/simulator.cpp:95-97) with its B1 and C, after ref_setup. */
extern "C" void ref_set_pear(float B1, float C) {
  P->B1 = B1;
  P->C = C;
  G->bulk_potential = &Bulk_Energy_Selinger_Pear;
}

/* The field strength, as electricEvolveN::run steps params->elecE
 * (src/evolve_electric.cpp:59). */
extern "C" void ref_set_field(float E) { P->elecE = E; }

/* Re-seeds the per-thread generators as thermalEvolveN::run does
 * (src/evolve_thermal.cpp:40-45): seed * 104729 + thread. */
extern "C" void ref_seed(unsigned long seed) {
  for (size_t t = 0; t < RNG.size(); t++) gsl_rng_set(RNG[t], seed * 104729 + t);
}
