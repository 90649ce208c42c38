/*
 * mcx_oracle.c -- CPU restatement of the McLiCS Metropolis hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.  The
 * product (the CUDA engine under mclics-backend_gb300/) never calls it.
 *
 * Every function restates the reference algorithm in FP64 and cites the
 * reference source it follows (paths relative to the McLiCS project root).
 * Layout is the reference's natural AoS layout: site index
 * s = i + Nx*(j + Ny*k), director ni[3*s + c] (include/define.h:10-12),
 * point type pt[s] (0 inactive, 1 bulk, >=2 surface id + 2), surface normal
 * ns[3*s + c].
 *
 * Pinning: the per-site energies, the sweep (fed the same uniforms) and the
 * E/Q/S observables are checked against the reference's own compiled C++
 * (oracle/_ref, built by oracle/Makefile with a test-only GSL shim); the RNG
 * is checked against the published Philox4x32-10 known-answer vectors.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "mcx_oracle.h"

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), written from the paper. */
/* ------------------------------------------------------------------------ */
void orc_philox(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; r++) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

/* The three uniforms of one site update.  Same-colour sites are paired along
 * x: site i of colour c = (i+j+k)%2 in row (j,k) has colour-row position
 * h = i/2, and positions 2q, 2q+1 form pair q.  One Philox4x32-10 draw per
 * pair, counter (row*pairs_per_row + q, sweep_lo, sweep_hi, tag | c), key
 * (seed, stream), gives 128 bits = six 21-bit uniforms: the even position
 * takes the top 21 bits of words 0, 1, 2; the odd one the top 21 bits of
 * word 3 and the low bits of words 0|1 and 2|3.  Multiples of 2^-21 are
 * exact in float and double. */
void orc_site_uniforms(int nx, int ny, long s, uint32_t seed, uint32_t stream, uint64_t sweep, uint32_t tag,
                       double u[3]) {
  int i = (int)(s % nx);
  long row = s / nx;
  int j = (int)(row % ny), k = (int)(row / ny);
  int c = (i + j + k) & 1;
  int hx = (nx + 1) / 2;
  int hp = (hx + 1) / 2;
  int h = i >> 1;
  uint32_t ctr[4] = {(uint32_t)(row * hp + (h >> 1)), (uint32_t)sweep, (uint32_t)(sweep >> 32), tag | (uint32_t)c};
  uint32_t key[2] = {seed, stream}, w[4];
  orc_philox(ctr, key, w);
  uint32_t a0, a1, a2;
  if ((h & 1) == 0) {
    a0 = w[0] >> 11;
    a1 = w[1] >> 11;
    a2 = w[2] >> 11;
  } else {
    a0 = w[3] >> 11;
    a1 = ((w[0] & 0x7FFu) << 10) | (w[1] & 0x3FFu);
    a2 = ((w[2] & 0x7FFu) << 10) | (w[3] & 0x3FFu);
  }
  const double sc = 1.0 / 2097152.0;
  u[0] = a0 * sc;
  u[1] = a1 * sc;
  u[2] = a2 * sc;
}

/* ------------------------------------------------------------------------ */
/* Pair, surface and field energies (FP64).                                  */
/* ------------------------------------------------------------------------ */

/* Neighbour displacement r_ij for direction d = 0..5 in the reference order
 * x+, x-, y+, y-, z+, z- (src/geometry.cpp:19-72). */
static const double RIJ[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};

static double dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* The chiral term as written in src/potential.cpp:30-32:
 * (a_z b_y - a_y b_z) r_x + (a_x b_z - a_z b_x) r_y + (a_y b_x - a_x b_y) r_z. */
static double cross_ref(const double a[3], const double b[3], const double r[3]) {
  return (a[2] * b[1] - a[1] * b[2]) * r[0] + (a[0] * b[2] - a[2] * b[0]) * r[1] + (a[1] * b[0] - a[0] * b[1]) * r[2];
}

/* GHRL bond form shared by the bulk pair (src/potential.cpp:22-38) and the
 * *_GHRL anchorings (src/anchoring_*.cpp): given ai, aj, nij and the chiral
 * term, E1*(rho*P2+lambda) + mu*(ai*aj*nij - c9) + nu*P2 + sigma*sgn(nij)*cross,
 * where c9 = 1/9 for the bulk pair and 0 for the anchorings (the reference
 * writes (1 / 9) there, an integer division). abs_out receives the sum of the
 * magnitudes of the terms (the scale used for relative-error checks). */
static double ghrl_form(const orc_params *p, double ai, double aj, double nij, double cross, double c9,
                        double *abs_out) {
  double P2 = 1.5 * nij * nij - 0.5;
  double E1 = 1.5 * ai * ai + 1.5 * aj * aj - 1.0;
  double sg = nij > 0 ? 1.0 : -1.0;
  double t1 = E1 * (p->rho * P2 + p->lam);
  double t2 = p->mu * (ai * aj * nij - c9);
  double t3 = p->nu * P2;
  double t4 = p->sigma * sg * cross;
  if (abs_out) *abs_out = fabs(t1) + fabs(t2) + fabs(t3) + fabs(t4);
  return t1 + t2 + t3 + t4;
}

double orc_pair(const orc_params *p, const double ni[3], const double nj[3], int d, double *abs_out) {
  const double *r = RIJ[d];
  if (p->potential == ORC_POT_LL) {
    /* src/potential.cpp:17-20: -A * 1.5 * (ni.nj)^2 */
    double nij = dot3(ni, nj);
    double e = -p->A * 1.5 * nij * nij;
    if (abs_out) *abs_out = fabs(e);
    return e;
  }
  if (p->potential == ORC_POT_PEAR) {
    /* src/potential.cpp:10-15: -A nij^2 - B1 nij - (C/4) (1 + 2 nij + nij^2) ((nj - ni) . rij) */
    double nij = dot3(ni, nj);
    double ps = (1 + 2 * nij + nij * nij) * ((nj[0] - ni[0]) * r[0] + (nj[1] - ni[1]) * r[1] + (nj[2] - ni[2]) * r[2]);
    double t1 = -p->A * nij * nij, t2 = -p->B1 * nij, t3 = -(p->C * 0.25) * ps;
    if (abs_out) *abs_out = fabs(t1) + fabs(t2) + fabs(t3);
    return t1 + t2 + t3;
  }
  /* src/potential.cpp:22-38 */
  double ai = dot3(ni, r), aj = dot3(nj, r), nij = dot3(ni, nj);
  return ghrl_form(p, ai, aj, nij, cross_ref(ni, nj, r), 1.0 / 9.0, abs_out);
}

double orc_surface(const orc_params *p, int sid, const double n[3], const double s[3], double *abs_out) {
  const double W = p->W[sid];
  const double *dir = p->dir[sid];
  double e, a = 0;
  switch (p->anch[sid]) {
    case ORC_ANCH_HOMEOTROPIC: { /* src/anchoring_homeotropic.cpp:29-34: -W (n.s)^2 */
      double c = dot3(n, s);
      e = -W * c * c;
      a = fabs(e);
      break;
    }
    case ORC_ANCH_FG: { /* src/anchoring_fg.cpp:29-34: +W (n.s)^2 */
      double c = dot3(n, s);
      e = W * c * c;
      a = fabs(e);
      break;
    }
    case ORC_ANCH_RP:          /* src/anchoring_rp.cpp:41-48 */
    case ORC_ANCH_STRONG:      /* src/anchoring_strong.cpp:41-48 */
    case ORC_ANCH_STRONG_GHRL: /* src/anchoring_strong.cpp:77-84 */
    {
      double c = dot3(n, dir);
      e = -W * c * c;
      a = fabs(e);
      break;
    }
    case ORC_ANCH_HOMEOTROPIC_GHRL: { /* src/anchoring_homeotropic.cpp:51-68 */
      double ai = dot3(n, s), nij = dot3(n, s);
      e = W * ghrl_form(p, ai, 1.0, nij, cross_ref(n, s, s), 0.0, &a);
      a *= fabs(W);
      break;
    }
    case ORC_ANCH_FG_GHRL: { /* src/anchoring_fg.cpp:51-74 */
      double m = sqrt(fabs(dot3(n, s)));
      double v[3] = {n[0] - s[0] * m, n[1] - s[1] * m, n[2] - s[2] * m};
      double L = sqrt(fabs(dot3(v, v)));
      double dv = L > 0 ? L : 1.0;
      v[0] /= dv;
      v[1] /= dv;
      v[2] /= dv;
      e = W * ghrl_form(p, dot3(n, s), dot3(v, s), dot3(n, v), cross_ref(n, v, s), 0.0, &a);
      a *= fabs(W);
      break;
    }
    case ORC_ANCH_RP_GHRL: { /* src/anchoring_rp.cpp:77-98 */
      e = W * ghrl_form(p, dot3(n, s), dot3(dir, s), dot3(n, dir), cross_ref(n, dir, s), 0.0, &a);
      a *= fabs(W);
      break;
    }
    default:
      e = 0;
  }
  if (abs_out) *abs_out = a;
  return e;
}

double orc_field(const orc_params *p, const double n[3]) {
  /* src/potential.cpp:39-43: -elecA * (elecE * (n . e))^2 */
  double ndE = p->elecE * (n[0] * p->ex + n[1] * p->ey + n[2] * p->ez);
  return -p->elecA * ndE * ndE;
}

/* Neighbour site of s in direction d with the reference's boundary rules
 * (src/potential.cpp:44-54: periodic wraps, free drops the bond at -1 / N).
 * Returns -1 when the neighbour does not exist. */
static long neighbour(const orc_params *p, int i, int j, int k, int d) {
  int N[3] = {p->nx, p->ny, p->nz};
  int b[3] = {p->xb, p->yb, p->zb};
  int c[3] = {i, j, k};
  int ax = d >> 1;
  c[ax] += (d & 1) ? -1 : 1;
  if (c[ax] < 0 || c[ax] >= N[ax]) {
    if (b[ax] == ORC_BOUND_PERIODIC)
      c[ax] = (c[ax] + N[ax]) % N[ax];
    else
      return -1;
  }
  return (long)c[0] + (long)p->nx * ((long)c[1] + (long)p->ny * c[2]);
}

/* Local energy of site s with director n (Geometry::latice_Potential:
 * src/geometry_bulk.cpp:63-72, src/geometry_slab.cpp:69-83,
 * src/geometry_sphere.cpp:56-69, src/geometry_custom.cpp:130-145):
 * sum over existing neighbours with pt != 0 of the pair energy, plus the
 * anchoring energy of surface pt-2 when pt > 1, plus the field energy when
 * elecA != 0.  The neighbour sum follows src/geometry.cpp:19-72. */
double orc_local_energy(const orc_params *p, const float *ni, const int *pt, const float *ns, long s,
                        const double n[3], double *abs_out) {
  int i = (int)(s % p->nx), j = (int)((s / p->nx) % p->ny), k = (int)(s / ((long)p->nx * p->ny));
  double E = 0, A = 0, a;
  for (int d = 0; d < 6; d++) {
    long t = neighbour(p, i, j, k, d);
    if (t < 0 || pt[t] == 0) continue;
    double nj[3] = {ni[3 * t], ni[3 * t + 1], ni[3 * t + 2]};
    E += orc_pair(p, n, nj, d, &a);
    A += a;
  }
  if (pt[s] > 1 && p->nsurf > 0) {
    double sv[3] = {ns[3 * s], ns[3 * s + 1], ns[3 * s + 2]};
    E += orc_surface(p, pt[s] - 2, n, sv, &a);
    A += a;
  }
  if (p->elecA != 0) {
    double f = orc_field(p, n);
    E += f;
    A += fabs(f);
  }
  if (abs_out) *abs_out = A;
  return E;
}

/* ------------------------------------------------------------------------ */
/* Proposal, acceptance and one pass of the sweep.                            */
/* ------------------------------------------------------------------------ */

/* Does site (i,j,k) belong to pass `pass` of the given order?
 * ORDER_EIGHT: the reference's 2x2x2 sub-lattice colours, tick t has
 * di = t%2, dj = (t/2)%2, dk = t/4 (src/evolve.cpp:89-112).
 * ORDER_REDBLACK: pass c updates (i+j+k) % 2 == c. */
static int in_pass(int order, int pass, int i, int j, int k) {
  if (order == ORC_ORDER_EIGHT) return (i & 1) == (pass & 1) && (j & 1) == ((pass >> 1) & 1) && (k & 1) == (pass >> 2);
  return ((i + j + k) & 1) == pass;
}

/* Rotated proposal (src/evolve.cpp:136-152): rotation by pi*va about x if
 * u1 < 0.333, about y if u1 < 0.666, else about z, va = (2 u0 - 1) * ang_var
 * (rounded to float as in the reference).  The GB300 engine renormalises the
 * result (as src/evolve.cu:160-163 does); flag ORC_F_NO_NORMALIZE reproduces
 * the CPU path, which does not. */
void orc_propose(const float n[3], double u0, double u1, float ang_var, int flags, double out[3]) {
  float va = (float)((2.0 * u0 - 1.0) * (double)ang_var);
  double th = M_PI * (double)va;
  double c = cos(th), s = sin(th);
  double x = n[0], y = n[1], z = n[2];
  if (u1 < 0.333) {
    out[0] = x;
    out[1] = y * c + z * s;
    out[2] = z * c - y * s;
  } else if (u1 < 0.666) {
    out[0] = x * c - z * s;
    out[1] = y;
    out[2] = z * c + x * s;
  } else {
    out[0] = x * c + y * s;
    out[1] = y * c - x * s;
    out[2] = z;
  }
  if (!(flags & ORC_F_NO_NORMALIZE)) {
    double L = sqrt(out[0] * out[0] + out[1] * out[1] + out[2] * out[2]);
    out[0] /= L;
    out[1] /= L;
    out[2] /= L;
  }
}

long orc_pass(const orc_params *p, float *ni, const int *pt, const float *ns, float T, float ang_var, uint32_t seed,
              uint32_t stream, uint64_t sweep, int order, int pass, int flags, double tie_eps, const double *feed,
              orc_trace *tr) {
  long acc = 0;
  long fed = 0;
  /* Sites of one pass are independent (no two are neighbours), so the
   * ORC_F_PARALLEL split over planes gives the same result as the serial
   * loop; fed uniforms are consumed in order and force the serial loop. */
  int par = (flags & ORC_F_PARALLEL) && feed == NULL;
#pragma omp parallel for reduction(+ : acc) schedule(static) if (par)
  for (int k = 0; k < p->nz; k++)
    for (int j = 0; j < p->ny; j++)
      for (int i = 0; i < p->nx; i++) {
        if (!in_pass(order, pass, i, j, k)) continue;
        long s = (long)i + (long)p->nx * ((long)j + (long)p->ny * k);
        if (pt[s] == 0) continue;
        double u0, u1, u2;
        if (feed) {
          u0 = feed[3 * fed];
          u1 = feed[3 * fed + 1];
          u2 = feed[3 * fed + 2];
          fed++;
        } else {
          double u[3];
          orc_site_uniforms(p->nx, p->ny, s, seed, stream, sweep, ORC_TAG_PLAIN, u);
          u0 = u[0];
          u1 = u[1];
          u2 = u[2];
        }
        float cur[3] = {ni[3 * s], ni[3 * s + 1], ni[3 * s + 2]};
        double nold[3] = {cur[0], cur[1], cur[2]}, nnew[3];
        orc_propose(cur, u0, u1, ang_var, flags, nnew);
        double a_old, a_new;
        double Eo = orc_local_energy(p, ni, pt, ns, s, nold, &a_old);
        double En = orc_local_energy(p, ni, pt, ns, s, nnew, &a_new);
        double dE = En - Eo;
        /* src/evolve.cpp:160: accept when u < exp(-(E_new - E_old)/T) */
        double pa = exp(-dE / (double)T);
        int accept = u2 < pa;
        int tie = 0;
        if (pa < 1.0 && fabs(u2 - pa) <= tie_eps * (1.0 + pa)) tie = 1;
        if (fabs(dE) <= tie_eps * (a_old + a_new) && T == 0.0f) tie = 1;
        if (tr) {
          tr->dE[s] = dE;
          tr->scale[s] = a_old + a_new;
          tr->acc[s] = (uint8_t)accept;
          tr->tie[s] = (uint8_t)tie;
          tr->visited[s] = 1;
        }
        if (accept) {
          ni[3 * s] = (float)nnew[0];
          ni[3 * s + 1] = (float)nnew[1];
          ni[3 * s + 2] = (float)nnew[2];
          acc++;
        }
      }
  return acc;
}

/* Step-size adaptation toward 50% acceptance (src/evolve.cpp:169-178),
 * with the reference's float/double rounding. */
float orc_adapt(float ang_var, long acc, long valid) {
  double ratio = 1.0 * (double)acc / (double)valid;
  if (ratio < 0.5) {
    ang_var = (float)((double)ang_var * 0.99);
    if ((double)ang_var < 0.01) ang_var = (float)0.01;
  } else if (ratio > 0.5) {
    ang_var = (float)((double)ang_var / 0.99);
    if ((double)ang_var > 1.0) ang_var = (float)((double)ang_var - 0.5);
  }
  return ang_var;
}

long orc_count_valid(const orc_params *p, const int *pt) {
  long n = (long)p->nx * p->ny * p->nz, v = 0;
  for (long s = 0; s < n; s++) v += pt[s] != 0;
  return v;
}

long orc_sweep(const orc_params *p, float *ni, const int *pt, const float *ns, float T, float *ang_var, uint32_t seed,
               uint32_t stream, uint64_t sweep, int order, int flags) {
  int npass = order == ORC_ORDER_EIGHT ? 8 : 2;
  long acc = 0;
  for (int q = 0; q < npass; q++)
    acc += orc_pass(p, ni, pt, ns, T, *ang_var, seed, stream, sweep, order, q, flags, 0.0, NULL, NULL);
  /* valid is counted once per call; the reference counts it once per
   * process (src/evolve.cpp:82-87) -- the same number for a fixed mask. */
  *ang_var = orc_adapt(*ang_var, acc, orc_count_valid(p, pt));
  return acc;
}

/* ------------------------------------------------------------------------ */
/* Observables.                                                               */
/* ------------------------------------------------------------------------ */

/* Cyclic Jacobi eigen-decomposition of a symmetric 3x3 matrix (Golub & Van
 * Loan, Matrix Computations, sec. 8.5).  Returns the largest eigenvalue and
 * its unit eigenvector (the reference sorts GSL's eigenvalues in descending
 * order and reports the first: src/parameter_order.cpp:11-28). */
double orc_eigmax(const double Qin[9], double vec[3]) {
  double a[3][3], v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) a[r][c] = 0.5 * (Qin[3 * r + c] + Qin[3 * c + r]);
  for (int sweep = 0; sweep < 64; sweep++) {
    double off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
    double scale = fabs(a[0][0]) + fabs(a[1][1]) + fabs(a[2][2]) + off;
    if (off <= 1e-300 || off <= 1e-17 * scale) break;
    for (int pq = 0; pq < 3; pq++) {
      int P = pq == 2 ? 1 : 0, Qi = pq == 0 ? 1 : 2;
      double apq = a[P][Qi];
      if (apq == 0) continue;
      double theta = (a[Qi][Qi] - a[P][P]) / (2 * apq);
      double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
      double c = 1 / sqrt(t * t + 1), s = t * c;
      for (int r = 0; r < 3; r++) { /* A <- A J */
        double arp = a[r][P], arq = a[r][Qi];
        a[r][P] = c * arp - s * arq;
        a[r][Qi] = s * arp + c * arq;
      }
      for (int r = 0; r < 3; r++) { /* A <- J^T A */
        double apr = a[P][r], aqr = a[Qi][r];
        a[P][r] = c * apr - s * aqr;
        a[Qi][r] = s * apr + c * aqr;
      }
      for (int r = 0; r < 3; r++) {
        double vrp = v[r][P], vrq = v[r][Qi];
        v[r][P] = c * vrp - s * vrq;
        v[r][Qi] = s * vrp + c * vrq;
      }
    }
  }
  int m = 0;
  if (a[1][1] > a[m][m]) m = 1;
  if (a[2][2] > a[m][m]) m = 2;
  if (vec) {
    vec[0] = v[0][m];
    vec[1] = v[1][m];
    vec[2] = v[2][m];
  }
  return a[m][m];
}

/* E, Q and S (EvolveN::energy_calculator, src/evolve.cpp:27-62;
 * Matrice_constructor, src/parameter_order.cpp:30-60):
 *   out[0] = E over all Nt sites (the CPU path: pt = 0 sites included with
 *            their stored director, divided by Nt)
 *   out[1] = E over active sites divided by the active count (the GPU
 *            path's normalisation, src/evolve.cu:72-75,435)
 *   out[2..10] = Q = sum_{pt!=0} (3 n n^T - I) / (2 points), Q_zz = -Q_xx - Q_yy
 *   out[11] = S = largest eigenvalue of Q, out[12..14] its eigenvector
 *   out[15] = number of active sites. */
void orc_measure(const orc_params *p, const float *ni, const int *pt, const float *ns, double out[16]) {
  long n = (long)p->nx * p->ny * p->nz;
  double Eall = 0, Ev = 0, q[6] = {0, 0, 0, 0, 0, 0};
  long v = 0;
  for (long s = 0; s < n; s++) {
    double nn[3] = {ni[3 * s], ni[3 * s + 1], ni[3 * s + 2]};
    double e = orc_local_energy(p, ni, pt, ns, s, nn, NULL);
    Eall += e;
    if (pt[s]) {
      Ev += e;
      v++;
      q[0] += 3.0 * nn[0] * nn[0] - 1;
      q[1] += 3.0 * nn[0] * nn[1];
      q[2] += 3.0 * nn[0] * nn[2];
      q[3] += 3.0 * nn[1] * nn[1] - 1;
      q[4] += 3.0 * nn[1] * nn[2];
    }
  }
  double Q[9];
  double d = 2.0 * (double)v;
  Q[0] = q[0] / d;
  Q[1] = q[1] / d;
  Q[2] = q[2] / d;
  Q[4] = q[3] / d;
  Q[5] = q[4] / d;
  Q[3] = Q[1];
  Q[6] = Q[2];
  Q[7] = Q[5];
  Q[8] = -Q[0] - Q[4];
  out[0] = Eall / (double)n;
  out[1] = v ? Ev / (double)v : 0.0;
  for (int c = 0; c < 9; c++) out[2 + c] = Q[c];
  double vec[3];
  out[11] = orc_eigmax(Q, vec);
  out[12] = vec[0];
  out[13] = vec[1];
  out[14] = vec[2];
  out[15] = (double)v;
}

/* ------------------------------------------------------------------------ */
/* Geometry masks.                                                            */
/* ------------------------------------------------------------------------ */

/* Point types and surface normals.
 * bulk: all 1 (src/geometry_bulk.cpp:57-61).
 * slab: k = 0 -> pt 2, ns = -z; k = Nz-1 -> pt 3, ns = +z; else 1
 *       (src/geometry_slab.cpp:47-67).
 * sphere: H = (float)(N/2) per axis, R = (i-Hx, j-Hy, k-Hz), r = |R| in
 *       float; r < radius-1 -> 1, r < radius+1 -> 2 with ns = R/r, else 0
 *       (src/geometry_sphere.cpp:28-54 with radius = Hz; radius > 0 here
 *       overrides it). */
void orc_geometry(int nx, int ny, int nz, int kind, float radius, int *pt, float *ns) {
  long n = (long)nx * ny * nz;
  memset(ns, 0, sizeof(float) * 3 * n);
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        long s = (long)i + (long)nx * ((long)j + (long)ny * k);
        if (kind == ORC_GEO_BULK) {
          pt[s] = 1;
        } else if (kind == ORC_GEO_SLAB) {
          if (k == nz - 1) {
            pt[s] = 3;
            ns[3 * s + 2] = 1;
          } else if (k == 0) {
            pt[s] = 2;
            ns[3 * s + 2] = -1;
          } else {
            pt[s] = 1;
          }
        } else if (kind == ORC_GEO_SPHERE) {
          float Hx = (float)(nx / 2), Hy = (float)(ny / 2), Hz = (float)(nz / 2);
          float R = radius > 0 ? radius : Hz;
          float Rx = (float)i - Hx, Ry = (float)j - Hy, Rz = (float)k - Hz;
          float r = sqrtf(Rx * Rx + Ry * Ry + Rz * Rz);
          if (r < R - 1) {
            pt[s] = 1;
          } else if (r < R + 1) {
            pt[s] = 2;
            ns[3 * s] = Rx / r;
            ns[3 * s + 1] = Ry / r;
            ns[3 * s + 2] = Rz / r;
          } else {
            pt[s] = 0;
          }
        }
      }
}
