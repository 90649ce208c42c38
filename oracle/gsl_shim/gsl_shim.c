/* Test-only implementation of the GSL entry points the McLiCS reference
 * calls, written from GSL's documented semantics.  Used only to build the
 * reference's own C++ into oracle/_ref for pinning the oracle and for the
 * CPU baseline.  The uniform generator is splitmix64 (Steele, Lea, Flood,
 * OOPSLA'14), not GSL's ranlxs0/taus, so trajectories differ from a
 * GSL-linked build; mcx_shim_feed() replaces it with an explicit list. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <gsl/gsl_rng.h>
#include <gsl/gsl_randist.h>
#include <gsl/gsl_eigen.h>

static const gsl_rng_type t_ranlxs0 = {"ranlxs0 (shim)"};
static const gsl_rng_type t_taus = {"taus (shim)"};
const gsl_rng_type *gsl_rng_ranlxs0 = &t_ranlxs0;
const gsl_rng_type *gsl_rng_taus = &t_taus;

static const double *g_feed = 0;
static long g_feed_n = 0, g_feed_pos = 0;

void mcx_shim_feed(const double *feed, long n) { g_feed = feed; g_feed_n = n; g_feed_pos = 0; }
long mcx_shim_feed_used(void) { return g_feed_pos; }

const gsl_rng_type *gsl_rng_env_setup(void) { return gsl_rng_ranlxs0; }
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T) {
  gsl_rng *r = (gsl_rng *)calloc(1, sizeof(gsl_rng));
  r->type = T;
  r->state = 0x853c49e6748fea9bULL;
  return r;
}
void gsl_rng_set(const gsl_rng *r, unsigned long int s) { ((gsl_rng *)r)->state = 0x9E3779B97F4A7C15ULL * (s + 1); }
void gsl_rng_free(gsl_rng *r) { free(r); }
double gsl_rng_uniform(const gsl_rng *r) {
  if (g_feed) {
    if (g_feed_pos >= g_feed_n) {
      fprintf(stderr, "gsl shim: uniform feed exhausted after %ld values\n", g_feed_n);
      abort();
    }
    return g_feed[g_feed_pos++];
  }
  gsl_rng *w = (gsl_rng *)r;
  unsigned long long z = (w->state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}
/* Uniform direction on the sphere: z uniform on [-1,1] and an azimuth
 * uniform on [0, 2pi) (Archimedes' hat-box theorem). */
void gsl_ran_dir_3d(const gsl_rng *r, double *x, double *y, double *z) {
  double zz = 2 * gsl_rng_uniform(r) - 1, ph = 2 * M_PI * gsl_rng_uniform(r);
  double rho = sqrt(1 - zz * zz);
  *x = rho * cos(ph);
  *y = rho * sin(ph);
  *z = zz;
}

gsl_vector *gsl_vector_alloc(size_t n) { gsl_vector *v = (gsl_vector *)calloc(1, sizeof(gsl_vector)); v->size = n; return v; }
gsl_matrix *gsl_matrix_alloc(size_t a, size_t b) { gsl_matrix *m = (gsl_matrix *)calloc(1, sizeof(gsl_matrix)); m->size1 = a; m->size2 = b; return m; }
void gsl_matrix_set(gsl_matrix *m, size_t i, size_t j, double x) { m->data[3 * i + j] = x; }
double gsl_matrix_get(const gsl_matrix *m, size_t i, size_t j) { return m->data[3 * i + j]; }
double gsl_vector_get(const gsl_vector *v, size_t i) { return v->data[i]; }
gsl_eigen_symmv_workspace *gsl_eigen_symmv_alloc(size_t n) { gsl_eigen_symmv_workspace *w = (gsl_eigen_symmv_workspace *)calloc(1, sizeof(*w)); w->size = n; return w; }

/* Cyclic Jacobi (Golub & Van Loan, sec. 8.5) on the lower triangle, as GSL
 * documents for gsl_eigen_symmv: eigenvalues in eval, unit eigenvectors in
 * the columns of evec. */
int gsl_eigen_symmv(gsl_matrix *A, gsl_vector *eval, gsl_matrix *evec, gsl_eigen_symmv_workspace *w) {
  (void)w;
  double a[3][3], v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j <= i; j++) a[i][j] = a[j][i] = A->data[3 * i + j];
  for (int it = 0; it < 64; it++) {
    double off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
    if (off == 0 || off < 1e-17 * (fabs(a[0][0]) + fabs(a[1][1]) + fabs(a[2][2]))) break;
    for (int p = 0; p < 2; p++)
      for (int q = p + 1; q < 3; q++) {
        if (a[p][q] == 0) continue;
        double th = (a[q][q] - a[p][p]) / (2 * a[p][q]);
        double t = (th >= 0 ? 1 : -1) / (fabs(th) + sqrt(th * th + 1));
        double c = 1 / sqrt(t * t + 1), s = t * c;
        for (int r = 0; r < 3; r++) { double x = a[r][p], y = a[r][q]; a[r][p] = c * x - s * y; a[r][q] = s * x + c * y; }
        for (int r = 0; r < 3; r++) { double x = a[p][r], y = a[q][r]; a[p][r] = c * x - s * y; a[q][r] = s * x + c * y; }
        for (int r = 0; r < 3; r++) { double x = v[r][p], y = v[r][q]; v[r][p] = c * x - s * y; v[r][q] = s * x + c * y; }
      }
  }
  for (int i = 0; i < 3; i++) {
    eval->data[i] = a[i][i];
    for (int r = 0; r < 3; r++) evec->data[3 * r + i] = v[r][i];
  }
  return 0;
}
int gsl_eigen_symmv_sort(gsl_vector *eval, gsl_matrix *evec, gsl_eigen_sort_t t) {
  for (int i = 0; i < 3; i++)
    for (int j = i + 1; j < 3; j++) {
      double a = eval->data[i], b = eval->data[j];
      int sw = t == GSL_EIGEN_SORT_VAL_DESC ? (b > a) : t == GSL_EIGEN_SORT_VAL_ASC ? (b < a)
             : t == GSL_EIGEN_SORT_ABS_DESC ? (fabs(b) > fabs(a)) : (fabs(b) < fabs(a));
      if (sw) {
        eval->data[i] = b; eval->data[j] = a;
        for (int r = 0; r < 3; r++) { double x = evec->data[3 * r + i]; evec->data[3 * r + i] = evec->data[3 * r + j]; evec->data[3 * r + j] = x; }
      }
    }
  return 0;
}
