/*
 * mcx_oracle.h -- CPU restatement of the McLiCS hot path (TEST INFRASTRUCTURE).
 * Only the test-suite, the smoke check and the benchmark's CPU-baseline leg
 * use this; the product never does.
 */
#ifndef MCX_ORACLE_H_
#define MCX_ORACLE_H_
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_POT_LL = 0, ORC_POT_GHRL = 1, ORC_POT_PEAR = 2 };
enum { ORC_BOUND_FREE = 0, ORC_BOUND_PERIODIC = 1 };
enum { ORC_GEO_BULK = 0, ORC_GEO_SLAB = 1, ORC_GEO_SPHERE = 2, ORC_GEO_CUSTOM = 3 };
enum {
  ORC_ANCH_HOMEOTROPIC = 0,
  ORC_ANCH_FG = 1,
  ORC_ANCH_RP = 2,
  ORC_ANCH_STRONG = 3,
  ORC_ANCH_HOMEOTROPIC_GHRL = 4,
  ORC_ANCH_FG_GHRL = 5,
  ORC_ANCH_RP_GHRL = 6,
  ORC_ANCH_STRONG_GHRL = 7
};
enum { ORC_ORDER_REDBLACK = 0, ORC_ORDER_EIGHT = 1 };
enum { ORC_F_NO_NORMALIZE = 1, ORC_F_PARALLEL = 2 };
enum { ORC_TAG_PLAIN = 0, ORC_TAG_VMF = 2 };
#define ORC_MAX_SURF 16

typedef struct {
  int nx, ny, nz;
  int xb, yb, zb;
  int potential;
  double A;
  double lam, mu, nu, rho, sigma;
  double elecA, elecE, ex, ey, ez;
  int nsurf;
  int anch[ORC_MAX_SURF];
  double W[ORC_MAX_SURF];
  double dir[ORC_MAX_SURF][3];
  double B1, C; /* Pear potential */
} orc_params;

typedef struct {
  double *dE;       /* per site: E_new - E_old */
  double *scale;    /* per site: sum of |terms| of E_old and E_new */
  uint8_t *acc;     /* per site: accepted */
  uint8_t *tie;     /* per site: |u - p| inside the tie band */
  uint8_t *visited; /* per site: updated in this pass */
} orc_trace;

void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void orc_site_uniforms(int nx, int ny, long s, uint32_t seed, uint32_t stream, uint64_t sweep, uint32_t tag,
                       double u[3]);
double orc_pair(const orc_params *p, const double ni[3], const double nj[3], int d, double *abs_out);
double orc_surface(const orc_params *p, int sid, const double n[3], const double s[3], double *abs_out);
double orc_field(const orc_params *p, const double n[3]);
double orc_local_energy(const orc_params *p, const float *ni, const int *pt, const float *ns, long s,
                        const double n[3], double *abs_out);
void orc_propose(const float n[3], double u0, double u1, float ang_var, int flags, double out[3]);
long orc_pass(const orc_params *p, float *ni, const int *pt, const float *ns, float T, float ang_var, uint32_t seed,
              uint32_t stream, uint64_t sweep, int order, int pass, int flags, double tie_eps, const double *feed,
              orc_trace *tr);
float orc_adapt(float ang_var, long acc, long valid);
long orc_count_valid(const orc_params *p, const int *pt);
long orc_sweep(const orc_params *p, float *ni, const int *pt, const float *ns, float T, float *ang_var, uint32_t seed,
               uint32_t stream, uint64_t sweep, int order, int flags);
double orc_eigmax(const double Q[9], double vec[3]);
void orc_measure(const orc_params *p, const float *ni, const int *pt, const float *ns, double out[16]);
void orc_geometry(int nx, int ny, int nz, int kind, float radius, int *pt, float *ns);
/* mcx_port.c: the reference's CPU sweep ported operation for operation (its
 * float / double arithmetic and 8-colour OpenMP loop), for timing. */
void *orc_port_rngs(unsigned long seed, int threads);
long orc_port_sweep(const orc_params *p, float *ni, const int *pt, const float *ns, float T, float *ang_var,
                    long vallid, void *rngs, int threads, float *scratch);

#ifdef __cplusplus
}
#endif
#endif
