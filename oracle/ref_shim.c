/* ref_shim.c -- flat entry points into the reference library compiled from
 * its own unmodified sources (see oracle/Makefile), for the parity tests.
 *
 * TEST INFRASTRUCTURE ONLY: built into oracle/_ref/libqcdref.so next to the
 * reference objects; nothing in the product links it.
 *
 * Each call builds a single-rank qcd_geometry with the reference's own
 * qcd_initGeometry and wraps the caller's arrays (reference host layout, no
 * halo tails at one rank) in qcd_vector / qcd_gaugeField structs.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <mpi.h>
#include <qcd.h>

/* gcr() as shipped in invert.c (compiled from that file, main renamed) */
qcd_int_4 gcr(qcd_vector *sol, qcd_vector *src, qcd_gaugeField *u, qcd_real_8 kappa,
              qcd_real_8 muTM, qcd_uint_4 n, qcd_geometry *geo);
void Exp(qcd_complex_16 M[][3]);

/* The drivers' file-I/O layer (qcd_io.c needs MPI-IO and c-lime and is not
 * built) is replaced by in-memory stand-ins: the parameter text, gauge field
 * and propagators come from arrays the test harness registers with
 * ref_io_set(). invert.c's main() is never called; twop.c's main() runs as
 * ref_twop_main() on those arrays. */
static const char *io_params;
static const double *io_gauge, *io_uprop, *io_dprop;

void ref_io_set(const char *params, const double *gauge, const double *uprop, const double *dprop)
{
  io_params = params;
  io_gauge = gauge;
  io_uprop = uprop;
  io_dprop = dprop;
}

char *qcd_getParams(char *fname, int *len)
{
  (void)fname;
  if (!io_params) return NULL;
  *len = (int)strlen(io_params) + 1;
  char *p = malloc((size_t)*len);
  memcpy(p, io_params, (size_t)*len);
  return p;
}

/* the text between `token` (an opening tag) and the next '<' */
char *qcd_getParam(char token[], char *params, int len)
{
  static char val[16][256];
  static int slot;
  char *out = val[slot++ % 16];
  out[0] = 0;
  const char *p = strstr(params, token);
  if (!p || p >= params + len) return out;
  p += strlen(token);
  int n = 0;
  while (p[n] && p[n] != '<' && n < 255) n++;
  memcpy(out, p, (size_t)n);
  out[n] = 0;
  return out;
}

int qcd_getGaugeField(char *fname, int type, qcd_gaugeField *u)
{
  (void)fname;
  (void)type;
  if (!io_gauge) return 1;
  memcpy(u->D, io_gauge, sizeof(qcd_complex_16) * 36 * u->geo->lV);
  return 0;
}

/* propagator file names "up..." / "down..." select the registered arrays */
int qcd_getPropagator(char *fname, int type, qcd_propagator *p)
{
  (void)type;
  const double *src = strstr(fname, "up") ? io_uprop : strstr(fname, "down") ? io_dprop : NULL;
  if (!src) return 1;
  memcpy(p->D, src, sizeof(qcd_complex_16) * 144 * p->geo->lV);
  return 0;
}

int qcd_getVector(char *fname, int type, qcd_uint_2 nu, qcd_uint_2 c2, qcd_vector *vec)
{ (void)fname; (void)type; (void)nu; (void)c2; (void)vec; return 1; }

/* twop.c (proton two-point function), main renamed */
int ref_twop_main(int argc, char *argv[]);
int ref_twop(const char *param_file)
{
  char *argv[3] = {(char *)"twop", (char *)param_file, NULL};
  return ref_twop_main(2, argv);
}

static int geo_make(qcd_geometry *geo, const int L[4], const double theta[4])
{
  qcd_uint_2 LL[4] = {(qcd_uint_2)L[0], (qcd_uint_2)L[1], (qcd_uint_2)L[2], (qcd_uint_2)L[3]};
  qcd_uint_2 P[4] = {1, 1, 1, 1};
  memset(geo, 0, sizeof(*geo));
  return qcd_initGeometry(geo, LL, P, theta, 0, 1);
}

static void vec_wrap(qcd_vector *v, double *d, qcd_geometry *geo)
{
  memset(v, 0, sizeof(*v));
  v->D = (qcd_complex_16(*)[4][3])d;
  v->geo = geo;
  v->initialized = 1;
}

static void gauge_wrap(qcd_gaugeField *u, double *d, qcd_geometry *geo)
{
  memset(u, 0, sizeof(*u));
  u->D = (qcd_complex_16(*)[4][3][3])d;
  u->geo = geo;
  u->initialized = 1;
}

size_t ref_sizeof_geometry(void) { return sizeof(qcd_geometry); }
size_t ref_sizeof_vector(void) { return sizeof(qcd_vector); }
size_t ref_sizeof_gauge(void) { return sizeof(qcd_gaugeField); }

/* variant: 0 qcd_applyWilsonTMOp, 1 ...NoOptim, 2 ...NoScripts, 3 qcd_applyQTMOp.
 * reps > 1 repeats the apply (CPU timing loops). */
int ref_dslash(double *out, const double *in, const double *gauge, const int L[4],
               const double theta[4], double m, double tm, int variant, int reps)
{
  qcd_geometry geo;
  if (geo_make(&geo, L, theta)) return 1;
  qcd_vector Dv, v;
  qcd_gaugeField u;
  vec_wrap(&Dv, out, &geo);
  vec_wrap(&v, (double *)in, &geo);
  gauge_wrap(&u, (double *)gauge, &geo);
  int rc = 0;
  for (int r = 0; r < (reps > 0 ? reps : 1); r++) {
    switch (variant) {
    case 0: rc = qcd_applyWilsonTMOp(&Dv, &v, &u, m, tm); break;
    case 1: rc = qcd_applyWilsonTMOpNoOptim(&Dv, &v, &u, m, tm); break;
    case 2: rc = qcd_applyWilsonTMOpNoScripts(&Dv, &v, &u, m, tm); break;
    default: rc = qcd_applyQTMOp(&Dv, &v, &u, m, tm); break;
    }
  }
  qcd_destroyGeometry(&geo);
  return rc;
}

/* one call of invert.c's gcr() */
int ref_gcr(double *sol, const double *src, const double *gauge, const int L[4],
            const double theta[4], double kappa, double mu, int n)
{
  qcd_geometry geo;
  if (geo_make(&geo, L, theta)) return 1;
  qcd_vector x, b;
  qcd_gaugeField u;
  vec_wrap(&x, sol, &geo);
  vec_wrap(&b, (double *)src, &geo);
  gauge_wrap(&u, (double *)gauge, &geo);
  int rc = gcr(&x, &b, &u, kappa, mu, (qcd_uint_4)n, &geo);
  qcd_destroyGeometry(&geo);
  return rc;
}

/* BLAS-1 through the reference: op 0 norm, 1 dot, 2 axpy, 3 add, 4 sub,
 * 5 scale, 6 mulC, 7 copy, 8 zero, 9 set, 10 gamma5 */
int ref_blas(int op, double *out, const double *a, const double *b, double cre, double cim,
             const int L[4], double res[2])
{
  double th[4] = {0, 0, 0, 0};
  qcd_geometry geo;
  if (geo_make(&geo, L, th)) return 1;
  qcd_vector o, x, y;
  vec_wrap(&o, out, &geo);
  vec_wrap(&x, (double *)a, &geo);
  vec_wrap(&y, (double *)b, &geo);
  qcd_complex_16 c = {cre, cim};
  switch (op) {
  case 0: res[0] = qcd_normVector(&x); break;
  case 1: { qcd_complex_16 d = qcd_mulAdjointVectorVector(&x, &y); res[0] = d.re; res[1] = d.im; } break;
  case 2: qcd_axpyVector(&o, c, &x, &y); break;
  case 3: qcd_addVector(&o, &x, &y); break;
  case 4: qcd_subVector(&o, &x, &y); break;
  case 5: qcd_scaleVector(&o, cre); break;
  case 6: qcd_mulVectorC(&o, c); break;
  case 7: qcd_copyVector(&o, &x); break;
  case 8: qcd_zeroVector(&o); break;
  case 9: qcd_setVector(&o, c); break;
  default: qcd_gamma5Vector(&o); break;
  }
  qcd_destroyGeometry(&geo);
  return 0;
}

double ref_plaquette(const double *gauge, const int L[4])
{
  double th[4] = {0, 0, 0, 0};
  qcd_geometry geo;
  if (geo_make(&geo, L, th)) return -1;
  qcd_gaugeField u;
  gauge_wrap(&u, (double *)gauge, &geo);
  double p = qcd_calculatePlaquette(&u);
  qcd_destroyGeometry(&geo);
  return p;
}

int ref_ape3d(double *out, const double *gauge, const int L[4], double alpha)
{
  double th[4] = {0, 0, 0, 0};
  qcd_geometry geo;
  if (geo_make(&geo, L, th)) return 1;
  qcd_gaugeField u, a;
  gauge_wrap(&u, (double *)gauge, &geo);
  gauge_wrap(&a, out, &geo);
  int rc = qcd_apeSmear3d(&a, &u, alpha);
  qcd_destroyGeometry(&geo);
  return rc;
}

int ref_gauss3d(double *vec, const double *gauge, const int L[4], double alpha, int t)
{
  double th[4] = {0, 0, 0, 0};
  qcd_geometry geo;
  if (geo_make(&geo, L, th)) return 1;
  qcd_vector v;
  qcd_gaugeField u;
  vec_wrap(&v, vec, &geo);
  gauge_wrap(&u, (double *)gauge, &geo);
  int rc = qcd_gaussIteration3d(&v, &u, alpha, (qcd_uint_4)t);
  qcd_destroyGeometry(&geo);
  return rc;
}

void ref_exp_iM(double *M) { Exp((qcd_complex_16(*)[3])M); }
void ref_project_su3(double *g) { qcd_projectSU33x3((qcd_complex_16(*)[3])g); }

/* geometry tables of the reference's qcd_initGeometry (one rank), for the
 * drop-in geometry parity test; arrays sized 4V, 4V, 4 V3, 4 V3, V, edges */
int ref_geometry(const int L[4], const double theta[4], unsigned long *plus, unsigned long *minus,
                 unsigned long *plus3d, unsigned long *minus3d, unsigned long *eo,
                 unsigned long *edge, unsigned long *edge0, unsigned long counts[4])
{
  qcd_geometry geo;
  if (geo_make(&geo, L, theta)) return 1;
  memcpy(plus, geo.plus, sizeof(qcd_uint_8) * 4 * geo.lV);
  memcpy(minus, geo.minus, sizeof(qcd_uint_8) * 4 * geo.lV);
  memcpy(plus3d, geo.plus3d, sizeof(qcd_uint_8) * 4 * geo.lV3);
  memcpy(minus3d, geo.minus3d, sizeof(qcd_uint_8) * 4 * geo.lV3);
  memcpy(eo, geo.eo, sizeof(qcd_uint_8) * geo.lV);
  memcpy(edge, geo.edge, sizeof(qcd_uint_8) * geo.edgePoints);
  memcpy(edge0, geo.edge0, sizeof(qcd_uint_8) * geo.edge0Points);
  counts[0] = geo.edgePoints;
  counts[1] = geo.edge0Points;
  counts[2] = geo.V;
  counts[3] = geo.V3;
  qcd_destroyGeometry(&geo);
  return 0;
}
