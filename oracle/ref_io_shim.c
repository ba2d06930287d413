/* Entry points into the reference's own file readers and writers
 * (lib/src/qcd_io.c, compiled unmodified into oracle/_ref/libqcdio.so with
 * the single-rank MPI-IO stand-in of mpi_stub/mpi.h and the LIME container
 * of lime_format.c). Test infrastructure only: the tests read files with
 * both the reference and the GPU library and compare the arrays.
 *
 * Arrays are the reference's host layouts: a vector [V][4][3] complex, a
 * gauge field [V][4][3][3] complex, V in qcd_LEXIC order (t fastest);
 * L = {T, X, Y, Z}.
 */
#include <string.h>

#include <mpi.h>
#include <qcd.h>

static int geo_init(qcd_geometry *geo, const int L[4])
{
  qcd_uint_2 LL[4] = {(qcd_uint_2)L[0], (qcd_uint_2)L[1], (qcd_uint_2)L[2], (qcd_uint_2)L[3]};
  qcd_uint_2 P[4] = {1, 1, 1, 1};
  qcd_real_8 theta[4] = {0, 0, 0, 0};
  memset(geo, 0, sizeof(*geo));
  return qcd_initGeometry(geo, LL, P, theta, 0, 1);
}

static void vec_on(qcd_vector *v, double *d, qcd_geometry *geo)
{
  memset(v, 0, sizeof(*v));
  v->D = (qcd_complex_16(*)[4][3])d;
  v->geo = geo;
  v->initialized = 1;
}

static void gauge_on(qcd_gaugeField *u, double *d, qcd_geometry *geo)
{
  memset(u, 0, sizeof(*u));
  u->D = (qcd_complex_16(*)[4][3][3])d;
  u->geo = geo;
  u->initialized = 1;
}

/* qcd_getVector (qcd_io.c:1386): type 0 CMI, 1 HMC, 2 HMCV, 3 LIME */
int refio_get_vector(double *out, const char *fname, const int L[4], int type, int nu, int c2)
{
  qcd_geometry geo;
  if (geo_init(&geo, L)) return 1;
  qcd_vector v;
  vec_on(&v, out, &geo);
  int rc = qcd_getVector((char *)fname, type, (qcd_uint_2)nu, (qcd_uint_2)c2, &v);
  qcd_destroyGeometry(&geo);
  return rc;
}

/* qcd_writeVector (qcd_io.c:1951): type 0 CMI, 3 LIME propagator, 4 LIME source */
int refio_write_vector(const double *in, const char *fname, const int L[4], int type, int nu, int c2)
{
  qcd_geometry geo;
  if (geo_init(&geo, L)) return 1;
  qcd_vector v;
  vec_on(&v, (double *)in, &geo);
  int rc = qcd_writeVector((char *)fname, type, (qcd_uint_2)nu, (qcd_uint_2)c2, &v);
  qcd_destroyGeometry(&geo);
  return rc;
}

/* qcd_getGaugeField (qcd_io.c:401): type 0, ILDG */
int refio_get_gauge(double *out, const char *fname, const int L[4])
{
  qcd_geometry geo;
  if (geo_init(&geo, L)) return 1;
  qcd_gaugeField u;
  gauge_on(&u, out, &geo);
  int rc = qcd_getGaugeField((char *)fname, qcd_GF_LIME, &u);
  qcd_destroyGeometry(&geo);
  return rc;
}

/* qcd_writeGaugeLime (qcd_io.c:421) */
int refio_write_gauge(const double *in, const char *fname, const int L[4], const char *message)
{
  qcd_geometry geo;
  if (geo_init(&geo, L)) return 1;
  qcd_gaugeField u;
  gauge_on(&u, (double *)in, &geo);
  int rc = qcd_writeGaugeLime((char *)fname, &u, (char *)message);
  qcd_destroyGeometry(&geo);
  return rc;
}
