/* qcd.h -- lets a qcd_lib driver (invert.c, b_minus_Dx.c, ...) compile
 * unmodified against this library: it includes <qcd.h>, and with this
 * directory on the include path that is the library's C ABI (qcdgpu.h),
 * which re-declares qcd_lib's data model and the entry points of the
 * operator, solve and file path under their qcd_lib names, plus the site
 * index and complex helpers those drivers use. Calls outside that path
 * (gauge fixing, three-point functions, ...) are not declared. */
#ifndef QCDGPU_QCD_H
#define QCDGPU_QCD_H 1

#include <math.h>

#include "qcdgpu.h"

/* include/qcd.h:144: site index, t fastest */
#define qcd_LEXIC(t, x, y, z, L) ((qcd_uint_8)((t) + (L)[0] * ((x) + (L)[1] * ((y) + (L)[2] * (z)))))

/* include/qcd_blas.h:12-35: complex arithmetic on qcd_complex_16 values */
static inline qcd_complex_16 qcd_CONJ(qcd_complex_16 a)
{
  qcd_complex_16 r = {a.re, -a.im};
  return r;
}
static inline qcd_complex_16 qcd_CMUL(qcd_complex_16 a, qcd_complex_16 b)
{
  qcd_complex_16 r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
  return r;
}
static inline qcd_complex_16 qcd_CADD(qcd_complex_16 a, qcd_complex_16 b)
{
  qcd_complex_16 r = {a.re + b.re, a.im + b.im};
  return r;
}
static inline qcd_complex_16 qcd_CSUB(qcd_complex_16 a, qcd_complex_16 b)
{
  qcd_complex_16 r = {a.re - b.re, a.im - b.im};
  return r;
}
static inline qcd_complex_16 qcd_CSCALE(qcd_complex_16 a, qcd_real_8 s)
{
  qcd_complex_16 r = {a.re * s, a.im * s};
  return r;
}
static inline qcd_real_8 qcd_NORMSQUARED(qcd_complex_16 a) { return a.re * a.re + a.im * a.im; }

#endif
