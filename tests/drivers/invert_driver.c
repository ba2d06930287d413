/* An inversion driver for the end-to-end file-path test, written against the
 * drop-in C ABI (include/qcd.h): the call sequence of qcd_lib's invert.c
 * (parameter file, ILDG gauge configuration, the twelve HMC source columns,
 * GCR on Q = i gamma5 D with iterative refinement until the true relative
 * residual |src - Q sol| / |src| is below <max_res>). Every solution is
 * written as an ETMC LIME propagator "<solution>.<column>" (column
 * nu * 3 + colour, two digits), for the test to check on the CPU.
 *
 *   invert_driver params.ini
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <qcd.h>

/* the value of tag <name> in the parameter text, copied to out; 1 if absent */
static int param(char *params, int len, const char *name, char *out, size_t n)
{
  char tag[64];
  snprintf(tag, sizeof(tag), "<%s>", name);
  const size_t tl = strlen(tag);
  for (int i = 0; i + (int)tl < len; i++)
    if (memcmp(params + i, tag, tl) == 0) {
      snprintf(out, n, "%s", qcd_getParam(tag, params, len));
      return 0;
    }
  return 1;
}

/* |src - Q sol| / |src| with res as scratch */
static double rel_residual(qcd_vector *res, qcd_vector *sol, qcd_vector *src, qcd_gaugeField *u, double kappa,
                           double mu)
{
  qcd_applyQTMOp(res, sol, u, 1.0 / (2.0 * kappa) - 4.0, mu);
  qcd_subVector(res, src, res);
  return qcd_normVector(res) / qcd_normVector(src);
}

int main(int argc, char *argv[])
{
  if (argc != 2) {
    fprintf(stderr, "usage: %s params.ini\n", argv[0]);
    return EXIT_FAILURE;
  }
  int len = 0;
  char *params = qcd_getParams(argv[1], &len);
  if (!params) return EXIT_FAILURE;
  char lat[64], cfg[qcd_MAX_STRING_LENGTH], src_name[qcd_MAX_STRING_LENGTH], sol_name[qcd_MAX_STRING_LENGTH];
  char buf[64];
  unsigned nrestart = 0;
  double kappa = 0, mu = 0, max_res = 1e-8;
  int max_rounds = 100;
  qcd_uint_2 L[4], P[4] = {1, 1, 1, 1};
  if (param(params, len, "lattice_txyz", lat, sizeof(lat)) ||
      sscanf(lat, "%hu %hu %hu %hu", &L[0], &L[1], &L[2], &L[3]) != 4 ||
      param(params, len, "cfg_name", cfg, sizeof(cfg)) || param(params, len, "source", src_name, sizeof(src_name)) ||
      param(params, len, "solution", sol_name, sizeof(sol_name)) ||
      param(params, len, "N_restart", buf, sizeof(buf)) || sscanf(buf, "%u", &nrestart) != 1 ||
      param(params, len, "kappa", buf, sizeof(buf)) || sscanf(buf, "%lf", &kappa) != 1 ||
      param(params, len, "mu", buf, sizeof(buf)) || sscanf(buf, "%lf", &mu) != 1) {
    fprintf(stderr, "incomplete parameter file %s\n", argv[1]);
    return EXIT_FAILURE;
  }
  if (!param(params, len, "max_res", buf, sizeof(buf))) sscanf(buf, "%lf", &max_res);
  free(params);

  qcd_real_8 theta[4] = {M_PI, 0.0, 0.0, 0.0};  /* antiperiodic in time */
  qcd_geometry geo;
  if (qcd_initGeometry(&geo, L, P, theta, 0, 1)) return EXIT_FAILURE;
  qcd_vector src, sol, res, corr;
  qcd_gaugeField u;
  if (qcd_initVector(&src, &geo) + qcd_initVector(&sol, &geo) + qcd_initVector(&res, &geo) +
          qcd_initVector(&corr, &geo) + qcd_initGaugeField(&u, &geo) != 0) {
    fprintf(stderr, "not enough memory\n");
    return EXIT_FAILURE;
  }
  if (qcd_getGaugeField(cfg, qcd_GF_LIME, &u)) return EXIT_FAILURE;
  printf("plaquette %.12f\n", qcd_calculatePlaquette(&u));

  int status = 0;
  for (int column = 0; column < 12 && !status; column++) {
    if (qcd_getVector(src_name, qcd_PROP_HMC, (qcd_uint_2)(column / 3), (qcd_uint_2)(column % 3), &src)) {
      status = 1;
      break;
    }
    gcr(&sol, &src, &u, kappa, mu, nrestart, &geo);
    double r = rel_residual(&res, &sol, &src, &u, kappa, mu);
    int rounds = 1;
    while (r > max_res && rounds < max_rounds) {  /* solve Q corr = res, sol += corr */
      gcr(&corr, &res, &u, kappa, mu, nrestart, &geo);
      qcd_addVector(&sol, &sol, &corr);
      r = rel_residual(&res, &sol, &src, &u, kappa, mu);
      rounds++;
    }
    printf("column %d rounds %d residual %.6e\n", column, rounds, r);
    char out[qcd_MAX_STRING_LENGTH + 8];
    snprintf(out, sizeof(out), "%s.%02d", sol_name, column);
    if (r > max_res || qcd_writeVector(out, qcd_PROP_LIME, 0, 0, &sol)) status = 1;
  }
  qcd_destroyVector(&src);
  qcd_destroyVector(&sol);
  qcd_destroyVector(&res);
  qcd_destroyVector(&corr);
  qcd_destroyGaugeField(&u);
  qcd_destroyGeometry(&geo);
  return status ? EXIT_FAILURE : EXIT_SUCCESS;
}
