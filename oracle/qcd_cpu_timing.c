/* qcd_cpu_timing.c -- the CPU baseline's timed Wilson-twisted-mass operator.
 *
 * BENCHMARK/TEST INFRASTRUCTURE ONLY: the CPU-baseline legs of the benchmark
 * time this routine and the tests check it; nothing in the GPU library links
 * or calls it. The parity checker stays orc_dslash (qcd_oracle.c, general
 * 4x4 gamma matrices, no FMA contraction); this file restates the ALGORITHM
 * of the reference's fast operator so that the CPU figure is the reference's
 * speed, not that of a slower formulation:
 *
 *   qcd_applyWilsonTMOp (lib/src/qcd_wilson.c:114-336): per site, project
 *   each of the eight neighbour spinors to a two-spin half spinor
 *   (1 -/+ gamma_mu) (qcd_wilson.h:47-387), multiply the half spinor by
 *   U_mu(x) or U_mu(x-mu)^dagger (qcd_wilson.h:449-509), multiply by the
 *   boundary phase e^{+/- i theta_mu / L_mu} where theta_mu != 0
 *   (qcd_wilson.h:605-624), and rebuild the lower two spins from the upper
 *   ones while summing with the mass term (qcd_wilson.h:389-417, 539-564).
 *   Neighbours come from plus/minus site tables, as qcd_initGeometry builds
 *   them (lib/src/qcd_init.c:110-124).
 *
 * It is compiled at -O3 with the compiler's default FMA contraction, like
 * the reference's own build (Makefile:1-5), so its results differ from the
 * checker's in the last bits only (tested at <= 1e-13 per site).
 *
 * Chiral basis (lib/src/qcd_gamma.c:46-103), s = +1 for (1 + gamma_mu) and
 * s = -1 for (1 - gamma_mu), h = the two upper spins of (1 + s gamma_mu) psi:
 *   mu = t: h0 = p0 - s p2,   h1 = p1 - s p3,   lower = (-s h0, -s h1)
 *   mu = x: h0 = p0 - i s p3, h1 = p1 - i s p2, lower = ( i s h1, i s h0)
 *   mu = y: h0 = p0 - s p3,   h1 = p1 + s p2,   lower = ( s h1, -s h0)
 *   mu = z: h0 = p0 - i s p2, h1 = p1 + i s p3, lower = ( i s h0, -i s h1)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* plus/minus neighbour tables [V][4], rebuilt when the lattice changes */
static uint64_t *tab_plus, *tab_minus;
static int tab_L[4];

static int tables(const int L[4])
{
  if (tab_plus && !memcmp(tab_L, L, sizeof(tab_L))) return 0;
  free(tab_plus);
  free(tab_minus);
  size_t V = (size_t)L[0] * L[1] * L[2] * L[3];
  tab_plus = malloc(V * 4 * sizeof(uint64_t));
  tab_minus = malloc(V * 4 * sizeof(uint64_t));
  if (!tab_plus || !tab_minus) {
    free(tab_plus);
    free(tab_minus);
    tab_plus = tab_minus = NULL;
    return 1;
  }
  memcpy(tab_L, L, sizeof(tab_L));
  size_t l = 0;
  for (int z = 0; z < L[3]; z++)
    for (int y = 0; y < L[2]; y++)
      for (int x = 0; x < L[1]; x++)
        for (int t = 0; t < L[0]; t++, l++) {
          int c[4] = {t, x, y, z};
          for (int mu = 0; mu < 4; mu++) {
            int cp[4] = {c[0], c[1], c[2], c[3]}, cm[4] = {c[0], c[1], c[2], c[3]};
            cp[mu] = (c[mu] + 1) % L[mu];
            cm[mu] = (c[mu] + L[mu] - 1) % L[mu];
            tab_plus[l * 4 + mu] = cp[0] + (uint64_t)L[0] * (cp[1] + (uint64_t)L[1] * (cp[2] + (uint64_t)L[2] * cp[3]));
            tab_minus[l * 4 + mu] = cm[0] + (uint64_t)L[0] * (cm[1] + (uint64_t)L[1] * (cm[2] + (uint64_t)L[2] * cm[3]));
          }
        }
  return 0;
}

/* a += c * b for a coefficient c in {+1, -1, +i, -i} given as (kind, sign):
 * kind 0 real, 1 imaginary */
static inline __attribute__((always_inline)) void acc_coef(double *a, const double *b, int kind, int sign)
{
  for (int k = 0; k < 3; k++) {
    double re = b[2 * k], im = b[2 * k + 1];
    if (kind == 0) {
      a[2 * k] += sign * re;
      a[2 * k + 1] += sign * im;
    } else { /* (i sign)(re + i im) = -sign im + i sign re */
      a[2 * k] -= sign * im;
      a[2 * k + 1] += sign * re;
    }
  }
}

/* one hop: project psi (24 doubles) along mu with sign s, multiply the half
 * spinor by U (dag = 0) or U^dagger (dag = 1), apply the phase (pr, pi) when
 * twisted, and add the rebuilt four-spin result to acc (24 doubles). mu, s and
 * dag are constants at every call site, so the branches fold away. */
static inline __attribute__((always_inline)) void hop(double *acc, const double *psi, const double *U, int mu, int s, int dag,
                       int twisted, double pr, double pi)
{
  double h[2][6];
  /* the partner spin of h0 / h1 and its coefficient (kind, sign) */
  int j0, j1, k0, k1, g0, g1;
  switch (mu) {
  case 0: j0 = 2; j1 = 3; k0 = 0; g0 = -s; k1 = 0; g1 = -s; break;
  case 1: j0 = 3; j1 = 2; k0 = 1; g0 = -s; k1 = 1; g1 = -s; break;
  case 2: j0 = 3; j1 = 2; k0 = 0; g0 = -s; k1 = 0; g1 = s; break;
  default: j0 = 2; j1 = 3; k0 = 1; g0 = -s; k1 = 1; g1 = s; break;
  }
  for (int c = 0; c < 6; c++) {
    h[0][c] = psi[c];
    h[1][c] = psi[6 + c];
  }
  acc_coef(h[0], psi + 6 * j0, k0, g0);
  acc_coef(h[1], psi + 6 * j1, k1, g1);
  /* colour multiply of both half-spinor rows */
  double w[2][6];
  for (int r = 0; r < 2; r++)
    for (int a = 0; a < 3; a++) {
      double re = 0.0, im = 0.0;
      for (int b = 0; b < 3; b++) {
        double ur, ui;
        if (!dag) {
          ur = U[(a * 3 + b) * 2];
          ui = U[(a * 3 + b) * 2 + 1];
        } else {
          ur = U[(b * 3 + a) * 2];
          ui = -U[(b * 3 + a) * 2 + 1];
        }
        double hr = h[r][2 * b], hi = h[r][2 * b + 1];
        re += ur * hr - ui * hi;
        im += ur * hi + ui * hr;
      }
      if (twisted) {
        double t = re * pr - im * pi;
        im = re * pi + im * pr;
        re = t;
      }
      w[r][2 * a] = re;
      w[r][2 * a + 1] = im;
    }
  /* upper spins: the half spinor itself; lower spins: coefficient times a row */
  for (int c = 0; c < 6; c++) {
    acc[c] += w[0][c];
    acc[6 + c] += w[1][c];
  }
  switch (mu) {
  case 0: acc_coef(acc + 12, w[0], 0, -s); acc_coef(acc + 18, w[1], 0, -s); break;
  case 1: acc_coef(acc + 12, w[1], 1, s); acc_coef(acc + 18, w[0], 1, s); break;
  case 2: acc_coef(acc + 12, w[1], 0, s); acc_coef(acc + 18, w[0], 0, -s); break;
  default: acc_coef(acc + 12, w[0], 1, s); acc_coef(acc + 18, w[1], 1, -s); break;
  }
}

/* Dv = D v, D = (m+4) + i tm gamma_5 - 1/2 sum_mu [(1 - gamma_mu) U_mu(x) e^{i th/L} v(x+mu)
 *                                                + (1 + gamma_mu) U_mu(x-mu)^+ e^{-i th/L} v(x-mu)]
 * Returns 0, or 1 when the neighbour tables cannot be allocated. */
int orc_dslash_fast(double *Dv, const double *v, const double *u, const int L[4], const double theta[4],
                    double m, double tm)
{
  if (tables(L)) return 1;
  size_t V = (size_t)L[0] * L[1] * L[2] * L[3];
  int tw[4];
  double pr[4], pi[4];
  for (int mu = 0; mu < 4; mu++) {
    tw[mu] = theta[mu] != 0.0;
    pr[mu] = cos(theta[mu] / L[mu]);
    pi[mu] = sin(theta[mu] / L[mu]);
  }
  const double mp4 = m + 4.0;
  for (size_t l = 0; l < V; l++) {
    double acc[24];
    memset(acc, 0, sizeof(acc));
    const uint64_t *P = tab_plus + l * 4, *M = tab_minus + l * 4;
    const double *ul = u + l * 72;
    hop(acc, v + P[0] * 24, ul + 0, 0, -1, 0, tw[0], pr[0], pi[0]);
    hop(acc, v + P[1] * 24, ul + 18, 1, -1, 0, tw[1], pr[1], pi[1]);
    hop(acc, v + P[2] * 24, ul + 36, 2, -1, 0, tw[2], pr[2], pi[2]);
    hop(acc, v + P[3] * 24, ul + 54, 3, -1, 0, tw[3], pr[3], pi[3]);
    hop(acc, v + M[0] * 24, u + M[0] * 72 + 0, 0, 1, 1, tw[0], pr[0], -pi[0]);
    hop(acc, v + M[1] * 24, u + M[1] * 72 + 18, 1, 1, 1, tw[1], pr[1], -pi[1]);
    hop(acc, v + M[2] * 24, u + M[2] * 72 + 36, 2, 1, 1, tw[2], pr[2], -pi[2]);
    hop(acc, v + M[3] * 24, u + M[3] * 72 + 54, 3, 1, 1, tw[3], pr[3], -pi[3]);
    const double *p = v + l * 24;
    double *o = Dv + l * 24;
    for (int k = 0; k < 12; k++) {
      /* (m+4) psi + i tm gamma_5 psi: gamma_5 = +1 on spins 0, 1 and -1 on 2, 3 */
      double g5 = k < 6 ? tm : -tm;
      double re = p[2 * k], im = p[2 * k + 1];
      o[2 * k] = mp4 * re - g5 * im - 0.5 * acc[2 * k];
      o[2 * k + 1] = mp4 * im + g5 * re - 0.5 * acc[2 * k + 1];
    }
  }
  return 0;
}
