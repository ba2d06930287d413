/* qcd_oracle.c -- CPU restatement of qcd_lib's Wilson-twisted-mass path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the parity oracle for the GPU
 * library: only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it. Nothing in the product links, imports or calls it.
 *
 * Every routine is written from the mathematics the reference implements and
 * cites the reference routine it restates (paths relative to the reference
 * project root). All fields use the reference's host layout:
 *   spinor  [V][4 spin][3 colour]{re,im}           (include/qcd.h:90-97)
 *   gauge   [V][4 mu][3 row][3 col]{re,im}         (include/qcd.h:119-126)
 *   site    l = t + L0*(x + L1*(y + L2*z))          (include/qcd.h:144)
 *   mu = 0 is t; 1,2,3 are x,y,z.
 * Parity of this restatement is pinned against the reference library itself,
 * compiled unmodified into oracle/_ref, and against committed golden vectors.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double re, im; } cx;

static inline cx cmk(double r, double i) { cx z = {r, i}; return z; }
static inline cx cadd(cx a, cx b) { return cmk(a.re + b.re, a.im + b.im); }
static inline cx csub(cx a, cx b) { return cmk(a.re - b.re, a.im - b.im); }
static inline cx cmul(cx a, cx b) { return cmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline cx cconj(cx a) { return cmk(a.re, -a.im); }
static inline cx cscale(cx a, double s) { return cmk(a.re * s, a.im * s); }

/* Chiral ("twisted-mass") Dirac basis, gamma_5 = diag(1,1,-1,-1).
 * Same matrices as qcd_GAMMA[0..3] (lib/src/qcd_gamma.c:46-103); the values
 * are a convention the operator's output depends on, so they must agree. */
static const cx GAM[4][4][4] = {
  { {{0,0},{0,0},{-1,0},{0,0}}, {{0,0},{0,0},{0,0},{-1,0}},
    {{-1,0},{0,0},{0,0},{0,0}}, {{0,0},{-1,0},{0,0},{0,0}} },
  { {{0,0},{0,0},{0,0},{0,-1}}, {{0,0},{0,0},{0,-1},{0,0}},
    {{0,0},{0,1},{0,0},{0,0}},  {{0,1},{0,0},{0,0},{0,0}} },
  { {{0,0},{0,0},{0,0},{-1,0}}, {{0,0},{0,0},{1,0},{0,0}},
    {{0,0},{1,0},{0,0},{0,0}},  {{-1,0},{0,0},{0,0},{0,0}} },
  { {{0,0},{0,0},{0,-1},{0,0}}, {{0,0},{0,0},{0,0},{0,1}},
    {{0,1},{0,0},{0,0},{0,0}},  {{0,0},{0,-1},{0,0},{0,0}} },
};

/* ---------------------------------------------------------------- geometry */

static inline size_t vol(const int L[4]) { return (size_t)L[0] * L[1] * L[2] * L[3]; }

/* neighbour of site l one step along +mu (dir=+1) or -mu (dir=-1), periodic
 * inside the lattice: the single-rank tables of qcd_initGeometry
 * (lib/src/qcd_init.c:110-124). */
static inline size_t hop(size_t l, int mu, int dir, const int L[4])
{
  size_t c[4];
  size_t r = l;
  c[0] = r % L[0]; r /= L[0];
  c[1] = r % L[1]; r /= L[1];
  c[2] = r % L[2]; r /= L[2];
  c[3] = r;
  c[mu] = (c[mu] + (size_t)L[mu] + (size_t)dir) % (size_t)L[mu];
  return c[0] + (size_t)L[0] * (c[1] + (size_t)L[1] * (c[2] + (size_t)L[2] * c[3]));
}

#define SP(v, l) ((const cx (*)[3])((v) + (size_t)(l) * 24))
#define SPW(v, l) ((cx (*)[3])((v) + (size_t)(l) * 24))
#define LINK(u, l, mu) ((const cx (*)[3])((u) + ((size_t)(l) * 4 + (mu)) * 18))

/* ------------------------------------------------------------ Dirac operator */

/* res = (1 + sign*gamma_mu) psi, full 4x3 spinor (lib/src/qcd_wilson.c:18-44) */
static void one_pm_gamma(cx res[4][3], const cx psi[4][3], int mu, int sign)
{
  for (int a = 0; a < 4; a++)
    for (int c = 0; c < 3; c++) {
      cx s = psi[a][c];
      for (int b = 0; b < 4; b++) {
        cx g = GAM[mu][a][b];
        if (g.re == 0.0 && g.im == 0.0) continue;
        cx t = cmul(g, psi[b][c]);
        s = sign > 0 ? cadd(s, t) : csub(s, t);
      }
      res[a][c] = s;
    }
}

/* res = U psi (dag=0) or U^dagger psi (dag=1) on every spin component
 * (lib/src/qcd_wilson.c:47-73) */
static void apply_link(cx res[4][3], const cx U[3][3], const cx psi[4][3], int dag)
{
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++) {
      cx s = cmk(0, 0);
      for (int j = 0; j < 3; j++)
        s = cadd(s, cmul(dag ? cconj(U[j][i]) : U[i][j], psi[a][j]));
      res[a][i] = s;
    }
}

/* Dv = D v with
 *   D = (m+4) + i tm gamma_5
 *       - 1/2 sum_mu [ (1-gamma_mu) U_mu(x) e^{+i th_mu/L_mu} v(x+mu)
 *                    + (1+gamma_mu) U_mu(x-mu)^dag e^{-i th_mu/L_mu} v(x-mu) ]
 * qcd_applyWilsonTMOp (lib/src/qcd_wilson.c:114-336); the phase is applied
 * on every hop along mu with theta_mu != 0 (:172-186, :238-257). */
void orc_dslash(double *Dv, const double *v, const double *u, const int L[4],
                const double theta[4], double m, double tm)
{
  size_t V = vol(L);
  cx ph[4];
  int twisted[4];
  for (int mu = 0; mu < 4; mu++) {
    twisted[mu] = theta[mu] != 0.0;
    ph[mu] = cmk(cos(theta[mu] / L[mu]), sin(theta[mu] / L[mu]));
  }
  double mp4 = m + 4.0;
  for (size_t l = 0; l < V; l++) {
    cx acc[4][3];
    memset(acc, 0, sizeof(acc));
    for (int mu = 0; mu < 4; mu++) {
      cx p[4][3], q[4][3];
      size_t fw = hop(l, mu, +1, L), bw = hop(l, mu, -1, L);
      one_pm_gamma(p, SP(v, fw), mu, -1);
      apply_link(q, LINK(u, l, mu), p, 0);
      for (int a = 0; a < 4; a++)
        for (int c = 0; c < 3; c++)
          acc[a][c] = cadd(acc[a][c], twisted[mu] ? cmul(q[a][c], ph[mu]) : q[a][c]);
      one_pm_gamma(p, SP(v, bw), mu, +1);
      apply_link(q, LINK(u, bw, mu), p, 1);
      for (int a = 0; a < 4; a++)
        for (int c = 0; c < 3; c++)
          acc[a][c] = cadd(acc[a][c], twisted[mu] ? cmul(q[a][c], cconj(ph[mu])) : q[a][c]);
    }
    const cx(*s)[3] = SP(v, l);
    cx(*o)[3] = SPW(Dv, l);
    for (int a = 0; a < 4; a++) {
      double g5 = a < 2 ? 1.0 : -1.0;
      for (int c = 0; c < 3; c++) {
        cx d = cscale(s[a][c], mp4);
        d = cadd(d, cmul(cmk(0, tm * g5), s[a][c]));
        o[a][c] = csub(d, cscale(acc[a][c], 0.5));
      }
    }
  }
}

/* Dv = i gamma_5 D v: spins 0,1 times +i, spins 2,3 times -i
 * (qcd_applyQTMOp, lib/src/qcd_wilson.c:795-814) */
void orc_qop(double *Dv, const double *v, const double *u, const int L[4],
             const double theta[4], double m, double tm)
{
  orc_dslash(Dv, v, u, L, theta, m, tm);
  size_t V = vol(L);
  for (size_t l = 0; l < V; l++) {
    cx(*o)[3] = SPW(Dv, l);
    for (int a = 0; a < 4; a++)
      for (int c = 0; c < 3; c++)
        o[a][c] = a < 2 ? cmk(-o[a][c].im, o[a][c].re) : cmk(o[a][c].im, -o[a][c].re);
  }
}

/* out = gamma_5 in (qcd_gamma5Vector, lib/src/qcd_gamma.c:521-533); in==out allowed */
void orc_gamma5(double *out, const double *in, size_t V)
{
  for (size_t l = 0; l < V; l++)
    for (int k = 0; k < 24; k++)
      out[l * 24 + k] = k < 12 ? in[l * 24 + k] : -in[l * 24 + k];
}

/* D(tm)^dagger = gamma_5 D(-tm) gamma_5 (gamma_5-hermiticity of the Wilson-TM
 * operator; no reference counterpart, used by the normal-equation solver). */
void orc_dslash_dag(double *Dv, const double *v, const double *u, const int L[4],
                    const double theta[4], double m, double tm)
{
  size_t V = vol(L);
  double *w = malloc(V * 24 * sizeof(double));
  orc_gamma5(w, v, V);
  orc_dslash(Dv, w, u, L, theta, m, -tm);
  orc_gamma5(Dv, Dv, V);
  free(w);
}

/* ------------------------------------------------------------------ BLAS-1 */

/* sqrt(sum v_i^2) accumulated in storage order (qcd_normVector,
 * lib/src/qcd_blas.c:478-492) */
double orc_norm(const double *v, size_t V)
{
  double s = 0;
  for (size_t i = 0; i < V * 24; i++) s += v[i] * v[i];
  return sqrt(s);
}

/* sum conj(a_i) b_i in storage order (qcd_mulAdjointVectorVector,
 * lib/src/qcd_blas.c:456-476) */
void orc_dot(double out[2], const double *a, const double *b, size_t V)
{
  double re = 0, im = 0;
  for (size_t i = 0; i < V * 12; i++) {
    re += a[2 * i] * b[2 * i] + a[2 * i + 1] * b[2 * i + 1];
    im += a[2 * i] * b[2 * i + 1] - a[2 * i + 1] * b[2 * i];
  }
  out[0] = re; out[1] = im;
}

/* out = a x + y, a complex; out may alias x or y (qcd_axpyVector,
 * lib/src/qcd_blas.c:414-432) */
void orc_axpy(double *out, double are, double aim, const double *x, const double *y, size_t V)
{
  for (size_t i = 0; i < V * 12; i++) {
    double xr = x[2 * i], xi = x[2 * i + 1];
    double yr = y[2 * i], yi = y[2 * i + 1];
    out[2 * i] = yr + xr * are - xi * aim;
    out[2 * i + 1] = yi + xi * are + xr * aim;
  }
}

/* out = s*in (qcd_scaleVector :301), out = c*in (qcd_mulVectorC :237),
 * out = a+b (qcd_addVector :403), out = a-b (qcd_subVector :345) */
void orc_scale(double *out, const double *in, double s, size_t V)
{ for (size_t i = 0; i < V * 24; i++) out[i] = in[i] * s; }
void orc_mulc(double *out, const double *in, double cre, double cim, size_t V)
{
  for (size_t i = 0; i < V * 12; i++) {
    double r = in[2 * i], m = in[2 * i + 1];
    out[2 * i] = r * cre - m * cim;
    out[2 * i + 1] = r * cim + m * cre;
  }
}
void orc_add(double *out, const double *a, const double *b, size_t V)
{ for (size_t i = 0; i < V * 24; i++) out[i] = a[i] + b[i]; }
void orc_sub(double *out, const double *a, const double *b, size_t V)
{ for (size_t i = 0; i < V * 24; i++) out[i] = a[i] - b[i]; }

/* ----------------------------------------------------------------- solvers */

typedef struct {
  const double *u;
  const int *L;
  const double *theta;
  double m, tm;
  int op; /* 0: D, 1: Q = i gamma_5 D, 2: D^dag D */
  double *tmp;
} opctx;

static void apply_op(const opctx *c, double *out, const double *in)
{
  if (c->op == 0) orc_dslash(out, in, c->u, c->L, c->theta, c->m, c->tm);
  else if (c->op == 1) orc_qop(out, in, c->u, c->L, c->theta, c->m, c->tm);
  else {
    orc_dslash(c->tmp, in, c->u, c->L, c->theta, c->m, c->tm);
    orc_dslash_dag(out, c->tmp, c->u, c->L, c->theta, c->m, c->tm);
  }
}

/* n-step GCR on Q = i gamma_5 D with modified Gram-Schmidt, following gcr()
 * in invert.c:20-113. With fixed=0 the solution update omits the first basis
 * term, exactly as shipped (invert.c:52-53 are commented out); with fixed=1
 * it starts from x = a00 c0 rho0 as the algorithm's specification gcr.m does.
 * Returns 0, or 1 when the Krylov space degenerates (NaN norm, :75-79). */
int orc_gcr(double *sol, const double *src, const double *u, const int L[4],
            const double theta[4], double kappa, double mu, int n, int fixed)
{
  size_t V = vol(L), N = V * 24;
  double m = 1.0 / (2.0 * kappa) - 4.0;
  double *chi = malloc((size_t)n * N * sizeof(double));
  double *res = malloc((size_t)n * N * sizeof(double));
  cx *a = calloc((size_t)n * n, sizeof(cx));
  cx *c = calloc((size_t)n, sizeof(cx));
  int rc = 0;
#define CHI(k) (chi + (size_t)(k) * N)
#define RES(k) (res + (size_t)(k) * N)
#define A(i, j) a[(size_t)(i) * n + (j)]
  memcpy(RES(0), src, N * sizeof(double));
  orc_qop(CHI(0), RES(0), u, L, theta, m, mu);
  A(0, 0) = cmk(1.0 / orc_norm(CHI(0), V), 0);
  orc_scale(CHI(0), CHI(0), A(0, 0).re, V);
  double d[2];
  orc_dot(d, CHI(0), src, V);
  c[0] = cmk(d[0], d[1]);
  memset(sol, 0, N * sizeof(double));
  if (fixed) {
    cx f = cmul(c[0], A(0, 0));
    orc_axpy(sol, f.re, f.im, RES(0), sol, V);
  }
  for (int k = 1; k < n; k++) {
    orc_axpy(RES(k), -c[k - 1].re, -c[k - 1].im, CHI(k - 1), RES(k - 1), V);
    orc_qop(CHI(k), RES(k), u, L, theta, m, mu);
    for (int j = 0; j < k; j++) {
      orc_dot(d, CHI(j), CHI(k), V);
      A(k, j) = cmk(-d[0], -d[1]);
      orc_axpy(CHI(k), A(k, j).re, A(k, j).im, CHI(j), CHI(k), V);
    }
    A(k, k) = cmk(1.0 / orc_norm(CHI(k), V), 0);
    if (isnan(A(k, k).re)) { rc = 1; break; }
    orc_scale(CHI(k), CHI(k), A(k, k).re, V);
    for (int j = 0; j < k; j++) A(k, j) = cscale(A(k, j), A(k, k).re);
    for (int j = 0; j < k; j++) {
      A(k, j) = cscale(A(k, j), A(j, j).re);
      for (int l = j + 1; l < k; l++) A(k, j) = cadd(A(k, j), cmul(A(k, l), A(l, j)));
    }
    orc_dot(d, CHI(k), src, V);
    c[k] = cmk(d[0], d[1]);
    for (int j = 0; j <= k; j++) {
      cx f = cmul(c[k], A(k, j));
      orc_axpy(sol, f.re, f.im, RES(j), sol, V);
    }
  }
#undef CHI
#undef RES
#undef A
  free(chi); free(res); free(a); free(c);
  return rc;
}

/* Restarted GCR with iterative refinement until |b - Qx|/|b| <= maxres, the
 * per-column loop of invert.c main (invert.c:255-294). Returns the number of
 * GCR cycles; *relres receives the final true relative residual. */
int orc_invert_gcr(double *sol, const double *src, const double *u, const int L[4],
                   const double theta[4], double kappa, double mu, int n, int fixed,
                   double maxres, int maxiter, double *relres)
{
  size_t V = vol(L), N = V * 24;
  double m = 1.0 / (2.0 * kappa) - 4.0;
  double *res = malloc(N * sizeof(double)), *cor = malloc(N * sizeof(double));
  double nsrc = orc_norm(src, V);
  int iter = 1;
  orc_gcr(sol, src, u, L, theta, kappa, mu, n, fixed);
  orc_qop(res, sol, u, L, theta, m, mu);
  orc_sub(res, src, res, V);
  double nr = orc_norm(res, V) / nsrc;
  while (nr > maxres && iter < maxiter) {
    orc_gcr(cor, res, u, L, theta, kappa, mu, n, fixed);
    orc_add(sol, sol, cor, V);
    orc_qop(res, sol, u, L, theta, m, mu);
    orc_sub(res, src, res, V);
    nr = orc_norm(res, V) / nsrc;
    iter++;
  }
  *relres = nr;
  free(res); free(cor);
  return iter;
}

/* BiCGstab (H. A. van der Vorst, SIAM J. Sci. Stat. Comput. 13 (1992) 631)
 * for A x = b with A = D (op 0) or Q (op 1), x0 = 0, stopping on the
 * iterated residual |r|/|b| <= tol. No reference counterpart: qcd_lib has
 * GCR only. Returns iterations, or -1 on breakdown (rho or omega = 0). */
int orc_bicgstab(double *x, const double *b, const double *u, const int L[4],
                 const double theta[4], double kappa, double mu, int op,
                 double tol, int maxiter, double *relres)
{
  size_t V = vol(L), N = V * 24;
  opctx c = {u, L, theta, 1.0 / (2.0 * kappa) - 4.0, mu, op, NULL};
  double *r = malloc(N * 8), *rh = malloc(N * 8), *p = calloc(N, 8), *v = calloc(N, 8);
  double *s = malloc(N * 8), *t = malloc(N * 8);
  memset(x, 0, N * 8);
  memcpy(r, b, N * 8);
  memcpy(rh, b, N * 8);
  cx rho = cmk(1, 0), alpha = cmk(1, 0), omega = cmk(1, 0);
  double nb = orc_norm(b, V), d[2];
  int it = 0, rc = 0;
  double rr = 1.0;
  if (nb == 0.0) { *relres = 0; goto done; }
  for (it = 1; it <= maxiter; it++) {
    orc_dot(d, rh, r, V);
    cx rho1 = cmk(d[0], d[1]);
    if (rho1.re == 0.0 && rho1.im == 0.0) { rc = -1; break; }
    /* beta = (rho1/rho) (alpha/omega) */
    cx num = cmul(rho1, alpha), den = cmul(rho, omega);
    double dd = den.re * den.re + den.im * den.im;
    cx beta = cmk((num.re * den.re + num.im * den.im) / dd, (num.im * den.re - num.re * den.im) / dd);
    /* p = r + beta (p - omega v) */
    for (size_t i = 0; i < N / 2; i++) {
      cx pv = cmk(p[2 * i], p[2 * i + 1]), vv = cmk(v[2 * i], v[2 * i + 1]);
      cx q = cadd(cmk(r[2 * i], r[2 * i + 1]), cmul(beta, csub(pv, cmul(omega, vv))));
      p[2 * i] = q.re; p[2 * i + 1] = q.im;
    }
    apply_op(&c, v, p);
    orc_dot(d, rh, v, V);
    dd = d[0] * d[0] + d[1] * d[1];
    alpha = cmk((rho1.re * d[0] + rho1.im * d[1]) / dd, (rho1.im * d[0] - rho1.re * d[1]) / dd);
    orc_axpy(s, -alpha.re, -alpha.im, v, r, V);
    rr = orc_norm(s, V) / nb;
    if (rr <= tol) { orc_axpy(x, alpha.re, alpha.im, p, x, V); break; }
    apply_op(&c, t, s);
    double ts[2];
    orc_dot(ts, t, s, V);
    double tt = orc_norm(t, V);
    tt *= tt;
    omega = cmk(ts[0] / tt, ts[1] / tt);
    if (omega.re == 0.0 && omega.im == 0.0) { rc = -1; break; }
    orc_axpy(x, alpha.re, alpha.im, p, x, V);
    orc_axpy(x, omega.re, omega.im, s, x, V);
    orc_axpy(r, -omega.re, -omega.im, t, s, V);
    rr = orc_norm(r, V) / nb;
    rho = rho1;
    if (rr <= tol) break;
  }
  *relres = rr;
done:
  free(r); free(rh); free(p); free(v); free(s); free(t);
  return rc < 0 ? -1 : it;
}

/* Conjugate gradient (Hestenes-Stiefel 1952) on the normal equations
 * D^dag D x = D^dag b, stopping on |D^dag(b - D x)| <= tol |D^dag b|.
 * No reference counterpart. Returns iterations. */
int orc_cgnr(double *x, const double *b, const double *u, const int L[4],
             const double theta[4], double kappa, double mu, double tol,
             int maxiter, double *relres)
{
  size_t V = vol(L), N = V * 24;
  double m = 1.0 / (2.0 * kappa) - 4.0;
  opctx c = {u, L, theta, m, mu, 2, malloc(N * 8)};
  double *r = malloc(N * 8), *p = malloc(N * 8), *q = malloc(N * 8);
  memset(x, 0, N * 8);
  orc_dslash_dag(r, b, u, L, theta, m, mu);
  memcpy(p, r, N * 8);
  double n0 = orc_norm(r, V), rr = n0 * n0;
  int it = 0;
  double rel = 1.0;
  if (n0 == 0.0) { rel = 0; goto done; }
  for (it = 1; it <= maxiter; it++) {
    apply_op(&c, q, p);
    double pq[2];
    orc_dot(pq, p, q, V);
    double alpha = rr / pq[0];
    orc_axpy(x, alpha, 0, p, x, V);
    orc_axpy(r, -alpha, 0, q, r, V);
    double rn = orc_norm(r, V);
    rel = rn / n0;
    if (rel <= tol) break;
    double beta = rn * rn / rr;
    rr = rn * rn;
    orc_axpy(p, beta, 0, p, r, V);
  }
done:
  *relres = rel;
  free(c.tmp); free(r); free(p); free(q);
  return it;
}

/* |b - A x| / |b| in FP64 with A = D (op 0) or Q (op 1): the check of
 * b_minus_Dx.c:152-169 */
double orc_true_residual(const double *x, const double *b, const double *u, const int L[4],
                         const double theta[4], double kappa, double mu, int op)
{
  size_t V = vol(L);
  double *t = malloc(V * 24 * 8);
  double m = 1.0 / (2.0 * kappa) - 4.0;
  if (op == 1) orc_qop(t, x, u, L, theta, m, mu);
  else orc_dslash(t, x, u, L, theta, m, mu);
  orc_sub(t, b, t, V);
  double r = orc_norm(t, V) / orc_norm(b, V);
  free(t);
  return r;
}

/* ------------------------------------------------------------ 3x3 algebra */

static void m3mul(cx c[3][3], const cx a[3][3], const cx b[3][3])
{
  cx t[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      cx s = cmk(0, 0);
      for (int k = 0; k < 3; k++) s = cadd(s, cmul(a[i][k], b[k][j]));
      t[i][j] = s;
    }
  memcpy(c, t, sizeof(t));
}
static void m3dag(cx c[3][3], const cx a[3][3])
{
  cx t[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) t[i][j] = cconj(a[j][i]);
  memcpy(c, t, sizeof(t));
}
static cx m3det(const cx m[3][3])
{
  cx d = cmul(m[0][0], csub(cmul(m[1][1], m[2][2]), cmul(m[1][2], m[2][1])));
  d = csub(d, cmul(m[0][1], csub(cmul(m[1][0], m[2][2]), cmul(m[1][2], m[2][0]))));
  return cadd(d, cmul(m[0][2], csub(cmul(m[1][0], m[2][1]), cmul(m[1][1], m[2][0]))));
}
static void m3inv(cx r[3][3], const cx m[3][3])
{
  cx d = m3det(m);
  double dd = d.re * d.re + d.im * d.im;
  cx id = cmk(d.re / dd, -d.im / dd);
  cx t[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      int i1 = (j + 1) % 3, i2 = (j + 2) % 3, j1 = (i + 1) % 3, j2 = (i + 2) % 3;
      cx cof = csub(cmul(m[i1][j1], m[i2][j2]), cmul(m[i1][j2], m[i2][j1]));
      t[i][j] = cmul(cof, id);
    }
  memcpy(r, t, sizeof(t));
}

/* exp(iM) for traceless Hermitian M by the Cayley-Hamilton formula of
 * C. Morningstar and M. Peardon, Phys. Rev. D 69 (2004) 054501
 * [hep-lat/0311018], eqs. (19)-(34): the reference's Exp()
 * (lib/src/qcd_smearing.c:293-371). M is overwritten. */
static double sinc_mp(double w)
{
  if (fabs(w) < 0.05) {
    double w2 = w * w;
    return 1.0 - w2 / 6.0 * (1.0 - w2 / 20.0 * (1.0 - w2 / 42.0));
  }
  return sin(w) / w;
}
void orc_exp_iM(double *Mflat)
{
  cx(*M)[3] = (cx(*)[3])Mflat;
  cx M2[3][3], M3[3][3];
  m3mul(M2, (const cx(*)[3])M, (const cx(*)[3])M);
  m3mul(M3, (const cx(*)[3])M2, (const cx(*)[3])M);
  double c0 = (M3[0][0].re + M3[1][1].re + M3[2][2].re) / 3.0;
  double c1 = (M2[0][0].re + M2[1][1].re + M2[2][2].re) / 2.0;
  int neg = c0 < 0;
  if (neg) c0 = -c0;
  double c0max = 2.0 * pow(c1 / 3.0, 1.5);
  double ratio = c0 / c0max;
  if (ratio > 1.0) ratio = 1.0; /* rounding guard for nearly degenerate spectra */
  double th = acos(ratio);
  double uu = sqrt(c1 / 3.0) * cos(th / 3.0);
  double w = sqrt(c1) * sin(th / 3.0);
  double xi = sinc_mp(w), cw = cos(w);
  cx e2iu = cmk(cos(2 * uu), sin(2 * uu)), emiu = cmk(cos(uu), -sin(uu));
  cx h0 = cadd(cmul(cmk(uu * uu - w * w, 0), e2iu),
               cmul(emiu, cmk(8 * uu * uu * cw, 2 * uu * (3 * uu * uu + w * w) * xi)));
  cx h1 = csub(cmul(cmk(2 * uu, 0), e2iu), cmul(emiu, cmk(2 * uu * cw, -(3 * uu * uu - w * w) * xi)));
  cx h2 = csub(e2iu, cmul(emiu, cmk(cw, 3 * uu * xi)));
  double den = 9 * uu * uu - w * w;
  cx f0 = cscale(h0, 1.0 / den), f1 = cscale(h1, 1.0 / den), f2 = cscale(h2, 1.0 / den);
  if (neg) { f0 = cconj(f0); f1 = cconj(cscale(f1, -1.0)); f2 = cconj(f2); }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      cx s = cadd(cmul(f1, M[i][j]), cmul(f2, M2[i][j]));
      if (i == j) s = cadd(s, f0);
      M[i][j] = s;
    }
}

/* Gram-Schmidt on the columns and col2 = conj(col0 x col1): the last stage
 * of qcd_projectSU33x3 (lib/src/qcd_blas.c:1700-1766) */
static void reunit_cols(cx U[3][3])
{
  double n = 0;
  for (int i = 0; i < 3; i++) n += U[i][0].re * U[i][0].re + U[i][0].im * U[i][0].im;
  cx w = cmk(0, 0);
  for (int i = 0; i < 3; i++) w = cadd(w, cmul(cconj(U[i][0]), U[i][1]));
  w = cscale(w, 1.0 / n);
  for (int i = 0; i < 3; i++) U[i][1] = csub(U[i][1], cmul(w, U[i][0]));
  double s = 1.0 / sqrt(n);
  for (int i = 0; i < 3; i++) U[i][0] = cscale(U[i][0], s);
  n = 0;
  for (int i = 0; i < 3; i++) n += U[i][1].re * U[i][1].re + U[i][1].im * U[i][1].im;
  s = 1.0 / sqrt(n);
  for (int i = 0; i < 3; i++) U[i][1] = cscale(U[i][1], s);
  U[0][2] = cconj(csub(cmul(U[1][0], U[2][1]), cmul(U[2][0], U[1][1])));
  U[1][2] = cconj(csub(cmul(U[2][0], U[0][1]), cmul(U[0][0], U[2][1])));
  U[2][2] = cconj(csub(cmul(U[0][0], U[1][1]), cmul(U[1][0], U[0][1])));
}

/* Projection onto SU(3): unitary polar factor W = M (M^dag M)^{-1/2}, times
 * exp(-i arg(det M)/3), then column re-orthonormalisation -- the result
 * qcd_projectSU33x3 computes (lib/src/qcd_blas.c:1376-1766, after
 * Phys. Lett. B307 (1993) 375). The polar factor is found here by Newton's
 * iteration W <- (W + W^{-dag})/2 (N. J. Higham, SIAM J. Sci. Stat. Comput.
 * 7 (1986) 1160), not by the reference's closed-form eigen-decomposition. */
void orc_project_su3(double *gflat)
{
  cx(*g)[3] = (cx(*)[3])gflat;
  cx M[3][3], W[3][3], Wi[3][3];
  memcpy(M, g, sizeof(M));
  cx d = m3det((const cx(*)[3])M);
  double phase = atan2(d.im, d.re) / 3.0;
  memcpy(W, M, sizeof(W));
  for (int it = 0; it < 100; it++) {
    m3inv(Wi, (const cx(*)[3])W);
    m3dag(Wi, (const cx(*)[3])Wi);
    double diff = 0, nrm = 0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        cx nw = cscale(cadd(W[i][j], Wi[i][j]), 0.5);
        diff += fabs(nw.re - W[i][j].re) + fabs(nw.im - W[i][j].im);
        nrm += fabs(nw.re) + fabs(nw.im);
        W[i][j] = nw;
      }
    if (diff <= 1e-15 * nrm) break;
  }
  cx ph = cmk(cos(phase), -sin(phase));
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) W[i][j] = cmul(W[i][j], ph);
  reunit_cols(W);
  memcpy(g, W, sizeof(W));
}

/* -------------------------------------------------------------- observables */

/* mean plaquette, Re tr over 6 planes, normalised to 1 on the unit field
 * (qcd_calculatePlaquette, lib/src/qcd_observables.c:15-36) */
double orc_plaquette(const double *u, const int L[4])
{
  size_t V = vol(L);
  double s = 0;
  for (size_t l = 0; l < V; l++)
    for (int mu = 0; mu < 3; mu++)
      for (int nu = mu + 1; nu < 4; nu++) {
        cx a[3][3], b[3][3];
        m3mul(a, LINK(u, l, mu), LINK(u, hop(l, mu, 1, L), nu));
        m3dag(b, LINK(u, hop(l, nu, 1, L), mu));
        m3mul(a, (const cx(*)[3])a, (const cx(*)[3])b);
        m3dag(b, LINK(u, l, nu));
        m3mul(a, (const cx(*)[3])a, (const cx(*)[3])b);
        s += a[0][0].re + a[1][1].re + a[2][2].re;
      }
  return s / ((double)V * 18.0);
}

/* ---------------------------------------------------------------- smearing */

/* one 3D APE step: spatial links -> Proj_SU3(U + alpha * sum of the four
 * spatial staples); temporal links copied (qcd_apeSmear3d,
 * lib/src/qcd_smearing.c:209-276 with qcd_projectSU33d, lib/src/qcd_blas.c:950) */
void orc_ape3d(double *out, const double *u, const int L[4], double alpha)
{
  size_t V = vol(L);
  for (size_t l = 0; l < V; l++) {
    memcpy(out + (l * 4) * 18, u + (l * 4) * 18, 18 * 8);
    for (int mu = 1; mu < 4; mu++) {
      cx S[3][3], t[3][3], w[3][3];
      memset(S, 0, sizeof(S));
      for (int nu = 1; nu < 4; nu++) {
        if (nu == mu) continue;
        /* forward: U_nu(x) U_mu(x+nu) U_nu(x+mu)^dag */
        m3mul(t, LINK(u, l, nu), LINK(u, hop(l, nu, 1, L), mu));
        m3dag(w, LINK(u, hop(l, mu, 1, L), nu));
        m3mul(t, (const cx(*)[3])t, (const cx(*)[3])w);
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) S[i][j] = cadd(S[i][j], t[i][j]);
        /* backward: U_nu(x-nu)^dag U_mu(x-nu) U_nu(x-nu+mu) */
        size_t b = hop(l, nu, -1, L);
        m3dag(w, LINK(u, b, nu));
        m3mul(t, (const cx(*)[3])w, LINK(u, b, mu));
        m3mul(t, (const cx(*)[3])t, LINK(u, hop(b, mu, 1, L), nu));
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) S[i][j] = cadd(S[i][j], t[i][j]);
      }
      const cx(*U)[3] = LINK(u, l, mu);
      cx(*O)[3] = (cx(*)[3])(out + (l * 4 + mu) * 18);
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) O[i][j] = cadd(U[i][j], cscale(S[i][j], alpha));
      orc_project_su3((double *)O);
    }
  }
}

/* one Gaussian smearing step on time-slice t: v -> (v + alpha H v)/(1+6 alpha)
 * with H v(x) = sum_{nu=1..3} U_nu(x) v(x+nu) + U_nu(x-nu)^dag v(x-nu);
 * other time-slices unchanged (qcd_gaussIteration3d,
 * lib/src/qcd_smearing.c:25-113) */
void orc_gauss3d(double *v, const double *u, const int L[4], double alpha, int t)
{
  size_t V = vol(L);
  double nrm = 1.0 / (1.0 + 6.0 * alpha);
  double *h = calloc(V * 24, 8);
  for (size_t l = 0; l < V; l++) {
    if ((int)(l % L[0]) != t) continue;
    cx(*o)[3] = SPW(h, l);
    for (int nu = 1; nu < 4; nu++) {
      cx q[4][3];
      apply_link(q, LINK(u, l, nu), SP(v, hop(l, nu, 1, L)), 0);
      for (int a = 0; a < 4; a++) for (int c = 0; c < 3; c++) o[a][c] = cadd(o[a][c], q[a][c]);
      size_t b = hop(l, nu, -1, L);
      apply_link(q, LINK(u, b, nu), SP(v, b), 1);
      for (int a = 0; a < 4; a++) for (int c = 0; c < 3; c++) o[a][c] = cadd(o[a][c], q[a][c]);
    }
  }
  for (size_t l = 0; l < V; l++) {
    if ((int)(l % L[0]) != t) continue;
    for (int k = 0; k < 24; k++) v[l * 24 + k] = (v[l * 24 + k] + alpha * h[l * 24 + k]) * nrm;
  }
  free(h);
}

/* ------------------------------------------------- seeded synthetic inputs */

/* Counter-based generator: the SplitMix64 output function (S. Vigna,
 * public domain) applied to a seed-keyed counter. Identical integer
 * arithmetic runs in the GPU library's input generator. */
static inline uint64_t mix64(uint64_t z)
{
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
uint64_t orc_rng_bits(uint64_t seed, uint64_t ctr)
{
  return mix64(mix64(seed * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull) ^ ctr);
}
/* uniform in (0,1) */
double orc_uniform(uint64_t seed, uint64_t ctr)
{
  return ((double)(orc_rng_bits(seed, ctr) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
/* standard normal by Box-Muller from counters 2k and 2k+1 */
double orc_gauss(uint64_t seed, uint64_t k)
{
  double u1 = orc_uniform(seed, 2 * k), u2 = orc_uniform(seed, 2 * k + 1);
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

/* spinor with re, im ~ N(0,1): component k of site l uses counter 24 l + k */
void orc_gaussian_spinor(double *v, size_t V, uint64_t seed)
{
  for (size_t i = 0; i < V * 24; i++) v[i] = orc_gauss(seed, i);
}

/* Z4 noise {+1,+i,-1,-i} per spin-colour component on every site, the
 * values of qcd_z2Vector (lib/src/qcd_stochastic.c:8-58); the stream is this
 * generator's (the reference draws from GSL's ranlux, absent here). */
/* Z4 (kind 4) or Z2 (kind 2) noise on time-slice ts (all sites when ts < 0),
 * the stochastic source of lib/src/qcd_stochastic.c:8-58 drawn from this
 * counter-based stream instead of GSL's ranlux: component k of site l from
 * counter 12 l + k (Z4: top two bits; Z2: top bit) */
void orc_noise_spinor(double *v, const int L[4], uint64_t seed, int ts, int kind)
{
  size_t V = vol(L);
  static const double re[4] = {1, 0, -1, 0}, im[4] = {0, 1, 0, -1};
  for (size_t l = 0; l < V; l++)
    for (int k = 0; k < 12; k++) {
      size_t i = l * 12 + k;
      uint64_t b = orc_rng_bits(seed, i);
      if (ts >= 0 && (int)(l % (size_t)L[0]) != ts) {
        v[2 * i] = 0.0; v[2 * i + 1] = 0.0;
      } else if (kind == 2) {
        v[2 * i] = (b >> 63) ? -1.0 : 1.0; v[2 * i + 1] = 0.0;
      } else {
        unsigned r = (unsigned)(b >> 62);
        v[2 * i] = re[r]; v[2 * i + 1] = im[r];
      }
    }
}

void orc_z4_spinor(double *v, size_t V, uint64_t seed)
{
  for (size_t i = 0; i < V * 12; i++) {
    unsigned r = (unsigned)(orc_rng_bits(seed, i) >> 62);
    static const double re[4] = {1, 0, -1, 0}, im[4] = {0, 1, 0, -1};
    v[2 * i] = re[r]; v[2 * i + 1] = im[r];
  }
}

/* Synthetic gauge field: U_mu(x) = exp(i eps H), H = sum_a g_a lambda_a / 2
 * with g_a ~ N(0,1) from counter 8 (4 l + mu) + a, exponentiated with the
 * Cayley-Hamilton formula and re-orthonormalised. */
void orc_gauge_synthetic(double *u, const int L[4], uint64_t seed, double eps)
{
  size_t V = vol(L);
  const double s3 = 1.0 / sqrt(3.0);
  for (size_t l = 0; l < V; l++)
    for (int mu = 0; mu < 4; mu++) {
      double g[8];
      for (int a = 0; a < 8; a++) g[a] = 0.5 * eps * orc_gauss(seed, (l * 4 + mu) * 8 + a);
      cx H[3][3];
      /* sum_a g_a lambda_a with the Gell-Mann matrices */
      H[0][0] = cmk(g[2] + g[7] * s3, 0);
      H[1][1] = cmk(-g[2] + g[7] * s3, 0);
      H[2][2] = cmk(-2.0 * g[7] * s3, 0);
      H[0][1] = cmk(g[0], -g[1]); H[1][0] = cmk(g[0], g[1]);
      H[0][2] = cmk(g[3], -g[4]); H[2][0] = cmk(g[3], g[4]);
      H[1][2] = cmk(g[5], -g[6]); H[2][1] = cmk(g[5], g[6]);
      orc_exp_iM((double *)H);
      reunit_cols(H);
      memcpy(u + (l * 4 + mu) * 18, H, 18 * 8);
    }
}

/* the unit gauge field U = 1 (unit_gaugefield.c) */
void orc_gauge_unit(double *u, size_t V)
{
  memset(u, 0, V * 4 * 18 * 8);
  for (size_t l = 0; l < V * 4; l++) { u[l * 18 + 0] = 1; u[l * 18 + 8] = 1; u[l * 18 + 16] = 1; }
}

/* ------------------------------------------------------- contractions */

/* Tables of the proton two-point function (kept identical to the
 * reference's): the antisymmetric colour permutations qcd_EPS / qcd_SGN_EPS
 * (lib/src/qcd_gamma.c:13-26), C gamma_5 and its bar (qcd_CGAMMA[5],
 * qcd_BAR_CGAMMA[5], lib/src/qcd_gamma.c:105-195) and the parity projector
 * PROJECTOR[13] (projectors.h). */
static const int TP_EPS[6][3] = {{0, 1, 2}, {2, 0, 1}, {1, 2, 0}, {2, 1, 0}, {0, 2, 1}, {1, 0, 2}};
static const int TP_SGN[6] = {+1, +1, +1, -1, -1, -1};
static const double TP_CG5[4][4] = {{0, 1, 0, 0}, {-1, 0, 0, 0}, {0, 0, 0, 1}, {0, 0, -1, 0}};
static const double TP_BCG5[4][4] = {{0, -1, 0, 0}, {1, 0, 0, 0}, {0, 0, 0, -1}, {0, 0, 1, 0}};
static const double TP_P13[4][4][2] = {{{0, .5}, {0, 0}, {-.5, 0}, {0, 0}},
                                       {{0, 0}, {0, .5}, {0, 0}, {-.5, 0}},
                                       {{-.5, 0}, {0, 0}, {0, -.5}, {0, 0}},
                                       {{0, 0}, {-.5, 0}, {0, 0}, {0, -.5}}};

void orc_twop_tables(double *cg5, double *bcg5, double *p13)
{
  memcpy(cg5, TP_CG5, sizeof(TP_CG5));
  memcpy(bcg5, TP_BCG5, sizeof(TP_BCG5));
  memcpy(p13, TP_P13, sizeof(TP_P13));
}

/* Proton two-point function of twop.c (twop.c:219-226 phases, :264-282
 * C g5 x bar C g5 entries, :324-399 block and Fourier sum): up and down
 * propagators D[v][mu][nu][c1][c2] (sink spin, source spin, sink colour,
 * source colour), source at xsrc (t, x, y, z), theta_t = pi. The
 * propagators are phased in place: time-slice (t + xsrc_t) % L_t times
 * exp(i pi t / L_t). corr[(t - t0) * nmom + j] (re, im) for t = t0..t1. */
void orc_twop_proton(double *up, double *dn, const int L[4], const int xsrc[4], int t0, int t1, const int *mom,
                     int nmom, double *corr)
{
  const size_t V = vol(L), V3 = V / (size_t)L[0];
  for (int t = 0; t < L[0]; t++) {
    const double ph = M_PI * t / L[0];
    const cx f = cmk(cos(ph), sin(ph));
    const int lt = (t + xsrc[0]) % L[0];
    for (size_t s = 0; s < V3; s++) {
      const size_t v = (size_t)lt + (size_t)L[0] * s;
      cx *pu = (cx *)(up + v * 288), *pd = (cx *)(dn + v * 288);
      for (int k = 0; k < 144; k++) {
        pu[k] = cmul(pu[k], f);
        pd[k] = cmul(pd[k], f);
      }
    }
  }
  cx *block = malloc(V3 * sizeof(cx));
  for (int t = t0; t <= t1; t++) {
    const int lt = (t + xsrc[0]) % L[0];
    for (size_t s = 0; s < V3; s++) block[s] = cmk(0, 0);
    for (int al = 0; al < 4; al++)
      for (int be = 0; be < 4; be++) {
        const cx P = cmk(TP_P13[al][be][0], TP_P13[al][be][1]);
        if (P.re * P.re + P.im * P.im <= 1e-8) continue;
        for (int mu = 0; mu < 4; mu++)
          for (int nu = 0; nu < 4; nu++)
            for (int ku = 0; ku < 4; ku++)
              for (int lu = 0; lu < 4; lu++) {
                const double C = TP_CG5[mu][nu] * TP_BCG5[ku][lu];
                if (fabs(C) <= 1e-3) continue;
                for (int e1 = 0; e1 < 6; e1++)
                  for (int e2 = 0; e2 < 6; e2++) {
                    const int c1 = TP_EPS[e1][0], c2 = TP_EPS[e1][1], c3 = TP_EPS[e1][2];
                    const int d1 = TP_EPS[e2][0], d2 = TP_EPS[e2][1], d3 = TP_EPS[e2][2];
                    const double sg = (double)(TP_SGN[e1] * TP_SGN[e2]);
                    for (size_t s = 0; s < V3; s++) {
                      const size_t v = (size_t)lt + (size_t)L[0] * s;
#define PR(p, a, b, c, d) (((const cx *)((p) + v * 288))[(((a) * 4 + (b)) * 3 + (c)) * 3 + (d)])
                      cx term = cmul(cmul(cmul(cmk(C, 0), PR(up, mu, ku, c1, d1)), PR(dn, nu, lu, c2, d2)),
                                     PR(up, be, al, c3, d3));
                      block[s] = csub(block[s], cmul(P, cscale(term, sg)));
                      term = cmul(cmul(cmul(cmk(C, 0), PR(up, mu, al, c1, d1)), PR(dn, nu, lu, c2, d2)),
                                  PR(up, be, ku, c3, d3));
                      block[s] = csub(block[s], cmul(P, cscale(term, sg)));
#undef PR
                    }
                  }
              }
      }
    for (int j = 0; j < nmom; j++) {
      cx c = cmk(0, 0);
      for (size_t s = 0; s < V3; s++) {
        /* spatial site s = x + Lx (y + Ly z) of the time-slice */
        const int x = (int)(s % (size_t)L[1]), y = (int)((s / (size_t)L[1]) % (size_t)L[2]),
                  z = (int)(s / ((size_t)L[1] * L[2]));
        const double a = 2 * M_PI * ((double)mom[3 * j] * (x - xsrc[1]) / L[1] +
                                     (double)mom[3 * j + 1] * (y - xsrc[2]) / L[2] +
                                     (double)mom[3 * j + 2] * (z - xsrc[3]) / L[3]);
        c = cadd(c, cmul(block[s], cmk(cos(a), -sin(a))));
      }
      corr[2 * ((size_t)(t - t0) * nmom + j)] = 0.5 * c.re;
      corr[2 * ((size_t)(t - t0) * nmom + j) + 1] = 0.5 * c.im;
    }
  }
  free(block);
}
