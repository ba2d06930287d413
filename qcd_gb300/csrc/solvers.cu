// solvers.cu -- Krylov solvers on device fields.
//
//  * gcr_dropin: n-step GCR with modified Gram-Schmidt on Q = i g5 D, the
//    algorithm of gcr() in invert.c:20-113 (with the first basis term of the
//    solution update that gcr.m has and the shipped invert.c omits; the
//    shipped variant is kept behind a flag).
//  * solve(): restarted GCR with refinement (invert.c:255-294), BiCGstab
//    (van der Vorst 1992) and CG on the normal equations (Hestenes-Stiefel
//    1952), each to a true relative residual |b - A x|/|b| computed in FP64.
//    Mixed precision:
//      - CGNR uses reliable updates (Sleijpen & van der Vorst, Computing 56
//        (1996) 141; as used for lattice QCD by Clark et al., Comput. Phys.
//        Commun. 181 (2010) 1517): the inner iteration runs in FP32 or FP16
//        storage; whenever the iterated residual has fallen by `delta` since
//        the last update, the solution is accumulated in FP64 and the true
//        residual is recomputed with the FP64 operator.
//      - BiCGstab uses defect correction: inner FP32/FP16 BiCGstab solves of
//        A e = r to relative accuracy `delta`, x += e and r = b - A x in FP64.
//    Scalars of the inner iteration live on the host; each reduction is one
//    synchronisation.
#include <math.h>
#include <string.h>

#include <complex>
#include <map>
#include <vector>

#include "internal.h"

namespace qg {

using cplx = std::complex<double>;

int g_gcr_shipped = 0;

// ------------------------------------------------------------- helpers
struct Work {
  std::vector<qcdgpu_field> fs;
  ~Work()
  {
    for (auto f : fs) work_put(f);
  }
  qcdgpu_field get(const int L[4], int prec)
  {
    qcdgpu_field f = work_get(L, prec);
    if (f) fs.push_back(f);
    return f;
  }
};

static bool norm(qcdgpu_field x, double *n)
{
  double n2;
  if (!blas_norm2(x, &n2)) return false;
  *n = sqrt(n2);
  return true;
}
static bool dot(qcdgpu_field a, qcdgpu_field b, cplx *d)
{
  double r[2];
  if (!blas_dot(a, b, r)) return false;
  *d = cplx(r[0], r[1]);
  return true;
}
// out = a x + y
static bool caxpy(qcdgpu_field out, cplx a, qcdgpu_field x, qcdgpu_field y)
{
  return blas_axpby(out, a.real(), a.imag(), x, 1.0, 0.0, y);
}
static bool scale(qcdgpu_field x, double s) { return blas_axpby(x, s, 0.0, x, 0.0, 0.0, x); }

// low-precision copies of gauge fields, keyed by the FP64 field
struct LowKey {
  qcdgpu_gauge g;
  int prec;
  bool operator<(const LowKey &o) const { return g < o.g || (g == o.g && prec < o.prec); }
};
static std::map<LowKey, qcdgpu_gauge> g_low;

qcdgpu_gauge gauge_at(qcdgpu_gauge g, int prec)
{
  if (g->prec == prec) return g;
  auto it = g_low.find({g, prec});
  if (it != g_low.end()) return it->second;
  const bool full32 = prec == kGaugeF32Full;
  qcdgpu_gauge lo = gauge_new(g->L, g->theta, full32 ? QCDGPU_F32 : prec, 18);
  if (!lo) return nullptr;
  // the full FP32 copy serves the multi-RHS kernels only; it carries the
  // boundary phases in its links
  if (!convert_gauge(lo, g, full32 ? 18 : 0) || (full32 && !gauge_fold_phases(lo))) {
    gauge_free(lo);
    return nullptr;
  }
  g_low[{g, prec}] = lo;
  return lo;
}

void gauge_forget(qcdgpu_gauge g)
{
  for (auto it = g_low.begin(); it != g_low.end();) {
    if (it->first.g == g) {
      gauge_free(it->second);
      it = g_low.erase(it);
    } else {
      ++it;
    }
  }
}

// ---------------------------------------------------------------- GCR
int gcr_dropin(qcdgpu_field sol, qcdgpu_field src, qcdgpu_gauge g, double mp4, double tm, int n, int shipped)
{
  if (n < 1) {
    set_error("gcr: n must be >= 1");
    return 1;
  }
  Work w;
  std::vector<qcdgpu_field> chi((size_t)n), res((size_t)n);
  for (int i = 0; i < n; i++) {
    chi[(size_t)i] = w.get(src->L, QCDGPU_F64);
    res[(size_t)i] = w.get(src->L, QCDGPU_F64);
    if (!chi[(size_t)i] || !res[(size_t)i]) {
      set_error("gcr: not enough device memory");
      return 1;
    }
  }
  std::vector<cplx> a((size_t)n * n), c((size_t)n);
  auto A = [&](int i, int j) -> cplx & { return a[(size_t)i * n + j]; };
  double nv;
  if (!blas_copy(res[0], src)) return 1;
  if (!dslash(chi[0], res[0], g, mp4, tm, QCDGPU_OP_Q, -1)) return 1;
  if (!norm(chi[0], &nv)) return 1;
  A(0, 0) = 1.0 / nv;
  if (!scale(chi[0], A(0, 0).real())) return 1;
  if (!dot(chi[0], src, &c[0])) return 1;
  if (!blas_zero(sol)) return 1;
  if (!shipped && !caxpy(sol, c[0] * A(0, 0), res[0], sol)) return 1;
  for (int k = 1; k < n; k++) {
    if (!caxpy(res[(size_t)k], -c[(size_t)k - 1], chi[(size_t)k - 1], res[(size_t)k - 1])) return 1;
    if (!dslash(chi[(size_t)k], res[(size_t)k], g, mp4, tm, QCDGPU_OP_Q, -1)) return 1;
    // Gram-Schmidt against the orthonormal chi_0 .. chi_{k-1}: the k
    // projections in one pass, then one batched update (classical form; for
    // an orthonormal basis its coefficients are modified Gram-Schmidt's,
    // invert.c:68-79)
    {
      std::vector<cplx> t((size_t)k);
      if (!blas_multi_dot(chi.data(), k, chi[(size_t)k], t.data())) return 1;
      for (int j = 0; j < k; j++) A(k, j) = -t[(size_t)j];
      if (!blas_multi_axpy(chi[(size_t)k], chi.data(), &A(k, 0), k)) return 1;
    }
    if (!norm(chi[(size_t)k], &nv)) return 1;
    A(k, k) = 1.0 / nv;
    if (std::isnan(A(k, k).real())) {
      set_error("gcr: Krylov space is sick (NaN norm)");
      return 1;
    }
    if (!scale(chi[(size_t)k], A(k, k).real())) return 1;
    for (int j = 0; j < k; j++) A(k, j) *= A(k, k).real();
    for (int j = 0; j < k; j++) {
      A(k, j) *= A(j, j).real();
      for (int l = j + 1; l < k; l++) A(k, j) += A(k, l) * A(l, j);
    }
    if (!dot(chi[(size_t)k], src, &c[(size_t)k])) return 1;
    {
      std::vector<cplx> coef((size_t)k + 1);
      for (int j = 0; j <= k; j++) coef[(size_t)j] = c[(size_t)k] * A(k, j);
      if (!blas_multi_axpy(sol, res.data(), coef.data(), k + 1)) return 1;
    }
  }
  return 0;
}

// ------------------------------------------------------- true residual
// r = b - A x in FP64; returns |r| / |b| via *rel
static bool true_residual(qcdgpu_field r, qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double mp4,
                          double tm, int op, double bnorm, double *rel)
{
  if (!dslash(r, x, g, mp4, tm, op, -1)) return false;
  if (!blas_axpby(r, 1.0, 0.0, b, -1.0, 0.0, r)) return false;
  double rn;
  if (!norm(r, &rn)) return false;
  *rel = bnorm > 0 ? rn / bnorm : 0.0;
  return true;
}

// ---------------------------------------------------------- BiCGstab
// Inner BiCGstab on A x = b in precision of (x, b), x0 = 0, stopping on the
// iterated residual <= tol |b|. Returns iterations, -1 on breakdown.
static int bicgstab_core(qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double mp4, double tm, int op,
                         double tol, int maxiter, bool *err)
{
  Work w;
  int prec = b->prec;
  qcdgpu_field r = w.get(b->L, prec), rh = w.get(b->L, prec), p = w.get(b->L, prec),
               v = w.get(b->L, prec), s = w.get(b->L, prec), t = w.get(b->L, prec);
  *err = true;
  if (!r || !rh || !p || !v || !s || !t) return -1;
  double bn;
  if (!norm(b, &bn)) return -1;
  if (!blas_zero(x) || !blas_copy(r, b) || !blas_zero(p) || !blas_zero(v)) return -1;
  // shadow residual: a fixed Z4 vector (a point source as shadow makes
  // <rh, r> vanish exactly because (1 - g_mu)(1 + g_mu) = 0)
  if (!field_z4(rh, 0x5EEDull)) return -1;
  *err = false;
  if (bn == 0.0) return 0;
  cplx rho = 1.0, alpha = 1.0, omega = 1.0;
  for (int it = 1; it <= maxiter; it++) {
    cplx rho1;
    if (!dot(rh, r, &rho1)) { *err = true; return -1; }
    if (std::abs(rho1) == 0.0) return -1;
    cplx beta = (rho1 / rho) * (alpha / omega);
    // p = r + beta (p - omega v)
    if (!blas_axpby(p, 1.0, 0.0, p, -omega.real(), -omega.imag(), v)) { *err = true; return -1; }
    if (!blas_axpby(p, 1.0, 0.0, r, beta.real(), beta.imag(), p)) { *err = true; return -1; }
    if (!dslash(v, p, g, mp4, tm, op, -1)) { *err = true; return -1; }
    cplx rv;
    if (!dot(rh, v, &rv)) { *err = true; return -1; }
    if (std::abs(rv) == 0.0) return -1;
    alpha = rho1 / rv;
    if (!caxpy(s, -alpha, v, r)) { *err = true; return -1; }
    double sn;
    if (!norm(s, &sn)) { *err = true; return -1; }
    if (sn <= tol * bn) {
      if (!caxpy(x, alpha, p, x)) { *err = true; return -1; }
      return it;
    }
    if (!dslash(t, s, g, mp4, tm, op, -1)) { *err = true; return -1; }
    cplx ts;
    double tn;
    if (!dot(t, s, &ts) || !norm(t, &tn)) { *err = true; return -1; }
    if (tn == 0.0) return -1;
    omega = ts / (tn * tn);
    if (std::abs(omega) == 0.0) return -1;
    if (!caxpy(x, alpha, p, x) || !caxpy(x, omega, s, x) || !caxpy(r, -omega, t, s)) { *err = true; return -1; }
    double rn;
    if (!norm(r, &rn)) { *err = true; return -1; }
    rho = rho1;
    if (rn <= tol * bn) return it;
  }
  return maxiter;
}

static int solve_bicgstab(qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double mp4, double tm,
                          qcdgpu_solve_params *p)
{
  Work w;
  qcdgpu_field r = w.get(b->L, QCDGPU_F64);
  if (!r) return 3;
  double bn;
  if (!norm(b, &bn)) return 3;
  int prec = p->inner_prec;
  qcdgpu_gauge gi = gauge_at(g, prec);
  qcdgpu_field ri = prec == QCDGPU_F64 ? nullptr : w.get(b->L, prec);
  qcdgpu_field ei = w.get(b->L, prec);
  if (!gi || !ei || (prec != QCDGPU_F64 && !ri)) return 3;
  if (!blas_zero(x)) return 3;
  double rel = 1.0;
  if (!blas_copy(r, b)) return 3;
  p->iters = 0;
  p->reliable_updates = 0;
  double inner_tol = prec == QCDGPU_F64 ? p->tol : (p->delta > 0 ? p->delta : 0.1);
  int stall = 0;
  double last = 1.0;
  while (p->iters < p->maxiter) {
    bool err;
    int it;
    double rn;
    if (!norm(r, &rn)) return 3;
    // inner solve A e = r to relative accuracy inner_tol (relative to |r|),
    // but never further than the outer target requires
    double want = p->tol * bn / (rn > 0 ? rn : 1.0);
    double itol = inner_tol > want ? inner_tol : want * 0.5;
    if (prec == QCDGPU_F64) {
      it = bicgstab_core(ei, r, gi, mp4, tm, p->op, itol, p->maxiter - p->iters, &err);
    } else {
      if (!convert_field(ri, r)) return 3;
      it = bicgstab_core(ei, ri, gi, mp4, tm, p->op, itol, p->maxiter - p->iters, &err);
    }
    if (err) return 3;
    if (it < 0) return 2;
    p->iters += it;
    // x += e in FP64
    if (prec == QCDGPU_F64) {
      if (!caxpy(x, 1.0, ei, x)) return 3;
    } else {
      if (!convert_field(r, ei)) return 3;
      if (!caxpy(x, 1.0, r, x)) return 3;
    }
    p->reliable_updates++;
    if (!true_residual(r, x, b, g, mp4, tm, p->op, bn, &rel)) return 3;
    p->true_residual = rel;
    if (rel <= p->tol) return 0;
    if (rel > 0.9 * last) {
      if (++stall >= 3) return 1;
    } else {
      stall = 0;
    }
    last = rel;
    if (it == 0) return 1;
  }
  return 1;
}

// CGNR with device-resident scalars: cg.cu
int solve_cgnr_eo(qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double mp4, double tm, qcdgpu_solve_params *p);
int solve_bicgstabl_eo(qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double mp4, double tm,
                       qcdgpu_solve_params *p);
int solve_cgnr_engine(qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double mp4, double tm,
                      qcdgpu_solve_params *p);

// -------------------------------------------------- GCR with refinement
static int solve_gcr(qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double mp4, double tm,
                     qcdgpu_solve_params *p)
{
  if (p->op != QCDGPU_OP_Q) {
    set_error("GCR solves Q = i g5 D (op Q) as invert.c does");
    return 3;
  }
  Work w;
  qcdgpu_field r = w.get(b->L, QCDGPU_F64), c = w.get(b->L, QCDGPU_F64);
  if (!r || !c) return 3;
  double bn;
  if (!norm(b, &bn)) return 3;
  int n = p->restart > 0 ? p->restart : 32;
  if (gcr_dropin(x, b, g, mp4, tm, n, g_gcr_shipped)) return 2;
  p->iters = n;
  double rel;
  if (!true_residual(r, x, b, g, mp4, tm, QCDGPU_OP_Q, bn, &rel)) return 3;
  p->true_residual = rel;
  p->reliable_updates = 1;
  while (rel > p->tol && p->iters < p->maxiter) {
    if (gcr_dropin(c, r, g, mp4, tm, n, g_gcr_shipped)) return 2;
    if (!caxpy(x, 1.0, c, x)) return 3;
    p->iters += n;
    if (!true_residual(r, x, b, g, mp4, tm, QCDGPU_OP_Q, bn, &rel)) return 3;
    p->true_residual = rel;
    p->reliable_updates++;
  }
  return rel <= p->tol ? 0 : 1;
}

int solve(qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double mp4, double tm, qcdgpu_solve_params *p)
{
  if (!same_shape(x, b) || x->prec != QCDGPU_F64 || b->prec != QCDGPU_F64 || g->prec != QCDGPU_F64 ||
      x->V != g->V) {
    set_error("solve: x, b and the gauge field must be FP64 and of one lattice");
    return 3;
  }
  if (x == b) {
    set_error("solve: x and b must differ");
    return 3;
  }
  if (p->op != QCDGPU_OP_D && p->op != QCDGPU_OP_Q) {
    set_error("solve: op must be D or Q");
    return 3;
  }
  if (p->inner_prec < QCDGPU_F64 || p->inner_prec > QCDGPU_F16) {
    set_error("solve: unknown inner precision");
    return 3;
  }
  if (p->maxiter <= 0) p->maxiter = 100000;
  p->true_residual = -1.0;
  int st;
  switch (p->solver) {
  case QCDGPU_SOLVER_GCR: st = solve_gcr(x, b, g, mp4, tm, p); break;
  case QCDGPU_SOLVER_BICGSTAB: st = solve_bicgstab(x, b, g, mp4, tm, p); break;
  case QCDGPU_SOLVER_CGNR: st = solve_cgnr_engine(x, b, g, mp4, tm, p); break;
  case QCDGPU_SOLVER_CGNR_EO: st = solve_cgnr_eo(x, b, g, mp4, tm, p); break;
  case QCDGPU_SOLVER_BICGSTABL_EO: st = solve_bicgstabl_eo(x, b, g, mp4, tm, p); break;
  default: set_error("solve: unknown solver %d", p->solver); st = 3;
  }
  p->status = st;
  return st;
}

}  // namespace qg

extern "C" {

int qcdgpu_solve(qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double kappa, double mu, qcdgpu_solve_params *p)
{
  if (!x || !b || !g || !p || !(kappa > 0.0)) {
    qg::set_error("solve: bad arguments");
    if (p) p->status = 3;
    return 3;
  }
  return qg::solve(x, b, g, 1.0 / (2.0 * kappa), mu, p);
}

void qcdgpu_set_gcr_compat(int shipped) { qg::g_gcr_shipped = shipped ? 1 : 0; }

}  // extern "C"
