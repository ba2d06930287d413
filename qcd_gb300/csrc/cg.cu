// cg.cu -- conjugate gradient on the normal equations D^+ D x = D^+ b with
// device-resident scalars and reliable updates.
//
// One inner iteration is five launches and no host synchronisation:
//   1. t = D p            (operator kernel; its epilogue also sums |t|^2 =
//                          p^+ D^+ D p per block)
//   2. scalar kernel:     pAp = sum of the block partials, alpha = rr / pAp
//   3. Ap = D^+ t         (operator kernel)
//   4. update kernel:     x' += alpha p, r -= alpha Ap, per-block |r|^2
//   5. scalar kernel:     rr' = sum, beta = rr'/rr, history[i] = rr'
//   6. p = r + beta p     (reads beta from device memory)
// The host enqueues a chunk of iterations, then reads the residual history
// once and decides. Reliable updates (Sleijpen & van der Vorst, Computing 56
// (1996) 141; Clark et al., Comput. Phys. Commun. 181 (2010) 1517): when the
// iterated residual has fallen by delta since the last update, or looks
// converged, the low-precision increment x' is added to the FP64 solution and
// the true residual b - D x is recomputed with the FP64 operator; the search
// direction p is kept. Convergence is declared on that true residual only.
// Reductions sum block partials in a fixed order, so a solve is
// deterministic.
#include <math.h>

#include <vector>

#include "dslash_args.h"

namespace qg {

using namespace qgd;

bool dslash_partials(qcdgpu_field out, qcdgpu_field in, qcdgpu_gauge g, double mp4, double tm, bool dag,
                     int arith, double *partials);
double *big_partials(int64_t n);

// scalar slots
enum { S_RR = 0, S_PAP = 1, S_RRNEW = 2, S_ALPHA = 3, S_BETA = 4, S_HIST = 8 };
constexpr int kChunk = 16;

template <int P, typename R>
__global__ void __launch_bounds__(128) k_cg_update(void *xs, float *xsn, const void *ps, const float *psn, void *rs,
                                                   float *rsn, const void *aps, const float *apsn, int64_t stride,
                                                   int V, const double *s, double *partials)
{
  int x = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  double n2 = 0.0;
  if (x < V) {
    // FP16 iterations keep the solution increment in FP32: rounding every
    // increment to 11 bits would cost iterations
    constexpr int PX = P == QCDGPU_F16 ? QCDGPU_F32 : P;
    const R alpha = (R)s[S_ALPHA];
    C<R> vx[12], vp[12];
    Spinor<PX, R>::load(xs, xsn, stride, x, vx);
    Spinor<P, R>::load(ps, psn, stride, x, vp);
#pragma unroll
    for (int k = 0; k < 12; k++) {
      vx[k].re = qfma(alpha, vp[k].re, vx[k].re);
      vx[k].im = qfma(alpha, vp[k].im, vx[k].im);
    }
    Spinor<PX, R>::store(xs, xsn, stride, x, vx);
    Spinor<P, R>::load(rs, rsn, stride, x, vx);
    Spinor<P, R>::load(aps, apsn, stride, x, vp);
#pragma unroll
    for (int k = 0; k < 12; k++) {
      vx[k].re = qfma(-alpha, vp[k].re, vx[k].re);
      vx[k].im = qfma(-alpha, vp[k].im, vx[k].im);
      n2 += (double)vx[k].re * (double)vx[k].re + (double)vx[k].im * (double)vx[k].im;
    }
    Spinor<P, R>::store(rs, rsn, stride, x, vx);
  }
  block_partial(n2, partials);
}

template <int P, typename R>
__global__ void __launch_bounds__(128) k_cg_p(void *ps, float *psn, const void *rs, const float *rsn, int64_t stride,
                                              int V, const double *s)
{
  int x = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (x >= V) return;
  const R beta = (R)s[S_BETA];
  C<R> vp[12], vr[12];
  Spinor<P, R>::load(ps, psn, stride, x, vp);
  Spinor<P, R>::load(rs, rsn, stride, x, vr);
#pragma unroll
  for (int k = 0; k < 12; k++) {
    vp[k].re = qfma(beta, vp[k].re, vr[k].re);
    vp[k].im = qfma(beta, vp[k].im, vr[k].im);
  }
  Spinor<P, R>::store(ps, psn, stride, x, vp);
}

// per-block Re <a, b> (used for p^+ A p when the storage rounds D p: with
// FP16 fields A p = D^+ round(D p), and |D p|^2 would not match it)
template <int P, typename R>
__global__ void __launch_bounds__(128) k_dot_re(const void *a, const float *an, const void *b, const float *bn,
                                                int64_t stride, int V, double *partials)
{
  int x = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  double d = 0.0;
  if (x < V) {
    C<R> va[12], vb[12];
    Spinor<P, R>::load(a, an, stride, x, va);
    Spinor<P, R>::load(b, bn, stride, x, vb);
#pragma unroll
    for (int k = 0; k < 12; k++) d += (double)va[k].re * (double)vb[k].re + (double)va[k].im * (double)vb[k].im;
  }
  block_partial(d, partials);
}

// one block: sum n partials in a fixed order and update the scalars
__global__ void k_cg_scalars(const double *partials, int n, double *s, int mode, int hist)
{
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v += partials[i];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += sh[i];
    if (mode == 0) {
      s[S_PAP] = t;
      s[S_ALPHA] = t > 0.0 ? s[S_RR] / t : nan("");  // p^+ A p <= 0: breakdown
    } else {
      s[S_RRNEW] = t;
      s[S_BETA] = t / s[S_RR];
      s[S_RR] = t;
      s[S_HIST + hist] = t;
    }
  }
}

#define QG_PREC_DISPATCH(prec, KERNEL, ...)                                          \
  do {                                                                               \
    if ((prec) == QCDGPU_F64) KERNEL<QCDGPU_F64, double><<<nb, 128, 0, st>>>(__VA_ARGS__); \
    else if ((prec) == QCDGPU_F32) KERNEL<QCDGPU_F32, float><<<nb, 128, 0, st>>>(__VA_ARGS__); \
    else KERNEL<QCDGPU_F16, float><<<nb, 128, 0, st>>>(__VA_ARGS__);                 \
  } while (0)

// true residual rt = b - D x (FP64 operator), returns |rt| / |b|
static bool true_res(qcdgpu_field rt, qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double mp4, double tm,
                     double bn, double *rel)
{
  if (!dslash(rt, x, g, mp4, tm, QCDGPU_OP_D, -1)) return false;
  if (!blas_axpby(rt, 1.0, 0.0, b, -1.0, 0.0, rt)) return false;
  double n2;
  if (!blas_norm2(rt, &n2)) return false;
  *rel = bn > 0 ? sqrt(n2) / bn : 0.0;
  return true;
}

int solve_cgnr_engine(qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double mp4, double tm, qcdgpu_solve_params *p)
{
  struct Held {
    std::vector<qcdgpu_field> f;
    ~Held()
    {
      for (auto q : f) work_put(q);
    }
    qcdgpu_field get(const int L[4], int prec)
    {
      qcdgpu_field q = work_get(L, prec);
      if (q) f.push_back(q);
      return q;
    }
  } w;
  const int prec = p->inner_prec;
  qcdgpu_gauge gi = gauge_at(g, prec);
  qcdgpu_field rt = w.get(b->L, QCDGPU_F64), r = w.get(b->L, QCDGPU_F64), up = w.get(b->L, QCDGPU_F64);
  qcdgpu_field rs = w.get(b->L, prec), ps = w.get(b->L, prec);
  qcdgpu_field xs = w.get(b->L, prec == QCDGPU_F16 ? QCDGPU_F32 : prec);
  qcdgpu_field t = w.get(b->L, prec), aps = w.get(b->L, prec);
  if (!gi || !rt || !r || !up || !rs || !xs || !ps || !t || !aps) return 3;
  const int V = (int)b->V;
  const unsigned nb = (unsigned)((V + 127) / 128);
  double *part = big_partials(nb);
  double *s = reduce_scratch();
  double *h = host_result();
  if (!part || !s || !h) return 3;
  s += 2 * kMaxPartials + 16;  // 16 + kChunk slots past the blas result words
  cudaStream_t st = stream();

  double bn2;
  if (!blas_norm2(b, &bn2)) return 3;
  double bn = sqrt(bn2);
  p->iters = 0;
  p->reliable_updates = 0;
  p->true_residual = 1.0;
  if (!blas_zero(x)) return 3;
  if (bn == 0.0) {
    p->true_residual = 0.0;
    return 0;
  }
  // the system matrix is D (op D) or Q = i g5 D (op Q): Q^+ Q = D^+ D and
  // Q x = b <=> D x = -i g5 b, so both run the D^+ D iteration
  qcdgpu_field bd = b;
  if (p->op == QCDGPU_OP_Q) {
    bd = w.get(b->L, QCDGPU_F64);
    if (!bd || !blas_ig5(bd, b) || !blas_axpby(bd, -1.0, 0.0, bd, 0.0, 0.0, bd)) return 3;
  }
  if (!blas_copy(rt, bd)) return 3;
  auto restart_residual = [&](double *rr_out) -> bool {
    // r = D^+ rt, rs = r (storage precision), s[RR] = |r|^2
    if (!dslash(r, rt, g, mp4, tm, QCDGPU_OP_DDAG, -1)) return false;
    double rr;
    if (!blas_norm2(r, &rr)) return false;
    if (!convert_field(rs, r)) return false;
    if (!QG_CUDA(cudaMemcpyAsync(s + S_RR, &rr, sizeof(double), cudaMemcpyHostToDevice, st))) return false;
    *rr_out = rr;
    return true;
  };
  double rr;
  if (!restart_residual(&rr)) return 3;
  if (!blas_copy(ps, rs) || !blas_zero(xs)) return 3;
  // the scalar upload above reads host memory asynchronously: wait for it
  if (!QG_CUDA(cudaStreamSynchronize(st))) return 3;
  double maxr = sqrt(rr), hint = p->tol * maxr;
  bool first = true;
  const double delta = p->delta > 0 ? p->delta : 0.1;
  const int arith = -1;
  int since_update = 0;
  while (true) {
    int chunk = kChunk;
    if (p->maxiter - p->iters < chunk) chunk = p->maxiter - p->iters;
    for (int j = 0; j < chunk; j++) {
      // p = r + beta p opens each iteration (not the first), so a reliable
      // update between chunks enters the next direction through beta
      if (!first) {
        QG_PREC_DISPATCH(prec, k_cg_p, ps->data, ps->norm, rs->data, rs->norm, ps->stride, V, s);
        if (!QG_LAUNCHED("cg_p")) return 3;
      }
      first = false;
      if (prec != QCDGPU_F16) {
        // p^+ A p = |D p|^2 summed in the epilogue of the first operator
        if (!dslash_partials(t, ps, gi, mp4, tm, false, arith, part)) return 3;
        k_cg_scalars<<<1, 256, 0, st>>>(part, (int)nb, s, 0, j);
        if (!QG_LAUNCHED("cg_scalars")) return 3;
        if (!dslash_partials(aps, t, gi, mp4, tm, true, arith, nullptr)) return 3;
      } else {
        if (!dslash_partials(t, ps, gi, mp4, tm, false, arith, nullptr)) return 3;
        if (!dslash_partials(aps, t, gi, mp4, tm, true, arith, nullptr)) return 3;
        k_dot_re<QCDGPU_F16, float><<<nb, 128, 0, st>>>(ps->data, ps->norm, aps->data, aps->norm, ps->stride, V, part);
        if (!QG_LAUNCHED("cg_dot")) return 3;
        k_cg_scalars<<<1, 256, 0, st>>>(part, (int)nb, s, 0, j);
        if (!QG_LAUNCHED("cg_scalars")) return 3;
      }
      QG_PREC_DISPATCH(prec, k_cg_update, xs->data, xs->norm, ps->data, ps->norm, rs->data, rs->norm, aps->data,
                       aps->norm, xs->stride, V, s, part);
      if (!QG_LAUNCHED("cg_update")) return 3;
      k_cg_scalars<<<1, 256, 0, st>>>(part, (int)nb, s, 1, j);
      if (!QG_LAUNCHED("cg_scalars")) return 3;
    }
    // history, and rr / beta of the last iteration (slots 0..S_HIST+kChunk)
    if (!QG_CUDA(cudaMemcpyAsync(h, s, sizeof(double) * (S_HIST + chunk), cudaMemcpyDeviceToHost, st)) ||
        !QG_CUDA(cudaStreamSynchronize(st)))
      return 3;
    const double rr_iter = h[S_RR], beta_iter = h[S_BETA];
    const double *hist = h + S_HIST;
    bool update = false, hinted = false;
    double rn = 0;
    for (int j = 0; j < chunk; j++) {
      rn = sqrt(hist[j]);
      if (!(rn == rn)) return 2;  // NaN: p^+ A p <= 0 or overflow
      p->iters++;
      since_update++;
      if (rn <= hint) hinted = true;
      if (prec != QCDGPU_F64 ? rn < delta * maxr : since_update >= 2 * kChunk) update = true;
      if (!update && rn > maxr) maxr = rn;
    }
    bool last = p->iters >= p->maxiter;
    if (update || hinted || last) {
      if (prec == QCDGPU_F64) {
        if (!blas_axpby(x, 1.0, 0.0, xs, 1.0, 0.0, x)) return 3;
      } else {
        if (!convert_field(up, xs) || !blas_axpby(x, 1.0, 0.0, up, 1.0, 0.0, x)) return 3;
      }
      if (!blas_zero(xs)) return 3;
      double rel;
      if (!true_res(rt, x, bd, g, mp4, tm, bn, &rel)) return 3;
      p->true_residual = rel;
      p->reliable_updates++;
      since_update = 0;
      if (rel <= p->tol) return 0;
      if (last) return 1;
      if (hinted) hint = rn * 0.3;
      if (!restart_residual(&rr)) return 3;
      // the next direction p = r_true + beta' p with beta' = |r_true|^2 / |r_prev|^2,
      // where |r_prev|^2 = rr_iter / beta_iter is the residual before the last iteration
      double beta_new = (beta_iter > 0.0 && rr_iter > 0.0) ? rr * beta_iter / rr_iter : 0.0;
      h[0] = beta_new;
      if (!QG_CUDA(cudaMemcpyAsync(s + S_BETA, h, sizeof(double), cudaMemcpyHostToDevice, st))) return 3;
      if (!QG_CUDA(cudaStreamSynchronize(st))) return 3;
      maxr = sqrt(rr);
    }
  }
}

}  // namespace qg
