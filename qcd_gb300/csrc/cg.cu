// cg.cu -- conjugate gradient on the normal equations D^+ D x = D^+ b with
// device-resident scalars and reliable updates.
//
// The iteration is written once (cgnr_core) for any system operator A given
// as kernels: A = D on the full lattice, or the even/odd Schur complement
// (solve_cgnr_eo). One inner iteration is four operations (five launches
// for the even/odd operator, whose A is two hops) and no host
// synchronisation:
//   1. t = A p            (operator kernel; its epilogue also sums |t|^2 =
//                          p^+ A^+ A p per block, and the block that
//                          finishes last forms alpha = rr / pAp)
//   2. Ap = A^+ t         (operator kernel)
//   3. update kernel:     x' += alpha p, r -= alpha Ap, per-block |r|^2; its
//                          last block forms rr', beta = rr'/rr, history[i]
//   4. p = r + beta p     (reads beta from device memory)
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
#include <string.h>

#include <complex>
#include <functional>
#include <vector>

#include "dslash_args.h"

namespace qg {

using namespace qgd;

bool dslash_partials(qcdgpu_field out, qcdgpu_field in, qcdgpu_gauge g, double mp4, double tm, bool dag,
                     int arith, double *partials, const CgFuse *fuse = nullptr);
double *big_partials(int64_t n);

constexpr int kChunk = 16;

// The two fused reductions run kCgSpt sites per thread in blocks of
// kCgThreads: fewer blocks, so the last block sums fewer partials.
constexpr int kCgThreads = 256, kCgSpt = 2, kCgSites = kCgThreads * kCgSpt;

template <int P, typename R>
__global__ void __launch_bounds__(kCgThreads) k_cg_update(void *xs, float *xsn, const void *ps, const float *psn,
                                                          void *rs, float *rsn, const void *aps, const float *apsn,
                                                          int64_t stride, int V, double *s, double *partials,
                                                          unsigned *done, int hist)
{
  double n2 = 0.0;
#pragma unroll
  for (int i = 0; i < kCgSpt; i++) {
  const int x = (int)(blockIdx.x * kCgSites + i * kCgThreads + threadIdx.x);
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
    R s2 = (R)0;  // per-site sum in the working precision, block sum in double
#pragma unroll
    for (int k = 0; k < 12; k++) {
      vx[k].re = qfma(-alpha, vp[k].re, vx[k].re);
      vx[k].im = qfma(-alpha, vp[k].im, vx[k].im);
      s2 = s2 + vx[k].re * vx[k].re + vx[k].im * vx[k].im;
    }
    n2 += (double)s2;
    Spinor<P, R>::store(rs, rsn, stride, x, vx);
  }
  }
  block_partial(n2, partials);
  cg_last_block(partials, done, s, 1, hist);
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

#define QG_PREC_DISPATCH(prec, KERNEL, ...)                                          \
  do {                                                                               \
    if ((prec) == QCDGPU_F64) KERNEL<QCDGPU_F64, double><<<nb, 128, 0, st>>>(__VA_ARGS__); \
    else if ((prec) == QCDGPU_F32) KERNEL<QCDGPU_F32, float><<<nb, 128, 0, st>>>(__VA_ARGS__); \
    else KERNEL<QCDGPU_F16, float><<<nb, 128, 0, st>>>(__VA_ARGS__);                 \
  } while (0)


// Operators of the system A y = c that cgnr_core solves through A^+ A.
struct CgOps {
  int L[4];  // lattice of the system's fields (the half lattice for even/odd)
  // inner precision: t = A p (with partials: |t|^2 per 128-site block, and
  // with fuse the CG step from them), aps = A^+ t
  std::function<bool(qcdgpu_field, qcdgpu_field, double *, const CgFuse *)> op;
  std::function<bool(qcdgpu_field, qcdgpu_field)> opdag;
  // FP64 storage (accurate arithmetic): out = A in, out = A^+ in
  std::function<bool(qcdgpu_field, qcdgpu_field)> op64, opdag64;
  // optional: rs = A^+ rt in the inner precision with |rs|^2 (instead of
  // opdag64 + conversion): the true residual rt is FP64-accurate, and its
  // image only seeds the low-precision iteration
  std::function<bool(qcdgpu_field, qcdgpu_field, double *)> restart;
};

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
};

// A chunk of solver iterations recorded once and replayed. Recording runs
// on a library-owned stream (the caller's stream may be the legacy default
// stream, which cannot be captured); the replay goes to the caller's stream.
// If recording fails the solver keeps launching the chunk directly.
struct ChunkGraph {
  cudaGraphExec_t exec = nullptr;
  uint64_t launches = 0;
  bool usable = true;
  ~ChunkGraph()
  {
    if (exec) cudaGraphExecDestroy(exec);
  }
  template <typename F>
  bool run(cudaStream_t st, F &&enqueue)
  {
    if (!exec) {
      static cudaStream_t cs = nullptr;
      if (!cs && cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) cs = nullptr;
      if (!cs) {
        usable = false;
        cudaGetLastError();
        return enqueue();
      }
      cudaGraph_t graph = nullptr;
      const uint64_t counted = g_launches.load();
      bool ok = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      if (ok) {
        const cudaStream_t prev = swap_stream(cs);
        ok = enqueue();
        swap_stream(prev);
        ok = cudaStreamEndCapture(cs, &graph) == cudaSuccess && ok;
      }
      launches = g_launches.load() - counted;
      g_launches.store(counted);  // recorded, not launched
      ok = ok && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
      if (graph) cudaGraphDestroy(graph);
      if (!ok) {
        exec = nullptr;
        usable = false;
        cudaGetLastError();
        return enqueue();
      }
    }
    if (!QG_CUDA(cudaGraphLaunch(exec, st))) return false;
    count_launches(launches);
    return true;
  }
};

// CG on A^+ A y = A^+ c, x0 = 0, chunked with reliable updates; convergence
// on the true residual |c - A y| / cn (cn: the norm the residual is relative
// to). Returns 0 converged, 1 maxiter, 2 breakdown, 3 CUDA error.
static int cgnr_core(qcdgpu_field y, qcdgpu_field c, double cn, const CgOps &ops, qcdgpu_solve_params *p)
{
  Held w;
  const int prec = p->inner_prec;
  qcdgpu_field rt = w.get(ops.L, QCDGPU_F64), r = w.get(ops.L, QCDGPU_F64), up = w.get(ops.L, QCDGPU_F64);
  qcdgpu_field rs = w.get(ops.L, prec), ps = w.get(ops.L, prec);
  qcdgpu_field xs = w.get(ops.L, prec == QCDGPU_F16 ? QCDGPU_F32 : prec);
  qcdgpu_field t = w.get(ops.L, prec), aps = w.get(ops.L, prec);
  if (!rt || !r || !up || !rs || !xs || !ps || !t || !aps) return 3;
  const int V = (int)rt->V;
  const unsigned nb = (unsigned)((V + 127) / 128);            // operator launches: 128 sites per block
  const unsigned nbr = (unsigned)((V + kCgSites - 1) / kCgSites);  // the fused reductions
  double *part = big_partials(nb);
  double *s = reduce_scratch();
  double *h = host_result();
  if (!part || !s || !h) return 3;
  s += 2 * kMaxPartials + 16;  // 16 + kChunk slots past the blas result words
  unsigned *done = (unsigned *)(s + S_HIST + kChunk);  // block counters of the fused reductions
  cudaStream_t st = stream();
  if (!QG_CUDA(cudaMemsetAsync(done, 0, 2 * sizeof(unsigned), st))) return 3;
  if (!blas_zero(y)) return 3;
  // true residual rt = c - A y (FP64), returns |rt| / cn
  auto true_res = [&](double *rel) -> bool {
    if (!ops.op64(rt, y) || !blas_axpby(rt, 1.0, 0.0, c, -1.0, 0.0, rt)) return false;
    double n2;
    if (!blas_norm2(rt, &n2)) return false;
    *rel = sqrt(n2) / cn;
    return true;
  };
  // r = A^+ rt, rs = r (storage precision), s[RR] = |r|^2
  auto restart_residual = [&](double *rr_out) -> bool {
    double rr;
    if (ops.restart) {
      if (!ops.restart(rs, rt, &rr)) return false;
    } else if (!ops.opdag64(r, rt) || !blas_norm2(r, &rr) || !convert_field(rs, r)) {
      return false;
    }
    h[0] = rr;
    if (!QG_CUDA(cudaMemcpyAsync(s + S_RR, h, sizeof(double), cudaMemcpyHostToDevice, st))) return false;
    if (!QG_CUDA(cudaStreamSynchronize(st))) return false;
    *rr_out = rr;
    return true;
  };
  if (!blas_copy(rt, c)) return 3;
  double rr;
  if (!restart_residual(&rr)) return 3;
  if (!blas_copy(ps, rs) || !blas_zero(xs)) return 3;
  double maxr = sqrt(rr), hint = p->tol * maxr;
  bool first = true;
  const double delta = p->delta > 0 ? p->delta : 0.1;
  int since_update = 0;
  // one chunk of iterations; every chunk after the first launches the same
  // kernels with the same arguments, so it is captured once as a CUDA graph
  // and replayed (the captured launches are counted at each replay)
  auto enqueue_chunk = [&](int chunk) -> bool {
    const cudaStream_t st = stream();  // the capture stream while a graph is recorded
    for (int j = 0; j < chunk; j++) {
      // p = r + beta p opens each iteration (not the first), so a reliable
      // update between chunks enters the next direction through beta
      if (!first) {
        QG_PREC_DISPATCH(prec, k_cg_p, ps->data, ps->norm, rs->data, rs->norm, ps->stride, V, s);
        if (!QG_LAUNCHED("cg_p")) return false;
      }
      first = false;
      // p^+ A^+ A p = |A p|^2, summed in the epilogue of the first operator;
      // its last block forms alpha
      const CgFuse fz{done, s, j};
      if (!ops.op(t, ps, part, &fz) || !ops.opdag(aps, t)) return false;
#define QG_CG_UPD(P, R)                                                                                           \
  k_cg_update<P, R><<<nbr, kCgThreads, 0, st>>>(xs->data, xs->norm, ps->data, ps->norm, rs->data, rs->norm, aps->data, \
                                                aps->norm, xs->stride, V, s, part, done + 1, j)
      // x += alpha p, r -= alpha A p, with |r|^2 and beta
      if (prec == QCDGPU_F64) QG_CG_UPD(QCDGPU_F64, double);
      else if (prec == QCDGPU_F32) QG_CG_UPD(QCDGPU_F32, float);
      else QG_CG_UPD(QCDGPU_F16, float);
#undef QG_CG_UPD
      if (!QG_LAUNCHED("cg_update")) return false;
    }
    return true;
  };
  ChunkGraph graph;
  while (true) {
    int chunk = kChunk;
    if (p->maxiter - p->iters < chunk) chunk = p->maxiter - p->iters;
    if (!first && chunk == kChunk && graph.usable) {
      if (!graph.run(st, [&] { return enqueue_chunk(chunk); })) return 3;
    } else {
      if (!enqueue_chunk(chunk)) return 3;
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
        if (!blas_axpby(y, 1.0, 0.0, xs, 1.0, 0.0, y)) return 3;
      } else {
        if (!convert_field(up, xs) || !blas_axpby(y, 1.0, 0.0, up, 1.0, 0.0, y)) return 3;
      }
      if (!blas_zero(xs)) return 3;
      double rel;
      if (!true_res(&rel)) return 3;
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

// b as seen by D: Q x = b <=> D x = -i g5 b (Q^+ Q = D^+ D)
static qcdgpu_field system_rhs(Held &w, qcdgpu_field b, int op)
{
  if (op != QCDGPU_OP_Q) return b;
  qcdgpu_field bd = w.get(b->L, QCDGPU_F64);
  if (!bd || !blas_ig5(bd, b) || !blas_axpby(bd, -1.0, 0.0, bd, 0.0, 0.0, bd)) return nullptr;
  return bd;
}

int solve_cgnr_engine(qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double mp4, double tm, qcdgpu_solve_params *p)
{
  Held w;
  p->iters = 0;
  p->reliable_updates = 0;
  p->true_residual = 1.0;
  double bn2;
  if (!blas_norm2(b, &bn2)) return 3;
  if (bn2 == 0.0) {
    p->true_residual = 0.0;
    return blas_zero(x) ? 0 : 3;
  }
  qcdgpu_field bd = system_rhs(w, b, p->op);
  qcdgpu_gauge gi = gauge_at(g, p->inner_prec);
  if (!bd || !gi) return 3;
  CgOps ops;
  memcpy(ops.L, b->L, sizeof(ops.L));
  ops.op = [&](qcdgpu_field o, qcdgpu_field i, double *part, const CgFuse *fuse) {
    return dslash_partials(o, i, gi, mp4, tm, false, -1, part, fuse);
  };
  ops.opdag = [&](qcdgpu_field o, qcdgpu_field i) { return dslash_partials(o, i, gi, mp4, tm, true, -1, nullptr); };
  ops.op64 = [&](qcdgpu_field o, qcdgpu_field i) { return dslash(o, i, g, mp4, tm, QCDGPU_OP_D, QCDGPU_ARITH_DF64); };
  ops.opdag64 = [&](qcdgpu_field o, qcdgpu_field i) {
    return dslash(o, i, g, mp4, tm, QCDGPU_OP_DDAG, QCDGPU_ARITH_DF64);
  };
  return cgnr_core(x, bd, sqrt(bn2), ops, p);
}

// Even/odd preconditioned CGNR. With D = A - H/2 (A = m+4 + i tm g5 on each
// site, H the hopping term) in even/odd blocks, x_o = A^{-1} (b_o + H_oe x_e / 2)
// and the even sites solve the Schur complement
//   M x_e = b_e + H_eo A^{-1} b_o / 2,   M = A - H_eo A^{-1} H_oe / 4,
// whose residual equals the full residual b - D x (its odd part vanishes).
// M is applied as two half-lattice kernels: t_o = A^{-1} H_oe x_e, then
// A x_e - H_eo t_o / 4 (with |M x_e|^2 summed in the second epilogue).
int solve_cgnr_eo(qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double mp4, double tm, qcdgpu_solve_params *p)
{
  if (!eo_lattice(b->L)) {
    set_error("even/odd solve: every lattice extent must be even");
    return 3;
  }
  Held w;
  p->iters = 0;
  p->reliable_updates = 0;
  p->true_residual = 1.0;
  double bn2;
  if (!blas_norm2(b, &bn2)) return 3;
  if (bn2 == 0.0) {
    p->true_residual = 0.0;
    return blas_zero(x) ? 0 : 3;
  }
  const int prec = p->inner_prec;
  qcdgpu_field bd = system_rhs(w, b, p->op);
  qcdgpu_gauge gi = gauge_at(g, prec);
  const int Lh[4] = {b->L[0] / 2, b->L[1], b->L[2], b->L[3]};
  qcdgpu_field be = w.get(Lh, QCDGPU_F64), bo = w.get(Lh, QCDGPU_F64), to = w.get(Lh, QCDGPU_F64);
  qcdgpu_field ce = w.get(Lh, QCDGPU_F64), xe = w.get(Lh, QCDGPU_F64), xo = w.get(Lh, QCDGPU_F64);
  qcdgpu_field ti = w.get(Lh, prec), t64 = w.get(Lh, QCDGPU_F64);  // odd intermediates
  qcdgpu_field tin = w.get(Lh, prec);
  if (!bd || !gi || !be || !bo || !to || !ce || !xe || !xo || !ti || !t64 || !tin) return 3;
  // c_e = b_e + H_eo A^{-1} b_o / 2
  if (!eo_split(be, bo, bd) || !eo_diag(to, bo, mp4, tm, true)) return 3;
  if (!dslash_eo(ce, to, be, g, mp4, tm, false, 0, 0.5, false, 1, nullptr, QCDGPU_ARITH_DF64)) return 3;
  CgOps ops;
  memcpy(ops.L, Lh, sizeof(ops.L));
  const int ar = QCDGPU_ARITH_DF64;  // FP64 fields: float-float arithmetic
  ops.op = [&](qcdgpu_field o, qcdgpu_field i, double *part, const CgFuse *fuse) {
    return dslash_eo(ti, i, nullptr, gi, mp4, tm, false, 1, 1.0, true, 0, nullptr, ar) &&
           dslash_eo(o, ti, i, gi, mp4, tm, false, 0, -0.25, false, 2, part, ar, fuse);
  };
  ops.opdag = [&](qcdgpu_field o, qcdgpu_field i) {
    return dslash_eo(ti, i, nullptr, gi, mp4, tm, true, 1, 1.0, true, 0, nullptr, ar) &&
           dslash_eo(o, ti, i, gi, mp4, tm, true, 0, -0.25, false, 2, nullptr, ar);
  };
  ops.op64 = [&](qcdgpu_field o, qcdgpu_field i) {
    return dslash_eo(t64, i, nullptr, g, mp4, tm, false, 1, 1.0, true, 0, nullptr, ar) &&
           dslash_eo(o, t64, i, g, mp4, tm, false, 0, -0.25, false, 2, nullptr, ar);
  };
  ops.opdag64 = [&](qcdgpu_field o, qcdgpu_field i) {
    return dslash_eo(t64, i, nullptr, g, mp4, tm, true, 1, 1.0, true, 0, nullptr, ar) &&
           dslash_eo(o, t64, i, g, mp4, tm, true, 0, -0.25, false, 2, nullptr, ar);
  };
  if (prec != QCDGPU_F64)
    ops.restart = [&](qcdgpu_field rs, qcdgpu_field rt, double *rr) {
      return convert_field(tin, rt) && ops.opdag(rs, tin) && blas_norm2(rs, rr);
    };
  const int st = cgnr_core(xe, ce, sqrt(bn2), ops, p);
  if (st == 3) return 3;
  // x_o = A^{-1} b_o + A^{-1} H_oe x_e / 2, then the full true residual
  if (!dslash_eo(xo, xe, to, g, mp4, tm, false, 1, 0.5, true, 1, nullptr, ar) || !eo_merge(x, xe, xo)) return 3;
  qcdgpu_field rt = w.get(b->L, QCDGPU_F64);
  double r2;
  if (!rt || !dslash(rt, x, g, mp4, tm, QCDGPU_OP_D, QCDGPU_ARITH_DF64) ||
      !blas_axpby(rt, 1.0, 0.0, bd, -1.0, 0.0, rt) || !blas_norm2(rt, &r2))
    return 3;
  p->true_residual = sqrt(r2 / bn2);
  return st == 0 && p->true_residual > p->tol ? 1 : st;
}

}  // namespace qg

// ------------------------------------------------------------ even/odd helpers
namespace qg {

// t-row parity trick: sites 2e and 2e + 1 of the full lattice have opposite
// parities (even t extent); the one of parity `par` goes to index e
__device__ __forceinline__ int eo_site(const Geom &g, int e, int par)
{
  int c[4];
  coords(g, 2 * e, c);
  return 2 * e + ((par ^ c[1] ^ c[2] ^ c[3]) & 1);
}

__global__ void k_eo_split(double2 *e, double2 *o, int64_t hstride, const double2 *f, int64_t fstride, Geom g, int Vh)
{
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= Vh) return;
  const int xe = eo_site(g, i, 0), xo = eo_site(g, i, 1);
#pragma unroll
  for (int k = 0; k < 12; k++) {
    e[k * hstride + i] = f[k * fstride + xe];
    o[k * hstride + i] = f[k * fstride + xo];
  }
}

__global__ void k_eo_merge(double2 *f, int64_t fstride, const double2 *e, const double2 *o, int64_t hstride, Geom g,
                           int Vh)
{
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= Vh) return;
  const int xe = eo_site(g, i, 0), xo = eo_site(g, i, 1);
#pragma unroll
  for (int k = 0; k < 12; k++) {
    f[k * fstride + xe] = e[k * hstride + i];
    f[k * fstride + xo] = o[k * hstride + i];
  }
}

// out = (ar + i ai g5) in
__global__ void k_eo_diag(double2 *out, const double2 *in, int64_t stride, int Vh, double ar, double ai)
{
  const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (i >= Vh) return;
#pragma unroll
  for (int k = 0; k < 12; k++) {
    const double2 v = in[k * stride + i];
    const double g = k < 6 ? ai : -ai;
    out[k * stride + i] = make_double2(ar * v.x - g * v.y, ar * v.y + g * v.x);
  }
}

static Geom full_geom(const int L[4])
{
  Geom g;
  for (int i = 0; i < 4; i++) g.L[i] = L[i];
  g.st[0] = 1;
  g.st[1] = L[0];
  g.st[2] = L[0] * L[1];
  g.st[3] = L[0] * L[1] * L[2];
  return g;
}

static bool halves_of(qcdgpu_field e, qcdgpu_field o, qcdgpu_field full)
{
  if (e->prec != QCDGPU_F64 || o->prec != QCDGPU_F64 || full->prec != QCDGPU_F64 || !same_shape(e, o) ||
      !eo_lattice(full->L) || e->L[0] * 2 != full->L[0] || e->L[1] != full->L[1] || e->L[2] != full->L[2] ||
      e->L[3] != full->L[3]) {
    set_error("even/odd split: FP64 half fields of the full field's lattice");
    return false;
  }
  return true;
}

bool eo_split(qcdgpu_field e, qcdgpu_field o, qcdgpu_field full)
{
  if (!halves_of(e, o, full)) return false;
  const int Vh = (int)e->V;
  k_eo_split<<<(unsigned)((Vh + 127) / 128), 128, 0, stream()>>>((double2 *)e->data, (double2 *)o->data, e->stride,
                                                                  (const double2 *)full->data, full->stride,
                                                                  full_geom(full->L), Vh);
  return QG_LAUNCHED("eo_split");
}

bool eo_merge(qcdgpu_field full, qcdgpu_field e, qcdgpu_field o)
{
  if (!halves_of(e, o, full)) return false;
  const int Vh = (int)e->V;
  k_eo_merge<<<(unsigned)((Vh + 127) / 128), 128, 0, stream()>>>((double2 *)full->data, full->stride,
                                                                  (const double2 *)e->data, (const double2 *)o->data,
                                                                  e->stride, full_geom(full->L), Vh);
  return QG_LAUNCHED("eo_merge");
}

bool eo_diag(qcdgpu_field out, qcdgpu_field in, double mp4, double tm, bool inverse)
{
  if (out->prec != QCDGPU_F64 || in->prec != QCDGPU_F64 || !same_shape(out, in)) {
    set_error("even/odd diagonal: FP64 fields of one shape");
    return false;
  }
  double ar = mp4, ai = tm;
  if (inverse) {
    const double den = mp4 * mp4 + tm * tm;
    ar = mp4 / den;
    ai = -tm / den;
  }
  k_eo_diag<<<(unsigned)((in->V + 127) / 128), 128, 0, stream()>>>((double2 *)out->data, (const double2 *)in->data,
                                                                    in->stride, (int)in->V, ar, ai);
  return QG_LAUNCHED("eo_diag");
}


// ------------------------------------------------- BiCGstab(l), even/odd
// BiCGstab(l) (Sleijpen & Fokkema, ETNA 1 (1993) 11) on the even/odd Schur
// complement M x_e = c_e of solve_cgnr_eo. Plain BiCGstab stagnates on this
// operator near the critical kappa (its one-step minimal-residual polynomial
// cannot damp eigenvalues of M that lie far off the real axis); BiCGstab(l)
// replaces it by a degree-l minimal-residual polynomial every l BiCG steps.
// One cycle: l BiCG steps (2 l applications of M, two dots each, read by
// the host), then the minimal-residual step from the Gram matrix
// G_ij = <r_i, r_j> of r_0 .. r_l (all dots queued, one synchronisation):
// gamma solves G[1..l][1..l] gamma = G[1..l][0], and
//   x += sum_j gamma_j r_{j-1},  r_0 -= sum_j gamma_j r_j,
//   u_0 -= sum_j gamma_j u_j,    omega = gamma_l.
// Mixed precision by reliable updates (Sleijpen & van der Vorst, Computing 56
// (1996) 141): one BiCGstab(l) recurrence runs in the inner precision; at a
// cycle's end, when the iterated residual has fallen by delta (p->delta in
// (0, 1), else 0.1) since the last update, looks converged, or the recurrence
// broke down, the increment is added to the FP64 x_e and r_0 is replaced by
// the FP64 true residual c_e - M x_e (float-float operator), keeping u_0 and
// the scalars (after a breakdown the recurrence restarts). The shadow
// residual is a fixed Z4 vector. Convergence is declared on the full true
// residual |b - D x| / |b|.

// gamma solving A gamma = c for the l x l Hermitian A (Gaussian elimination
// with partial pivoting); false when A is singular
static bool small_solve(int n, std::vector<std::complex<double>> A, std::vector<std::complex<double>> c,
                        std::vector<std::complex<double>> &x)
{
  for (int k = 0; k < n; k++) {
    int piv = k;
    for (int i = k + 1; i < n; i++)
      if (std::abs(A[i * n + k]) > std::abs(A[piv * n + k])) piv = i;
    if (std::abs(A[piv * n + k]) == 0.0) return false;
    if (piv != k) {
      for (int j = 0; j < n; j++) std::swap(A[k * n + j], A[piv * n + j]);
      std::swap(c[k], c[piv]);
    }
    for (int i = k + 1; i < n; i++) {
      const std::complex<double> f = A[i * n + k] / A[k * n + k];
      for (int j = k; j < n; j++) A[i * n + j] -= f * A[k * n + j];
      c[i] -= f * c[k];
    }
  }
  x.assign(n, 0.0);
  for (int i = n - 1; i >= 0; i--) {
    std::complex<double> t = c[i];
    for (int j = i + 1; j < n; j++) t -= A[i * n + j] * x[j];
    x[i] = t / A[i * n + i];
  }
  return true;
}

int solve_bicgstabl_eo(qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double mp4, double tm,
                       qcdgpu_solve_params *p)
{
  using cplx = std::complex<double>;
  if (!eo_lattice(b->L)) {
    set_error("even/odd solve: every lattice extent must be even");
    return 3;
  }
  Held w;
  p->iters = 0;
  p->reliable_updates = 0;
  p->true_residual = 1.0;
  double bn2;
  if (!blas_norm2(b, &bn2)) return 3;
  if (bn2 == 0.0) {
    p->true_residual = 0.0;
    return blas_zero(x) ? 0 : 3;
  }
  const int ell = p->restart >= 1 && p->restart <= 16 ? p->restart : 8;
  const int prec = p->inner_prec;
  const int xprec = prec == QCDGPU_F16 ? QCDGPU_F32 : prec;  // the inner increment keeps FP32 at least
  const int ar = QCDGPU_ARITH_DF64;
  qcdgpu_field bd = system_rhs(w, b, p->op);
  qcdgpu_gauge gi = gauge_at(g, prec);
  const int Lh[4] = {b->L[0] / 2, b->L[1], b->L[2], b->L[3]};
  qcdgpu_field be = w.get(Lh, QCDGPU_F64), bo = w.get(Lh, QCDGPU_F64), to = w.get(Lh, QCDGPU_F64);
  qcdgpu_field ce = w.get(Lh, QCDGPU_F64), xe = w.get(Lh, QCDGPU_F64), xo = w.get(Lh, QCDGPU_F64);
  qcdgpu_field re = w.get(Lh, QCDGPU_F64), t64 = w.get(Lh, QCDGPU_F64), e64 = w.get(Lh, QCDGPU_F64);
  qcdgpu_field ti = w.get(Lh, prec), rh = w.get(Lh, prec), xi = w.get(Lh, xprec);
  // FP16 vectors reach the FP32 increment through this conversion buffer
  qcdgpu_field cv = xprec != prec ? w.get(Lh, xprec) : nullptr;
  if (xprec != prec && !cv) return 3;
  auto add_to_x = [&](cplx a, qcdgpu_field v) {
    if (cv) {
      if (!convert_field(cv, v)) return false;
      v = cv;
    }
    return blas_axpby(xi, a.real(), a.imag(), v, 1.0, 0.0, xi);
  };
  std::vector<qcdgpu_field> R(ell + 1), U(ell + 1);
  for (int j = 0; j <= ell; j++) {
    R[j] = w.get(Lh, prec);
    U[j] = w.get(Lh, prec);
    if (!R[j] || !U[j]) return 3;
  }
  if (!bd || !gi || !be || !bo || !to || !ce || !xe || !xo || !re || !t64 || !e64 || !ti || !rh || !xi) return 3;
  // the Gram matrix's dots land in one device buffer and come back together
  static double *gram_dev = nullptr, *gram_host = nullptr;
  const int npair = (ell + 1) * (ell + 2) / 2;
  if (!gram_dev) {
    if (!QG_CUDA(cudaMalloc(&gram_dev, sizeof(double) * 2 * 153)) ||
        !QG_CUDA(cudaMallocHost(&gram_host, sizeof(double) * 2 * 153)))
      return 3;
  }
  // c_e = b_e + H_eo A^{-1} b_o / 2
  if (!eo_split(be, bo, bd) || !eo_diag(to, bo, mp4, tm, true)) return 3;
  if (!dslash_eo(ce, to, be, g, mp4, tm, false, 0, 0.5, false, 1, nullptr, ar)) return 3;
  auto M = [&](qcdgpu_field o, qcdgpu_field i) {
    return dslash_eo(ti, i, nullptr, gi, mp4, tm, false, 1, 1.0, true, 0, nullptr, ar) &&
           dslash_eo(o, ti, i, gi, mp4, tm, false, 0, -0.25, false, 2, nullptr, ar);
  };
  auto M64 = [&](qcdgpu_field o, qcdgpu_field i) {
    return dslash_eo(t64, i, nullptr, g, mp4, tm, false, 1, 1.0, true, 0, nullptr, ar) &&
           dslash_eo(o, t64, i, g, mp4, tm, false, 0, -0.25, false, 2, nullptr, ar);
  };
  auto dotc = [&](qcdgpu_field a, qcdgpu_field c, cplx *d) {
    double r[2];
    if (!blas_dot(a, c, r)) return false;
    *d = cplx(r[0], r[1]);
    return true;
  };
  const double bn = sqrt(bn2), target = p->tol * bn;
  // reliable-update threshold: FP64 iterations update only to confirm convergence
  const double delta = prec == QCDGPU_F64 ? 0.0 : (p->delta > 0.0 && p->delta < 1.0 ? p->delta : 0.1);
  if (!blas_zero(xe) || !blas_copy(re, ce) || !field_z4(rh, 0x5EEDull)) return 3;
  double rn2;
  if (!blas_norm2(re, &rn2)) return 3;
  double rn = sqrt(rn2);
  if (!convert_field(R[0], re) || !blas_zero(U[0]) || !blas_zero(xi)) return 3;
  cplx rho0 = 1.0, alpha = 0.0, omega = 1.0;
  double rmax = rn, best = rn;  // largest iterated residual since the last update; smallest true residual
  int st = rn <= target ? 0 : 1, since = 0, stall = 0;
  while (st != 0 && p->iters < p->maxiter) {
    bool breakdown = false;
    rho0 = -omega * rho0;
    for (int j = 0; j < ell && !breakdown; j++) {
      cplx rho1, gam;
      if (!dotc(rh, R[j], &rho1)) return 3;
      if (std::abs(rho1) == 0.0 || std::abs(rho0) == 0.0) {
        breakdown = true;
        break;
      }
      const cplx beta = alpha * rho1 / rho0;
      rho0 = rho1;
      for (int i = 0; i <= j; i++)  // u_i = r_i - beta u_i
        if (!blas_axpby(U[i], 1.0, 0.0, R[i], -beta.real(), -beta.imag(), U[i])) return 3;
      if (!M(U[j + 1], U[j])) return 3;
      if (!dotc(rh, U[j + 1], &gam)) return 3;
      if (std::abs(gam) == 0.0) {
        breakdown = true;
        break;
      }
      alpha = rho0 / gam;
      for (int i = 0; i <= j; i++)  // r_i -= alpha u_{i+1}
        if (!blas_axpby(R[i], -alpha.real(), -alpha.imag(), U[i + 1], 1.0, 0.0, R[i])) return 3;
      if (!M(R[j + 1], R[j])) return 3;
      if (!add_to_x(alpha, U[0])) return 3;
      p->iters += 2;
    }
    double rr = 0.0;
    if (!breakdown) {
      // minimal-residual step from the Gram matrix of r_0 .. r_l
      int k = 0;
      for (int i = 0; i <= ell; i++)
        for (int j = i; j <= ell; j++, k++)
          if (!blas_dot_dev(R[i], R[j], gram_dev + 2 * k)) return 3;
      if (!QG_CUDA(cudaMemcpyAsync(gram_host, gram_dev, sizeof(double) * 2 * npair, cudaMemcpyDeviceToHost,
                                   stream())) ||
          !QG_CUDA(cudaStreamSynchronize(stream())))
        return 3;
      std::vector<cplx> G((ell + 1) * (ell + 1));
      k = 0;
      for (int i = 0; i <= ell; i++)
        for (int j = i; j <= ell; j++, k++) {
          G[i * (ell + 1) + j] = cplx(gram_host[2 * k], gram_host[2 * k + 1]);
          G[j * (ell + 1) + i] = std::conj(G[i * (ell + 1) + j]);
        }
      std::vector<cplx> A(ell * ell), c(ell), gm;
      for (int i = 0; i < ell; i++) {
        c[i] = G[(i + 1) * (ell + 1)];
        for (int j = 0; j < ell; j++) A[i * ell + j] = G[(i + 1) * (ell + 1) + j + 1];
      }
      if (!small_solve(ell, A, c, gm) || std::abs(gm[ell - 1]) == 0.0) {
        breakdown = true;
      } else {
        for (int j = 1; j <= ell; j++) {
          const cplx gj = gm[j - 1];
          if (!add_to_x(gj, R[j - 1]) || !blas_axpby(R[0], -gj.real(), -gj.imag(), R[j], 1.0, 0.0, R[0]) ||
              !blas_axpby(U[0], -gj.real(), -gj.imag(), U[j], 1.0, 0.0, U[0]))
            return 3;
        }
        omega = gm[ell - 1];
        // |r_0 - R gamma|^2 = G_00 - c^+ gamma at the minimum
        cplx cg = 0.0;
        for (int i = 0; i < ell; i++) cg += std::conj(c[i]) * gm[i];
        const double r2 = G[0].real() - cg.real();
        rr = r2 > 0.0 ? sqrt(r2) : 0.0;
      }
    }
    since++;
    // reliable update: the iterated residual fell by delta (or looks
    // converged, or the recurrence broke down, or a long plateau): fold the
    // increment into x_e and continue from the FP64 true residual
    if (breakdown || rr <= delta * rmax || rr <= target || since >= 256) {
      if (!convert_field(e64, xi) || !blas_axpby(xe, 1.0, 0.0, e64, 1.0, 0.0, xe) || !blas_zero(xi)) return 3;
      if (!M64(e64, xe) || !blas_axpby(re, 1.0, 0.0, ce, -1.0, 0.0, e64) || !blas_norm2(re, &rn2)) return 3;
      rn = sqrt(rn2);
      p->reliable_updates++;
      since = 0;
      if (rn <= target) {
        st = 0;
        break;
      }
      if (rn < 0.9 * best) {
        best = rn;
        stall = 0;
      } else if (++stall >= 8) {
        st = breakdown ? 2 : 1;
        break;
      }
      if (!convert_field(R[0], re)) return 3;
      rmax = rn;
      if (breakdown) {  // start the recurrence afresh from the true residual
        if (!blas_zero(U[0])) return 3;
        rho0 = 1.0;
        alpha = 0.0;
        omega = 1.0;
      }
    } else if (rr > rmax) {
      rmax = rr;
    }
  }
  // x_o = A^{-1} b_o + A^{-1} H_oe x_e / 2, then the full true residual
  if (!dslash_eo(xo, xe, to, g, mp4, tm, false, 1, 0.5, true, 1, nullptr, ar) || !eo_merge(x, xe, xo)) return 3;
  qcdgpu_field rt = w.get(b->L, QCDGPU_F64);
  double r2;
  if (!rt || !dslash(rt, x, g, mp4, tm, QCDGPU_OP_D, QCDGPU_ARITH_DF64) ||
      !blas_axpby(rt, 1.0, 0.0, bd, -1.0, 0.0, rt) || !blas_norm2(rt, &r2))
    return 3;
  p->true_residual = sqrt(r2 / bn2);
  return st == 0 && p->true_residual > p->tol ? 1 : st;
}

}  // namespace qg
