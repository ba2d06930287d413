// dslash.cu -- the Wilson-twisted-mass operator on the GPU.
//
//   D psi(x) = (m+4) psi(x) + i tm g5 psi(x)
//     - 1/2 sum_mu [ (1 - g_mu) U_mu(x)      e^{+i th_mu/L_mu} psi(x+mu)
//                  + (1 + g_mu) U_mu(x-mu)^+ e^{-i th_mu/L_mu} psi(x-mu) ]
//
// (qcd_applyWilsonTMOp, lib/src/qcd_wilson.c:114-336; chiral basis of
// lib/src/qcd_gamma.c:46-103, g5 = diag(1,1,-1,-1)). D^+ swaps the two
// projectors and flips the sign of tm. Q = i g5 D (qcd_wilson.c:795-814).
//
// Kernel template: wilson_kernel.cuh. This file instantiates it for native
// double (FP64 fields) and float (FP32 and FP16 fields) arithmetic and holds
// the operator dispatch.
#include "wilson_kernel.cuh"

namespace qg {

using namespace qgd;


// float-float kernel for FP64 storage (dslash_df64.cu)
bool dslash_df64(const DArgs &a, bool dag, bool eo = false);

template <bool DAG>
static bool launch_native(const DArgs &a, int prec, int recon)
{
  unsigned grid = (unsigned)((a.V - a.x0 + 127) / 128);
  cudaStream_t s = stream();
  // FP64 arithmetic is the bottleneck of the native FP64 kernel (GB300 runs
  // DFMA at ~1/60 of the FP32 rate): read all 18 link reals, no rebuild
  if (prec == QCDGPU_F64) k_wilson<DAG, QCDGPU_F64, QCDGPU_F64, 18, double><<<grid, 128, 0, s>>>(a);
  else if (prec == QCDGPU_F32 && recon == 12) k_wilson<DAG, QCDGPU_F32, QCDGPU_F32, 12, float><<<grid, 128, 0, s>>>(a);
  else if (prec == QCDGPU_F32) k_wilson<DAG, QCDGPU_F32, QCDGPU_F32, 18, float><<<grid, 128, 0, s>>>(a);
  else k_wilson<DAG, QCDGPU_F16, QCDGPU_F16, 12, float><<<grid, 128, 0, s>>>(a);
  return QG_LAUNCHED("wilson");
}

// in_aos / out_aos (float-float arithmetic only): read and write spinors in
// the host layout at these device addresses instead of in / out's data
static bool dslash_once(qcdgpu_field out, qcdgpu_field in, qcdgpu_gauge g, double mp4, double tm,
                        bool dag, bool q, int arith, double *partials = nullptr, int x0 = 0, int x1 = -1,
                        const void *in_aos = nullptr, void *out_aos = nullptr, const CgFuse *fuse = nullptr)
{
  DArgs a;
  a.partials = partials;
  if (partials && fuse) {
    a.cg_done = fuse->done;
    a.cg_s = fuse->s;
    a.cg_hist = fuse->hist;
  }
  a.x0 = x0;
  a.out = out->data;
  a.out_norm = out->norm;
  a.in = in->data;
  a.in_norm = in->norm;
  a.gauge = g->data;
  for (int i = 0; i < 4; i++) a.geo.L[i] = in->L[i];
  a.geo.st[0] = 1;
  a.geo.st[1] = in->L[0];
  a.geo.st[2] = in->L[0] * in->L[1];
  a.geo.st[3] = in->L[0] * in->L[1] * in->L[2];
  a.V = x1 < 0 ? (int)in->V : x1;
  a.stride = in->stride;
  a.gstride = g->stride;
  a.twist_mask = 0;
  for (int mu = 0; mu < 4; mu++) {
    if (g->theta[mu] != 0.0) {
      a.twist_mask |= 1 << mu;
      a.phr[mu] = cos(g->theta[mu] / (double)g->L[mu]);
      a.phi[mu] = sin(g->theta[mu] / (double)g->L[mu]);
    } else {
      a.phr[mu] = 1.0;
      a.phi[mu] = 0.0;
    }
  }
  a.mp4 = mp4;
  a.tm = dag ? -tm : tm;
  a.op_q = q ? 1 : 0;
  for (int mu = 0; mu < 4; mu++) {
    split_host(a.phr[mu], &a.phr_h[mu], &a.phr_l[mu]);
    split_host(a.phi[mu], &a.phi_h[mu], &a.phi_l[mu]);
  }
  split_host(a.mp4, &a.mp4_h, &a.mp4_l);
  split_host(a.tm, &a.tm_h, &a.tm_l);
  if (in->prec == QCDGPU_F64 && arith == QCDGPU_ARITH_DF64) {
    // float-pair copy of the links (made once per field, phases folded in)
    qcdgpu_gauge gf = gauge_at(g, kGaugeFF);
    if (!gf) return false;
    a.gauge = gf->data;
    a.gstride = gf->stride;
    if (in_aos) {
      a.in = in_aos;
      a.out = out_aos;
      a.in_norm = a.out_norm = nullptr;
      a.aos = 1;
    }
    return dslash_df64(a, dag);
  }
  if (in_aos) {
    set_error("dslash on host-layout spinors: float-float arithmetic only");
    return false;
  }
  return dag ? launch_native<true>(a, in->prec, g->recon) : launch_native<false>(a, in->prec, g->recon);
}

bool dslash(qcdgpu_field out, qcdgpu_field in, qcdgpu_gauge g, double mp4, double tm, int op, int arith)
{
  if (!out || !in || !g) {
    set_error("dslash: null field");
    return false;
  }
  if (!same_shape(out, in) || in->V != g->V || in->L[0] != g->L[0] || in->L[1] != g->L[1] ||
      in->L[2] != g->L[2] || in->L[3] != g->L[3]) {
    set_error("dslash: lattice shapes of the fields differ");
    return false;
  }
  if (out == in || out->data == in->data) {
    set_error("dslash: output must not alias the input");
    return false;
  }
  if (in->prec != out->prec || in->prec != g->prec) {
    set_error("dslash: spinor and gauge precisions must agree (%d, %d, %d)", in->prec, out->prec, g->prec);
    return false;
  }
  if (arith < 0) arith = g_f64_arith;
  switch (op) {
  case QCDGPU_OP_D: return dslash_once(out, in, g, mp4, tm, false, false, arith);
  case QCDGPU_OP_Q: return dslash_once(out, in, g, mp4, tm, false, true, arith);
  case QCDGPU_OP_DDAG: return dslash_once(out, in, g, mp4, tm, true, false, arith);
  case QCDGPU_OP_DDAGD: {
    qcdgpu_field t = work_get(in->L, in->prec);
    if (!t) return false;
    bool ok = dslash_once(t, in, g, mp4, tm, false, false, arith) &&
              dslash_once(out, t, g, mp4, tm, true, false, arith);
    work_put(t);
    return ok;
  }
  default: set_error("dslash: unknown operator %d", op); return false;
  }
}

// Even/odd kernel on half fields (FP64, FP32 or FP16 with a gauge field of
// the same precision): out (parity par) = ch * [A^{-1}] H in + {0 | z | A z}
// with A = mp4 + i tm g5 (D^+: tm -> -tm and the hopping term of D^+).
// in, out, z are fields on the half lattice {L_t / 2, L_x, L_y, L_z}.
bool dslash_eo(qcdgpu_field out, qcdgpu_field in, qcdgpu_field z, qcdgpu_gauge g, double mp4, double tm, bool dag,
               int par, double ch, bool ainv, int zmode, double *partials, int arith, const CgFuse *fuse)
{
  if (!out || !in || !g || out == in || (zmode && (!z || z == out)) || in->prec != out->prec ||
      in->prec != g->prec || (z && z->prec != in->prec) || !eo_lattice(g->L) || in->L[0] * 2 != g->L[0] ||
      in->L[1] != g->L[1] || in->L[2] != g->L[2] || in->L[3] != g->L[3] || !same_shape(out, in) ||
      (z && !same_shape(z, in))) {
    set_error("even/odd operator: half fields of one precision on the gauge field's half lattice (every extent "
              "even)");
    return false;
  }
  DArgs a;
  a.partials = partials;
  if (partials && fuse) {
    a.cg_done = fuse->done;
    a.cg_s = fuse->s;
    a.cg_hist = fuse->hist;
  }
  a.x0 = 0;
  a.out = out->data;
  a.out_norm = out->norm;
  a.in = in->data;
  a.in_norm = in->norm;
  a.z = z ? z->data : nullptr;
  a.z_norm = z ? z->norm : nullptr;
  a.gauge = g->data;
  for (int i = 0; i < 4; i++) a.geo.L[i] = g->L[i];
  a.geo.st[0] = 1;
  a.geo.st[1] = g->L[0];
  a.geo.st[2] = g->L[0] * g->L[1];
  a.geo.st[3] = g->L[0] * g->L[1] * g->L[2];
  a.V = (int)in->V;
  a.stride = in->stride;
  a.gstride = g->stride;
  a.twist_mask = 0;
  for (int mu = 0; mu < 4; mu++) {
    a.phr[mu] = 1.0;
    a.phi[mu] = 0.0;
    if (g->theta[mu] != 0.0) {
      a.twist_mask |= 1 << mu;
      a.phr[mu] = cos(g->theta[mu] / (double)g->L[mu]);
      a.phi[mu] = sin(g->theta[mu] / (double)g->L[mu]);
    }
    split_host(a.phr[mu], &a.phr_h[mu], &a.phr_l[mu]);
    split_host(a.phi[mu], &a.phi_h[mu], &a.phi_l[mu]);
  }
  a.mp4 = mp4;
  a.tm = dag ? -tm : tm;
  a.op_q = 0;
  a.eo_par = par;
  a.zmode = zmode;
  a.ainv = ainv ? 1 : 0;
  a.ch = ch;
  const double den = a.mp4 * a.mp4 + a.tm * a.tm;
  a.ai_r = a.mp4 / den;
  a.ai_i = -a.tm / den;
  split_host(a.mp4, &a.mp4_h, &a.mp4_l);
  split_host(a.tm, &a.tm_h, &a.tm_l);
  split_host(a.ch, &a.ch_h, &a.ch_l);
  split_host(a.ai_r, &a.ai_r_h, &a.ai_r_l);
  split_host(a.ai_i, &a.ai_i_h, &a.ai_i_l);
  if (in->prec == QCDGPU_F64 && arith == QCDGPU_ARITH_DF64) {
    // float-pair copy of the links (phases folded in)
    qcdgpu_gauge gf = gauge_at(g, kGaugeFF);
    if (!gf) return false;
    a.gauge = gf->data;
    a.gstride = gf->stride;
    return dslash_df64(a, dag, true);
  }
  const unsigned grid = (unsigned)((a.V + 127) / 128);
  cudaStream_t s = stream();
#define QG_EO(SP, RECON, R)                                                        \
  if (dag) k_wilson_eo<true, SP, SP, RECON, R><<<grid, 128, 0, s>>>(a);            \
  else k_wilson_eo<false, SP, SP, RECON, R><<<grid, 128, 0, s>>>(a);
  if (in->prec == QCDGPU_F64) {
    QG_EO(QCDGPU_F64, 18, double)
  } else if (in->prec == QCDGPU_F32 && g->recon == 12) {
    QG_EO(QCDGPU_F32, 12, float)
  } else if (in->prec == QCDGPU_F32) {
    QG_EO(QCDGPU_F32, 18, float)
  } else {
    QG_EO(QCDGPU_F16, 12, float)
  }
#undef QG_EO
  return QG_LAUNCHED("wilson_eo");
}

// out = op(in) (op D or Q) on sites x0 .. x1-1 only: the pieces of a
// pipelined apply. The neighbours' values must be in place.
bool dslash_sites(qcdgpu_field out, qcdgpu_field in, qcdgpu_gauge g, double mp4, double tm, int op, int arith,
                  int x0, int x1)
{
  if (!out || !in || !g || out == in || in->prec != out->prec || in->prec != g->prec || in->V != g->V ||
      !same_shape(out, in) || (op != QCDGPU_OP_D && op != QCDGPU_OP_Q) || x0 < 0 || x1 > in->V || x0 >= x1) {
    set_error("dslash over a site range: fields of one shape, op D or Q, 0 <= x0 < x1 <= V");
    return false;
  }
  if (arith < 0) arith = g_f64_arith;
  return dslash_once(out, in, g, mp4, tm, false, op == QCDGPU_OP_Q, arith, nullptr, x0, x1);
}

// D or Q on sites [x0, x1) of spinors in the host layout (12 double2 per
// site) at device addresses in_aos / out_aos, computed by the float-float
// kernel; `shape` is an FP64 field of the lattice (its data is not used)
bool dslash_sites_aos(void *out_aos, const void *in_aos, qcdgpu_field shape, qcdgpu_gauge g, double mp4, double tm,
                      int op, int x0, int x1)
{
  if (!out_aos || !in_aos || !shape || !g || out_aos == in_aos || shape->prec != QCDGPU_F64 ||
      g->prec != QCDGPU_F64 || shape->V != g->V || (op != QCDGPU_OP_D && op != QCDGPU_OP_Q) || x0 < 0 ||
      x1 > shape->V || x0 >= x1) {
    set_error("dslash over a site range of host-layout spinors: FP64, op D or Q, 0 <= x0 < x1 <= V");
    return false;
  }
  return dslash_once(shape, shape, g, mp4, tm, false, op == QCDGPU_OP_Q, QCDGPU_ARITH_DF64, nullptr, x0, x1, in_aos,
                     out_aos);
}

// out = D in (dag: D^+ in) on fields checked by the caller; when partials is
// non-null, block b of the launch (128 sites each) also writes the sum of
// |out|^2 over its sites to partials[b], and with fuse the block that
// finishes last forms the CG step from them
bool dslash_partials(qcdgpu_field out, qcdgpu_field in, qcdgpu_gauge g, double mp4, double tm, bool dag,
                     int arith, double *partials, const CgFuse *fuse)
{
  if (arith < 0) arith = g_f64_arith;
  return dslash_once(out, in, g, mp4, tm, dag, false, arith, partials, 0, -1, nullptr, nullptr, fuse);
}

// float-float by default: GB300 runs FP64 at ~1/58 of its FP32 rate, and
// the float-float operator meets the same per-site parity 3.6x faster
int g_f64_arith = QCDGPU_ARITH_DF64;

}  // namespace qg

extern "C" {

int qcdgpu_dslash(qcdgpu_field out, qcdgpu_field in, qcdgpu_gauge g, double kappa, double mu, int op, int arith)
{
  if (!(kappa > 0.0)) {
    qg::set_error("dslash: kappa must be positive");
    return 1;
  }
  return qg::dslash(out, in, g, 1.0 / (2.0 * kappa), mu, op, arith) ? 0 : 1;
}

int qcdgpu_set_f64_arith(int arith)
{
  if (arith != QCDGPU_ARITH_F64 && arith != QCDGPU_ARITH_DF64) return 1;
  qg::g_f64_arith = arith;
  return 0;
}

}  // extern "C"
