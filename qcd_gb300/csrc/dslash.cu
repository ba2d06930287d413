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
// One thread per site. Each of the eight neighbour spinors is projected to a
// two-spin half spinor straight after its load, multiplied by the link,
// phased when theta_mu != 0, and expanded back into the 4-spin accumulator.
// Links arrive as 12 reals (third row rebuilt) when the field is SU(3).
#include "internal.h"

namespace qg {

using namespace qgd;

struct DArgs {
  void *out;
  float *out_norm;
  const void *in;
  const float *in_norm;
  const void *gauge;
  Geom geo;
  int64_t V;
  int64_t stride;   // spinor block stride
  int64_t gstride;  // gauge block stride
  double phr[4], phi[4];
  int twist_mask;
  double mp4, tm;  // tm already negated for D^+
  int op_q;        // multiply the result by i g5
};

// h = (1 + S g_mu) p restricted to spins 0,1 (the independent half)
template <int MU, int S, typename R>
__device__ __forceinline__ void project(const C<R> p[12], C<R> h[6])
{
#pragma unroll
  for (int c = 0; c < 3; c++) {
    C<R> p0 = p[c], p1 = p[3 + c], p2 = p[6 + c], p3 = p[9 + c];
    if (MU == 0) {
      h[c] = S > 0 ? p0 - p2 : p0 + p2;
      h[3 + c] = S > 0 ? p1 - p3 : p1 + p3;
    } else if (MU == 1) {
      h[c] = S > 0 ? p0 - mul_i(p3) : p0 + mul_i(p3);
      h[3 + c] = S > 0 ? p1 - mul_i(p2) : p1 + mul_i(p2);
    } else if (MU == 2) {
      h[c] = S > 0 ? p0 - p3 : p0 + p3;
      h[3 + c] = S > 0 ? p1 + p2 : p1 - p2;
    } else {
      h[c] = S > 0 ? p0 - mul_i(p2) : p0 + mul_i(p2);
      h[3 + c] = S > 0 ? p1 + mul_i(p3) : p1 - mul_i(p3);
    }
  }
}

// acc += (1 + S g_mu) spinor rebuilt from its upper half h
template <int MU, int S, typename R>
__device__ __forceinline__ void accumulate(C<R> acc[12], const C<R> h[6])
{
#pragma unroll
  for (int c = 0; c < 3; c++) {
    C<R> h0 = h[c], h1 = h[3 + c];
    acc[c] = acc[c] + h0;
    acc[3 + c] = acc[3 + c] + h1;
    if (MU == 0) {
      acc[6 + c] = S > 0 ? acc[6 + c] - h0 : acc[6 + c] + h0;
      acc[9 + c] = S > 0 ? acc[9 + c] - h1 : acc[9 + c] + h1;
    } else if (MU == 1) {
      acc[6 + c] = S > 0 ? acc[6 + c] + mul_i(h1) : acc[6 + c] - mul_i(h1);
      acc[9 + c] = S > 0 ? acc[9 + c] + mul_i(h0) : acc[9 + c] - mul_i(h0);
    } else if (MU == 2) {
      acc[6 + c] = S > 0 ? acc[6 + c] + h1 : acc[6 + c] - h1;
      acc[9 + c] = S > 0 ? acc[9 + c] - h0 : acc[9 + c] + h0;
    } else {
      acc[6 + c] = S > 0 ? acc[6 + c] + mul_i(h0) : acc[6 + c] - mul_i(h0);
      acc[9 + c] = S > 0 ? acc[9 + c] - mul_i(h1) : acc[9 + c] + mul_i(h1);
    }
  }
}

template <int MU, bool DAG, int SP, int GP, int RECON, typename R>
__device__ __forceinline__ void hop_pair(const DArgs &a, int64_t x, const int c[4], C<R> acc[12])
{
  constexpr int SF = DAG ? +1 : -1;  // projector sign of the forward hop
  const bool twisted = (a.twist_mask >> MU) & 1;
  {
    int64_t y = fwd(a.geo, x, c, MU);
    C<R> s[12], h[6], uh[6], U[9];
    Spinor<SP, R>::load(a.in, a.in_norm, a.stride, y, s);
    project<MU, SF>(s, h);
    Link<GP, RECON, R>::load(a.gauge, a.gstride, x, MU, U);
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
      for (int i = 0; i < 3; i++)
        uh[3 * j + i] = U[3 * i] * h[3 * j] + U[3 * i + 1] * h[3 * j + 1] + U[3 * i + 2] * h[3 * j + 2];
    if (twisted) {
      C<R> ph{(R)a.phr[MU], (R)a.phi[MU]};
#pragma unroll
      for (int k = 0; k < 6; k++) uh[k] = uh[k] * ph;
    }
    accumulate<MU, SF>(acc, uh);
  }
  {
    int64_t y = bwd(a.geo, x, c, MU);
    C<R> s[12], h[6], uh[6], U[9];
    Spinor<SP, R>::load(a.in, a.in_norm, a.stride, y, s);
    project<MU, -SF>(s, h);
    Link<GP, RECON, R>::load(a.gauge, a.gstride, y, MU, U);
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
      for (int i = 0; i < 3; i++)
        uh[3 * j + i] = cdot(U[i], h[3 * j]) + cdot(U[3 + i], h[3 * j + 1]) + cdot(U[6 + i], h[3 * j + 2]);
    if (twisted) {
      C<R> ph{(R)a.phr[MU], -(R)a.phi[MU]};
#pragma unroll
      for (int k = 0; k < 6; k++) uh[k] = uh[k] * ph;
    }
    accumulate<MU, -SF>(acc, uh);
  }
}

template <bool DAG, int SP, int GP, int RECON, typename R>
__global__ void __launch_bounds__(128) k_wilson(const DArgs a)
{
  int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= a.V) return;
  int c[4];
  coords(a.geo, x, c);
  C<R> acc[12];
#pragma unroll
  for (int k = 0; k < 12; k++) acc[k] = C<R>{(R)0, (R)0};
  hop_pair<0, DAG, SP, GP, RECON, R>(a, x, c, acc);
  hop_pair<1, DAG, SP, GP, RECON, R>(a, x, c, acc);
  hop_pair<2, DAG, SP, GP, RECON, R>(a, x, c, acc);
  hop_pair<3, DAG, SP, GP, RECON, R>(a, x, c, acc);
  C<R> s[12];
  Spinor<SP, R>::load(a.in, a.in_norm, a.stride, x, s);
  const R mp4 = (R)a.mp4, tm = (R)a.tm, half = (R)0.5;
#pragma unroll
  for (int k = 0; k < 12; k++) {
    // (m+4) s + i tm g5 s - acc/2 ; g5 = +1 for spins 0,1, -1 for spins 2,3
    R g5tm = k < 6 ? tm : -tm;
    C<R> d{mp4 * s[k].re - g5tm * s[k].im, mp4 * s[k].im + g5tm * s[k].re};
    d = d - half * acc[k];
    if (a.op_q) d = k < 6 ? mul_i(d) : -mul_i(d);
    acc[k] = d;
  }
  Spinor<SP, R>::store(a.out, a.out_norm, a.stride, x, acc);
}

// float-float kernel for FP64 storage (dslash_df64.cu)
bool dslash_df64(const DArgs &a, bool dag, int recon);

template <bool DAG>
static bool launch_native(const DArgs &a, int prec, int recon)
{
  unsigned grid = (unsigned)((a.V + 127) / 128);
  cudaStream_t s = stream();
  if (prec == QCDGPU_F64 && recon == 12) k_wilson<DAG, QCDGPU_F64, QCDGPU_F64, 12, double><<<grid, 128, 0, s>>>(a);
  else if (prec == QCDGPU_F64) k_wilson<DAG, QCDGPU_F64, QCDGPU_F64, 18, double><<<grid, 128, 0, s>>>(a);
  else if (prec == QCDGPU_F32 && recon == 12) k_wilson<DAG, QCDGPU_F32, QCDGPU_F32, 12, float><<<grid, 128, 0, s>>>(a);
  else if (prec == QCDGPU_F32) k_wilson<DAG, QCDGPU_F32, QCDGPU_F32, 18, float><<<grid, 128, 0, s>>>(a);
  else k_wilson<DAG, QCDGPU_F16, QCDGPU_F16, 12, float><<<grid, 128, 0, s>>>(a);
  return QG_LAUNCHED("wilson");
}

static bool dslash_once(qcdgpu_field out, qcdgpu_field in, qcdgpu_gauge g, double mp4, double tm,
                        bool dag, bool q, int arith)
{
  DArgs a;
  a.out = out->data;
  a.out_norm = out->norm;
  a.in = in->data;
  a.in_norm = in->norm;
  a.gauge = g->data;
  for (int i = 0; i < 4; i++) a.geo.L[i] = in->L[i];
  a.geo.st[0] = 1;
  a.geo.st[1] = in->L[0];
  a.geo.st[2] = (int64_t)in->L[0] * in->L[1];
  a.geo.st[3] = (int64_t)in->L[0] * in->L[1] * in->L[2];
  a.V = in->V;
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
  if (in->prec == QCDGPU_F64 && arith == QCDGPU_ARITH_DF64) return dslash_df64(a, dag, g->recon);
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

int g_f64_arith = QCDGPU_ARITH_F64;

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
