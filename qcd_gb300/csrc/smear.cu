// smear.cu -- source construction on the GPU: 3D APE smearing of the links,
// 3D Gaussian smearing of a spinor on one time-slice, and the smeared point
// source built from both (the setup of the 24^3 x 48 single-RHS workload).
//
// APE step (qcd_apeSmear3d, lib/src/qcd_smearing.c:209-276): for spatial
// mu, U'_mu(x) = Proj_SU3( U_mu(x) + alpha * sum over spatial nu != mu of
//   U_nu(x) U_mu(x+nu) U_nu(x+mu)^+  +  U_nu(x-nu)^+ U_mu(x-nu) U_nu(x-nu+mu) );
// temporal links are copied. Proj_SU3 (qcd_projectSU33d, lib/src/qcd_blas.c:
// 950) is the unitary polar factor of M times exp(-i arg(det M) / 3) with
// the columns re-orthonormalised; the polar factor comes from Newton's
// iteration W <- (W + W^{-+}) / 2 (N. J. Higham, SIAM J. Sci. Stat. Comput.
// 7 (1986) 1160), run to a relative step of 1e-15.
//
// Gaussian step (qcd_gaussIteration3d, lib/src/qcd_smearing.c:25-113): on
// time-slice t, v <- (v + alpha H v) / (1 + 6 alpha) with
//   H v(x) = sum_{nu=1..3} U_nu(x) v(x+nu) + U_nu(x-nu)^+ v(x-nu);
// other time-slices are unchanged. One thread per site of the slice, FP64.
#include <math.h>

#include "su3.cuh"

namespace qg {

__device__ __forceinline__ void m3dag(const C<double> a[9], C<double> r[9])
{
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) r[3 * i + j] = conj(a[3 * j + i]);
}

__device__ __forceinline__ C<double> m3det(const C<double> m[9])
{
  C<double> d = m[0] * (m[4] * m[8] - m[5] * m[7]);
  d = d - m[1] * (m[3] * m[8] - m[5] * m[6]);
  return d + m[2] * (m[3] * m[7] - m[4] * m[6]);
}

// r = (m^{-1})^+ by cofactors
__device__ __forceinline__ void m3inv_dag(const C<double> m[9], C<double> r[9])
{
  const C<double> d = m3det(m);
  const double dd = d.re * d.re + d.im * d.im;
  const C<double> id{d.re / dd, -d.im / dd};
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int i1 = (j + 1) % 3, i2 = (j + 2) % 3, j1 = (i + 1) % 3, j2 = (i + 2) % 3;
      const C<double> cof = m[3 * i1 + j1] * m[3 * i2 + j2] - m[3 * i1 + j2] * m[3 * i2 + j1];
      r[3 * j + i] = conj(cof * id);  // (m^{-1})_{ij} = cof_ij / det, stored transposed and conjugated
    }
}

__device__ void project_su3(C<double> W[9])
{
  const C<double> d = m3det(W);
  const double phase = atan2(d.im, d.re) / 3.0;
  for (int it = 0; it < 100; it++) {
    C<double> Wi[9];
    m3inv_dag(W, Wi);
    double diff = 0, nrm = 0;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      const C<double> nw{0.5 * (W[k].re + Wi[k].re), 0.5 * (W[k].im + Wi[k].im)};
      diff += fabs(nw.re - W[k].re) + fabs(nw.im - W[k].im);
      nrm += fabs(nw.re) + fabs(nw.im);
      W[k] = nw;
    }
    if (diff <= 1e-15 * nrm) break;
  }
  double s, c;
  sincos(phase, &s, &c);
  const C<double> ph{c, -s};
#pragma unroll
  for (int k = 0; k < 9; k++) W[k] = W[k] * ph;
  reunit_cols(W);
}

__device__ __forceinline__ void load_link(const double2 *u, int64_t stride, int x, int mu, C<double> U[9])
{
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const double2 v = __ldg(u + ((int64_t)mu * 9 + k) * stride + x);
    U[k] = C<double>{v.x, v.y};
  }
}

__global__ void __launch_bounds__(128) k_ape3d(double2 *out, const double2 *in, int64_t stride, Geom geo, int V,
                                               double alpha)
{
  const int x = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (x >= V) return;
  int c[4];
  coords(geo, x, c);
#pragma unroll
  for (int k = 0; k < 9; k++) out[(int64_t)k * stride + x] = in[(int64_t)k * stride + x];
  for (int mu = 1; mu < 4; mu++) {
    C<double> S[9];
#pragma unroll
    for (int k = 0; k < 9; k++) S[k] = C<double>{0.0, 0.0};
    for (int nu = 1; nu < 4; nu++) {
      if (nu == mu) continue;
      C<double> A[9], B[9], T[9], Bd[9];
      // U_nu(x) U_mu(x+nu) U_nu(x+mu)^+
      load_link(in, stride, x, nu, A);
      load_link(in, stride, fwd(geo, x, c, nu), mu, B);
      m3mul(A, B, T);
      load_link(in, stride, fwd(geo, x, c, mu), nu, B);
      m3dag(B, Bd);
      m3mul(T, Bd, A);
#pragma unroll
      for (int k = 0; k < 9; k++) S[k] = S[k] + A[k];
      // U_nu(x-nu)^+ U_mu(x-nu) U_nu(x-nu+mu)
      const int b = bwd(geo, x, c, nu);
      int cb[4];
      coords(geo, b, cb);
      load_link(in, stride, b, nu, A);
      m3dag(A, Bd);
      load_link(in, stride, b, mu, B);
      m3mul(Bd, B, T);
      load_link(in, stride, fwd(geo, b, cb, mu), nu, B);
      m3mul(T, B, A);
#pragma unroll
      for (int k = 0; k < 9; k++) S[k] = S[k] + A[k];
    }
    C<double> U[9];
    load_link(in, stride, x, mu, U);
#pragma unroll
    for (int k = 0; k < 9; k++) U[k] = C<double>{U[k].re + alpha * S[k].re, U[k].im + alpha * S[k].im};
    project_su3(U);
#pragma unroll
    for (int k = 0; k < 9; k++) out[((int64_t)mu * 9 + k) * stride + x] = make_double2(U[k].re, U[k].im);
  }
}

// out = (in + alpha H in) / (1 + 6 alpha) on the sites of time-slice t
__global__ void __launch_bounds__(128) k_gauss3d(double2 *out, const double2 *in, int64_t fstride,
                                                 const double2 *u, int64_t gstride, Geom geo, int V3, int t,
                                                 double alpha, double nrm)
{
  const int s = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (s >= V3) return;
  const int x = t + geo.L[0] * s;
  int c[4];
  coords(geo, x, c);
  C<double> h[12];
#pragma unroll
  for (int k = 0; k < 12; k++) h[k] = C<double>{0.0, 0.0};
  for (int nu = 1; nu < 4; nu++) {
    C<double> U[9];
    const int y = fwd(geo, x, c, nu);
    load_link(u, gstride, x, nu, U);
#pragma unroll
    for (int sp = 0; sp < 4; sp++) {
      C<double> p[3];
#pragma unroll
      for (int b = 0; b < 3; b++) {
        const double2 v = in[(int64_t)(3 * sp + b) * fstride + y];
        p[b] = C<double>{v.x, v.y};
      }
#pragma unroll
      for (int a = 0; a < 3; a++) h[3 * sp + a] = h[3 * sp + a] + U[3 * a] * p[0] + U[3 * a + 1] * p[1] + U[3 * a + 2] * p[2];
    }
    const int z = bwd(geo, x, c, nu);
    load_link(u, gstride, z, nu, U);
#pragma unroll
    for (int sp = 0; sp < 4; sp++) {
      C<double> p[3];
#pragma unroll
      for (int b = 0; b < 3; b++) {
        const double2 v = in[(int64_t)(3 * sp + b) * fstride + z];
        p[b] = C<double>{v.x, v.y};
      }
#pragma unroll
      for (int a = 0; a < 3; a++)
        h[3 * sp + a] = h[3 * sp + a] + cdot(U[a], p[0]) + cdot(U[3 + a], p[1]) + cdot(U[6 + a], p[2]);
    }
  }
#pragma unroll
  for (int k = 0; k < 12; k++) {
    const double2 v = in[(int64_t)k * fstride + x];
    out[(int64_t)k * fstride + x] = make_double2((v.x + alpha * h[k].re) * nrm, (v.y + alpha * h[k].im) * nrm);
  }
}

static Geom make_geom(const int L[4])
{
  Geom g;
  for (int i = 0; i < 4; i++) g.L[i] = L[i];
  g.st[0] = 1;
  g.st[1] = L[0];
  g.st[2] = L[0] * L[1];
  g.st[3] = L[0] * L[1] * L[2];
  return g;
}

static bool same_lattice(qcdgpu_gauge a, qcdgpu_gauge b)
{
  return a->L[0] == b->L[0] && a->L[1] == b->L[1] && a->L[2] == b->L[2] && a->L[3] == b->L[3];
}

// one APE step out <- in (FP64 fields, out != in)
bool ape3d(qcdgpu_gauge out, qcdgpu_gauge in, double alpha)
{
  if (!out || !in || out == in || out->prec != QCDGPU_F64 || in->prec != QCDGPU_F64 || !same_lattice(out, in)) {
    set_error("APE smearing: two distinct FP64 gauge fields on the same lattice");
    return false;
  }
  const unsigned nb = (unsigned)((in->V + 127) / 128);
  k_ape3d<<<nb, 128, 0, stream()>>>((double2 *)out->data, (const double2 *)in->data, in->stride,
                                    make_geom(in->L), (int)in->V, alpha);
  if (!QG_LAUNCHED("ape3d")) return false;
  out->recon = 12;  // SU(3) by construction
  gauge_forget(out);
  return true;
}

// n Gaussian steps of v on time-slice t with links g
bool gauss3d(qcdgpu_field v, qcdgpu_gauge g, double alpha, int t, int n)
{
  if (!v || !g || v->prec != QCDGPU_F64 || g->prec != QCDGPU_F64 || v->V != g->V ||
      memcmp(v->L, g->L, sizeof(v->L)) != 0 || t < 0 || t >= v->L[0] || n < 0) {
    set_error("Gaussian smearing: FP64 field and gauge on one lattice, 0 <= t < L_t, n >= 0");
    return false;
  }
  if (n == 0) return true;
  qcdgpu_field w = work_get(v->L, QCDGPU_F64);
  if (!w) return false;
  bool ok = blas_copy(w, v);
  const int V3 = (int)(v->V / v->L[0]);
  const unsigned nb = (unsigned)((V3 + 127) / 128);
  const Geom geo = make_geom(v->L);
  const double nrm = 1.0 / (1.0 + 6.0 * alpha);
  qcdgpu_field a = v, b = w;  // a holds the current value
  for (int i = 0; ok && i < n; i++) {
    k_gauss3d<<<nb, 128, 0, stream()>>>((double2 *)b->data, (const double2 *)a->data, v->stride,
                                        (const double2 *)g->data, g->stride, geo, V3, t, alpha, nrm);
    ok = QG_LAUNCHED("gauss3d");
    qcdgpu_field tmp = a;
    a = b;
    b = tmp;
  }
  if (ok && a != v) ok = blas_copy(v, a);
  work_put(w);
  return ok;
}

bool ape3d_steps(qcdgpu_gauge out, qcdgpu_gauge in, double alpha, int n)
{
  if (!out || !in || out == in || n < 1) {
    set_error("APE smearing: distinct fields and n >= 1");
    return false;
  }
  if (n == 1) return ape3d(out, in, alpha);
  qcdgpu_gauge w = gauge_new(in->L, in->theta, QCDGPU_F64, 18);
  if (!w) return false;
  // ping-pong so that the last step writes `out`
  qcdgpu_gauge src = in;
  bool ok = true;
  for (int i = 0; ok && i < n; i++) {
    qcdgpu_gauge dst = ((n - 1 - i) % 2 == 0) ? out : w;
    ok = ape3d(dst, src, alpha);
    src = dst;
  }
  if (!QG_CUDA(cudaStreamSynchronize(stream()))) ok = false;
  gauge_forget(w);
  gauge_free(w);
  return ok;
}

}  // namespace qg

extern "C" {

int qcdgpu_gauge_ape3d(qcdgpu_gauge out, qcdgpu_gauge in, double alpha, int n)
{
  return qg::ape3d_steps(out, in, alpha, n) ? 0 : 1;
}

int qcdgpu_field_gauss3d(qcdgpu_field v, qcdgpu_gauge g, double alpha, int t, int n)
{
  return qg::gauss3d(v, g, alpha, t, n) ? 0 : 1;
}

int qcdgpu_smeared_source(qcdgpu_field f, qcdgpu_gauge g, const int x[4], int spin, int colour, double ape_alpha,
                          int ape_n, double gauss_alpha, int gauss_n)
{
  if (!f || !g || f->prec != QCDGPU_F64) {
    qg::set_error("smeared source: FP64 field and gauge field");
    return 1;
  }
  if (!qg::field_point(f, x, spin, colour)) return 1;
  if (gauss_n == 0) return 0;
  qcdgpu_gauge ga = g;
  if (ape_n > 0) {
    ga = qg::gauge_new(g->L, g->theta, QCDGPU_F64, 18);
    if (!ga) return 1;
    if (!qg::ape3d_steps(ga, g, ape_alpha, ape_n)) {
      qg::gauge_free(ga);
      return 1;
    }
  }
  bool ok = qg::gauss3d(f, ga, gauss_alpha, x[0], gauss_n);
  if (ga != g) {
    if (!QG_CUDA(cudaStreamSynchronize(qg::stream()))) ok = false;
    qg::gauge_forget(ga);
    qg::gauge_free(ga);
  }
  return ok ? 0 : 1;
}

}  // extern "C"
