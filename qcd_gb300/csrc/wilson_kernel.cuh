// wilson_kernel.cuh -- the operator kernel template, shared by the native
// (double / float) and the float-float instantiations.
//
// One thread per site. Each of the eight neighbour spinors is projected to a
// two-spin half spinor straight after its load, multiplied by the link,
// phased when theta_mu != 0, and expanded back into the 4-spin accumulator
// (projectors of the chiral basis, qcd_wilson.h:17-387). Links arrive as 12
// reals (third row rebuilt) when the field is SU(3). R is the arithmetic
// type: any type with +, -, * and unary - and conversions from/to double.
#pragma once

#include "dslash_args.h"

namespace qg {

using namespace qgd;

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

// acc += sc (1 + S g_mu) spinor rebuilt from its upper half h: the same as
// accumulate<MU, S> applied to sc h, with the scale folded into the
// multiply-adds
template <int MU, int S>
__device__ __forceinline__ void accumulate_scaled(C<float> acc[12], const C<float> h[6], float sc)
{
  const float p = S > 0 ? sc : -sc;  // sign of the rebuilt lower spins' terms
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const C<float> h0 = h[c], h1 = h[3 + c];
    acc[c] = C<float>{qfma(sc, h0.re, acc[c].re), qfma(sc, h0.im, acc[c].im)};
    acc[3 + c] = C<float>{qfma(sc, h1.re, acc[3 + c].re), qfma(sc, h1.im, acc[3 + c].im)};
    if (MU == 0) {  // -S h0, -S h1
      acc[6 + c] = C<float>{qfma(-p, h0.re, acc[6 + c].re), qfma(-p, h0.im, acc[6 + c].im)};
      acc[9 + c] = C<float>{qfma(-p, h1.re, acc[9 + c].re), qfma(-p, h1.im, acc[9 + c].im)};
    } else if (MU == 1) {  // S i h1, S i h0
      acc[6 + c] = C<float>{qfma(-p, h1.im, acc[6 + c].re), qfma(p, h1.re, acc[6 + c].im)};
      acc[9 + c] = C<float>{qfma(-p, h0.im, acc[9 + c].re), qfma(p, h0.re, acc[9 + c].im)};
    } else if (MU == 2) {  // S h1, -S h0
      acc[6 + c] = C<float>{qfma(p, h1.re, acc[6 + c].re), qfma(p, h1.im, acc[6 + c].im)};
      acc[9 + c] = C<float>{qfma(-p, h0.re, acc[9 + c].re), qfma(-p, h0.im, acc[9 + c].im)};
    } else {  // S i h0, -S i h1
      acc[6 + c] = C<float>{qfma(-p, h0.im, acc[6 + c].re), qfma(p, h0.re, acc[6 + c].im)};
      acc[9 + c] = C<float>{qfma(p, h1.im, acc[9 + c].re), qfma(-p, h1.re, acc[9 + c].im)};
    }
  }
}

// h = upper half of (1 + S g_mu) s for the spinor s at index y: any storage
// loads the twelve components, then projects. kScaled: h is returned
// without the site's norm, which comes back in sc for the accumulation.
template <int MU, int S, int SP, typename R>
struct LoadProject {
  static constexpr bool kScaled = false;
  __device__ __forceinline__ static void run(const void *base, const float *norm, int64_t stride, int64_t y,
                                             C<R> h[6], float &sc)
  {
    C<R> s[12];
    Spinor<SP, R>::load(base, norm, stride, y, s);
    project<MU, S>(s, h);
    sc = 1.0f;
  }
};

// a + sg b (IM: a + sg i b) on packed (re, im) half pairs
template <bool IM>
__device__ __forceinline__ __half2 hcomb(__half2 a, __half2 b, int sg)
{
  if (IM) return __hfma2(__lowhigh2highlow(b), sg > 0 ? __floats2half2_rn(-1.f, 1.f) : __floats2half2_rn(1.f, -1.f), a);
  return sg > 0 ? __hadd2(a, b) : __hsub2(a, b);
}

// FP16 storage (component k = 3 spin + colour is the k-th (re, im) half pair
// of the site's three 16-byte words): the projection adds the stored half
// pairs directly (one FP16 rounding per projected component, below the
// storage's own 2^-11), and only the six projected components are converted
// -- half the conversions of decoding all twelve (measured: 57.4 -> 54.0 us
// per 24^3x48 apply). The site norm is applied in the accumulation
// (accumulate_scaled), not to the six components.
template <int MU, int S>
struct LoadProject<MU, S, QCDGPU_F16, float> {
  static constexpr bool kScaled = true;
  __device__ __forceinline__ static void run(const void *base, const float *norm, int64_t stride, int64_t y,
                                             C<float> h[6], float &sc)
  {
    const uint4 *p = (const uint4 *)base + y;
    sc = __ldg(norm + y);
    uint4 w[3];
#pragma unroll
    for (int j = 0; j < 3; j++) w[j] = __ldg(p + j * stride);
    const __half2 *hv = reinterpret_cast<const __half2 *>(w);
    constexpr bool IM = MU & 1;
    // partner spins and signs of the two projected halves (as in project())
    constexpr int B0 = (MU == 0 || MU == 3) ? 2 : 3, B1 = 5 - B0;
    constexpr int SG0 = S > 0 ? -1 : 1, SG1 = MU < 2 ? SG0 : -SG0;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float2 f0 = __half22float2(hcomb<IM>(hv[c], hv[3 * B0 + c], SG0));
      const float2 f1 = __half22float2(hcomb<IM>(hv[3 + c], hv[3 * B1 + c], SG1));
      h[c] = C<float>{f0.x, f0.y};
      h[3 + c] = C<float>{f1.x, f1.y};
    }
  }
};

template <int MU, bool DAG, int SP, int GP, int RECON, typename R, bool EO = false>
__device__ __forceinline__ void hop_pair(const DArgs &a, int x, const int c[4], C<R> acc[12])
{
  constexpr int SF = DAG ? +1 : -1;  // projector sign of the forward hop
  const bool twisted = (a.twist_mask >> MU) & 1;
  {
    int y = fwd(a.geo, x, c, MU);
    C<R> h[6], uh[6], U[9];
    float sc;
    LoadProject<MU, SF, SP, R>::run(a.in, a.in_norm, a.stride, EO ? (y >> 1) : y, h, sc);
    Link<GP, RECON, R>::load(a.gauge, a.gstride, x, MU, U);
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
      for (int i = 0; i < 3; i++)
        uh[3 * j + i] = cmadd(U[3 * i + 2], h[3 * j + 2], cmadd(U[3 * i + 1], h[3 * j + 1], U[3 * i] * h[3 * j]));
    if (twisted) {
      C<R> ph{Scalar<R>::get(a.phr[MU], a.phr_h[MU], a.phr_l[MU]), Scalar<R>::get(a.phi[MU], a.phi_h[MU], a.phi_l[MU])};
#pragma unroll
      for (int k = 0; k < 6; k++) uh[k] = uh[k] * ph;
    }
    if constexpr (LoadProject<MU, SF, SP, R>::kScaled) accumulate_scaled<MU, SF>(acc, uh, sc);
    else accumulate<MU, SF>(acc, uh);
  }
  {
    int y = bwd(a.geo, x, c, MU);
    C<R> h[6], uh[6], U[9];
    float sc;
    LoadProject<MU, -SF, SP, R>::run(a.in, a.in_norm, a.stride, EO ? (y >> 1) : y, h, sc);
    Link<GP, RECON, R>::load(a.gauge, a.gstride, y, MU, U);
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
      for (int i = 0; i < 3; i++)
        uh[3 * j + i] = cmadd_conj(U[6 + i], h[3 * j + 2], cmadd_conj(U[3 + i], h[3 * j + 1], cdot(U[i], h[3 * j])));
    if (twisted) {
      C<R> ph{Scalar<R>::get(a.phr[MU], a.phr_h[MU], a.phr_l[MU]), -Scalar<R>::get(a.phi[MU], a.phi_h[MU], a.phi_l[MU])};
#pragma unroll
      for (int k = 0; k < 6; k++) uh[k] = uh[k] * ph;
    }
    if constexpr (LoadProject<MU, -SF, SP, R>::kScaled) accumulate_scaled<MU, -SF>(acc, uh, sc);
    else accumulate<MU, -SF>(acc, uh);
  }
}

// FP32 / FP16 storage: registers capped for seven blocks per SM (72; 80
// uncapped), measured at 24^3x48: FP16 48.9 -> 47.1 us, FP32 57.3 -> 55.3 us
// per apply (a cap of 64 spills and loses). The even/odd kernel below keeps
// the uncapped form, which solves 0.7 % faster.
template <bool DAG, int SP, int GP, int RECON, typename R>
__global__ void __launch_bounds__(128, SP != QCDGPU_F64 ? 7 : 1) k_wilson(const DArgs a)
{
  int x = a.x0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  double n2 = 0.0;
  if (x < a.V) {
    int c[4];
    coords(a.geo, x, c);
    C<R> acc[12];
    const R zero = Scalar<R>::get(0.0, 0.0f, 0.0f);
#pragma unroll
    for (int k = 0; k < 12; k++) acc[k] = C<R>{zero, zero};
    hop_pair<0, DAG, SP, GP, RECON, R>(a, x, c, acc);
    hop_pair<1, DAG, SP, GP, RECON, R>(a, x, c, acc);
    hop_pair<2, DAG, SP, GP, RECON, R>(a, x, c, acc);
    hop_pair<3, DAG, SP, GP, RECON, R>(a, x, c, acc);
    C<R> s[12];
    Spinor<SP, R>::load(a.in, a.in_norm, a.stride, x, s);
    const R mp4 = Scalar<R>::get(a.mp4, a.mp4_h, a.mp4_l), tm = Scalar<R>::get(a.tm, a.tm_h, a.tm_l);
    const R half = Scalar<R>::get(0.5, 0.5f, 0.0f);
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
    if (a.partials) {
      // per-site sum in the working precision (FP64 arithmetic is scarce on
      // this part); the block sum is double
      R s2 = acc[0].re * acc[0].re + acc[0].im * acc[0].im;
#pragma unroll
      for (int k = 1; k < 12; k++) s2 = s2 + acc[k].re * acc[k].re + acc[k].im * acc[k].im;
      n2 = (double)s2;
    }
  }
  if (a.partials) block_partial_cg(n2, a);
}

// Even/odd kernel: thread e handles the site of parity a.eo_par whose full
// index is 2e or 2e + 1 (the t extent is even, so the two sites 2e, 2e + 1
// of a t-row have opposite parities); neighbours are read from the half
// field of the other parity at (full index) >> 1.
template <bool DAG, int SP, int GP, int RECON, typename R>
__global__ void __launch_bounds__(128) k_wilson_eo(const DArgs a)
{
  const int e = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  double n2 = 0.0;
  if (e < a.V) {
    int c[4];
    coords(a.geo, 2 * e, c);
    const int b = (a.eo_par ^ c[1] ^ c[2] ^ c[3]) & 1;
    const int x = 2 * e + b;
    c[0] += b;
    C<R> acc[12];
    const R zero = Scalar<R>::get(0.0, 0.0f, 0.0f);
#pragma unroll
    for (int k = 0; k < 12; k++) acc[k] = C<R>{zero, zero};
    hop_pair<0, DAG, SP, GP, RECON, R, true>(a, x, c, acc);
    hop_pair<1, DAG, SP, GP, RECON, R, true>(a, x, c, acc);
    hop_pair<2, DAG, SP, GP, RECON, R, true>(a, x, c, acc);
    hop_pair<3, DAG, SP, GP, RECON, R, true>(a, x, c, acc);
    const R ch = Scalar<R>::get(a.ch, a.ch_h, a.ch_l);
    if (a.ainv) {  // ch A^{-1}: the scale folded into the coefficients
      const R ar = ch * Scalar<R>::get(a.ai_r, a.ai_r_h, a.ai_r_l), ai = ch * Scalar<R>::get(a.ai_i, a.ai_i_h, a.ai_i_l);
#pragma unroll
      for (int k = 0; k < 12; k++) {
        const R g5ai = k < 6 ? ai : -ai;
        acc[k] = C<R>{ar * acc[k].re - g5ai * acc[k].im, ar * acc[k].im + g5ai * acc[k].re};
      }
    } else if (!a.zmode) {
#pragma unroll
      for (int k = 0; k < 12; k++) acc[k] = C<R>{ch * acc[k].re, ch * acc[k].im};
    }
    if (a.zmode) {
      C<R> s[12];
      Spinor<SP, R>::load(a.z, a.z_norm, a.stride, e, s);
      if (a.zmode == 2) {
        const R mp4 = Scalar<R>::get(a.mp4, a.mp4_h, a.mp4_l), tm = Scalar<R>::get(a.tm, a.tm_h, a.tm_l);
#pragma unroll
        for (int k = 0; k < 12; k++) {
          const R g5tm = k < 6 ? tm : -tm;
          s[k] = C<R>{mp4 * s[k].re - g5tm * s[k].im, mp4 * s[k].im + g5tm * s[k].re};
        }
      }
      if (a.ainv) {
#pragma unroll
        for (int k = 0; k < 12; k++) acc[k] = acc[k] + s[k];
      } else {  // ch H in + z as one multiply-add per real
#pragma unroll
        for (int k = 0; k < 12; k++) acc[k] = C<R>{qfma(ch, acc[k].re, s[k].re), qfma(ch, acc[k].im, s[k].im)};
      }
    }
    Spinor<SP, R>::store(a.out, a.out_norm, a.stride, e, acc);
    if (a.partials) {
      R s2 = acc[0].re * acc[0].re + acc[0].im * acc[0].im;
#pragma unroll
      for (int k = 1; k < 12; k++) s2 = s2 + acc[k].re * acc[k].re + acc[k].im * acc[k].im;
      n2 = (double)s2;
    }
  }
  if (a.partials) block_partial_cg(n2, a);
}

}  // namespace qg
