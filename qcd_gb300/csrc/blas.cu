// blas.cu -- BLAS-1 and reductions on device spinor fields
// (qcd_blas.c:137-492: zero, set, copy, scale, mulC, add, sub, axpy, the
// complex dot <a,b> = sum conj(a) b and the 2-norm).
//
// Kernels work one site per thread through the precision accessors, so the
// same code serves FP64, FP32 and FP16(+norm) storage. Reductions accumulate
// in double: each block reduces with warp shuffles into one partial, and a
// single block sums the partials in a fixed order, so results do not depend
// on scheduling (the reference's MPI_Allreduce becomes this second pass).
#include <string.h>

#include <complex>

#include "internal.h"

namespace qg {

using namespace qgd;

static inline unsigned grid_sites(int64_t V) { return (unsigned)((V + 127) / 128); }

// -------------------------------------------------------------- elementwise
template <int P, typename R>
__global__ void k_axpby(void *out, float *onorm, R ar, R ai, const void *x, const float *xn, R br,
                        R bi, const void *y, const float *yn, int64_t stride, int64_t V)
{
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= V) return;
  C<R> a{ar, ai}, b{br, bi}, vx[12], vy[12];
  Spinor<P, R>::load(x, xn, stride, s, vx);
  Spinor<P, R>::load(y, yn, stride, s, vy);
#pragma unroll
  for (int k = 0; k < 12; k++) vx[k] = a * vx[k] + b * vy[k];
  Spinor<P, R>::store(out, onorm, stride, s, vx);
}

// out = a x + b y with real a, b: b y + x (a = 1: exact for b = +-1) or
// b y + (a x); one or two FP64 operations per real instead of the complex
// form's six (GB300's FP64 pipe, not HBM, bounds the complex form)
template <int P, typename R>
__global__ void k_axpby_real(void *out, float *onorm, R a, const void *x, const float *xn, R b, const void *y,
                             const float *yn, int64_t stride, int64_t V)
{
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= V) return;
  C<R> vx[12], vy[12];
  Spinor<P, R>::load(x, xn, stride, s, vx);
  Spinor<P, R>::load(y, yn, stride, s, vy);
  const bool unit = a == (R)1;
#pragma unroll
  for (int k = 0; k < 12; k++) {
    const R xr = unit ? vx[k].re : a * vx[k].re, xi = unit ? vx[k].im : a * vx[k].im;
    vx[k].re = qfma(b, vy[k].re, xr);
    vx[k].im = qfma(b, vy[k].im, xi);
  }
  Spinor<P, R>::store(out, onorm, stride, s, vx);
}

// y = a x + y with real a: one fused multiply-add per real
template <int P, typename R>
__global__ void k_axpy_real(void *y, float *yn, R a, const void *x, const float *xn, int64_t stride,
                            int64_t V)
{
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= V) return;
  C<R> vx[12], vy[12];
  Spinor<P, R>::load(x, xn, stride, s, vx);
  Spinor<P, R>::load(y, yn, stride, s, vy);
#pragma unroll
  for (int k = 0; k < 12; k++) {
    vy[k].re = qfma(a, vx[k].re, vy[k].re);
    vy[k].im = qfma(a, vx[k].im, vy[k].im);
  }
  Spinor<P, R>::store(y, yn, stride, s, vy);
}

template <int P, typename R>
__global__ void k_set(void *out, float *onorm, R cr, R ci, int64_t stride, int64_t V)
{
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= V) return;
  C<R> v[12];
#pragma unroll
  for (int k = 0; k < 12; k++) v[k] = C<R>{cr, ci};
  Spinor<P, R>::store(out, onorm, stride, s, v);
}

// mode 0: g5 in ; mode 1: i g5 in
template <int P, typename R>
__global__ void k_g5(void *out, float *onorm, const void *in, const float *inorm, int mode,
                     int64_t stride, int64_t V)
{
  int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= V) return;
  C<R> v[12];
  Spinor<P, R>::load(in, inorm, stride, s, v);
#pragma unroll
  for (int k = 0; k < 12; k++) {
    C<R> w = mode ? mul_i(v[k]) : v[k];
    v[k] = k < 6 ? w : -w;
  }
  Spinor<P, R>::store(out, onorm, stride, s, v);
}

// --------------------------------------------------------------- reductions
__device__ __forceinline__ double warp_sum(double v)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-level sum of (v0, v1) into partials[2*blockIdx.x + {0,1}]
__device__ __forceinline__ void block_sum2(double v0, double v1, double *partials)
{
  __shared__ double sh[2][32];
  v0 = warp_sum(v0);
  v1 = warp_sum(v1);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = v0;
    sh[1][w] = v1;
  }
  __syncthreads();
  if (w == 0) {
    int nw = blockDim.x >> 5;
    v0 = l < nw ? sh[0][l] : 0.0;
    v1 = l < nw ? sh[1][l] : 0.0;
    v0 = warp_sum(v0);
    v1 = warp_sum(v1);
    if (l == 0) {
      partials[2 * blockIdx.x] = v0;
      partials[2 * blockIdx.x + 1] = v1;
    }
  }
}

// kind 0: |a|^2 ; kind 1: <a,b> ; kind 2: b = b + (ar,ai) a, then |b|^2
template <int P, typename R, int KIND>
__global__ void __launch_bounds__(256) k_reduce(const void *a, const float *an, void *b, float *bn,
                                                R ar, R ai, int64_t stride, int64_t V, double *partials)
{
  double s0 = 0, s1 = 0;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < V;
       s += (int64_t)gridDim.x * blockDim.x) {
    C<R> va[12];
    Spinor<P, R>::load(a, an, stride, s, va);
    // FP64 fields: FP64 products and sums; FP32 / FP16 fields: the site's
    // twelve terms in FP32 (their own precision), the sum over sites in FP64
    // (FP64 arithmetic per component would make these kernels FP64-pipe bound)
    constexpr bool F = sizeof(R) == 4;
    if (KIND == 0) {
      if (F) {
        R t = (R)0;
#pragma unroll
        for (int k = 0; k < 12; k++) t += va[k].re * va[k].re + va[k].im * va[k].im;
        s0 += (double)t;
      } else {
#pragma unroll
        for (int k = 0; k < 12; k++) s0 += (double)va[k].re * va[k].re + (double)va[k].im * va[k].im;
      }
    } else if (KIND == 1) {
      C<R> vb[12];
      Spinor<P, R>::load(b, bn, stride, s, vb);
      if (F) {
        R t0 = (R)0, t1 = (R)0;
#pragma unroll
        for (int k = 0; k < 12; k++) {
          t0 += va[k].re * vb[k].re + va[k].im * vb[k].im;
          t1 += va[k].re * vb[k].im - va[k].im * vb[k].re;
        }
        s0 += (double)t0;
        s1 += (double)t1;
      } else {
#pragma unroll
        for (int k = 0; k < 12; k++) {
          s0 += (double)va[k].re * vb[k].re + (double)va[k].im * vb[k].im;
          s1 += (double)va[k].re * vb[k].im - (double)va[k].im * vb[k].re;
        }
      }
    } else {
      C<R> vb[12], c{ar, ai};
      Spinor<P, R>::load(b, bn, stride, s, vb);
      R t = (R)0;
#pragma unroll
      for (int k = 0; k < 12; k++) {
        vb[k] = vb[k] + c * va[k];
        if (F) t += vb[k].re * vb[k].re + vb[k].im * vb[k].im;
        else s0 += (double)vb[k].re * vb[k].re + (double)vb[k].im * vb[k].im;
      }
      if (F) s0 += (double)t;
      Spinor<P, R>::store(b, bn, stride, s, vb);
    }
  }
  block_sum2(s0, s1, partials);
}

// one block: res[0..1] = sum of n partial pairs, in index order per lane
__global__ void k_finalize(const double *partials, int n, double *res)
{
  double v0 = 0, v1 = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    v0 += partials[2 * i];
    v1 += partials[2 * i + 1];
  }
  __shared__ double sh[2][32];
  v0 = warp_sum(v0);
  v1 = warp_sum(v1);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = v0;
    sh[1][w] = v1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
      a += sh[0][i];
      b += sh[1][i];
    }
    res[0] = a;
    res[1] = b;
  }
}

static int reduce_blocks(int64_t V)
{
  int64_t n = (V + 255) / 256;
  return (int)(n < kMaxPartials ? n : kMaxPartials);
}

// --------------------------------------------------------------- dispatch
#define QG_DISPATCH(prec, F64CALL, F32CALL, F16CALL) \
  do {                                               \
    if ((prec) == QCDGPU_F64) { F64CALL; }           \
    else if ((prec) == QCDGPU_F32) { F32CALL; }      \
    else { F16CALL; }                                \
  } while (0)

bool blas_zero(qcdgpu_field x) { return QG_CUDA(cudaMemsetAsync(x->data, 0, x->bytes, stream())); }

bool blas_copy(qcdgpu_field d, qcdgpu_field s)
{
  if (!same_shape(d, s) || d->prec != s->prec) {
    set_error("copy: fields differ in shape or precision");
    return false;
  }
  if (d == s) return true;
  return QG_CUDA(cudaMemcpyAsync(d->data, s->data, d->bytes, cudaMemcpyDeviceToDevice, stream()));
}

bool blas_axpby(qcdgpu_field out, double ar, double ai, qcdgpu_field x, double br, double bi, qcdgpu_field y)
{
  if (!same_shape(out, x) || !same_shape(out, y) || out->prec != x->prec || out->prec != y->prec) {
    set_error("axpby: fields differ in shape or precision");
    return false;
  }
  unsigned g = grid_sites(out->V);
  cudaStream_t st = stream();
  if (ai == 0.0 && br == 1.0 && bi == 0.0 && out == y) {
    QG_DISPATCH(out->prec,
                (k_axpy_real<QCDGPU_F64, double><<<g, 128, 0, st>>>(y->data, y->norm, ar, x->data, x->norm, out->stride, out->V)),
                (k_axpy_real<QCDGPU_F32, float><<<g, 128, 0, st>>>(y->data, y->norm, (float)ar, x->data, x->norm, out->stride, out->V)),
                (k_axpy_real<QCDGPU_F16, float><<<g, 128, 0, st>>>(y->data, y->norm, (float)ar, x->data, x->norm, out->stride, out->V)));
    return QG_LAUNCHED("axpy_real");
  }
  if (ai == 0.0 && bi == 0.0) {
    QG_DISPATCH(out->prec,
                (k_axpby_real<QCDGPU_F64, double><<<g, 128, 0, st>>>(out->data, out->norm, ar, x->data, x->norm, br, y->data, y->norm, out->stride, out->V)),
                (k_axpby_real<QCDGPU_F32, float><<<g, 128, 0, st>>>(out->data, out->norm, (float)ar, x->data, x->norm, (float)br, y->data, y->norm, out->stride, out->V)),
                (k_axpby_real<QCDGPU_F16, float><<<g, 128, 0, st>>>(out->data, out->norm, (float)ar, x->data, x->norm, (float)br, y->data, y->norm, out->stride, out->V)));
    return QG_LAUNCHED("axpby_real");
  }
  QG_DISPATCH(out->prec,
              (k_axpby<QCDGPU_F64, double><<<g, 128, 0, st>>>(out->data, out->norm, ar, ai, x->data, x->norm, br, bi, y->data, y->norm, out->stride, out->V)),
              (k_axpby<QCDGPU_F32, float><<<g, 128, 0, st>>>(out->data, out->norm, (float)ar, (float)ai, x->data, x->norm, (float)br, (float)bi, y->data, y->norm, out->stride, out->V)),
              (k_axpby<QCDGPU_F16, float><<<g, 128, 0, st>>>(out->data, out->norm, (float)ar, (float)ai, x->data, x->norm, (float)br, (float)bi, y->data, y->norm, out->stride, out->V)));
  return QG_LAUNCHED("axpby");
}

bool blas_set(qcdgpu_field x, double cr, double ci)
{
  unsigned g = grid_sites(x->V);
  cudaStream_t st = stream();
  QG_DISPATCH(x->prec,
              (k_set<QCDGPU_F64, double><<<g, 128, 0, st>>>(x->data, x->norm, cr, ci, x->stride, x->V)),
              (k_set<QCDGPU_F32, float><<<g, 128, 0, st>>>(x->data, x->norm, (float)cr, (float)ci, x->stride, x->V)),
              (k_set<QCDGPU_F16, float><<<g, 128, 0, st>>>(x->data, x->norm, (float)cr, (float)ci, x->stride, x->V)));
  return QG_LAUNCHED("set");
}

static bool g5_common(qcdgpu_field out, qcdgpu_field in, int mode)
{
  if (!same_shape(out, in) || out->prec != in->prec) {
    set_error("gamma5: fields differ in shape or precision");
    return false;
  }
  unsigned g = grid_sites(out->V);
  cudaStream_t st = stream();
  QG_DISPATCH(out->prec,
              (k_g5<QCDGPU_F64, double><<<g, 128, 0, st>>>(out->data, out->norm, in->data, in->norm, mode, out->stride, out->V)),
              (k_g5<QCDGPU_F32, float><<<g, 128, 0, st>>>(out->data, out->norm, in->data, in->norm, mode, out->stride, out->V)),
              (k_g5<QCDGPU_F16, float><<<g, 128, 0, st>>>(out->data, out->norm, in->data, in->norm, mode, out->stride, out->V)));
  return QG_LAUNCHED("gamma5");
}
bool blas_gamma5(qcdgpu_field out, qcdgpu_field in) { return g5_common(out, in, 0); }
bool blas_ig5(qcdgpu_field out, qcdgpu_field in) { return g5_common(out, in, 1); }

template <int KIND>
static bool reduce_common(qcdgpu_field a, qcdgpu_field b, double ar, double ai, double *res)
{
  double *part = reduce_scratch();
  if (!part) return false;
  int nb = reduce_blocks(a->V);
  cudaStream_t st = stream();
  const void *bd = b ? b->data : nullptr;
  float *bn = b ? b->norm : nullptr;
  QG_DISPATCH(a->prec,
              (k_reduce<QCDGPU_F64, double, KIND><<<nb, 256, 0, st>>>(a->data, a->norm, (void *)bd, bn, ar, ai, a->stride, a->V, part)),
              (k_reduce<QCDGPU_F32, float, KIND><<<nb, 256, 0, st>>>(a->data, a->norm, (void *)bd, bn, (float)ar, (float)ai, a->stride, a->V, part)),
              (k_reduce<QCDGPU_F16, float, KIND><<<nb, 256, 0, st>>>(a->data, a->norm, (void *)bd, bn, (float)ar, (float)ai, a->stride, a->V, part)));
  if (!QG_LAUNCHED("reduce")) return false;
  k_finalize<<<1, 256, 0, st>>>(part, nb, res);
  return QG_LAUNCHED("reduce_finalize");
}

bool blas_norm2_dev(qcdgpu_field x, double *res) { return reduce_common<0>(x, nullptr, 0, 0, res); }

bool blas_dot_dev(qcdgpu_field a, qcdgpu_field b, double *res)
{
  if (!same_shape(a, b) || a->prec != b->prec) {
    set_error("dot: fields differ in shape or precision");
    return false;
  }
  return reduce_common<1>(a, b, 0, 0, res);
}

bool blas_axpy_norm2_dev(qcdgpu_field y, double ar, double ai, qcdgpu_field x, double *res)
{
  if (!same_shape(x, y) || x->prec != y->prec) {
    set_error("axpy_norm: fields differ in shape or precision");
    return false;
  }
  return reduce_common<2>(x, y, ar, ai, res);
}

static bool fetch(double *dev_res, double *out, int n)
{
  double *h = host_result();
  if (!h) return false;
  if (!QG_CUDA(cudaMemcpyAsync(h, dev_res, sizeof(double) * n, cudaMemcpyDeviceToHost, stream()))) return false;
  if (!QG_CUDA(cudaStreamSynchronize(stream()))) return false;
  memcpy(out, h, sizeof(double) * n);
  return true;
}

bool blas_norm2(qcdgpu_field x, double *out)
{
  double *r = reduce_scratch();
  if (!r) return false;
  r += 2 * kMaxPartials;
  return blas_norm2_dev(x, r) && fetch(r, out, 1);
}

bool blas_dot(qcdgpu_field a, qcdgpu_field b, double out[2])
{
  double *r = reduce_scratch();
  if (!r) return false;
  r += 2 * kMaxPartials;
  return blas_dot_dev(a, b, r) && fetch(r, out, 2);
}


// ------------------------------------------------ multi-dot, multi-axpy
// Gram-Schmidt and solution updates of the Krylov solvers: k dot products
// against one field in one pass, and one field plus k scaled fields in one
// pass (FP64 fields of one shape, taken as flat arrays of 12 x stride complex
// numbers: the padding holds zeros). Up to kMulti fields per launch; block
// partial sums are added in a fixed order, so the results are deterministic.
constexpr int kMulti = 8, kMultiThreads = 256, kMultiBlocks = 1024;

struct MultiPtr {
  const double2 *p[kMulti];
  double2 a[kMulti];
};

template <int J>
__global__ void __launch_bounds__(kMultiThreads) k_multi_dot(MultiPtr x, const double2 *y, int64_t n, double *part)
{
  double re[J], im[J];
#pragma unroll
  for (int j = 0; j < J; j++) re[j] = im[j] = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kMultiThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kMultiThreads) {
    const double2 b = y[i];
#pragma unroll
    for (int j = 0; j < J; j++) {
      const double2 a = x.p[j][i];  // conj(a) b
      re[j] = fma(a.x, b.x, fma(a.y, b.y, re[j]));
      im[j] = fma(a.x, b.y, fma(-a.y, b.x, im[j]));
    }
  }
  __shared__ double sh[kMultiThreads / 32][2 * kMulti];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < J; j++) {
    for (int o = 16; o > 0; o >>= 1) {
      re[j] += __shfl_xor_sync(0xffffffffu, re[j], o);
      im[j] += __shfl_xor_sync(0xffffffffu, im[j], o);
    }
    if (lane == 0) {
      sh[w][2 * j] = re[j];
      sh[w][2 * j + 1] = im[j];
    }
  }
  __syncthreads();
  if (threadIdx.x < 2 * J) {
    double t = 0.0;
    for (int k = 0; k < kMultiThreads / 32; k++) t += sh[k][threadIdx.x];
    part[(int64_t)blockIdx.x * 2 * kMulti + threadIdx.x] = t;
  }
}

template <int J>
__global__ void __launch_bounds__(kMultiThreads) k_multi_axpy(MultiPtr x, double2 *y, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * kMultiThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kMultiThreads) {
    double2 v = y[i];
#pragma unroll
    for (int j = 0; j < J; j++) {
      const double2 b = x.p[j][i], c = x.a[j];
      v.x = fma(c.x, b.x, fma(-c.y, b.y, v.x));
      v.y = fma(c.x, b.y, fma(c.y, b.x, v.y));
    }
    y[i] = v;
  }
}

static unsigned multi_blocks(int64_t n)
{
  const int64_t b = (n + kMultiThreads - 1) / kMultiThreads;
  return (unsigned)(b < kMultiBlocks ? b : kMultiBlocks);
}

bool blas_multi_dot(const qcdgpu_field *x, int k, qcdgpu_field y, std::complex<double> *out)
{
  if (k <= 0) return true;
  for (int j = 0; j < k; j++)
    if (!same_shape(x[j], y) || x[j]->prec != QCDGPU_F64 || y->prec != QCDGPU_F64) {
      set_error("multi-dot: FP64 fields of one shape");
      return false;
    }
  static double *part = nullptr, *host = nullptr;
  if (!part) {
    if (!QG_CUDA(cudaMalloc(&part, sizeof(double) * 2 * kMulti * kMultiBlocks))) return false;
    if (!QG_CUDA(cudaMallocHost(&host, sizeof(double) * 2 * kMulti * kMultiBlocks))) return false;
  }
  const int64_t n = 12 * y->stride;
  const unsigned nb = multi_blocks(n);
  cudaStream_t st = stream();
  for (int j0 = 0; j0 < k; j0 += kMulti) {
    const int J = k - j0 < kMulti ? k - j0 : kMulti;
    MultiPtr mp{};
    for (int j = 0; j < J; j++) mp.p[j] = (const double2 *)x[j0 + j]->data;
    const double2 *yy = (const double2 *)y->data;
    switch (J) {
    case 1: k_multi_dot<1><<<nb, kMultiThreads, 0, st>>>(mp, yy, n, part); break;
    case 2: k_multi_dot<2><<<nb, kMultiThreads, 0, st>>>(mp, yy, n, part); break;
    case 3: k_multi_dot<3><<<nb, kMultiThreads, 0, st>>>(mp, yy, n, part); break;
    case 4: k_multi_dot<4><<<nb, kMultiThreads, 0, st>>>(mp, yy, n, part); break;
    case 5: k_multi_dot<5><<<nb, kMultiThreads, 0, st>>>(mp, yy, n, part); break;
    case 6: k_multi_dot<6><<<nb, kMultiThreads, 0, st>>>(mp, yy, n, part); break;
    case 7: k_multi_dot<7><<<nb, kMultiThreads, 0, st>>>(mp, yy, n, part); break;
    default: k_multi_dot<8><<<nb, kMultiThreads, 0, st>>>(mp, yy, n, part); break;
    }
    if (!QG_LAUNCHED("multi_dot")) return false;
    if (!QG_CUDA(cudaMemcpyAsync(host, part, sizeof(double) * 2 * kMulti * nb, cudaMemcpyDeviceToHost, st)) ||
        !QG_CUDA(cudaStreamSynchronize(st)))
      return false;
    for (int j = 0; j < J; j++) {
      double re = 0.0, im = 0.0;  // block order: deterministic
      for (unsigned b = 0; b < nb; b++) {
        re += host[(size_t)b * 2 * kMulti + 2 * j];
        im += host[(size_t)b * 2 * kMulti + 2 * j + 1];
      }
      out[j0 + j] = std::complex<double>(re, im);
    }
  }
  return true;
}

bool blas_multi_axpy(qcdgpu_field y, const qcdgpu_field *x, const std::complex<double> *a, int k)
{
  for (int j = 0; j < k; j++)
    if (!same_shape(x[j], y) || x[j]->prec != QCDGPU_F64 || y->prec != QCDGPU_F64) {
      set_error("multi-axpy: FP64 fields of one shape");
      return false;
    }
  const int64_t n = 12 * y->stride;
  const unsigned nb = multi_blocks(n);
  cudaStream_t st = stream();
  for (int j0 = 0; j0 < k; j0 += kMulti) {
    const int J = k - j0 < kMulti ? k - j0 : kMulti;
    MultiPtr mp{};
    for (int j = 0; j < J; j++) {
      mp.p[j] = (const double2 *)x[j0 + j]->data;
      mp.a[j] = make_double2(a[j0 + j].real(), a[j0 + j].imag());
    }
    double2 *yy = (double2 *)y->data;
    switch (J) {
    case 1: k_multi_axpy<1><<<nb, kMultiThreads, 0, st>>>(mp, yy, n); break;
    case 2: k_multi_axpy<2><<<nb, kMultiThreads, 0, st>>>(mp, yy, n); break;
    case 3: k_multi_axpy<3><<<nb, kMultiThreads, 0, st>>>(mp, yy, n); break;
    case 4: k_multi_axpy<4><<<nb, kMultiThreads, 0, st>>>(mp, yy, n); break;
    case 5: k_multi_axpy<5><<<nb, kMultiThreads, 0, st>>>(mp, yy, n); break;
    case 6: k_multi_axpy<6><<<nb, kMultiThreads, 0, st>>>(mp, yy, n); break;
    case 7: k_multi_axpy<7><<<nb, kMultiThreads, 0, st>>>(mp, yy, n); break;
    default: k_multi_axpy<8><<<nb, kMultiThreads, 0, st>>>(mp, yy, n); break;
    }
    if (!QG_LAUNCHED("multi_axpy")) return false;
  }
  return true;
}

}  // namespace qg

extern "C" {

int qcdgpu_axpy(qcdgpu_field out, double are, double aim, qcdgpu_field x, qcdgpu_field y)
{
  return qg::blas_axpby(out, are, aim, x, 1.0, 0.0, y) ? 0 : 1;
}

int qcdgpu_norm2(qcdgpu_field x, double *result) { return qg::blas_norm2(x, result) ? 0 : 1; }

int qcdgpu_dot(qcdgpu_field a, qcdgpu_field b, double result[2]) { return qg::blas_dot(a, b, result) ? 0 : 1; }

}  // extern "C"
