// layout.cu -- host layout (qcd_vector / qcd_gaugeField, array-of-structs,
// FP64) <-> device structure-of-arrays, and precision conversion.
//
// Uploads copy the host bytes unchanged into a staging buffer and reorder on
// the device; downloads do the reverse. A gauge upload also measures how far
// each link's third row is from conj(row0 x row1): at <= 2e-14 the field is
// stored with 12 reals per link, else with all 18.
#include <string.h>

#include <mutex>

#include "internal.h"

namespace qg {

using namespace qgd;

static void *g_stage = nullptr;
static size_t g_stage_bytes = 0;
static std::mutex g_stage_mu;

static void *stage(size_t bytes)
{
  if (bytes > g_stage_bytes) {
    if (g_stage) {
      cudaStreamSynchronize(stream());
      cudaFree(g_stage);
    }
    g_stage = nullptr;
    g_stage_bytes = 0;
    if (!QG_CUDA(cudaMalloc(&g_stage, bytes))) return nullptr;
    g_stage_bytes = bytes;
  }
  return g_stage;
}

static inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

// ------------------------------------------------------------ spinors
template <int P>
__global__ void k_spinor_aos_to_soa(void *dst, float *norm, int64_t stride, const double2 *src,
                                    int64_t V, int64_t x0 = 0)
{
  int64_t x = x0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= V) return;
  C<double> s[12];
  const double2 *p = src + x * 12;
#pragma unroll
  for (int k = 0; k < 12; k++) {
    double2 v = p[k];
    s[k] = C<double>{v.x, v.y};
  }
  Spinor<P, double>::store(dst, norm, stride, x, s);
}

template <int P>
__global__ void k_spinor_soa_to_aos(double2 *dst, const void *src, const float *norm,
                                    int64_t stride, int64_t V, int64_t x0 = 0)
{
  int64_t x = x0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= V) return;
  C<double> s[12];
  Spinor<P, double>::load(src, norm, stride, x, s);
  double2 *p = dst + x * 12;
#pragma unroll
  for (int k = 0; k < 12; k++) p[k] = make_double2(s[k].re, s[k].im);
}

bool upload_spinor_aos(qcdgpu_field f, const double *host)
{
  std::lock_guard<std::mutex> lk(g_stage_mu);
  size_t bytes = (size_t)f->V * 24 * 8;
  void *st = stage(bytes);
  if (!st) return false;
  if (!QG_CUDA(cudaMemcpyAsync(st, host, bytes, cudaMemcpyHostToDevice, stream()))) return false;
  unsigned g = grid_for(f->V, 128);
  switch (f->prec) {
  case QCDGPU_F64:
    k_spinor_aos_to_soa<QCDGPU_F64><<<g, 128, 0, stream()>>>(f->data, f->norm, f->stride, (const double2 *)st, f->V);
    break;
  case QCDGPU_F32:
    k_spinor_aos_to_soa<QCDGPU_F32><<<g, 128, 0, stream()>>>(f->data, f->norm, f->stride, (const double2 *)st, f->V);
    break;
  default:
    k_spinor_aos_to_soa<QCDGPU_F16><<<g, 128, 0, stream()>>>(f->data, f->norm, f->stride, (const double2 *)st, f->V);
  }
  return QG_LAUNCHED("spinor_aos_to_soa");
}

bool download_spinor_aos(qcdgpu_field f, double *host)
{
  std::lock_guard<std::mutex> lk(g_stage_mu);
  size_t bytes = (size_t)f->V * 24 * 8;
  void *st = stage(bytes);
  if (!st) return false;
  unsigned g = grid_for(f->V, 128);
  switch (f->prec) {
  case QCDGPU_F64:
    k_spinor_soa_to_aos<QCDGPU_F64><<<g, 128, 0, stream()>>>((double2 *)st, f->data, f->norm, f->stride, f->V);
    break;
  case QCDGPU_F32:
    k_spinor_soa_to_aos<QCDGPU_F32><<<g, 128, 0, stream()>>>((double2 *)st, f->data, f->norm, f->stride, f->V);
    break;
  default:
    k_spinor_soa_to_aos<QCDGPU_F16><<<g, 128, 0, stream()>>>((double2 *)st, f->data, f->norm, f->stride, f->V);
  }
  if (!QG_LAUNCHED("spinor_soa_to_aos")) return false;
  if (!QG_CUDA(cudaMemcpyAsync(host, st, bytes, cudaMemcpyDeviceToHost, stream()))) return false;
  return QG_CUDA(cudaStreamSynchronize(stream()));
}

template <int SP, int DP>
__global__ void k_convert_spinor(void *dst, float *dnorm, const void *src, const float *snorm,
                                 int64_t stride, int64_t V)
{
  int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= V) return;
  C<double> s[12];
  Spinor<SP, double>::load(src, snorm, stride, x, s);
  Spinor<DP, double>::store(dst, dnorm, stride, x, s);
}

template <int SP>
static void launch_convert(qcdgpu_field d, qcdgpu_field s)
{
  unsigned g = grid_for(d->V, 128);
  switch (d->prec) {
  case QCDGPU_F64:
    k_convert_spinor<SP, QCDGPU_F64><<<g, 128, 0, stream()>>>(d->data, d->norm, s->data, s->norm, d->stride, d->V);
    break;
  case QCDGPU_F32:
    k_convert_spinor<SP, QCDGPU_F32><<<g, 128, 0, stream()>>>(d->data, d->norm, s->data, s->norm, d->stride, d->V);
    break;
  default:
    k_convert_spinor<SP, QCDGPU_F16><<<g, 128, 0, stream()>>>(d->data, d->norm, s->data, s->norm, d->stride, d->V);
  }
}

bool convert_field(qcdgpu_field d, qcdgpu_field s)
{
  if (!same_shape(d, s)) {
    set_error("field copy: shapes differ");
    return false;
  }
  if (d->prec == s->prec) return blas_copy(d, s);
  switch (s->prec) {
  case QCDGPU_F64: launch_convert<QCDGPU_F64>(d, s); break;
  case QCDGPU_F32: launch_convert<QCDGPU_F32>(d, s); break;
  default: launch_convert<QCDGPU_F16>(d, s);
  }
  return QG_LAUNCHED("convert_spinor");
}

// -------------------------------------------------------------- gauge
// max over links of |row2 - conj(row0 x row1)| (as float bits, >= 0)
__global__ void k_gauge_su3_dev(const double2 *src, int64_t nlinks, unsigned int *out)
{
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float dev = 0.f;
  if (i < nlinks) {
    C<double> U[9];
    const double2 *p = src + i * 9;
#pragma unroll
    for (int k = 0; k < 9; k++) U[k] = C<double>{p[k].x, p[k].y};
    C<double> r[9];
#pragma unroll
    for (int k = 0; k < 6; k++) r[k] = U[k];
    rebuild_row2(r);
    double m = 0;
#pragma unroll
    for (int k = 6; k < 9; k++) m = fmax(m, fmax(fabs(r[k].re - U[k].re), fabs(r[k].im - U[k].im)));
    dev = (float)m;
    if (!(m == m)) dev = 1e30f;  // NaN links must not pass
  }
  for (int o = 16; o > 0; o >>= 1) dev = fmaxf(dev, __shfl_xor_sync(0xffffffffu, dev, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(dev));
}

template <int P>
__device__ __forceinline__ void put_link(void *dst, int64_t stride, int64_t x, int mu, int recon,
                                         const C<double> U[9])
{
  if (P == QCDGPU_F64) {
    // FP64 links are stored complete whatever recon says (see internal.h)
    double2 *d = (double2 *)dst + (int64_t)mu * 9 * stride + x;
    for (int k = 0; k < 9; k++) d[k * stride] = make_double2(U[k].re, U[k].im);
  } else if (P == QCDGPU_F32) {
    if (recon == 12) {
      float4 *d = (float4 *)dst + (int64_t)mu * 3 * stride + x;
      for (int j = 0; j < 3; j++)
        d[j * stride] = make_float4((float)U[2 * j].re, (float)U[2 * j].im, (float)U[2 * j + 1].re,
                                    (float)U[2 * j + 1].im);
    } else {
      float2 *d = (float2 *)dst + (int64_t)mu * 9 * stride + x;
      for (int k = 0; k < 9; k++) d[k * stride] = make_float2((float)U[k].re, (float)U[k].im);
    }
  } else {
    uint2 *d = (uint2 *)dst + (int64_t)mu * 3 * stride + x;
    for (int j = 0; j < 3; j++) {
      uint2 v;
      __half2 *h = reinterpret_cast<__half2 *>(&v);
      h[0] = __floats2half2_rn((float)U[2 * j].re, (float)U[2 * j].im);
      h[1] = __floats2half2_rn((float)U[2 * j + 1].re, (float)U[2 * j + 1].im);
      d[j * stride] = v;
    }
  }
}

template <int P>
__global__ void k_gauge_aos_to_soa(void *dst, int64_t stride, int recon, const double2 *src, int64_t V)
{
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V * 4) return;
  int64_t x = i >> 2;
  int mu = (int)(i & 3);
  C<double> U[9];
  const double2 *p = src + i * 9;
#pragma unroll
  for (int k = 0; k < 9; k++) U[k] = C<double>{p[k].x, p[k].y};
  put_link<P>(dst, stride, x, mu, recon, U);
}

template <int P, int R>
__global__ void k_gauge_soa_to_aos(double2 *dst, const void *src, int64_t stride, int64_t V)
{
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V * 4) return;
  int64_t x = i >> 2;
  int mu = (int)(i & 3);
  C<double> U[9];
  Link<P, R, double>::load(src, stride, x, mu, U);
  double2 *p = dst + i * 9;
#pragma unroll
  for (int k = 0; k < 9; k++) p[k] = make_double2(U[k].re, U[k].im);
}

template <int SP, int SR, int DP>
__global__ void k_convert_gauge(void *dst, int64_t dstride, int drecon, const void *src,
                                int64_t sstride, int64_t V)
{
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V * 4) return;
  int64_t x = i >> 2;
  int mu = (int)(i & 3);
  C<double> U[9];
  Link<SP, SR, double>::load(src, sstride, x, mu, U);
  put_link<DP>(dst, dstride, x, mu, drecon, U);
}

static unsigned *g_devflag = nullptr;

// SU(3) check and packing of a gauge field held on the device in the host layout
bool pack_gauge(qcdgpu_gauge g, const void *dev_aos)
{
  if (!g_devflag && !QG_CUDA(cudaMalloc(&g_devflag, sizeof(unsigned)))) return false;
  unsigned *hres = (unsigned *)host_result();
  if (!hres) return false;
  if (!QG_CUDA(cudaMemsetAsync(g_devflag, 0, sizeof(unsigned), stream()))) return false;
  int64_t nl = g->V * 4;
  k_gauge_su3_dev<<<grid_for(nl, 256), 256, 0, stream()>>>((const double2 *)dev_aos, nl, g_devflag);
  if (!QG_LAUNCHED("gauge_su3_dev")) return false;
  if (!QG_CUDA(cudaMemcpyAsync(hres, g_devflag, sizeof(unsigned), cudaMemcpyDeviceToHost, stream())))
    return false;
  if (!QG_CUDA(cudaStreamSynchronize(stream()))) return false;
  float dev;
  memcpy(&dev, hres, sizeof(dev));
  int recon = dev <= 2e-14f ? 12 : 18;
  if (g->prec == QCDGPU_F16 && recon == 18) {
    set_error("half-precision gauge fields need SU(3) links (third-row deviation %g)", dev);
    return false;
  }
  g->recon = recon;
  unsigned gr = grid_for(nl, 128);
  const double2 *st = (const double2 *)dev_aos;
  switch (g->prec) {
  case QCDGPU_F64: k_gauge_aos_to_soa<QCDGPU_F64><<<gr, 128, 0, stream()>>>(g->data, g->stride, recon, st, g->V); break;
  case QCDGPU_F32: k_gauge_aos_to_soa<QCDGPU_F32><<<gr, 128, 0, stream()>>>(g->data, g->stride, recon, st, g->V); break;
  default: k_gauge_aos_to_soa<QCDGPU_F16><<<gr, 128, 0, stream()>>>(g->data, g->stride, recon, st, g->V);
  }
  return QG_LAUNCHED("gauge_aos_to_soa");
}

void *stage_buffer(size_t bytes) { return stage(bytes); }

// spinor field <-> the host layout [V][4][3] complex double held in device memory
bool spinor_from_aos_dev(qcdgpu_field f, const void *dev_aos)
{
  unsigned g = grid_for(f->V, 128);
  const double2 *a = (const double2 *)dev_aos;
  switch (f->prec) {
  case QCDGPU_F64: k_spinor_aos_to_soa<QCDGPU_F64><<<g, 128, 0, stream()>>>(f->data, f->norm, f->stride, a, f->V); break;
  case QCDGPU_F32: k_spinor_aos_to_soa<QCDGPU_F32><<<g, 128, 0, stream()>>>(f->data, f->norm, f->stride, a, f->V); break;
  default: k_spinor_aos_to_soa<QCDGPU_F16><<<g, 128, 0, stream()>>>(f->data, f->norm, f->stride, a, f->V);
  }
  return QG_LAUNCHED("spinor_aos_to_soa");
}

bool spinor_to_aos_dev(qcdgpu_field f, void *dev_aos)
{
  unsigned g = grid_for(f->V, 128);
  double2 *a = (double2 *)dev_aos;
  switch (f->prec) {
  case QCDGPU_F64: k_spinor_soa_to_aos<QCDGPU_F64><<<g, 128, 0, stream()>>>(a, f->data, f->norm, f->stride, f->V); break;
  case QCDGPU_F32: k_spinor_soa_to_aos<QCDGPU_F32><<<g, 128, 0, stream()>>>(a, f->data, f->norm, f->stride, f->V); break;
  default: k_spinor_soa_to_aos<QCDGPU_F16><<<g, 128, 0, stream()>>>(a, f->data, f->norm, f->stride, f->V);
  }
  return QG_LAUNCHED("spinor_soa_to_aos");
}

// sites x0 .. x1-1 of an FP64 field from / to the host layout held in device
// memory (the whole field's array; only the range is touched)
bool spinor_from_aos_sites(qcdgpu_field f, const void *dev_aos, int64_t x0, int64_t x1)
{
  if (f->prec != QCDGPU_F64) return false;
  k_spinor_aos_to_soa<QCDGPU_F64><<<grid_for(x1 - x0, 128), 128, 0, stream()>>>(f->data, f->norm, f->stride,
                                                                                 (const double2 *)dev_aos, x1, x0);
  return QG_LAUNCHED("spinor_aos_to_soa");
}

bool spinor_to_aos_sites(qcdgpu_field f, void *dev_aos, int64_t x0, int64_t x1)
{
  if (f->prec != QCDGPU_F64) return false;
  k_spinor_soa_to_aos<QCDGPU_F64><<<grid_for(x1 - x0, 128), 128, 0, stream()>>>((double2 *)dev_aos, f->data, f->norm,
                                                                                 f->stride, x1, x0);
  return QG_LAUNCHED("spinor_soa_to_aos");
}

// gauge field -> the host layout [V][4][3][3] complex double in device memory
bool gauge_to_aos_dev(qcdgpu_gauge g, void *dev_aos)
{
  unsigned gr = grid_for(g->V * 4, 128);
  double2 *d = (double2 *)dev_aos;
  if (g->prec == QCDGPU_F64) k_gauge_soa_to_aos<QCDGPU_F64, 18><<<gr, 128, 0, stream()>>>(d, g->data, g->stride, g->V);
  else if (g->prec == QCDGPU_F32 && g->recon == 12) k_gauge_soa_to_aos<QCDGPU_F32, 12><<<gr, 128, 0, stream()>>>(d, g->data, g->stride, g->V);
  else if (g->prec == QCDGPU_F32) k_gauge_soa_to_aos<QCDGPU_F32, 18><<<gr, 128, 0, stream()>>>(d, g->data, g->stride, g->V);
  else k_gauge_soa_to_aos<QCDGPU_F16, 12><<<gr, 128, 0, stream()>>>(d, g->data, g->stride, g->V);
  return QG_LAUNCHED("gauge_soa_to_aos");
}

bool upload_gauge_aos(qcdgpu_gauge g, const double *host)
{
  std::lock_guard<std::mutex> lk(g_stage_mu);
  size_t bytes = (size_t)g->V * 4 * 18 * 8;
  void *st = stage(bytes);
  if (!st) return false;
  if (!QG_CUDA(cudaMemcpyAsync(st, host, bytes, cudaMemcpyHostToDevice, stream()))) return false;
  return pack_gauge(g, st);
}

bool download_gauge_aos(qcdgpu_gauge g, double *host)
{
  std::lock_guard<std::mutex> lk(g_stage_mu);
  size_t bytes = (size_t)g->V * 4 * 18 * 8;
  void *st = stage(bytes);
  if (!st) return false;
  unsigned gr = grid_for(g->V * 4, 128);
  double2 *d = (double2 *)st;
  if (g->prec == QCDGPU_F64) k_gauge_soa_to_aos<QCDGPU_F64, 18><<<gr, 128, 0, stream()>>>(d, g->data, g->stride, g->V);
  else if (g->prec == QCDGPU_F32 && g->recon == 12) k_gauge_soa_to_aos<QCDGPU_F32, 12><<<gr, 128, 0, stream()>>>(d, g->data, g->stride, g->V);
  else if (g->prec == QCDGPU_F32) k_gauge_soa_to_aos<QCDGPU_F32, 18><<<gr, 128, 0, stream()>>>(d, g->data, g->stride, g->V);
  else k_gauge_soa_to_aos<QCDGPU_F16, 12><<<gr, 128, 0, stream()>>>(d, g->data, g->stride, g->V);
  if (!QG_LAUNCHED("gauge_soa_to_aos")) return false;
  if (!QG_CUDA(cudaMemcpyAsync(host, st, bytes, cudaMemcpyDeviceToHost, stream()))) return false;
  return QG_CUDA(cudaStreamSynchronize(stream()));
}

bool gauge_to_ff(qcdgpu_gauge d, qcdgpu_gauge s);  // dslash_df64.cu

// links of direction mu times e^{i theta_mu / L_mu} (FP32, all 18 reals):
// the multi-RHS kernels' copy carries the boundary phases, so its forward
// hops need no phase multiply and its backward hops get the conjugate from U^+
__global__ void k_fold_phases(float2 *d, int64_t stride, int64_t V, float4 phr, float4 phi)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V * 4) return;
  const int mu = (int)(i / V);
  const int64_t x = i % V;
  const float pr = mu == 0 ? phr.x : mu == 1 ? phr.y : mu == 2 ? phr.z : phr.w;
  const float pi = mu == 0 ? phi.x : mu == 1 ? phi.y : mu == 2 ? phi.z : phi.w;
  float2 *p = d + (int64_t)mu * 9 * stride + x;
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const float2 u = p[k * stride];
    p[k * stride] = make_float2(pr * u.x - pi * u.y, pr * u.y + pi * u.x);
  }
}

bool gauge_fold_phases(qcdgpu_gauge g)
{
  if (g->prec != QCDGPU_F32 || g->recon != 18) {
    set_error("phase folding: FP32 18-real gauge copies only");
    return false;
  }
  double pr[4], pi[4];
  bool any = false;
  for (int mu = 0; mu < 4; mu++) {
    pr[mu] = cos(g->theta[mu] / (double)g->L[mu]);
    pi[mu] = sin(g->theta[mu] / (double)g->L[mu]);
    any = any || g->theta[mu] != 0.0;
  }
  if (!any) return true;
  const float4 fr = make_float4((float)pr[0], (float)pr[1], (float)pr[2], (float)pr[3]);
  const float4 fi = make_float4((float)pi[0], (float)pi[1], (float)pi[2], (float)pi[3]);
  k_fold_phases<<<grid_for(g->V * 4, 128), 128, 0, stream()>>>((float2 *)g->data, g->stride, g->V, fr, fi);
  return QG_LAUNCHED("fold_phases");
}

bool convert_gauge(qcdgpu_gauge d, qcdgpu_gauge s, int force_recon)
{
  if (d->prec == kGaugeFF) return gauge_to_ff(d, s);
  if (d->V != s->V) {
    set_error("gauge convert: volumes differ");
    return false;
  }
  if (d->prec == QCDGPU_F16 && s->recon != 12) {
    set_error("half-precision gauge fields need SU(3) links");
    return false;
  }
  d->recon = force_recon ? force_recon : s->recon;
  memcpy(d->theta, s->theta, sizeof(d->theta));
  unsigned gr = grid_for(s->V * 4, 128);
#define QG_CONV(SP, SR)                                                                          \
  switch (d->prec) {                                                                             \
  case QCDGPU_F64: k_convert_gauge<SP, SR, QCDGPU_F64><<<gr, 128, 0, stream()>>>(d->data, d->stride, d->recon, s->data, s->stride, s->V); break; \
  case QCDGPU_F32: k_convert_gauge<SP, SR, QCDGPU_F32><<<gr, 128, 0, stream()>>>(d->data, d->stride, d->recon, s->data, s->stride, s->V); break; \
  default: k_convert_gauge<SP, SR, QCDGPU_F16><<<gr, 128, 0, stream()>>>(d->data, d->stride, d->recon, s->data, s->stride, s->V); \
  }
  if (s->prec == QCDGPU_F64 && s->recon == 12) { QG_CONV(QCDGPU_F64, 12) }
  else if (s->prec == QCDGPU_F64) { QG_CONV(QCDGPU_F64, 18) }
  else if (s->prec == QCDGPU_F32 && s->recon == 12) { QG_CONV(QCDGPU_F32, 12) }
  else if (s->prec == QCDGPU_F32) { QG_CONV(QCDGPU_F32, 18) }
  else { QG_CONV(QCDGPU_F16, 12) }
#undef QG_CONV
  return QG_LAUNCHED("convert_gauge");
}

}  // namespace qg

extern "C" {

int qcdgpu_field_load(qcdgpu_field f, const double *host) { return qg::upload_spinor_aos(f, host) ? 0 : 1; }
int qcdgpu_field_store(qcdgpu_field f, double *host) { return qg::download_spinor_aos(f, host) ? 0 : 1; }
int qcdgpu_field_copy(qcdgpu_field d, qcdgpu_field s) { return qg::convert_field(d, s) ? 0 : 1; }
int qcdgpu_gauge_load(qcdgpu_gauge g, const double *host)
{
  qg::gauge_forget(g);  // derived low-precision copies are stale now
  return qg::upload_gauge_aos(g, host) ? 0 : 1;
}
int qcdgpu_gauge_store(qcdgpu_gauge g, double *host) { return qg::download_gauge_aos(g, host) ? 0 : 1; }
int qcdgpu_gauge_convert(qcdgpu_gauge d, qcdgpu_gauge s)
{
  qg::gauge_forget(d);
  return qg::convert_gauge(d, s) ? 0 : 1;
}

}  // extern "C"
