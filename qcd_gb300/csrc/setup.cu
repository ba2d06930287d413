// setup.cu -- synthetic inputs and the plaquette on the GPU.
//
// Generators use a counter-based stream: the SplitMix64 output function
// (S. Vigna, public domain) of a seed-keyed counter, so every site draws its
// numbers independently and the result does not depend on the launch shape.
// Counters:  spinor component (site, spin, colour, re/im) -> 24 site + 6 spin
//            + 2 colour + reim ; gauge link (site, mu) draws 8 normals from
//            counters 8 (4 site + mu) + a.
// Gauge links are U = exp(i eps H) with H = sum_a g_a lambda_a / 2,
// g_a ~ N(0,1), exponentiated by the Cayley-Hamilton formula of Morningstar
// and Peardon (Phys. Rev. D 69 (2004) 054501; the reference's Exp(),
// lib/src/qcd_smearing.c:293-371) and re-orthonormalised by columns (the last
// stage of qcd_projectSU33x3, lib/src/qcd_blas.c:1700-1766).
#include <string.h>

#include <vector>

#include "internal.h"
#include "su3.cuh"

namespace qg {

using namespace qgd;

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t rng_bits(uint64_t key, uint64_t ctr) { return mix64(key ^ ctr); }
__host__ __device__ inline uint64_t rng_key(uint64_t seed)
{
  // mix64 of the scrambled seed, computed on the host once per launch
  uint64_t z = seed * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull;
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double uniform01(uint64_t key, uint64_t ctr)
{
  return ((double)(rng_bits(key, ctr) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
__device__ __forceinline__ double normal(uint64_t key, uint64_t k)
{
  double u1 = uniform01(key, 2 * k), u2 = uniform01(key, 2 * k + 1);
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

// ------------------------------------------------------------------ spinors
template <int P>
__global__ void k_gaussian(void *d, float *n, int64_t stride, int64_t V, uint64_t key)
{
  int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= V) return;
  C<double> s[12];
#pragma unroll
  for (int k = 0; k < 12; k++)
    s[k] = C<double>{normal(key, (uint64_t)x * 24 + 2 * k), normal(key, (uint64_t)x * 24 + 2 * k + 1)};
  Spinor<P, double>::store(d, n, stride, x, s);
}

// Noise spinors (the stochastic sources of qcd_stochastic.c:8-58): every
// spin-colour component of the sites on time-slice tslice (all sites when
// tslice < 0) is an independent draw from Z4 = {1, i, -1, -i} (kind 4, the
// two top bits of the site's counter-based stream at 12 x + k) or Z2 = {1, -1}
// (kind 2, the top bit); the other sites are zero. The reference draws from
// GSL's ranlux (absent here); this stream is the library's own, seeded.
template <int P>
__global__ void k_noise(void *d, float *n, int64_t stride, int64_t V, uint64_t key, int L0, int tslice, int kind)
{
  int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= V) return;
  const bool on = tslice < 0 || (int)(x % L0) == tslice;
  C<double> s[12];
#pragma unroll
  for (int k = 0; k < 12; k++) {
    const uint64_t b = rng_bits(key, (uint64_t)x * 12 + k);
    if (!on) {
      s[k] = C<double>{0.0, 0.0};
    } else if (kind == 2) {
      s[k] = C<double>{(b >> 63) ? -1.0 : 1.0, 0.0};
    } else {
      const unsigned r = (unsigned)(b >> 62);
      s[k] = C<double>{r == 0 ? 1.0 : r == 2 ? -1.0 : 0.0, r == 1 ? 1.0 : r == 3 ? -1.0 : 0.0};
    }
  }
  Spinor<P, double>::store(d, n, stride, x, s);
}

template <int P>
__global__ void k_point(void *d, float *n, int64_t stride, int64_t x, int k)
{
  C<double> s[12];
#pragma unroll
  for (int j = 0; j < 12; j++) s[j] = C<double>{j == k ? 1.0 : 0.0, 0.0};
  Spinor<P, double>::store(d, n, stride, x, s);
}

static unsigned blocks(int64_t n, int b) { return (unsigned)((n + b - 1) / b); }

bool field_gaussian(qcdgpu_field f, uint64_t seed)
{
  uint64_t key = rng_key(seed);
  unsigned g = blocks(f->V, 128);
  if (f->prec == QCDGPU_F64) k_gaussian<QCDGPU_F64><<<g, 128, 0, stream()>>>(f->data, f->norm, f->stride, f->V, key);
  else if (f->prec == QCDGPU_F32) k_gaussian<QCDGPU_F32><<<g, 128, 0, stream()>>>(f->data, f->norm, f->stride, f->V, key);
  else k_gaussian<QCDGPU_F16><<<g, 128, 0, stream()>>>(f->data, f->norm, f->stride, f->V, key);
  return QG_LAUNCHED("gaussian_spinor");
}

bool field_noise(qcdgpu_field f, uint64_t seed, int tslice, int kind)
{
  if (!f || (kind != 2 && kind != 4)) {
    set_error("noise: kind 2 (Z2) or 4 (Z4)");
    return false;
  }
  uint64_t key = rng_key(seed);
  unsigned g = blocks(f->V, 128);
  const int L0 = f->L[0];
  if (f->prec == QCDGPU_F64)
    k_noise<QCDGPU_F64><<<g, 128, 0, stream()>>>(f->data, f->norm, f->stride, f->V, key, L0, tslice, kind);
  else if (f->prec == QCDGPU_F32)
    k_noise<QCDGPU_F32><<<g, 128, 0, stream()>>>(f->data, f->norm, f->stride, f->V, key, L0, tslice, kind);
  else
    k_noise<QCDGPU_F16><<<g, 128, 0, stream()>>>(f->data, f->norm, f->stride, f->V, key, L0, tslice, kind);
  return QG_LAUNCHED("noise_spinor");
}

bool field_z4(qcdgpu_field f, uint64_t seed) { return field_noise(f, seed, -1, 4); }

bool field_point(qcdgpu_field f, const int x[4], int spin, int colour)
{
  for (int i = 0; i < 4; i++)
    if (x[i] < 0 || x[i] >= f->L[i]) {
      set_error("point source outside the lattice");
      return false;
    }
  if (spin < 0 || spin > 3 || colour < 0 || colour > 2) {
    set_error("point source: spin 0..3, colour 0..2");
    return false;
  }
  if (!blas_zero(f)) return false;
  int64_t s = x[0] + (int64_t)f->L[0] * (x[1] + (int64_t)f->L[1] * (x[2] + (int64_t)f->L[2] * x[3]));
  int k = spin * 3 + colour;
  if (f->prec == QCDGPU_F64) k_point<QCDGPU_F64><<<1, 1, 0, stream()>>>(f->data, f->norm, f->stride, s, k);
  else if (f->prec == QCDGPU_F32) k_point<QCDGPU_F32><<<1, 1, 0, stream()>>>(f->data, f->norm, f->stride, s, k);
  else k_point<QCDGPU_F16><<<1, 1, 0, stream()>>>(f->data, f->norm, f->stride, s, k);
  return QG_LAUNCHED("point_source");
}

// -------------------------------------------------------------------- gauge
__device__ double sinc_mp(double w)
{
  if (fabs(w) < 0.05) {
    double w2 = w * w;
    return 1.0 - w2 / 6.0 * (1.0 - w2 / 20.0 * (1.0 - w2 / 42.0));
  }
  return sin(w) / w;
}

// M <- exp(i M) for traceless Hermitian M
__device__ void exp_iM(C<double> M[9])
{
  C<double> M2[9], M3[9];
  m3mul(M, M, M2);
  m3mul(M2, M, M3);
  double c0 = (M3[0].re + M3[4].re + M3[8].re) / 3.0;
  double c1 = (M2[0].re + M2[4].re + M2[8].re) / 2.0;
  bool neg = c0 < 0;
  if (neg) c0 = -c0;
  double r3 = sqrt(c1 / 3.0);
  double c0max = 2.0 * r3 * r3 * r3;
  double ratio = c0 / c0max;
  if (ratio > 1.0) ratio = 1.0;
  double th = acos(ratio);
  double u = r3 * cos(th / 3.0);
  double w = sqrt(c1) * sin(th / 3.0);
  double xi = sinc_mp(w), cw = cos(w);
  C<double> e2iu{cos(2 * u), sin(2 * u)}, emiu{cos(u), -sin(u)};
  C<double> h0 = C<double>{u * u - w * w, 0} * e2iu + emiu * C<double>{8 * u * u * cw, 2 * u * (3 * u * u + w * w) * xi};
  C<double> h1 = C<double>{2 * u, 0} * e2iu - emiu * C<double>{2 * u * cw, -(3 * u * u - w * w) * xi};
  C<double> h2 = e2iu - emiu * C<double>{cw, 3 * u * xi};
  double den = 1.0 / (9 * u * u - w * w);
  C<double> f0 = den * h0, f1 = den * h1, f2 = den * h2;
  if (neg) {
    f0 = conj(f0);
    f1 = conj(-f1);
    f2 = conj(f2);
  }
#pragma unroll
  for (int k = 0; k < 9; k++) {
    C<double> s = f1 * M[k] + f2 * M2[k];
    if (k == 0 || k == 4 || k == 8) s = s + f0;
    M[k] = s;
  }
}


// writes links in the host layout into aos[(4 site + mu) * 9 + k]
__global__ void k_gauge_synth(double2 *aos, int64_t V, uint64_t key, double eps)
{
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V * 4) return;
  double g[8];
#pragma unroll
  for (int a = 0; a < 8; a++) g[a] = 0.5 * eps * normal(key, (uint64_t)i * 8 + a);
  const double s3 = 0.57735026918962576451;  // 1/sqrt(3)
  C<double> H[9];
  H[0] = C<double>{g[2] + g[7] * s3, 0};
  H[4] = C<double>{-g[2] + g[7] * s3, 0};
  H[8] = C<double>{-2.0 * g[7] * s3, 0};
  H[1] = C<double>{g[0], -g[1]};
  H[3] = C<double>{g[0], g[1]};
  H[2] = C<double>{g[3], -g[4]};
  H[6] = C<double>{g[3], g[4]};
  H[5] = C<double>{g[5], -g[6]};
  H[7] = C<double>{g[5], g[6]};
  exp_iM(H);
  reunit_cols(H);
#pragma unroll
  for (int k = 0; k < 9; k++) aos[i * 9 + k] = make_double2(H[k].re, H[k].im);
}

bool gauge_synthetic(qcdgpu_gauge g, uint64_t seed, double eps)
{
  // generate in the host layout into the staging buffer, then pack
  size_t bytes = (size_t)g->V * 4 * 18 * 8;
  double2 *aos = (double2 *)stage_buffer(bytes);
  if (!aos) return false;
  k_gauge_synth<<<blocks(g->V * 4, 128), 128, 0, stream()>>>(aos, g->V, rng_key(seed), eps);
  if (!QG_LAUNCHED("gauge_synthetic")) return false;
  return pack_gauge(g, aos);
}

// ---------------------------------------------------------------- plaquette
template <int P, int R>
__global__ void __launch_bounds__(256) k_plaquette(const void *u, int64_t stride, Geom geo, int64_t V,
                                                   double *partials)
{
  double acc = 0;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < V;
       x += (int64_t)gridDim.x * blockDim.x) {
    int c[4];
    coords(geo, x, c);
#pragma unroll
    for (int mu = 0; mu < 3; mu++)
#pragma unroll
      for (int nu = mu + 1; nu < 4; nu++) {
        C<double> A[9], B[9], T[9];
        Link<P, R, double>::load(u, stride, x, mu, A);
        Link<P, R, double>::load(u, stride, fwd(geo, x, c, mu), nu, B);
        m3mul(A, B, T);  // U_mu(x) U_nu(x+mu)
        Link<P, R, double>::load(u, stride, fwd(geo, x, c, nu), mu, A);
        Link<P, R, double>::load(u, stride, x, nu, B);
        // Re tr( T U_mu(x+nu)^+ U_nu(x)^+ ) = Re tr( T (B A)^+ )
        C<double> BA[9];
        m3mul(B, A, BA);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int k = 0; k < 3; k++) {
            C<double> t = T[3 * i + k], b = BA[3 * i + k];
            acc += t.re * b.re + t.im * b.im;  // Re( t conj(b) )
          }
      }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double sh[8];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += sh[i];
    partials[blockIdx.x] = s;
  }
}

double plaquette(qcdgpu_gauge g)
{
  double *part = reduce_scratch();
  double *h = host_result();
  if (!part || !h) return -1.0;
  Geom geo;
  for (int i = 0; i < 4; i++) geo.L[i] = g->L[i];
  geo.st[0] = 1;
  geo.st[1] = g->L[0];
  geo.st[2] = (int64_t)g->L[0] * g->L[1];
  geo.st[3] = geo.st[2] * g->L[2];
  int nb = (int)((g->V + 255) / 256);
  if (nb > kMaxPartials) nb = kMaxPartials;
  cudaStream_t st = stream();
  if (g->prec == QCDGPU_F64 && g->recon == 12) k_plaquette<QCDGPU_F64, 12><<<nb, 256, 0, st>>>(g->data, g->stride, geo, g->V, part);
  else if (g->prec == QCDGPU_F64) k_plaquette<QCDGPU_F64, 18><<<nb, 256, 0, st>>>(g->data, g->stride, geo, g->V, part);
  else if (g->prec == QCDGPU_F32 && g->recon == 12) k_plaquette<QCDGPU_F32, 12><<<nb, 256, 0, st>>>(g->data, g->stride, geo, g->V, part);
  else if (g->prec == QCDGPU_F32) k_plaquette<QCDGPU_F32, 18><<<nb, 256, 0, st>>>(g->data, g->stride, geo, g->V, part);
  else k_plaquette<QCDGPU_F16, 12><<<nb, 256, 0, st>>>(g->data, g->stride, geo, g->V, part);
  if (!QG_LAUNCHED("plaquette")) return -1.0;
  // fixed-order final sum on the host of nb partials
  std::vector<double> hp((size_t)nb);
  if (!QG_CUDA(cudaMemcpyAsync(hp.data(), part, sizeof(double) * nb, cudaMemcpyDeviceToHost, st)) ||
      !QG_CUDA(cudaStreamSynchronize(st)))
    return -1.0;
  double s = 0;
  for (int i = 0; i < nb; i++) s += hp[(size_t)i];
  return s / ((double)g->V * 18.0);
}

}  // namespace qg

extern "C" {

int qcdgpu_gauge_synthetic(qcdgpu_gauge g, uint64_t seed, double eps)
{
  qg::gauge_forget(g);
  return qg::gauge_synthetic(g, seed, eps) ? 0 : 1;
}
double qcdgpu_plaquette(qcdgpu_gauge g) { return qg::plaquette(g); }
int qcdgpu_field_gaussian(qcdgpu_field f, uint64_t seed) { return qg::field_gaussian(f, seed) ? 0 : 1; }
int qcdgpu_field_noise(qcdgpu_field f, uint64_t seed, int t_slice, int kind)
{
  return qg::field_noise(f, seed, t_slice, kind) ? 0 : 1;
}
int qcdgpu_field_point(qcdgpu_field f, const int x[4], int spin, int colour)
{
  return qg::field_point(f, x, spin, colour) ? 0 : 1;
}

}  // extern "C"
