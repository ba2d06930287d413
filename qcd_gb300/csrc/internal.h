// internal.h -- shared declarations of the GB300 Wilson-TM library.
//
// Device data layout (site-major structure-of-arrays; every block holds one
// component for all sites, so a warp reading consecutive sites issues fully
// coalesced 128-bit loads):
//
//   spinor F64 : 12 blocks of double2  -- block k = spin*3+colour
//   spinor F32 :  6 blocks of float4   -- block j = complex components 2j,2j+1
//   spinor F16 :  3 blocks of uint4    -- 8 halves = complex 4j..4j+3, values
//                 divided by a per-site float norm (max |real| of the site)
//   gauge  F64 : 4 mu x 9 double2, always complete; when every link is in
//                SU(3) (recon 12) kernels may read rows 0,1 only and rebuild
//                row 2 -- memory-bound kernels do, FP64-compute-bound ones
//                read all 9 and skip the rebuild
//   gauge  F32 : recon 12 -> 4 mu x 3 float4  ; recon 18 -> 4 mu x 9 float2
//   gauge  F16 : recon 12 -> 4 mu x 3 uint2 (4 halves each)
//
// A block has `stride` elements, stride = V rounded up to a multiple of 128;
// the padding sites hold zeros so whole-buffer reductions are exact.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <stdio.h>

#include <atomic>
#include <complex>
#include <string>

#include "../../include/qcdgpu.h"

namespace qg {

// ------------------------------------------------------------------ errors
void set_error(const char *fmt, ...);
// true when the allocation about to be made must fail (fault injection for
// tests, qcdgpu_inject_alloc_failures)
bool alloc_fault();
bool cuda_ok(cudaError_t e, const char *what);
#define QG_CUDA(call) ::qg::cuda_ok((call), #call)
#define QG_LAUNCHED(what) ::qg::after_launch(what)
bool after_launch(const char *what);
extern std::atomic<uint64_t> g_launches;

cudaStream_t stream();
cudaStream_t swap_stream(cudaStream_t s);  // returns the previous stream
inline void count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// the library's calls go to `s` while the scope lives
struct StreamScope {
  cudaStream_t prev;
  explicit StreamScope(cudaStream_t s) : prev(swap_stream(s)) {}
  ~StreamScope() { swap_stream(prev); }
  StreamScope(const StreamScope &) = delete;
  StreamScope &operator=(const StreamScope &) = delete;
};

// ------------------------------------------------------------------ fields
inline int64_t pad_stride(int64_t V) { return (V + 127) / 128 * 128; }

// The even/odd (checkerboard) decomposition holds on a periodic lattice only
// when every extent is even: across the boundary of an odd extent a site's
// neighbour has its own parity. The half fields pair the sites 2e, 2e + 1
// of a t-row, which needs the even t extent as well.
inline bool eo_lattice(const int L[4]) { return L[0] % 2 == 0 && L[1] % 2 == 0 && L[2] % 2 == 0 && L[3] % 2 == 0; }

// Internal gauge storage used by the float-float operator: every link entry
// as a float pair (re_hi, re_lo, im_hi, im_lo) in one float4, 4 mu x 9 blocks,
// with the boundary phase e^{i theta_mu / L_mu} already multiplied into the
// links of every direction whose theta is non-zero.
constexpr int kGaugeFF = 3;
// Internal key of the FP32 copy with all 18 reals per link (4 mu x 9 float2),
// read by the multi-RHS operator kernels, with the boundary phase
// e^{i theta_mu / L_mu} multiplied into the links (gauge_fold_phases).
constexpr int kGaugeF32Full = 4;
bool gauge_fold_phases(qcdgpu_gauge g);

}  // namespace qg

struct qcdgpu_field_s {
  int L[4];
  int64_t V;
  int64_t stride;
  int prec;
  void *data;
  float *norm;  // F16 only
  size_t bytes;
  bool view;    // data lies in another field's allocation (not freed with it)
};

struct qcdgpu_gauge_s {
  int L[4];
  int64_t V;
  int64_t stride;
  double theta[4];
  int prec;
  int recon;  // 12 or 18
  void *data;
  size_t bytes;
};

namespace qg {

// field allocation helpers (runtime.cu)
qcdgpu_field field_new(const int L[4], int prec);
// a field of lattice L whose data starts at `data`, inside an allocation
// the caller keeps alive (F64 or F32); field_free releases only the handle
qcdgpu_field field_view(const int L[4], int prec, void *data);
void field_free(qcdgpu_field f);
qcdgpu_gauge gauge_new(const int L[4], const double theta[4], int prec, int recon);
void gauge_free(qcdgpu_gauge g);
bool same_shape(qcdgpu_field a, qcdgpu_field b);

// pooled work fields (runtime.cu): returned fields are zero-free garbage
qcdgpu_field work_get(const int L[4], int prec);
void work_put(qcdgpu_field f);
void work_trim();  // frees the pooled fields

// scratch for reductions: 2 * kMaxPartials doubles + result slots
constexpr int kMaxPartials = 2048;
double *reduce_scratch();
double *host_result();  // pinned host slots, 64 doubles

// layout.cu
bool upload_spinor_aos(qcdgpu_field f, const double *host);
bool download_spinor_aos(qcdgpu_field f, double *host);
bool upload_gauge_aos(qcdgpu_gauge g, const double *host);  // decides recon
bool download_gauge_aos(qcdgpu_gauge g, double *host);
bool convert_field(qcdgpu_field dst, qcdgpu_field src);
// force_recon = 18 stores all 18 reals even for SU(3) links (FP32 targets)
bool convert_gauge(qcdgpu_gauge dst, qcdgpu_gauge src, int force_recon = 0);
// device staging buffer of at least `bytes` (single-threaded use) and the
// SU(3)-check + packing of a gauge field held there in the host layout
void *stage_buffer(size_t bytes);
bool pack_gauge(qcdgpu_gauge g, const void *dev_aos);
// the same conversions from / to the host layout held in device memory
bool spinor_from_aos_dev(qcdgpu_field f, const void *dev_aos);
bool spinor_to_aos_dev(qcdgpu_field f, void *dev_aos);
bool gauge_to_aos_dev(qcdgpu_gauge g, void *dev_aos);
// sites x0 .. x1-1 of an FP64 field from / to the host layout held in device
// memory (the whole field's array; only the range is touched)
bool spinor_from_aos_sites(qcdgpu_field f, const void *dev_aos, int64_t x0, int64_t x1);
bool spinor_to_aos_sites(qcdgpu_field f, void *dev_aos, int64_t x0, int64_t x1);
// dslash.cu: op D or Q on sites x0 .. x1-1 only
bool dslash_sites(qcdgpu_field out, qcdgpu_field in, qcdgpu_gauge g, double mp4, double tm, int op, int arith,
                  int x0, int x1);
// the same with the spinors in the host layout (12 double2 per site) at
// device addresses, float-float arithmetic; `shape` gives the lattice
bool dslash_sites_aos(void *out_aos, const void *in_aos, qcdgpu_field shape, qcdgpu_gauge g, double mp4, double tm,
                      int op, int x0, int x1);

// lime.cu: LIME files (ILDG gauge fields, ETMC spinors) <-> the host layout
// [V][4][3][3] / [V][4][3] complex double in device memory
bool lime_read_gauge(const char *fname, const int L[4], void *dev_aos);
bool lime_write_gauge(const char *fname, const int L[4], const void *dev_aos, const char *message);
bool lime_read_spinor(const char *fname, const int L[4], void *dev_aos);
// legacy CMI (type 0), HMC (1) and HMCV (2) vector files, column col (HMC)
bool legacy_read_spinor(const char *fname, const int L[4], int type, int col, void *dev_aos);
// CMI vector file (big-endian float32, [x][y][z][t][spin][colour][re, im])
bool cmi_write_spinor(const char *fname, const int L[4], const void *dev_aos);
bool lime_write_spinor(const char *fname, const int L[4], const void *dev_aos, bool source);

// dslash.cu: out = op(in) with diagonal mp4 = m + 4 and twisted mass tm
bool dslash(qcdgpu_field out, qcdgpu_field in, qcdgpu_gauge g, double mp4, double tm, int op,
            int arith);
// even/odd kernel on half fields {L_t/2, L_x, L_y, L_z} (native arithmetic):
// out (parity par) = ch * [A^{-1}] H in + {0 | z | A z}, A = mp4 + i tm g5
// arith: QCDGPU_ARITH_DF64 runs FP64 fields in float-float arithmetic
// with partials and fuse, the block that finishes last also forms the CG
// step alpha from the partials (dslash_args.h: CgFuse)
struct CgFuse;
bool dslash_eo(qcdgpu_field out, qcdgpu_field in, qcdgpu_field z, qcdgpu_gauge g, double mp4, double tm, bool dag,
               int par, double ch, bool ainv, int zmode, double *partials, int arith = QCDGPU_ARITH_F64,
               const CgFuse *fuse = nullptr);

// cg.cu: even/odd helpers -- full FP64 field <-> its two half fields, and
// out = A in or A^{-1} in on a half field (A = mp4 + i tm g5)
bool eo_split(qcdgpu_field e, qcdgpu_field o, qcdgpu_field full);
bool eo_merge(qcdgpu_field full, qcdgpu_field e, qcdgpu_field o);
bool eo_diag(qcdgpu_field out, qcdgpu_field in, double mp4, double tm, bool inverse);

// blas.cu (all precisions; arithmetic in the storage's working precision,
// reductions accumulated in double)
bool blas_zero(qcdgpu_field x);
bool blas_copy(qcdgpu_field dst, qcdgpu_field src);  // same precision
// out = a*x + b*y with complex a, b (out may alias x or y)
bool blas_axpby(qcdgpu_field out, double ar, double ai, qcdgpu_field x, double br, double bi,
                qcdgpu_field y);
bool blas_set(qcdgpu_field x, double cr, double ci);
bool blas_gamma5(qcdgpu_field out, qcdgpu_field in);
// out = i*g5*in  (spins 0,1 times +i, spins 2,3 times -i)
bool blas_ig5(qcdgpu_field out, qcdgpu_field in);
// reductions; result written to device slot res (double[2]) on the stream
bool blas_norm2_dev(qcdgpu_field x, double *res);
bool blas_dot_dev(qcdgpu_field a, qcdgpu_field b, double *res);
// host-returning versions (synchronise)
bool blas_norm2(qcdgpu_field x, double *out);
// FP64 fields: out[j] = <x_j, y> for j < k in one pass per 8 fields (host
// results, fixed summation order); y += sum_j a_j x_j in one pass per 8
bool blas_multi_dot(const qcdgpu_field *x, int k, qcdgpu_field y, std::complex<double> *out);
bool blas_multi_axpy(qcdgpu_field y, const qcdgpu_field *x, const std::complex<double> *a, int k);
bool blas_dot(qcdgpu_field a, qcdgpu_field b, double out[2]);
// fused: y = y + a*x  followed by |y|^2 (device result)
bool blas_axpy_norm2_dev(qcdgpu_field y, double ar, double ai, qcdgpu_field x, double *res);

// setup.cu
bool gauge_synthetic(qcdgpu_gauge g, uint64_t seed, double eps);
bool field_gaussian(qcdgpu_field f, uint64_t seed);
bool field_z4(qcdgpu_field f, uint64_t seed);
// Z2 (kind 2) or Z4 (kind 4) noise on time-slice tslice (all when negative)
bool field_noise(qcdgpu_field f, uint64_t seed, int tslice, int kind);
bool field_point(qcdgpu_field f, const int x[4], int spin, int colour);
double plaquette(qcdgpu_gauge g);

// smear.cu: one 3D APE step out <- in, and n Gaussian steps of v on
// time-slice t (both FP64)
bool ape3d(qcdgpu_gauge out, qcdgpu_gauge in, double alpha);
bool gauss3d(qcdgpu_field v, qcdgpu_gauge g, double alpha, int t, int n);

// solvers.cu
int solve(qcdgpu_field x, qcdgpu_field b, qcdgpu_gauge g, double mp4, double tm,
          qcdgpu_solve_params *p);
int gcr_dropin(qcdgpu_field sol, qcdgpu_field src, qcdgpu_gauge g, double mp4, double tm, int n,
               int shipped);

// low-precision copies of a gauge field made for mixed-precision solves;
// gauge_forget drops them (the field was reloaded or destroyed)
qcdgpu_gauge gauge_at(qcdgpu_gauge g, int prec);
void gauge_forget(qcdgpu_gauge g);

extern int g_gcr_shipped;
extern int g_f64_arith;

}  // namespace qg

// ------------------------------------------------------------ device helpers
namespace qgd {

template <typename R>
struct C {
  R re, im;
};

template <typename R>
__device__ __forceinline__ C<R> cmk(R a, R b) { return C<R>{a, b}; }
template <typename R>
__device__ __forceinline__ C<R> operator+(C<R> a, C<R> b) { return {a.re + b.re, a.im + b.im}; }
template <typename R>
__device__ __forceinline__ C<R> operator-(C<R> a, C<R> b) { return {a.re - b.re, a.im - b.im}; }
template <typename R>
__device__ __forceinline__ C<R> operator-(C<R> a) { return {-a.re, -a.im}; }
template <typename R>
__device__ __forceinline__ C<R> operator*(C<R> a, C<R> b)
{
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename R>
__device__ __forceinline__ C<R> operator*(R s, C<R> a) { return {s * a.re, s * a.im}; }
template <typename R>
__device__ __forceinline__ C<R> conj(C<R> a) { return {a.re, -a.im}; }
__device__ __forceinline__ float qfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double qfma(double a, double b, double c) { return __fma_rn(a, b, c); }

// i * a
template <typename R>
__device__ __forceinline__ C<R> mul_i(C<R> a) { return {-a.im, a.re}; }
// conj(a) * b
template <typename R>
__device__ __forceinline__ C<R> cdot(C<R> a, C<R> b)
{
  return {a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re};
}
// acc + a b, acc + conj(a) b and acc - a b as multiply-add chains into the
// accumulator: four FMAs, no separate product and add (a sum of three
// complex products costs 2 multiplies + 10 FMAs instead of 6 + 6 + 4 adds)
template <typename R>
__device__ __forceinline__ C<R> cmadd(C<R> a, C<R> b, C<R> acc)
{
  return {qfma(-a.im, b.im, qfma(a.re, b.re, acc.re)), qfma(a.im, b.re, qfma(a.re, b.im, acc.im))};
}
template <typename R>
__device__ __forceinline__ C<R> cmadd_conj(C<R> a, C<R> b, C<R> acc)
{
  return {qfma(a.im, b.im, qfma(a.re, b.re, acc.re)), qfma(-a.im, b.re, qfma(a.re, b.im, acc.im))};
}
template <typename R>
__device__ __forceinline__ C<R> cmsub(C<R> a, C<R> b, C<R> acc)
{
  return {qfma(a.im, b.im, qfma(-a.re, b.re, acc.re)), qfma(-a.im, b.re, qfma(-a.re, b.im, acc.im))};
}

// ---------------------------------------------------------- spinor access
// Spinor<P, R>::load fills s[12] (k = spin*3 + colour) in working precision R.
template <int P, typename R>
struct Spinor;

template <typename R>
struct Spinor<QCDGPU_F64, R> {
  __device__ __forceinline__ static void load(const void *base, const float *, int64_t stride,
                                              int64_t x, C<R> s[12])
  {
    const double2 *p = (const double2 *)base + x;
#pragma unroll
    for (int k = 0; k < 12; k++) {
      double2 v = __ldg(p + k * stride);
      s[k] = C<R>{(R)v.x, (R)v.y};
    }
  }
  __device__ __forceinline__ static void store(void *base, float *, int64_t stride, int64_t x,
                                               const C<R> s[12])
  {
    double2 *p = (double2 *)base + x;
#pragma unroll
    for (int k = 0; k < 12; k++) p[k * stride] = make_double2((double)s[k].re, (double)s[k].im);
  }
};

template <typename R>
struct Spinor<QCDGPU_F32, R> {
  __device__ __forceinline__ static void load(const void *base, const float *, int64_t stride,
                                              int64_t x, C<R> s[12])
  {
    const float4 *p = (const float4 *)base + x;
#pragma unroll
    for (int j = 0; j < 6; j++) {
      float4 v = __ldg(p + j * stride);
      s[2 * j] = C<R>{(R)v.x, (R)v.y};
      s[2 * j + 1] = C<R>{(R)v.z, (R)v.w};
    }
  }
  __device__ __forceinline__ static void store(void *base, float *, int64_t stride, int64_t x,
                                               const C<R> s[12])
  {
    float4 *p = (float4 *)base + x;
#pragma unroll
    for (int j = 0; j < 6; j++)
      p[j * stride] = make_float4((float)s[2 * j].re, (float)s[2 * j].im, (float)s[2 * j + 1].re,
                                  (float)s[2 * j + 1].im);
  }
};

template <typename R>
struct Spinor<QCDGPU_F16, R> {
  __device__ __forceinline__ static void load(const void *base, const float *norm, int64_t stride,
                                              int64_t x, C<R> s[12])
  {
    const uint4 *p = (const uint4 *)base + x;
    R nrm = (R)__ldg(norm + x);
#pragma unroll
    for (int j = 0; j < 3; j++) {
      uint4 v = __ldg(p + j * stride);
      const __half2 *h = reinterpret_cast<const __half2 *>(&v);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        float2 f = __half22float2(h[q]);
        s[4 * j + q] = C<R>{nrm * (R)f.x, nrm * (R)f.y};
      }
    }
  }
  __device__ __forceinline__ static void store(void *base, float *norm, int64_t stride, int64_t x,
                                               const C<R> s[12])
  {
    float m = 0.f;
#pragma unroll
    for (int k = 0; k < 12; k++) m = fmaxf(m, fmaxf(fabsf((float)s[k].re), fabsf((float)s[k].im)));
    // a site whose largest component is below the smallest normal float
    // (1.2e-38) is stored as zero: 1/m would overflow and 0 * inf is NaN
    if (!(m >= 1.17549435e-38f)) m = 0.f;
    float inv = m > 0.f ? 1.0f / m : 0.f;
    uint4 *p = (uint4 *)base + x;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      uint4 v;
      __half2 *h = reinterpret_cast<__half2 *>(&v);
#pragma unroll
      for (int q = 0; q < 4; q++)
        h[q] = __floats2half2_rn((float)s[4 * j + q].re * inv, (float)s[4 * j + q].im * inv);
      p[j * stride] = v;
    }
    norm[x] = m;
  }
};

// ------------------------------------------------------------ gauge access
// Link<P, RECON, R>::load fills U[9] (row-major 3x3) for link (x, mu).
template <int P, int RECON, typename R>
struct Link;

template <typename R>
__device__ __forceinline__ void rebuild_row2(C<R> U[9])
{
  // row2 = conj(row0 x row1), exact for U in SU(3)
  U[6] = conj(cmsub(U[2], U[4], U[1] * U[5]));
  U[7] = conj(cmsub(U[0], U[5], U[2] * U[3]));
  U[8] = conj(cmsub(U[1], U[3], U[0] * U[4]));
}

template <typename R>
struct Link<QCDGPU_F64, 18, R> {
  __device__ __forceinline__ static void load(const void *base, int64_t stride, int64_t x, int mu,
                                              C<R> U[9])
  {
    const double2 *p = (const double2 *)base + (int64_t)mu * 9 * stride + x;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      double2 v = __ldg(p + k * stride);
      U[k] = C<R>{(R)v.x, (R)v.y};
    }
  }
};
template <typename R>
struct Link<QCDGPU_F64, 12, R> {
  __device__ __forceinline__ static void load(const void *base, int64_t stride, int64_t x, int mu,
                                              C<R> U[9])
  {
    // FP64 links always hold all 9 entries; this reader takes rows 0 and 1
    const double2 *p = (const double2 *)base + (int64_t)mu * 9 * stride + x;
#pragma unroll
    for (int k = 0; k < 6; k++) {
      double2 v = __ldg(p + k * stride);
      U[k] = C<R>{(R)v.x, (R)v.y};
    }
    rebuild_row2(U);
  }
};
template <typename R>
struct Link<QCDGPU_F32, 12, R> {
  __device__ __forceinline__ static void load(const void *base, int64_t stride, int64_t x, int mu,
                                              C<R> U[9])
  {
    const float4 *p = (const float4 *)base + (int64_t)mu * 3 * stride + x;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      float4 v = __ldg(p + j * stride);
      U[2 * j] = C<R>{(R)v.x, (R)v.y};
      U[2 * j + 1] = C<R>{(R)v.z, (R)v.w};
    }
    rebuild_row2(U);
  }
};
template <typename R>
struct Link<QCDGPU_F32, 18, R> {
  __device__ __forceinline__ static void load(const void *base, int64_t stride, int64_t x, int mu,
                                              C<R> U[9])
  {
    const float2 *p = (const float2 *)base + (int64_t)mu * 9 * stride + x;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      float2 v = __ldg(p + k * stride);
      U[k] = C<R>{(R)v.x, (R)v.y};
    }
  }
};
template <typename R>
struct Link<QCDGPU_F16, 12, R> {
  __device__ __forceinline__ static void load(const void *base, int64_t stride, int64_t x, int mu,
                                              C<R> U[9])
  {
    const uint2 *p = (const uint2 *)base + (int64_t)mu * 3 * stride + x;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      uint2 v = __ldg(p + j * stride);
      const __half2 *h = reinterpret_cast<const __half2 *>(&v);
      float2 a = __half22float2(h[0]), b = __half22float2(h[1]);
      U[2 * j] = C<R>{(R)a.x, (R)a.y};
      U[2 * j + 1] = C<R>{(R)b.x, (R)b.y};
    }
    rebuild_row2(U);
  }
};

// site coordinates (t fastest) and neighbour offsets with periodic wrap
// Lattice geometry for kernels. Site indices fit in 32 bits (the library
// rejects volumes of 2^31 sites or more), so coordinates are recovered with
// 32-bit unsigned divisions.
struct Geom {
  int L[4];
  int st[4];  // 1, Lt, Lt*Lx, Lt*Lx*Ly
};

__device__ __forceinline__ void coords(const Geom &g, int x, int c[4])
{
  unsigned r = (unsigned)x;
  unsigned q = r / (unsigned)g.L[0];
  c[0] = (int)(r - q * (unsigned)g.L[0]);
  r = q;
  q = r / (unsigned)g.L[1];
  c[1] = (int)(r - q * (unsigned)g.L[1]);
  r = q;
  q = r / (unsigned)g.L[2];
  c[2] = (int)(r - q * (unsigned)g.L[2]);
  c[3] = (int)q;
}
__device__ __forceinline__ int fwd(const Geom &g, int x, const int c[4], int mu)
{
  return c[mu] == g.L[mu] - 1 ? x - (g.L[mu] - 1) * g.st[mu] : x + g.st[mu];
}
__device__ __forceinline__ int bwd(const Geom &g, int x, const int c[4], int mu)
{
  return c[mu] == 0 ? x + (g.L[mu] - 1) * g.st[mu] : x - g.st[mu];
}

}  // namespace qgd
