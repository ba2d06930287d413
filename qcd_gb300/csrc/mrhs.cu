// mrhs.cu -- many right-hand sides sharing one gauge-field read.
//
// A multi-RHS field holds N spinors in FP16 with one float norm per
// (site, RHS), laid out [component 0..11][site][rhs] as half2 (re, im), so
// the RHS of one site and component are contiguous.
//
// Operator: three kernels, picked per (volume, slot count) by timing. SIMT:
// one thread per site and one or two slots, links shared through L1.
// tcgen05: one FP16 GEMM per site with the eight hops concatenated along K
// (see k_wilson_mrhs_tc). mma.sync (below): one warp per site. For each of
// the eight hops the warp builds, for 16 RHS at a time, the matrix A (16 RHS x 12 reals of the
// projected half spinor, padded to 16) and multiplies it with
//   B = realified ( R_mu (x) U_mu )   (12 x 24, padded to 16 x 24)
// where U_mu is the link (or U^+ for backward hops, phase e^{+-i th/L}
// folded in) and R_mu the 4 x 2 spin matrix that rebuilds the lower spinor
// half from the upper one (qcd_wilson.h:17-387). The eight products
// accumulate in the same FP32 MMA accumulators (mma.sync m16n8k8, TF32
// operands), so the link is read once per site for all N RHS and the
// per-RHS arithmetic runs on the tensor pipe; the diagonal term and the FP16
// re-normalisation are the epilogue. TF32 keeps the FP32 exponent range, so
// small residual vectors need no rescaling.
#include <string.h>

#include <map>
#include <utility>

#include "mrhs.h"
#include "wilson_kernel.cuh"

namespace qg {

using namespace qgd;

struct MArgs {
  __half2 *out;
  float *out_norm;
  const __half2 *in;
  const float *in_norm;
  const float2 *gauge;  // FP32, 4 mu x 9 float2 blocks
  Geom geo;
  int V, N, nact;
  int64_t gstride;
  float phr[4], phi[4];
  int twist_mask;
  float mp4, tm;  // tm negated for D^+
  // per-slot diagonal (m+4 and tm of each RHS) when non-null; the hopping
  // term does not depend on kappa or mu, so one batch may mix both
  const float *mp4s, *tms;
  // SIMT kernel epilogue: out = ch * [A^{-1}] H in + {0 | z | A z} with A the
  // slot's diagonal (m+4) + i tm g5; the full-lattice operator is ch = -1/2,
  // z = in, zmode 2. Even/odd kernels: sites of parity eo_par, fields on the
  // half lattice (V = half volume) indexed by (full site index) >> 1.
  const __half2 *z;
  const float *z_norm;
  int zmode, ainv, eo_par;
  float ch;
};

__device__ __forceinline__ float2 mload(const __half2 *d, const float *nrm, int V, int N, int k, int site, int r)
{
  float2 f = __half22float2(d[mhalf2_index(V, N, k, site, r)]);
  float s = nrm[(int64_t)site * N + r];
  return make_float2(f.x * s, f.y * s);
}

__device__ __forceinline__ unsigned to_tf32(float x)
{
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void mma_tf32(float c[4], const unsigned a[4], unsigned b0, unsigned b1)
{
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// MT = number of 16-RHS tiles (N <= 16 MT)
template <bool DAG, int MT>
__global__ void __launch_bounds__(128) k_wilson_mrhs(const MArgs a)
{
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int x = blockIdx.x * 4 + wp;
  if (x >= a.V) return;  // the whole warp leaves together
  const int g = lane >> 2, t = lane & 3;
  int c[4];
  coords(a.geo, x, c);
  float acc[MT][3][4];
#pragma unroll
  for (int m = 0; m < MT; m++)
#pragma unroll
    for (int n = 0; n < 3; n++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[m][n][q] = 0.f;
  constexpr int SF = DAG ? +1 : -1;
#pragma unroll 1
  for (int d = 0; d < 8; d++) {
    const int mu = d >> 1;
    const bool back = d & 1;
    const int S = back ? -SF : SF;
    const int cm = mu == 0 ? c[0] : mu == 1 ? c[1] : mu == 2 ? c[2] : c[3];
    const int Lm = a.geo.L[mu], st = a.geo.st[mu];
    int y;
    if (back) y = cm == 0 ? x + (Lm - 1) * st : x - st;
    else y = cm == Lm - 1 ? x - (Lm - 1) * st : x + st;
    const int ly = back ? y : x;
    // spin structure of (1 + S g_mu): see wilson_kernel / dslash_df64 tables
    const bool odd = mu & 1;
    const int b0 = (mu == 0 || mu == 3) ? 2 : 3, b1 = 5 - b0;
    const bool neg0 = S > 0, neg1 = mu < 2 ? S > 0 : S < 0;
    const int jA = (mu == 1 || mu == 2) ? 1 : 0;
    const bool negA = mu == 0 ? S > 0 : S < 0, negB = mu == 1 ? S < 0 : S > 0;
    const bool tw = (a.twist_mask >> mu) & 1;
    const float pr = a.phr[mu], pi = back ? -a.phi[mu] : a.phi[mu];
    // B fragments: element (row kk, col n) of the realified R (x) U
    unsigned bf[2][3][2];
#pragma unroll
    for (int ks = 0; ks < 2; ks++)
#pragma unroll
      for (int nt = 0; nt < 3; nt++)
#pragma unroll
        for (int hf = 0; hf < 2; hf++) {
          const int kk = 8 * ks + t + 4 * hf, n = 8 * nt + g;
          float v = 0.f;
          if (kk < 12) {
            const int j = kk / 6, cp = (kk % 6) >> 1, rip = kk & 1;
            const int s = n / 6, cc = (n % 6) >> 1, ri = n & 1;
            bool nz, rodd = false, rneg = false;
            if (s < 2) {
              nz = s == j;
            } else if (s == 2) {
              nz = j == jA;
              rodd = odd;
              rneg = negA;
            } else {
              nz = j == 1 - jA;
              rodd = odd;
              rneg = negB;
            }
            if (nz) {
              float2 u = __ldg(a.gauge + ((int64_t)mu * 9 + (back ? 3 * cp + cc : 3 * cc + cp)) * a.gstride + ly);
              float wr = u.x, wi = back ? -u.y : u.y;
              if (tw) {
                float tr = wr * pr - wi * pi;
                wi = wr * pi + wi * pr;
                wr = tr;
              }
              if (rodd) {
                float tr = -wi;
                wi = wr;
                wr = tr;
              }
              if (rneg) {
                wr = -wr;
                wi = -wi;
              }
              v = rip == 0 ? (ri == 0 ? wr : wi) : (ri == 0 ? -wi : wr);
            }
          }
          bf[ks][nt][hf] = to_tf32(v);
        }
#pragma unroll
    for (int m = 0; m < MT; m++) {
      float hv[2][3];
#pragma unroll
      for (int row = 0; row < 2; row++) {
        const int r = 16 * m + g + 8 * row;
#pragma unroll
        for (int q = 0; q < 3; q++) {
          const int kk = t + 4 * q, j = kk / 6, cc = (kk % 6) >> 1;
          float val = 0.f;
          if (r < a.nact) {
            float2 p = mload(a.in, a.in_norm, a.V, a.N, 3 * j + cc, y, r);
            float2 pb = mload(a.in, a.in_norm, a.V, a.N, 3 * (j == 0 ? b0 : b1) + cc, y, r);
            if (odd) pb = make_float2(-pb.y, pb.x);
            if (j == 0 ? neg0 : neg1) pb = make_float2(-pb.x, -pb.y);
            val = (t & 1) ? p.y + pb.y : p.x + pb.x;
          }
          hv[row][q] = val;
        }
      }
      const unsigned a0[4] = {to_tf32(hv[0][0]), to_tf32(hv[1][0]), to_tf32(hv[0][1]), to_tf32(hv[1][1])};
      const unsigned a1[4] = {to_tf32(hv[0][2]), to_tf32(hv[1][2]), 0u, 0u};
#pragma unroll
      for (int nt = 0; nt < 3; nt++) {
        mma_tf32(acc[m][nt], a0, bf[0][nt][0], bf[0][nt][1]);
        mma_tf32(acc[m][nt], a1, bf[1][nt][0], bf[1][nt][1]);
      }
    }
  }
  // epilogue: out = (m+4) psi + i tm g5 psi - acc/2, stored as FP16 + norm
#pragma unroll
  for (int m = 0; m < MT; m++)
#pragma unroll
    for (int row = 0; row < 2; row++) {
      const int r = 16 * m + g + 8 * row;
      const bool live = r < a.nact;
      const float mp4r = (a.mp4s && live) ? a.mp4s[r] : a.mp4;
      const float tmr = (a.tms && live) ? (DAG ? -a.tms[r] : a.tms[r]) : a.tm;
      float2 o[3];
      float mx = 0.f;
#pragma unroll
      for (int nt = 0; nt < 3; nt++) {
        const int q = 4 * nt + t, s = q / 3;
        float2 cq = make_float2(acc[m][nt][2 * row], acc[m][nt][2 * row + 1]);
        float2 ps = live ? mload(a.in, a.in_norm, a.V, a.N, q, x, r) : make_float2(0.f, 0.f);
        const float g5tm = s < 2 ? tmr : -tmr;
        o[nt] = make_float2(mp4r * ps.x - g5tm * ps.y - 0.5f * cq.x, mp4r * ps.y + g5tm * ps.x - 0.5f * cq.y);
        mx = fmaxf(mx, fmaxf(fabsf(o[nt].x), fabsf(o[nt].y)));
      }
      // the 12 components of RHS r are spread over the 4 lanes of its quad
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 2));
      if (!(mx >= 1.17549435e-38f)) mx = 0.f;
      const float inv = mx > 0.f ? 1.0f / mx : 0.f;
      if (live) {
#pragma unroll
        for (int nt = 0; nt < 3; nt++) {
          const int q = 4 * nt + t;
          a.out[mhalf2_index(a.V, a.N, q, x, r)] = __floats2half2_rn(o[nt].x * inv, o[nt].y * inv);
        }
        if (t == 0) a.out_norm[(int64_t)x * a.N + r] = mx;
      }
    }
}

// ------------------------------------------------ SIMT variant (FP32 cores)
// One thread per site and RP adjacent RHS slots, block (N / RP threads, SB
// sites): the threads of one site read the same links (L1 broadcast), so
// the gauge field is fetched once per site for all RHS, while the per-RHS
// spin projection, link products and reconstruction run as FP32 FMAs. With
// RP = 2 a thread loads the two slots' half2 values of a component as one
// 8-byte word and applies each link it loads to both. With `partials` the
// epilogue also writes, per block and slot, the sum of |out|^2 over the
// block's sites (partials[block * N + slot]) in a fixed order.
template <int RP>
__device__ __forceinline__ void mload_rp(const MArgs &a, const __half2 *d, const float *dn, int y, int r0,
                                         C<float> s[RP][12], float nrm[RP])
{
  if (RP == 2) {
    const float2 n2 = *(const float2 *)(dn + (int64_t)y * a.N + r0);
    nrm[0] = n2.x;
    nrm[RP - 1] = n2.y;
  } else {
    nrm[0] = dn[(int64_t)y * a.N + r0];
  }
#pragma unroll
  for (int q = 0; q < RP; q++) {
    float2 v[12];
    mload_raw(d, a.V, a.N, y, r0 + q, v);
#pragma unroll
    for (int k = 0; k < 12; k++) s[q][k] = C<float>{v[k].x, v[k].y};
  }
}

// h = nrm * upper half of (1 + S g_mu) s for the spinor s held as its three
// 16-byte words, projected on packed half pairs (as the single-RHS FP16
// kernel does)
template <int MU, int S>
__device__ __forceinline__ void project_words(const uint4 w[3], float nrm, C<float> h[6])
{
  const __half2 *hv = reinterpret_cast<const __half2 *>(w);
  constexpr bool IM = MU & 1;
  constexpr int B0 = (MU == 0 || MU == 3) ? 2 : 3, B1 = 5 - B0;
  constexpr int SG0 = S > 0 ? -1 : 1, SG1 = MU < 2 ? SG0 : -SG0;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const float2 f0 = __half22float2(hcomb<IM>(hv[c], hv[3 * B0 + c], SG0));
    const float2 f1 = __half22float2(hcomb<IM>(hv[3 + c], hv[3 * B1 + c], SG1));
    h[c] = C<float>{nrm * f0.x, nrm * f0.y};
    h[3 + c] = C<float>{nrm * f1.x, nrm * f1.y};
  }
}

// the same for slot r of the multi-RHS spinor at y
template <int MU, int S>
__device__ __forceinline__ void mload_project(const __half2 *d, int64_t V, int N, int y, int r, float nrm,
                                              C<float> h[6])
{
  const uint4 *p = (const uint4 *)d;
  uint4 w[3];
#pragma unroll
  for (int j = 0; j < 3; j++) w[j] = p[((int64_t)j * V + y) * N + r];
  project_words<MU, S>(w, nrm, h);
}

template <int MU, bool DAG, int RP, bool EO>
__device__ __forceinline__ void mhop_pair(const MArgs &a, int x, const int c[4], int r0, C<float> acc[RP][12])
{
  constexpr int SF = DAG ? +1 : -1;
  const bool twisted = (a.twist_mask >> MU) & 1;
#pragma unroll
  for (int dir = 0; dir < 2; dir++) {
    const bool back = dir == 1;
    const int y = back ? bwd(a.geo, x, c, MU) : fwd(a.geo, x, c, MU);
    C<float> U[9];
    const int ys = EO ? (y >> 1) : y;
    float nrm[RP];
    if (RP == 2) {
      const float2 n2 = *(const float2 *)(a.in_norm + (int64_t)ys * a.N + r0);
      nrm[0] = n2.x;
      nrm[RP - 1] = n2.y;
    } else {
      nrm[0] = a.in_norm[(int64_t)ys * a.N + r0];
    }
    Link<QCDGPU_F32, 18, float>::load(a.gauge, a.gstride, back ? y : x, MU, U);
#pragma unroll
    for (int q = 0; q < RP; q++) {
      C<float> h[6], uh[6];
      // the projection adds the stored half pairs, then the six projected
      // components are converted and scaled by the slot's site norm
      if (back) mload_project<MU, -SF>(a.in, a.V, a.N, ys, r0 + q, nrm[q], h);
      else mload_project<MU, SF>(a.in, a.V, a.N, ys, r0 + q, nrm[q], h);
#pragma unroll
      for (int j = 0; j < 2; j++)
#pragma unroll
        for (int i = 0; i < 3; i++)
          uh[3 * j + i] = back ? cdot(U[i], h[3 * j]) + cdot(U[3 + i], h[3 * j + 1]) + cdot(U[6 + i], h[3 * j + 2])
                               : U[3 * i] * h[3 * j] + U[3 * i + 1] * h[3 * j + 1] + U[3 * i + 2] * h[3 * j + 2];
      if (twisted) {
        C<float> ph{a.phr[MU], back ? -a.phi[MU] : a.phi[MU]};
#pragma unroll
        for (int k = 0; k < 6; k++) uh[k] = uh[k] * ph;
      }
      if (back) accumulate<MU, -SF>(acc[q], uh);
      else accumulate<MU, SF>(acc[q], uh);
    }
  }
}

// MODE 0: full lattice, out = A in - H in / 2. Even/odd (half fields): MODE 1
// out = A^{-1} H in; MODE 2 out = A z - H in / 4 (the two halves of the Schur
// complement). The epilogue is fixed at compile time for each mode.
template <bool DAG, int RP, int MODE>
__global__ void __launch_bounds__(256, 2) k_wilson_mrhs_simt(const MArgs a, double *partials)
{
  constexpr bool EO = MODE != 0;
  const int r0 = threadIdx.x * RP;
  const int e = blockIdx.x * blockDim.y + threadIdx.y;  // output index
  double n2[RP];
#pragma unroll
  for (int q = 0; q < RP; q++) n2[q] = 0.0;
  if (r0 < a.nact && e < a.V) {
    int c[4], x = e;
    if (EO) {  // the site of parity eo_par among full indices 2e, 2e + 1 (even t extent)
      coords(a.geo, 2 * e, c);
      const int b = (a.eo_par ^ c[1] ^ c[2] ^ c[3]) & 1;
      x = 2 * e + b;
      c[0] += b;
    } else {
      coords(a.geo, x, c);
    }
    C<float> acc[RP][12];
#pragma unroll
    for (int q = 0; q < RP; q++)
#pragma unroll
      for (int k = 0; k < 12; k++) acc[q][k] = C<float>{0.f, 0.f};
    mhop_pair<0, DAG, RP, EO>(a, x, c, r0, acc);
    mhop_pair<1, DAG, RP, EO>(a, x, c, r0, acc);
    mhop_pair<2, DAG, RP, EO>(a, x, c, r0, acc);
    mhop_pair<3, DAG, RP, EO>(a, x, c, r0, acc);
    constexpr int zmode = MODE == 1 ? 0 : 2;
    constexpr bool ainv = MODE == 1;
    constexpr float ch = MODE == 0 ? -0.5f : MODE == 1 ? 1.0f : -0.25f;
    C<float> s[RP][12];
    float nrm[RP];
    if (zmode) mload_rp<RP>(a, EO ? a.z : a.in, EO ? a.z_norm : a.in_norm, e, r0, s, nrm);
#pragma unroll
    for (int q = 0; q < RP; q++) {
      const int r = r0 + q;
      // slots past nact hold zeros; their results are not stored
      const float mp4r = a.mp4s ? a.mp4s[r] : a.mp4;
      const float tmr = a.tms ? (DAG ? -a.tms[r] : a.tms[r]) : a.tm;
      if (ainv) {  // A^{-1} = (mp4 - i tm g5) / (mp4^2 + tm^2)
        const float den = 1.0f / (mp4r * mp4r + tmr * tmr), ar = mp4r * den, ai = -tmr * den;
#pragma unroll
        for (int k = 0; k < 12; k++) {
          const float g5ai = k < 6 ? ai : -ai;
          acc[q][k] = C<float>{ar * acc[q][k].re - g5ai * acc[q][k].im, ar * acc[q][k].im + g5ai * acc[q][k].re};
        }
      }
      const float zs = zmode ? nrm[q] : 0.f;
      const float zm = zmode == 2 ? mp4r * zs : zs, zt = zmode == 2 ? tmr * zs : 0.f;
      float mx = 0.f;
#pragma unroll
      for (int k = 0; k < 12; k++) {
        const float g5tm = k < 6 ? zt : -zt;
        const C<float> zk = zmode ? s[q][k] : C<float>{0.f, 0.f};
        acc[q][k] = C<float>{zm * zk.re - g5tm * zk.im + ch * acc[q][k].re,
                             zm * zk.im + g5tm * zk.re + ch * acc[q][k].im};
        mx = fmaxf(mx, fmaxf(fabsf(acc[q][k].re), fabsf(acc[q][k].im)));
      }
      if (!(mx >= 1.17549435e-38f)) mx = 0.f;
      const float inv = mx > 0.f ? 1.0f / mx : 0.f;
      if (r < a.nact) {
        float2 o[12];
#pragma unroll
        for (int k = 0; k < 12; k++) o[k] = make_float2(acc[q][k].re, acc[q][k].im);
        mstore_raw(a.out, a.V, a.N, e, r, o, inv);
        float s2 = 0.f;
        if (partials) {  // |out|^2 of the stored (rounded) values
#pragma unroll
          for (int k = 0; k < 12; k++) {
            const float2 f = __half22float2(__floats2half2_rn(o[k].x * inv, o[k].y * inv));
            s2 += f.x * f.x + f.y * f.y;
          }
        }
        a.out_norm[(int64_t)e * a.N + r] = mx;
        n2[q] = (double)(s2 * mx * mx);  // per-site sum in FP32, block sum in double
      }
    }
  }
  if (partials) {
    // the block covers slots 0 .. NS-1 (the occupied ones); partials keep
    // the field's slot stride N
    extern __shared__ double sh[];
    const int N = a.N, y = threadIdx.y, NS = min(N, (int)blockDim.x * RP);
#pragma unroll
    for (int q = 0; q < RP; q++)
      if (threadIdx.x * RP + q < NS) sh[y * NS + threadIdx.x * RP + q] = n2[q];
    __syncthreads();
    for (int r = threadIdx.x; r < NS; r += blockDim.x)
      if (y == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)blockDim.y; i++) t += sh[i * NS + r];
        partials[(int64_t)blockIdx.x * N + r] = t;
      }
  }
}

// ------------------------------------------------------------ fields
qcdgpu_mfield mfield_new(const int L[4], int N)
{
  if (N < 1 || N > 64) {
    set_error("multi-RHS fields hold 1..64 right-hand sides (got %d)", N);
    return nullptr;
  }
  qcdgpu_field probe = field_new(L, QCDGPU_F16);  // validates L and the volume
  if (!probe) return nullptr;
  field_free(probe);
  auto *m = new qcdgpu_mfield_s();
  memcpy(m->L, L, sizeof(m->L));
  m->V = (int64_t)L[0] * L[1] * L[2] * L[3];
  m->N = N;
  size_t nd = (size_t)12 * m->V * N * sizeof(__half2), nn = (size_t)m->V * N * sizeof(float);
  m->bytes = nd + nn;
  if (!QG_CUDA(cudaMalloc(&m->data, m->bytes))) {
    delete m;
    return nullptr;
  }
  m->norm = (float *)((char *)m->data + nd);
  if (!QG_CUDA(cudaMemsetAsync(m->data, 0, m->bytes, stream()))) {
    cudaFree(m->data);
    delete m;
    return nullptr;
  }
  return m;
}

void mfield_free(qcdgpu_mfield m)
{
  if (!m) return;
  cudaFree(m->data);
  delete m;
}

// slot r of m <- f (f in any storage precision)
template <int P>
__global__ void k_pack(__half2 *d, float *dn, int V, int N, int r, const void *f, const float *fn, int64_t stride)
{
  int x = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (x >= V) return;
  C<float> s[12];
  Spinor<P, float>::load(f, fn, stride, x, s);
  float mx = 0.f;
#pragma unroll
  for (int k = 0; k < 12; k++) mx = fmaxf(mx, fmaxf(fabsf(s[k].re), fabsf(s[k].im)));
  if (!(mx >= 1.17549435e-38f)) mx = 0.f;
  float inv = mx > 0.f ? 1.0f / mx : 0.f;
  float2 v[12];
#pragma unroll
  for (int k = 0; k < 12; k++) v[k] = make_float2(s[k].re, s[k].im);
  mstore_raw(d, V, N, x, r, v, inv);
  dn[(int64_t)x * N + r] = mx;
}

// f <- slot r of m
template <int P>
__global__ void k_unpack(void *f, float *fn, int64_t stride, const __half2 *d, const float *dn, int V, int N, int r)
{
  int x = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (x >= V) return;
  C<double> s[12];
#pragma unroll
  for (int k = 0; k < 12; k++) {
    float2 v = mload(d, dn, V, N, k, x, r);
    s[k] = C<double>{(double)v.x, (double)v.y};
  }
  Spinor<P, double>::store(f, fn, stride, x, s);
}

bool mfield_set(qcdgpu_mfield m, int r, qcdgpu_field f)
{
  if (!m || !f || r < 0 || r >= m->N || f->V != m->V) {
    set_error("multi-RHS set: bad slot or shape");
    return false;
  }
  unsigned g = (unsigned)((m->V + 127) / 128);
  __half2 *d = (__half2 *)m->data;
  if (f->prec == QCDGPU_F64) k_pack<QCDGPU_F64><<<g, 128, 0, stream()>>>(d, m->norm, (int)m->V, m->N, r, f->data, f->norm, f->stride);
  else if (f->prec == QCDGPU_F32) k_pack<QCDGPU_F32><<<g, 128, 0, stream()>>>(d, m->norm, (int)m->V, m->N, r, f->data, f->norm, f->stride);
  else k_pack<QCDGPU_F16><<<g, 128, 0, stream()>>>(d, m->norm, (int)m->V, m->N, r, f->data, f->norm, f->stride);
  return QG_LAUNCHED("mrhs_pack");
}

bool mfield_get(qcdgpu_field f, qcdgpu_mfield m, int r)
{
  if (!m || !f || r < 0 || r >= m->N || f->V != m->V) {
    set_error("multi-RHS get: bad slot or shape");
    return false;
  }
  unsigned g = (unsigned)((m->V + 127) / 128);
  const __half2 *d = (const __half2 *)m->data;
  if (f->prec == QCDGPU_F64) k_unpack<QCDGPU_F64><<<g, 128, 0, stream()>>>(f->data, f->norm, f->stride, d, m->norm, (int)m->V, m->N, r);
  else if (f->prec == QCDGPU_F32) k_unpack<QCDGPU_F32><<<g, 128, 0, stream()>>>(f->data, f->norm, f->stride, d, m->norm, (int)m->V, m->N, r);
  else k_unpack<QCDGPU_F16><<<g, 128, 0, stream()>>>(f->data, f->norm, f->stride, d, m->norm, (int)m->V, m->N, r);
  return QG_LAUNCHED("mrhs_unpack");
}

// out = D in (dag: D^+ in) for the first nact RHS of the two fields; with
// mp4s / tms (device float arrays) each slot r uses its own diagonal
// ------------------------------------------------------------ launch + tuner
// per-slot sum of |v|^2 over the block's sites (for the tensor-core variant,
// whose epilogue has no reduction); block (N, SB) like the SIMT variant
__global__ void k_mnorm(const __half2 *d, const float *dn, int V, int N, int nact, double *partials)
{
  const int r = threadIdx.x, x = blockIdx.x * blockDim.y + threadIdx.y;
  double n2 = 0.0;
  if (r < nact && x < V) {
    const float s = dn[(int64_t)x * N + r];
    float s2 = 0.f;  // per-site sum in FP32, block sum in double
#pragma unroll
    for (int k = 0; k < 12; k++) {
      float2 f = __half22float2(d[mhalf2_index(V, N, k, x, r)]);
      s2 += (f.x * s) * (f.x * s) + (f.y * s) * (f.y * s);
    }
    n2 = (double)s2;
  }
  extern __shared__ double sh[];
  const int y = threadIdx.y;
  sh[y * N + r] = n2;
  __syncthreads();
  if (y == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)blockDim.y; i++) t += sh[i * N + r];
    partials[(int64_t)blockIdx.x * N + r] = t;
  }
}

// ------------------------------------------------- tensor cores (tcgen05)
// One GEMM per site and 16-slot group holds all eight hops:
//   D^T (24 x 16) = L (24 x 96) H^T (96 x 16),
// FP16 operands, FP32 accumulator in tensor memory. Row o = (spin S, colour
// i, re/im) of L is the site's link matrix: in K block h (12 values: input
// spin s, colour j, re/im) it holds the realified c M_ij, where M = U_mu (or
// U_mu^+ for backward hops, boundary phase folded in) and c the entry (0, 1,
// +-1 or +-i) of the 4 x 2 matrix that rebuilds spin S from the projected
// upper half of (1 +- g_mu); L is built once per site for all slots. Row n of
// H is slot n's projected half spinor at each of the eight neighbours (packed
// half pairs, as the FP16 kernels project them), scaled by that neighbour's
// norm over the slot's largest. The MMA is issued with M = 64 (the smallest
// M): rows 24..63 of the A operand read whatever follows in shared memory and
// land in accumulator rows that are never read. Per tile of 8 sites: 128
// threads build L (two threads per site and hop) and H (one thread per site
// and slot), one thread issues 8 x 6 MMAs (M = 64, N = 16, K = 16) into 128
// tensor-memory columns and commits them to an mbarrier, warps 0 and 1 read
// the 24 accumulator rows back, and the epilogue (diagonal term, A^{-1}, FP16
// rounding with per-site norm, per-slot |out|^2) runs one thread per site and
// slot. The slot's rescale factor multiplies the accumulator back.
constexpr int kTcSites = 8;     // sites per tile (one MMA chain each)
constexpr int kTcTiles = 16;    // tiles per CTA
constexpr int kTcThreads = 128;
constexpr int kTcK = 96;                                       // 8 hops x 12
constexpr uint32_t kTcSbo = (kTcK / 8) * 128;                  // bytes per 8-row group
constexpr size_t kTcLBytes = (size_t)kTcSites * 3 * kTcSbo;    // 24 rows per site
constexpr size_t kTcHBytes = (size_t)kTcSites * 2 * kTcSbo;    // 16 rows per site
constexpr size_t kTcSmem = kTcLBytes + kTcHBytes + sizeof(double) * kTcSites * 16;
// the M = 64 operand of the last site reads 64 rows from its start: inside the allocation
static_assert((kTcSites - 1) * 3 * kTcSbo + 8 * kTcSbo <= kTcSmem, "tcgen05 A operand overruns shared memory");

__device__ unsigned g_mrhs_tc_timeouts;  // rounds abandoned after a bounded mbarrier wait

// launch controls of the tensor-core kernel: the bound of each wait for the
// MMAs (mbarrier polls), a test hook that issues no MMA (so the waits run
// out), and a host-mapped flag the kernel sets when a wait ran out
struct TcCtl {
  int polls;
  int skip_mma;
  volatile unsigned *fail;
};

__device__ __forceinline__ uint32_t tc_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: no swizzle, K-major core matrices of 8
// rows x 16 bytes; lbo = byte step between K-adjacent core matrices, sbo =
// byte step between 8-row groups; bits 46-48 hold the fixed value 0b001
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B FP16
// (bits 7-12 = 0), both K-major (bits 15, 16 = 0), N >> 3 at bit 17, M >> 4
// at bit 24
constexpr uint32_t tc_idesc(int M, int N) { return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24); }

__device__ __forceinline__ uint32_t pack_h2(float a, float b)
{
  const __half2 h = __floats2half2_rn(a, b);
  return *(const uint32_t *)&h;
}

// shared stores that the compiler may reorder against global loads (the
// tensor cores read them after a fence and a barrier)
__device__ __forceinline__ void sts128(uint32_t a, uint32_t x, uint32_t y, uint32_t z, uint32_t w)
{
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(a), "r"(x), "r"(y), "r"(z), "r"(w));
}
__device__ __forceinline__ void sts64(uint32_t a, uint32_t x, uint32_t y)
{
  asm volatile("st.shared.v2.b32 [%0], {%1, %2};" ::"r"(a), "r"(x), "r"(y));
}

// the 12 halves (6 words) v of K block h in the row at `row` (address of
// the row inside its core-matrix group): block h starts at K = 12 h, i.e.
// at a whole core matrix (h even) or half-way through one (h odd)
__device__ __forceinline__ void tc_put12(uint32_t row, int h, const uint32_t v[6])
{
  const uint32_t c = (uint32_t)(12 * h) >> 3;  // first core matrix
  if ((h & 1) == 0) {
    sts128(row + c * 128, v[0], v[1], v[2], v[3]);
    sts64(row + (c + 1) * 128, v[4], v[5]);
  } else {
    sts64(row + c * 128 + 8, v[0], v[1]);
    sts128(row + (c + 1) * 128, v[2], v[3], v[4], v[5]);
  }
}

// entry (c, source spin) of the matrix that rebuilds spin sp (0..3) from the
// projected upper half of (1 + S g_mu) (the rules of accumulate<MU, S>)
__device__ __forceinline__ void tc_rebuild(int mu, int S, int sp, int &src, float &cr, float &ci)
{
  const float s = (float)S;
  cr = 0.f;
  ci = 0.f;
  if (sp < 2) {
    src = sp;
    cr = 1.f;
  } else if (mu == 0) {
    src = sp - 2;
    cr = -s;
  } else if (mu == 1) {
    src = 3 - sp;
    ci = s;
  } else if (mu == 2) {
    src = 3 - sp;
    cr = sp == 2 ? s : -s;
  } else {
    src = sp - 2;
    ci = sp == 2 ? s : -s;
  }
}

// neighbour of x in hop dd (2 mu + backward)
__device__ __forceinline__ int tc_nb(const Geom &g, int x, const int c[4], int dd)
{
  return (dd & 1) ? bwd(g, x, c, dd >> 1) : fwd(g, x, c, dd >> 1);
}

// slot r's row of H, K block DD: the projected half spinor at neighbour ys,
// scaled by sc2
template <bool DAG, int DD>
__device__ __forceinline__ void tc_h_block(const MArgs &a, int ys, int r, __half2 sc2, uint32_t row)
{
  constexpr int MU = DD >> 1, SF = DAG ? +1 : -1, S = (DD & 1) ? -SF : SF;
  constexpr bool IM = MU & 1;
  constexpr int B0 = (MU == 0 || MU == 3) ? 2 : 3, B1 = 5 - B0;
  constexpr int SG0 = S > 0 ? -1 : 1, SG1 = MU < 2 ? SG0 : -SG0;
  const uint4 *p = (const uint4 *)a.in;
  uint4 w[3];
#pragma unroll
  for (int j = 0; j < 3; j++) w[j] = p[((int64_t)j * a.V + ys) * a.N + r];
  const __half2 *hv = reinterpret_cast<const __half2 *>(w);
  uint32_t v[6];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const __half2 h0 = __hmul2(hcomb<IM>(hv[c], hv[3 * B0 + c], SG0), sc2);
    const __half2 h1 = __hmul2(hcomb<IM>(hv[3 + c], hv[3 * B1 + c], SG1), sc2);
    v[c] = *(const uint32_t *)&h0;
    v[3 + c] = *(const uint32_t *)&h1;
  }
  tc_put12(row, DD, v);
}

template <bool DAG, int MODE>
__global__ void __launch_bounds__(kTcThreads, 3) k_wilson_mrhs_tc(const MArgs a, double *partials, const TcCtl ctl)
{
  extern __shared__ __align__(16) unsigned char tc_dyn[];
  unsigned char *Ls = tc_dyn, *Hs = tc_dyn + kTcLBytes;
  double *red = (double *)(tc_dyn + kTcLBytes + kTcHBytes);
  float *X = (float *)Hs;  // accumulators [site][slot][24], over H once the MMAs are done
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tbase;
  constexpr bool EO = MODE != 0;
  constexpr int SF = DAG ? +1 : -1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int s = tid >> 4, rl = tid & 15;  // this thread's site in the tile and slot in the group
  const uint32_t Lb = tc_smem(Ls), Hb = tc_smem(Hs);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(tc_smem(&tbase)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tbase;
  const int G = a.N >> 4;
  uint32_t phase = 0;
  double run[4] = {0.0, 0.0, 0.0, 0.0};  // per-slot |out|^2 of the CTA (threads 0..15)
  bool failed = false;
  for (int tile = 0; tile < kTcTiles && !failed; tile++) {
    const int base = (blockIdx.x * kTcTiles + tile) * kTcSites;
    if (base >= a.V) break;
    const int e = base + s;  // output index
    const bool act = e < a.V;
    int c[4], x = e;
    if (act) {
      if (EO) {
        coords(a.geo, 2 * e, c);
        const int b = (a.eo_par ^ c[1] ^ c[2] ^ c[3]) & 1;
        x = 2 * e + b;
        c[0] += b;
      } else {
        coords(a.geo, x, c);
      }
    }
    // L: thread (site s, hop h, half) writes the rows of output spins 2 half, 2 half + 1
    {
      const int h = rl >> 1, half = rl & 1, mu = h >> 1;
      const bool back = h & 1;
      const int S = back ? -SF : SF;
      C<float> M[9];
      if (act) {
        const int y = tc_nb(a.geo, x, c, h);
        C<float> U[9];
        Link<QCDGPU_F32, 18, float>::load(a.gauge, a.gstride, back ? y : x, mu, U);
        const bool tw = (a.twist_mask >> mu) & 1;
        const C<float> ph{tw ? a.phr[mu] : 1.f, tw ? (back ? -a.phi[mu] : a.phi[mu]) : 0.f};
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int j = 0; j < 3; j++) M[3 * i + j] = ph * (back ? conj(U[3 * j + i]) : U[3 * i + j]);
      } else {
#pragma unroll
        for (int k = 0; k < 9; k++) M[k] = C<float>{0.f, 0.f};
      }
#pragma unroll
      for (int q = 0; q < 2; q++) {
        const int sp = 2 * half + q;
        int src;
        float cr, ci;
        tc_rebuild(mu, S, sp, src, cr, ci);
#pragma unroll
        for (int i = 0; i < 3; i++) {
          uint32_t vre[6], vim[6];
#pragma unroll
          for (int j = 0; j < 3; j++) {
            // z = c M_ij; row re: (Re z, -Im z), row im: (Im z, Re z), in the source spin's columns
            const float zr = cr * M[3 * i + j].re - ci * M[3 * i + j].im;
            const float zi = cr * M[3 * i + j].im + ci * M[3 * i + j].re;
            const uint32_t pre = pack_h2(zr, -zi), pim = pack_h2(zi, zr);
            vre[j] = src == 0 ? pre : 0u;
            vre[3 + j] = src == 1 ? pre : 0u;
            vim[j] = src == 0 ? pim : 0u;
            vim[3 + j] = src == 1 ? pim : 0u;
          }
          const int o = 6 * sp + 2 * i;  // rows o (re) and o + 1 (im)
          const uint32_t site = Lb + (uint32_t)s * 3 * kTcSbo;
          tc_put12(site + (uint32_t)(o >> 3) * kTcSbo + (uint32_t)(o & 7) * 16, h, vre);
          tc_put12(site + (uint32_t)((o + 1) >> 3) * kTcSbo + (uint32_t)((o + 1) & 7) * 16, h, vim);
        }
      }
    }
    // neighbours are the same for every slot group
    int ys[8];
#pragma unroll
    for (int dd = 0; dd < 8; dd++) {
      const int y = act ? tc_nb(a.geo, x, c, dd) : 0;
      ys[dd] = EO ? (y >> 1) : y;
    }
    for (int grp = 0; grp < G && !failed; grp++) {
      const int r = grp * 16 + rl;
      // H row rl of site s
      const uint32_t hrow = Hb + (uint32_t)s * 2 * kTcSbo + (uint32_t)(rl >> 3) * kTcSbo + (uint32_t)(rl & 7) * 16;
      float sc = 0.f;  // the slot's rescale: its largest neighbour norm
      if (act) {
        float nr[8];
#pragma unroll
        for (int dd = 0; dd < 8; dd++) {
          nr[dd] = a.in_norm[(int64_t)ys[dd] * a.N + r];
          sc = fmaxf(sc, nr[dd]);
        }
        const float inv = sc > 0.f ? 1.0f / sc : 0.f;
        tc_h_block<DAG, 0>(a, ys[0], r, __float2half2_rn(nr[0] * inv), hrow);
        tc_h_block<DAG, 1>(a, ys[1], r, __float2half2_rn(nr[1] * inv), hrow);
        tc_h_block<DAG, 2>(a, ys[2], r, __float2half2_rn(nr[2] * inv), hrow);
        tc_h_block<DAG, 3>(a, ys[3], r, __float2half2_rn(nr[3] * inv), hrow);
        tc_h_block<DAG, 4>(a, ys[4], r, __float2half2_rn(nr[4] * inv), hrow);
        tc_h_block<DAG, 5>(a, ys[5], r, __float2half2_rn(nr[5] * inv), hrow);
        tc_h_block<DAG, 6>(a, ys[6], r, __float2half2_rn(nr[6] * inv), hrow);
        tc_h_block<DAG, 7>(a, ys[7], r, __float2half2_rn(nr[7] * inv), hrow);
      } else {
        const uint32_t z[6] = {0u, 0u, 0u, 0u, 0u, 0u};
#pragma unroll
        for (int dd = 0; dd < 8; dd++) tc_put12(hrow, dd, z);
      }
      // the tensor cores read what the threads wrote
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      if (tid == 0 && !ctl.skip_mma) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        constexpr uint32_t idesc = tc_idesc(64, 16);
#pragma unroll 1
        for (int t = 0; t < kTcSites; t++) {
#pragma unroll
          for (int kk = 0; kk < kTcK / 16; kk++) {
            const uint64_t ad = tc_sdesc(Lb + (uint32_t)t * 3 * kTcSbo + kk * 256, 128, kTcSbo);
            const uint64_t bd = tc_sdesc(Hb + (uint32_t)t * 2 * kTcSbo + kk * 256, 128, kTcSbo);
            const uint32_t dt = tmem + (uint32_t)(t * 16), acc = kk > 0;
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(dt),
                "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         tc_smem(&mbar))
                     : "memory");
      }
      // the z term of the epilogue does not wait for the tensor cores
      constexpr int zmode = MODE == 1 ? 0 : 2;
      C<float> zs[1][12];
      float znrm[1] = {0.f};
      if (zmode && act) mload_rp<1>(a, EO ? a.z : a.in, EO ? a.z_norm : a.in_norm, e, r, zs, znrm);
      // bounded wait for the commit; a timeout abandons the kernel's work
      uint32_t done = 0;
      for (int it = 0; it < ctl.polls && !done; it++)
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(tc_smem(&mbar)), "r"(phase)
            : "memory");
      if (__syncthreads_or(!done)) {
        // the MMAs may still be in flight: wait once more, bounded, before
        // the tensor memory is released
        for (int it = 0; it < ctl.polls && !done; it++)
          asm volatile(
              "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
              : "=r"(done)
              : "r"(tc_smem(&mbar)), "r"(phase)
              : "memory");
        if (tid == 0) {
          atomicAdd(&g_mrhs_tc_timeouts, 1u);
          *ctl.fail = 1u;
        }
        failed = true;
        break;
      }
      phase ^= 1u;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // accumulator rows 0..23 (warp 0 lanes 0..15, warp 1 lanes 0..7) -> X[site][slot][row]
      if (warp < 2) {
#pragma unroll
        for (int t = 0; t < kTcSites; t++) {
          uint32_t v[16];
          const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(t * 16);
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
              : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
              : "r"(ta));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          const int o = warp * 16 + lane;  // accumulator row
          if (lane < 16 && o < 24) {
#pragma unroll
            for (int n = 0; n < 16; n++) X[(t * 16 + n) * 24 + o] = __uint_as_float(v[n]);
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      // epilogue: one thread per (site, slot)
      double n2 = 0.0;
      if (act) {
        C<float> acc[12];
        const float *xi = X + (s * 16 + rl) * 24;
#pragma unroll
        for (int k = 0; k < 12; k++) acc[k] = C<float>{sc * xi[2 * k], sc * xi[2 * k + 1]};
        constexpr bool ainv = MODE == 1;
        constexpr float ch = MODE == 0 ? -0.5f : MODE == 1 ? 1.0f : -0.25f;
        const float mp4r = a.mp4s ? a.mp4s[r] : a.mp4;
        const float tmr = a.tms ? (DAG ? -a.tms[r] : a.tms[r]) : a.tm;
        if (ainv) {  // A^{-1} = (mp4 - i tm g5) / (mp4^2 + tm^2)
          const float den = 1.0f / (mp4r * mp4r + tmr * tmr), ar = mp4r * den, ai = -tmr * den;
#pragma unroll
          for (int k = 0; k < 12; k++) {
            const float g5ai = k < 6 ? ai : -ai;
            acc[k] = C<float>{ar * acc[k].re - g5ai * acc[k].im, ar * acc[k].im + g5ai * acc[k].re};
          }
        }
        const float zsc = zmode ? znrm[0] : 0.f;
        const float zm = zmode == 2 ? mp4r * zsc : zsc, zt = zmode == 2 ? tmr * zsc : 0.f;
        float mx = 0.f;
#pragma unroll
        for (int k = 0; k < 12; k++) {
          const float g5tm = k < 6 ? zt : -zt;
          const C<float> zk = zmode ? zs[0][k] : C<float>{0.f, 0.f};
          acc[k] = C<float>{zm * zk.re - g5tm * zk.im + ch * acc[k].re, zm * zk.im + g5tm * zk.re + ch * acc[k].im};
          mx = fmaxf(mx, fmaxf(fabsf(acc[k].re), fabsf(acc[k].im)));
        }
        if (!(mx >= 1.17549435e-38f)) mx = 0.f;
        const float inv = mx > 0.f ? 1.0f / mx : 0.f;
        if (r < a.nact) {
          float2 o[12];
#pragma unroll
          for (int k = 0; k < 12; k++) o[k] = make_float2(acc[k].re, acc[k].im);
          mstore_raw(a.out, a.V, a.N, e, r, o, inv);
          a.out_norm[(int64_t)e * a.N + r] = mx;
          if (partials) {  // |out|^2 of the stored (rounded) values
            float s2 = 0.f;
#pragma unroll
            for (int k = 0; k < 12; k++) {
              const float2 f = __half22float2(__floats2half2_rn(o[k].x * inv, o[k].y * inv));
              s2 += f.x * f.x + f.y * f.y;
            }
            n2 = (double)(s2 * mx * mx);
          }
        }
      }
      if (partials) {  // the CTA's per-slot sums, in a fixed order
        red[s * 16 + rl] = n2;
        __syncthreads();
        if (tid < 16) {
          double t = 0.0;
          for (int i = 0; i < kTcSites; i++) t += red[i * 16 + tid];
          run[grp] += t;
        }
      }
      __syncthreads();  // X (over H) and red are rewritten by the next group
    }
  }
  if (partials && tid < 16)
    for (int grp = 0; grp < G; grp++) partials[(int64_t)blockIdx.x * a.N + grp * 16 + tid] = run[grp];
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem));
}

unsigned mrhs_tc_grid(int64_t V) { return (unsigned)((V + kTcSites * kTcTiles - 1) / (kTcSites * kTcTiles)); }

template <bool D, int M>
static void launch_tc(const MArgs &a, double *partials, unsigned grid, cudaStream_t s, const TcCtl &ctl)
{
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_wilson_mrhs_tc<D, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
    attr = true;
  }
  k_wilson_mrhs_tc<D, M><<<grid, kTcThreads, kTcSmem, s>>>(a, partials, ctl);
}

// host side of the tensor-core kernel's failure reporting
static int g_tc_polls = 1 << 24;
static int g_tc_skip_mma = 0;
static volatile unsigned *g_tc_fail_host = nullptr;  // page-locked, mapped
static unsigned *g_tc_fail_dev = nullptr;

static bool tc_fail_setup()
{
  if (g_tc_fail_host) return true;
  void *h = nullptr, *d = nullptr;
  if (!QG_CUDA(cudaHostAlloc(&h, sizeof(unsigned), cudaHostAllocMapped))) return false;
  if (!QG_CUDA(cudaHostGetDevicePointer(&d, h, 0))) {
    cudaFreeHost(h);
    return false;
  }
  *(volatile unsigned *)h = 0u;
  g_tc_fail_dev = (unsigned *)d;
  g_tc_fail_host = (volatile unsigned *)h;
  return true;
}

bool mrhs_tc_failed() { return g_tc_fail_host && *g_tc_fail_host; }

struct MrhsTune {
  int variant;  // MRHS_SIMT, MRHS_MMA or MRHS_TC
  int threads;  // SIMT: N x (sites per block) target, 64, 128 or 256
  int rp;       // SIMT: RHS slots per thread (1, or 2 when N is even)
};

static int g_mrhs_variant = MRHS_AUTO;
static std::map<std::pair<int64_t, int>, MrhsTune> g_mrhs_tuned;

// block (N / rp slot threads, sites per block). `threads` / N sites is the
// target; of the counts from half to twice that (at least up to 4, at most
// 256 threads) the one that leaves the fewest idle lanes in the block's last
// warp is taken, the nearest to the target on a tie (48 slots at two per
// thread: 4 sites of 24 threads fill three warps, where 1 site leaves a
// quarter of its warp idle)
static dim3 simt_block(int N, int threads, int rp = 1)
{
  const int x = (N + rp - 1) / rp;  // threads per site
  const int sb = threads / N > 0 ? threads / N : 1;
  const int hi = 2 * sb > 4 ? 2 * sb : 4;
  int best = sb;
  int best_idle = 1 << 30, best_warps = 1;
  for (int c = sb / 2 > 1 ? sb / 2 : 1; c <= hi && x * c <= 256; c++) {
    const int t = x * c, warps = (t + 31) / 32, idle = warps * 32 - t;
    // idle / (32 warps) compared exactly: fewer idle lanes per lane, then nearer the target
    const long long lhs = (long long)idle * best_warps, rhs = (long long)best_idle * warps;
    if (best_idle == 1 << 30 || lhs < rhs || (lhs == rhs && abs(c - sb) < abs(best - sb))) {
      best = c;
      best_idle = idle;
      best_warps = warps;
    }
  }
  return dim3((unsigned)x, (unsigned)best);
}

// the largest block count of any shape that writes per-slot partial sums
unsigned mrhs_max_blocks(int64_t V, int N)
{
  unsigned m = 0;
  for (int threads : {64, 128, 256})
    for (int rp : {1, 2}) {
      const dim3 b = simt_block(N, threads, rp);
      const unsigned nb = (unsigned)((V + b.y - 1) / b.y);
      if (nb > m) m = nb;
    }
  return m;
}

static bool launch_mrhs(const MArgs &a, bool dag, MrhsTune t, double *partials, unsigned *nblocks)
{
  cudaStream_t s = stream();
  if (t.variant == MRHS_TC) {
    if (a.N % 16 != 0 || a.N > 64) {
      set_error("tensor-core (tcgen05) multi-RHS kernel: slot count a multiple of 16, at most 64 (got %d)", a.N);
      return false;
    }
    if (!tc_fail_setup()) return false;
    if (*g_tc_fail_host) {
      set_error("tensor-core multi-RHS kernel: an earlier launch abandoned its work after a bounded wait for the "
                "tensor cores ran out (its output is invalid); qcdgpu_mrhs_tc_reset clears the state");
      return false;
    }
    const TcCtl ctl{g_tc_polls, g_tc_skip_mma, g_tc_fail_dev};
    const unsigned grid = mrhs_tc_grid(a.V);
    const int mode = a.eo_par < 0 ? 0 : a.ainv ? 1 : 2;
    if (dag) {
      if (mode == 0) launch_tc<true, 0>(a, partials, grid, s, ctl);
      else if (mode == 1) launch_tc<true, 1>(a, partials, grid, s, ctl);
      else launch_tc<true, 2>(a, partials, grid, s, ctl);
    } else {
      if (mode == 0) launch_tc<false, 0>(a, partials, grid, s, ctl);
      else if (mode == 1) launch_tc<false, 1>(a, partials, grid, s, ctl);
      else launch_tc<false, 2>(a, partials, grid, s, ctl);
    }
    if (!QG_LAUNCHED("wilson_mrhs_tc")) return false;
    if (nblocks) *nblocks = grid;
    return true;
  }
  const bool simt = t.variant == MRHS_SIMT;
  // threads for the occupied slots only (the tuned block size holds more
  // sites when fewer slots are occupied), except when the launch writes
  // per-slot partial sums: their grouping into blocks, and so their summation
  // order, must not depend on which other slots are occupied
  const dim3 blk = simt_block(simt && !partials ? a.nact : a.N, simt ? t.threads : 256, simt ? t.rp : 1);
  const unsigned nb = (unsigned)((a.V + blk.y - 1) / blk.y);
  const size_t shm = sizeof(double) * a.N * blk.y;
  if (simt) {
    const int ns = (int)blk.x * t.rp < a.N ? (int)blk.x * t.rp : a.N;
    const size_t sm = partials ? sizeof(double) * ns * blk.y : 0;
    // kernel mode from the epilogue (see k_wilson_mrhs_simt)
    const int mode = a.eo_par < 0 ? 0 : a.ainv ? 1 : 2;
#define QG_SIMT(RP, MODE)                                                           \
  if (dag) k_wilson_mrhs_simt<true, RP, MODE><<<nb, blk, sm, s>>>(a, partials);     \
  else k_wilson_mrhs_simt<false, RP, MODE><<<nb, blk, sm, s>>>(a, partials);
    if (t.rp == 2) {
      if (mode == 0) {
        QG_SIMT(2, 0)
      } else if (mode == 1) {
        QG_SIMT(2, 1)
      } else {
        QG_SIMT(2, 2)
      }
    } else {
      if (mode == 0) {
        QG_SIMT(1, 0)
      } else if (mode == 1) {
        QG_SIMT(1, 1)
      } else {
        QG_SIMT(1, 2)
      }
    }
#undef QG_SIMT
    if (!QG_LAUNCHED("wilson_mrhs_simt")) return false;
  } else {
    unsigned grid = (unsigned)((a.V + 3) / 4);
    int mt = (a.nact + 15) / 16;
#define QG_MRHS(MT)                                                      \
  if (dag) k_wilson_mrhs<true, MT><<<grid, 128, 0, s>>>(a);              \
  else k_wilson_mrhs<false, MT><<<grid, 128, 0, s>>>(a);
    switch (mt) {
    case 1: QG_MRHS(1) break;
    case 2: QG_MRHS(2) break;
    case 3: QG_MRHS(3) break;
    default: QG_MRHS(4) break;
    }
#undef QG_MRHS
    if (!QG_LAUNCHED("wilson_mrhs")) return false;
    if (partials) {
      k_mnorm<<<nb, simt_block(a.N, 256), shm, s>>>(a.out, a.out_norm, a.V, a.N, a.nact, partials);
      if (!QG_LAUNCHED("mrhs_norm")) return false;
    }
  }
  if (nblocks) *nblocks = nb;
  return true;
}

// Pick the variant and block shape for (V, N) by timing each candidate
// three times on the caller's fields (the output is overwritten with the
// same result). Not while the stream is being captured: then the SIMT
// variant with 256-thread blocks runs until a tuned choice exists.
static MrhsTune mrhs_tune(const MArgs &a, bool dag)
{
  if (g_mrhs_variant == MRHS_MMA) return MrhsTune{MRHS_MMA, 256, 1};
  if (g_mrhs_variant == MRHS_TC) return MrhsTune{MRHS_TC, kTcThreads, 1};
  if (g_mrhs_variant >= 64) {  // forced block size; +1: two slots per thread
    const int rp = (g_mrhs_variant & 1) && a.N % 2 == 0 ? 2 : 1;
    return MrhsTune{MRHS_SIMT, g_mrhs_variant & ~1, rp};
  }
  // even/odd kernels are tuned separately (key: minus the half volume)
  const auto key = std::make_pair(a.eo_par < 0 ? (int64_t)a.V : -(int64_t)a.V, a.N);
  auto it = g_mrhs_tuned.find(key);
  if (it != g_mrhs_tuned.end()) return it->second;
  const MrhsTune fallback{MRHS_SIMT, 128, 1};
  cudaStream_t s = stream();
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return fallback;
  const MrhsTune cands[] = {{MRHS_SIMT, 64, 1},  {MRHS_SIMT, 128, 1}, {MRHS_SIMT, 256, 1},
                            {MRHS_SIMT, 64, 2},  {MRHS_SIMT, 128, 2}, {MRHS_SIMT, 256, 2},
                            {MRHS_TC, kTcThreads, 1}, {MRHS_MMA, 256, 1}};
  const int ncand = a.eo_par < 0 ? 8 : 7;  // the mma.sync kernel has no even/odd mode
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return fallback;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return fallback;
  }
  MrhsTune best = fallback;
  float best_ms = 1e30f;
  for (int ic = 0; ic < ncand; ic++) {
    const MrhsTune &c = cands[ic];
    if (c.variant == MRHS_SIMT && (c.threads < a.N || (c.rp == 2 && a.N % 2 != 0))) continue;
    if (c.variant == MRHS_TC && a.N % 16 != 0) continue;
    if (!launch_mrhs(a, dag, c, nullptr, nullptr)) break;  // warm-up
    cudaEventRecord(e0, s);
    bool ok = true;
    for (int i = 0; i < 3 && ok; i++) ok = launch_mrhs(a, dag, c, nullptr, nullptr);
    cudaEventRecord(e1, s);
    if (!ok || cudaEventSynchronize(e1) != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_ms) {
      best_ms = ms;
      best = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  g_mrhs_tuned[key] = best;
  return best;
}

bool dslash_mrhs(qcdgpu_mfield out, qcdgpu_mfield in, qcdgpu_gauge g, double mp4, double tm, bool dag, int nact,
                 const float *mp4s, const float *tms, double *partials, unsigned *nblocks)
{
  if (!out || !in || !g || out == in || out->N != in->N || out->V != in->V || in->V != g->V ||
      memcmp(out->L, in->L, sizeof(in->L)) != 0 || memcmp(in->L, g->L, sizeof(g->L)) != 0) {
    set_error("multi-RHS operator: fields differ in shape or alias");
    return false;
  }
  if (nact < 0 || nact > in->N) {
    set_error("multi-RHS operator: %d active RHS of %d slots", nact, in->N);
    return false;
  }
  if (g->prec != QCDGPU_F64) {
    set_error("multi-RHS operator takes the FP64 gauge field (it keeps its own FP32 copy)");
    return false;
  }
  qcdgpu_gauge g32 = gauge_at(g, kGaugeF32Full);
  if (!g32) return false;
  MArgs a;
  a.out = (__half2 *)out->data;
  a.out_norm = out->norm;
  a.in = (const __half2 *)in->data;
  a.in_norm = in->norm;
  a.gauge = (const float2 *)g32->data;
  for (int i = 0; i < 4; i++) a.geo.L[i] = in->L[i];
  a.geo.st[0] = 1;
  a.geo.st[1] = in->L[0];
  a.geo.st[2] = in->L[0] * in->L[1];
  a.geo.st[3] = in->L[0] * in->L[1] * in->L[2];
  a.V = (int)in->V;
  a.N = in->N;
  a.nact = nact;
  a.gstride = g32->stride;
  a.twist_mask = 0;
  for (int mu = 0; mu < 4; mu++) {
    a.phr[mu] = 1.f;
    a.phi[mu] = 0.f;
    if (g->theta[mu] != 0.0) {
      a.twist_mask |= 1 << mu;
      a.phr[mu] = (float)cos(g->theta[mu] / (double)g->L[mu]);
      a.phi[mu] = (float)sin(g->theta[mu] / (double)g->L[mu]);
    }
  }
  a.mp4 = (float)mp4;
  a.tm = (float)(dag ? -tm : tm);
  a.mp4s = mp4s;
  a.tms = tms;
  a.z = a.in;  // full-lattice operator: (m+4) in + i tm g5 in - H in / 2
  a.z_norm = a.in_norm;
  a.zmode = 2;
  a.ainv = 0;
  a.ch = -0.5f;
  a.eo_par = -1;
  if (nact == 0) {
    if (nblocks) *nblocks = 0;
    return true;
  }
  const MrhsTune tune = mrhs_tune(a, dag);
  if (!launch_mrhs(a, dag, tune, partials, nblocks)) return false;
  return true;
}

// Even/odd multi-RHS kernel (SIMT) on half-lattice fields: slots 0..nact-1 of
// out (parity par) = ch * [A^{-1}] H in + {0 | z | A z}, A the slot's diagonal
// (mp4s, tms; D^+: tm -> -tm and the hopping term of D^+). partials as in
// dslash_mrhs. g is the FP64 gauge field of the full lattice.
bool dslash_mrhs_eo(qcdgpu_mfield out, qcdgpu_mfield in, qcdgpu_mfield z, qcdgpu_gauge g, bool dag, int nact,
                    const float *mp4s, const float *tms, int par, double ch, bool ainv, int zmode, double *partials,
                    unsigned *nblocks)
{
  if (!out || !in || !g || out == in || out->N != in->N || out->V != in->V || (zmode && (!z || z == out)) ||
      (z && (z->N != in->N || z->V != in->V)) || g->prec != QCDGPU_F64 || g->L[0] % 2 != 0 ||
      in->L[0] * 2 != g->L[0] || in->L[1] != g->L[1] || in->L[2] != g->L[2] || in->L[3] != g->L[3] ||
      memcmp(out->L, in->L, sizeof(in->L)) != 0 || nact < 0 || nact > in->N || !mp4s || !tms) {
    set_error("even/odd multi-RHS operator: half-lattice fields of one shape, per-slot diagonal");
    return false;
  }
  qcdgpu_gauge g32 = gauge_at(g, kGaugeF32Full);
  if (!g32) return false;
  MArgs a;
  a.out = (__half2 *)out->data;
  a.out_norm = out->norm;
  a.in = (const __half2 *)in->data;
  a.in_norm = in->norm;
  a.gauge = (const float2 *)g32->data;
  for (int i = 0; i < 4; i++) a.geo.L[i] = g->L[i];
  a.geo.st[0] = 1;
  a.geo.st[1] = g->L[0];
  a.geo.st[2] = g->L[0] * g->L[1];
  a.geo.st[3] = g->L[0] * g->L[1] * g->L[2];
  a.V = (int)in->V;
  a.N = in->N;
  a.nact = nact;
  a.gstride = g32->stride;
  a.twist_mask = 0;
  for (int mu = 0; mu < 4; mu++) {
    a.phr[mu] = 1.f;
    a.phi[mu] = 0.f;
    if (g->theta[mu] != 0.0) {
      a.twist_mask |= 1 << mu;
      a.phr[mu] = (float)cos(g->theta[mu] / (double)g->L[mu]);
      a.phi[mu] = (float)sin(g->theta[mu] / (double)g->L[mu]);
    }
  }
  a.mp4 = 4.f;
  a.tm = 0.f;
  a.mp4s = mp4s;
  a.tms = tms;
  a.z = z ? (const __half2 *)z->data : nullptr;
  a.z_norm = z ? z->norm : nullptr;
  a.zmode = zmode;
  a.ainv = ainv ? 1 : 0;
  a.ch = (float)ch;
  a.eo_par = par;
  // the kernels implement the two halves of the Schur complement
  if (!((ainv && zmode == 0 && ch == 1.0) || (!ainv && zmode == 2 && ch == -0.25))) {
    set_error("even/odd multi-RHS operator: epilogue A^{-1} H in or A z - H in / 4 only");
    return false;
  }
  if (nact == 0) {
    if (nblocks) *nblocks = 0;
    return true;
  }
  return launch_mrhs(a, dag, mrhs_tune(a, dag), partials, nblocks);
}

}  // namespace qg

extern "C" {

int qcdgpu_mfield_create(qcdgpu_mfield *m, const int L[4], int nrhs)
{
  *m = qg::mfield_new(L, nrhs);
  return *m ? 0 : 1;
}
int qcdgpu_mfield_destroy(qcdgpu_mfield m)
{
  qg::mfield_free(m);
  return 0;
}
int qcdgpu_mfield_set(qcdgpu_mfield m, int r, qcdgpu_field f) { return qg::mfield_set(m, r, f) ? 0 : 1; }
int qcdgpu_mfield_get(qcdgpu_field f, qcdgpu_mfield m, int r) { return qg::mfield_get(f, m, r) ? 0 : 1; }
int qcdgpu_set_mrhs_variant(int v)
{
  if (v != qg::MRHS_AUTO && v != qg::MRHS_MMA && v != qg::MRHS_TC && v != 64 && v != 128 && v != 256 && v != 65 &&
      v != 129 && v != 257) {
    qg::set_error("multi-RHS variant: -1 (tuned), 1 (tensor cores, mma.sync), 2 (tensor cores, tcgen05; slot "
                  "counts that are multiples of 16), 64 / 128 / 256 (SIMT, slots x sites per block), +1 for two "
                  "slots per thread");
    return 1;
  }
  qg::g_mrhs_variant = v;
  return 0;
}

int qcdgpu_mrhs_tc_timeouts(unsigned *n)
{
  if (!QG_CUDA(cudaStreamSynchronize(qg::stream()))) return 1;
  return QG_CUDA(cudaMemcpyFromSymbol(n, qg::g_mrhs_tc_timeouts, sizeof(unsigned))) ? 0 : 1;
}

int qcdgpu_mrhs_tc_reset(void)
{
  if (!QG_CUDA(cudaStreamSynchronize(qg::stream()))) return 1;
  const unsigned z = 0;
  if (!QG_CUDA(cudaMemcpyToSymbol(qg::g_mrhs_tc_timeouts, &z, sizeof(z)))) return 1;
  if (qg::g_tc_fail_host) *qg::g_tc_fail_host = 0u;
  return 0;
}

int qcdgpu_mrhs_tc_test_hook(int skip_mma, int polls)
{
  qg::g_tc_skip_mma = skip_mma ? 1 : 0;
  qg::g_tc_polls = polls > 0 ? polls : 1 << 24;
  return 0;
}

int qcdgpu_mrhs_tuned(const int L[4], int nrhs, int *variant, int *threads)
{
  const int64_t V = (int64_t)L[0] * L[1] * L[2] * L[3];
  auto it = qg::g_mrhs_tuned.find(std::make_pair(V, nrhs));
  if (it == qg::g_mrhs_tuned.end()) return 1;
  *variant = it->second.variant;
  *threads = it->second.threads + (it->second.rp == 2 ? 1 : 0);
  return 0;
}

int qcdgpu_dslash_mrhs(qcdgpu_mfield out, qcdgpu_mfield in, qcdgpu_gauge g, double kappa, double mu, int op,
                       int nact)
{
  if (!(kappa > 0.0) || (op != QCDGPU_OP_D && op != QCDGPU_OP_DDAG)) {
    qg::set_error("multi-RHS operator: kappa > 0 and op D or DDAG");
    return 1;
  }
  return qg::dslash_mrhs(out, in, g, 1.0 / (2.0 * kappa), mu, op == QCDGPU_OP_DDAG, nact, nullptr, nullptr) ? 0 : 1;
}

}  // extern "C"
