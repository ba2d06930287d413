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

// h = upper half of (1 + S g_mu) s for the spinor s held as its three
// 16-byte words (without its norm, which the accumulation applies),
// projected on packed half pairs (as the single-RHS FP16 kernel does)
template <int MU, int S>
__device__ __forceinline__ void project_words(const uint4 w[3], C<float> h[6])
{
  const __half2 *hv = reinterpret_cast<const __half2 *>(w);
  constexpr bool IM = MU & 1;
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

// the same for slot r of the multi-RHS spinor at y
template <int MU, int S>
__device__ __forceinline__ void mload_project(const __half2 *d, int64_t V, int N, int y, int r, C<float> h[6])
{
  const uint4 *p = (const uint4 *)d;
  uint4 w[3];
#pragma unroll
  for (int j = 0; j < 3; j++) w[j] = p[((int64_t)j * V + y) * N + r];
  project_words<MU, S>(w, h);
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
      // components are converted; the slot's site norm scales the accumulation
      if (back) mload_project<MU, -SF>(a.in, a.V, a.N, ys, r0 + q, h);
      else mload_project<MU, SF>(a.in, a.V, a.N, ys, r0 + q, h);
#pragma unroll
      for (int j = 0; j < 2; j++)
#pragma unroll
        for (int i = 0; i < 3; i++)
          uh[3 * j + i] =
              back ? cmadd_conj(U[6 + i], h[3 * j + 2], cmadd_conj(U[3 + i], h[3 * j + 1], cdot(U[i], h[3 * j])))
                   : cmadd(U[3 * i + 2], h[3 * j + 2], cmadd(U[3 * i + 1], h[3 * j + 1], U[3 * i] * h[3 * j]));
      if (twisted) {
        C<float> ph{a.phr[MU], back ? -a.phi[MU] : a.phi[MU]};
#pragma unroll
        for (int k = 0; k < 6; k++) uh[k] = uh[k] * ph;
      }
      if (back) accumulate_scaled<MU, -SF>(acc[q], uh, nrm[q]);
      else accumulate_scaled<MU, SF>(acc[q], uh, nrm[q]);
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
      float mx = 0.f;
      if constexpr (ainv) {  // ch A^{-1} = ch (mp4 - i tm g5) / (mp4^2 + tm^2), no addend
        const float den = ch / (mp4r * mp4r + tmr * tmr), ar = mp4r * den, ai = -tmr * den;
#pragma unroll
        for (int k = 0; k < 12; k++) {
          const float g5ai = k < 6 ? ai : -ai;
          acc[q][k] = C<float>{ar * acc[q][k].re - g5ai * acc[q][k].im, ar * acc[q][k].im + g5ai * acc[q][k].re};
          mx = fmaxf(mx, fmaxf(fabsf(acc[q][k].re), fabsf(acc[q][k].im)));
        }
      } else {  // ch H in + A z
        const float zs = nrm[q];
        const float zm = zmode == 2 ? mp4r * zs : zs, zt = zmode == 2 ? tmr * zs : 0.f;
#pragma unroll
        for (int k = 0; k < 12; k++) {
          const float g5tm = k < 6 ? zt : -zt;
          const C<float> zk = s[q][k];
          acc[q][k] = C<float>{qfma(ch, acc[q][k].re, qfma(-g5tm, zk.im, zm * zk.re)),
                               qfma(ch, acc[q][k].im, qfma(g5tm, zk.re, zm * zk.im))};
          mx = fmaxf(mx, fmaxf(fabsf(acc[q][k].re), fabsf(acc[q][k].im)));
        }
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
//   D^T (24 x 16) = L (24 x 128) H^T (128 x 16),
// FP16 operands, FP32 accumulator in tensor memory. K = (hop h, input spin
// s, colour j, re/im) in blocks of 8: each (hop, spin) is the six values of
// three colours and two zero pads, one 16-byte core-matrix row, so every
// operand row is written with aligned 16-byte stores. Row o = (spin S,
// colour i, re/im) of L holds, in block (h, src), the realified c M_ij
// (row re: (Re z, -Im z), row im: (Im z, Re z), z = c M_ij), where M = U_mu
// (or U_mu^+ for backward hops, boundary phase folded in) and c (1, -1, i or
// -i) and src the coefficient and source spin that rebuild spin S from the
// projected upper half of (1 +- g_mu) (the rules of accumulate<MU, S>); the
// blocks of the other source spin are zero. L is built once per site for all
// slot groups. Row n of H is slot n's projected half spinor at each of the
// eight neighbours (packed half pairs, as the FP16 kernels project them),
// scaled by that neighbour's norm over the slot's largest. The MMA is issued
// with M = 64 (the smallest): rows 24..63 of the A operand read whatever
// follows in shared memory and land in accumulator rows that are never read.
//
// A CTA (two per SM, persistent over tiles of 4 sites) is a pipeline of warp
// roles over work items (tile, slot group), with the operand buffers and the
// tensor-memory accumulators double-buffered:
//  - warps 0..3 build L (first group of a tile) and H of item n into buffer
//    n % 2, once the MMAs of item n - 2 have completed (every global load of
//    the item is issued before that wait), and arrive on full;
//  - one thread of warp 6 issues the item's 4 sites x 8 MMAs (M = 64, N = 16,
//    K = 16, no-swizzle K-major descriptors) into 64 tensor-memory columns
//    once full has completed and the epilogue has drained that accumulator
//    buffer, and commits them to the item's done barrier (it also arrives on
//    sready, which hands the producers' per-slot rescale factors, read from
//    shared memory, on to the epilogue with release / acquire ordering);
//  - warps 4 and 5 wait for done, copy the 24 accumulator rows (TMEM lanes
//    0..15 and 32..39) to shared memory, release the accumulator buffer and
//    run the epilogue (slot rescale, diagonal term, A^{-1}, FP16 rounding with
//    the per-site norm, per-slot |out|^2 in a fixed order), one thread per
//    site and slot.
// Every mbarrier wait is bounded (ctl.polls); a wait that runs out sets the
// failure flag and its thread stops waiting, so the launch always ends (with
// its output invalid and the failure reported to the host).
constexpr int kTcSites = 4;                                 // sites per tile
constexpr int kTcK = 128;                                   // 8 hops x 2 spins x 8
constexpr uint32_t kTcSbo = (kTcK / 8) * 128;               // bytes per 8-row group
constexpr uint32_t kTcLSite = 3 * kTcSbo;                   // 24 rows of L per site
constexpr uint32_t kTcHSite = 2 * kTcSbo;                   // 16 rows of H per site
constexpr uint32_t kTcLBuf = kTcSites * kTcLSite, kTcHBuf = kTcSites * kTcHSite;
constexpr int kTcPairs = kTcSites * 16;                     // (site, slot) pairs of an item
constexpr int kTcProd = 2 * kTcPairs, kTcEpi = kTcPairs;    // producer and epilogue threads
constexpr int kTcThreads = kTcProd + kTcEpi + 32;           // + the MMA warp
constexpr int kTcEpiWarp0 = kTcProd / 32;                   // warps 4, 5 (TMEM lanes 0..31, 32..63)
constexpr int kTcMmaWarp = kTcEpiWarp0 + kTcEpi / 32;       // warp 6
constexpr uint32_t kTcCols = 2 * kTcSites * 16;             // tensor-memory columns (two buffers)
static_assert(kTcEpiWarp0 % 4 == 0 && kTcEpi == 64, "epilogue warps must cover TMEM lanes 0..63");
// dynamic shared memory: L[2], H[2], X (accumulators for the epilogue), the
// slots' rescale factors of four items, per-slot partial sums, neighbours
constexpr uint32_t kTcOffH = 2 * kTcLBuf;
constexpr uint32_t kTcOffX = kTcOffH + 2 * kTcHBuf;
constexpr uint32_t kTcOffScl = kTcOffX + kTcSites * 16 * 24 * 4;
constexpr uint32_t kTcOffRed = kTcOffScl + 4 * kTcPairs * 4;
constexpr uint32_t kTcOffNb = kTcOffRed + kTcPairs * 8;
constexpr size_t kTcSmem = kTcOffNb + kTcSites * 9 * 4;
// the M = 64 operand of the last site of L[1] reads 64 rows from its start:
// inside the allocation
static_assert(kTcLBuf + (kTcSites - 1) * kTcLSite + 8 * kTcSbo <= kTcSmem, "tcgen05 A operand overruns shared memory");
static_assert(2 * kTcSmem <= 226 * 1024, "tcgen05 kernel: two CTAs per SM");

__device__ unsigned g_mrhs_tc_timeouts;  // launches that abandoned work after a bounded wait

// launch controls of the tensor-core kernel: the bound of each wait (mbarrier
// polls), a test hook that issues no MMA (so the waits run out), and a
// host-mapped flag the kernel sets when a wait ran out
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

// shared stores of the operands: volatile asm, so they stay in order with
// the fences and barriers that hand the operands to the tensor cores, while
// global loads may move across them
__device__ __forceinline__ void sts128(uint32_t a, uint32_t x, uint32_t y, uint32_t z, uint32_t w)
{
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(a), "r"(x), "r"(y), "r"(z), "r"(w));
}

__device__ __forceinline__ void tc_named_bar(int id, int n)
{
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t bar, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}" ::"r"(bar) : "memory");
}

// wait for the phase of parity `parity` of the barrier to complete, at most
// `polls` polls; false if the wait ran out
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int polls)
{
  uint32_t done = 0;
  for (int it = 0; it < polls && !done; it++)
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
  return done != 0;
}

// a bounded wait of a pipeline role; after one wait ran out the thread stops
// waiting (its work is void, the launch reports the failure)
__device__ __forceinline__ void tc_wait(uint32_t bar, uint32_t parity, const TcCtl &ctl, bool &failed)
{
  if (failed) return;
  if (!mbar_wait(bar, parity, ctl.polls)) {
    failed = true;
    *ctl.fail = 1u;
  }
}

// a row of H, K blocks of hop DD: the projected half spinor of the
// neighbour's three 16-byte words w, scaled by sc2
template <bool DAG, int DD>
__device__ __forceinline__ void tc_h_block(const uint4 w[3], __half2 sc2, uint32_t row)
{
  constexpr int MU = DD >> 1, SF = DAG ? +1 : -1, S = (DD & 1) ? -SF : SF;
  constexpr bool IM = MU & 1;
  constexpr int B0 = (MU == 0 || MU == 3) ? 2 : 3, B1 = 5 - B0;
  constexpr int SG0 = S > 0 ? -1 : 1, SG1 = MU < 2 ? SG0 : -SG0;
  const __half2 *hv = reinterpret_cast<const __half2 *>(w);
  uint32_t v0[3], v1[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const __half2 h0 = __hmul2(hcomb<IM>(hv[c], hv[3 * B0 + c], SG0), sc2);
    const __half2 h1 = __hmul2(hcomb<IM>(hv[3 + c], hv[3 * B1 + c], SG1), sc2);
    v0[c] = *(const uint32_t *)&h0;
    v1[c] = *(const uint32_t *)&h1;
  }
  sts128(row + (2 * DD) * 128, v0[0], v0[1], v0[2], 0u);
  sts128(row + (2 * DD + 1) * 128, v1[0], v1[1], v1[2], 0u);
}

// neighbour of x in hop dd (2 mu + backward)
__device__ __forceinline__ int tc_nb(const Geom &g, int x, const int c[4], int dd)
{
  return (dd & 1) ? bwd(g, x, c, dd >> 1) : fwd(g, x, c, dd >> 1);
}

// source spin and coefficient (0: 1, 1: -1, 2: i, 3: -i) that rebuild spin sp
// from the projected upper half of (1 + S g_mu)
__device__ __forceinline__ void tc_rebuild(int mu, int S, int sp, int &src, int &kind)
{
  const int neg = S > 0 ? 0 : 1;  // c = S or i S: negative when S < 0
  if (sp < 2) {
    src = sp;
    kind = 0;
  } else if (mu == 0) {  // c = -S
    src = sp - 2;
    kind = 1 - neg;
  } else if (mu == 1) {  // c = i S
    src = 3 - sp;
    kind = 2 + neg;
  } else if (mu == 2) {  // c = S (spin 2), -S (spin 3)
    src = 3 - sp;
    kind = sp == 2 ? neg : 1 - neg;
  } else {  // c = i S (spin 2), -i S (spin 3)
    src = sp - 2;
    kind = sp == 2 ? 2 + neg : 3 - neg;
  }
}

template <bool DAG, int MODE>
__global__ void __launch_bounds__(kTcThreads, 2) k_wilson_mrhs_tc(const MArgs a, double *partials, const TcCtl ctl)
{
  extern __shared__ __align__(128) unsigned char tc_dyn[];
  __shared__ __align__(8) uint64_t bars[8];  // full[2], done[2], tfree[2], sready[2]
  __shared__ uint32_t tbase;
  constexpr bool EO = MODE != 0;
  constexpr int SF = DAG ? +1 : -1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t Lb = tc_smem(tc_dyn), Hb = Lb + kTcOffH;
  float *X = (float *)(tc_dyn + kTcOffX);
  float *scl = (float *)(tc_dyn + kTcOffScl);
  double *red = (double *)(tc_dyn + kTcOffRed);
  int *nb = (int *)(tc_dyn + kTcOffNb);
  const uint32_t bfull = tc_smem(&bars[0]), bdone = tc_smem(&bars[2]), btfree = tc_smem(&bars[4]);
  const uint32_t bsready = tc_smem(&bars[6]);
  if (tid == 0) {
    mbar_init(bfull, kTcProd);
    mbar_init(bfull + 8, kTcProd);
    mbar_init(bdone, 1);
    mbar_init(bdone + 8, 1);
    mbar_init(btfree, 2);
    mbar_init(btfree + 8, 2);
    mbar_init(bsready, 1);
    mbar_init(bsready + 8, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // zero both L buffers: the blocks of the other source spin and the pads
  // are never written again
  for (uint32_t i = tid; i < 2 * kTcLBuf / 16; i += kTcThreads) sts128(Lb + 16 * i, 0u, 0u, 0u, 0u);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (warp == kTcMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&tbase)), "n"(kTcCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tbase;
  const int G = a.N >> 4;
  const int ntiles = (a.V + kTcSites - 1) / kTcSites;
  const int my_tiles = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  bool failed = false;
  int last_item = -1;  // MMA thread: the last item committed

  if (warp < kTcEpiWarp0) {
    // ------------------------------------------------------ producers
    const int pt = tid;
    int n = 0;
    for (int lt = 0; lt < my_tiles; lt++) {
      const int base = ((int)blockIdx.x + lt * (int)gridDim.x) * kTcSites;
      tc_named_bar(2, kTcProd);  // the previous tile's neighbours are no longer read
      if (pt < kTcSites) {
        const int e = base + pt;
        int x = -1;
        if (e < a.V) {
          int c[4];
          x = e;
          if (EO) {
            coords(a.geo, 2 * e, c);
            const int b = (a.eo_par ^ c[1] ^ c[2] ^ c[3]) & 1;
            x = 2 * e + b;
            c[0] += b;
          } else {
            coords(a.geo, x, c);
          }
#pragma unroll
          for (int dd = 0; dd < 8; dd++) nb[pt * 9 + dd] = tc_nb(a.geo, x, c, dd);
        }
        nb[pt * 9 + 8] = x;
      }
      tc_named_bar(2, kTcProd);
      for (int g = 0; g < G; g++, n++) {
        const int b = n & 1;
        // every global load of the item first, so that their latency overlaps
        // the wait for the buffers and one another
        // L: thread (site, hop, colour row i) of the first 192 reads row i of its link
        const bool lbuild = g == 0 && pt < kTcSites * 24;
        const int ls = pt / 24, lh = (pt % 24) / 3, li = pt % 3;
        const int lx = lbuild ? nb[ls * 9 + 8] : -1;
        C<float> m[3];
        if (lx >= 0) {
          const int mu = lh >> 1;
          const bool back = lh & 1;
          const int y = nb[ls * 9 + lh];
          const float2 *gp = a.gauge + (int64_t)mu * 9 * a.gstride + (back ? y : lx);
#pragma unroll
          for (int j = 0; j < 3; j++) {
            const float2 v = __ldg(gp + (int64_t)(back ? 3 * j + li : 3 * li + j) * a.gstride);
            m[j] = C<float>{v.x, back ? -v.y : v.y};
          }
        }
        // H: thread (site, slot) of the first half of the producers takes hops 0..3, of the second hops 4..7
        const int pair = pt % kTcPairs, hh = pt / kTcPairs;
        const int hs = pair >> 4, rl = pair & 15, r = g * 16 + rl;
        const int hx = nb[hs * 9 + 8];
        float nr[8];
        uint4 w[4][3];
        if (hx >= 0) {
#pragma unroll
          for (int dd = 0; dd < 8; dd++) {
            const int y = nb[hs * 9 + dd];
            nr[dd] = a.in_norm[(int64_t)(EO ? (y >> 1) : y) * a.N + r];
          }
          const uint4 *p = (const uint4 *)a.in;
#pragma unroll
          for (int q = 0; q < 4; q++) {
            const int y = nb[hs * 9 + 4 * hh + q];
            const int64_t ys = EO ? (y >> 1) : y;
#pragma unroll
            for (int j = 0; j < 3; j++) w[q][j] = p[((int64_t)j * a.V + ys) * a.N + r];
          }
        }
        if (n >= 2) tc_wait(bdone + 8 * b, ((n >> 1) & 1) ^ 1, ctl, failed);  // the MMAs of item n - 2
        if (lx >= 0) {
          const int mu = lh >> 1;
          const bool back = lh & 1;
          if ((a.twist_mask >> mu) & 1) {
            const C<float> ph{a.phr[mu], back ? -a.phi[mu] : a.phi[mu]};
#pragma unroll
            for (int j = 0; j < 3; j++) m[j] = ph * m[j];
          }
          uint32_t p1[3], p2[3];  // (Re, -Im) and (Im, Re) of M_ij
#pragma unroll
          for (int j = 0; j < 3; j++) {
            p1[j] = pack_h2(m[j].re, -m[j].im);
            p2[j] = pack_h2(m[j].im, m[j].re);
          }
          const int S = back ? -SF : SF;
          const uint32_t Ls = Lb + (uint32_t)(lt & 1) * kTcLBuf + (uint32_t)ls * kTcLSite;
#pragma unroll
          for (int sp = 0; sp < 4; sp++) {
            int src, kind;
            tc_rebuild(mu, S, sp, src, kind);
            // c M in the two rows: 1: (P1, P2); -1: (-P1, -P2); i: (-P2, P1); -i: (P2, -P1)
            const bool swap = kind >= 2;
            const uint32_t nre = (kind == 1 || kind == 2) ? 0x80008000u : 0u;
            const uint32_t nim = (kind == 1 || kind == 3) ? 0x80008000u : 0u;
            uint32_t wr[3], wi[3];
#pragma unroll
            for (int j = 0; j < 3; j++) {
              wr[j] = (swap ? p2[j] : p1[j]) ^ nre;
              wi[j] = (swap ? p1[j] : p2[j]) ^ nim;
            }
            const int o = 6 * sp + 2 * li;  // rows o (re) and o + 1 (im)
            const uint32_t core = (uint32_t)(2 * lh + src) * 128;
            sts128(Ls + (uint32_t)(o >> 3) * kTcSbo + (uint32_t)(o & 7) * 16 + core, wr[0], wr[1], wr[2], 0u);
            sts128(Ls + (uint32_t)((o + 1) >> 3) * kTcSbo + (uint32_t)((o + 1) & 7) * 16 + core, wi[0], wi[1], wi[2],
                   0u);
          }
        }
        if (hx >= 0) {
          float mx = 0.f;
#pragma unroll
          for (int dd = 0; dd < 8; dd++) mx = fmaxf(mx, nr[dd]);
          const float inv = mx > 0.f ? 1.0f / mx : 0.f;
          const uint32_t hrow = Hb + (uint32_t)b * kTcHBuf + (uint32_t)hs * kTcHSite + (uint32_t)(rl >> 3) * kTcSbo +
                                (uint32_t)(rl & 7) * 16;
          if (hh == 0) {
            scl[(n & 3) * kTcPairs + pair] = mx;
            tc_h_block<DAG, 0>(w[0], __float2half2_rn(nr[0] * inv), hrow);
            tc_h_block<DAG, 1>(w[1], __float2half2_rn(nr[1] * inv), hrow);
            tc_h_block<DAG, 2>(w[2], __float2half2_rn(nr[2] * inv), hrow);
            tc_h_block<DAG, 3>(w[3], __float2half2_rn(nr[3] * inv), hrow);
          } else {
            tc_h_block<DAG, 4>(w[0], __float2half2_rn(nr[4] * inv), hrow);
            tc_h_block<DAG, 5>(w[1], __float2half2_rn(nr[5] * inv), hrow);
            tc_h_block<DAG, 6>(w[2], __float2half2_rn(nr[6] * inv), hrow);
            tc_h_block<DAG, 7>(w[3], __float2half2_rn(nr[7] * inv), hrow);
          }
        }
        // the tensor cores read what this thread wrote
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(bfull + 8 * b);
      }
    }
  } else if (warp == kTcMmaWarp) {
    // ------------------------------------------------------ MMA issue
    if (lane == 0) {
      constexpr uint32_t idesc = tc_idesc(64, 16);
      int n = 0;
      for (int lt = 0; lt < my_tiles; lt++) {
        for (int g = 0; g < G; g++, n++) {
          const int b = n & 1;
          tc_wait(bfull + 8 * b, (n >> 1) & 1, ctl, failed);
          if (n >= 2) tc_wait(btfree + 8 * b, ((n >> 1) & 1) ^ 1, ctl, failed);  // epilogue of item n - 2
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          // the producers' rescale factors of item n, released to the epilogue
          mbar_arrive(bsready + 8 * b);
          if (ctl.skip_mma) continue;
          // descriptors of the item's first operands; later sites and K steps
          // add their byte offsets / 16 to the 14-bit address field
          const uint64_t ad0 = tc_sdesc(Lb + (uint32_t)(lt & 1) * kTcLBuf, 128, kTcSbo);
          const uint64_t bd0 = tc_sdesc(Hb + (uint32_t)b * kTcHBuf, 128, kTcSbo);
#pragma unroll
          for (int t = 0; t < kTcSites; t++) {
#pragma unroll
            for (int kk = 0; kk < kTcK / 16; kk++) {
              const uint64_t ad = ad0 + (uint64_t)((t * kTcLSite + kk * 256) >> 4);
              const uint64_t bd = bd0 + (uint64_t)((t * kTcHSite + kk * 256) >> 4);
              const uint32_t dt = tmem + (uint32_t)(b * kTcSites * 16 + t * 16);
              if (kk == 0)
                asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, 0;" ::"r"(dt), "l"(ad), "l"(bd),
                             "r"(idesc));
              else
                asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, 1;" ::"r"(dt), "l"(ad), "l"(bd),
                             "r"(idesc));
            }
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bdone + 8 * b)
                       : "memory");
          last_item = n;
        }
      }
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------ epilogue
    const int et = tid - kTcEpiWarp0 * 32;  // (site, slot) pair
    const int s = et >> 4, rl = et & 15;
    // warp sub = 0 reads accumulator rows 0..15 (lanes 0..15), sub = 1 rows
    // 16..23 (lanes 32..39) of the M = 64 layout (row i in lane 32 (i / 16) + i % 16)
    const int sub = warp & 3;
    const bool reader = true;
    constexpr int zmode = MODE == 1 ? 0 : 2;
    constexpr bool ainv = MODE == 1;
    constexpr float ch = MODE == 0 ? -0.5f : MODE == 1 ? 1.0f : -0.25f;
    double run[4] = {0.0, 0.0, 0.0, 0.0};  // per-slot |out|^2 of the CTA (threads 0..15)
    int n = 0;
    for (int lt = 0; lt < my_tiles; lt++) {
      const int base = ((int)blockIdx.x + lt * (int)gridDim.x) * kTcSites;
      const int e = base + s;
      const bool act = e < a.V;
      for (int g = 0; g < G; g++, n++) {
        const int b = n & 1, r = g * 16 + rl;
        // the diagonal term does not wait for the tensor cores
        C<float> zs[1][12];
        float znrm[1] = {0.f};
        if (zmode && act) mload_rp<1>(a, EO ? a.z : a.in, EO ? a.z_norm : a.in_norm, e, r, zs, znrm);
        tc_wait(bdone + 8 * b, (n >> 1) & 1, ctl, failed);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        tc_wait(bsready + 8 * b, (n >> 1) & 1, ctl, failed);
        const float sc = scl[(n & 3) * kTcPairs + et];
        if (reader) {
#pragma unroll
          for (int t0 = 0; t0 < kTcSites; t0 += 4) {  // four sites per batch of loads
            uint32_t v[4][16];
#pragma unroll
            for (int q = 0; q < 4; q++) {
              const uint32_t ta = tmem + ((uint32_t)(sub * 32) << 16) + (uint32_t)(b * kTcSites * 16 + (t0 + q) * 16);
              asm volatile(
                  "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                  "[%16];"
                  : "=r"(v[q][0]), "=r"(v[q][1]), "=r"(v[q][2]), "=r"(v[q][3]), "=r"(v[q][4]), "=r"(v[q][5]),
                    "=r"(v[q][6]), "=r"(v[q][7]), "=r"(v[q][8]), "=r"(v[q][9]), "=r"(v[q][10]), "=r"(v[q][11]),
                    "=r"(v[q][12]), "=r"(v[q][13]), "=r"(v[q][14]), "=r"(v[q][15])
                  : "r"(ta));
            }
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            const int o = sub * 16 + lane;  // accumulator row
            if (lane < 16 && o < 24) {
#pragma unroll
              for (int q = 0; q < 4; q++)
#pragma unroll
                for (int c = 0; c < 16; c++) X[((t0 + q) * 16 + c) * 24 + o] = __uint_as_float(v[q][c]);
            }
          }
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        }
        tc_named_bar(1, kTcEpi);  // X complete, every thread has read its rescale
        if (reader && lane == 0) mbar_arrive(btfree + 8 * b);
        double n2 = 0.0;
        if (act) {
          C<float> acc[12];
          const float *xi = X + et * 24;
#pragma unroll
          for (int k = 0; k < 12; k++) acc[k] = C<float>{sc * xi[2 * k], sc * xi[2 * k + 1]};
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
          red[et] = n2;
          tc_named_bar(1, kTcEpi);
          if (et < 16) {
            double t = 0.0;
            for (int i = 0; i < kTcSites; i++) t += red[i * 16 + et];
            run[g] += t;
          }
        }
        tc_named_bar(1, kTcEpi);  // X and red are rewritten by the next item
      }
    }
    if (partials && et < 16)
      for (int g = 0; g < G; g++) partials[(int64_t)blockIdx.x * a.N + g * 16 + et] = run[g];
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == kTcMmaWarp) {
    // a role that stopped waiting may have left MMAs in flight: wait for the
    // last commit (bounded) before the tensor memory is released
    if (lane == 0 && last_item >= 0) {
      const int b = last_item & 1;
      tc_wait(bdone + 8 * b, (last_item >> 1) & 1, ctl, failed);
    }
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(kTcCols));
  }
  if (failed) atomicAdd(&g_mrhs_tc_timeouts, 1u);
}

// two CTAs per SM (the kernel's shared memory allows no third), at most one per tile
unsigned mrhs_tc_grid(int64_t V)
{
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
      sms = 1;
  }
  const int64_t tiles = (V + kTcSites - 1) / kTcSites;
  return (unsigned)(tiles < 2 * sms ? tiles : 2 * sms);
}

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
static int g_tc_polls = 1 << 20;
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
  // the FP32 copy holds the boundary phases folded into its links
  a.twist_mask = 0;
  for (int mu = 0; mu < 4; mu++) {
    a.phr[mu] = 1.f;
    a.phi[mu] = 0.f;
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
      (z && (z->N != in->N || z->V != in->V)) || g->prec != QCDGPU_F64 || !eo_lattice(g->L) ||
      in->L[0] * 2 != g->L[0] || in->L[1] != g->L[1] || in->L[2] != g->L[2] || in->L[3] != g->L[3] ||
      memcmp(out->L, in->L, sizeof(in->L)) != 0 || nact < 0 || nact > in->N || !mp4s || !tms) {
    set_error("even/odd multi-RHS operator: half-lattice fields of one shape (every extent even), per-slot "
              "diagonal");
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
  // the FP32 copy holds the boundary phases folded into its links
  a.twist_mask = 0;
  for (int mu = 0; mu < 4; mu++) {
    a.phr[mu] = 1.f;
    a.phi[mu] = 0.f;
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
  qg::g_tc_polls = polls > 0 ? polls : 1 << 20;
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
