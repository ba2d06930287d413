// dslash_args.h -- launch arguments shared by the operator kernels.
#pragma once

#include "internal.h"

namespace qg {

struct DArgs {
  void *out;
  float *out_norm;
  const void *in;
  const float *in_norm;
  const void *gauge;
  qgd::Geom geo;
  int x0;  // sites x0 .. V-1 (a range of a full-lattice launch; 0 otherwise)
  int V;
  int64_t stride;   // spinor block stride
  int64_t gstride;  // gauge block stride
  // scalars in double and as float pairs (hi + lo), so kernels of every
  // arithmetic type read them without converting on the FP64 pipe
  double phr[4], phi[4], mp4, tm;  // tm already negated for D^+
  float phr_h[4], phr_l[4], phi_h[4], phi_l[4], mp4_h, mp4_l, tm_h, tm_l;
  int twist_mask;
  int op_q;          // multiply the result by i g5
  double *partials;  // non-null: block b writes sum over its sites of |out|^2 to partials[b]
  // even/odd kernels (k_wilson_eo): the sites of parity eo_par only, V = half
  // volume; in, out and z are half fields indexed by (full site index) >> 1
  // (t extent even). out = ch * [A^{-1}] H in + {0 | z | A z}, with
  // A = mp4 + i tm g5 and H the hopping sum of the operator.
  int eo_par;
  const void *z;
  const float *z_norm;
  int zmode;  // 0: no addend, 1: + z, 2: + A z
  int ainv;   // 1: hopping term multiplied by A^{-1}
  double ch, ai_r, ai_i;  // A^{-1} = ai_r + i ai_i g5
  float ch_h, ch_l, ai_r_h, ai_r_l, ai_i_h, ai_i_l;
  // 1: in and out are in the host layout, [site][spin][colour] complex
  // double (12 double2 per site), instead of component blocks of `stride`
  // sites (full-lattice float-float kernel only)
  int aos = 0;
  // non-null (with partials): the CG step alpha = rr / (sum of the partials)
  // is formed by the block that finishes last (cg_last_block, mode 0)
  unsigned *cg_done = nullptr;
  double *cg_s = nullptr;
  int cg_hist = 0;
};

// the CG scalars a launch of the operator may update at its end
struct CgFuse {
  unsigned *done;  // arrival counter (zero between launches)
  double *s;       // the solver's scalar slots
  int hist;
};

// |v|^2 summed over the block into partials[blockIdx.x]; every thread of the
// block must call it (blockDim.x a multiple of 32, at most 1024)
__device__ __forceinline__ void block_partial(double v, double *partials)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += sh[i];
    partials[blockIdx.x] = s;
  }
}

// scalar slots
enum { S_RR = 0, S_PAP = 1, S_RRNEW = 2, S_ALPHA = 3, S_BETA = 4, S_HIST = 8 };

// the CG scalars from a reduced total: mode 0 t = p^+ A p -> alpha;
// mode 1 t = |r|^2 -> beta and the residual history
__device__ __forceinline__ void cg_scalars_from(double t, double *s, int mode, int hist)
{
  if (mode == 0) {
    s[S_PAP] = t;
    s[S_ALPHA] = t > 0.0 ? s[S_RR] / t : nan("");  // p^+ A p <= 0: breakdown
  } else {
    s[S_RRNEW] = t;
    s[S_BETA] = t / s[S_RR];
    s[S_RR] = t;
    s[S_HIST + hist] = t;
  }
}

// Called by every thread of a 128-thread block after block_partial wrote the
// block's partial: the block that finishes last sums all gridDim.x partials
// in index order (the same order whichever block is last), updates the
// scalars and re-arms the counter. No block waits for another.
__device__ __forceinline__ void cg_last_block(const double *partials, unsigned *done, double *s, int mode, int hist)
{
  __shared__ unsigned last;
  __shared__ double sh[32];
  if (threadIdx.x == 0) {
    __threadfence();  // this block's partial before its count
    last = atomicAdd(done, 1u) == gridDim.x - 1 ? 1u : 0u;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // eight independent loads in flight per thread, summed in a fixed order
  const int n = (int)gridDim.x;
  double v = 0.0;
  const int nt = (int)blockDim.x;
  for (int i0 = threadIdx.x; i0 < n; i0 += 8 * nt) {
    double w[8];
#pragma unroll
    for (int k = 0; k < 8; k++) w[k] = i0 + k * nt < n ? __ldcg(partials + i0 + k * nt) : 0.0;
#pragma unroll
    for (int k = 0; k < 8; k++) v += w[k];
  }
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < nt >> 5; i++) t += sh[i];
    cg_scalars_from(t, s, mode, hist);
    *done = 0u;
  }
}

// the kernels' end with partials: the block partial, then (cg_done) the CG
// step from all of them
__device__ __forceinline__ void block_partial_cg(double v, const DArgs &a)
{
  block_partial(v, a.partials);
  if (a.cg_done) cg_last_block(a.partials, a.cg_done, a.cg_s, 0, a.cg_hist);
}

// a launch scalar in the kernel's arithmetic type R
template <typename R>
struct Scalar;
template <>
struct Scalar<double> {
  __device__ __forceinline__ static double get(double d, float, float) { return d; }
};
template <>
struct Scalar<float> {
  __device__ __forceinline__ static float get(double, float h, float) { return h; }
};

inline void split_host(double d, float *h, float *l)
{
  *h = (float)d;
  *l = (float)(d - (double)*h);
}

}  // namespace qg
