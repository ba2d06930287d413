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
