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
  int V;
  int64_t stride;   // spinor block stride
  int64_t gstride;  // gauge block stride
  // scalars in double and as float pairs (hi + lo), so kernels of every
  // arithmetic type read them without converting on the FP64 pipe
  double phr[4], phi[4], mp4, tm;  // tm already negated for D^+
  float phr_h[4], phr_l[4], phi_h[4], phi_l[4], mp4_h, mp4_l, tm_h, tm_l;
  int twist_mask;
  int op_q;  // multiply the result by i g5
};

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
