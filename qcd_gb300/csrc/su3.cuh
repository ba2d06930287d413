// su3.cuh -- 3x3 complex matrix helpers for the gauge-field kernels
// (generator, smearing, plaquette). Matrices are row-major C<double>[9].
#pragma once

#include "internal.h"

namespace qg {

using namespace qgd;

__device__ __forceinline__ void m3mul(const C<double> a[9], const C<double> b[9], C<double> c[9])
{
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) c[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
}

// Gram-Schmidt on columns 0,1 and col2 = conj(col0 x col1)
__device__ __forceinline__ void reunit_cols(C<double> U[9])
{
  double n = 0;
#pragma unroll
  for (int i = 0; i < 3; i++) n += U[3 * i].re * U[3 * i].re + U[3 * i].im * U[3 * i].im;
  C<double> w{0, 0};
#pragma unroll
  for (int i = 0; i < 3; i++) w = w + cdot(U[3 * i], U[3 * i + 1]);
  w = (1.0 / n) * w;
#pragma unroll
  for (int i = 0; i < 3; i++) U[3 * i + 1] = U[3 * i + 1] - w * U[3 * i];
  double s = 1.0 / sqrt(n);
#pragma unroll
  for (int i = 0; i < 3; i++) U[3 * i] = s * U[3 * i];
  n = 0;
#pragma unroll
  for (int i = 0; i < 3; i++) n += U[3 * i + 1].re * U[3 * i + 1].re + U[3 * i + 1].im * U[3 * i + 1].im;
  s = 1.0 / sqrt(n);
#pragma unroll
  for (int i = 0; i < 3; i++) U[3 * i + 1] = s * U[3 * i + 1];
  U[2] = conj(U[3] * U[7] - U[6] * U[4]);
  U[5] = conj(U[6] * U[1] - U[0] * U[7]);
  U[8] = conj(U[0] * U[4] - U[3] * U[1]);
}

}  // namespace qg
