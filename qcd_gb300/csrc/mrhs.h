// mrhs.h -- multi-RHS fields and operator, shared by the operator (mrhs.cu)
// and the batched solver (mrhs_cg.cu).
#pragma once

#include "internal.h"

// N spinors in FP16 with one float norm per (site, RHS). The 12 complex
// components of a spinor form three groups of four; group j of slot r at
// site x is one 16-byte word (8 halves: re, im of components 4j..4j+3) at
// uint4 index (j * V + x) * N + r. A thread reads a whole spinor with three
// 128-bit loads, and the threads of consecutive (site, slot) pairs read
// consecutive words. Norms are [site][slot] floats.
struct qcdgpu_mfield_s {
  int L[4];
  int64_t V;
  int N;  // RHS slots
  void *data;
  float *norm;
  size_t bytes;
};

namespace qg {

// spinor (x, r) of a multi-RHS field as 12 float2 (without the norm)
__device__ __forceinline__ void mload_raw(const __half2 *d, int64_t V, int N, int x, int r, float2 v[12])
{
  const uint4 *p = (const uint4 *)d;
#pragma unroll
  for (int j = 0; j < 3; j++) {
    const uint4 w = p[((int64_t)j * V + x) * N + r];
    v[4 * j + 0] = __half22float2(*(const __half2 *)&w.x);
    v[4 * j + 1] = __half22float2(*(const __half2 *)&w.y);
    v[4 * j + 2] = __half22float2(*(const __half2 *)&w.z);
    v[4 * j + 3] = __half22float2(*(const __half2 *)&w.w);
  }
}

// spinor (x, r) <- 12 float2 multiplied by inv, rounded to FP16
__device__ __forceinline__ void mstore_raw(__half2 *d, int64_t V, int N, int x, int r, const float2 v[12], float inv)
{
  uint4 *p = (uint4 *)d;
#pragma unroll
  for (int j = 0; j < 3; j++) {
    __half2 h[4];
#pragma unroll
    for (int i = 0; i < 4; i++) h[i] = __floats2half2_rn(v[4 * j + i].x * inv, v[4 * j + i].y * inv);
    uint4 w;
    w.x = *(const unsigned *)&h[0];
    w.y = *(const unsigned *)&h[1];
    w.z = *(const unsigned *)&h[2];
    w.w = *(const unsigned *)&h[3];
    p[((int64_t)j * V + x) * N + r] = w;
  }
}

// component k of spinor (x, r) as one half2
__device__ __forceinline__ int64_t mhalf2_index(int64_t V, int N, int k, int x, int r)
{
  return (((int64_t)(k >> 2) * V + x) * N + r) * 4 + (k & 3);
}

qcdgpu_mfield mfield_new(const int L[4], int N);
void mfield_free(qcdgpu_mfield m);
bool mfield_set(qcdgpu_mfield m, int r, qcdgpu_field f);
bool mfield_get(qcdgpu_field f, qcdgpu_mfield m, int r);

// out = D in (dag: D^+ in) for slots 0..nact-1. With mp4s / tms (device
// float arrays) slot r uses its own diagonal. With `partials` the call also
// leaves, per block b and slot r, partials[b * N + r] = the sum of |out_r|^2
// over the block's sites, and *nblocks = the number of blocks; partials must
// hold mrhs_max_blocks(V, N) * N doubles.
bool dslash_mrhs(qcdgpu_mfield out, qcdgpu_mfield in, qcdgpu_gauge g, double mp4, double tm, bool dag, int nact,
                 const float *mp4s, const float *tms, double *partials = nullptr, unsigned *nblocks = nullptr);
unsigned mrhs_max_blocks(int64_t V, int N);
// even/odd kernel on half-lattice fields (SIMT): out (parity par) =
// ch * [A^{-1}] H in + {0 | z | A z} with the slots' diagonals A
bool dslash_mrhs_eo(qcdgpu_mfield out, qcdgpu_mfield in, qcdgpu_mfield z, qcdgpu_gauge g, bool dag, int nact,
                    const float *mp4s, const float *tms, int par, double ch, bool ainv, int zmode, double *partials,
                    unsigned *nblocks);

// a tensor-core launch ran out of a bounded wait and abandoned its work (a
// host-mapped flag the kernel sets: reading it needs no synchronisation)
bool mrhs_tc_failed();

// operator variants picked by the tuner
enum { MRHS_AUTO = -1, MRHS_SIMT = 0, MRHS_MMA = 1, MRHS_TC = 2 };

}  // namespace qg

namespace qg {

// batched solver pieces used by the request server (serve.cu): enqueue one
// chunk of iterations of every occupied slot on the batch's own stream, and
// wait for it and apply reliable updates / retirement
bool batch_launch(qcdgpu_batch B);
bool batch_finish(qcdgpu_batch B);
// a chunk is launched and not yet finished
bool batch_in_flight(qcdgpu_batch B);
// the launched chunk's work has completed on the device (batch_finish will
// not wait)
bool batch_chunk_done(qcdgpu_batch B);

}  // namespace qg
