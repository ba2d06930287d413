// mrhs.h -- multi-RHS fields and operator, shared by the operator (mrhs.cu)
// and the batched solver (mrhs_cg.cu).
#pragma once

#include "internal.h"

// N spinors in FP16 with one float norm per (site, RHS), laid out
// [component 0..11][site][rhs] as half2 (re, im): the RHS of one site and
// component are contiguous
struct qcdgpu_mfield_s {
  int L[4];
  int64_t V;
  int N;  // RHS slots
  void *data;
  float *norm;
  size_t bytes;
};

namespace qg {

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

// operator variants picked by the tuner
enum { MRHS_AUTO = -1, MRHS_SIMT = 0, MRHS_MMA = 1 };

}  // namespace qg

namespace qg {

// batched solver pieces used by the request server (serve.cu): enqueue one
// chunk of iterations of every occupied slot on the batch's own stream, and
// wait for it and apply reliable updates / retirement
bool batch_launch(qcdgpu_batch B);
bool batch_finish(qcdgpu_batch B);

}  // namespace qg
