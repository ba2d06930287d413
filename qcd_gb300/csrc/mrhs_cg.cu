// mrhs_cg.cu -- batched CG on the normal equations for many right-hand sides,
// with continuous admission and retirement (the engine behind the serving
// loop).
//
// A batch owns multi-RHS work fields (FP16 with per-(site, slot) norms; the
// solution increments in FP32) with a fixed number of slots and runs the
// mixed-precision reliable-update CG of cg.cu for all occupied slots at once:
// every inner iteration is two multi-RHS operator launches (the first also
// sums |D p|^2 per slot) plus three small per-(site, slot) kernels, with
// per-slot scalars kept on the device; a chunk of 16 iterations is one CUDA
// graph launch. The operator's hopping term does not
// depend on kappa or mu, so each slot carries its own diagonal and a batch
// mixes requests of different kappa and twisted mass on one gauge field.
// Between chunks of iterations the host reads the per-slot residual
// histories, performs reliable updates (FP64 true residual per slot),
// retires converged slots by moving the last occupied slot into their place,
// and admits new right-hand sides into free slots -- while the others keep
// iterating. Every reduction sums in a fixed order per slot, independent of
// which other slots are occupied, so a right-hand side converges to the same
// result alone and in any mix.
#include <math.h>
#include <string.h>

#include <vector>

#include "mrhs.h"

namespace qg {

using namespace qgd;

struct MV {
  __half2 *d;
  float *n;
  int V, N;
};
static MV mv(qcdgpu_mfield m) { return MV{(__half2 *)m->data, m->norm, (int)m->V, m->N}; }

__device__ __forceinline__ void mv_load(const MV &m, int x, int r, float2 v[12])
{
  const float s = m.n[(int64_t)x * m.N + r];
  mload_raw(m.d, m.V, m.N, x, r, v);
#pragma unroll
  for (int k = 0; k < 12; k++) v[k] = make_float2(v[k].x * s, v[k].y * s);
}
__device__ __forceinline__ void mv_store(const MV &m, int x, int r, const float2 v[12])
{
  float mx = 0.f;
#pragma unroll
  for (int k = 0; k < 12; k++) mx = fmaxf(mx, fmaxf(fabsf(v[k].x), fabsf(v[k].y)));
  if (!(mx >= 1.17549435e-38f)) mx = 0.f;
  const float inv = mx > 0.f ? 1.0f / mx : 0.f;
  mstore_raw(m.d, m.V, m.N, x, r, v, inv);
  m.n[(int64_t)x * m.N + r] = mx;
}

// Launch shape of the per-(site, slot) kernels: block (N, SB) -- x = slot,
// y = site within the block -- so a warp reads the slots of one site
// contiguously; partials[block * N + slot] receives the block's sum for each
// slot in a fixed order.
static dim3 mblock(int N) { return dim3((unsigned)N, (unsigned)(256 / N > 0 ? 256 / N : 1)); }
static unsigned mgrid(int V, int N) { return (unsigned)((V + mblock(N).y - 1) / mblock(N).y); }

// block partials of the blockDim.x occupied slots, at slot stride N
__device__ __forceinline__ void slot_partial(double v, double *partials, int N)
{
  extern __shared__ double sh[];
  const int NS = blockDim.x, r = threadIdx.x, y = threadIdx.y;
  sh[y * NS + r] = v;
  __syncthreads();
  if (y == 0) {
    double s = 0.0;
    for (int i = 0; i < (int)blockDim.y; i++) s += sh[i * NS + r];
    partials[(int64_t)blockIdx.x * N + r] = s;
  }
}

// FP32 solution increments of the slots: components 2j, 2j+1 of slot r at
// site x form the float4 at index (j * V + x) * N + r, j = 0..5. FP16 would
// round every increment to 11 bits and cost iterations.
struct MX {
  float4 *d;
  int V, N;
};

// xs += alpha p ; rs -= alpha Ap ; partials <- |rs|^2 per slot
__global__ void k_mupdate(MX xs, MV ps, MV rs, MV aps, int nact, const double *alpha, double *partials)
{
  const int r = threadIdx.x, x = blockIdx.x * blockDim.y + threadIdx.y;
  double n2 = 0.0;
  if (r < nact && x < xs.V) {
    const float al = (float)alpha[r];
    float2 a[12], b[12];
    mv_load(ps, x, r, b);
#pragma unroll
    for (int j = 0; j < 6; j++) {
      float4 &v = xs.d[((int64_t)j * xs.V + x) * xs.N + r];
      const float4 w = v;
      v = make_float4(__fmaf_rn(al, b[2 * j].x, w.x), __fmaf_rn(al, b[2 * j].y, w.y),
                      __fmaf_rn(al, b[2 * j + 1].x, w.z), __fmaf_rn(al, b[2 * j + 1].y, w.w));
    }
    mv_load(rs, x, r, a);
    mv_load(aps, x, r, b);
    float s2 = 0.f;  // per-site sum in FP32, block sum in double
#pragma unroll
    for (int k = 0; k < 12; k++) {
      a[k] = make_float2(__fmaf_rn(-al, b[k].x, a[k].x), __fmaf_rn(-al, b[k].y, a[k].y));
      s2 += a[k].x * a[k].x + a[k].y * a[k].y;
    }
    mv_store(rs, x, r, a);
    n2 = (double)s2;
  }
  slot_partial(n2, partials, xs.N);
}

// f (FP64 field) += slot r of xs, then slot r of xs <- 0
__global__ void k_mx_flush(double2 *f, int64_t fstride, MX xs, int r)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= xs.V) return;
#pragma unroll
  for (int j = 0; j < 6; j++) {
    float4 &v = xs.d[((int64_t)j * xs.V + x) * xs.N + r];
    double2 &o0 = f[(int64_t)(2 * j) * fstride + x];
    double2 &o1 = f[(int64_t)(2 * j + 1) * fstride + x];
    const float4 w = v;
    o0.x += (double)w.x;
    o0.y += (double)w.y;
    o1.x += (double)w.z;
    o1.y += (double)w.w;
    v = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// slot `to` of xs <- slot `from` (zero == 1: <- 0)
__global__ void k_mx_copy(MX xs, int from, int to, int zero)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= xs.V) return;
#pragma unroll
  for (int j = 0; j < 6; j++)
    xs.d[((int64_t)j * xs.V + x) * xs.N + to] =
        zero ? make_float4(0.f, 0.f, 0.f, 0.f) : xs.d[((int64_t)j * xs.V + x) * xs.N + from];
}

// ps = rs + beta ps
__global__ void k_mp(MV ps, MV rs, int nact, const double *beta)
{
  const int r = threadIdx.x, x = blockIdx.x * blockDim.y + threadIdx.y;
  if (r >= nact || x >= ps.V) return;
  const float be = (float)beta[r];
  float2 p[12], q[12];
  mv_load(ps, x, r, p);
  mv_load(rs, x, r, q);
#pragma unroll
  for (int k = 0; k < 12; k++) p[k] = make_float2(__fmaf_rn(be, p[k].x, q[k].x), __fmaf_rn(be, p[k].y, q[k].y));
  mv_store(ps, x, r, p);
}

// slot `to` <- slot `from` (zero == 1: slot `to` <- 0)
__global__ void k_mcopy(MV m, int from, int to, int zero)
{
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= m.V) return;
  uint4 *p = (uint4 *)m.d;
#pragma unroll
  for (int j = 0; j < 3; j++)
    p[((int64_t)j * m.V + x) * m.N + to] = zero ? make_uint4(0u, 0u, 0u, 0u) : p[((int64_t)j * m.V + x) * m.N + from];
  m.n[(int64_t)x * m.N + to] = zero ? 0.f : m.n[(int64_t)x * m.N + from];
}

// scalar layout, per slot r of N: rr, pAp, alpha, beta, then history[j]
enum { M_RR = 0, M_PAP = 1, M_ALPHA = 2, M_BETA = 3, M_HIST = 4 };
constexpr int kMChunk = 16;

// Per-slot sums of the nb block partials, in two levels: block g of kMSGroups sums a contiguous
// range of the nb block partials for every slot (consecutive threads read
// consecutive slots: coalesced), and the block that finishes last sums the
// kMSGroups group sums per slot, both in a fixed order, and updates the
// scalars of the nact occupied slots. No block waits for another.
constexpr int kMSGroups = 128;
__global__ void __launch_bounds__(256) k_mscalars2(const double *partials, int nb, int N, int nact, double *s,
                                                   int mode, int hist, double *l1, unsigned *done)
{
  const int K = (int)blockDim.x / N;  // thread groups per slot (N <= 64)
  const int r = (int)threadIdx.x % N, k = (int)threadIdx.x / N;
  const int per = (nb + (int)gridDim.x - 1) / (int)gridDim.x;
  const int b0 = (int)blockIdx.x * per, b1 = min(nb, b0 + per);
  double v = 0.0;
  if (k < K)
    for (int b = b0 + k; b < b1; b += K) v += partials[(int64_t)b * N + r];
  __shared__ double sh[256];
  __shared__ unsigned last;
  sh[threadIdx.x] = v;
  __syncthreads();
  if ((int)threadIdx.x < N) {
    double t = 0.0;
    for (int kk = 0; kk < K; kk++) t += sh[kk * N + threadIdx.x];
    l1[(int64_t)blockIdx.x * N + threadIdx.x] = t;
  }
  __threadfence();  // the group sums before the count
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1 ? 1u : 0u;
  __syncthreads();
  if (!last) return;
  __threadfence();
  // slot r's group sums split over the K thread groups, eight loads in flight
  const int G = (int)gridDim.x;
  double w = 0.0;
  if (k < K)
    for (int g0 = k; g0 < G; g0 += 8 * K) {
      double q[8];
#pragma unroll
      for (int i = 0; i < 8; i++) q[i] = g0 + i * K < G ? __ldcg(l1 + (int64_t)(g0 + i * K) * N + r) : 0.0;
#pragma unroll
      for (int i = 0; i < 8; i++) w += q[i];
    }
  __syncthreads();
  sh[threadIdx.x] = w;
  __syncthreads();
  if ((int)threadIdx.x < nact) {
    const int rr = threadIdx.x;
    double t = 0.0;
    for (int kk = 0; kk < K; kk++) t += sh[kk * N + rr];
    if (mode == 0) {
      s[M_PAP * N + rr] = t;
      s[M_ALPHA * N + rr] = t > 0.0 ? s[M_RR * N + rr] / t : nan("");
    } else {
      s[M_BETA * N + rr] = t / s[M_RR * N + rr];
      s[M_RR * N + rr] = t;
      s[(M_HIST + hist) * N + rr] = t;
    }
  }
  if (threadIdx.x == 0) *done = 0u;
}

}  // namespace qg

// ----------------------------------------------------------------- engine
namespace qg {

struct BSlot {
  int tag;
  qcdgpu_field x, b;  // caller's FP64 fields
  // even/odd batches: the slot's FP64 half fields -- system right-hand side
  // c_e = b_e + H_eo A^{-1} b_o / 2, A^{-1} b_o, and the solution x_e. x is
  // written only when the slot retires, so c_e and A^{-1} b_o are kept in
  // x's own memory until then (views; their own allocations when x has no
  // room for two half fields); x_e comes from the batch's per-slot pool.
  qcdgpu_field ce, to, xe;
  int op;             // QCDGPU_OP_D or QCDGPU_OP_Q
  double mp4, tm, bn, tol, delta, maxr, hint, true_res;
  int iters, maxiter, updates, since;
};

struct BDone {
  int tag, status, iters, updates;
  double true_res;
};

}  // namespace qg

struct qcdgpu_batch_s {
  qcdgpu_gauge g;
  int cap, nact;
  // even/odd: the slots solve the Schur complement M x_e = c_e on the half
  // lattice (Ls, Vs); otherwise D^+ D on the full lattice
  bool eo;
  int Ls[4];
  int64_t Vs;
  qcdgpu_mfield rs, ps, t, aps, u;  // u: odd intermediate (even/odd only)
  float4 *xs;                  // FP32 solution increments (layout of MX)
  qcdgpu_field rt, r, up, bd;  // FP64 work shared by the slots' reliable updates
  qcdgpu_field u64, r32, u32, s32;  // even/odd: FP64 odd temp; FP32 restart fields
  std::vector<qcdgpu_field> spare;  // even/odd: free per-slot x_e fields
  double *s;                   // device scalars, (M_HIST + kMChunk) * cap
  float *mp4s, *tms;           // device per-slot diagonal
  double *part;                // device partials
  double *l1;                  // group sums of the two-level reduction, kMSGroups * cap
  unsigned *msdone;            // its block counter
  double *hs;                  // pinned host copy of the scalars
  double *rudev, *ruhost;      // reliable updates' norms, 4 per slot (device, pinned host)
  std::vector<qg::BSlot> slots;
  std::vector<qg::BDone> done;
  cudaStream_t st;             // the stream the batch's work runs on
  cudaEvent_t ev;              // end of the launched chunk
  cudaEvent_t ev_in;           // caller's stream at admission
  int nchunk;                  // occupied slots of the launched chunk
  bool use_graphs;
  bool tuned;                  // the operator variant has been chosen
  std::vector<cudaGraphExec_t> graphs;  // chunk graph per occupied-slot count
  std::vector<uint64_t> graph_launches;  // kernels in each graph
};

namespace qg {

static MX mx(qcdgpu_batch B) { return MX{B->xs, (int)B->Vs, B->cap}; }

static void batch_free(qcdgpu_batch b)
{
  if (!b) return;
  if (b->st) cudaStreamSynchronize(b->st);  // a chunk may still be running
  for (auto m : {b->rs, b->ps, b->t, b->aps, b->u}) mfield_free(m);
  cudaFree(b->xs);
  for (auto f : {b->rt, b->r, b->up, b->bd, b->u64, b->r32, b->u32, b->s32}) field_free(f);
  for (auto &sl : b->slots)
    for (auto f : {sl.ce, sl.to, sl.xe}) field_free(f);
  for (auto f : b->spare) field_free(f);
  cudaFree(b->s);
  cudaFree(b->mp4s);
  cudaFree(b->tms);
  cudaFree(b->part);
  cudaFree(b->l1);
  cudaFree(b->rudev);
  cudaFreeHost(b->ruhost);
  cudaFreeHost(b->hs);
  for (auto e : b->graphs)
    if (e) cudaGraphExecDestroy(e);
  if (b->ev) cudaEventDestroy(b->ev);
  if (b->ev_in) cudaEventDestroy(b->ev_in);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
}

static qcdgpu_batch batch_new(qcdgpu_gauge g, int cap, bool eo)
{
  if (!g || g->prec != QCDGPU_F64 || cap < 1 || cap > 64 || (eo && !eo_lattice(g->L))) {
    set_error("batch: FP64 gauge field, 1..64 slots, every extent even for even/odd");
    return nullptr;
  }
  auto *b = new qcdgpu_batch_s();
  b->g = g;
  b->cap = cap;
  b->eo = eo;
  memcpy(b->Ls, g->L, sizeof(b->Ls));
  if (eo) b->Ls[0] /= 2;
  b->Vs = (int64_t)b->Ls[0] * b->Ls[1] * b->Ls[2] * b->Ls[3];
  b->nact = 0;
  b->st = nullptr;
  b->nchunk = 0;
  b->use_graphs = true;
  b->graphs.assign((size_t)cap + 1, nullptr);
  b->graph_launches.assign((size_t)cap + 1, 0);
  b->rs = mfield_new(b->Ls, cap);
  b->ps = mfield_new(b->Ls, cap);
  b->t = mfield_new(b->Ls, cap);
  b->aps = mfield_new(b->Ls, cap);
  b->rt = field_new(b->Ls, QCDGPU_F64);
  b->r = field_new(b->Ls, QCDGPU_F64);
  b->up = field_new(b->Ls, QCDGPU_F64);
  b->bd = field_new(g->L, QCDGPU_F64);
  bool ok = b->rs && b->ps && b->t && b->aps && b->rt && b->r && b->up && b->bd;
  if (eo) {
    b->u = mfield_new(b->Ls, cap);
    b->u64 = field_new(b->Ls, QCDGPU_F64);
    b->r32 = field_new(b->Ls, QCDGPU_F32);
    b->u32 = field_new(b->Ls, QCDGPU_F32);
    b->s32 = field_new(b->Ls, QCDGPU_F32);
    ok = ok && b->u && b->u64 && b->r32 && b->u32 && b->s32;
    for (int k = 0; ok && k < cap; k++) {
      b->spare.push_back(field_new(b->Ls, QCDGPU_F64));
      ok = b->spare.back() != nullptr;
    }
  }
  size_t ns = (size_t)(M_HIST + kMChunk) * cap;
  unsigned nb = mgrid((int)b->Vs, cap);
  if (mrhs_max_blocks(b->Vs, cap) > nb) nb = mrhs_max_blocks(b->Vs, cap);
  ok = ok && QG_CUDA(cudaMalloc(&b->xs, (size_t)12 * b->Vs * cap * sizeof(float2))) &&
            QG_CUDA(cudaMalloc(&b->s, ns * sizeof(double))) && QG_CUDA(cudaMalloc(&b->mp4s, cap * sizeof(float))) &&
            QG_CUDA(cudaMalloc(&b->tms, cap * sizeof(float))) &&
            QG_CUDA(cudaMalloc(&b->part, (size_t)nb * cap * sizeof(double))) &&
            QG_CUDA(cudaMalloc(&b->l1, (size_t)kMSGroups * cap * sizeof(double) + 256)) &&
            QG_CUDA(cudaMalloc(&b->rudev, (size_t)4 * cap * sizeof(double))) &&
            QG_CUDA(cudaMallocHost(&b->ruhost, (size_t)4 * cap * sizeof(double))) &&
            QG_CUDA(cudaMallocHost(&b->hs, ns * sizeof(double))) &&
            QG_CUDA(cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming)) &&
            QG_CUDA(cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming)) &&
            QG_CUDA(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
  // the reduction's counter starts at zero, on the batch's own stream
  ok = ok && QG_CUDA(cudaMemsetAsync(b->l1, 0, (size_t)kMSGroups * cap * sizeof(double) + 256, b->st));
  if (ok) b->msdone = (unsigned *)(b->l1 + (size_t)kMSGroups * cap);
  if (!ok) {
    batch_free(b);
    return nullptr;
  }
  return b;
}

// bd = b as seen by D (Q x = b  <=>  D x = -i g5 b)
static bool slot_bd(qcdgpu_batch B, const BSlot &sl)
{
  if (sl.op == QCDGPU_OP_Q) return blas_ig5(B->bd, sl.b) && blas_axpby(B->bd, -1.0, 0.0, B->bd, 0.0, 0.0, B->bd);
  return blas_copy(B->bd, sl.b);
}

// rt = bd - D x (FP64), r = D^+ rt; slot k of rs <- r. |rt|^2 and |r|^2 are
// left on the device at res[0] and res[2]: the residuals of all updating
// slots are enqueued back to back and read with one synchronisation.
// Even/odd: rt = c_e - M x_e in FP64 (equal to the full residual), and the
// restart residual M^+ rt in FP32 (it only seeds the FP16 iteration).
static bool slot_residual(qcdgpu_batch B, int k, const BSlot &sl, double *res)
{
  if (B->eo) {
    qcdgpu_gauge g32 = gauge_at(B->g, QCDGPU_F32);
    const int ar = QCDGPU_ARITH_DF64;
    return g32 && dslash_eo(B->u64, sl.xe, nullptr, B->g, sl.mp4, sl.tm, false, 1, 1.0, true, 0, nullptr, ar) &&
           dslash_eo(B->rt, B->u64, sl.xe, B->g, sl.mp4, sl.tm, false, 0, -0.25, false, 2, nullptr, ar) &&
           blas_axpby(B->rt, 1.0, 0.0, sl.ce, -1.0, 0.0, B->rt) && blas_norm2_dev(B->rt, res) &&
           convert_field(B->r32, B->rt) &&
           dslash_eo(B->u32, B->r32, nullptr, g32, sl.mp4, sl.tm, true, 1, 1.0, true, 0, nullptr) &&
           dslash_eo(B->s32, B->u32, B->r32, g32, sl.mp4, sl.tm, true, 0, -0.25, false, 2, nullptr) &&
           blas_norm2_dev(B->s32, res + 2) && mfield_set(B->rs, k, B->s32);
  }
  return slot_bd(B, sl) && dslash(B->rt, sl.x, B->g, sl.mp4, sl.tm, QCDGPU_OP_D, QCDGPU_ARITH_DF64) &&
         blas_axpby(B->rt, 1.0, 0.0, B->bd, -1.0, 0.0, B->rt) && blas_norm2_dev(B->rt, res) &&
         dslash(B->r, B->rt, B->g, sl.mp4, sl.tm, QCDGPU_OP_DDAG, QCDGPU_ARITH_DF64) &&
         blas_norm2_dev(B->r, res + 2) && mfield_set(B->rs, k, B->r);
}

// rr and beta of up to 64 slots after their reliable updates, in one launch
struct SlotRestart {
  int n;
  int slot[64];
  double rr[64], beta[64];
};
__global__ void k_set_restart(double *s, int cap, SlotRestart r)
{
  const int i = threadIdx.x;
  if (i >= r.n) return;
  s[M_RR * cap + r.slot[i]] = r.rr[i];
  s[M_BETA * cap + r.slot[i]] = r.beta[i];
}

static bool set_scalar(qcdgpu_batch B, int slot_kind, int k, double v)
{
  B->hs[0] = v;
  return QG_CUDA(cudaMemcpyAsync(B->s + slot_kind * B->cap + k, B->hs, sizeof(double), cudaMemcpyHostToDevice,
                                 stream())) &&
         QG_CUDA(cudaStreamSynchronize(stream()));
}

static bool copy_slot(qcdgpu_batch B, int from, int to)
{
  unsigned g = (unsigned)((B->Vs + 127) / 128);
  for (auto m : {B->rs, B->ps}) {
    k_mcopy<<<g, 128, 0, stream()>>>(mv(m), from, to, 0);
    if (!QG_LAUNCHED("mrhs_copy_slot")) return false;
  }
  k_mx_copy<<<g, 128, 0, stream()>>>(mx(B), from, to, 0);
  if (!QG_LAUNCHED("mrhs_copy_slot")) return false;
  return QG_CUDA(cudaMemcpyAsync(B->mp4s + to, B->mp4s + from, sizeof(float), cudaMemcpyDeviceToDevice, stream())) &&
         QG_CUDA(cudaMemcpyAsync(B->tms + to, B->tms + from, sizeof(float), cudaMemcpyDeviceToDevice, stream()));
}

// an even/odd slot's half fields go back: x_e to the pool, the handles of
// c_e and A^{-1} b_o freed (with their memory when they are not views)
static void slot_release_eo(qcdgpu_batch B, BSlot &sl)
{
  if (sl.xe) B->spare.push_back(sl.xe);
  field_free(sl.ce);
  field_free(sl.to);
  sl.ce = sl.to = sl.xe = nullptr;
}

// x = (x_e, x_o), x_o = A^{-1} b_o + A^{-1} H_oe x_e / 2, written over the
// views of c_e and A^{-1} b_o in x (A^{-1} b_o is read into r first); then
// the slot's half fields go back
static bool slot_finish_eo(qcdgpu_batch B, BSlot &sl)
{
  const bool ok =
      dslash_eo(B->r, sl.xe, sl.to, B->g, sl.mp4, sl.tm, false, 1, 0.5, true, 1, nullptr, QCDGPU_ARITH_DF64) &&
      eo_merge(sl.x, sl.xe, B->r);
  slot_release_eo(B, sl);
  return ok;
}

int batch_add(qcdgpu_batch B, qcdgpu_field x, qcdgpu_field b, double kappa, double mu, int op, double tol,
              int maxiter, double delta, int tag)
{
  if (!x || !b || x->prec != QCDGPU_F64 || b->prec != QCDGPU_F64 || !same_shape(x, B->bd) ||
      !same_shape(b, B->bd) || x == b || !(kappa > 0.0) || (op != QCDGPU_OP_D && op != QCDGPU_OP_Q)) {
    set_error("batch add: FP64 x, b on the batch's lattice, kappa > 0, op D or Q");
    return -2;
  }
  for (const BSlot &o : B->slots)
    if (o.x == x || o.x == b || o.b == x) {
      set_error("batch add: x or b is a field of a right-hand side still in the batch");
      return -2;
    }
  if (B->nact >= B->cap) return -1;
  // the batch's stream starts after the caller's work on x and b
  if (!QG_CUDA(cudaEventRecord(B->ev_in, stream())) || !QG_CUDA(cudaStreamWaitEvent(B->st, B->ev_in, 0))) return -2;
  StreamScope scope(B->st);
  BSlot sl;
  sl.tag = tag;
  sl.x = x;
  sl.b = b;
  sl.op = op;
  sl.mp4 = 1.0 / (2.0 * kappa);
  sl.tm = mu;
  sl.tol = tol;
  sl.delta = delta > 0 ? delta : 0.1;
  sl.iters = 0;
  sl.updates = 0;
  sl.since = 0;
  sl.maxiter = maxiter > 0 ? maxiter : 100000;
  double bn2;
  if (!blas_norm2(b, &bn2) || !blas_zero(x)) return -2;
  sl.bn = sqrt(bn2);
  const int k = B->nact;
  sl.ce = sl.to = sl.xe = nullptr;
  if (B->eo) {
    // c_e = b_e + H_eo A^{-1} b_o / 2 with the slot's own half fields; c_e
    // and A^{-1} b_o in x's memory when it holds two half fields
    sl.xe = B->spare.back();
    B->spare.pop_back();
    const size_t hb = B->rt->bytes;
    if (x->bytes >= 2 * hb) {
      sl.ce = field_view(B->Ls, QCDGPU_F64, x->data);
      sl.to = field_view(B->Ls, QCDGPU_F64, (char *)x->data + hb);
    } else {
      sl.ce = field_new(B->Ls, QCDGPU_F64);
      sl.to = field_new(B->Ls, QCDGPU_F64);
    }
    const bool ok = sl.ce && sl.to && slot_bd(B, sl) && eo_split(B->rt, B->r, B->bd) &&
                    eo_diag(sl.to, B->r, sl.mp4, mu, true) &&
                    dslash_eo(sl.ce, sl.to, B->rt, B->g, sl.mp4, mu, false, 0, 0.5, false, 1, nullptr,
                              QCDGPU_ARITH_DF64) &&
                    blas_zero(sl.xe);
    if (!ok) {
      slot_release_eo(B, sl);
      return -2;
    }
  }
  auto give_back = [&]() {
    if (B->eo) slot_release_eo(B, sl);
  };
  if (!slot_residual(B, k, sl, B->rudev + 4 * k) ||
      !QG_CUDA(cudaMemcpyAsync(B->ruhost + 4 * k, B->rudev + 4 * k, sizeof(double) * 4, cudaMemcpyDeviceToHost,
                               stream())) ||
      !QG_CUDA(cudaStreamSynchronize(stream()))) {
    give_back();
    return -2;
  }
  const double rel = sl.bn > 0 ? sqrt(B->ruhost[4 * k]) / sl.bn : 0.0, rr = B->ruhost[4 * k + 2];
  sl.true_res = rel;
  sl.maxr = sqrt(rr);
  sl.hint = tol * sl.maxr;
  unsigned g = (unsigned)((B->Vs + 127) / 128);
  k_mx_copy<<<g, 128, 0, stream()>>>(mx(B), 0, k, 1);
  float mp = (float)sl.mp4, tmf = (float)mu;
  // p = r (slot_residual left r in B->s32 for even/odd batches, else in B->r);
  // a fresh slot starts with beta = 0, so the shared p update leaves p = r
  if (!QG_LAUNCHED("mrhs_zero_slot") || !mfield_set(B->ps, k, B->eo ? B->s32 : B->r) ||
      !QG_CUDA(cudaMemcpyAsync(B->mp4s + k, &mp, sizeof(float), cudaMemcpyHostToDevice, stream())) ||
      !QG_CUDA(cudaMemcpyAsync(B->tms + k, &tmf, sizeof(float), cudaMemcpyHostToDevice, stream())) ||
      !set_scalar(B, M_RR, k, rr) || !set_scalar(B, M_BETA, k, 0.0)) {
    give_back();
    return -2;
  }
  if (bn2 == 0.0 || rel <= tol) {
    // solved by x_e = 0: x = (0, A^{-1} b_o) for even/odd batches
    if (B->eo && !slot_finish_eo(B, sl)) return -2;
    B->done.push_back(BDone{tag, 0, 0, 0, rel});
    return k;
  }
  B->slots.push_back(sl);
  B->nact++;
  return k;
}

// retire slot k: the last occupied slot moves into it
static bool retire(qcdgpu_batch B, int k, int status)
{
  BSlot &sl = B->slots[(size_t)k];
  if (B->eo && !slot_finish_eo(B, sl)) return false;
  B->done.push_back(BDone{sl.tag, status, sl.iters, sl.updates, sl.true_res});
  const int last = B->nact - 1;
  if (k != last) {
    if (!copy_slot(B, last, k)) return false;
    // scalars of the moved slot
    if (!QG_CUDA(cudaMemcpyAsync(B->hs, B->s, sizeof(double) * (M_HIST + kMChunk) * B->cap, cudaMemcpyDeviceToHost,
                                 stream())) ||
        !QG_CUDA(cudaStreamSynchronize(stream())))
      return false;
    for (int q = 0; q < M_HIST + kMChunk; q++) B->hs[q * B->cap + k] = B->hs[q * B->cap + last];
    if (!QG_CUDA(cudaMemcpyAsync(B->s, B->hs, sizeof(double) * (M_HIST + kMChunk) * B->cap, cudaMemcpyHostToDevice,
                                 stream())))
      return false;
    B->slots[(size_t)k] = B->slots[(size_t)last];
  }
  B->slots.pop_back();
  B->nact--;
  return QG_CUDA(cudaStreamSynchronize(stream()));
}

// Enqueue one chunk (kMChunk iterations of every occupied slot) and the copy
// of the per-slot scalars to the host; the chunk is a CUDA graph per number
// of occupied slots, captured on first use.
static bool chunk_enqueue(qcdgpu_batch B, int n)
{
  const int cap = B->cap;
  const int V = (int)B->Vs;
  // the update writes per-slot partial sums: its block shape follows the
  // capacity, so their summation order does not depend on the mix; the
  // direction update uses threads for the n occupied slots only
  const dim3 blk = mblock(cap), blkp = mblock(n);
  const unsigned nb = mgrid(V, cap), nbp = mgrid(V, n);
  const size_t shm = sizeof(double) * blk.x * blk.y;
  cudaStream_t st = stream();
  for (int j = 0; j < kMChunk; j++) {
    // p = r + beta p (beta = 0 keeps a fresh slot's p = r)
    k_mp<<<nbp, blkp, 0, st>>>(mv(B->ps), mv(B->rs), n, B->s + M_BETA * cap);
    if (!QG_LAUNCHED("mrhs_p")) return false;
    // p^+ A^+ A p = |A p|^2, summed per slot in the epilogue of t = A p
    // (A = D, or the Schur complement M = A_ee - H_eo A_oo^{-1} H_oe / 4 as
    // u = A^{-1} H_oe p, t = A p - H_eo u / 4)
    unsigned nbo = 0;
    if (B->eo) {
      if (!dslash_mrhs_eo(B->u, B->ps, nullptr, B->g, false, n, B->mp4s, B->tms, 1, 1.0, true, 0, nullptr, nullptr) ||
          !dslash_mrhs_eo(B->t, B->u, B->ps, B->g, false, n, B->mp4s, B->tms, 0, -0.25, false, 2, B->part, &nbo))
        return false;
    } else if (!dslash_mrhs(B->t, B->ps, B->g, 4.0, 0.0, false, n, B->mp4s, B->tms, B->part, &nbo)) {
      return false;
    }
    k_mscalars2<<<kMSGroups, 256, 0, st>>>(B->part, (int)nbo, cap, n, B->s, 0, j, B->l1, B->msdone);
    if (!QG_LAUNCHED("mrhs_scalars")) return false;
    if (B->eo) {
      if (!dslash_mrhs_eo(B->u, B->t, nullptr, B->g, true, n, B->mp4s, B->tms, 1, 1.0, true, 0, nullptr, nullptr) ||
          !dslash_mrhs_eo(B->aps, B->u, B->t, B->g, true, n, B->mp4s, B->tms, 0, -0.25, false, 2, nullptr, nullptr))
        return false;
    } else if (!dslash_mrhs(B->aps, B->t, B->g, 4.0, 0.0, true, n, B->mp4s, B->tms)) {
      return false;
    }
    k_mupdate<<<nb, blk, shm, st>>>(mx(B), mv(B->ps), mv(B->rs), mv(B->aps), n, B->s + M_ALPHA * cap, B->part);
    if (!QG_LAUNCHED("mrhs_update")) return false;
    k_mscalars2<<<kMSGroups, 256, 0, st>>>(B->part, (int)nb, cap, n, B->s, 1, j, B->l1, B->msdone);
    if (!QG_LAUNCHED("mrhs_scalars")) return false;
  }
  return QG_CUDA(cudaMemcpyAsync(B->hs, B->s, sizeof(double) * (M_HIST + kMChunk) * cap, cudaMemcpyDeviceToHost, st));
}

bool batch_launch(qcdgpu_batch B)
{
  B->nchunk = B->nact;
  if (B->nchunk == 0) return true;
  StreamScope scope(B->st);
  const int n = B->nchunk;
  if (!gauge_at(B->g, kGaugeF32Full)) return false;  // resident before any capture
  if (!B->tuned) {
    // the operator's tuner times its variants outside stream capture; t and
    // u are scratch (recomputed by every iteration)
    const bool ok = B->eo ? dslash_mrhs_eo(B->u, B->ps, nullptr, B->g, false, n, B->mp4s, B->tms, 1, 1.0, true, 0,
                                           nullptr, nullptr) &&
                                dslash_mrhs_eo(B->t, B->u, B->ps, B->g, false, n, B->mp4s, B->tms, 0, -0.25, false, 2,
                                               nullptr, nullptr)
                          : dslash_mrhs(B->t, B->ps, B->g, 4.0, 0.0, false, n, B->mp4s, B->tms);
    if (!ok) return false;
    B->tuned = true;
  }
  if (B->use_graphs) {
    cudaGraphExec_t &ex = B->graphs[(size_t)n];
    if (!ex) {
      cudaGraph_t graph = nullptr;
      if (!QG_CUDA(cudaStreamBeginCapture(B->st, cudaStreamCaptureModeThreadLocal))) return false;
      const uint64_t counted = g_launches.load();
      bool ok = chunk_enqueue(B, n);
      cudaError_t e = cudaStreamEndCapture(B->st, &graph);
      B->graph_launches[(size_t)n] = g_launches.load() - counted;
      g_launches.store(counted);  // captured, not launched: counted at each graph launch
      if (!ok || !QG_CUDA(e)) {
        if (graph) cudaGraphDestroy(graph);
        return false;
      }
      ok = QG_CUDA(cudaGraphInstantiate(&ex, graph, 0));
      cudaGraphDestroy(graph);
      if (!ok) {
        ex = nullptr;
        return false;
      }
    }
    if (!QG_CUDA(cudaGraphLaunch(ex, B->st))) return false;
    count_launches(B->graph_launches[(size_t)n]);
  } else if (!chunk_enqueue(B, n)) {
    return false;
  }
  return QG_CUDA(cudaEventRecord(B->ev, B->st));
}

bool batch_in_flight(qcdgpu_batch B) { return B->nchunk > 0; }

bool batch_chunk_done(qcdgpu_batch B)
{
  if (B->nchunk == 0) return true;
  const cudaError_t e = cudaEventQuery(B->ev);
  if (e == cudaErrorNotReady) {
    if (cudaPeekAtLastError() == cudaErrorNotReady) cudaGetLastError();  // not an error
    return false;
  }
  return true;  // done, or an error that batch_finish reports
}

// Wait for the launched chunk, then reliable updates and retirement
bool batch_finish(qcdgpu_batch B)
{
  const int n = B->nchunk;
  B->nchunk = 0;
  if (n == 0) return true;
  StreamScope scope(B->st);
  const int cap = B->cap;
  const int V = (int)B->Vs;
  cudaStream_t st = B->st;
  if (!QG_CUDA(cudaEventSynchronize(B->ev))) return false;
  if (mrhs_tc_failed()) {
    set_error("batch: the tensor-core multi-RHS kernel abandoned an apply after a bounded wait for the tensor "
              "cores ran out; the chunk's results are invalid");
    return false;
  }
  std::vector<double> rr_iter(n), beta_iter(n);
  std::vector<int> need(n, 0), fail(n, 0);
  for (int k = 0; k < n; k++) {
    BSlot &sl = B->slots[(size_t)k];
    rr_iter[k] = B->hs[M_RR * cap + k];
    beta_iter[k] = B->hs[M_BETA * cap + k];
    bool update = false, hinted = false;
    for (int j = 0; j < kMChunk; j++) {
      double rn = sqrt(B->hs[(M_HIST + j) * cap + k]);
      if (!(rn == rn)) {
        fail[k] = 1;
        break;
      }
      sl.iters++;
      if (rn <= sl.hint) hinted = true;
      if (rn < sl.delta * sl.maxr) update = true;
      if (!update && rn > sl.maxr) sl.maxr = rn;
    }
    need[k] = fail[k] || update || hinted || sl.iters >= sl.maxiter;
    if (hinted) sl.hint *= 0.3;
  }
  // reliable updates: every updating slot's FP64 residual and restart are
  // enqueued back to back, their norms read with one synchronisation, and
  // the continuing slots' rr and beta written with one launch; then
  // retirement from the highest slot down
  std::vector<int> retire_status(n, -1), upd;
  for (int k = 0; k < n; k++) {
    if (!need[k]) continue;
    BSlot &sl = B->slots[(size_t)k];
    qcdgpu_field acc = B->eo ? sl.xe : sl.x;  // the slot's FP64 solution
    k_mx_flush<<<(unsigned)((V + 127) / 128), 128, 0, st>>>((double2 *)acc->data, acc->stride, mx(B), k);
    if (!QG_LAUNCHED("mrhs_flush_slot")) return false;
    if (!slot_residual(B, k, sl, B->rudev + 4 * k)) return false;
    upd.push_back(k);
  }
  if (!upd.empty()) {
    if (!QG_CUDA(cudaMemcpyAsync(B->ruhost, B->rudev, sizeof(double) * 4 * (size_t)n, cudaMemcpyDeviceToHost, st)) ||
        !QG_CUDA(cudaStreamSynchronize(st)))
      return false;
    SlotRestart rs;
    rs.n = 0;
    for (int k : upd) {
      BSlot &sl = B->slots[(size_t)k];
      const double n2 = B->ruhost[4 * k], rr = B->ruhost[4 * k + 2];
      const double rel = sl.bn > 0 ? sqrt(n2) / sl.bn : 0.0;
      sl.true_res = rel;
      sl.updates++;
      if (rel <= sl.tol) {
        retire_status[k] = 0;
      } else if (fail[k]) {
        retire_status[k] = 2;
      } else if (sl.iters >= sl.maxiter) {
        retire_status[k] = 1;
      } else {
        rs.slot[rs.n] = k;
        rs.rr[rs.n] = rr;
        rs.beta[rs.n] = (beta_iter[k] > 0.0 && rr_iter[k] > 0.0) ? rr * beta_iter[k] / rr_iter[k] : 0.0;
        rs.n++;
        sl.maxr = sqrt(rr);
      }
    }
    if (rs.n > 0) {
      k_set_restart<<<1, 64, 0, st>>>(B->s, cap, rs);
      if (!QG_LAUNCHED("mrhs_set_restart")) return false;
    }
  }
  for (int k = n - 1; k >= 0; k--)
    if (retire_status[k] >= 0 && !retire(B, k, retire_status[k])) return false;
  return true;
}

// run up to `iters` iterations (whole chunks) with reliable updates and
// retirement at chunk boundaries; returns 0, or 3 on error
int batch_step(qcdgpu_batch B, int iters)
{
  for (int done_it = 0; done_it < iters && B->nact > 0; done_it += kMChunk)
    if (!batch_launch(B) || !batch_finish(B)) return 3;
  return 0;
}

}  // namespace qg

extern "C" {

int qcdgpu_batch_create(qcdgpu_batch *b, qcdgpu_gauge g, int capacity)
{
  *b = qg::batch_new(g, capacity, false);
  return *b ? 0 : 1;
}
int qcdgpu_batch_create_eo(qcdgpu_batch *b, qcdgpu_gauge g, int capacity)
{
  *b = qg::batch_new(g, capacity, true);
  return *b ? 0 : 1;
}
int qcdgpu_batch_destroy(qcdgpu_batch b)
{
  qg::batch_free(b);
  return 0;
}
int qcdgpu_batch_add(qcdgpu_batch b, qcdgpu_field x, qcdgpu_field rhs, double kappa, double mu, int op, double tol,
                     int maxiter, double delta, int tag)
{
  return qg::batch_add(b, x, rhs, kappa, mu, op, tol, maxiter, delta, tag);
}
int qcdgpu_batch_step(qcdgpu_batch b, int iterations) { return qg::batch_step(b, iterations); }
int qcdgpu_batch_active(qcdgpu_batch b) { return b ? b->nact : 0; }
int qcdgpu_batch_free_slots(qcdgpu_batch b) { return b ? b->cap - b->nact : 0; }
int qcdgpu_batch_poll(qcdgpu_batch b, int *tags, int *status, int *iters, double *true_residual, int max)
{
  int n = 0;
  while (n < max && !b->done.empty()) {
    qg::BDone d = b->done.front();
    b->done.erase(b->done.begin());
    tags[n] = d.tag;
    status[n] = d.status;
    iters[n] = d.iters;
    true_residual[n] = d.true_res;
    n++;
  }
  return n;
}
size_t qcdgpu_batch_bytes(qcdgpu_batch b)
{
  if (!b) return 0;
  size_t n = 4 * b->rs->bytes + (size_t)12 * b->Vs * b->cap * sizeof(float2) + 3 * b->rt->bytes + b->bd->bytes;
  if (b->eo) n += b->u->bytes + b->u64->bytes + 3 * b->r32->bytes + (size_t)b->cap * b->rt->bytes;
  for (const auto &sl : b->slots)  // c_e, A^{-1} b_o outside x (x too small for both)
    for (auto f : {sl.ce, sl.to})
      if (f && !f->view) n += f->bytes;
  return n;
}

}  // extern "C"
