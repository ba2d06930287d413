// noalloc.cu -- the complex dot product <a,b> = sum_i conj(a_i) b_i over the
// caller's device arrays, with no device memory allocated at any point.
//
// Who needs this: code that cannot call cudaMalloc -- a process whose device
// heap is owned by someone else (a framework's caching allocator, or a
// serving engine that reserved its whole memory budget up front), a
// latency-critical loop that cannot afford the device-wide synchronisation
// cudaMalloc may imply, or a path that must not fail on allocation. The
// regular reductions take their per-block partial sums from a buffer the
// library allocates on first use; this variant keeps them in a file-scope
// __device__ array instead:
//
//   * the array holds 2 x 2048 doubles (32 KB) and lives on every GPU that
//     loads the library until the process exits;
//   * each block sums one chunk of 65,536 complex elements, so an input may
//     hold at most 2048 x 65,536 = 134,217,728 complex elements; larger inputs
//     are rejected with an error (return 1);
//   * every call shares the array and leaves its partial sums behind: each
//     call writes every partial it reads before reading it, so nothing has to
//     start at zero -- but calls that overlap on the GPU (different streams,
//     or different host threads on one device) race on the array;
//   * host code cannot use the array's name as a device address, so the
//     first call on each device resolves it with cudaGetSymbolAddress while
//     that device is current and caches the result. That first call is the
//     set-up: make it before any stream capture begins.
#include <stdint.h>

#include <mutex>

#include "internal.h"

namespace qg {

constexpr int kNaBlocks = 2048;
constexpr int64_t kNaChunk = 65536;
constexpr int64_t kNaMaxN = (int64_t)kNaBlocks * kNaChunk;
constexpr int kNaMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[2 * kNaBlocks];

static std::mutex g_na_mu;
static double *g_na_addr[kNaMaxDevices];

// device address of g_noalloc_partials on the current device
static double *noalloc_partials()
{
  int dev = -1;
  if (!QG_CUDA(cudaGetDevice(&dev))) return nullptr;
  if (dev < 0 || dev >= kNaMaxDevices) {
    set_error("dot_noalloc: device ordinal %d out of range", dev);
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (!g_na_addr[dev]) {
    void *p = nullptr;
    if (!QG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_partials))) return nullptr;
    g_na_addr[dev] = (double *)p;
  }
  return g_na_addr[dev];
}

__device__ __forceinline__ double na_warp_sum(double v)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block i: partials[2i..2i+1] = sum over chunk i of conj(a) b
__global__ void __launch_bounds__(256) k_dot_chunks(const double2 *a, const double2 *b, int64_t n,
                                                    double *partials)
{
  int64_t begin = (int64_t)blockIdx.x * kNaChunk;
  int64_t end = begin + kNaChunk < n ? begin + kNaChunk : n;
  double re = 0.0, im = 0.0;
  for (int64_t i = begin + threadIdx.x; i < end; i += blockDim.x) {
    double2 x = a[i], y = b[i];
    re += x.x * y.x + x.y * y.y;
    im += x.x * y.y - x.y * y.x;
  }
  __shared__ double sh[2][8];
  re = na_warp_sum(re);
  im = na_warp_sum(im);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = re;
    sh[1][w] = im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sr = 0.0, si = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
      sr += sh[0][k];
      si += sh[1][k];
    }
    partials[2 * blockIdx.x] = sr;
    partials[2 * blockIdx.x + 1] = si;
  }
}

// one block sums the nb partial pairs in a fixed order into result[0..1]
__global__ void k_dot_final(const double *partials, int nb, double *result)
{
  double re = 0.0, im = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    re += partials[2 * i];
    im += partials[2 * i + 1];
  }
  __shared__ double sh[2][8];
  re = na_warp_sum(re);
  im = na_warp_sum(im);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = re;
    sh[1][w] = im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sr = 0.0, si = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
      sr += sh[0][k];
      si += sh[1][k];
    }
    result[0] = sr;
    result[1] = si;
  }
}

}  // namespace qg

extern "C" int qcdgpu_dot_noalloc(const double *a, const double *b, int64_t n, double *result, void *stream)
{
  using namespace qg;
  if (n < 0 || n > kNaMaxN) {
    set_error("dot_noalloc: %lld complex elements requested, the maximum is %lld (2048 chunks of 65536)",
              (long long)n, (long long)kNaMaxN);
    return 1;
  }
  if (!result || (n > 0 && (!a || !b))) {
    set_error("dot_noalloc: null pointer");
    return 1;
  }
  if (((uintptr_t)a | (uintptr_t)b) % 16 != 0 || (uintptr_t)result % 8 != 0) {
    set_error("dot_noalloc: a and b must be 16-byte aligned, result 8-byte aligned");
    return 1;
  }
  double *partials = noalloc_partials();
  if (!partials) return 1;
  cudaStream_t s = (cudaStream_t)stream;
  int nb = (int)((n + kNaChunk - 1) / kNaChunk);
  if (nb > 0) {
    k_dot_chunks<<<nb, 256, 0, s>>>((const double2 *)a, (const double2 *)b, n, partials);
    if (!QG_LAUNCHED("dot_noalloc_chunks")) return 1;
  }
  k_dot_final<<<1, 256, 0, s>>>(partials, nb, result);
  return QG_LAUNCHED("dot_noalloc_final") ? 0 : 1;
}
