// peaks.cu -- arithmetic-pipe throughput of this GPU, measured for the
// benchmark's compute ceilings (FP64 FMA for the native FP64 operator, FP32
// FMA for the float-float operator). Each thread runs 8 independent FMA
// chains; the result is written so the chains are not removed.
#include "internal.h"

namespace qg {

template <typename T>
__global__ void __launch_bounds__(256) k_fma_rate(T *out, int iters, T x, T y)
{
  T a[8];
#pragma unroll
  for (int k = 0; k < 8; k++) a[k] = (T)(threadIdx.x + k);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = fma(a[k], x, y);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace qg

extern "C" {

/* FMA throughput of this GPU in TFLOP/s (2 flops per FMA): kind 0 FP64,
 * kind 1 FP32. Times a kernel of independent FMA chains on every SM with
 * CUDA events (best of three launches). Returns 0, or 1 on error. */
int qcdgpu_measure_fma_rate(int kind, double *tflops)
{
  int dev = 0, sms = 0;
  if (!QG_CUDA(cudaGetDevice(&dev)) || !QG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)))
    return 1;
  const int blocks = sms * 8, threads = 256, iters = kind == 0 ? 2048 : 16384;
  void *out = nullptr;
  if (!QG_CUDA(cudaMalloc(&out, sizeof(double) * blocks * threads))) return 1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaStream_t s = qg::stream();
  float best = 1e30f;
  bool ok = true;
  for (int rep = 0; rep < 4 && ok; rep++) {
    cudaEventRecord(e0, s);
    if (kind == 0) qg::k_fma_rate<double><<<blocks, threads, 0, s>>>((double *)out, iters, 0.999999, 1e-7);
    else qg::k_fma_rate<float><<<blocks, threads, 0, s>>>((float *)out, iters, 0.999999f, 1e-7f);
    cudaEventRecord(e1, s);
    ok = QG_LAUNCHED("fma_rate") && QG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;  // the first launch warms up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (!ok) return 1;
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
  return 0;
}

}  // extern "C"
