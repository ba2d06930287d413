// runtime.cu -- error reporting, stream selection, device field allocation,
// the pooled work fields solvers draw from, and reduction scratch.
#include <stdarg.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "internal.h"
#include "mrhs.h"

namespace qg {

std::atomic<uint64_t> g_launches{0};
static thread_local std::string t_last_error;
static cudaStream_t g_stream = nullptr;

void set_error(const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_last_error = buf;
  fprintf(stderr, "qcdgpu: %s\n", buf);
}

// fault injection (tests): the next g_alloc_faults allocations of fields,
// gauge fields and host vectors fail as if memory were exhausted
static std::atomic<int> g_alloc_faults{0};

bool alloc_fault()
{
  int n = g_alloc_faults.load();
  while (n > 0)
    if (g_alloc_faults.compare_exchange_weak(n, n - 1)) return true;
  return false;
}

bool cuda_ok(cudaError_t e, const char *what)
{
  if (e == cudaSuccess) return true;
  set_error("CUDA error %s in %s", cudaGetErrorString(e), what);
  return false;
}

bool after_launch(const char *what)
{
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return cuda_ok(cudaGetLastError(), what);
}

cudaStream_t stream() { return g_stream; }
cudaStream_t swap_stream(cudaStream_t s)
{
  cudaStream_t p = g_stream;
  g_stream = s;
  return p;
}

static size_t spinor_bytes(int prec, int64_t stride)
{
  switch (prec) {
  case QCDGPU_F64: return (size_t)stride * 24 * 8;
  case QCDGPU_F32: return (size_t)stride * 24 * 4;
  default: return (size_t)stride * 24 * 2 + (size_t)stride * 4;
  }
}

qcdgpu_field field_new(const int L[4], int prec)
{
  for (int i = 0; i < 4; i++)
    if (L[i] < 2) {
      set_error("lattice extents must be >= 2 (got %d)", L[i]);
      return nullptr;
    }
  if (prec < QCDGPU_F64 || prec > QCDGPU_F16) {
    set_error("unknown precision %d", prec);
    return nullptr;
  }
  auto *f = new qcdgpu_field_s();
  memcpy(f->L, L, sizeof(f->L));
  f->V = (int64_t)L[0] * L[1] * L[2] * L[3];
  if (f->V >= (1ll << 31) - 128) {
    set_error("lattice of %lld sites: kernels index sites with 32-bit integers", (long long)f->V);
    delete f;
    return nullptr;
  }
  f->stride = pad_stride(f->V);
  f->prec = prec;
  f->bytes = spinor_bytes(prec, f->stride);
  if (alloc_fault()) {
    set_error("out of device memory (injected) for a %zu-byte field", f->bytes);
    delete f;
    return nullptr;
  }
  if (!QG_CUDA(cudaMalloc(&f->data, f->bytes))) {
    delete f;
    return nullptr;
  }
  f->norm = prec == QCDGPU_F16 ? (float *)((char *)f->data + (size_t)f->stride * 48) : nullptr;
  if (!QG_CUDA(cudaMemsetAsync(f->data, 0, f->bytes, g_stream))) {
    cudaFree(f->data);
    delete f;
    return nullptr;
  }
  return f;
}

qcdgpu_field field_view(const int L[4], int prec, void *data)
{
  if (prec != QCDGPU_F64 && prec != QCDGPU_F32) {
    set_error("field view: F64 or F32 only");
    return nullptr;
  }
  auto *f = new qcdgpu_field_s();
  memcpy(f->L, L, sizeof(f->L));
  f->V = (int64_t)L[0] * L[1] * L[2] * L[3];
  f->stride = pad_stride(f->V);
  f->prec = prec;
  f->bytes = spinor_bytes(prec, f->stride);
  f->data = data;
  f->view = true;
  return f;
}

void field_free(qcdgpu_field f)
{
  if (!f) return;
  if (!f->view) cudaFree(f->data);
  delete f;
}

qcdgpu_gauge gauge_new(const int L[4], const double theta[4], int prec, int recon)
{
  for (int i = 0; i < 4; i++)
    if (L[i] < 2) {
      set_error("lattice extents must be >= 2 (got %d)", L[i]);
      return nullptr;
    }
  auto *g = new qcdgpu_gauge_s();
  memcpy(g->L, L, sizeof(g->L));
  for (int i = 0; i < 4; i++) g->theta[i] = theta ? theta[i] : 0.0;
  g->V = (int64_t)L[0] * L[1] * L[2] * L[3];
  if (g->V >= (1ll << 31) - 128) {
    set_error("lattice of %lld sites: kernels index sites with 32-bit integers", (long long)g->V);
    delete g;
    return nullptr;
  }
  g->stride = pad_stride(g->V);
  g->prec = prec;
  g->recon = recon;
  size_t reals = (size_t)4 * recon;
  size_t esz = (prec == QCDGPU_F64 || prec == kGaugeFF) ? 8 : prec == QCDGPU_F32 ? 4 : 2;
  g->bytes = reals * esz * (size_t)g->stride;
  if (alloc_fault()) {
    set_error("out of device memory (injected) for a %zu-byte gauge field", g->bytes);
    delete g;
    return nullptr;
  }
  if (!QG_CUDA(cudaMalloc(&g->data, g->bytes))) {
    delete g;
    return nullptr;
  }
  if (!QG_CUDA(cudaMemsetAsync(g->data, 0, g->bytes, g_stream))) {
    cudaFree(g->data);
    delete g;
    return nullptr;
  }
  return g;
}

void gauge_free(qcdgpu_gauge g)
{
  if (!g) return;
  cudaFree(g->data);
  delete g;
}

bool same_shape(qcdgpu_field a, qcdgpu_field b)
{
  return a && b && a->V == b->V && a->L[0] == b->L[0] && a->L[1] == b->L[1] &&
         a->L[2] == b->L[2] && a->L[3] == b->L[3];
}

// ------------------------------------------------------------ work pool
static std::mutex g_pool_mu;
static std::vector<qcdgpu_field> g_pool;

qcdgpu_field work_get(const int L[4], int prec)
{
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    for (size_t i = 0; i < g_pool.size(); i++) {
      qcdgpu_field f = g_pool[i];
      if (f->prec == prec && f->L[0] == L[0] && f->L[1] == L[1] && f->L[2] == L[2] &&
          f->L[3] == L[3]) {
        g_pool.erase(g_pool.begin() + (long)i);
        return f;
      }
    }
  }
  qcdgpu_field f = field_new(L, prec);
  if (!f) {  // out of device memory: give back the pooled fields and retry once
    work_trim();
    f = field_new(L, prec);
  }
  return f;
}

void work_put(qcdgpu_field f)
{
  if (!f) return;
  std::lock_guard<std::mutex> lk(g_pool_mu);
  g_pool.push_back(f);
}

void work_trim()
{
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if (!g_pool.empty()) cudaStreamSynchronize(g_stream);
  for (qcdgpu_field f : g_pool) field_free(f);
  g_pool.clear();
}

// ------------------------------------------------------- reduction scratch
static double *g_scratch = nullptr;
static double *g_host_res = nullptr;

double *reduce_scratch()
{
  if (!g_scratch) {
    if (!QG_CUDA(cudaMalloc(&g_scratch, sizeof(double) * (2 * kMaxPartials + 64)))) return nullptr;
  }
  return g_scratch;
}

// per-block partial sums of launches with one block per 128 sites; grows
// (outside any timed loop: solvers call it before iterating)
static double *g_big = nullptr;
static int64_t g_big_n = 0;

double *big_partials(int64_t n)
{
  if (n > g_big_n) {
    if (g_big) {
      cudaStreamSynchronize(g_stream);
      cudaFree(g_big);
    }
    g_big = nullptr;
    g_big_n = 0;
    if (!QG_CUDA(cudaMalloc(&g_big, sizeof(double) * (size_t)n))) return nullptr;
    g_big_n = n;
  }
  return g_big;
}

double *host_result()
{
  if (!g_host_res) {
    if (!QG_CUDA(cudaMallocHost(&g_host_res, sizeof(double) * 64))) return nullptr;
  }
  return g_host_res;
}

}  // namespace qg

// ------------------------------------------------------------ C entry points
extern "C" {

const char *qcdgpu_last_error(void) { return qg::t_last_error.c_str(); }

int qcdgpu_set_stream(void *s)
{
  qg::g_stream = (cudaStream_t)s;
  return 0;
}

int qcdgpu_sync(void)
{
  if (!QG_CUDA(cudaStreamSynchronize(qg::g_stream))) return 1;
  if (qg::mrhs_tc_failed()) {
    qg::set_error("the tensor-core multi-RHS kernel abandoned an apply after a bounded wait ran out");
    return 1;
  }
  return 0;
}

int qcdgpu_inject_alloc_failures(int n)
{
  qg::g_alloc_faults.store(n > 0 ? n : 0);
  return 0;
}

int64_t qcdgpu_scratch_bytes(void)
{
  return (qg::g_scratch ? (int64_t)sizeof(double) * (2 * qg::kMaxPartials + 64) : 0) +
         (int64_t)sizeof(double) * qg::g_big_n;
}

int qcdgpu_release_work(void)
{
  qg::work_trim();
  return 0;
}

uint64_t qcdgpu_kernel_launches(void) { return qg::g_launches.load(); }

int qcdgpu_field_create(qcdgpu_field *f, const int L[4], int prec)
{
  *f = qg::field_new(L, prec);
  return *f ? 0 : 1;
}

int qcdgpu_field_destroy(qcdgpu_field f)
{
  qg::field_free(f);
  return 0;
}

size_t qcdgpu_field_bytes(qcdgpu_field f) { return f ? f->bytes : 0; }
size_t qcdgpu_gauge_bytes(qcdgpu_gauge g) { return g ? g->bytes : 0; }
void *qcdgpu_field_data(qcdgpu_field f) { return f ? f->data : nullptr; }

int qcdgpu_gauge_create(qcdgpu_gauge *g, const int L[4], const double theta[4], int prec)
{
  // storage is sized for 18 reals per link until the first load decides
  *g = qg::gauge_new(L, theta, prec, 18);
  return *g ? 0 : 1;
}

int qcdgpu_gauge_destroy(qcdgpu_gauge g)
{
  qg::gauge_forget(g);
  qg::gauge_free(g);
  return 0;
}

int qcdgpu_gauge_recon(qcdgpu_gauge g) { return g ? g->recon : 0; }

}  // extern "C"
