// api.cu -- qcd_lib entry points on the caller's host structs.
//
// Every qcd_vector / qcd_gaugeField seen by an entry point gets a device
// mirror, found by its data pointer D. Unless the object was made device
// resident, an entry point uploads each input it reads and writes each
// output back to host memory before returning, so the caller observes the
// reference's synchronous semantics. qcd_initVector / qcd_initGaugeField
// allocate page-locked host memory so these copies run at full link speed.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "internal.h"

namespace qg {

qcdgpu_gauge gauge_at(qcdgpu_gauge g, int prec);
void gauge_forget(qcdgpu_gauge g);

struct VecMirror {
  qcdgpu_field f = nullptr;
  bool resident = false;
};
struct GaugeMirror {
  qcdgpu_gauge g = nullptr;
  bool resident = false;
};

static std::mutex g_mu;
static std::unordered_map<const void *, VecMirror> g_vec;
static std::unordered_map<const void *, GaugeMirror> g_gauge;
static std::unordered_set<const void *> g_pinned;  // host blocks from cudaMallocHost

static void *host_alloc(size_t bytes)
{
  if (alloc_fault()) return nullptr;
  void *p = nullptr;
  if (cudaMallocHost(&p, bytes) == cudaSuccess) {
    g_pinned.insert(p);
    return p;
  }
  cudaGetLastError();  // no usable GPU here: plain host memory still works
  return malloc(bytes);
}

static void host_free(void *p)
{
  if (!p) return;
  auto it = g_pinned.find(p);
  if (it != g_pinned.end()) {
    g_pinned.erase(it);
    cudaFreeHost(p);
  } else {
    free(p);
  }
}

static void geo_L(const qcd_geometry *geo, int L[4])
{
  for (int i = 0; i < 4; i++) L[i] = geo->L[i];
}

static bool same_L(const int a[4], const int b[4])
{
  return a[0] == b[0] && a[1] == b[1] && a[2] == b[2] && a[3] == b[3];
}

static VecMirror *vec_mirror(qcd_vector *v)
{
  if (!v || !v->initialized || !v->D || !v->geo || v->geo->initialized != 1) {
    set_error("vector not properly initialized");
    return nullptr;
  }
  int L[4];
  geo_L(v->geo, L);
  VecMirror &m = g_vec[(const void *)v->D];
  if (m.f && !same_L(m.f->L, L)) {
    field_free(m.f);
    m.f = nullptr;
    m.resident = false;
  }
  if (!m.f) m.f = field_new(L, QCDGPU_F64);
  return m.f ? &m : nullptr;
}

// device field holding v's current value
static qcdgpu_field vec_in(qcd_vector *v)
{
  VecMirror *m = vec_mirror(v);
  if (!m) return nullptr;
  if (!m->resident && !upload_spinor_aos(m->f, (const double *)v->D)) return nullptr;
  return m->f;
}

// device field that will receive v's new value
static qcdgpu_field vec_out(qcd_vector *v)
{
  VecMirror *m = vec_mirror(v);
  return m ? m->f : nullptr;
}

// publish the device result to the host unless v is resident
static bool vec_done(qcd_vector *v)
{
  auto it = g_vec.find((const void *)v->D);
  if (it == g_vec.end() || !it->second.f) return false;
  // uploads from page-locked memory are asynchronous: finish them before the
  // caller may touch its host buffers again
  if (it->second.resident) return QG_CUDA(cudaStreamSynchronize(stream()));
  return download_spinor_aos(it->second.f, (double *)v->D);
}

static qcdgpu_gauge gauge_in(qcd_gaugeField *u)
{
  if (!u || !u->initialized || !u->D || !u->geo || u->geo->initialized != 1) {
    set_error("gauge field not properly initialized");
    return nullptr;
  }
  int L[4];
  geo_L(u->geo, L);
  GaugeMirror &m = g_gauge[(const void *)u->D];
  if (m.g && (!same_L(m.g->L, L) || memcmp(m.g->theta, u->geo->theta, sizeof(m.g->theta)) != 0)) {
    gauge_forget(m.g);
    gauge_free(m.g);
    m.g = nullptr;
    m.resident = false;
  }
  if (m.resident && m.g) return m.g;
  if (!m.g) m.g = gauge_new(L, u->geo->theta, QCDGPU_F64, 18);
  if (!m.g) return nullptr;
  gauge_forget(m.g);  // host data may have changed: drop derived copies
  if (!upload_gauge_aos(m.g, (const double *)u->D)) return nullptr;
  return m.g;
}

// the reference's argument checks (qcd_wilson.c:139-166)
static bool check_op_args(qcd_vector *Dv, qcd_vector *v, qcd_gaugeField *u)
{
  if (!v || !v->initialized) {
    set_error("Error in qcd_ApplyWilsonTMOp! Vector must be properly initialized");
    return false;
  }
  if (!u || !u->initialized) {
    set_error("Error in qcd_ApplyWilsonTMOp! Gauge field must be properly initialized");
    return false;
  }
  const qcd_geometry *a = v->geo, *b = u->geo;
  if (!a || !b || a->initialized != 1 || b->initialized != 1 || memcmp(a->L, b->L, sizeof(a->L)) != 0 ||
      memcmp(a->lL, b->lL, sizeof(a->lL)) != 0 || memcmp(a->Pos, b->Pos, sizeof(a->Pos)) != 0) {
    set_error("Error in qcd_ApplyWilsonTMOp! Geometry not initialized or missmatched");
    return false;
  }
  if (!Dv || !Dv->initialized || !Dv->D) {
    set_error("Error in qcd_ApplyWilsonTMOp! Output vector must be properly initialized");
    return false;
  }
  if (Dv->D == v->D) {
    set_error("Error in qcd_ApplyWilsonTMOp! Output and input vectors must differ");
    return false;
  }
  return true;
}

// Pipelined apply for page-locked host vectors: the lattice is cut into S
// slabs of whole z-planes (up to 24). Each stage runs on its own stream,
// chained per slab by events, so the copy engines stream their slabs back
// to back: c_in copies slab k in, the operator runs as soon as slabs
// k-1..k+1 are in (consecutive slabs rotating over three streams, so thin
// slabs share the GPU) and c_out copies the result out. With float-float
// arithmetic the operator reads and writes the host layout in the staging
// buffers directly; with native FP64 s_in reorders each slab to the field
// layout first and s_out reorders the result back. Slabs 0 and S-1 need
// each other (periodic z), so the order of application is 1 .. S-2, S-1, 0.
// The host link bounds it: 254 MB per 24^3x48 apply at the 340 GB/s both
// directions reach together is 0.75 ms.
static cudaStream_t g_c_in, g_s_in, g_s_out, g_c_out, g_s_op2, g_s_op3;
static std::vector<cudaEvent_t> g_ev_cin, g_ev_in, g_ev_op, g_ev_rout;
static cudaEvent_t g_ev_start, g_ev_done, g_ev_op2, g_ev_op3;
static void *g_stage_in, *g_stage_out;  // device copies of the host layout
static size_t g_stage_bytes;

static int g_pipe_slabs = 0;  // 0: the largest of 24, 16, 12, 8, 6, 4, 3 dividing L_z

static int pipeline_slabs(const qcdgpu_field f)
{
  if (g_pipe_slabs > 0) return f->L[3] % g_pipe_slabs == 0 && g_pipe_slabs >= 3 ? g_pipe_slabs : 0;
  for (int S : {24, 16, 12, 8, 6, 4, 3})
    if (f->L[3] % S == 0) return S;
  return 0;
}

static bool pipeline_ready(int S)
{
  if (!g_s_in) {
    for (cudaStream_t *q : {&g_c_in, &g_s_in, &g_s_out, &g_c_out, &g_s_op2, &g_s_op3})
      if (!QG_CUDA(cudaStreamCreateWithFlags(q, cudaStreamNonBlocking))) return false;
    if (!QG_CUDA(cudaEventCreateWithFlags(&g_ev_start, cudaEventDisableTiming)) ||
        !QG_CUDA(cudaEventCreateWithFlags(&g_ev_done, cudaEventDisableTiming)) ||
        !QG_CUDA(cudaEventCreateWithFlags(&g_ev_op2, cudaEventDisableTiming)) ||
        !QG_CUDA(cudaEventCreateWithFlags(&g_ev_op3, cudaEventDisableTiming)))
      return false;
  }
  while ((int)g_ev_in.size() < S) {
    cudaEvent_t e[4];
    for (auto &x : e)
      if (!QG_CUDA(cudaEventCreateWithFlags(&x, cudaEventDisableTiming))) return false;
    g_ev_cin.push_back(e[0]);
    g_ev_in.push_back(e[1]);
    g_ev_op.push_back(e[2]);
    g_ev_rout.push_back(e[3]);
  }
  return true;
}

// the whole pipeline enqueued behind stream `origin` (which it joins again)
static bool enqueue_pipeline(cudaStream_t origin, qcdgpu_field out, qcdgpu_field in, qcdgpu_gauge g,
                             const double *vin, double *vout, double mp4, double tm, int op, int S)
{
  const int64_t V = in->V, slab = V / S;
  const size_t sbytes = (size_t)V * 24 * sizeof(double) / S;
  const bool direct = g_f64_arith == QCDGPU_ARITH_DF64;
  // the event that marks slab k as readable by the operator
  const std::vector<cudaEvent_t> &ready = direct ? g_ev_cin : g_ev_in;
  if (!QG_CUDA(cudaEventRecord(g_ev_start, origin))) return false;
  for (cudaStream_t q : {g_c_in, g_s_in, g_s_out, g_c_out, g_s_op2, g_s_op3})
    if (!QG_CUDA(cudaStreamWaitEvent(q, g_ev_start, 0))) return false;
  // The stages are enqueued slab by slab, interleaved across the streams,
  // so the first slabs' results are already queued for copy-out while the
  // host is still enqueueing later slabs (enqueueing all copy-ins, then all
  // operators, ... leaves the copy-out stream empty until the host has
  // issued every call of the apply). Each stream sees its own operations in
  // the same order either way.
  auto copy_in = [&](int k) {
    if (!QG_CUDA(cudaMemcpyAsync((char *)g_stage_in + k * sbytes, (const char *)vin + k * sbytes, sbytes,
                                 cudaMemcpyHostToDevice, g_c_in)) ||
        !QG_CUDA(cudaEventRecord(g_ev_cin[k], g_c_in)))
      return false;
    if (direct) return true;
    StreamScope scope(g_s_in);
    return QG_CUDA(cudaStreamWaitEvent(g_s_in, g_ev_cin[k], 0)) &&
           spinor_from_aos_sites(in, g_stage_in, k * slab, (k + 1) * slab) &&
           QG_CUDA(cudaEventRecord(g_ev_in[k], g_s_in));
  };
  // operator on slab k once slab `need` is in (slabs arrive in order), then
  // the reorder and copy-out of its result; consecutive slabs rotate over
  // three streams, so a thin slab's launch shares the GPU with the next ones
  // (the last three slabs all wait for the last copy-in)
  int nop = 0;
  auto apply_out = [&](int k, int need) {
    const int r = nop++ % 3;
    const cudaStream_t q = r == 0 ? origin : r == 1 ? g_s_op2 : g_s_op3;
    {
      StreamScope scope(q);
      if (!QG_CUDA(cudaStreamWaitEvent(q, ready[need], 0)) ||
          !(direct ? dslash_sites_aos(g_stage_out, g_stage_in, in, g, mp4, tm, op, (int)(k * slab),
                                      (int)((k + 1) * slab))
                   : dslash_sites(out, in, g, mp4, tm, op, -1, (int)(k * slab), (int)((k + 1) * slab))) ||
          !QG_CUDA(cudaEventRecord(g_ev_op[k], q)))
        return false;
    }
    if (direct) return QG_CUDA(cudaStreamWaitEvent(g_c_out, g_ev_op[k], 0)) &&
                       QG_CUDA(cudaMemcpyAsync((char *)vout + k * sbytes, (const char *)g_stage_out + k * sbytes,
                                               sbytes, cudaMemcpyDeviceToHost, g_c_out));
    {
      StreamScope scope(g_s_out);
      if (!QG_CUDA(cudaStreamWaitEvent(g_s_out, g_ev_op[k], 0)) ||
          !spinor_to_aos_sites(out, g_stage_out, k * slab, (k + 1) * slab) ||
          !QG_CUDA(cudaEventRecord(g_ev_rout[k], g_s_out)))
        return false;
    }
    return QG_CUDA(cudaStreamWaitEvent(g_c_out, g_ev_rout[k], 0)) &&
           QG_CUDA(cudaMemcpyAsync((char *)vout + k * sbytes, (const char *)g_stage_out + k * sbytes, sbytes,
                                   cudaMemcpyDeviceToHost, g_c_out));
  };
  // slabs 1 .. S-2 as their upper neighbours arrive; 0 and S-1 need each
  // other (periodic z), so they go last
  if (!copy_in(0) || !copy_in(1)) return false;
  for (int k = 2; k < S; k++)
    if (!copy_in(k) || !apply_out(k - 1, k)) return false;
  if (!apply_out(S - 1, S - 1) || !apply_out(0, S - 1)) return false;
  // join every side stream back into the origin
  if (!QG_CUDA(cudaEventRecord(g_ev_done, g_c_out)) || !QG_CUDA(cudaStreamWaitEvent(origin, g_ev_done, 0)) ||
      !QG_CUDA(cudaEventRecord(g_ev_op2, g_s_op2)) || !QG_CUDA(cudaStreamWaitEvent(origin, g_ev_op2, 0)) ||
      !QG_CUDA(cudaEventRecord(g_ev_op3, g_s_op3)) || !QG_CUDA(cudaStreamWaitEvent(origin, g_ev_op3, 0)))
    return false;
  return true;
}

static bool apply_pipelined(qcdgpu_field out, qcdgpu_field in, qcdgpu_gauge g, const double *vin, double *vout,
                            double mp4, double tm, int op, int S)
{
  if (!pipeline_ready(S)) return false;
  const size_t bytes = (size_t)in->V * 24 * sizeof(double);
  if (bytes > g_stage_bytes) {
    cudaFree(g_stage_in);
    cudaFree(g_stage_out);
    g_stage_in = g_stage_out = nullptr;
    g_stage_bytes = 0;
    if (!QG_CUDA(cudaMalloc(&g_stage_in, bytes)) || !QG_CUDA(cudaMalloc(&g_stage_out, bytes))) return false;
    g_stage_bytes = bytes;
  }
  cudaStream_t st = stream();
  return enqueue_pipeline(st, out, in, g, vin, vout, mp4, tm, op, S) && QG_CUDA(cudaStreamSynchronize(st));
}

static int apply_op(qcd_vector *Dv, qcd_vector *v, qcd_gaugeField *u, double m, double tm, int op)
{
  std::lock_guard<std::mutex> lk(g_mu);
  if (!check_op_args(Dv, v, u)) return 1;
  if (v->geo->numOfRequests != 0) {
    set_error("process %u: Error in qcd_communicateVectorPMGaugeP! Previous communication not finished",
              v->geo->myid);
    return 1;
  }
  qcdgpu_gauge g = gauge_in(u);
  if (!g) return 1;
  VecMirror *mi = vec_mirror(v), *mo = vec_mirror(Dv);
  if (!mi || !mo) return 1;
  const int S = pipeline_slabs(mi->f);
  if (!mi->resident && !mo->resident && S && g_pinned.count((const void *)v->D) &&
      g_pinned.count((const void *)Dv->D) && (op == QCDGPU_OP_D || op == QCDGPU_OP_Q))
    return apply_pipelined(mo->f, mi->f, g, (const double *)v->D, (double *)Dv->D, 4.0 + m, tm, op, S) ? 0 : 1;
  qcdgpu_field in = vec_in(v);
  qcdgpu_field out = vec_out(Dv);
  if (!in || !out) return 1;
  if (!dslash(out, in, g, 4.0 + m, tm, op, -1)) return 1;
  return vec_done(Dv) ? 0 : 1;
}

}  // namespace qg

using namespace qg;

extern "C" {

// ------------------------------------------------------------- geometry
int qcd_initGeometry(qcd_geometry *geo, const qcd_uint_2 L[], const qcd_uint_2 P[], const qcd_real_8 theta[],
                     const int myid, const int numprocs)
{
  // checks of qcd_init.c:31-52, plus the single-GPU restriction
  if (L[0] % P[0] || L[1] % P[1] || L[2] % P[2] || L[3] % P[3]) {
    set_error("process %i: Error in qcd_initGeometry! %i x %i x %i x %i cannot be subdivided in %i x %i x %i x %i",
              myid, L[0], L[1], L[2], L[3], P[0], P[1], P[2], P[3]);
    return 1;
  }
  if (P[0] != 1 || P[1] != 1 || P[2] != 1 || P[3] != 1 || numprocs != 1 || myid != 0) {
    set_error("process %i: Error in qcd_initGeometry! one GPU holds the whole lattice: P must be 1 1 1 1 "
              "with one process", myid);
    return 1;
  }
  if (L[0] < 2 || L[1] < 2 || L[2] < 2 || L[3] < 2) {
    set_error("process %i: Error in qcd_initGeometry! Local lattices must be at least 2x2x2x2", myid);
    return 1;
  }
  if (((uint64_t)L[0] * L[1] * L[2] * L[3]) % 2) {
    set_error("process %i: Error in qcd_initGeometry! Local volume must be multiple of 2.", myid);
    return 1;
  }
  memset(geo, 0, sizeof(*geo));
  for (int i = 0; i < 4; i++) {
    geo->L[i] = L[i];
    geo->lL[i] = L[i];
    geo->theta[i] = theta[i];
  }
  const uint64_t Lt = L[0], Lx = L[1], Ly = L[2], Lz = L[3];
  geo->V = geo->lV = Lt * Lx * Ly * Lz;
  geo->V3 = geo->lV3 = Lx * Ly * Lz;
  geo->myid = 0;
  geo->nproc = 1;
  geo->plus = (qcd_uint_8(*)[4])malloc(sizeof(qcd_uint_8) * 4 * geo->lV);
  geo->minus = (qcd_uint_8(*)[4])malloc(sizeof(qcd_uint_8) * 4 * geo->lV);
  geo->plus3d = (qcd_uint_8(*)[4])malloc(sizeof(qcd_uint_8) * 4 * geo->lV3);
  geo->minus3d = (qcd_uint_8(*)[4])malloc(sizeof(qcd_uint_8) * 4 * geo->lV3);
  geo->eo = (qcd_uint_8(*)[2])malloc(sizeof(qcd_uint_8) * geo->lV);
  geo->edgePoints = geo->lV - (Lt - 2) * (Lx - 2) * (Ly - 2) * (Lz - 2);
  geo->edge0Points = geo->lV3 - (Lx - 2) * (Ly - 2) * (Lz - 2);
  geo->edge = (qcd_uint_8 *)malloc(sizeof(qcd_uint_8) * (geo->edgePoints ? geo->edgePoints : 1));
  geo->edge0 = (qcd_uint_8 *)malloc(sizeof(qcd_uint_8) * (geo->edge0Points ? geo->edge0Points : 1));
  if (!geo->plus || !geo->minus || !geo->plus3d || !geo->minus3d || !geo->eo || !geo->edge || !geo->edge0) {
    set_error("process %i: Error in qcd_initGeometry! Out of memory", myid);
    return 1;
  }
  // periodic neighbour tables (qcd_init.c:110-124 at one rank), t fastest
  auto lex = [&](uint64_t t, uint64_t x, uint64_t y, uint64_t z) { return t + Lt * (x + Lx * (y + Ly * z)); };
  uint64_t j = 0, ne = 0, no = 0;
  for (uint64_t z = 0; z < Lz; z++)
    for (uint64_t y = 0; y < Ly; y++)
      for (uint64_t x = 0; x < Lx; x++)
        for (uint64_t t = 0; t < Lt; t++) {
          uint64_t i = lex(t, x, y, z);
          geo->plus[i][0] = lex((t + 1) % Lt, x, y, z);
          geo->plus[i][1] = lex(t, (x + 1) % Lx, y, z);
          geo->plus[i][2] = lex(t, x, (y + 1) % Ly, z);
          geo->plus[i][3] = lex(t, x, y, (z + 1) % Lz);
          geo->minus[i][0] = lex((t + Lt - 1) % Lt, x, y, z);
          geo->minus[i][1] = lex(t, (x + Lx - 1) % Lx, y, z);
          geo->minus[i][2] = lex(t, x, (y + Ly - 1) % Ly, z);
          geo->minus[i][3] = lex(t, x, y, (z + Lz - 1) % Lz);
          if (z == 0 || z == Lz - 1 || y == 0 || y == Ly - 1 || x == 0 || x == Lx - 1 || t == 0 || t == Lt - 1)
            geo->edge[j++] = i;
          // even/odd split (qcd_init.c:315-335): (0,0,0,0) is even at one rank
          // when sum_mu P_mu lL_mu = sum_mu L_mu is even
          uint64_t b = (Lt + Lx + Ly + Lz) % 2;
          if ((t + x + y + z + b) % 2) geo->eo[no++][1] = i;
          else geo->eo[ne++][0] = i;
        }
  j = 0;
  for (uint64_t z = 0; z < Lz; z++)
    for (uint64_t y = 0; y < Ly; y++)
      for (uint64_t x = 0; x < Lx; x++) {
        uint64_t i = x + Lx * (y + Ly * z);
        geo->plus3d[i][1] = ((x + 1) % Lx) + Lx * (y + Ly * z);
        geo->plus3d[i][2] = x + Lx * (((y + 1) % Ly) + Ly * z);
        geo->plus3d[i][3] = x + Lx * (y + Ly * ((z + 1) % Lz));
        geo->minus3d[i][1] = ((x + Lx - 1) % Lx) + Lx * (y + Ly * z);
        geo->minus3d[i][2] = x + Lx * (((y + Ly - 1) % Ly) + Ly * z);
        geo->minus3d[i][3] = x + Lx * (y + Ly * ((z + Lz - 1) % Lz));
        if (z == 0 || z == Lz - 1 || y == 0 || y == Ly - 1 || x == 0 || x == Lx - 1) geo->edge0[j++] = i;
      }
  geo->numOfRequests = 0;
  geo->initialized = 1;
  return 0;
}

void qcd_destroyGeometry(const qcd_geometry *geo)
{
  free(geo->plus);
  free(geo->minus);
  free(geo->plus3d);
  free(geo->minus3d);
  free(geo->edge);
  free(geo->edge0);
  free(geo->eo);
}

// --------------------------------------------------------------- fields
int qcd_initVector(qcd_vector *vec, qcd_geometry *geo)
{
  if (!geo->initialized) {
    set_error("error in qcd_initVector! Geometry must be properly initialized.");
    return 1;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  memset(vec, 0, sizeof(*vec));
  vec->D = (qcd_complex_16(*)[4][3])host_alloc(sizeof(qcd_complex_16) * 12 * geo->lV);
  if (!vec->D) {
    set_error("process %i: Error in qcd_initVector! Out of memory", geo->myid);
    return 1;
  }
  vec->geo = geo;
  vec->initialized = 1;
  return 0;
}

void qcd_destroyVector(qcd_vector *vec)
{
  if (!vec->initialized) {
    fprintf(stderr, "Error in qcd_destroyVector! Vector not initialized\n");
    return;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_vec.find((const void *)vec->D);
  if (it != g_vec.end()) {
    field_free(it->second.f);
    g_vec.erase(it);
  }
  host_free(vec->D);
}

int qcd_initGaugeField(qcd_gaugeField *u, qcd_geometry *geo)
{
  if (!geo->initialized) {
    set_error("error in qcd_initGaugeField! Geometry must be properly initialized.");
    return 1;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  memset(u, 0, sizeof(*u));
  u->D = (qcd_complex_16(*)[4][3][3])host_alloc(sizeof(qcd_complex_16) * 36 * geo->lV);
  if (!u->D) {
    set_error("process %i: Error in qcd_initGaugeField! Out of memory", geo->myid);
    return 1;
  }
  u->geo = geo;
  u->initialized = 1;
  return 0;
}

void qcd_destroyGaugeField(qcd_gaugeField *u)
{
  if (!u->initialized) {
    fprintf(stderr, "Error in qcd_destroyGaugeField! Gauge field not initialized\n");
    return;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_gauge.find((const void *)u->D);
  if (it != g_gauge.end()) {
    gauge_forget(it->second.g);
    gauge_free(it->second.g);
    g_gauge.erase(it);
  }
  host_free(u->D);
}

// ------------------------------------------------------------ operators
int qcd_applyWilsonTMOp(qcd_vector *Dv, qcd_vector *v, qcd_gaugeField *u, qcd_real_8 m, qcd_real_8 tm)
{
  return apply_op(Dv, v, u, m, tm, QCDGPU_OP_D);
}
int qcd_applyWilsonTMOpNoScripts(qcd_vector *Dv, qcd_vector *v, qcd_gaugeField *u, qcd_real_8 m, qcd_real_8 tm)
{
  return apply_op(Dv, v, u, m, tm, QCDGPU_OP_D);
}
int qcd_applyWilsonTMOpNoOptim(qcd_vector *Dv, qcd_vector *v, qcd_gaugeField *u, qcd_real_8 m, qcd_real_8 tm)
{
  return apply_op(Dv, v, u, m, tm, QCDGPU_OP_D);
}
int qcd_applyQTMOp(qcd_vector *Dv, qcd_vector *v, qcd_gaugeField *u, qcd_real_8 m, qcd_real_8 tm)
{
  return apply_op(Dv, v, u, m, tm, QCDGPU_OP_Q);
}

// ----------------------------------------------------------------- BLAS
#define QG_BLAS_GUARD std::lock_guard<std::mutex> lk(g_mu)

void qcd_zeroVector(qcd_vector *vec)
{
  QG_BLAS_GUARD;
  qcdgpu_field f = vec_out(vec);
  if (f && blas_zero(f)) vec_done(vec);
}

void qcd_setVector(qcd_vector *vec, qcd_complex_16 c)
{
  QG_BLAS_GUARD;
  qcdgpu_field f = vec_out(vec);
  if (f && blas_set(f, c.re, c.im)) vec_done(vec);
}

void qcd_copyVector(qcd_vector *dest, qcd_vector *src)
{
  QG_BLAS_GUARD;
  qcdgpu_field s = vec_in(src);
  qcdgpu_field d = s ? vec_out(dest) : nullptr;
  if (d && blas_copy(d, s)) vec_done(dest);
}

void qcd_mulVectorC(qcd_vector *vec, qcd_complex_16 c)
{
  QG_BLAS_GUARD;
  qcdgpu_field f = vec_in(vec);
  if (f && blas_axpby(f, c.re, c.im, f, 0.0, 0.0, f)) vec_done(vec);
}

void qcd_scaleVector(qcd_vector *vec, qcd_real_8 r)
{
  QG_BLAS_GUARD;
  qcdgpu_field f = vec_in(vec);
  if (f && blas_axpby(f, r, 0.0, f, 0.0, 0.0, f)) vec_done(vec);
}

static void lincomb(qcd_vector *out, double ar, double ai, qcd_vector *x, double br, double bi, qcd_vector *y)
{
  qcdgpu_field fx = vec_in(x);
  qcdgpu_field fy = fx ? (y->D == x->D ? fx : vec_in(y)) : nullptr;
  qcdgpu_field fo = fy ? vec_out(out) : nullptr;
  if (fo && blas_axpby(fo, ar, ai, fx, br, bi, fy)) vec_done(out);
}

void qcd_subVector(qcd_vector *difference, qcd_vector *minuend, qcd_vector *subtrahend)
{
  QG_BLAS_GUARD;
  lincomb(difference, 1.0, 0.0, minuend, -1.0, 0.0, subtrahend);
}

void qcd_addVector(qcd_vector *sum, qcd_vector *summand1, qcd_vector *summand2)
{
  QG_BLAS_GUARD;
  lincomb(sum, 1.0, 0.0, summand1, 1.0, 0.0, summand2);
}

void qcd_axpyVector(qcd_vector *axpy, qcd_complex_16 a, qcd_vector *x, qcd_vector *y)
{
  QG_BLAS_GUARD;
  lincomb(axpy, a.re, a.im, x, 1.0, 0.0, y);
}

qcd_complex_16 qcd_mulAdjointVectorVector(qcd_vector *factor1, qcd_vector *factor2)
{
  QG_BLAS_GUARD;
  qcd_complex_16 r = {NAN, NAN};
  qcdgpu_field a = vec_in(factor1);
  qcdgpu_field b = a ? (factor2->D == factor1->D ? a : vec_in(factor2)) : nullptr;
  double d[2];
  if (b && blas_dot(a, b, d)) {
    r.re = d[0];
    r.im = d[1];
  }
  return r;
}

qcd_real_8 qcd_normVector(qcd_vector *vec)
{
  QG_BLAS_GUARD;
  qcdgpu_field f = vec_in(vec);
  double n2;
  if (f && blas_norm2(f, &n2)) return sqrt(n2);
  return NAN;
}

void qcd_gamma5Vector(qcd_vector *v)
{
  QG_BLAS_GUARD;
  qcdgpu_field f = vec_in(v);
  if (f && blas_gamma5(f, f)) vec_done(v);
}

// ------------------------------------------------------------- noise
// The reference's qcd_z2Vector (lib/src/qcd_stochastic.c:8-58) fills a vector
// with Z4 noise {1, i, -1, -i} on one time-slice (every site when t_slice < 0;
// a zero vector when t_slice is past the lattice) from GSL's ranlux stream.
// Here every call draws a new vector from the library's own counter-based
// stream: key (seed, call number), counter 12 x + spin-colour component.
static uint64_t g_noise_seed = 1, g_noise_calls = 0;

void qcd_z2Vector(qcd_vector *vec, int t_slice)
{
  QG_BLAS_GUARD;
  qcdgpu_field f = vec_out(vec);
  const uint64_t seed = g_noise_seed * 0x9E3779B97F4A7C15ull + g_noise_calls++;
  if (f && field_noise(f, seed, t_slice, 4)) vec_done(vec);
}

// --------------------------------------------- per-site operator helpers
// lib/src/qcd_wilson.c:18-103 (include/qcd_wilson.h:628-633): host functions
// on one site's 4 x 3 spin-colour vector. gamma_mu (mu = 0..5) in the chiral
// basis of qcd_gamma.c:46-103 (gamma_4 = -gamma_0, gamma_5 = diag(1, 1, -1,
// -1)); each row has one non-zero entry: column kGamCol[mu][row], value
// kGamVal[mu][row] in {1, -1, i, -i} as (re, im).
static const int kGamCol[6][4] = {{2, 3, 0, 1}, {3, 2, 1, 0}, {3, 2, 1, 0}, {2, 3, 0, 1}, {2, 3, 0, 1}, {0, 1, 2, 3}};
static const double kGamVal[6][4][2] = {{{-1, 0}, {-1, 0}, {-1, 0}, {-1, 0}}, {{0, -1}, {0, -1}, {0, 1}, {0, 1}},
                                        {{-1, 0}, {1, 0}, {1, 0}, {-1, 0}},   {{0, -1}, {0, 1}, {0, 1}, {0, -1}},
                                        {{1, 0}, {1, 0}, {1, 0}, {1, 0}},     {{1, 0}, {1, 0}, {-1, 0}, {-1, 0}}};

static inline qcd_complex_16 cmul16(qcd_complex_16 a, qcd_complex_16 b)
{
  return qcd_complex_16{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}

// result = (1 + sign gamma_mu) vec; entries are 0, +-1, +-i, so the sum of
// the row's two terms is exact
static void one_pm_gamma(qcd_complex_16 result[][3], qcd_complex_16 vec[][3], int mu, double sign)
{
  for (int al = 0; al < 4; al++) {
    const int be = kGamCol[mu][al];
    const qcd_complex_16 g{sign * kGamVal[mu][al][0], sign * kGamVal[mu][al][1]};
    for (int c = 0; c < 3; c++) {
      const qcd_complex_16 t = cmul16(g, vec[be][c]);
      result[al][c] = qcd_complex_16{vec[al][c].re + t.re, vec[al][c].im + t.im};
    }
  }
}

void qcd_onePlusGamma(qcd_complex_16 result[][3], qcd_complex_16 vec[][3], qcd_uint_2 mu)
{
  if (mu > 5) return;
  one_pm_gamma(result, vec, mu, 1.0);
}

void qcd_oneMinusGamma(qcd_complex_16 result[][3], qcd_complex_16 vec[][3], qcd_uint_2 mu)
{
  if (mu > 5) return;
  one_pm_gamma(result, vec, mu, -1.0);
}

// result = u vec on every spin (colour matrix u[row][col])
void qcd_applyU(qcd_complex_16 result[][3], qcd_complex_16 u[][3], qcd_complex_16 vec[][3])
{
  for (int al = 0; al < 4; al++)
    for (int c1 = 0; c1 < 3; c1++) {
      qcd_complex_16 s{0.0, 0.0};
      for (int c2 = 0; c2 < 3; c2++) {
        const qcd_complex_16 t = cmul16(u[c1][c2], vec[al][c2]);
        s = qcd_complex_16{s.re + t.re, s.im + t.im};
      }
      result[al][c1] = s;
    }
}

// result = u^+ vec on every spin
void qcd_applyUDagger(qcd_complex_16 result[][3], qcd_complex_16 u[][3], qcd_complex_16 vec[][3])
{
  for (int al = 0; al < 4; al++)
    for (int c1 = 0; c1 < 3; c1++) {
      qcd_complex_16 s{0.0, 0.0};
      for (int c2 = 0; c2 < 3; c2++) {
        const qcd_complex_16 t = cmul16(qcd_complex_16{u[c2][c1].re, -u[c2][c1].im}, vec[al][c2]);
        s = qcd_complex_16{s.re + t.re, s.im + t.im};
      }
      result[al][c1] = s;
    }
}

// result = (mp4 + i tm gamma_5) vec
void qcd_massTerms(qcd_complex_16 result[][3], qcd_complex_16 vec[][3], qcd_real_8 mp4, qcd_real_8 tm)
{
  const qcd_complex_16 itm{0.0, tm};
  for (int al = 0; al < 4; al++)
    for (int c = 0; c < 3; c++) {
      const qcd_complex_16 g5v = cmul16(qcd_complex_16{kGamVal[5][al][0], 0.0}, vec[al][c]);
      const qcd_complex_16 t = cmul16(g5v, itm);
      result[al][c] = qcd_complex_16{vec[al][c].re * mp4 + t.re, vec[al][c].im * mp4 + t.im};
    }
}

// vec <- vec phi
void qcd_phaseMul(qcd_complex_16 vec[][3], qcd_complex_16 phi)
{
  for (int al = 0; al < 4; al++)
    for (int c = 0; c < 3; c++) vec[al][c] = cmul16(vec[al][c], phi);
}

// -------------------------------------------------------- communication
int qcd_communicateVectorPMGaugeP(qcd_vector *v, qcd_gaugeField *u)
{
  (void)u;
  if (v->geo->numOfRequests != 0) {
    set_error("process %u: Error in qcd_communicateVectorPMGaugeP! Previous communication not finished",
              v->geo->myid);
    return 1;
  }
  return 0;  // one GPU holds the whole lattice: there is no halo to send
}

void qcd_waitall(qcd_geometry *geo) { geo->numOfRequests = 0; }

// ------------------------------------------------------ source construction
// include/qcd_smearing.h:41 (lib/src/qcd_smearing.c:209): one 3D APE step
int qcd_apeSmear3d(qcd_gaugeField *apeu, qcd_gaugeField *u, qcd_real_8 alpha)
{
  std::lock_guard<std::mutex> lk(g_mu);
  if (!apeu || !apeu->initialized || !apeu->D || !apeu->geo || apeu->geo->initialized != 1 || apeu->D == u->D) {
    set_error("qcd_apeSmear3d: output gauge field not initialized or the same as the input");
    return 1;
  }
  qcdgpu_gauge gin = gauge_in(u);
  if (!gin) return 1;
  int L[4];
  geo_L(apeu->geo, L);
  if (!same_L(L, gin->L)) {
    set_error("qcd_apeSmear3d: lattices differ");
    return 1;
  }
  GaugeMirror &m = g_gauge[(const void *)apeu->D];
  if (m.g && (!same_L(m.g->L, L) || memcmp(m.g->theta, apeu->geo->theta, sizeof(m.g->theta)) != 0)) {
    gauge_forget(m.g);
    gauge_free(m.g);
    m.g = nullptr;
    m.resident = false;
  }
  if (!m.g) m.g = gauge_new(L, apeu->geo->theta, QCDGPU_F64, 18);
  if (!m.g || !ape3d(m.g, gin, alpha)) return 1;
  if (m.resident) return QG_CUDA(cudaStreamSynchronize(stream())) ? 0 : 1;
  return download_gauge_aos(m.g, (double *)apeu->D) ? 0 : 1;
}

// include/qcd_smearing.h:39 (lib/src/qcd_smearing.c:25): one Gaussian step on time-slice t
int qcd_gaussIteration3d(qcd_vector *v, qcd_gaugeField *u, qcd_real_8 alpha, qcd_uint_4 t)
{
  std::lock_guard<std::mutex> lk(g_mu);
  qcdgpu_field f = vec_in(v);
  qcdgpu_gauge g = f ? gauge_in(u) : nullptr;
  if (!f || !g) return 1;
  if (!gauss3d(f, g, alpha, (int)t, 1)) return 1;
  return vec_done(v) ? 0 : 1;
}

// include/qcd_observables.h:12 (lib/src/qcd_observables.c:15): mean plaquette
qcd_real_8 qcd_calculatePlaquette(qcd_gaugeField *u)
{
  std::lock_guard<std::mutex> lk(g_mu);
  qcdgpu_gauge g = gauge_in(u);
  if (!g) return NAN;
  return plaquette(g);
}

// ------------------------------------------------------- parameter files
// include/qcd_io.h:21 (lib/src/qcd_io.c:83-110): the whole file in a new
// buffer (the caller frees it); *len = file size + 1, as the reference counts
// it. The last byte is a terminating zero (the reference leaves it unset).
char *qcd_getParams(char *fname, int *len)
{
  FILE *f = fname ? fopen(fname, "rb") : nullptr;
  if (!f) {
    set_error("Error, cannot open %s for reading", fname ? fname : "(null)");
    return nullptr;
  }
  long n = -1;
  if (fseek(f, 0, SEEK_END) == 0) n = ftell(f);
  char *p = n >= 0 && n < INT32_MAX ? (char *)malloc((size_t)n + 1) : nullptr;
  if (!p || fseek(f, 0, SEEK_SET) != 0 || fread(p, 1, (size_t)n, f) != (size_t)n) {
    set_error("Error, cannot read %s", fname);
    free(p);
    fclose(f);
    return nullptr;
  }
  fclose(f);
  p[n] = '\0';
  *len = (int)n + 1;
  return p;
}

// include/qcd_io.h:22 (lib/src/qcd_io.c:114-129): the text after the first
// occurrence of token, cut at the next '<' (written into params, as the
// reference does). A missing token gives an empty string (the reference
// returns the buffer's last bytes).
char *qcd_getParam(char token[], char *params, int len)
{
  const int tl = (int)strlen(token);
  for (int i = 0; i + tl < len; i++) {
    if (memcmp(token, params + i, (size_t)tl) == 0) {
      char *v = params + i + tl;
      char *end = (char *)memchr(v, '<', (size_t)(len - i - tl));
      if (end) *end = '\0';
      return v;
    }
  }
  static char empty[1];
  empty[0] = '\0';
  return empty;
}

// ------------------------------------------------------------ LIME files
// include/qcd_io.h:26 (lib/src/qcd_io.c:204): ILDG configuration into u
int qcd_getGaugeLime(char *fname, qcd_gaugeField *u)
{
  std::lock_guard<std::mutex> lk(g_mu);
  if (!u || !u->initialized || !u->D || !u->geo || u->geo->initialized != 1) {
    set_error("qcd_getGaugeLime: gauge field must be properly initialized");
    return 1;
  }
  int L[4];
  geo_L(u->geo, L);
  const size_t bytes = (size_t)u->geo->V * 72 * sizeof(double);
  void *dev = nullptr;
  bool ok = QG_CUDA(cudaMalloc(&dev, bytes)) && lime_read_gauge(fname, L, dev) &&
            QG_CUDA(cudaMemcpy(u->D, dev, bytes, cudaMemcpyDeviceToHost));
  auto it = g_gauge.find((const void *)u->D);
  if (ok && it != g_gauge.end() && it->second.g) {
    gauge_forget(it->second.g);
    if (it->second.resident) ok = pack_gauge(it->second.g, dev) && QG_CUDA(cudaStreamSynchronize(stream()));
  }
  if (dev) cudaFree(dev);
  return ok ? 0 : 1;
}

// include/qcd_io.h:27 (lib/src/qcd_io.c:401): type qcd_GF_LIME (0) only
int qcd_getGaugeField(char *fname, int type, qcd_gaugeField *u)
{
  if (type != 0) {
    set_error("qcd_getGaugeField: unknown type %d (LIME = 0)", type);
    return 1;
  }
  return qcd_getGaugeLime(fname, u);
}

// include/qcd_io.h:29 (lib/src/qcd_io.c:419): FP64 ILDG file with an xlf-info message
int qcd_writeGaugeLime(char *fname, qcd_gaugeField *u, char *message)
{
  std::lock_guard<std::mutex> lk(g_mu);
  qcdgpu_gauge g = gauge_in(u);  // the device copy (uploaded unless resident)
  if (!g) return 1;
  const size_t bytes = (size_t)g->V * 72 * sizeof(double);
  void *dev = nullptr;
  bool ok = QG_CUDA(cudaMalloc(&dev, bytes)) && gauge_to_aos_dev(g, dev) &&
            lime_write_gauge(fname, g->L, dev, message);
  if (dev) cudaFree(dev);
  return ok ? 0 : 1;
}

// include/qcd_io.h:36 (lib/src/qcd_io.c:984): ETMC spinor file into v
int qcd_getVectorLime(char *fname, qcd_vector *v)
{
  std::lock_guard<std::mutex> lk(g_mu);
  qcdgpu_field f = vec_out(v);
  if (!f) return 1;
  const size_t bytes = (size_t)f->V * 24 * sizeof(double);
  void *dev = nullptr;
  bool ok = QG_CUDA(cudaMalloc(&dev, bytes)) && lime_read_spinor(fname, f->L, dev) && spinor_from_aos_dev(f, dev);
  if (dev) {
    cudaStreamSynchronize(stream());
    cudaFree(dev);
  }
  return ok && vec_done(v) ? 0 : 1;
}

// include/qcd_io.h:35-39 (lib/src/qcd_io.c:907-1340, :1386): the legacy
// vector formats and the dispatcher by type (0 CMI, 1 HMC, 2 HMCV, 3 LIME)
static int get_legacy(char *fname, int type, qcd_uint_2 nu, qcd_uint_2 c2, qcd_vector *v)
{
  std::lock_guard<std::mutex> lk(g_mu);
  qcdgpu_field f = vec_out(v);
  if (!f) return 1;
  const size_t bytes = (size_t)f->V * 24 * sizeof(double);
  void *dev = nullptr;
  bool ok = QG_CUDA(cudaMalloc(&dev, bytes)) && legacy_read_spinor(fname, f->L, type, nu * 3 + c2, dev) &&
            spinor_from_aos_dev(f, dev);
  if (dev) {
    cudaStreamSynchronize(stream());
    cudaFree(dev);
  }
  return ok && vec_done(v) ? 0 : 1;
}

int qcd_getVectorCMI(char *fname, qcd_uint_2 nu, qcd_uint_2 c2, qcd_vector *v) { return get_legacy(fname, 0, nu, c2, v); }
int qcd_getVectorHMC(char *fname, qcd_uint_2 nu, qcd_uint_2 c2, qcd_vector *v) { return get_legacy(fname, 1, nu, c2, v); }
int qcd_getVectorHMCV(char *fname, qcd_uint_2 nu, qcd_uint_2 c2, qcd_vector *v) { return get_legacy(fname, 2, nu, c2, v); }

int qcd_getVector(char *fname, int type, qcd_uint_2 nu, qcd_uint_2 c2, qcd_vector *v)
{
  if (!v || !v->initialized) {
    set_error("Error in qcd_getVector! Vector must be properly initialized.");
    return 1;
  }
  if (type >= 0 && type <= 2) return get_legacy(fname, type, nu, c2, v);
  if (type == 3) return qcd_getVectorLime(fname, v);
  set_error("process %i: Error in qcd_getVector! Unknown type.", v->geo ? (int)v->geo->myid : 0);
  return 1;
}

// include/qcd_io.h:43 (lib/src/qcd_io.c:1766): type qcd_PROP_LIME (3) or qcd_SOURCE_LIME (4)
int qcd_writeVectorLime(char *fname, int type, qcd_vector *v)
{
  std::lock_guard<std::mutex> lk(g_mu);
  if (type != 3 && type != 4) {
    set_error("qcd_writeVectorLime: type must be qcd_PROP_LIME (3) or qcd_SOURCE_LIME (4)");
    return 1;
  }
  qcdgpu_field f = vec_in(v);
  if (!f) return 1;
  const size_t bytes = (size_t)f->V * 24 * sizeof(double);
  void *dev = nullptr;
  bool ok = QG_CUDA(cudaMalloc(&dev, bytes)) && spinor_to_aos_dev(f, dev) &&
            lime_write_spinor(fname, f->L, dev, type == 4);
  if (dev) cudaFree(dev);
  return ok ? 0 : 1;
}

// include/qcd_io.h:42 (lib/src/qcd_io.c:1685): one vector as a CMI file;
// nu and c2 are unused there too
int qcd_writeVectorCMI(char *fname, qcd_uint_2 nu, qcd_uint_2 c2, qcd_vector *v)
{
  std::lock_guard<std::mutex> lk(g_mu);
  (void)nu;
  (void)c2;
  qcdgpu_field f = vec_in(v);
  if (!f) return 1;
  const size_t bytes = (size_t)f->V * 24 * sizeof(double);
  void *dev = nullptr;
  bool ok = QG_CUDA(cudaMalloc(&dev, bytes)) && spinor_to_aos_dev(f, dev) && cmi_write_spinor(fname, f->L, dev);
  if (dev) cudaFree(dev);
  return ok ? 0 : 1;
}

// include/qcd_io.h:44 (lib/src/qcd_io.c:1951): 0 CMI, 3 / 4 LIME propagator
// / source (the reference's HMC writer is commented out)
int qcd_writeVector(char *fname, int type, qcd_uint_2 nu, qcd_uint_2 c2, qcd_vector *v)
{
  if (!v || !v->initialized) {
    set_error("Error in qcd_writeVector! Vector must be properly initialized.");
    return 1;
  }
  if (type == 0) return qcd_writeVectorCMI(fname, nu, c2, v);
  if (type == 3 || type == 4) return qcd_writeVectorLime(fname, type, v);
  set_error("process %i: Error in qcd_writeVector! Unknown type.", v->geo ? (int)v->geo->myid : 0);
  return 1;
}

// --------------------------------------------------------------- solvers
qcd_int_4 gcr(qcd_vector *sol, qcd_vector *src, qcd_gaugeField *u, qcd_real_8 kappa, qcd_real_8 muTM,
              qcd_uint_4 n, qcd_geometry *geo)
{
  std::lock_guard<std::mutex> lk(g_mu);
  (void)geo;
  if (!check_op_args(sol, src, u)) return EXIT_FAILURE;
  qcdgpu_gauge g = gauge_in(u);
  qcdgpu_field b = g ? vec_in(src) : nullptr;
  qcdgpu_field x = b ? vec_out(sol) : nullptr;
  if (!x) return EXIT_FAILURE;
  // m = 1/(2 kappa) - 4 as the callers pass it (invert.c:46), diagonal m + 4
  double mp4 = (1.0 / (2.0 * kappa) - 4.0) + 4.0;
  if (gcr_dropin(x, b, g, mp4, muTM, (int)n, g_gcr_shipped)) return EXIT_FAILURE;
  return vec_done(sol) ? 0 : EXIT_FAILURE;
}

static qcd_int_4 solve_dropin(int solver, qcd_vector *sol, qcd_vector *src, qcd_gaugeField *u, double kappa,
                              double mu, double tol, unsigned maxiter)
{
  std::lock_guard<std::mutex> lk(g_mu);
  if (!check_op_args(sol, src, u)) return -1;
  qcdgpu_gauge g = gauge_in(u);
  qcdgpu_field b = g ? vec_in(src) : nullptr;
  qcdgpu_field x = b ? vec_out(sol) : nullptr;
  if (!x) return -1;
  qcdgpu_solve_params p;
  memset(&p, 0, sizeof(p));
  p.solver = solver;
  p.op = QCDGPU_OP_D;
  p.inner_prec = QCDGPU_F64;
  p.tol = tol;
  p.maxiter = (int)maxiter;
  double mp4 = (1.0 / (2.0 * kappa) - 4.0) + 4.0;
  int st = solve(x, b, g, mp4, mu, &p);
  if (!vec_done(sol)) return -1;
  return st == 0 ? p.iters : -1;
}

qcd_int_4 bicgstab(qcd_vector *sol, qcd_vector *src, qcd_gaugeField *u, qcd_real_8 kappa, qcd_real_8 muTM,
                   qcd_real_8 tol, qcd_uint_4 maxiter, qcd_geometry *geo)
{
  (void)geo;
  return solve_dropin(QCDGPU_SOLVER_BICGSTAB, sol, src, u, kappa, muTM, tol, maxiter);
}

qcd_int_4 cgnr(qcd_vector *sol, qcd_vector *src, qcd_gaugeField *u, qcd_real_8 kappa, qcd_real_8 muTM,
               qcd_real_8 tol, qcd_uint_4 maxiter, qcd_geometry *geo)
{
  (void)geo;
  return solve_dropin(QCDGPU_SOLVER_CGNR, sol, src, u, kappa, muTM, tol, maxiter);
}

// ------------------------------------------------------------ residency
int qcdgpu_set_noise_seed(uint64_t seed)
{
  g_noise_seed = seed;
  g_noise_calls = 0;
  return 0;
}

int qcdgpu_vector_make_resident(qcd_vector *v)
{
  std::lock_guard<std::mutex> lk(g_mu);
  VecMirror *m = vec_mirror(v);
  if (!m) return 1;
  if (!m->resident && !upload_spinor_aos(m->f, (const double *)v->D)) return 1;
  if (!QG_CUDA(cudaStreamSynchronize(stream()))) return 1;
  m->resident = true;
  return 0;
}

int qcdgpu_vector_to_host(qcd_vector *v)
{
  std::lock_guard<std::mutex> lk(g_mu);
  VecMirror *m = vec_mirror(v);
  return m && download_spinor_aos(m->f, (double *)v->D) ? 0 : 1;
}

int qcdgpu_vector_to_device(qcd_vector *v)
{
  std::lock_guard<std::mutex> lk(g_mu);
  VecMirror *m = vec_mirror(v);
  return m && upload_spinor_aos(m->f, (const double *)v->D) && QG_CUDA(cudaStreamSynchronize(stream())) ? 0 : 1;
}

int qcdgpu_vector_release(qcd_vector *v)
{
  std::lock_guard<std::mutex> lk(g_mu);
  VecMirror *m = vec_mirror(v);
  if (!m) return 1;
  if (m->resident && !download_spinor_aos(m->f, (double *)v->D)) return 1;
  m->resident = false;
  return 0;
}

int qcdgpu_gauge_upload(qcd_gaugeField *u)
{
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_gauge.find((const void *)u->D);
  if (it != g_gauge.end()) it->second.resident = false;  // force a fresh upload
  qcdgpu_gauge g = gauge_in(u);
  if (!g) return 1;
  g_gauge[(const void *)u->D].resident = true;
  return 0;
}

int qcdgpu_gauge_release(qcd_gaugeField *u)
{
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_gauge.find((const void *)u->D);
  if (it != g_gauge.end()) it->second.resident = false;
  return 0;
}

}  // extern "C"

extern "C" int qcdgpu_set_pipeline_slabs(int S)
{
  if (S < 0 || S == 1 || S == 2) {
    qg::set_error("pipeline slabs: 0 (automatic) or at least 3 (got %d)", S);
    return 1;
  }
  qg::g_pipe_slabs = S;
  return 0;
}
