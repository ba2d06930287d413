// serve.cu -- request server: continuous batching of solve requests over
// resident gauge fields, HBM-budget admission, per-request latency.
//
// Scheduling round (qcdgpu_server_progress):
//   1. admission: requests are admitted strictly in arrival order while the
//      head's bytes (FP64 x and b per RHS, plus its gauge field's batch when
//      that is not yet built) fit in the budget -- idle batches of other
//      gauge fields are freed to make room; admission allocates and fills
//      the request's fields;
//   2. slot filling: each gauge field's pending RHS (admitted requests in
//      order, columns in order) enter its batch while slots are free;
//   3. iteration: one chunk is launched on every busy batch -- each on its
//      own stream, so batches of different gauge fields overlap on the GPU --
//      and then each chunk is finished (reliable updates, retirement);
//   4. accounting: retired RHS update their request; a request whose last
//      RHS retired is completed with its latency.
#include <chrono>
#include <deque>
#include <map>
#include <vector>

#include <thread>

#include "mrhs.h"

namespace qg {

struct SrvRequest {
  int tag = 0, gauge = 0, nrhs = 0, op = QCDGPU_OP_D, maxiter = 0;
  uint64_t seed = 0;
  double kappa = 0, mu = 0, tol = 0;
  std::vector<qcdgpu_field> src;  // caller's sources (may be empty)
  std::vector<qcdgpu_field> x, b;
  bool admitted = false, complete = false;
  int next_col = 0, retired = 0, status = 0, max_iters = 0, total_iters = 0;
  double max_res = 0;
  double t_submit = 0, t_admit = 0, t_done = 0;
  size_t bytes = 0;
};

struct SrvGauge {
  qcdgpu_gauge g = nullptr;
  qcdgpu_batch batch = nullptr;
  std::deque<int> pending;  // admitted request ids with columns left to enter
};

}  // namespace qg

struct qcdgpu_server_s {
  size_t budget = 0, used = 0;
  int slots = 0;
  int next_id = 0;
  std::vector<qg::SrvGauge> gauges;
  std::map<int, qg::SrvRequest> reqs;  // by request id
  std::deque<int> queue;               // not yet admitted, arrival order
  std::map<int, int> by_tag;           // tag -> request id
  std::deque<qcdgpu_server_result> results;
  std::chrono::steady_clock::time_point t0;
};

namespace qg {

static double now_s(qcdgpu_server S)
{
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - S->t0).count();
}

static size_t field_bytes_f64(const int L[4])
{
  return (size_t)pad_stride((int64_t)L[0] * L[1] * L[2] * L[3]) * 12 * sizeof(double2);
}

// batches of lattices with even extents solve the even/odd system
static bool use_eo(const int L[4]) { return eo_lattice(L); }

// device bytes of a batch of `slots` slots on lattice L (mirrors batch_new)
static size_t batch_bytes_est(const int L[4], int slots)
{
  const bool eo = use_eo(L);
  const int Ls[4] = {eo ? L[0] / 2 : L[0], L[1], L[2], L[3]};
  const int64_t Vs = (int64_t)Ls[0] * Ls[1] * Ls[2] * Ls[3];
  const size_t mf = (size_t)12 * Vs * slots * sizeof(__half2) + (size_t)Vs * slots * sizeof(float);
  const size_t f64 = field_bytes_f64(Ls), f32 = f64 / 2;
  size_t n = 4 * mf + (size_t)12 * Vs * slots * sizeof(float2) + 3 * f64 + field_bytes_f64(L);
  if (eo) {
    n += mf + f64 + 3 * f32 + (size_t)slots * f64;
    // c_e and A^{-1} b_o get their own memory when x cannot hold both
    if (2 * f64 > field_bytes_f64(L)) n += (size_t)2 * slots * f64;
  }
  return n;
}

static void free_request_fields(SrvRequest &r)
{
  for (auto f : r.x) field_free(f);
  for (auto f : r.b) field_free(f);
  r.x.clear();
  r.b.clear();
}

// point-source position of column group k of a request
static void point_position(uint64_t seed, int k, const int L[4], int pos[4])
{
  for (int mu = 0; mu < 4; mu++) {
    uint64_t z = seed * 0x9E3779B97F4A7C15ull + (uint64_t)(k * 4 + mu + 1) * 0xBF58476D1CE4E5B9ull;
    z ^= z >> 31;
    z *= 0x94D049BB133111EBull;
    z ^= z >> 29;
    pos[mu] = (int)(z % (uint64_t)L[mu]);
  }
}

static bool admit(qcdgpu_server S, SrvRequest &r)
{
  SrvGauge &G = S->gauges[(size_t)r.gauge];
  if (!G.batch) {
    G.batch = [&]() {
      qcdgpu_batch b = nullptr;
      const int rc = use_eo(G.g->L) ? qcdgpu_batch_create_eo(&b, G.g, S->slots) : qcdgpu_batch_create(&b, G.g, S->slots);
      return rc == 0 ? b : nullptr;
    }();
    if (!G.batch) return false;
    S->used += qcdgpu_batch_bytes(G.batch);
  }
  for (int c = 0; c < r.nrhs; c++) {
    qcdgpu_field x = field_new(G.g->L, QCDGPU_F64), b = field_new(G.g->L, QCDGPU_F64);
    if (x) r.x.push_back(x);
    if (b) r.b.push_back(b);
    if (!x || !b) return false;
    if (!r.src.empty()) {
      if (!blas_copy(b, r.src[(size_t)c])) return false;
    } else {
      int pos[4];
      point_position(r.seed, c / 12, G.g->L, pos);
      if (!field_point(b, pos, (c % 12) / 3, c % 3)) return false;
    }
  }
  r.src.clear();
  S->used += r.bytes;
  r.admitted = true;
  r.t_admit = now_s(S);
  G.pending.push_back(r.tag);
  return true;
}

static void complete(qcdgpu_server S, SrvRequest &r)
{
  r.complete = true;
  r.t_done = now_s(S);
  qcdgpu_server_result res;
  res.tag = r.tag;
  res.status = r.status;
  res.nrhs = r.nrhs;
  res.max_iters = r.max_iters;
  res.max_true_residual = r.max_res;
  res.queue_s = r.t_admit - r.t_submit;
  res.latency_s = r.t_done - r.t_submit;
  res.total_iters = r.total_iters;
  S->results.push_back(res);
}

// collect the RHS a batch retired; batch tags are request id * 64 + column
static void collect(qcdgpu_server S, SrvGauge &G)
{
  int tags[64], st[64], it[64];
  double tr[64];
  int n;
  while ((n = qcdgpu_batch_poll(G.batch, tags, st, it, tr, 64)) > 0) {
    for (int i = 0; i < n; i++) {
      auto f = S->reqs.find(tags[i] / 64);
      if (f == S->reqs.end()) continue;
      SrvRequest &r = f->second;
      r.retired++;
      if (st[i] > r.status) r.status = st[i];
      if (it[i] > r.max_iters) r.max_iters = it[i];
      r.total_iters += it[i];
      if (tr[i] > r.max_res) r.max_res = tr[i];
      if (r.retired == r.nrhs) complete(S, r);
    }
  }
}

// free slots of G's batch <- right-hand sides of its admitted requests, in
// arrival order; then collect what was solved at admission
static bool fill_slots(qcdgpu_server S, SrvGauge &G)
{
  while (G.batch && !G.pending.empty() && qcdgpu_batch_free_slots(G.batch) > 0) {
    const int id = S->by_tag[G.pending.front()];
    SrvRequest &r = S->reqs[id];
    const int c = r.next_col;
    int k = qcdgpu_batch_add(G.batch, r.x[(size_t)c], r.b[(size_t)c], r.kappa, r.mu, r.op, r.tol, r.maxiter, 0.1,
                             id * 64 + c);
    if (k == -2) return false;
    if (k == -1) break;
    if (++r.next_col == r.nrhs) G.pending.pop_front();
  }
  if (G.batch) collect(S, G);  // right-hand sides solved at admission
  return true;
}

int progress(qcdgpu_server S)
{
  // 1. admission in arrival order
  while (!S->queue.empty()) {
    SrvRequest &r = S->reqs[S->queue.front()];
    SrvGauge &G = S->gauges[(size_t)r.gauge];
    size_t need = r.bytes + (G.batch ? 0 : batch_bytes_est(G.g->L, S->slots));
    if (S->used + need > S->budget) {
      // free the batches of idle gauge fields (no RHS in or waiting for
      // them): they are rebuilt when a request for them is admitted again
      for (SrvGauge &O : S->gauges)
        if (&O != &G && O.batch && O.pending.empty() && qcdgpu_batch_active(O.batch) == 0) {
          collect(S, O);
          S->used -= qcdgpu_batch_bytes(O.batch);
          qcdgpu_batch_destroy(O.batch);
          O.batch = nullptr;
        }
      if (S->used + need > S->budget) break;
    }
    if (!admit(S, r)) {
      free_request_fields(r);
      return 3;
    }
    S->queue.pop_front();
  }
  // 2. slot filling (batches with a chunk running are filled when it ends)
  for (SrvGauge &G : S->gauges) {
    if (!G.batch || batch_in_flight(G.batch)) continue;
    if (!fill_slots(S, G)) return 3;
  }
  // 3. every batch runs on its own stream, independently of the others:
  // an idle batch with work starts a chunk; a batch whose chunk has ended is
  // finished (reliable updates, retirement), refilled and relaunched at
  // once. The call returns when at least one chunk has ended, or at once if
  // none is running, so small lattices' batches are not held to the pace of
  // a large one's chunks.
  for (SrvGauge &G : S->gauges)
    if (G.batch && !batch_in_flight(G.batch) && qcdgpu_batch_active(G.batch) > 0 && !batch_launch(G.batch))
      return 3;
  for (;;) {
    bool running = false, ended = false;
    for (SrvGauge &G : S->gauges) {
      if (!G.batch || !batch_in_flight(G.batch)) continue;
      if (!batch_chunk_done(G.batch)) {
        running = true;
        continue;
      }
      if (!batch_finish(G.batch)) return 3;
      collect(S, G);
      ended = true;
      if (!fill_slots(S, G)) return 3;
      if (qcdgpu_batch_active(G.batch) > 0 && !batch_launch(G.batch)) return 3;
    }
    if (ended || !running) return 0;
    std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

}  // namespace qg

extern "C" {

int qcdgpu_server_create(qcdgpu_server *s, size_t hbm_budget_bytes, int slots)
{
  *s = nullptr;
  if (slots < 1 || slots > 64) {
    qg::set_error("server: 1..64 slots per batch");
    return 1;
  }
  auto *S = new qcdgpu_server_s();
  S->budget = hbm_budget_bytes;
  S->slots = slots;
  S->t0 = std::chrono::steady_clock::now();
  *s = S;
  return 0;
}

int qcdgpu_server_destroy(qcdgpu_server S)
{
  if (!S) return 0;
  for (auto &kv : S->reqs) qg::free_request_fields(kv.second);
  for (auto &G : S->gauges) qcdgpu_batch_destroy(G.batch);
  delete S;
  return 0;
}

int qcdgpu_server_add_gauge(qcdgpu_server S, qcdgpu_gauge g)
{
  if (!S || !g || g->prec != QCDGPU_F64) {
    qg::set_error("server: FP64 gauge field required");
    return -1;
  }
  qg::SrvGauge G;
  G.g = g;
  S->gauges.push_back(G);
  return (int)S->gauges.size() - 1;
}

int qcdgpu_server_submit(qcdgpu_server S, int gauge_id, int nrhs, const qcdgpu_field *sources, uint64_t seed,
                         double kappa, double mu, int op, double tol, int maxiter, int tag)
{
  if (!S || gauge_id < 0 || gauge_id >= (int)S->gauges.size() || nrhs < 1 || nrhs > 64 || !(kappa > 0.0) ||
      !(tol > 0.0) || (op != QCDGPU_OP_D && op != QCDGPU_OP_Q) || S->by_tag.count(tag)) {
    qg::set_error("server submit: bad gauge id, nrhs (1..64), kappa, tol, op, or a tag in use");
    return 1;
  }
  const qcdgpu_gauge g = S->gauges[(size_t)gauge_id].g;
  qg::SrvRequest r;
  r.tag = tag;
  r.gauge = gauge_id;
  r.nrhs = nrhs;
  r.op = op;
  r.seed = seed;
  r.kappa = kappa;
  r.mu = mu;
  r.tol = tol;
  r.maxiter = maxiter;
  r.bytes = (size_t)2 * nrhs * qg::field_bytes_f64(g->L);
  if (sources) {
    for (int c = 0; c < nrhs; c++) {
      qcdgpu_field f = sources[c];
      if (!f || f->prec != QCDGPU_F64 || memcmp(f->L, g->L, sizeof(g->L)) != 0) {
        qg::set_error("server submit: sources must be FP64 fields on the gauge field's lattice");
        return 1;
      }
      r.src.push_back(f);
    }
  }
  if (r.bytes + qg::batch_bytes_est(g->L, S->slots) > S->budget) {
    qg::set_error("server submit: request needs %zu bytes, more than the budget", r.bytes);
    return 1;
  }
  r.t_submit = qg::now_s(S);
  const int id = S->next_id++;
  S->reqs[id] = r;
  S->by_tag[tag] = id;
  S->queue.push_back(id);
  return 0;
}

int qcdgpu_server_progress(qcdgpu_server S) { return S ? qg::progress(S) : 1; }

int qcdgpu_server_poll(qcdgpu_server S, qcdgpu_server_result *out, int max)
{
  int n = 0;
  while (S && n < max && !S->results.empty()) {
    out[n++] = S->results.front();
    S->results.pop_front();
  }
  return n;
}

int qcdgpu_server_fetch(qcdgpu_server S, int tag, int col, qcdgpu_field dst)
{
  auto t = S ? S->by_tag.find(tag) : decltype(S->by_tag.end()){};
  if (!S || t == S->by_tag.end() || !S->reqs[t->second].complete || col < 0 || col >= S->reqs[t->second].nrhs) {
    qg::set_error("server fetch: no completed request with this tag and column");
    return 1;
  }
  return qg::blas_copy(dst, S->reqs[t->second].x[(size_t)col]) ? 0 : 1;
}

int qcdgpu_server_release(qcdgpu_server S, int tag)
{
  auto t = S ? S->by_tag.find(tag) : decltype(S->by_tag.end()){};
  if (!S || t == S->by_tag.end() || !S->reqs[t->second].complete) {
    qg::set_error("server release: no completed request with this tag");
    return 1;
  }
  qg::SrvRequest &r = S->reqs[t->second];
  qg::free_request_fields(r);
  S->used -= r.bytes;
  S->reqs.erase(t->second);
  S->by_tag.erase(t);
  return 0;
}

int qcdgpu_server_stats(qcdgpu_server S, size_t *bytes_used, int *queued, int *active_rhs)
{
  if (!S) return 1;
  *bytes_used = S->used;
  *queued = (int)S->queue.size();
  int a = 0;
  for (auto &G : S->gauges) {
    if (G.batch) a += qcdgpu_batch_active(G.batch);
    for (int tag : G.pending) {  // admitted, waiting for a slot
      const qg::SrvRequest &r = S->reqs[S->by_tag[tag]];
      a += r.nrhs - r.next_col;
    }
  }
  *active_rhs = a;
  return 0;
}

}  // extern "C"
