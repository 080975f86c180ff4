// mc_serve.cu -- continuous batching of fixed-source requests on one context.
//
// A context keeps its mesh and cross sections resident; requests (a source,
// a history count, a seed) arrive over time.  Each admitted request owns a
// tally slot and a range of the event pipeline's birth sequence, so the
// particles of every request in flight share the bank: new requests are born
// into bank slots as older ones drain, with no drain between requests.
// Because a request's histories take their random numbers from its own seed
// and local history index, and score only into its own slot, its result is
// the same whether it runs alone or among others (tallies up to FP64
// summation order).
#include <cuda_runtime.h>

#include <algorithm>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/macaw_gb300.h"
#include "mc_ctx_view.h"
#include "mc_kernels.h"

namespace {

using namespace mc;

struct Active {
  int64_t ticket;
  int slot;
  DevRequest dr;
};

struct Serve {
  int max_slots = 0;
  int64_t bank = 0;
  int precision = MC_PREC_MIXED, max_seg = 0;
  double* slots = nullptr;     // max_slots x n_tally tallies
  int* live = nullptr;         // in-flight particles per slot
  DevRequest* table = nullptr; // active requests, sorted by start
  DevRequest* h_table[2] = {nullptr, nullptr};  // pinned staging
  long long* h_limit[2] = {nullptr, nullptr};
  int* h_live = nullptr;
  cudaEvent_t staged[2] = {nullptr, nullptr};
  int stage = 0;
  bool table_dirty = false;
  std::deque<std::pair<int64_t, mc_request>> queue;
  std::vector<Active> active;
  std::vector<int> free_slots;
  std::map<int64_t, std::vector<double>> results;
  int64_t seq_end = 0, next_ticket = 1;
  int par = 0;
  CtxEvent ev;
  CtxView v;
};

std::mutex g_mu;
std::map<mc_ctx*, Serve*> g_serve;

Serve* find(mc_ctx* c) {
  std::lock_guard<std::mutex> g(g_mu);
  auto it = g_serve.find(c);
  return it == g_serve.end() ? nullptr : it->second;
}

void release(Serve* s) {
  if (s->slots) cudaFree(s->slots);
  if (s->live) cudaFree(s->live);
  if (s->table) cudaFree(s->table);
  for (int k = 0; k < 2; ++k) {
    if (s->h_table[k]) cudaFreeHost(s->h_table[k]);
    if (s->h_limit[k]) cudaFreeHost(s->h_limit[k]);
    if (s->staged[k]) cudaEventDestroy(s->staged[k]);
  }
  if (s->h_live) cudaFreeHost(s->h_live);
  delete s;
}

int cuda_fail(mc_ctx* c, cudaError_t e, const char* what) {
  return ctx_fail(c, MC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define SCK(expr, what)                              \
  do {                                               \
    cudaError_t e_ = (expr);                         \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
  } while (0)

RunArgs args(const Serve& s) {
  RunArgs a{};
  a.first = 0;
  a.n = (int64_t)1 << 62;
  a.master = 0;
  a.tally = s.slots;
  a.tally2 = s.slots + s.v.n_tally;
  a.n_tally = s.v.n_tally;
  a.ts = s.v.ts;
  a.req = s.table;
  a.n_req = (int)s.active.size();
  a.live = s.live;
  a.traces = nullptr;
  a.counters = s.ev.counters;
  a.leak_w = s.ev.leak_w;
  a.sites = nullptr;
  a.n_mat = s.v.n_mat;
  a.precision = s.precision;
  a.tol = s.v.tol;
  a.max_seg = s.max_seg;
  a.refill = 0;
  a.two_d = s.v.two_d;
  a.z2d = s.v.z2d;
  a.sort_shift = -1;
  return a;
}

// Active-request table to the device, ordered in the stream after the work
// already queued (pinned staging buffers alternate; each is reused only
// after its previous copy completed).
int upload_table(mc_ctx* c, Serve& s) {
  const int k = s.stage;
  SCK(cudaEventSynchronize(s.staged[k]), "serve staging");
  for (size_t i = 0; i < s.active.size(); ++i) s.h_table[k][i] = s.active[i].dr;
  *s.h_limit[k] = s.seq_end;
  cudaStream_t st = s.v.stream;
  if (!s.active.empty())
    SCK(cudaMemcpyAsync(s.table, s.h_table[k], sizeof(DevRequest) * s.active.size(), cudaMemcpyHostToDevice, st),
        "upload request table");
  SCK(cudaMemcpyAsync(&s.ev.ctl->birth_limit, s.h_limit[k], sizeof(long long), cudaMemcpyHostToDevice, st),
      "upload birth limit");
  SCK(cudaEventRecord(s.staged[k], st), "serve staging");
  s.stage ^= 1;
  s.table_dirty = false;
  return MC_OK;
}

}  // namespace

extern "C" int mc_serve_open(mc_ctx* c, int32_t max_slots, int64_t bank_size, int32_t precision,
                             int32_t max_seg) {
  if (!c) return MC_ERR_ARG;
  if (find(c)) return ctx_fail(c, MC_ERR_STATE, "serving already open on this context");
  if (max_slots < 1 || max_slots > 4096) return ctx_fail(c, MC_ERR_ARG, "max_slots must be in [1, 4096]");
  if (bank_size < 1 || bank_size > ((int64_t)1 << 30)) return ctx_fail(c, MC_ERR_ARG, "bank size out of range");
  if (precision != MC_PREC_FP64 && precision != MC_PREC_MIXED) return ctx_fail(c, MC_ERR_ARG, "unknown precision");
  std::lock_guard<std::mutex> g(ctx_mutex(c));
  int rc = ctx_prepare(c);
  if (rc) return rc;
  Serve* s = new Serve();
  ctx_view(c, &s->v);  // requests bring their own sources; only the tables are needed
  if (!s->v.M.planes || !s->v.X.gE) {
    delete s;
    return ctx_fail(c, MC_ERR_STATE, "mesh and cross sections must be uploaded before serving");
  }
  s->max_slots = max_slots;
  s->bank = bank_size;
  s->precision = precision;
  s->max_seg = max_seg > 0 ? max_seg : 0;
  rc = ctx_event_state(c, bank_size, &s->ev);
  if (rc) {
    delete s;
    return rc;
  }
  auto bad = [&](cudaError_t e, const char* what) {
    release(s);
    return cuda_fail(c, e, what);
  };
  cudaError_t e;
  if ((e = cudaMalloc(&s->slots, sizeof(double) * (size_t)max_slots * (size_t)s->v.n_tally)) != cudaSuccess)
    return bad(e, "allocate request tallies");
  if ((e = cudaMalloc(&s->live, sizeof(int) * (size_t)max_slots)) != cudaSuccess) return bad(e, "allocate slots");
  if ((e = cudaMalloc(&s->table, sizeof(DevRequest) * (size_t)max_slots)) != cudaSuccess)
    return bad(e, "allocate request table");
  for (int k = 0; k < 2; ++k) {
    if ((e = cudaMallocHost(&s->h_table[k], sizeof(DevRequest) * (size_t)max_slots)) != cudaSuccess)
      return bad(e, "allocate staging");
    if ((e = cudaMallocHost(&s->h_limit[k], sizeof(long long))) != cudaSuccess) return bad(e, "allocate staging");
    if ((e = cudaEventCreateWithFlags(&s->staged[k], cudaEventDisableTiming)) != cudaSuccess)
      return bad(e, "create event");
  }
  if ((e = cudaMallocHost(&s->h_live, sizeof(int) * (size_t)max_slots)) != cudaSuccess)
    return bad(e, "allocate staging");
  // every bank slot starts free: the free ring holds them all
  const int64_t cap = s->ev.B.cap;
  std::vector<int> iota((size_t)cap);
  for (int64_t i = 0; i < cap; ++i) iota[i] = (int)i;
  EventCtl h{};
  h.free_head = 0;
  h.free_tail = (unsigned long long)cap;
  cudaStream_t st = s->v.stream;
  if ((e = cudaMemcpyAsync(s->ev.Q.free_slots, iota.data(), sizeof(int) * (size_t)cap, cudaMemcpyHostToDevice, st)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(s->ev.ctl, &h, sizeof(EventCtl), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(s->live, 0, sizeof(int) * (size_t)max_slots, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(s->ev.counters, 0, sizeof(unsigned long long) * kNumCounters, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return bad(e, "initialise serving state");
  for (int k = max_slots - 1; k >= 0; --k) s->free_slots.push_back(k);
  ctx_set_serving(c, true);
  std::lock_guard<std::mutex> g2(g_mu);
  g_serve[c] = s;
  return MC_OK;
}

extern "C" int mc_serve_submit(mc_ctx* c, const mc_request* r, int64_t* ticket) {
  if (!c || !r) return MC_ERR_ARG;
  Serve* s = find(c);
  if (!s) return ctx_fail(c, MC_ERR_STATE, "serving is not open (mc_serve_open)");
  if (r->n_histories < 1) return ctx_fail(c, MC_ERR_ARG, "a request needs at least one history");
  const mc_source_desc& q = r->source;
  if (q.space != MC_SRC_POINT && q.space != MC_SRC_BOX)
    return ctx_fail(c, MC_ERR_ARG, "requests take point or box sources");
  if (q.energy == MC_SRC_MONO && !(q.mono_E >= s->v.X.E_lo && q.mono_E < s->v.X.E_hi))
    return ctx_fail(c, MC_ERR_ARG, "source energy outside the tabulated range");
  if (q.energy == MC_SRC_WATT && (!(q.watt_a > 0.0) || !(q.watt_b > 0.0)))
    return ctx_fail(c, MC_ERR_ARG, "Watt parameters must be positive");
  std::lock_guard<std::mutex> g(ctx_mutex(c));
  const int64_t t = s->next_ticket++;
  s->queue.emplace_back(t, *r);
  if (ticket) *ticket = t;
  return MC_OK;
}

// Admits queued requests into free slots, then launches `iterations`
// event iterations on the context stream (asynchronous).
extern "C" int mc_serve_step(mc_ctx* c, int32_t iterations) {
  if (!c) return MC_ERR_ARG;
  Serve* s = find(c);
  if (!s) return ctx_fail(c, MC_ERR_STATE, "serving is not open (mc_serve_open)");
  std::lock_guard<std::mutex> g(ctx_mutex(c));
  cudaSetDevice(s->v.device);
  cudaStream_t st = s->v.stream;
  while (!s->queue.empty() && !s->free_slots.empty()) {
    const auto qr = s->queue.front();
    s->queue.pop_front();
    const int slot = s->free_slots.back();
    s->free_slots.pop_back();
    SCK(cudaMemsetAsync(s->slots + (size_t)slot * (size_t)s->v.n_tally, 0, sizeof(double) * (size_t)s->v.n_tally, st),
        "clear request tally");
    Active a;
    a.ticket = qr.first;
    a.slot = slot;
    a.dr = DevRequest{};
    a.dr.start = s->seq_end;
    a.dr.end = s->seq_end + qr.second.n_histories;
    a.dr.first_id = 0;
    a.dr.seed = qr.second.seed;
    a.dr.slot = slot;
    a.dr.has_src = 1;
    const mc_source_desc& q = qr.second.source;
    DevSource& d = a.dr.src;
    d = DevSource{};
    d.space = q.space;
    d.energy = q.energy;
    for (int k = 0; k < 3; ++k) {
      d.point[k] = q.point[k];
      d.box_lo[k] = q.box_lo[k];
      d.box_hi[k] = q.box_hi[k];
    }
    d.watt_a = q.watt_a;
    d.watt_b = q.watt_b;
    d.mono_E = q.mono_E;
    s->seq_end = a.dr.end;
    s->active.push_back(a);
    s->table_dirty = true;
  }
  if (s->table_dirty) {
    int rc = upload_table(c, *s);
    if (rc) return rc;
  }
  if (s->active.empty()) return MC_OK;
  const RunArgs a = args(*s);
  const int block = 256;
  const int grid = std::max(1, s->v.n_sm * (2048 / block));
  for (int i = 0; i < iterations; ++i) {
    SCK(launch_event_iteration(s->v.M, s->v.X, s->v.S, a, s->ev.B, s->ev.Q, s->ev.ctl, s->par, block, grid, st,
                               nullptr),
        "launch event iteration");
    s->par ^= 1;
  }
  return MC_OK;
}

// Waits for the launched work, retires finished requests (their FP64
// element tallies are copied out) and lists their tickets.
extern "C" int mc_serve_poll(mc_ctx* c, int64_t* done, int32_t capacity, int32_t* n_done) {
  if (!c || !n_done) return MC_ERR_ARG;
  Serve* s = find(c);
  if (!s) return ctx_fail(c, MC_ERR_STATE, "serving is not open (mc_serve_open)");
  std::lock_guard<std::mutex> g(ctx_mutex(c));
  cudaSetDevice(s->v.device);
  cudaStream_t st = s->v.stream;
  *n_done = 0;
  EventCtl h;
  SCK(cudaMemcpyAsync(&h, s->ev.ctl, sizeof(EventCtl), cudaMemcpyDeviceToHost, st), "read event control");
  SCK(cudaMemcpyAsync(s->h_live, s->live, sizeof(int) * (size_t)s->max_slots, cudaMemcpyDeviceToHost, st),
      "read slots");
  SCK(cudaStreamSynchronize(st), "serve poll");
  std::vector<Active> keep;
  for (const Active& a : s->active) {
    if (h.next_hist >= a.dr.end && s->h_live[a.slot] == 0 && *n_done < capacity) {
      std::vector<double>& out = s->results[a.ticket];
      out.resize((size_t)s->v.n_tally);
      SCK(cudaMemcpy(out.data(), s->slots + (size_t)a.slot * (size_t)s->v.n_tally, sizeof(double) * (size_t)s->v.n_tally,
                     cudaMemcpyDeviceToHost),
          "copy request tally");
      s->free_slots.push_back(a.slot);
      if (done) done[*n_done] = a.ticket;
      ++*n_done;
      s->table_dirty = true;
    } else {
      keep.push_back(a);
    }
  }
  s->active.swap(keep);
  return MC_OK;
}

extern "C" int mc_serve_result(mc_ctx* c, int64_t ticket, double* tally, int64_t n) {
  if (!c || !tally) return MC_ERR_ARG;
  Serve* s = find(c);
  if (!s) return ctx_fail(c, MC_ERR_STATE, "serving is not open (mc_serve_open)");
  std::lock_guard<std::mutex> g(ctx_mutex(c));
  auto it = s->results.find(ticket);
  if (it == s->results.end()) return ctx_fail(c, MC_ERR_ARG, "no finished request with this ticket");
  if (n != (int64_t)it->second.size()) return ctx_fail(c, MC_ERR_ARG, "tally length must equal mc_tally_size");
  std::copy(it->second.begin(), it->second.end(), tally);
  s->results.erase(it);
  return MC_OK;
}

extern "C" int mc_serve_status(mc_ctx* c, int32_t* queued, int32_t* active, int32_t* free_slots) {
  if (!c) return MC_ERR_ARG;
  Serve* s = find(c);
  if (!s) return ctx_fail(c, MC_ERR_STATE, "serving is not open (mc_serve_open)");
  std::lock_guard<std::mutex> g(ctx_mutex(c));
  if (queued) *queued = (int32_t)s->queue.size();
  if (active) *active = (int32_t)s->active.size();
  if (free_slots) *free_slots = (int32_t)s->free_slots.size();
  return MC_OK;
}

extern "C" int mc_serve_close(mc_ctx* c) {
  if (!c) return MC_ERR_ARG;
  Serve* s = nullptr;
  {
    std::lock_guard<std::mutex> g(g_mu);
    auto it = g_serve.find(c);
    if (it == g_serve.end()) return MC_OK;
    s = it->second;
    g_serve.erase(it);
  }
  std::lock_guard<std::mutex> g(ctx_mutex(c));
  cudaSetDevice(s->v.device);
  cudaStreamSynchronize(s->v.stream);
  release(s);
  ctx_set_serving(c, false);
  return MC_OK;
}
