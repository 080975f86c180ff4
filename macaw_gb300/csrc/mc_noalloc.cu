// mc_noalloc.cu -- event-form batch run that allocates no device memory.
//
// mc_run keeps its particle bank, event queues and counters in buffers the
// library cudaMalloc's on first use.  Some callers cannot allow that:
// applications that hand the whole device to their own memory pool (a MOOSE
// run sharing the GPU with other solvers, a serving process that budgets
// HBM up front), and code that runs where a device allocation would stall
// or is forbidden.  mc_run_noalloc tracks the same histories with that
// scratch in one fixed file-scope __device__ array instead, and writes its
// results into buffers the caller owns.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/macaw_gb300.h"
#include "mc_ctx_view.h"
#include "mc_kernels.h"

namespace {

using namespace mc;

constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// Per particle slot: its kBankRec-byte record, its element index and 6
// four-byte queue entries.
constexpr size_t kSlotArrays4 = 1 + 6;
constexpr size_t kScratchBytes =
    align_up((size_t)kBankRec * MC_NOALLOC_MAX_BANK) + kSlotArrays4 * align_up(4 * (size_t)MC_NOALLOC_MAX_BANK) +
    align_up(sizeof(EventCtl)) + align_up(sizeof(unsigned long long) * kNumCounters) +
    align_up(sizeof(double));

// The scratch (220 bytes per particle slot plus the control block and
// counters: about 3.61 MB at 16,384 slots).  It lives in this translation
// unit's module, which the CUDA driver loads onto a device the first time
// host code asks for the array's address; mc_ctx_create does that
// (noalloc_prepare), so every device that has had a context holds these
// bytes until the process exits, and every call on a device shares them.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];
static_assert(kScratchBytes < 4u * 1024u * 1024u, "no-allocation scratch above 4 MB");

// Device address of g_scratch, looked up once per device (the host-side
// name g_scratch is only a stand-in and must never be passed to a kernel).
constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};

int scratch_address(int device, void** out, std::string& err) {
  if (device < 0 || device >= kMaxDevices) {
    err = "device index out of range for the no-allocation scratch table";
    return MC_ERR_ARG;
  }
  std::lock_guard<std::mutex> g(g_setup_mu);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);  // device is current here
    if (e != cudaSuccess || !p) {
      err = std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e);
      return MC_ERR_CUDA;
    }
    g_scratch_addr[device] = p;
  }
  *out = g_scratch_addr[device];
  return MC_OK;
}

}  // namespace

namespace mc {

// Called by mc_ctx_create with `device` current: resolves the scratch
// address (loading this module, and with it the array, onto the device) and
// loads the event-form kernels, once per device.
int noalloc_prepare(int device, std::string& err) {
  void* p = nullptr;
  int rc = scratch_address(device, &p, err);
  if (rc) return rc;
  static bool loaded[kMaxDevices] = {};
  std::lock_guard<std::mutex> g(g_setup_mu);
  if (!loaded[device]) {
    const cudaError_t e = preload_event_kernels();
    if (e != cudaSuccess) {
      err = std::string("load event kernels: ") + cudaGetErrorString(e);
      return MC_ERR_CUDA;
    }
    loaded[device] = true;
  }
  return MC_OK;
}

}  // namespace mc

namespace {

struct Carve {
  unsigned char* p;
  template <class T>
  T* take(size_t count) {
    T* r = (T*)p;
    p += align_up(sizeof(T) * count);
    return r;
  }
};

}  // namespace

extern "C" int mc_run_noalloc(mc_ctx* ctx, const mc_run_desc* d, double* tally, mc_trace* traces) {
  if (!ctx || !d) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(ctx_mutex(ctx));
  CtxView v;
  const bool ok = ctx_view(ctx, &v);
  auto fail = [&](int code, const std::string& m) {
    ctx_set_error(ctx, m);
    return code;
  };
  if (!ok)
    return fail(MC_ERR_STATE,
                "mc_run_noalloc: mesh, tables, block map, boundary conditions and source must already be "
                "on the device (call mc_run once, e.g. with n_histories = 0, after the last change)");
  if (d->n_histories < 0 || d->first_history < 0) return fail(MC_ERR_ARG, "negative history range");
  if (d->mode != MC_MODE_EVENT) return fail(MC_ERR_ARG, "mc_run_noalloc runs the event form only");
  if (d->precision != MC_PREC_FP64 && d->precision != MC_PREC_MIXED)
    return fail(MC_ERR_ARG, "unknown precision form");
  const int64_t cap = d->bank_size > 0 ? d->bank_size : MC_NOALLOC_MAX_BANK;
  if (cap > MC_NOALLOC_MAX_BANK)
    return fail(MC_ERR_ARG, "mc_run_noalloc: bank_size " + std::to_string(d->bank_size) +
                                " exceeds the no-allocation maximum of " +
                                std::to_string(MC_NOALLOC_MAX_BANK) + " particles");
  if (d->sites) return fail(MC_ERR_ARG, "mc_run_noalloc: host source sites would need a device copy");
  if (d->accumulate) return fail(MC_ERR_ARG, "mc_run_noalloc: accumulate uses the context's tallies");
  if (d->profile) return fail(MC_ERR_ARG, "mc_run_noalloc: profiling creates events");
  // what mc_run would honour but this form cannot: reject rather than drop
  if (d->n_batches > 1 || d->batch_sizes || d->batch_sum_out)
    return fail(MC_ERR_ARG, "mc_run_noalloc: pipelined batches need per-batch tally slots; run one batch per call");
  if (d->sort_queue > 0)
    return fail(MC_ERR_ARG, "mc_run_noalloc: ordering the advance queue needs scratch beyond the fixed array");
  if (d->graph) return fail(MC_ERR_ARG, "mc_run_noalloc: instantiating a CUDA graph allocates");
  if (v.rays_on) return fail(MC_ERR_ARG, "mc_run_noalloc: ray recording is on (mc_rays_enable); turn it off");
  if (!tally) return fail(MC_ERR_ARG, "mc_run_noalloc: null tally buffer");
  if (d->record_traces && !traces) return fail(MC_ERR_ARG, "mc_run_noalloc: null trace buffer");
  const int block = d->block_size > 0 ? d->block_size : 256;
  if (block % 32 != 0 || block > 256)
    return fail(MC_ERR_ARG, "block size must be a multiple of 32, at most 256");
  if (d->walk_blocks != 0 && d->walk_blocks != 4 && d->walk_blocks != 5)
    return fail(MC_ERR_ARG, "walk_blocks must be 0, 4 or 5");

  cudaError_t e = cudaSetDevice(v.device);
  if (e != cudaSuccess) return fail(MC_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  void* base = nullptr;
  std::string err;
  int rc = scratch_address(v.device, &base, err);
  if (rc) return fail(rc, err);

  Carve cv{(unsigned char*)base};
  const size_t n = (size_t)cap;
  unsigned char* rec = cv.take<unsigned char>(n * (size_t)kBankRec);
  Bank B = bank_at(rec, cv.take<int>(n), cap);
  if (!bank_complete(B)) return fail(MC_ERR_STATE, "internal: particle bank incomplete");
  EventQueues Q{};
  Q.xs[0] = cv.take<int>(n); Q.xs[1] = cv.take<int>(n);
  Q.adv[0] = cv.take<int>(n); Q.adv[1] = cv.take<int>(n);
  Q.coll = cv.take<int>(n); Q.free_slots = cv.take<int>(n);
  EventCtl* ctl = cv.take<EventCtl>(1);
  unsigned long long* counters = cv.take<unsigned long long>(kNumCounters);
  double* leak_w = cv.take<double>(1);

  // the array keeps the previous call's contents: counters start at zero
  // here, the control block is cleared by the first launch
  cudaStream_t st = v.stream;
  e = cudaMemsetAsync(counters, 0, sizeof(unsigned long long) * kNumCounters, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(leak_w, 0, sizeof(double), st);
  if (e != cudaSuccess) return fail(MC_ERR_CUDA, std::string("clear scratch: ") + cudaGetErrorString(e));

  RunArgs a{};
  a.first = d->first_history;
  a.n = d->n_histories;
  a.master = d->seed;
  a.tally = tally;
  a.tally2 = tally;
  a.req = nullptr;
  a.n_req = 0;
  a.n_tally = v.n_tally;
  a.ts = v.ts;
  a.live = nullptr;
  a.traces = d->record_traces ? traces : nullptr;
  a.counters = counters;
  a.leak_w = leak_w;
  a.sites = nullptr;
  a.n_mat = v.n_mat;
  a.precision = d->precision;
  a.tol = v.tol;
  a.max_seg = d->max_seg_per_advance;
  a.refill = d->refill;
  a.walk_blocks = d->walk_blocks;
  a.two_d = v.two_d;
  a.z2d = v.z2d;
  a.sort_shift = -1;  // ordering needs scratch beyond the fixed array
  a.sort_buckets = 0;
  a.sort_tmp = nullptr;
  a.sort_cnt = nullptr;
  const int grid = std::max(1, v.n_sm * (2048 / block));
  int n_launch = 0;
  if (d->n_histories > 0) {
    e = launch_event_init(v.M, v.X, v.S, a, B, Q, ctl, block, grid, st, a.n);
    if (e != cudaSuccess) return fail(MC_ERR_CUDA, std::string("event init: ") + cudaGetErrorString(e));
    n_launch = 1;
    int par = 0;
    EventCtl h;
    const int64_t tail = d->tail > 0 ? (int64_t)d->tail : d->tail < 0 ? -1 : std::max<int64_t>(1024, cap / tail_divisor(a));
    for (int64_t it = 0;; ++it) {
      for (int gi = 0; gi < 4; ++gi) {
        e = launch_event_iteration(v.M, v.X, v.S, a, B, Q, ctl, par, block, grid, st, &n_launch);
        if (e != cudaSuccess) return fail(MC_ERR_CUDA, std::string("event iteration: ") + cudaGetErrorString(e));
        par ^= 1;
      }
      e = cudaMemcpyAsync(&h, ctl, sizeof(EventCtl), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) return fail(MC_ERR_CUDA, std::string("event loop: ") + cudaGetErrorString(e));
      const int64_t inflight = (int64_t)h.n_xs[par] + h.n_adv[par];
      if (inflight == 0 && h.next_hist >= a.n) break;
      if (h.next_hist >= a.n && inflight <= tail) {
        // a few particles per warp, spread over every SM (as mc_run does)
        e = launch_event_finish(v.M, v.X, v.S, a, B, Q, ctl, par, tail_block(a.precision),
                                (int)std::max<int64_t>(1, (inflight + tail_block(a.precision) - 1) /
                                                              tail_block(a.precision)),
                                st);
        if (e != cudaSuccess) return fail(MC_ERR_CUDA, std::string("event finish: ") + cudaGetErrorString(e));
        ++n_launch;
        break;
      }
      if (it > 100000000) return fail(MC_ERR_DEVICE, "event loop did not terminate");
    }
  }
  unsigned long long cnt[kNumCounters];
  double lw = 0.0;
  e = cudaMemcpyAsync(cnt, counters, sizeof cnt, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&lw, leak_w, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(MC_ERR_CUDA, std::string("read counters: ") + cudaGetErrorString(e));
  mc_stats s{};
  s.n_hist = (int64_t)cnt[kCntHist];
  s.n_seg = (int64_t)cnt[kCntSeg];
  s.n_seg_advance = (int64_t)cnt[kCntSegWalk];
  s.n_coll = (int64_t)cnt[kCntColl];
  s.n_leak = (int64_t)cnt[kCntLeak];
  s.n_absorb = (int64_t)cnt[kCntAbsorb];
  s.n_cutoff = (int64_t)cnt[kCntCutoff];
  s.n_stuck = (int64_t)cnt[kCntStuck];
  s.n_lost = (int64_t)cnt[kCntLost];
  s.n_badxs = (int64_t)cnt[kCntBadXS];
  s.n_fallback = (int64_t)cnt[kCntFallback];
  s.n_xs = (int64_t)cnt[kCntXS];
  s.n_launch = n_launch;
  s.leak_weight = lw;
  ctx_set_stats(ctx, s);
  if (s.n_hist != d->n_histories)
    return fail(MC_ERR_DEVICE, "device finished " + std::to_string(s.n_hist) + " of " +
                                   std::to_string(d->n_histories) + " histories");
  return MC_OK;
}
