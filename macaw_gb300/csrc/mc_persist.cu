// mc_persist.cu -- many batches, of one or more problems, in one kernel launch.
//
// mc_run streams pipelined batches through a cycle of event launches that
// the host drives.  mc_run_persistent instead launches one persistent
// kernel (k_persist, mc_kernels.cu) over a table of batches: every lane
// takes the next history of the run, tracks it with its batch's problem
// (mesh, cross sections, source, tally definition) and, when it ends a
// batch's last history, makes that batch's tally available for folding into
// its problem's SUM/SUM_SQ.  Each problem's batches take a fixed number of
// tally slots in turn; a history whose batch's slot is still being folded
// waits, folding meanwhile, and gives up after wait_limit polls.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/macaw_gb300.h"
#include "mc_ctx_view.h"
#include "mc_kernels.h"

using namespace mc;

namespace {

constexpr int kFoldChunk = 4096;               // tally values per fold chunk
constexpr long long kDefaultWaitLimit = 10000000;  // polls, about a microsecond apart

struct Dev {
  void* p = nullptr;
  ~Dev() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t n) { return cudaMalloc(&p, n < 16 ? 16 : n); }
  template <class T>
  T* as() const {
    return (T*)p;
  }
};

}  // namespace

extern "C" int mc_run_persistent(const mc_persist_desc* d, int32_t n_jobs, const mc_job* jobs, mc_stats* stats) {
  if (!d || !jobs || n_jobs < 1) return MC_ERR_ARG;
  mc_ctx* c0 = jobs[0].ctx;
  if (!c0) return MC_ERR_ARG;
  // the problems of the run, in order of first appearance; their locks are
  // taken in address order
  std::vector<mc_ctx*> probs;
  std::map<mc_ctx*, int> index;
  for (int j = 0; j < n_jobs; ++j) {
    if (!jobs[j].ctx) return MC_ERR_ARG;
    if (!index.count(jobs[j].ctx)) {
      index[jobs[j].ctx] = (int)probs.size();
      probs.push_back(jobs[j].ctx);
    }
  }
  std::vector<mc_ctx*> order(probs);
  std::sort(order.begin(), order.end());
  std::vector<std::unique_lock<std::mutex>> locks;
  for (mc_ctx* c : order) locks.emplace_back(ctx_mutex(c));
  auto fail = [&](int code, const std::string& m) {
    for (mc_ctx* c : probs) ctx_set_error(c, "mc_run_persistent: " + m);
    return code;
  };
  if ((int)probs.size() > kMaxPersistProblems)
    return fail(MC_ERR_ARG, "at most " + std::to_string(kMaxPersistProblems) + " problems per run");
  if (d->precision != MC_PREC_FP64 && d->precision != MC_PREC_MIXED) return fail(MC_ERR_ARG, "unknown precision form");
  const int block = d->block_size > 0 ? d->block_size : 128;
  if (block % 32 != 0 || block > 128) return fail(MC_ERR_ARG, "block size must be a multiple of 32, at most 128");
  if (d->slots < 0) return fail(MC_ERR_ARG, "negative slot count");
  if (d->record_traces && !d->traces) return fail(MC_ERR_ARG, "record_traces without a trace buffer");

  // problem views and per-problem batch counts
  std::vector<CtxView> views(probs.size());
  std::vector<int> jobs_of(probs.size(), 0);
  for (size_t i = 0; i < probs.size(); ++i) {
    if (!ctx_view(probs[i], &views[i]))
      return fail(MC_ERR_STATE, "every problem's mesh, tables, block map, boundary conditions and source must be on "
                                "the device (call mc_run once after the last set-up call)");
    if (ctx_serving(probs[i])) return fail(MC_ERR_STATE, "a serving session holds one of the problems");
    if (views[i].device != views[0].device) return fail(MC_ERR_ARG, "every problem must be on the same device");
    double *s, *q;
    if (!ctx_sums(probs[i], &s, &q)) return fail(MC_ERR_STATE, "a problem has no tallies");
  }
  unsigned long long total = 0;
  std::vector<PersistJob> J(n_jobs);
  for (int j = 0; j < n_jobs; ++j) {
    if (jobs[j].n_histories < 1 || jobs[j].first_history < 0) return fail(MC_ERR_ARG, "empty or negative batch");
    const int p = index[jobs[j].ctx];
    J[j].start = (int64_t)total;
    J[j].end = (int64_t)(total + (unsigned long long)jobs[j].n_histories);
    J[j].first = jobs[j].first_history;
    J[j].seed = jobs[j].seed;
    J[j].inv_n = 1.0 / (double)jobs[j].n_histories;
    J[j].prob = p;
    J[j].order = jobs_of[p]++;
    total += (unsigned long long)jobs[j].n_histories;
  }

  cudaError_t e = cudaSetDevice(views[0].device);
  if (e != cudaSuccess) return fail(MC_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  cudaStream_t st = views[0].stream;
  for (size_t i = 0; i < probs.size(); ++i) {
    // earlier work of the other problems' contexts lands first
    if (views[i].stream != st) {
      e = cudaStreamSynchronize(views[i].stream);
      if (e != cudaSuccess) return fail(MC_ERR_CUDA, std::string("synchronize: ") + cudaGetErrorString(e));
    }
  }

  // device tables
  std::vector<std::unique_ptr<Dev>> slot_mem;
  std::vector<PersistProblem> P(probs.size());
  std::vector<int> slot_base(probs.size()), turn;
  bool fold_in_run = false;  // the batches of some problem share tally slots
  for (size_t i = 0; i < probs.size(); ++i) {
    const CtxView& v = views[i];
    PersistProblem& q = P[i];
    q.M = v.M;
    q.X = v.X;
    q.S = v.S;
    q.ts = v.ts;
    q.ts.rays = nullptr;  // ray segments are recorded by mc_run only
    q.n_tally = v.n_tally;
    q.n_slots = d->slots > 0 ? std::min(d->slots, jobs_of[i]) : jobs_of[i];
    if (q.n_slots < jobs_of[i]) fold_in_run = true;
    q.two_d = v.two_d;
    q.z2d = v.z2d;
    q.tol = v.tol;
    q.n_chunks = (int)((v.n_tally + kFoldChunk - 1) / kFoldChunk);
    ctx_sums(probs[i], &q.sum, &q.sumsq);
    slot_mem.emplace_back(new Dev());
    const size_t bytes = sizeof(double) * (size_t)q.n_slots * (size_t)q.n_tally;
    e = slot_mem.back()->alloc(bytes);
    if (e != cudaSuccess) return fail(MC_ERR_NOMEM, "tally slots (" + std::to_string(bytes >> 20) + " MiB): " +
                                                        cudaGetErrorString(e) + "; ask for fewer slots");
    q.slots = slot_mem.back()->as<double>();
    e = cudaMemsetAsync(q.slots, 0, bytes, st);
    if (e != cudaSuccess) return fail(MC_ERR_CUDA, std::string("clear slots: ") + cudaGetErrorString(e));
    slot_base[i] = (int)turn.size();
    for (int k = 0; k < q.n_slots; ++k) turn.push_back(k);  // the problem's k-th batch takes slot k first
  }
  std::vector<int> live(n_jobs);
  for (int j = 0; j < n_jobs; ++j) live[j] = (int)jobs[j].n_histories;
  for (int j = 0; j < n_jobs; ++j)
    if (jobs[j].n_histories > 0x7fffffff) return fail(MC_ERR_ARG, "a batch of more than 2^31 - 1 histories");
  Dev d_probs, d_jobs, d_live, d_next, d_done, d_ready, d_turn, d_base, d_ctl, d_cnt, d_traces;
  const size_t nj = (size_t)n_jobs;
  if ((e = d_probs.alloc(sizeof(PersistProblem) * P.size())) != cudaSuccess ||
      (e = d_jobs.alloc(sizeof(PersistJob) * nj)) != cudaSuccess || (e = d_live.alloc(sizeof(int) * nj)) != cudaSuccess ||
      (e = d_next.alloc(sizeof(int) * nj)) != cudaSuccess || (e = d_done.alloc(sizeof(int) * nj)) != cudaSuccess ||
      (e = d_ready.alloc(sizeof(int) * nj)) != cudaSuccess || (e = d_turn.alloc(sizeof(int) * turn.size())) != cudaSuccess ||
      (e = d_base.alloc(sizeof(int) * P.size())) != cudaSuccess || (e = d_ctl.alloc(sizeof(PersistCtl))) != cudaSuccess ||
      (e = d_cnt.alloc(sizeof(unsigned long long) * kNumCounters + sizeof(double))) != cudaSuccess ||
      (d->record_traces && (e = d_traces.alloc(sizeof(mc_trace) * (size_t)total)) != cudaSuccess))
    return fail(MC_ERR_NOMEM, std::string("run tables: ") + cudaGetErrorString(e));
  std::vector<int> minus1(nj, -1);
  if ((e = cudaMemcpyAsync(d_probs.p, P.data(), sizeof(PersistProblem) * P.size(), cudaMemcpyHostToDevice, st)) ||
      (e = cudaMemcpyAsync(d_jobs.p, J.data(), sizeof(PersistJob) * nj, cudaMemcpyHostToDevice, st)) ||
      (e = cudaMemcpyAsync(d_live.p, live.data(), sizeof(int) * nj, cudaMemcpyHostToDevice, st)) ||
      (e = cudaMemsetAsync(d_next.p, 0, sizeof(int) * nj, st)) || (e = cudaMemsetAsync(d_done.p, 0, sizeof(int) * nj, st)) ||
      (e = cudaMemcpyAsync(d_ready.p, minus1.data(), sizeof(int) * nj, cudaMemcpyHostToDevice, st)) ||
      (e = cudaMemcpyAsync(d_turn.p, turn.data(), sizeof(int) * turn.size(), cudaMemcpyHostToDevice, st)) ||
      (e = cudaMemcpyAsync(d_base.p, slot_base.data(), sizeof(int) * P.size(), cudaMemcpyHostToDevice, st)) ||
      (e = cudaMemsetAsync(d_ctl.p, 0, sizeof(PersistCtl), st)) ||
      (e = cudaMemsetAsync(d_cnt.p, 0, sizeof(unsigned long long) * kNumCounters + sizeof(double), st)))
    return fail(MC_ERR_CUDA, std::string("upload run tables: ") + cudaGetErrorString(e));

  PersistArgs a{};
  a.probs = d_probs.as<PersistProblem>();
  a.n_probs = (int)P.size();
  a.n_jobs = n_jobs;
  a.jobs = d_jobs.as<PersistJob>();
  a.total = total;
  a.live = d_live.as<int>();
  a.chunk_next = d_next.as<int>();
  a.chunk_done = d_done.as<int>();
  a.ready_list = d_ready.as<int>();
  a.slot_turn = d_turn.as<int>();
  a.slot_base = d_base.as<int>();
  a.chunk = kFoldChunk;
  a.ctl = d_ctl.as<PersistCtl>();
  a.traces = d->record_traces ? d_traces.as<mc_trace>() : nullptr;
  a.counters = d_cnt.as<unsigned long long>();
  a.leak_w = (double*)(a.counters + kNumCounters);
  a.wait_limit = d->wait_limit > 0 ? d->wait_limit : kDefaultWaitLimit;
  // with a slot per batch nothing waits for a fold: k_persist_fold_rest
  // folds every batch after the run (10M histories of the 41M-tet core:
  // FP64 1.90 s against 2.11 s with lanes folding during the run, mixed
  // 1.52 s against 1.76-1.92 s)
  a.fold_in_run = fold_in_run ? 1 : 0;

  const int grid = views[0].n_sm * persistent_blocks_per_sm(d->precision, block);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, st);
  e = launch_persistent(a, d->precision, block, grid, st);
  cudaEventRecord(e1, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  float ms = 0.0f;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return fail(MC_ERR_CUDA, std::string("persistent kernel: ") + cudaGetErrorString(e));

  PersistCtl h;
  unsigned long long cnt[kNumCounters];
  double lw = 0.0;
  if ((e = cudaMemcpy(&h, d_ctl.p, sizeof h, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(cnt, d_cnt.p, sizeof cnt, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(&lw, a.leak_w, sizeof(double), cudaMemcpyDeviceToHost)))
    return fail(MC_ERR_CUDA, std::string("read run state: ") + cudaGetErrorString(e));
  mc_stats s{};
  s.n_hist = (int64_t)cnt[kCntHist];
  s.n_seg = (int64_t)cnt[kCntSeg];
  s.n_coll = (int64_t)cnt[kCntColl];
  s.n_leak = (int64_t)cnt[kCntLeak];
  s.n_absorb = (int64_t)cnt[kCntAbsorb];
  s.n_cutoff = (int64_t)cnt[kCntCutoff];
  s.n_stuck = (int64_t)cnt[kCntStuck];
  s.n_lost = (int64_t)cnt[kCntLost];
  s.n_badxs = (int64_t)cnt[kCntBadXS];
  s.n_fallback = (int64_t)cnt[kCntFallback];
  s.n_xs = (int64_t)cnt[kCntXS];
  s.n_launch = 2;
  s.leak_weight = lw;
  s.ms_total = ms;
  for (mc_ctx* c : probs) ctx_set_stats(c, s);
  if (stats) *stats = s;
  if (h.error)
    return fail(MC_ERR_DEVICE, "a history of batch " + std::to_string(h.err_job) + " waited " +
                                   std::to_string(h.err_polls) + " polls for its tally slot (wait_limit " +
                                   std::to_string(a.wait_limit) + ") and the run stopped; the problems' SUM/SUM_SQ "
                                   "hold the batches folded before that (mc_tally_reset clears them)");
  if (s.n_hist != (int64_t)total)
    return fail(MC_ERR_DEVICE, "device finished " + std::to_string(s.n_hist) + " of " + std::to_string(total) +
                                   " histories");
  for (size_t i = 0; i < probs.size(); ++i) ctx_add_batches(probs[i], jobs_of[i]);
  if (d->record_traces) {
    e = cudaMemcpy(d->traces, d_traces.p, sizeof(mc_trace) * (size_t)total, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(MC_ERR_CUDA, std::string("read traces: ") + cudaGetErrorString(e));
  }
  return MC_OK;
}
