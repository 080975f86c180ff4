// mc_tune.cpp -- autotuner for the event form's execution parameters.
//
// Bank size, block shape, segments per walk launch, the advance-queue
// ordering granularity, lane refill, CUDA-graph replay and the FP64 walk's
// register budget all move throughput, and their best values depend on the
// mesh, the cross sections and the precision form.
// mc_autotune measures them on trial runs of the context's own problem
// (device time from the CUDA events inside mc_run) by coordinate descent:
// each parameter in turn over its candidate values, the others held at
// their best so far, two passes; a candidate replaces the current value
// only when the best of three trial runs beats it by more than 1%.  A trial is four pipelined batches of a
// quarter of the trial size each, the way production runs stream batches
// through the bank, so that the tail of one batch overlaps the next as it
// will in use.  SUM/SUM_SQ and the batch count are set aside before the
// trials and put back after them; the batch tally is left cleared.
#include <algorithm>
#include <vector>

#include "../../include/macaw_gb300.h"

namespace mc {
int accum_snapshot(mc_ctx* c, int restore);
}

namespace {

double measure(mc_ctx* ctx, const mc_run_desc& d, int reps) {
  double best = 0.0;
  for (int r = 0; r < reps; ++r) {
    if (mc_run(ctx, &d) != MC_OK) return -1.0;
    mc_stats s;
    mc_stats_get(ctx, &s);
    if (s.ms_total > 0.0) best = std::max(best, (double)d.n_histories / (s.ms_total * 1e-3));
  }
  return best;
}

}  // namespace

extern "C" int mc_autotune(mc_ctx* ctx, const mc_run_desc* base, int64_t trial_histories, mc_run_desc* best,
                           double* best_rate) {
  if (!ctx || !base || !best || trial_histories < 1024) return MC_ERR_ARG;
  const int64_t quarter = trial_histories / 4;
  const int64_t sizes[4] = {quarter, quarter, quarter, trial_histories - 3 * quarter};
  mc_run_desc cur = *base;
  cur.n_histories = trial_histories;
  cur.mode = MC_MODE_EVENT;
  cur.accumulate = 1;
  cur.record_traces = 0;
  cur.profile = 0;
  cur.sites = nullptr;
  cur.n_batches = 4;
  cur.batch_sizes = sizes;
  if (cur.bank_size <= 0 || cur.bank_size > trial_histories) cur.bank_size = trial_histories;
  if (cur.block_size <= 0) cur.block_size = 256;
  if (cur.max_seg_per_advance < 0) cur.max_seg_per_advance = 0;
  if (mc::accum_snapshot(ctx, 0) != MC_OK) return MC_ERR_STATE;
  struct Restore {
    mc_ctx* c;
    ~Restore() {
      mc::accum_snapshot(c, 1);
      mc_tally_clear(c, MC_TALLY_BATCH);
    }
  } restore{ctx};
  double rate = measure(ctx, cur, 3);
  if (rate < 0.0) return MC_ERR_STATE;

  struct Knob {
    int kind;
    std::vector<int64_t> values;
  };
  const int64_t t = trial_histories;
  std::vector<Knob> knobs = {
      {0, {0, 16, 32, 48, 64, 96, 128, 256}},                      // segments per walk launch
      {1, {64, 128, 256}},                                         // threads per block
      {2, {0, 1, 5, 9, 13}},                                       // queue ordering granularity
      {3, {std::max<int64_t>(16384, t / 8), std::max<int64_t>(16384, t / 4), std::max<int64_t>(16384, t / 2)}},
      // (bank sizes only when the caller left the bank open)
      {4, {0, 1}},                                                 // lane refill
      {5, {0, 1}},                                                 // CUDA-graph event cycles
      {6, {5, 4}},                                                 // FP64 walk: resident blocks per SM
  };
  auto apply = [](mc_run_desc& d, int kind, int64_t v) {
    switch (kind) {
      case 0: d.max_seg_per_advance = (int32_t)v; break;
      case 1: d.block_size = (int32_t)v; break;
      case 2: d.sort_queue = (int32_t)v; break;
      case 3: d.bank_size = v; break;
      case 4: d.refill = (int32_t)v; break;
      case 5: d.graph = (int32_t)v; break;
      default: d.walk_blocks = (int32_t)v; break;
    }
  };
  for (int pass = 0; pass < 2; ++pass) {
    for (const Knob& k : knobs) {
      if (k.kind == 3 && base->bank_size > 0) continue;
      if (k.kind == 6 && cur.precision != MC_PREC_FP64) continue;
      mc_run_desc keep = cur;
      for (int64_t v : k.values) {
        mc_run_desc trial = keep;
        apply(trial, k.kind, v);
        // best of three repeats, and a change must win by more than 1%:
        // trials are short, and noise must not pick the parameters
        const double r = measure(ctx, trial, 3);
        if (r > rate * 1.01) {
          rate = r;
          cur = trial;
        }
      }
    }
  }
  *best = *base;
  best->mode = MC_MODE_EVENT;
  best->max_seg_per_advance = cur.max_seg_per_advance;
  best->block_size = cur.block_size;
  best->sort_queue = cur.sort_queue;
  best->refill = cur.refill;
  best->graph = cur.graph;
  best->walk_blocks = cur.walk_blocks;
  best->bank_size = base->bank_size > 0 ? base->bank_size : cur.bank_size;
  if (best_rate) *best_rate = rate;
  return MC_OK;
}
