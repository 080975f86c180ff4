// mc_ctx_view.h -- what other translation units may see of a context.
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/macaw_gb300.h"
#include "mc_device.cuh"
#include "mc_kernels.h"

namespace mc {

struct CtxView {
  int device = 0, n_sm = 0, n_mat = 0;
  cudaStream_t stream = nullptr;
  int64_t n_tet = 0;
  int64_t n_tally = 0;  // values per tally: elements x energy bins x scores
  TallySpec ts{};       // the context's tally definition
  int two_d = 0;        // 2-D mode and its z coordinate
  double z2d = 0.0;
  float tol = 0.0f;
  bool rays_on = false; // ray recording is enabled (mc_rays_enable)
  bool ready = false;  // mesh, tables, block map, BCs and source resident on the device
                       // (M, X and S are filled whenever the tables are resident)
  DevMesh M;
  DevXS X;
  DevSource S;
};

std::mutex& ctx_mutex(mc_ctx* c);
void ctx_set_error(mc_ctx* c, const std::string& msg);
void ctx_set_stats(mc_ctx* c, const mc_stats& s);
// Fills v; false (with v->ready false) when the device tables are not resident.
bool ctx_view(mc_ctx* c, CtxView* v);

// Device event state of a context (bank of at least cap slots, queues,
// control block, counters), allocated on first use.
struct CtxEvent {
  Bank B;
  EventQueues Q;
  EventCtl* ctl;
  unsigned long long* counters;
  double* leak_w;
};
int ctx_prepare(mc_ctx* c);  // puts mesh, tables, block map, BCs on the device
int ctx_event_state(mc_ctx* c, int64_t cap, CtxEvent* out);
int ctx_fail(mc_ctx* c, int code, const std::string& msg);
void ctx_set_serving(mc_ctx* c, bool on);
// The context's SUM and SUM_SQ tallies (false while not allocated), its
// count of folded batches, and whether a serving session holds it.
bool ctx_sums(mc_ctx* c, double** sum, double** sumsq);
void ctx_add_batches(mc_ctx* c, int64_t n);
bool ctx_serving(mc_ctx* c);
// Puts the no-allocation run's fixed scratch array and kernels on the
// current device (once per device; mc_noalloc.cu).  Called at context
// creation so that mc_run_noalloc itself never makes the driver commit
// device memory.
int noalloc_prepare(int device, std::string& err);

}  // namespace mc
