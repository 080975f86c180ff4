// mc_ctx_view.h -- what other translation units may see of a context.
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/macaw_gb300.h"
#include "mc_device.cuh"

namespace mc {

struct CtxView {
  int device = 0, n_sm = 0, n_mat = 0;
  cudaStream_t stream = nullptr;
  int64_t n_tet = 0;
  float tol = 0.0f;
  bool ready = false;  // mesh, tables, block map, BCs and source resident on the device
  DevMesh M;
  DevXS X;
  DevSource S;
};

std::mutex& ctx_mutex(mc_ctx* c);
void ctx_set_error(mc_ctx* c, const std::string& msg);
void ctx_set_stats(mc_ctx* c, const mc_stats& s);
// Fills v; false (with v->ready false) when the device tables are not resident.
bool ctx_view(mc_ctx* c, CtxView* v);

}  // namespace mc
