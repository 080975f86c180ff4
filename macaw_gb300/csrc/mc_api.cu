// mc_api.cu -- context, uploads, run loop and readback behind the C ABI.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/macaw_gb300.h"
#include "mc_host.h"
#include "mc_ctx_view.h"
#include "mc_kernels.h"

using namespace mc;

namespace {

// Owning device allocation.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t alloc(size_t n) {
    if (n == bytes && p) return cudaSuccess;
    release();
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    else p = nullptr;
    return e;
  }
  template <class T>
  T* as() const {
    return (T*)p;
  }
};

}  // namespace

struct mc_ctx {
  int device = 0;
  int n_sm = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // host source sites of later batches
  std::vector<cudaEvent_t> prof_ev;
  std::vector<cudaEvent_t> site_ev;  // batch b's sites are on the device
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_a0 = nullptr, ev_a1 = nullptr;
  std::mutex mu;
  std::string err;

  // host model
  MeshTables mesh;
  bool have_mesh = false;
  std::vector<int32_t> bc_type = std::vector<int32_t>(1024, MC_BC_VACUUM);
  std::vector<Nuclide> nucs;
  std::vector<Material> mats;
  std::vector<int32_t> map_blocks, map_mats;
  int32_t n_bins = 8000;
  XSTables xs;
  bool xs_dirty = true, tmat_dirty = true, bc_dirty = true;
  mc_source_desc src{};
  std::vector<double> src_cyl;
  bool have_src = false;

  // device copies
  DevBuf d_planes, d_tet, d_teto, d_tmat, d_bc, d_gstart, d_gtets, d_gseed;
  DevBuf d_gE, d_goff, d_gn, d_ghidx, d_nuc_grid, d_nuc_off, d_sig, d_awr, d_mat_off, d_mat_nuc, d_mat_dens;
  DevBuf d_nusf, d_nuc_fiss, d_mat_fiss;
  DevBuf d_cyl;
  DevBuf d_tally, d_sum, d_sumsq;
  DevBuf d_counters, d_leak_w;
  DevBuf d_traces;
  int64_t trace_n = 0;
  DevBuf d_sites;
  DevBuf d_tally2, d_batch_end, d_live;
  DevBuf d_accum_save;  // SUM and SUM_SQ kept aside while the autotuner runs pipelined trials
  int64_t batches_save = 0;
  DevBuf d_sort_tmp, d_sort_cnt;
  bool tally2_clear = false;  // d_tally2 is all zeros between runs
  // tally definition (mc_tally_configure); the default scores the
  // track-length flux, one value per element
  TallySpec tspec{};           // device view (edges point into d_edges)
  DevBuf d_edges;
  int64_t n_tally = 0;         // values per tally: elements x energy bins x scores
  // recorded ray segments (mc_rays_enable): ray_n rays of ray_cap segments
  DevBuf d_rays;
  // 2-D mode (mc_set_2d)
  int two_d = 0;
  double z2d = 0.0;
  // largest L1 error of an octahedral record's decoded unit normal
  double oct_err = 0.0;
  // segments a history may walk before it ends as stuck (mc_set_segment_limit;
  // 0: default_segment_limit of the mesh)
  int64_t seg_limit = 0;
  int32_t ray_n = 0, ray_cap = 0;
  int64_t ray_first = 0;       // first_history of the last run that recorded
  long long h_limit = 0;
  // event bank
  DevBuf b_rec, b_elem;                // particle records (kBankRec bytes a slot), element indices
  DevBuf b_nuf, b_ktl, b_cn, b_nprog;  // k-eigenvalue runs only
  // k-eigenvalue state (mc_eigen_run): source sites of the next generation,
  // the last generation's fission bank (append order, then sorted),
  // per-history estimator sums and site counts, scan scratch
  DevBuf e_src, e_bank, e_sorted, e_ktl, e_kcol, e_kabs, e_prog, e_off, e_cnt, e_pos, e_tmp, e_part, e_nbank;
  int64_t e_n = 0;      // sites in e_src
  int64_t e_m = 0;      // sites in e_sorted
  DevBuf q_xs0, q_xs1, q_adv0, q_adv1, q_coll, q_free, d_ctl;
  int64_t bank_cap = 0;

  int64_t batches = 0;
  mc_stats last{};
  bool serving = false;  // the event state belongs to an open serving session
};

namespace {

int run_locked(mc_ctx* c, const mc_run_desc* d, const mc_site* dev_sites, const EigArgs* eig);

int set_err(mc_ctx* c, int code, const std::string& msg) {
  c->err = msg;
  return code;
}

int cuda_err(mc_ctx* c, cudaError_t e, const char* what) {
  c->err = std::string(what) + ": " + cudaGetErrorString(e);
  return MC_ERR_CUDA;
}

template <class T>
cudaError_t upload(DevBuf& b, const std::vector<T>& v, cudaStream_t st) {
  cudaError_t e = b.alloc(std::max<size_t>(16, v.size() * sizeof(T)));
  if (e != cudaSuccess) return e;
  if (v.empty()) return cudaSuccess;
  return cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
}

#define CK(expr, what)                      \
  do {                                      \
    cudaError_t e_ = (expr);                \
    if (e_ != cudaSuccess) return cuda_err(c, e_, what); \
  } while (0)

int ensure_device_tables(mc_ctx* c) {
  if (!c->have_mesh) return set_err(c, MC_ERR_STATE, "no mesh uploaded (mc_mesh_upload)");
  if (c->nucs.empty()) return set_err(c, MC_ERR_STATE, "no nuclides (mc_nuclide_add)");
  if (c->mats.empty()) return set_err(c, MC_ERR_STATE, "no materials (mc_material_add)");
  if (c->xs_dirty) {
    std::string m = build_xs_tables(c->nucs, c->mats, c->n_bins, c->xs);
    if (!m.empty()) return set_err(c, MC_ERR_ARG, m);
    CK(upload(c->d_gE, c->xs.gE, c->stream), "upload xs grids");
    CK(upload(c->d_goff, c->xs.g_off, c->stream), "upload xs grids");
    CK(upload(c->d_gn, c->xs.g_n, c->stream), "upload xs grids");
    CK(upload(c->d_ghidx, c->xs.ghidx, c->stream), "upload xs hash index");
    CK(upload(c->d_nuc_grid, c->xs.nuc_grid, c->stream), "upload xs grid map");
    CK(upload(c->d_nuc_off, c->xs.nuc_off, c->stream), "upload xs offsets");
    CK(upload(c->d_sig, c->xs.sig, c->stream), "upload xs values");
    CK(upload(c->d_awr, c->xs.awr, c->stream), "upload awr");
    CK(upload(c->d_mat_off, c->xs.mat_off, c->stream), "upload materials");
    CK(upload(c->d_mat_nuc, c->xs.mat_nuc, c->stream), "upload materials");
    CK(upload(c->d_mat_dens, c->xs.mat_dens, c->stream), "upload materials");
    CK(upload(c->d_nusf, c->xs.nusf, c->stream), "upload fission data");
    CK(upload(c->d_nuc_fiss, c->xs.nuc_fiss, c->stream), "upload fission data");
    CK(upload(c->d_mat_fiss, c->xs.mat_fiss, c->stream), "upload fission data");
    c->xs_dirty = false;
    c->tmat_dirty = true;
  }
  if (c->tmat_dirty) {
    // element -> material index via the block map (material id, then the
    // index of that id among the uploaded materials)
    std::vector<int32_t> tmat((size_t)c->mesh.n_tet, -1);
    for (int64_t t = 0; t < c->mesh.n_tet; ++t) {
      const int32_t blk = c->mesh.block[t];
      for (size_t i = 0; i < c->map_blocks.size(); ++i)
        if (c->map_blocks[i] == blk) {
          for (size_t m = 0; m < c->xs.mat_ids.size(); ++m)
            if (c->xs.mat_ids[m] == c->map_mats[i]) {
              tmat[t] = (int32_t)m;
              break;
            }
          break;
        }
    }
    CK(upload(c->d_tmat, tmat, c->stream), "upload element materials");
    // packed float record per tet: planes, and neighbour entries flagged
    // where the material changes across the side
    std::vector<Tet32> rec((size_t)c->mesh.n_tet);
    for (int64_t t = 0; t < c->mesh.n_tet; ++t) {
      Tet32& r = rec[t];
      const float* q = &c->mesh.planes32[16 * t];
      r.p[0] = make_float4(q[0], q[1], q[2], q[3]);
      r.p[1] = make_float4(q[4], q[5], q[6], q[7]);
      r.p[2] = make_float4(q[8], q[9], q[10], q[11]);
      r.p[3] = make_float4(q[12], q[13], q[14], q[15]);
      int e[4];
      for (int f = 0; f < 4; ++f) {
        e[f] = c->mesh.nbr[4 * t + f];
        if (e[f] >= 0 && tmat[(size_t)(e[f] >> 2)] != tmat[t]) e[f] |= kMatChange;
      }
      r.nbr = make_int4(e[0], e[1], e[2], e[3]);
    }
    CK(upload(c->d_tet, rec, c->stream), "upload tet records");
    // octahedral records: the FP64 unit normal n -> (a, b) = n.xy / |n|_1,
    // folded over the lower half (z < 0), rounded to float; the offset is
    // scaled by the length of the normal the walk decodes from (a, b)
    std::vector<TetOct> oct((size_t)c->mesh.n_tet);
    double oct_err = 0.0;
    for (int64_t t = 0; t < c->mesh.n_tet; ++t) {
      float ab[8], dd[4];
      for (int f = 0; f < 4; ++f) {
        const double* q = &c->mesh.planes[16 * t + 4 * f];
        const double l1 = fabs(q[0]) + fabs(q[1]) + fabs(q[2]);
        double a = q[0] / l1, b = q[1] / l1;
        if (q[2] < 0.0) {
          const double fa = (1.0 - fabs(b)) * (a >= 0.0 ? 1.0 : -1.0);
          const double fb = (1.0 - fabs(a)) * (b >= 0.0 ? 1.0 : -1.0);
          a = fa;
          b = fb;
        }
        // of the float pairs next to (a, b), the one whose decoded normal
        // points closest to n
        const float a0 = (float)a, b0 = (float)b;
        float best_a = a0, best_b = b0;
        double best = -2.0;
        for (int i = -1; i <= 1; ++i)
          for (int j = -1; j <= 1; ++j) {
            const float ca = i < 0 ? nextafterf(a0, -2.0f) : i > 0 ? nextafterf(a0, 2.0f) : a0;
            const float cb = j < 0 ? nextafterf(b0, -2.0f) : j > 0 ? nextafterf(b0, 2.0f) : b0;
            float x, y, z;
            oct_normal(ca, cb, x, y, z);
            const double l = sqrt((double)x * x + (double)y * y + (double)z * z);
            const double cosang = ((double)x * q[0] + (double)y * q[1] + (double)z * q[2]) / l;
            if (cosang > best) {
              best = cosang;
              best_a = ca;
              best_b = cb;
            }
          }
        ab[2 * f] = best_a;
        ab[2 * f + 1] = best_b;
        float nx, ny, nz;
        oct_normal(best_a, best_b, nx, ny, nz);
        const double len = sqrt((double)nx * nx + (double)ny * ny + (double)nz * nz);
        dd[f] = (float)(q[3] * len);
        // the decoded normal's direction error (L1), for the FP64 walk's
        // certified side choice on these records
        const double err = fabs(nx / len - q[0]) + fabs(ny / len - q[1]) + fabs(nz / len - q[2]);
        if (err > oct_err) oct_err = err;
      }
      TetOct& o = oct[t];
      o.oct01 = make_float4(ab[0], ab[1], ab[2], ab[3]);
      o.oct23 = make_float4(ab[4], ab[5], ab[6], ab[7]);
      o.d = make_float4(dd[0], dd[1], dd[2], dd[3]);
      o.nbr = rec[t].nbr;
    }
    CK(upload(c->d_teto, oct, c->stream), "upload octahedral records");
    c->oct_err = oct_err;
    CK(cudaStreamSynchronize(c->stream), "upload tet records");
    c->tmat_dirty = false;
  }
  if (c->bc_dirty) {
    CK(upload(c->d_bc, c->bc_type, c->stream), "upload boundary conditions");
    c->bc_dirty = false;
  }
  return MC_OK;
}

DevMesh dev_mesh(mc_ctx* c) {
  DevMesh M{};
  M.planes = c->d_planes.as<double4_32a>();
  M.tet = c->d_tet.as<Tet32>();
  M.teto = c->d_teto.as<TetOct>();
  M.tmat = c->d_tmat.as<int>();
  M.bc_type = c->d_bc.as<int>();
  M.n_bid = (int)c->bc_type.size();
  M.n_tet = c->mesh.n_tet;
  M.max_seg = (int)(c->seg_limit > 0 ? c->seg_limit : default_segment_limit(c->mesh.n_tet));
  // with margin for the float rounding of the bound itself
  M.oct_err = (float)(c->oct_err * 1.25 + 1e-9);
  for (int k = 0; k < 3; ++k) {
    M.glo[k] = c->mesh.glo[k];
    M.gh[k] = c->mesh.gh[k];
    M.ginv[k] = 1.0 / c->mesh.gh[k];
    M.gn[k] = c->mesh.gn[k];
  }
  M.gstart = c->d_gstart.as<int64_t>();
  M.gtets = c->d_gtets.as<int>();
  M.gseed = c->d_gseed.as<int>();
  return M;
}

DevXS dev_xs(mc_ctx* c) {
  DevXS X{};
  X.gE = c->d_gE.as<double>();
  X.g_off = c->d_goff.as<int64_t>();
  X.g_n = c->d_gn.as<int>();
  X.ghidx = c->d_ghidx.as<int>();
  X.nuc_grid = c->d_nuc_grid.as<int>();
  X.nuc_off = c->d_nuc_off.as<int64_t>();
  X.sig = c->d_sig.as<double2>();
  X.awr = c->d_awr.as<double>();
  X.mat_off = c->d_mat_off.as<int>();
  X.mat_nuc = c->d_mat_nuc.as<int>();
  X.mat_dens = c->d_mat_dens.as<double>();
  X.nusf = c->xs.nusf.empty() ? nullptr : c->d_nusf.as<double>();
  X.nuc_fiss = c->d_nuc_fiss.as<int>();
  X.mat_fiss = c->d_mat_fiss.as<int>();
  X.n_nuc = (int)c->xs.nuc_grid.size();
  X.n_grid = (int)c->xs.g_n.size();
  X.n_bins = c->xs.n_bins;
  X.E_lo = c->xs.E_lo;
  X.E_hi = c->xs.E_hi;
  X.lE_lo = c->xs.lE_lo;
  X.du = c->xs.du;
  return X;
}

DevSource dev_source(mc_ctx* c) {
  DevSource S{};
  S.space = c->src.space;
  S.energy = c->src.energy;
  for (int k = 0; k < 3; ++k) {
    S.point[k] = c->src.point[k];
    S.box_lo[k] = c->src.box_lo[k];
    S.box_hi[k] = c->src.box_hi[k];
  }
  S.n_cyl = c->src.n_cyl;
  S.cyl_xy = c->d_cyl.as<double>();
  S.cyl_r = c->src.cyl_r;
  S.cyl_z0 = c->src.cyl_z0;
  S.cyl_z1 = c->src.cyl_z1;
  S.watt_a = c->src.watt_a;
  S.watt_b = c->src.watt_b;
  S.mono_E = c->src.mono_E;
  return S;
}

int ensure_bank(mc_ctx* c, int64_t cap) {
  if (c->bank_cap == cap) return MC_OK;
  const size_t n = (size_t)cap;
  CK(c->b_rec.alloc(n * (size_t)kBankRec), "allocate particle bank");
  DevBuf* d4[] = {&c->b_elem, &c->q_xs0, &c->q_xs1, &c->q_adv0, &c->q_adv1, &c->q_coll, &c->q_free};
  for (DevBuf* b : d4) CK(b->alloc(n * 4), "allocate particle bank");
  CK(c->d_ctl.alloc(sizeof(EventCtl)), "allocate event control");
  c->bank_cap = cap;
  return MC_OK;
}

// k-eigenvalue fields of the particle bank, sized to the bank.
int ensure_eig_bank(mc_ctx* c) {
  const size_t n = (size_t)c->bank_cap;
  if (c->b_cn.bytes >= n * 32 && c->b_cn.p) return MC_OK;
  CK(c->b_nuf.alloc(n * 8), "allocate eigenvalue bank fields");
  CK(c->b_ktl.alloc(n * 8), "allocate eigenvalue bank fields");
  CK(c->b_cn.alloc(n * 32), "allocate eigenvalue bank fields");
  CK(c->b_nprog.alloc(n * 4), "allocate eigenvalue bank fields");
  return MC_OK;
}

Bank dev_bank(mc_ctx* c) {
  Bank B = bank_at(c->b_rec.p, c->b_elem.as<int>(), c->bank_cap);
  if (c->b_cn.p && c->b_cn.bytes >= (size_t)c->bank_cap * 32) {
    B.nuf = c->b_nuf.as<double>();
    B.ktl = c->b_ktl.as<double>();
    B.cn = c->b_cn.as<double4_32a>();
    B.n_prog = c->b_nprog.as<int>();
  }
  B.cap = c->bank_cap;
  return B;
}

EventQueues dev_queues(mc_ctx* c) {
  EventQueues Q{};
  Q.xs[0] = c->q_xs0.as<int>();
  Q.xs[1] = c->q_xs1.as<int>();
  Q.adv[0] = c->q_adv0.as<int>();
  Q.adv[1] = c->q_adv1.as<int>();
  Q.coll = c->q_coll.as<int>();
  Q.free_slots = c->q_free.as<int>();
  return Q;
}

}  // namespace

// ===========================================================================
extern "C" {

int mc_version(void) { return 1; }

int mc_ctx_create(int device, mc_ctx** out) {
  if (!out) return MC_ERR_ARG;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return MC_ERR_CUDA;
  if (device < 0 || device >= n) return MC_ERR_ARG;
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return MC_ERR_CUDA;
  mc_ctx* c = new mc_ctx();
  c->device = device;
  cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      cudaEventCreate(&c->ev_a0) != cudaSuccess || cudaEventCreate(&c->ev_a1) != cudaSuccess) {
    delete c;
    return MC_ERR_CUDA;
  }
  c->stream = c->own_stream;
  if (c->d_counters.alloc(sizeof(unsigned long long) * kNumCounters) != cudaSuccess ||
      c->d_leak_w.alloc(sizeof(double)) != cudaSuccess) {
    delete c;
    return MC_ERR_NOMEM;
  }
  // the no-allocation run's scratch array and kernels go on the device now,
  // while the caller can still let the library take memory
  std::string err;
  if (noalloc_prepare(device, err) != MC_OK) {
    delete c;
    return MC_ERR_CUDA;
  }
  *out = c;
  return MC_OK;
}

int mc_ctx_destroy(mc_ctx* c) {
  if (!c) return MC_ERR_ARG;
  {
    std::lock_guard<std::mutex> g(c->mu);
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
  }
  cudaEventDestroy(c->ev0);
  cudaEventDestroy(c->ev1);
  cudaEventDestroy(c->ev_a0);
  cudaEventDestroy(c->ev_a1);
  for (cudaEvent_t e : c->prof_ev) cudaEventDestroy(e);
  for (cudaEvent_t e : c->site_ev) cudaEventDestroy(e);
  cudaStreamSynchronize(c->copy_stream);
  cudaStreamDestroy(c->copy_stream);
  cudaStreamDestroy(c->own_stream);
  delete c;
  return MC_OK;
}

const char* mc_last_error(mc_ctx* c) { return c ? c->err.c_str() : "null context"; }

int mc_mesh_upload(mc_ctx* c, int64_t n_vtx, const double* xyz, int64_t n_tet,
                   const int32_t* tet_vtx, const int32_t* tet_block, const int32_t* tet_side_bid) {
  if (!c) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (!xyz || !tet_vtx || !tet_block) return set_err(c, MC_ERR_ARG, "null mesh array");
  MeshTables M;
  std::string m = build_mesh_tables(n_vtx, xyz, n_tet, tet_vtx, tet_block, tet_side_bid, M);
  if (!m.empty()) return set_err(c, MC_ERR_ARG, m);
  for (int64_t s = 0; s < 4 * n_tet; ++s)
    if (M.nbr[s] < 0 && -1 - M.nbr[s] >= (int64_t)c->bc_type.size())
      return set_err(c, MC_ERR_ARG, "sideset id out of range [0, 1024)");
  cudaSetDevice(c->device);
  c->mesh = std::move(M);
  CK(upload(c->d_planes, c->mesh.planes, c->stream), "upload planes");

  CK(upload(c->d_gstart, c->mesh.gstart, c->stream), "upload locator");
  CK(upload(c->d_gtets, c->mesh.gtets, c->stream), "upload locator");
  CK(upload(c->d_gseed, c->mesh.gseed, c->stream), "upload locator");
  c->tspec = TallySpec{};
  c->tspec.est = MC_EST_TRACKLENGTH;
  c->tspec.nb = 1;
  c->tspec.ns = 1;
  c->n_tally = n_tet;
  c->tally2_clear = false;
  CK(c->d_tally.alloc(sizeof(double) * (size_t)c->n_tally), "allocate tally");
  CK(c->d_sum.alloc(sizeof(double) * (size_t)c->n_tally), "allocate tally");
  CK(c->d_sumsq.alloc(sizeof(double) * (size_t)c->n_tally), "allocate tally");
  CK(cudaMemsetAsync(c->d_tally.p, 0, c->d_tally.bytes, c->stream), "clear tally");
  CK(cudaMemsetAsync(c->d_sum.p, 0, c->d_sum.bytes, c->stream), "clear tally");
  CK(cudaMemsetAsync(c->d_sumsq.p, 0, c->d_sumsq.bytes, c->stream), "clear tally");
  CK(cudaStreamSynchronize(c->stream), "mesh upload");
  c->have_mesh = true;
  c->tmat_dirty = true;
  c->batches = 0;
  return MC_OK;
}

int mc_bc_set(mc_ctx* c, int32_t bid, int32_t type) {
  if (!c) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (bid < 0 || bid >= (int32_t)c->bc_type.size()) return set_err(c, MC_ERR_ARG, "boundary id out of range [0, 1024)");
  if (type != MC_BC_VACUUM && type != MC_BC_REFLECT) return set_err(c, MC_ERR_ARG, "unknown boundary condition type");
  c->bc_type[bid] = type;
  c->bc_dirty = true;
  return MC_OK;
}

int mc_nuclide_add(mc_ctx* c, int64_t n_pts, const double* E, const double* sig_t,
                   const double* sig_s, double awr, int32_t* out_index) {
  if (!c) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (n_pts < 2 || !E || !sig_t || !sig_s) return set_err(c, MC_ERR_ARG, "nuclide grid needs at least 2 points");
  if (n_pts > (int64_t)1 << 30) return set_err(c, MC_ERR_ARG, "nuclide grid too large");
  if (!(E[0] > 0.0)) return set_err(c, MC_ERR_ARG, "nuclide energies must be positive");
  for (int64_t i = 0; i + 1 < n_pts; ++i)
    if (!(E[i] < E[i + 1])) return set_err(c, MC_ERR_ARG, "nuclide energy grid must be strictly increasing");
  if (!std::isfinite(E[n_pts - 1])) return set_err(c, MC_ERR_ARG, "nuclide energies must be finite");
  for (int64_t i = 0; i < n_pts; ++i) {
    if (!std::isfinite(sig_t[i]) || !std::isfinite(sig_s[i]))
      return set_err(c, MC_ERR_ARG, "cross sections must be finite (point " + std::to_string(i) + ")");
    if (!(sig_t[i] >= 0.0) || !(sig_s[i] >= 0.0) || sig_s[i] > sig_t[i])
      return set_err(c, MC_ERR_ARG, "cross sections must satisfy 0 <= sigma_s <= sigma_t (point " +
                                        std::to_string(i) + ")");
  }
  if (!(awr > 0.0) || !std::isfinite(awr)) return set_err(c, MC_ERR_ARG, "atomic weight ratio must be positive");
  Nuclide n;
  n.E.assign(E, E + n_pts);
  n.st.assign(sig_t, sig_t + n_pts);
  n.ss.assign(sig_s, sig_s + n_pts);
  n.awr = awr;
  c->nucs.push_back(std::move(n));
  if (out_index) *out_index = (int32_t)c->nucs.size() - 1;
  c->xs_dirty = true;
  return MC_OK;
}

int mc_nuclide_set_fission(mc_ctx* c, int32_t nuclide, const double* nu_sig_f) {
  if (!c) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (nuclide < 0 || nuclide >= (int32_t)c->nucs.size()) return set_err(c, MC_ERR_ARG, "nuclide index out of range");
  Nuclide& n = c->nucs[nuclide];
  if (!nu_sig_f) {
    n.nusf.clear();
  } else {
    for (size_t i = 0; i < n.E.size(); ++i)
      if (!(nu_sig_f[i] >= 0.0) || !(nu_sig_f[i] < 1e300))
        return set_err(c, MC_ERR_ARG, "nu*sigma_f must be finite and non-negative");
    n.nusf.assign(nu_sig_f, nu_sig_f + n.E.size());
  }
  c->xs_dirty = true;
  return MC_OK;
}

int mc_material_add(mc_ctx* c, int32_t material_id, int32_t n, const int32_t* nuclides,
                    const double* densities) {
  if (!c) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (n < 1 || !nuclides || !densities) return set_err(c, MC_ERR_ARG, "material needs at least one nuclide");
  for (int i = 0; i < n; ++i) {
    if (nuclides[i] < 0 || nuclides[i] >= (int32_t)c->nucs.size())
      return set_err(c, MC_ERR_ARG, "material nuclide index out of range");
    if (!(densities[i] >= 0.0) || !std::isfinite(densities[i]))
      return set_err(c, MC_ERR_ARG, "atom densities must be finite and non-negative");
  }
  for (const auto& m : c->mats)
    if (m.id == material_id) return set_err(c, MC_ERR_ARG, "duplicate material id");
  Material m;
  m.id = material_id;
  m.nuc.assign(nuclides, nuclides + n);
  m.dens.assign(densities, densities + n);
  c->mats.push_back(std::move(m));
  c->xs_dirty = true;
  return MC_OK;
}

int mc_block_material_map(mc_ctx* c, int32_t n, const int32_t* blocks, const int32_t* materials) {
  if (!c) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (n < 0 || (n > 0 && (!blocks || !materials))) return set_err(c, MC_ERR_ARG, "null block map");
  c->map_blocks.assign(blocks, blocks + n);
  c->map_mats.assign(materials, materials + n);
  c->tmat_dirty = true;
  return MC_OK;
}

int mc_set_hash_bins(mc_ctx* c, int32_t n_bins) {
  if (!c) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (n_bins < 1 || n_bins > (1 << 24)) return set_err(c, MC_ERR_ARG, "hash bins must be in [1, 2^24]");
  c->n_bins = n_bins;
  c->xs_dirty = true;
  return MC_OK;
}

int mc_source_set(mc_ctx* c, const mc_source_desc* s) {
  if (!c || !s) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (s->space < 0 || s->space > 2) return set_err(c, MC_ERR_ARG, "unknown source space kind");
  if (s->energy < 0 || s->energy > 1) return set_err(c, MC_ERR_ARG, "unknown source energy kind");
  if (s->space == MC_SRC_CYLINDERS && (s->n_cyl < 1 || !s->cyl_xy || !(s->cyl_r > 0.0)))
    return set_err(c, MC_ERR_ARG, "cylinder source needs cylinders and a positive radius");
  if (s->energy == MC_SRC_WATT && (!(s->watt_a > 0.0) || !(s->watt_b > 0.0)))
    return set_err(c, MC_ERR_ARG, "Watt parameters must be positive");
  if (s->energy == MC_SRC_MONO && !(s->mono_E > 0.0))
    return set_err(c, MC_ERR_ARG, "source energy must be positive");
  c->src = *s;
  if (s->space == MC_SRC_CYLINDERS) {
    c->src_cyl.assign(s->cyl_xy, s->cyl_xy + 2 * (size_t)s->n_cyl);
    cudaSetDevice(c->device);
    CK(upload(c->d_cyl, c->src_cyl, c->stream), "upload source");
    CK(cudaStreamSynchronize(c->stream), "upload source");
  }
  c->src.cyl_xy = nullptr;
  c->have_src = true;
  return MC_OK;
}

int mc_run(mc_ctx* c, const mc_run_desc* d) {
  if (!c || !d) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  const int rc = run_locked(c, d, nullptr, nullptr);
  // copies of later batches' host sites run on the copy stream and read the
  // caller's buffer; a run that stopped early may leave some queued, so
  // every return waits for them (a finished run has already waited)
  if (d->sites) {
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->copy_stream);
  }
  return rc;
}

}  // extern "C"

namespace {

// One run of histories (mc_run's body, with the context lock held).
// dev_sites: DEVICE source sites of the n_histories histories (instead of
// d->sites or sampling); eig: k-eigenvalue generation state, or null.
int run_locked(mc_ctx* c, const mc_run_desc* d, const mc_site* dev_sites, const EigArgs* eig) {
  if (d->n_histories < 0 || d->first_history < 0) return set_err(c, MC_ERR_ARG, "negative history range");
  if (d->precision != MC_PREC_FP64 && d->precision != MC_PREC_MIXED)
    return set_err(c, MC_ERR_ARG, "unknown precision form");
  if (d->mode != MC_MODE_HISTORY && d->mode != MC_MODE_EVENT) return set_err(c, MC_ERR_ARG, "unknown execution form");
  if (!c->have_src) return set_err(c, MC_ERR_STATE, "no source (mc_source_set)");
  if (c->serving && d->mode == MC_MODE_EVENT)
    return set_err(c, MC_ERR_STATE, "a serving session holds this context's event state (mc_serve_close)");
  cudaSetDevice(c->device);
  int rc = ensure_device_tables(c);
  if (rc) return rc;
  const int block = d->block_size > 0 ? d->block_size : 256;
  if (block % 32 != 0 || block > 256) return set_err(c, MC_ERR_ARG, "block size must be a multiple of 32, at most 256");
  if (d->walk_blocks != 0 && d->walk_blocks != 4 && d->walk_blocks != 5)
    return set_err(c, MC_ERR_ARG, "walk_blocks must be 0, 4 or 5");
  if (d->record_traces) {
    if (c->trace_n < d->n_histories) {
      CK(c->d_traces.alloc(sizeof(mc_trace) * (size_t)std::max<int64_t>(1, d->n_histories)), "allocate traces");
      c->trace_n = d->n_histories;
    }
  }
  CK(cudaMemsetAsync(c->d_counters.p, 0, c->d_counters.bytes, c->stream), "clear counters");
  CK(cudaMemsetAsync(c->d_leak_w.p, 0, sizeof(double), c->stream), "clear counters");
  RunArgs a{};
  a.first = d->first_history;
  a.n = d->n_histories;
  a.master = d->seed;
  a.tally = c->d_tally.as<double>();
  a.traces = d->record_traces ? c->d_traces.as<mc_trace>() : nullptr;
  a.counters = c->d_counters.as<unsigned long long>();
  a.leak_w = c->d_leak_w.as<double>();
  a.precision = d->precision;
  a.max_seg = d->max_seg_per_advance;
  a.refill = d->refill;
  a.walk_blocks = d->walk_blocks;
  a.two_d = c->two_d;
  a.z2d = c->z2d;
  a.sort_shift = -1;
  a.sort_buckets = 0;
  a.sort_tmp = nullptr;
  a.sort_cnt = nullptr;
  if (d->sort_queue > 0 && d->mode == MC_MODE_EVENT) {
    // key = elem >> shift with at most 65536 buckets
    int shift = d->sort_queue - 1;
    while ((c->mesh.n_tet >> shift) >= 65536) ++shift;
    a.sort_shift = shift;
    a.sort_buckets = (int)(c->mesh.n_tet >> shift) + 1;
    CK(c->d_sort_cnt.alloc(sizeof(int) * (size_t)(a.sort_buckets + 1)), "allocate sort counters");
  }
  a.sites = nullptr;
  a.n_mat = (int)c->xs.mat_ids.size();
  {
    double dg = 0.0;
    for (int k = 0; k < 3; ++k) {
      const double e = c->mesh.bbox_hi[k] - c->mesh.bbox_lo[k];
      dg += e * e;
    }
    a.tol = (float)(1e-6 * sqrt(dg));
  }
  if (dev_sites) a.sites = dev_sites;
  a.eig = EigArgs{};
  a.eig.keff = 1.0;
  if (eig) a.eig = *eig;
  const DevMesh M = dev_mesh(c);
  const DevXS X = dev_xs(c);
  const DevSource S = dev_source(c);
  const int per_sm = 2048 / block;
  const int grid = std::max(1, c->n_sm * per_sm);
  int n_launch = 0, n_adv = 0;
  float ms_adv = 0.0f;
  // batches run through one pipeline: batch b scores into tally slot
  // b % slots and is folded into SUM/SUM_SQ (normalised by its size) once
  // its last particle ends; births of batch b+slots wait until then, so the
  // long walks of one batch overlap the bulk of the next slots-1 batches
  const int nb = d->n_batches > 1 ? d->n_batches : 1;
  if (d->batch_sum_out && !d->accumulate) return set_err(c, MC_ERR_ARG, "batch results need accumulate = 1");
  // Each slot is one batch tally.  More slots let births run further
  // ahead of a batch's last long histories, so the bank stays full: on the
  // 2M-tet lattice, 10 x 1e6 histories ran 172.4M (mixed) and 60.9M (FP64)
  // histories/s with all ten batches in flight against 157.8M and 58.5M
  // with eight.  The slots' tallies are held to kSlotBudget bytes and a
  // quarter of the free device memory.
  int slots = std::min(nb, kPipeSlots);
  if (nb > 1) {
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b), "memory info");
    const size_t per = std::max<size_t>(1, sizeof(double) * (size_t)c->n_tally);
    const size_t budget = std::min<size_t>(kSlotBudget, free_b / 4);
    slots = std::max(2, std::min(slots, (int)std::min<size_t>(kPipeSlots, budget / per + 1)));
  }
  std::vector<int64_t> bend((size_t)nb);
  if (nb > 1) {
    if (!d->batch_sizes) return set_err(c, MC_ERR_ARG, "n_batches > 1 needs batch_sizes");
    if (!d->accumulate) return set_err(c, MC_ERR_ARG, "pipelined batches need accumulate = 1");
    int64_t acc = 0;
    for (int b = 0; b < nb; ++b) {
      if (d->batch_sizes[b] < 1) return set_err(c, MC_ERR_ARG, "batch sizes must be positive");
      acc += d->batch_sizes[b];
      bend[b] = acc;
    }
    if (acc != d->n_histories) return set_err(c, MC_ERR_ARG, "batch sizes must add up to n_histories");
    std::vector<DevRequest> rq((size_t)nb);
    for (int b = 0; b < nb; ++b) {
      DevRequest& q = rq[b];
      q = DevRequest{};
      q.start = b ? bend[b - 1] : 0;
      q.end = bend[b];
      q.first_id = a.first + q.start;
      q.seed = d->seed;
      q.slot = b % slots;
      q.has_src = 0;
    }
    CK(upload(c->d_batch_end, rq, c->stream), "upload batch table");
    const size_t need = sizeof(double) * (size_t)c->n_tally * (size_t)(slots - 1);
    if (c->d_tally2.bytes < need) {
      CK(c->d_tally2.alloc(need), "allocate batch tallies");
      c->tally2_clear = false;
    }
    if (!c->tally2_clear) {
      CK(cudaMemsetAsync(c->d_tally2.p, 0, c->d_tally2.bytes, c->stream), "clear batch tally");
      c->tally2_clear = true;
    }
    a.tally2 = c->d_tally2.as<double>();
    a.req = c->d_batch_end.as<DevRequest>();
    a.n_req = nb;
  } else {
    bend[0] = d->n_histories;
    a.tally2 = a.tally;
    a.req = nullptr;
    a.n_req = 0;
  }
  a.n_tally = c->n_tally;
  a.ts = c->tspec;
  if (c->ray_n > 0 && d->n_histories > 0) {
    CK(cudaMemsetAsync(c->d_rays.p, 0, c->d_rays.bytes, c->stream), "clear ray segments");
    a.ts.rays = c->d_rays.as<mc_ray_segment>();
    a.ts.ray_first = d->first_history;
    a.ts.ray_n = c->ray_n;
    a.ts.ray_cap = c->ray_cap;
    c->ray_first = d->first_history;
  }
  a.live = nullptr;
  // history-form batches all score into slot 0 (one runs at a time);
  // event-form batch b scores into slot b % slots
  // Host source sites: the first batch's sites are copied in stream order;
  // in the event form the rest go on the copy stream, one copy per batch,
  // and the birth limit reaches batch b only after the tracker's stream
  // has waited for b's copy, so the copies overlap the first batch's walks.
  // (Copying two batches first ran within the spread on a box whose host
  // copies were fast, and costs a batch's copy where they are slow.)
  int pre_b = nb;  // batches whose sites are copied in stream order
  if (!dev_sites && d->sites && d->n_histories > 0) {
    CK(cudaStreamSynchronize(c->copy_stream), "copy stream");
    CK(c->d_sites.alloc(std::max(c->d_sites.bytes, sizeof(mc_site) * (size_t)d->n_histories)), "allocate sites");
    a.sites = c->d_sites.as<mc_site>();
    if (d->mode == MC_MODE_EVENT && nb > 1) pre_b = 1;
    CK(cudaMemcpyAsync(c->d_sites.p, d->sites, sizeof(mc_site) * (size_t)bend[pre_b - 1], cudaMemcpyHostToDevice,
                       c->stream),
       "upload sites");
    if (pre_b < nb) {
      while (c->site_ev.size() < (size_t)nb) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
        c->site_ev.push_back(e);
      }
      // the copies start after the tracker's stream reached this point
      CK(cudaEventRecord(c->site_ev[0], c->stream), "event");
      CK(cudaStreamWaitEvent(c->copy_stream, c->site_ev[0], 0), "copy stream wait");
      for (int b = pre_b; b < nb; ++b) {
        CK(cudaMemcpyAsync(c->d_sites.as<mc_site>() + bend[b - 1], d->sites + bend[b - 1],
                           sizeof(mc_site) * (size_t)(bend[b] - bend[b - 1]), cudaMemcpyHostToDevice,
                           c->copy_stream),
           "upload sites");
        CK(cudaEventRecord(c->site_ev[b], c->copy_stream), "event");
      }
    }
  }
  auto fold = [&](int b) -> int {
    const int64_t size = bend[b] - (b ? bend[b - 1] : 0);
    const int sl = (d->mode == MC_MODE_EVENT) ? b % slots : 0;
    double* buf = sl ? a.tally2 + (int64_t)(sl - 1) * c->n_tally : a.tally;
    CK(launch_accumulate(buf, c->d_sum.as<double>(), c->d_sumsq.as<double>(),
                         c->n_tally, size > 0 ? 1.0 / (double)size : 0.0, c->stream),
       "launch accumulate");
    if (d->batch_sum_out && d->batch_sum_out[b])
      CK(cudaMemcpyAsync(d->batch_sum_out[b], c->d_sum.p, sizeof(double) * (size_t)c->n_tally,
                         cudaMemcpyDeviceToHost, c->stream),
         "copy batch result");
    c->batches += 1;
    return MC_OK;
  };
  CK(cudaEventRecord(c->ev0, c->stream), "event");
  int folded = 0;
  if (d->n_histories > 0) {
    if (d->mode == MC_MODE_HISTORY) {
      for (int b = 0; b < nb; ++b) {
        RunArgs ab = a;
        ab.first = a.first + (b ? bend[b - 1] : 0);
        ab.n = bend[b] - (b ? bend[b - 1] : 0);
        ab.req = nullptr;
        ab.n_req = 0;
        ab.tally2 = ab.tally;
        ab.traces = a.traces ? a.traces + (ab.first - a.first) : nullptr;
        CK(launch_history(M, X, S, ab, block, grid, c->stream), "launch history kernel");
        ++n_launch;
        if (nb > 1) {
          rc = fold(b);
          if (rc) return rc;
          ++folded;
        }
      }
      n_adv = n_launch;
    } else {
      int64_t cap = d->bank_size > 0 ? std::min(d->bank_size, d->n_histories) : d->n_histories;
      cap = std::max<int64_t>(cap, 1);
      if (cap > ((int64_t)1 << 30)) return set_err(c, MC_ERR_ARG, "bank too large");
      rc = ensure_bank(c, std::max(cap, c->bank_cap));
      if (rc) return rc;
      if (a.eig.on) {
        rc = ensure_eig_bank(c);
        if (rc) return rc;
      }
      const Bank B = dev_bank(c);
      if (!bank_complete(B)) return set_err(c, MC_ERR_STATE, "internal: particle bank incomplete");
      if (a.eig.on && !(B.nuf && B.ktl && B.cn && B.n_prog))
        return set_err(c, MC_ERR_STATE, "internal: eigenvalue bank fields missing");
      const EventQueues Q = dev_queues(c);
      EventCtl* ctl = c->d_ctl.as<EventCtl>();
      int h_live[kPipeSlots] = {0};
      if (nb > 1) {
        if (c->d_live.bytes < sizeof(int) * kPipeSlots) CK(c->d_live.alloc(sizeof(int) * kPipeSlots), "allocate live");
        CK(cudaMemsetAsync(c->d_live.p, 0, sizeof(int) * kPipeSlots, c->stream), "clear live");
        a.live = c->d_live.as<int>();
      }
      if (a.sort_shift >= 0) {
        CK(c->d_sort_tmp.alloc(std::max(c->d_sort_tmp.bytes, sizeof(int) * (size_t)c->bank_cap)), "allocate sort");
        a.sort_tmp = c->d_sort_tmp.as<int>();
        a.sort_cnt = c->d_sort_cnt.as<int>();
      }
      // births are allowed up to the end of batch lim_b
      int lim_b = std::min(slots, pre_b) - 1;
      int64_t limit = nb > 1 ? bend[lim_b] : d->n_histories;
      CK(launch_event_init(M, X, S, a, B, Q, ctl, block, grid, c->stream, limit), "launch event init");
      n_launch = 1;
      int par = 0;
      int oldest = 0;
      EventCtl h;
      const int kGroup = 4;
      const int64_t tail = d->tail > 0 ? (int64_t)d->tail : d->tail < 0 ? -1
                                                          : std::max<int64_t>(4096, cap / tail_divisor(a));
      // a graph replays one group of iterations (parity 0,1,0,1: the group
      // always starts at parity 0), captured on first use
      const bool use_graph = d->graph && !d->profile;
      cudaGraphExec_t gexec = nullptr;
      struct GraphGuard {
        cudaGraphExec_t* e;
        ~GraphGuard() {
          if (*e) cudaGraphExecDestroy(*e);
        }
      } gguard{&gexec};
      if (use_graph) {
        int nl = 0;
        cudaGraph_t graph = nullptr;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin graph capture");
        cudaError_t ce = cudaSuccess;
        for (int gi = 0; gi < kGroup && ce == cudaSuccess; ++gi)
          ce = launch_event_iteration(M, X, S, a, B, Q, ctl, gi & 1, block, grid, c->stream, &nl);
        const cudaError_t ee = cudaStreamEndCapture(c->stream, &graph);
        if (ce != cudaSuccess) return cuda_err(c, ce, "capture event iterations");
        if (ee != cudaSuccess) return cuda_err(c, ee, "end graph capture");
        ce = cudaGraphInstantiate(&gexec, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) return cuda_err(c, ce, "instantiate event graph");
      }
      for (int64_t it = 0;; ++it) {
        if (use_graph) {
          CK(cudaGraphLaunch(gexec, c->stream), "launch event graph");
          n_launch += kGroup * (5 + (a.sort_shift >= 0 ? 4 : 0));
          n_adv += kGroup;
        }
        for (int gi = 0; gi < kGroup && !use_graph; ++gi) {
          cudaEvent_t e0 = nullptr, e1 = nullptr;
          if (d->profile) {
            while (c->prof_ev.size() < (size_t)(2 * n_adv + 2)) {
              cudaEvent_t e;
              CK(cudaEventCreate(&e), "event");
              c->prof_ev.push_back(e);
            }
            e0 = c->prof_ev[2 * n_adv];
            e1 = c->prof_ev[2 * n_adv + 1];
          }
          CK(launch_event_iteration(M, X, S, a, B, Q, ctl, par, block, grid, c->stream, &n_launch, e0, e1),
             "launch event iteration");
          n_adv += 1;
          par ^= 1;
        }
        CK(cudaMemcpyAsync(&h, ctl, sizeof(EventCtl), cudaMemcpyDeviceToHost, c->stream), "read event control");
        if (nb > 1)
          CK(cudaMemcpyAsync(h_live, a.live, sizeof(int) * slots, cudaMemcpyDeviceToHost, c->stream),
             "read live counters");
        CK(cudaStreamSynchronize(c->stream), "event loop");
        if (nb > 1) {
          // retire drained batches, then let the next batches be born
          while (oldest < nb && h.next_hist >= bend[oldest] && h_live[oldest % slots] == 0) {
            rc = fold(oldest);
            if (rc) return rc;
            ++oldest;
            ++folded;
          }
          // the limit moves over the batches within the slot window whose
          // sites have landed (a copy still running is not waited for)
          const int target = std::min(oldest + slots - 1, nb - 1);
          int reach = lim_b;
          while (oldest < nb && reach < target) {
            const int b = reach + 1;
            if (b >= pre_b) {
              const cudaError_t q = cudaEventQuery(c->site_ev[b]);
              if (q == cudaErrorNotReady) break;
              CK(q, "site copy");
              CK(cudaStreamWaitEvent(c->stream, c->site_ev[b], 0), "wait for sites");
            }
            reach = b;
          }
          if (reach > lim_b) {
            lim_b = reach;
            c->h_limit = bend[reach];
            CK(cudaMemcpyAsync(&ctl->birth_limit, &c->h_limit, sizeof(long long), cudaMemcpyHostToDevice,
                               c->stream),
               "raise birth limit");
            CK(cudaStreamSynchronize(c->stream), "raise birth limit");
          }
          if (oldest >= nb) break;
        }
        const int64_t inflight = (int64_t)h.n_xs[par] + h.n_adv[par];
        if (nb == 1 && inflight == 0 && h.next_hist >= a.n) break;
        if (h.next_hist >= a.n && inflight <= tail) {
          // a few particles per warp (tail_block): the long histories left
          // are latency chains, spread over every SM instead of serialised
          // by divergence inside full warps
          const int tb = tail_block(a.precision);
          const int fgrid = (int)std::max<int64_t>(1, (inflight + tb - 1) / tb);
          CK(launch_event_finish(M, X, S, a, B, Q, ctl, par, tb, fgrid, c->stream), "launch event finish");
          ++n_launch;
          break;
        }
        if (it > 10000000) return set_err(c, MC_ERR_DEVICE, "event loop did not terminate");
      }
    }
  }
  CK(cudaEventRecord(c->ev1, c->stream), "event");
  if (d->accumulate) {
    if (nb == 1) {
      rc = fold(0);
      if (rc) return rc;
    } else {
      for (int b = folded; b < nb; ++b) {
        rc = fold(b);
        if (rc) return rc;
      }
    }
  }
  unsigned long long cnt[kNumCounters];
  double leak_w = 0.0;
  CK(cudaMemcpyAsync(cnt, c->d_counters.p, sizeof cnt, cudaMemcpyDeviceToHost, c->stream), "read counters");
  CK(cudaMemcpyAsync(&leak_w, c->d_leak_w.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream), "read counters");
  CK(cudaStreamSynchronize(c->stream), "run");
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  if (d->mode == MC_MODE_HISTORY) {
    ms_adv = ms;
  } else if (d->profile) {
    for (int i = 0; i < n_adv; ++i) {
      float t = 0.0f;
      cudaEventElapsedTime(&t, c->prof_ev[2 * i], c->prof_ev[2 * i + 1]);
      ms_adv += t;
    }
  }
  mc_stats& s = c->last;
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
  s.n_launch = n_launch;
  s.leak_weight = leak_w;
  s.ms_total = ms;
  s.ms_advance = ms_adv;
  s.n_advance_launch = n_adv;
  s.n_seg_advance = (int64_t)cnt[kCntSegWalk];
  if (s.n_hist != d->n_histories)
    return set_err(c, MC_ERR_DEVICE, "device finished " + std::to_string(s.n_hist) + " of " +
                                         std::to_string(d->n_histories) + " histories");
  return MC_OK;
}

}  // namespace

extern "C" {

int mc_source_sample(mc_ctx* c, int64_t first, int64_t n, uint64_t seed, mc_site* out) {
  if (!c || (!out && n > 0)) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (n < 0 || first < 0) return set_err(c, MC_ERR_ARG, "negative history range");
  if (!c->have_src) return set_err(c, MC_ERR_STATE, "no source (mc_source_set)");
  if (n == 0) return MC_OK;
  cudaSetDevice(c->device);
  int rc = ensure_device_tables(c);
  if (rc) return rc;
  CK(c->d_sites.alloc(std::max(c->d_sites.bytes, sizeof(mc_site) * (size_t)n)), "allocate sites");
  CK(launch_sample(dev_xs(c), dev_source(c), first, n, seed, c->d_sites.as<mc_site>(), c->stream),
     "launch source sampling");
  CK(cudaMemcpyAsync(out, c->d_sites.p, sizeof(mc_site) * (size_t)n, cudaMemcpyDeviceToHost, c->stream),
     "download sites");
  CK(cudaStreamSynchronize(c->stream), "source sampling");
  return MC_OK;
}

int mc_ctx_set_stream(mc_ctx* c, void* stream) {
  if (!c) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  cudaSetDevice(c->device);
  CK(cudaStreamSynchronize(c->stream), "sync before stream change");
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return MC_OK;
}

int mc_sync(mc_ctx* c) {
  if (!c) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  cudaSetDevice(c->device);
  CK(cudaStreamSynchronize(c->stream), "sync");
  return MC_OK;
}

int mc_tally_download(mc_ctx* c, int32_t kind, double* out, int64_t n) {
  if (!c || !out) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (!c->have_mesh) return set_err(c, MC_ERR_STATE, "no mesh");
  if (n != c->n_tally)
    return set_err(c, MC_ERR_ARG, "tally length must equal mc_tally_size (" + std::to_string(c->n_tally) + ")");
  DevBuf* b = kind == MC_TALLY_BATCH ? &c->d_tally : kind == MC_TALLY_SUM ? &c->d_sum
              : kind == MC_TALLY_SUM_SQ ? &c->d_sumsq : nullptr;
  if (!b) return set_err(c, MC_ERR_ARG, "unknown tally kind");
  cudaSetDevice(c->device);
  CK(cudaMemcpyAsync(out, b->p, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, c->stream), "download tally");
  CK(cudaStreamSynchronize(c->stream), "download tally");
  return MC_OK;
}

int mc_tally_reset(mc_ctx* c) {
  if (!c) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (!c->have_mesh) return set_err(c, MC_ERR_STATE, "no mesh");
  cudaSetDevice(c->device);
  CK(cudaMemsetAsync(c->d_tally.p, 0, c->d_tally.bytes, c->stream), "clear tally");
  CK(cudaMemsetAsync(c->d_sum.p, 0, c->d_sum.bytes, c->stream), "clear tally");
  CK(cudaMemsetAsync(c->d_sumsq.p, 0, c->d_sumsq.bytes, c->stream), "clear tally");
  CK(cudaStreamSynchronize(c->stream), "clear tally");
  c->batches = 0;
  return MC_OK;
}

int mc_tally_configure(mc_ctx* c, const mc_tally_desc* d) {
  if (!c || !d) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (!c->have_mesh) return set_err(c, MC_ERR_STATE, "no mesh");
  if (c->serving) return set_err(c, MC_ERR_STATE, "the tally cannot change while serving is open");
  if (d->estimator != MC_EST_TRACKLENGTH && d->estimator != MC_EST_COLLISION)
    return set_err(c, MC_ERR_ARG, "estimator must be MC_EST_TRACKLENGTH or MC_EST_COLLISION");
  if (d->n_scores < 1 || d->n_scores > MC_MAX_SCORES) return set_err(c, MC_ERR_ARG, "1 to 4 scores");
  int sc = 0;
  bool need_ss = false;
  for (int j = 0; j < d->n_scores; ++j) {
    const int s = d->scores[j];
    if (s < MC_SCORE_FLUX || s > MC_SCORE_ABSORPTION) return set_err(c, MC_ERR_ARG, "unknown score");
    if (d->estimator == MC_EST_TRACKLENGTH && s != MC_SCORE_FLUX && s != MC_SCORE_TOTAL)
      return set_err(c, MC_ERR_ARG, "the track-length estimator scores flux and total only");
    for (int i = 0; i < j; ++i)
      if (d->scores[i] == s) return set_err(c, MC_ERR_ARG, "repeated score");
    if (s == MC_SCORE_SCATTER || s == MC_SCORE_ABSORPTION) need_ss = true;
    sc |= s << (8 * j);
  }
  const int nb = d->n_energy_bins > 0 ? d->n_energy_bins : 1;
  if (d->n_energy_bins > MC_MAX_ENERGY_BINS) return set_err(c, MC_ERR_ARG, "too many energy bins");
  if (d->n_energy_bins > 0) {
    if (!d->energy_edges) return set_err(c, MC_ERR_ARG, "null energy edges");
    for (int b = 0; b < d->n_energy_bins; ++b)
      if (!(d->energy_edges[b + 1] > d->energy_edges[b]))
        return set_err(c, MC_ERR_ARG, "energy edges must ascend strictly");
  }
  cudaSetDevice(c->device);
  TallySpec t{};
  t.general = 1;
  t.est = d->estimator;
  t.nb = nb;
  t.ns = d->n_scores;
  t.sc = sc;
  t.need_ss = need_ss;
  t.edges = nullptr;
  if (d->n_energy_bins > 0) {
    std::vector<double> e(d->energy_edges, d->energy_edges + d->n_energy_bins + 1);
    CK(upload(c->d_edges, e, c->stream), "upload energy edges");
    t.edges = c->d_edges.as<double>();
  }
  // the default definition keeps the one-value-per-element fast path
  if (t.est == MC_EST_TRACKLENGTH && t.ns == 1 && sc == MC_SCORE_FLUX && d->n_energy_bins <= 0) t.general = 0;
  c->tspec = t;
  c->n_tally = c->mesh.n_tet * (int64_t)nb * (int64_t)t.ns;
  c->tally2_clear = false;
  c->d_tally2.release();
  CK(c->d_tally.alloc(sizeof(double) * (size_t)c->n_tally), "allocate tally");
  CK(c->d_sum.alloc(sizeof(double) * (size_t)c->n_tally), "allocate tally");
  CK(c->d_sumsq.alloc(sizeof(double) * (size_t)c->n_tally), "allocate tally");
  CK(cudaMemsetAsync(c->d_tally.p, 0, c->d_tally.bytes, c->stream), "clear tally");
  CK(cudaMemsetAsync(c->d_sum.p, 0, c->d_sum.bytes, c->stream), "clear tally");
  CK(cudaMemsetAsync(c->d_sumsq.p, 0, c->d_sumsq.bytes, c->stream), "clear tally");
  CK(cudaStreamSynchronize(c->stream), "configure tally");
  c->batches = 0;
  return MC_OK;
}

int mc_rays_enable(mc_ctx* c, int32_t n_rays, int32_t max_segments) {
  if (!c) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (n_rays < 0 || max_segments < 0) return set_err(c, MC_ERR_ARG, "negative ray count or segment limit");
  if (n_rays == 0 || max_segments == 0) {
    c->ray_n = c->ray_cap = 0;
    c->d_rays.release();
    return MC_OK;
  }
  const size_t bytes = sizeof(mc_ray_segment) * (size_t)n_rays * (size_t)max_segments;
  if (bytes > ((size_t)16 << 30)) return set_err(c, MC_ERR_ARG, "ray segment buffer over 16 GiB");
  cudaSetDevice(c->device);
  CK(c->d_rays.alloc(bytes), "allocate ray segments");
  CK(cudaMemsetAsync(c->d_rays.p, 0, bytes, c->stream), "clear ray segments");
  CK(cudaStreamSynchronize(c->stream), "clear ray segments");
  c->ray_n = n_rays;
  c->ray_cap = max_segments;
  return MC_OK;
}

int mc_rays_download(mc_ctx* c, mc_ray_segment* out, int64_t capacity, int64_t* n_out) {
  if (!c || !n_out || (capacity > 0 && !out)) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  *n_out = 0;
  if (c->ray_n == 0) return set_err(c, MC_ERR_STATE, "ray recording is not enabled");
  cudaSetDevice(c->device);
  std::vector<mc_ray_segment> all((size_t)c->ray_n * (size_t)c->ray_cap);
  CK(cudaMemcpyAsync(all.data(), c->d_rays.p, c->d_rays.bytes, cudaMemcpyDeviceToHost, c->stream), "download rays");
  CK(cudaStreamSynchronize(c->stream), "download rays");
  int64_t n = 0;
  for (const mc_ray_segment& s : all) {
    if (s.id == 0) continue;  // slots past a ray's last segment stay empty
    if (n < capacity) out[n] = s;
    ++n;
  }
  *n_out = n;
  if (n > capacity) return set_err(c, MC_ERR_ARG, "capacity below the " + std::to_string(n) + " recorded segments");
  return MC_OK;
}

int mc_set_2d(mc_ctx* c, int32_t on, double z_coord) {
  if (!c) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (on && !(z_coord == z_coord)) return set_err(c, MC_ERR_ARG, "z_coord must be a number");
  c->two_d = on ? 1 : 0;
  c->z2d = on ? z_coord : 0.0;
  return MC_OK;
}

int mc_set_segment_limit(mc_ctx* c, int64_t max_segments) {
  if (!c) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (max_segments < 0 || max_segments > 2000000000LL)
    return set_err(c, MC_ERR_ARG, "segment limit must be in [0, 2e9] (0: the mesh-size default)");
  c->seg_limit = max_segments;
  return MC_OK;
}

int mc_segment_limit(mc_ctx* c, int64_t* out) {
  if (!c || !out) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (!c->have_mesh) return set_err(c, MC_ERR_STATE, "no mesh");
  *out = c->seg_limit > 0 ? c->seg_limit : default_segment_limit(c->mesh.n_tet);
  return MC_OK;
}

int mc_tally_size(mc_ctx* c, int64_t* n) {
  if (!c || !n) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (!c->have_mesh) return set_err(c, MC_ERR_STATE, "no mesh");
  *n = c->n_tally;
  return MC_OK;
}

int mc_tally_clear(mc_ctx* c, int32_t kind) {
  if (!c) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (!c->have_mesh) return set_err(c, MC_ERR_STATE, "no mesh");
  DevBuf* b = kind == MC_TALLY_BATCH ? &c->d_tally : kind == MC_TALLY_SUM ? &c->d_sum
              : kind == MC_TALLY_SUM_SQ ? &c->d_sumsq : nullptr;
  if (!b) return set_err(c, MC_ERR_ARG, "unknown tally kind");
  cudaSetDevice(c->device);
  CK(cudaMemsetAsync(b->p, 0, b->bytes, c->stream), "clear tally");
  CK(cudaStreamSynchronize(c->stream), "clear tally");
  return MC_OK;
}

int mc_trace_download(mc_ctx* c, mc_trace* out, int64_t n) {
  if (!c || !out) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (n > c->trace_n) return set_err(c, MC_ERR_ARG, "more traces requested than recorded");
  cudaSetDevice(c->device);
  CK(cudaMemcpyAsync(out, c->d_traces.p, sizeof(mc_trace) * (size_t)n, cudaMemcpyDeviceToHost, c->stream),
     "download traces");
  CK(cudaStreamSynchronize(c->stream), "download traces");
  return MC_OK;
}

int mc_stats_get(mc_ctx* c, mc_stats* out) {
  if (!c || !out) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  *out = c->last;
  return MC_OK;
}

int mc_batches_done(mc_ctx* c, int64_t* out) {
  if (!c || !out) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  *out = c->batches;
  return MC_OK;
}

// k-eigenvalue generations (OpenMCStudy's batch loop in eigenvalue mode:
// defineRays from the source bank, execute, postExecuteStudy ->
// finalize_generation -> sort, synchronize_bank, calculate_generation_keff,
// calculate_average_keff; src/userobjects/OpenMCStudy.C:297-607).
int mc_eigen_run(mc_ctx* c, const mc_eigen_desc* d, mc_eigen_gen* out) {
  if (!c || !d || !out) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  const int64_t n = d->n_particles;
  if (n < 1 || n > ((int64_t)1 << 30)) return set_err(c, MC_ERR_ARG, "particles must be in [1, 2^30]");
  if (d->n_batches < 1) return set_err(c, MC_ERR_ARG, "batches must be at least 1");
  if (d->n_inactive < 0 || d->n_inactive >= d->n_batches)
    return set_err(c, MC_ERR_ARG, "inactive batches must be in [0, batches)");
  if (!d->initial_source && !c->have_src) return set_err(c, MC_ERR_STATE, "no source (mc_source_set)");
  if (c->serving && d->mode == MC_MODE_EVENT)
    return set_err(c, MC_ERR_STATE, "a serving session holds this context's event state (mc_serve_close)");
  if (d->watt_a < 0.0 || d->watt_b < 0.0 || d->keff0 < 0.0)
    return set_err(c, MC_ERR_ARG, "keff0 and the fission spectrum parameters must be non-negative");
  cudaSetDevice(c->device);
  int rc = ensure_device_tables(c);
  if (rc) return rc;
  if (c->xs.nusf.empty()) return set_err(c, MC_ERR_STATE, "no fissionable nuclide (mc_nuclide_set_fission)");
  const int64_t cap = d->fission_bank_capacity > 0 ? d->fission_bank_capacity : 3 * n;
  if (cap > ((int64_t)1 << 31) - 1) return set_err(c, MC_ERR_ARG, "fission bank capacity too large");
  auto grow = [&](DevBuf& b, size_t need) -> cudaError_t {
    return b.bytes >= need && b.p ? cudaSuccess : b.alloc(need);
  };
  const int64_t nt = (n + kReduceTile - 1) / kReduceTile;
  CK(grow(c->e_src, sizeof(mc_site) * (size_t)n), "allocate source bank");
  CK(grow(c->e_bank, sizeof(mc_fission_site) * (size_t)cap), "allocate fission bank");
  CK(grow(c->e_sorted, sizeof(mc_fission_site) * (size_t)cap), "allocate fission bank");
  CK(grow(c->e_ktl, sizeof(double) * (size_t)n), "allocate estimators");
  CK(grow(c->e_kcol, sizeof(double) * (size_t)n), "allocate estimators");
  CK(grow(c->e_kabs, sizeof(double) * (size_t)n), "allocate estimators");
  CK(grow(c->e_prog, sizeof(int) * (size_t)n), "allocate site counts");
  CK(grow(c->e_off, sizeof(int64_t) * (size_t)(n + 1)), "allocate bank offsets");
  CK(grow(c->e_cnt, sizeof(int) * (size_t)cap), "allocate resampling counts");
  CK(grow(c->e_pos, sizeof(int64_t) * (size_t)(cap + 1)), "allocate resampling offsets");
  CK(grow(c->e_tmp, sizeof(int64_t) * (size_t)std::max(scan_tmp_size(n), scan_tmp_size(cap))), "allocate scan");
  CK(grow(c->e_part, sizeof(double) * (size_t)(3 * nt)), "allocate partial sums");
  CK(grow(c->e_nbank, sizeof(unsigned long long)), "allocate site counter");
  c->e_n = 0;
  c->e_m = 0;
  if (d->initial_source) {
    CK(cudaMemcpyAsync(c->e_src.p, d->initial_source, sizeof(mc_site) * (size_t)n, cudaMemcpyHostToDevice,
                       c->stream),
       "upload initial source");
  } else {
    // OpenMC initialize_source: site i from the source stream of id i+1
    CK(launch_sample(dev_xs(c), dev_source(c), 0, n, d->seed, c->e_src.as<mc_site>(), c->stream),
       "sample initial source");
  }
  cudaEvent_t g0 = nullptr, g1 = nullptr;
  CK(cudaEventCreate(&g0), "event");
  struct EvGuard {
    cudaEvent_t* a;
    cudaEvent_t* b;
    ~EvGuard() {
      if (*a) cudaEventDestroy(*a);
      if (*b) cudaEventDestroy(*b);
    }
  } evg{&g0, &g1};
  CK(cudaEventCreate(&g1), "event");
  std::vector<double> part((size_t)(3 * nt));
  double keff = d->keff0 > 0.0 ? d->keff0 : 1.0;
  double k_sum0 = 0.0, k_sum1 = 0.0, keff_std = 0.0;
  int n_active = 0;
  for (int gen = 0; gen < d->n_batches; ++gen) {
    const bool active = gen >= d->n_inactive;
    const int64_t first = (int64_t)gen * n;
    CK(cudaEventRecord(g0, c->stream), "event");
    CK(cudaMemsetAsync(c->e_ktl.p, 0, sizeof(double) * (size_t)n, c->stream), "clear estimators");
    CK(cudaMemsetAsync(c->e_kcol.p, 0, sizeof(double) * (size_t)n, c->stream), "clear estimators");
    CK(cudaMemsetAsync(c->e_kabs.p, 0, sizeof(double) * (size_t)n, c->stream), "clear estimators");
    CK(cudaMemsetAsync(c->e_prog.p, 0, sizeof(int) * (size_t)n, c->stream), "clear site counts");
    CK(cudaMemsetAsync(c->e_nbank.p, 0, sizeof(unsigned long long), c->stream), "clear site counter");
    EigArgs e{};
    e.on = 1;
    e.keff = keff;
    e.fa = d->watt_a > 0.0 ? d->watt_a : 0.988e6;
    e.fb = d->watt_b > 0.0 ? d->watt_b : 2.249e-6;
    e.first = first;
    e.bank = c->e_bank.as<mc_fission_site>();
    e.n_bank = c->e_nbank.as<unsigned long long>();
    e.cap = cap;
    e.ktl = c->e_ktl.as<double>();
    e.kcol = c->e_kcol.as<double>();
    e.kabs = c->e_kabs.as<double>();
    e.prog = c->e_prog.as<int>();
    mc_run_desc rd{};
    rd.first_history = first;
    rd.n_histories = n;
    rd.bank_size = d->bank_size;
    rd.seed = d->seed;
    rd.precision = d->precision;
    rd.mode = d->mode;
    rd.block_size = d->block_size;
    rd.max_seg_per_advance = d->max_seg_per_advance;
    rd.sort_queue = d->sort_queue;
    rd.graph = d->graph;
    rd.tail = d->tail;
    rd.accumulate = active ? 1 : 0;  // OpenMC scores tallies in active batches only
    rc = run_locked(c, &rd, c->e_src.as<mc_site>(), &e);
    if (rc) return rc;
    if (!active) CK(cudaMemsetAsync(c->d_tally.p, 0, c->d_tally.bytes, c->stream), "clear batch tally");
    const mc_stats st = c->last;
    // estimator sums in a fixed order: tree per tile of 1024, then tiles in order
    double* dp = c->e_part.as<double>();
    CK(launch_tile_sums(c->e_ktl.as<double>(), n, dp, c->stream), "sum estimators");
    CK(launch_tile_sums(c->e_kcol.as<double>(), n, dp + nt, c->stream), "sum estimators");
    CK(launch_tile_sums(c->e_kabs.as<double>(), n, dp + 2 * nt, c->stream), "sum estimators");
    unsigned long long m_all = 0;
    CK(cudaMemcpyAsync(part.data(), dp, sizeof(double) * (size_t)(3 * nt), cudaMemcpyDeviceToHost, c->stream),
       "read estimators");
    CK(cudaMemcpyAsync(&m_all, c->e_nbank.p, sizeof m_all, cudaMemcpyDeviceToHost, c->stream), "read site count");
    CK(cudaStreamSynchronize(c->stream), "generation");
    double s_tl = 0.0, s_col = 0.0, s_abs = 0.0;
    for (int64_t b = 0; b < nt; ++b) {
      s_tl = s_tl + part[(size_t)b];
      s_col = s_col + part[(size_t)(nt + b)];
      s_abs = s_abs + part[(size_t)(2 * nt + b)];
    }
    if (m_all > (unsigned long long)cap)
      return set_err(c, MC_ERR_DEVICE, "fission bank full: " + std::to_string(m_all) + " sites for a capacity of " +
                                           std::to_string(cap) + " (fission_bank_capacity)");
    const int64_t m = (int64_t)m_all;
    if (m == 0) return set_err(c, MC_ERR_DEVICE, "no fission sites sampled, cannot sample a new generation");
    // sort_fission_bank: (parent, progeny) order via the per-history counts
    CK(launch_scan(c->e_prog.as<int>(), n, c->e_off.as<int64_t>(), c->e_tmp.as<int64_t>(), c->stream),
       "scan site counts");
    CK(launch_bank_sort(c->e_bank.as<mc_fission_site>(), m, c->e_off.as<int64_t>(), first, n,
                        c->e_sorted.as<mc_fission_site>(), c->stream),
       "sort fission bank");
    // synchronize_bank with one rank (start = 0)
    const int64_t needed = m < n ? n % m : n;
    const double p_sample = (double)needed / (double)m;
    const int copies = m < n ? (int)(n / m) : 0;
    const uint64_t seed0 = stream_seed(skip_ahead((uint64_t)(gen + 1) * kPrnStride), d->seed, kStreamTracking);
    CK(launch_bank_counts(m, seed0, copies, p_sample, c->e_cnt.as<int>(), c->stream), "resample fission bank");
    CK(launch_scan(c->e_cnt.as<int>(), m, c->e_pos.as<int64_t>(), c->e_tmp.as<int64_t>(), c->stream),
       "resample fission bank");
    CK(launch_bank_fill(c->e_sorted.as<mc_fission_site>(), m, c->e_pos.as<int64_t>(), n, c->e_src.as<mc_site>(),
                        c->stream),
       "resample fission bank");
    int64_t off_n = 0;
    CK(cudaMemcpyAsync(&off_n, c->e_off.as<int64_t>() + n, sizeof off_n, cudaMemcpyDeviceToHost, c->stream),
       "read bank size");
    CK(cudaEventRecord(g1, c->stream), "event");
    CK(cudaStreamSynchronize(c->stream), "resample fission bank");
    if (off_n != m)
      return set_err(c, MC_ERR_DEVICE, "fission bank holds " + std::to_string(m) + " sites but histories counted " +
                                           std::to_string(off_n));
    c->e_n = n;
    c->e_m = m;
    // calculate_generation_keff / calculate_average_keff
    const double k_gen = s_tl / (double)n;
    if (!active) {
      keff = k_gen;
    } else {
      ++n_active;
      k_sum0 += k_gen;
      k_sum1 += k_gen * k_gen;
      keff = k_sum0 / (double)n_active;
      if (n_active > 1) keff_std = sqrt((k_sum1 / (double)n_active - keff * keff) / (double)(n_active - 1));
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, g0, g1);
    mc_eigen_gen& o = out[gen];
    o.k_generation = k_gen;
    o.k_collision = s_col / (double)n;
    o.k_absorption = s_abs / (double)n;
    o.keff = keff;
    o.keff_std = keff_std;
    o.leakage = st.leak_weight / (double)n;
    o.n_sites = m;
    o.n_seg = st.n_seg;
    o.n_coll = st.n_coll;
    o.ms = ms;
  }
  return MC_OK;
}

int mc_eigen_source_download(mc_ctx* c, mc_site* out, int64_t n) {
  if (!c || (!out && n > 0)) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  if (n != c->e_n) return set_err(c, MC_ERR_ARG, "n must equal the last eigenvalue run's particles");
  if (n == 0) return MC_OK;
  cudaSetDevice(c->device);
  CK(cudaMemcpyAsync(out, c->e_src.p, sizeof(mc_site) * (size_t)n, cudaMemcpyDeviceToHost, c->stream),
     "download source bank");
  CK(cudaStreamSynchronize(c->stream), "download source bank");
  return MC_OK;
}

int mc_eigen_fission_bank_download(mc_ctx* c, mc_fission_site* out, int64_t capacity, int64_t* n_out) {
  if (!c || !n_out || (!out && capacity > 0)) return MC_ERR_ARG;
  std::lock_guard<std::mutex> g(c->mu);
  *n_out = c->e_m;
  const int64_t k = std::min(capacity, c->e_m);
  if (k <= 0) return MC_OK;
  cudaSetDevice(c->device);
  CK(cudaMemcpyAsync(out, c->e_sorted.p, sizeof(mc_fission_site) * (size_t)k, cudaMemcpyDeviceToHost, c->stream),
     "download fission bank");
  CK(cudaStreamSynchronize(c->stream), "download fission bank");
  return MC_OK;
}

}  // extern "C"

// ===========================================================================
// Read-only views of a context for entry points defined in other files.
namespace mc {

std::mutex& ctx_mutex(mc_ctx* c) { return c->mu; }

void ctx_set_error(mc_ctx* c, const std::string& msg) { c->err = msg; }

void ctx_set_stats(mc_ctx* c, const mc_stats& s) { c->last = s; }

bool ctx_sums(mc_ctx* c, double** sum, double** sumsq) {
  *sum = c->d_sum.as<double>();
  *sumsq = c->d_sumsq.as<double>();
  return *sum && *sumsq;
}

void ctx_add_batches(mc_ctx* c, int64_t n) { c->batches += n; }

bool ctx_serving(mc_ctx* c) { return c->serving; }

bool ctx_view(mc_ctx* c, CtxView* v) {
  v->device = c->device;
  v->n_sm = c->n_sm;
  v->stream = c->stream;
  v->n_tet = c->mesh.n_tet;
  v->n_tally = c->n_tally;
  v->ts = c->tspec;
  v->two_d = c->two_d;
  v->z2d = c->z2d;
  v->n_mat = (int)c->xs.mat_ids.size();
  v->rays_on = c->ray_n > 0 && c->ray_cap > 0;
  const bool tables = c->have_mesh && !c->nucs.empty() && !c->mats.empty() && !c->xs_dirty && !c->tmat_dirty &&
                      !c->bc_dirty;
  v->ready = tables && c->have_src;
  double dg = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double e = c->mesh.bbox_hi[k] - c->mesh.bbox_lo[k];
    dg += e * e;
  }
  v->tol = (float)(1e-6 * sqrt(dg));
  if (!tables) return false;
  v->M = dev_mesh(c);
  v->X = dev_xs(c);
  v->S = dev_source(c);
  return v->ready;
}

void ctx_set_serving(mc_ctx* c, bool on) { c->serving = on; }

}  // namespace mc

namespace mc {

int ctx_prepare(mc_ctx* c) {
  cudaSetDevice(c->device);
  return ensure_device_tables(c);
}

int ctx_event_state(mc_ctx* c, int64_t cap, CtxEvent* out) {
  int rc = ensure_bank(c, std::max(cap, c->bank_cap));
  if (rc) return rc;
  out->B = dev_bank(c);
  if (!bank_complete(out->B)) return set_err(c, MC_ERR_STATE, "internal: particle bank incomplete");
  out->Q = dev_queues(c);
  out->ctl = c->d_ctl.as<EventCtl>();
  out->counters = c->d_counters.as<unsigned long long>();
  out->leak_w = c->d_leak_w.as<double>();
  return MC_OK;
}

int ctx_fail(mc_ctx* c, int code, const std::string& msg) { return set_err(c, code, msg); }

// Copies SUM and SUM_SQ (and the batch count) aside (restore = 0) or back
// (restore = 1), so that trial runs which fold batches leave no trace.
int accum_snapshot(mc_ctx* c, int restore) {
  std::lock_guard<std::mutex> lock(c->mu);
  if (!c->d_sum.p || !c->d_sumsq.p) return MC_OK;  // nothing accumulated yet
  const size_t n = c->d_sum.bytes;
  cudaError_t e = cudaSuccess;
  if (!restore) {
    if (c->d_accum_save.bytes != 2 * n) e = c->d_accum_save.alloc(2 * n);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(c->d_accum_save.p, c->d_sum.p, n, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync((char*)c->d_accum_save.p + n, c->d_sumsq.p, n, cudaMemcpyDeviceToDevice, c->stream);
    c->batches_save = c->batches;
  } else {
    if (c->d_accum_save.bytes != 2 * n) return set_err(c, MC_ERR_STATE, "no saved accumulators");
    e = cudaMemcpyAsync(c->d_sum.p, c->d_accum_save.p, n, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(c->d_sumsq.p, (char*)c->d_accum_save.p + n, n, cudaMemcpyDeviceToDevice, c->stream);
    c->batches = c->batches_save;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return set_err(c, MC_ERR_CUDA, std::string("accumulator snapshot: ") + cudaGetErrorString(e));
  return MC_OK;
}

}  // namespace mc
