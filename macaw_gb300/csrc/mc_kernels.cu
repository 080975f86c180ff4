// mc_kernels.cu -- tracking kernels for sm_103a.
//
// Two execution forms over the same per-particle steps (mc_device.cuh):
//  * history: a persistent grid where each thread runs whole histories,
//    birth to death, one after another;
//  * event: a device-resident particle bank and four event queues (XS
//    lookup, advance, collide, refill).  Each launch works on one event
//    type, so warps stay coherent; queues are filled with warp-aggregated
//    atomics.  Grids are persistent and loop over the device-side queue
//    lengths, so the host never needs the counts to launch.
#include <cooperative_groups.h>

#include "mc_kernels.h"

namespace cg = cooperative_groups;

namespace mc {

namespace {

// Event counters of one launch, accumulated in shared memory (one set per
// block) so that no thread carries them in registers through its walk.
// Declared by MC_COUNTERS at the top of a kernel, which every thread of the
// block executes; flush() is reached by every thread at the end.
struct LocalCounters {
  unsigned long long* c;
  double* leak_w;
  __device__ __forceinline__ void add(int k, unsigned long long v) {
    if (v) atomicAdd(c + k, v);
  }
  __device__ __forceinline__ void add_leak(double w) { atomicAdd(leak_w, w); }
};

#define MC_COUNTERS(L)                                          \
  __shared__ unsigned long long L##_c[kNumCounters];            \
  __shared__ double L##_w;                                      \
  LocalCounters L{L##_c, &L##_w};                               \
  for (int i_ = threadIdx.x; i_ < kNumCounters; i_ += blockDim.x) L##_c[i_] = 0; \
  if (threadIdx.x == 0) L##_w = 0.0;                            \
  __syncthreads()

__device__ __forceinline__ void flush(LocalCounters& L, unsigned long long* g, double* leak_w) {
  __syncthreads();
  for (int i = threadIdx.x; i < kNumCounters; i += blockDim.x)
    if (L.c[i]) atomicAdd(g + i, L.c[i]);
  if (threadIdx.x == 0 && *L.leak_w != 0.0) atomicAdd(leak_w, *L.leak_w);
}

// In-flight counter of a tally slot, one atomic per group of converged
// lanes with the same slot (births and deaths come in warp-wide bursts on
// a handful of addresses).
__device__ __forceinline__ void live_add(int* live, int tag, int v) {
  cg::coalesced_group g = cg::coalesced_threads();
  cg::coalesced_group same = cg::labeled_partition(g, tag);
  if (same.thread_rank() == 0) atomicAdd(live + tag, v * (int)same.size());
}

// Batch tally a particle scores into.
__device__ __forceinline__ double* tally_of(const RunArgs& a, int tag) {
  return tag ? a.tally2 + (int64_t)(tag - 1) * a.n_tally : a.tally;
}

// End of a history: closing hash word, counters, optional trace record.
__device__ __forceinline__ void finish(Particle& p, const RunArgs& a, LocalCounters& L) {
  if (a.live) live_add(a.live, p.tag, -1);
  p.hash = fnv(p.hash, (uint64_t)(16 + p.status));
  L.add(kCntSeg, (unsigned long long)p.n_seg);
  L.add(kCntColl, (unsigned long long)p.n_coll);
  L.add(kCntHist, 1);
  switch (p.status) {
    case kLeaked: L.add(kCntLeak, 1); L.add_leak(p.wgt); break;
    case kAbsorbed: L.add(kCntAbsorb, 1); break;
    case kCutoff: L.add(kCntCutoff, 1); break;
    case kStuck: L.add(kCntStuck, 1); break;
    case kLost: L.add(kCntLost, 1); break;
    default: L.add(kCntBadXS, 1); break;
  }
  if (a.eig.on) {  // the history's keff sum and site count (OpenMC event_death)
    const int64_t h = p.id - 1 - a.eig.first;
    a.eig.ktl[h] = p.ktl;
    a.eig.prog[h] = p.n_prog;
  }
  if (a.traces) {
    mc_trace t;
    t.id = p.id;
    t.hash = p.hash;
    t.status = p.status;
    t.n_seg = p.n_seg;
    t.n_coll = p.n_coll;
    t.elem = p.elem;
    t.face = p.face;
    t.pad = 0;
    t.E = p.E;
    t.x = p.x;
    t.y = p.y;
    t.z = p.z;
    a.traces[p.id - 1 - a.first] = t;
  }
}

// Cross-section event: Sigma_t of the current element's material (and, when
// the problem has at most four materials, of every material, so later
// material changes at this energy hit the cache); false if unusable.
// f32: the mixed-precision form's float interpolation (macro_total32).
// eig: nu*Sigma_f of each evaluated material too.
// c, c32: grid cursors shared by every material evaluated at this energy.
__device__ __forceinline__ double eval_xs(const DevXS& X, int mat, double E, int k, bool f32, bool eig,
                                          double& nf, GridCursor& c, GridCursor32& c32) {
  nf = 0.0;
  if (f32) {
    float n32 = 0.0f;
    const double s = eig ? widen(macro_total32<true>(X, mat, E, k, c32, &n32))
                         : widen(macro_total32(X, mat, E, k, c32));
    nf = widen(n32);
    return s;
  }
  return eig ? macro_total_nuf(X, mat, E, k, nf, c) : macro_total(X, mat, E, k, c);
}

__device__ __forceinline__ bool refresh_xs(const DevMesh& M, const DevXS& X, int n_mat, bool f32, bool eig,
                                          Particle& p, LocalCounters& L) {
  const int mat = __ldg(M.tmat + p.elem);
  if (mat < 0) {
    p.status = kBadXS;
    return false;
  }
  const int k = xs_bucket32(X, p.E);
  double nf;
  GridCursor c;
  GridCursor32 c32;
  const double s = eval_xs(X, mat, p.E, k, f32, eig, nf, c, c32);
  L.add(kCntXS, 1);
  if (!(s > 0.0) || s != s) {
    p.status = kBadXS;
    return false;
  }
  p.sigt = s;
  p.nuf = nf;
  p.mat = mat;
  xs_cache_put<true>(p, mat, s, nf);
  if (n_mat <= 4) {
    for (int m = 0; m < n_mat; ++m) {
      if (m == mat) continue;
      double onf;
      const double o = eval_xs(X, m, p.E, k, f32, eig, onf, c, c32);
      L.add(kCntXS, 1);
      if (o > 0.0) xs_cache_put<true>(p, m, o, onf);
    }
  }
  return true;
}

// eig: also the k-eigenvalue fields (a constant in the walk kernels).
__device__ __forceinline__ void load(const Bank& B, int s, Particle& p, bool eig = false) {
  if (eig) {
    p.nuf = B.nuf[s];
    p.ktl = B.ktl[s];
    p.n_prog = B.n_prog[s];
    const double4_32a n = B.cn[s];
    p.cn0 = n.x; p.cn1 = n.y; p.cn2 = n.z; p.cn3 = n.w;
  }
  p.x = B.x[s]; p.y = B.y[s]; p.z = B.z[s];
  p.u = B.u[s]; p.v = B.v[s]; p.w = B.w[s];
  p.E = B.E[s]; p.wgt = B.wgt[s]; p.sigt = B.sigt[s];
  p.seed = B.seed[s]; p.hash = B.hash[s]; p.id = B.id[s];
  p.elem = B.elem[s]; p.mat = B.mat[s]; p.n_seg = B.n_seg[s]; p.n_coll = B.n_coll[s];
  p.zero_run = B.zero_run[s];
  p.fin = B.fin[s];
  p.tag = B.tag[s];
  p.cm = B.cm[s];
  const double4_32a c = B.cs[s];
  p.cs0 = c.x; p.cs1 = c.y; p.cs2 = c.z; p.cs3 = c.w;
  p.status = kAlive;
  p.face = -1;
}

__device__ __forceinline__ void store(const Bank& B, int s, const Particle& p, bool eig = false) {
  if (eig) {
    B.nuf[s] = p.nuf;
    B.ktl[s] = p.ktl;
    B.n_prog[s] = p.n_prog;
    double4_32a n;
    n.x = p.cn0; n.y = p.cn1; n.z = p.cn2; n.w = p.cn3;
    B.cn[s] = n;
  }
  B.x[s] = p.x; B.y[s] = p.y; B.z[s] = p.z;
  B.u[s] = p.u; B.v[s] = p.v; B.w[s] = p.w;
  B.E[s] = p.E; B.wgt[s] = p.wgt; B.sigt[s] = p.sigt;
  B.seed[s] = p.seed; B.hash[s] = p.hash; B.id[s] = p.id;
  B.elem[s] = p.elem; B.mat[s] = p.mat; B.n_seg[s] = p.n_seg; B.n_coll[s] = p.n_coll;
  B.zero_run[s] = p.zero_run;
  B.fin[s] = p.fin;
  B.tag[s] = p.tag;
  B.cm[s] = p.cm;
  double4_32a c;
  c.x = p.cs0; c.y = p.cs1; c.z = p.cs2; c.w = p.cs3;
  B.cs[s] = c;
}

// The fields one visit of the FP64 walk reads: all but the particle id and
// the eigenvalue site count, which only the end of a history reads.
__device__ __forceinline__ void load_walk(const Bank& B, int s, Particle& p, bool eig) {
  if (eig) {
    p.nuf = B.nuf[s];
    p.ktl = B.ktl[s];
    const double4_32a n = B.cn[s];
    p.cn0 = n.x; p.cn1 = n.y; p.cn2 = n.z; p.cn3 = n.w;
  }
  p.x = B.x[s]; p.y = B.y[s]; p.z = B.z[s];
  p.u = B.u[s]; p.v = B.v[s]; p.w = B.w[s];
  p.E = B.E[s]; p.wgt = B.wgt[s]; p.sigt = B.sigt[s];
  p.seed = B.seed[s]; p.hash = B.hash[s];
  p.elem = B.elem[s]; p.mat = B.mat[s]; p.n_seg = B.n_seg[s]; p.n_coll = B.n_coll[s];
  p.zero_run = B.zero_run[s];
  p.fin = B.fin[s];
  p.tag = B.tag[s];
  p.cm = B.cm[s];
  const double4_32a c = B.cs[s];
  p.cs0 = c.x; p.cs1 = c.y; p.cs2 = c.z; p.cs3 = c.w;
  p.status = kAlive;
  p.face = -1;
}

// The fields one visit of the FP64 walk can change: position, direction
// (reflections), Sigma_t and material (cache hits on entering a material),
// RNG state, hash, element, counts and entry side (with nu*Sigma_f and the
// keff sum in eigenvalue runs).  Energy, id and the cross-section cache
// stay as they are in the bank: the walk hands a cache miss to the XS
// kernel instead of filling the cache itself.
__device__ __forceinline__ void store_walk(const Bank& B, int s, const Particle& p, bool eig) {
  if (eig) {
    B.nuf[s] = p.nuf;
    B.ktl[s] = p.ktl;
  }
  B.x[s] = p.x; B.y[s] = p.y; B.z[s] = p.z;
  B.u[s] = p.u; B.v[s] = p.v; B.w[s] = p.w;
  B.seed[s] = p.seed; B.hash[s] = p.hash;
  // the record's third sector written whole (weight and tag unchanged)
  B.wgt[s] = p.wgt; B.fin[s] = p.fin; B.mat[s] = p.mat; B.n_seg[s] = p.n_seg;
  B.zero_run[s] = p.zero_run; B.tag[s] = p.tag; B.n_coll[s] = p.n_coll;
  B.sigt[s] = p.sigt;
  B.elem[s] = p.elem;
}

__device__ __forceinline__ void birth(const DevMesh& M, const DevXS& X, const DevSource& S,
                                      const RunArgs& a, int64_t h, Particle& p) {
  // which batch / request of the birth sequence this history belongs to
  int64_t id = h + 1;
  uint64_t master = a.master;
  int tag = 0;
  const DevSource* src = &S;
  if (a.req) {
    const int64_t r = h - a.first;
    int lo = 0, hi = a.n_req - 1;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (r < a.req[mid].end) hi = mid;
      else lo = mid + 1;
    }
    const DevRequest& q = a.req[lo];
    id = q.first_id + (r - q.start) + 1;
    master = q.seed;
    tag = q.slot;
    if (q.has_src) src = &q.src;
  }
  mc_site o;
  const Skip k = skip_ahead((uint64_t)id * kPrnStride);
  if (a.sites) o = a.sites[h - a.first];
  else if (a.precision == MC_PREC_MIXED) sample_source32(X, *src, k, master, o);
  else sample_source(X, *src, k, master, o);
  if (a.two_d) {
    o.z = a.z2d;
    planar_dir(o.u, o.v, o.w);
  }
  start(M, o, id - 1, k, master, p);
  p.tag = tag;
  if (a.live) live_add(a.live, p.tag, 1);
}

// Append slot to a queue with one atomic per converged group of lanes.
__device__ __forceinline__ void push(int* q, int* cnt, int slot) {
  cg::coalesced_group g = cg::coalesced_threads();
  int base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(cnt, (int)g.size());
  base = g.shfl(base, 0);
  q[base + g.thread_rank()] = slot;
}

// Return a slot to the free ring (slots of ended histories wait there until
// births are allowed).
__device__ __forceinline__ void push_free(const EventQueues& Q, EventCtl* ctl, int slot, int64_t cap) {
  cg::coalesced_group g = cg::coalesced_threads();
  unsigned long long base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(&ctl->free_tail, (unsigned long long)g.size());
  base = g.shfl(base, 0);
  Q.free_slots[(base + g.thread_rank()) % (unsigned long long)cap] = slot;
}

// Births allowed in this iteration: free slots available, histories left
// below the birth limit.
__device__ __forceinline__ long long births_now(const EventCtl* ctl, int64_t n) {
  const long long base = *(volatile const long long*)&ctl->next_hist;
  const long long lim0 = *(volatile const long long*)&ctl->birth_limit;
  const long long lim = lim0 < n ? lim0 : n;
  const long long avail = (long long)(*(volatile const unsigned long long*)&ctl->free_tail -
                                      *(volatile const unsigned long long*)&ctl->free_head);
  const long long left = lim - base;
  return left < avail ? (left > 0 ? left : 0) : avail;
}

// ---------------------------------------------------------------------------
// History form.
template <int kPrec, bool kEig>
__global__ void __launch_bounds__(256) k_history(DevMesh M, DevXS X, DevSource S, RunArgs a) {
  MC_COUNTERS(L);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    Particle p;
    birth(M, X, S, a, a.first + i, p);
    unsigned long long nxs = 0, nfb = 0;
    if (kPrec == MC_PREC_FP64) {
      float sigt32 = 0.0f;
      float uf = narrow(p.u), vf = narrow(p.v), wf = narrow(p.w);
      while (p.status == kAlive) {
        const int r = segment_fp64g<true, false, true, kEig>(M, X, p, uf, vf, wf, tally_of(a, p.tag), a.ts,
                                                             sigt32, nxs);
        if (r == 1) {
          score_collision(X, a.ts, tally_of(a, p.tag), p);
          collide<kEig>(X, p, a.two_d, a.eig);
        }
        if (r == 1 || r == 5) {
          uf = narrow(p.u);
          vf = narrow(p.v);
          wf = narrow(p.w);
        }
      }
    } else {
      Geo32 g;
      geo_load(p, g);
      float inv_sig = 0.0f;
      while (p.status == kAlive) {
        const int r = segment_mixed<true, false, kEig>(M, X, p, g, tally_of(a, p.tag), a.ts, inv_sig, a.tol, nxs,
                                                        nfb);
        if (r == 1) {
          geo_store(g, p);
          score_collision(X, a.ts, tally_of(a, p.tag), p);
          collide<kEig>(X, p, a.two_d, a.eig);
          geo_load(p, g);
        }
      }
      geo_store(g, p);
    }
    L.add(kCntXS, nxs);
    L.add(kCntFallback, nfb);
    finish(p, a, L);
  }
  flush(L, a.counters, a.leak_w);
}

// ---------------------------------------------------------------------------
// Event form.

// Births of histories [0, min(n, cap)) into slots of the same index.
__global__ void __launch_bounds__(256) k_ev_init(DevMesh M, DevXS X, DevSource S, RunArgs a,
                                                 Bank B, EventQueues Q, EventCtl* ctl, int64_t limit) {
  MC_COUNTERS(L);
  int64_t m = a.n < B.cap ? a.n : B.cap;
  if (limit < m) m = limit;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
    Particle p;
    birth(M, X, S, a, a.first + i, p);
    if (p.status != kAlive) {
      finish(p, a, L);
      push_free(Q, ctl, (int)i, B.cap);
      continue;
    }
    store(B, (int)i, p, a.eig.on);
    push(Q.xs[0], &ctl->n_xs[0], (int)i);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->next_hist = m;
    ctl->birth_limit = limit;
  }
  flush(L, a.counters, a.leak_w);
}

template <bool kEig>
__global__ void __launch_bounds__(256) k_ev_xs(DevMesh M, DevXS X, RunArgs a, Bank B,
                                               EventQueues Q, EventCtl* ctl, int par) {
  MC_COUNTERS(L);
  const int n = *(volatile int*)&ctl->n_xs[par];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int s = Q.xs[par][i];
    // only the fields a cross-section event reads: element, energy, cache
    Particle p;
    p.elem = B.elem[s];
    p.E = B.E[s];
    p.cm = B.cm[s];
    const double4_32a c0 = B.cs[s];
    p.cs0 = c0.x; p.cs1 = c0.y; p.cs2 = c0.z; p.cs3 = c0.w;
    const bool eig = kEig;
    if (eig) {
      const double4_32a n0 = B.cn[s];
      p.cn0 = n0.x; p.cn1 = n0.y; p.cn2 = n0.z; p.cn3 = n0.w;
    }
    p.status = kAlive;
    const bool f32 = a.precision == MC_PREC_MIXED;
    if (refresh_xs(M, X, a.n_mat, f32, eig, p, L)) {
      B.sigt[s] = p.sigt;
      B.mat[s] = p.mat;
      B.cm[s] = p.cm;
      double4_32a c;
      c.x = p.cs0; c.y = p.cs1; c.z = p.cs2; c.w = p.cs3;
      B.cs[s] = c;
      if (eig) {
        B.nuf[s] = p.nuf;
        double4_32a n;
        n.x = p.cn0; n.y = p.cn1; n.z = p.cn2; n.w = p.cn3;
        B.cn[s] = n;
      }
      if (f32) {  // the cached values are floats widened: their float inverses
        B.cinv[s] = make_float4(p.cm.x >= 0 ? 1.0f / narrow(p.cs0) : 0.0f, p.cm.y >= 0 ? 1.0f / narrow(p.cs1) : 0.0f,
                                p.cm.z >= 0 ? 1.0f / narrow(p.cs2) : 0.0f, p.cm.w >= 0 ? 1.0f / narrow(p.cs3) : 0.0f);
      }
      push(Q.adv[par], &ctl->n_adv[par], s);
    } else {
      load(B, s, p, eig);  // the history ends: all of it
      p.status = kBadXS;
      finish(p, a, L);
      push_free(Q, ctl, s, B.cap);
    }
  }
  flush(L, a.counters, a.leak_w);
}

// Next 32 advance-queue entries for the calling warp (all 32 lanes call it
// together).  Warps take chunks as they finish, so a warp whose particles
// walk far never holds up queue entries a faster warp could take.
__device__ __forceinline__ int take_chunk(int* head) {
  int base = 0;
  if ((threadIdx.x & 31) == 0) base = atomicAdd(head, 32);
  return __shfl_sync(0xffffffffu, base, 0);
}

// Segment walk, one queued particle per lane, queue entries taken by warp
// chunks.
template <int kPrec, bool kRays, bool kEig>
__global__ void __launch_bounds__(256) k_ev_advance_static(DevMesh M, DevXS X, RunArgs a, Bank B,
                                                           EventQueues Q, EventCtl* ctl, int par) {
  MC_COUNTERS(L);
  const int n = *(volatile int*)&ctl->n_adv[par];
  const int nxt = par ^ 1;
  for (;;) {
    const int i = take_chunk(&ctl->adv_head) + (int)(threadIdx.x & 31);
    if (__shfl_sync(0xffffffffu, i, 0) >= n) break;
    if (i >= n) continue;
    const int s = Q.adv[par][i];
    Particle p;
    load(B, s, p, kEig);
    const int seg0 = p.n_seg;
    unsigned long long nxs = 0, nfb = 0;
    int r = 0;
    int k = 0;
    if (kPrec == MC_PREC_FP64) {
      float sigt32 = narrow(p.sigt);
      float uf = narrow(p.u), vf = narrow(p.v), wf = narrow(p.w);
      for (;;) {
        r = segment_fp64g<false, false, kRays, kEig>(M, X, p, uf, vf, wf, tally_of(a, p.tag), a.ts, sigt32, nxs);
        if (r == 5) {
          uf = narrow(p.u);
          vf = narrow(p.v);
          wf = narrow(p.w);
          r = 0;
        }
        if (r != 0) break;
        if (a.max_seg > 0 && ++k >= a.max_seg) {
          r = 4;
          break;
        }
      }
    } else {
      Geo32 g;
      geo_load(p, g);
      float inv_sig = (float)(1.0 / p.sigt);
      for (;;) {
        r = segment_mixed<false, false, kEig>(M, X, p, g, tally_of(a, p.tag), a.ts, inv_sig, a.tol, nxs, nfb);
        if (r != 0) break;
        if (a.max_seg > 0 && ++k >= a.max_seg) {
          r = 4;
          break;
        }
      }
      geo_store(g, p);
    }
    L.add(kCntFallback, nfb);
    L.add(kCntSegWalk, (unsigned long long)(p.n_seg - seg0));
    if (r == 2) {
      finish(p, a, L);
      push_free(Q, ctl, s, B.cap);
      continue;
    }
    store(B, s, p, kEig);
    if (r == 1) push(Q.coll, &ctl->n_coll, s);
    else if (r == 3) push(Q.xs[nxt], &ctl->n_xs[nxt], s);
    else push(Q.adv[nxt], &ctl->n_adv[nxt], s);
  }
  flush(L, a.counters, a.leak_w);
}

// A fixed-source FP64 visit also ends, for every lane still walking, once
// fewer than this many lanes of a full warp are: the FP64 pipe issues for
// all 32 lanes, so a warp kept busy by a few long visits wastes it (the
// particles are re-queued where they stand).  12-16 lanes ran 98.2-98.7M
// histories/s on the 2M-tet lattice against 96.8M without; 20 ran 97.2M.
// The mixed walk, bound by its record loads instead, gained nothing.
constexpr int kWalkMinLanes = 14;

// FP64 segment walk for the default tally (no ray recording): each lane
// walks the particles of its warp's queue chunks one visit at a time with
// segment_fp64c, whose element records are loaded one step ahead.
// kBlocks: resident 128-thread blocks per SM it is compiled for.  Five cap
// it at 96 registers (a few spilled bytes; the keff score's variant spills
// more) and give 20 warps per SM, four leave it the registers it takes
// unconstrained and 16 warps.  Which is faster depends on the workload: on
// the 2M-tet lattice five ran 78.5M histories/s against 76.8M, on the
// 41M-tet core four ran 5.57M against 5.37M, and the k-eigenvalue walk
// ran 20.7M with four against 20.0M with five.
template <bool kEig, int kBlocks>
__global__ void __launch_bounds__(128, kBlocks) k_ev_advance_fp64(DevMesh M, DevXS X, RunArgs a, Bank B, EventQueues Q,
                                                         EventCtl* ctl, int par) {
  MC_COUNTERS(L);
  const int n = *(volatile int*)&ctl->n_adv[par];
  const int nxt = par ^ 1;
  for (;;) {
    const int i = take_chunk(&ctl->adv_head) + (int)(threadIdx.x & 31);
    if (__shfl_sync(0xffffffffu, i, 0) >= n) break;
    // the lane floor applies to full chunks only: the queue's last, partial
    // chunk would otherwise end its visits after every segment
    const int min_lanes = (!kEig && __ballot_sync(0xffffffffu, i < n) == 0xffffffffu) ? kWalkMinLanes : 0;
    if (i >= n) continue;
    const int s = Q.adv[par][i];
    Particle p;
    load_walk(B, s, p, kEig);
    float4 O01, O23, D;
    int4 nb4;
    load_oct(M, p.elem, O01, O23, D, nb4);
    int mnext = p.mat < 0 ? __ldg(M.tmat + p.elem) : 0;
    const int seg0 = p.n_seg;
    unsigned long long nxs = 0;
    int r = 0, k = 0;
    float sigt32 = narrow(p.sigt);
    float uf = narrow(p.u), vf = narrow(p.v), wf = narrow(p.w);
    double* const tal = tally_of(a, p.tag);
    for (;;) {
      r = segment_fp64c<kEig>(M, X, p, uf, vf, wf, O01, O23, D, nb4, mnext, tal, a.ts, sigt32, nxs);
      if (r == 5) {
        uf = narrow(p.u);
        vf = narrow(p.v);
        wf = narrow(p.w);
        r = 0;
      }
      if (r != 0) break;
      if (a.max_seg > 0 && ++k >= a.max_seg) {
        r = 4;
        break;
      }
      if (__popc(__activemask()) < min_lanes) {
        r = 4;
        break;
      }
    }
    L.add(kCntSegWalk, (unsigned long long)(p.n_seg - seg0));
    if (r == 2) {
      p.id = B.id[s];
      if (kEig) p.n_prog = B.n_prog[s];
      finish(p, a, L);
      push_free(Q, ctl, s, B.cap);
      continue;
    }
    store_walk(B, s, p, kEig);
    if (r == 1) push(Q.coll, &ctl->n_coll, s);
    else if (r == 3) push(Q.xs[nxt], &ctl->n_xs[nxt], s);
    else push(Q.adv[nxt], &ctl->n_adv[nxt], s);
  }
  flush(L, a.counters, a.leak_w);
}

// Take the next advance-queue entry (one atomic per converged lane group).
__device__ __forceinline__ int take(int* head) {
  cg::coalesced_group g = cg::coalesced_threads();
  int base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(head, (int)g.size());
  return g.shfl(base, 0) + (int)g.thread_rank();
}

// Segment walk.  A lane whose particle reaches an event (collision, XS
// miss, end of history, segment budget) hands it on and immediately takes
// the next queued particle, so warps stay full until the queue drains
// instead of waiting for their longest walk.
template <int kPrec>
__global__ void __launch_bounds__(256) k_ev_advance(DevMesh M, DevXS X, RunArgs a, Bank B,
                                                    EventQueues Q, EventCtl* ctl, int par) {
  MC_COUNTERS(L);
  const int n = *(volatile int*)&ctl->n_adv[par];
  const int nxt = par ^ 1;
  const int* q = Q.adv[par];
  Particle p;
  Geo32 g;
  float f32 = 0.0f;  // FP64: float Sigma_t; mixed: float 1/Sigma_t
  int s = -1, k = 0, seg0 = 0;
  unsigned long long nxs = 0, nfb = 0, nwalk = 0;
  {
    const int i = take(&ctl->adv_head);
    if (i < n) {
      s = q[i];
      load(B, s, p);
      seg0 = p.n_seg;
      geo_load(p, g);
      f32 = (kPrec == MC_PREC_FP64) ? narrow(p.sigt) : (float)(1.0 / p.sigt);
    }
  }
  while (__any_sync(0xffffffffu, s >= 0)) {
    if (s < 0) continue;
    int r;
    if (kPrec == MC_PREC_FP64) {
      r = segment_fp64g<false>(M, X, p, g.u, g.v, g.w, tally_of(a, p.tag), a.ts, f32, nxs);
      if (r == 5) {
        g.u = narrow(p.u);
        g.v = narrow(p.v);
        g.w = narrow(p.w);
        r = 0;
      }
    } else {
      r = segment_mixed<false>(M, X, p, g, tally_of(a, p.tag), a.ts, f32, a.tol, nxs, nfb);
    }
    if (r == 0) {
      if (a.max_seg <= 0 || ++k < a.max_seg) continue;
      r = 4;
    }
    if (kPrec != MC_PREC_FP64) geo_store(g, p);
    nwalk += (unsigned long long)(p.n_seg - seg0);
    if (r == 2) {
      finish(p, a, L);
      push_free(Q, ctl, s, B.cap);
    } else {
      store(B, s, p);
      if (r == 1) push(Q.coll, &ctl->n_coll, s);
      else if (r == 3) push(Q.xs[nxt], &ctl->n_xs[nxt], s);
      else push(Q.adv[nxt], &ctl->n_adv[nxt], s);
    }
    k = 0;
    s = -1;
    const int i = take(&ctl->adv_head);
    if (i < n) {
      s = q[i];
      load(B, s, p);
      seg0 = p.n_seg;
      geo_load(p, g);
      f32 = (kPrec == MC_PREC_FP64) ? narrow(p.sigt) : (float)(1.0 / p.sigt);
    }
  }
  L.add(kCntFallback, nfb);
  L.add(kCntSegWalk, nwalk);
  flush(L, a.counters, a.leak_w);
}

// One visit of the compact mixed-precision walk to the particle in bank
// slot s: float position and direction, float 1/Sigma_t for the cached
// materials, 64-bit RNG state and trace hash; only the bank fields the walk
// reads or changes move, the rest of a particle is touched only when its
// history ends here.  Same arithmetic as segment_mixed.  Walks until an
// event or max_seg segments (max_seg <= 0: until an event) and returns r:
// 1 collision, 2 history ended (finished here), 3 cross-section event due,
// 4 segment budget.  queue: hand the particle to the queue of its next
// event (the event loop); otherwise the caller handles the event.
// x + xl += d * u with the rounding error of the float sum kept in xl
// (Knuth's TwoSum, exact for any magnitudes).
__device__ __forceinline__ void advance2(float& x, float& xl, float d, float u) {
  const float t = fmaf(d, u, xl);
  const float s2 = x + t;
  const float bb = s2 - x;
  xl = (x - (s2 - bb)) + (t - bb);
  x = s2;
}

template <bool kEig = false>
__device__ __forceinline__ int mixed_visit(const DevMesh& M, const RunArgs& a, const Bank& B, const EventQueues& Q,
                                           EventCtl* ctl, int nxt, int s, int max_seg, float tol, bool hashing,
                                           bool queue, LocalCounters& L) {
  // (queue = false: the tail kernel; its segments are not walk-launch segments)
  // bank state is read once and written once per visit: streaming
  // (evict-first) accesses, so the L2 keeps the element records
  // position as float (x, y, z) plus a float low part (xl, yl, zl): the
  // walk's plane tests use the float part; the low part carries what each
  // advance rounds away, so float rounding does not accumulate along the
  // walk (the bank keeps the double sum between visits)
  const double xd = __ldcs(B.x + s), yd = __ldcs(B.y + s), zd = __ldcs(B.z + s);
  float x = narrow(xd), y = narrow(yd), z = narrow(zd);
  float xl = narrow(xd - widen(x)), yl = narrow(yd - widen(y)), zl = narrow(zd - widen(z));
  float u = narrow(__ldcs(B.u + s)), v = narrow(__ldcs(B.v + s)), w = narrow(__ldcs(B.w + s));
  int elem = __ldcs(B.elem + s), fin = __ldcs(B.fin + s), mat = __ldcs(B.mat + s), n_seg = __ldcs(B.n_seg + s),
      zrun = __ldcs(B.zero_run + s);
  const int seg0 = n_seg;
  uint64_t seed = __ldcs((const unsigned long long*)(B.seed + s));
  uint64_t hash = __ldcs((const unsigned long long*)(B.hash + s));
  const double wgt = __ldcs(B.wgt + s);
  const bool unit_w = __double_as_longlong(wgt) == __double_as_longlong(1.0);
  double* const tal = tally_of(a, B.tag[s]);
  const int4 cm = B.cm[s];
  const float4 ci = B.cinv[s];
  int slot = -1;  // cache slot whose Sigma_t is current, if the walk changed material
  // the cached float 1/Sigma_t of the current material (set below when mat < 0)
  float inv_sig = 0.0f;
  // k-eigenvalue runs: nu*Sigma_f of the cached materials (float) and the
  // visit's sum of score * nu*Sigma_f, added to the history's FP64
  // track-length keff sum when the visit ends
  float4 cnf = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  float nuf = 0.0f, kacc = 0.0f;
  if (kEig) {
    const double4_32a c = B.cn[s];
    cnf = make_float4(narrow(c.x), narrow(c.y), narrow(c.z), narrow(c.w));
  }
  if (mat >= 0) {
    const int sl = xs_cache_slot(cm, mat);
    inv_sig = sl == 0 ? ci.x : sl == 1 ? ci.y : sl == 2 ? ci.z : ci.w;
    if (kEig) nuf = sl == 0 ? cnf.x : sl == 1 ? cnf.y : sl == 2 ? cnf.z : cnf.w;
  }
  int r = 0, face = -1;
  int k = 0;
  // The record of the element being walked is loaded one step ahead: at
  // each crossing the neighbour's planes, entries and (after a flagged
  // side) material are requested before that segment's tally, hash and
  // position update, so the loads are in flight while those run.
  float4 O01, O23, D;  // octahedral record (two 32-byte sectors)
  int4 nb4;
  int mnext = 0;  // material of elem, valid while mat < 0
  {
    const TetOct* T = M.teto + elem;
    O01 = __ldg(&T->oct01);
    O23 = __ldg(&T->oct23);
    D = __ldg(&T->d);
    nb4 = __ldg(&T->nbr);
    if (mat < 0) mnext = __ldg(M.tmat + elem);
  }
  for (;;) {
    if (n_seg >= M.max_seg || zrun >= kMaxZeroRun) {
      r = 2;
      face = -2;  // stuck
      break;
    }
    // this segment's draw depends on no load: formed while they land,
    // committed to the RNG state only when the segment is scored
    const uint64_t seed_n = kPrnMult * seed + kPrnAdd;
    uint64_t wv = ((seed_n >> ((seed_n >> 59u) + 5u)) ^ seed_n) * 12605985483714917081ULL;
    wv = (wv >> 43u) ^ wv;
    const float lnxi = -__logf((float)(uint32_t)(wv >> 32) * 2.3283064365386963e-10f);
    if (mat < 0) {  // after a side flagged kMatChange
      const int m = mnext;
      const int sl = m < 0 ? -1 : xs_cache_slot(cm, m);
      if (sl < 0) {
        r = (m < 0) ? 2 : 3;
        if (m < 0) face = -3;  // no material: bad cross section
        break;
      }
      mat = m;
      slot = sl;
      inv_sig = sl == 0 ? ci.x : sl == 1 ? ci.y : sl == 2 ? ci.z : ci.w;
      if (kEig) nuf = sl == 0 ? cnf.x : sl == 1 ? cnf.y : sl == 2 ? cnf.z : cnf.w;
    }
    int bf = -1;
    float t1 = 3.0e38f, t2 = 3.0e38f;
    // branch-free: every lane runs the same instructions for every side
    // (a side that is the entry side or faces away gets t = 3e38)
    auto side = [&](const float4& pl, int f) {
      const float den = fmaf(pl.x, u, fmaf(pl.y, v, pl.z * w));
      const float num = pl.w - fmaf(pl.x, x, fmaf(pl.y, y, pl.z * z));
      const float t = (f != fin && den > 0.0f) ? __fdividef(num, den) : 3.0e38f;
      const bool lt1 = t < t1;
      t2 = lt1 ? t1 : fminf(t2, t);
      bf = lt1 ? f : bf;
      t1 = lt1 ? t : t1;
    };
    const float4 P0 = oct_plane(O01.x, O01.y, D.x), P1 = oct_plane(O01.z, O01.w, D.y);
    const float4 P2 = oct_plane(O23.x, O23.y, D.z), P3 = oct_plane(O23.z, O23.w, D.w);
    side(P0, 0);
    side(P1, 1);
    side(P2, 2);
    side(P3, 3);
    float Ls;
    if (bf < 0 || t2 - t1 <= tol || t1 < -tol) {
      L.add(kCntFallback, 1);
      Geo32 g{x, y, z, u, v, w};
      double Ld = 0.0;
      bf = exit_fp64(M, elem, fin, g, Ld);
      if (bf < 0) {
        r = 2;
        face = -2;
        break;
      }
      Ls = (float)Ld;
    } else {
      Ls = fmaxf(t1, 0.0f);
    }
    seed = seed_n;
    const float dist = lnxi * inv_sig;
    const bool cross = dist > Ls;
    const int nb = side_entry(nb4, bf);
    const int next = (nb & (kMatChange - 1)) >> 2;
    if (cross && nb >= 0) {
      const TetOct* T = M.teto + next;
      O01 = __ldg(&T->oct01);
      O23 = __ldg(&T->oct23);
      D = __ldg(&T->d);
      nb4 = __ldg(&T->nbr);
      if (nb & kMatChange) mnext = __ldg(M.tmat + next);
    }
    const float score = cross ? Ls : dist;
    atomicAdd(tal + elem, unit_w ? widen(score) : wgt * widen(score));
    if (kEig) kacc = fmaf(score, nuf, kacc);  // CollisionKernel.C:153-154
    ++n_seg;
    if (Ls == 0.0f) ++zrun;
    else zrun = 0;
    if (!cross) {
      if (hashing) hash = fnv(hash, (uint64_t)elem * 8ULL + 4ULL);
      advance2(x, xl, dist, u);
      advance2(y, yl, dist, v);
      advance2(z, zl, dist, w);
      zrun = 0;
      r = 1;
      break;
    }
    if (hashing) hash = fnv(hash, (uint64_t)elem * 8ULL + (uint64_t)bf);
    advance2(x, xl, Ls, u);
    advance2(y, yl, Ls, v);
    advance2(z, zl, Ls, w);
    if (nb >= 0) {
      if (nb & kMatChange) mat = -2;
      elem = next;
      fin = nb & 3;
    } else {
      const int bid = -1 - nb;
      if (bid < M.n_bid && M.bc_type[bid] == 1) {
        // no load is issued for a boundary side: the record is still this element's
        float4 pb = bf == 0 ? oct_plane(O01.x, O01.y, D.x) : bf == 1 ? oct_plane(O01.z, O01.w, D.y)
                  : bf == 2 ? oct_plane(O23.x, O23.y, D.z) : oct_plane(O23.z, O23.w, D.w);
        const float rn = rsqrtf(fmaf(pb.x, pb.x, fmaf(pb.y, pb.y, pb.z * pb.z)));  // unit normal
        pb.x *= rn;
        pb.y *= rn;
        pb.z *= rn;
        const float t2r = 2.0f * fmaf(u, pb.x, fmaf(v, pb.y, w * pb.z));
        u = fmaf(-t2r, pb.x, u);
        v = fmaf(-t2r, pb.y, v);
        w = fmaf(-t2r, pb.z, w);
        const float nrm = rsqrtf(fmaf(u, u, fmaf(v, v, w * w)));
        u *= nrm;
        v *= nrm;
        w *= nrm;
        fin = -1;
      } else {
        r = 2;
        face = bf;  // leaked through side bf
        break;
      }
    }
    if (a.max_seg > 0 && ++k >= a.max_seg) {
      r = 4;
      break;
    }
  }
  if (queue) L.add(kCntSegWalk, (unsigned long long)(n_seg - seg0));
  if (r == 2) {
    Particle p;
    load(B, s, p, kEig);
    if (kEig) p.ktl = p.ktl + wgt * widen(kacc);
    p.x = widen(x) + widen(xl); p.y = widen(y) + widen(yl); p.z = widen(z) + widen(zl);
    p.u = widen(u); p.v = widen(v); p.w = widen(w);
    p.elem = elem; p.fin = fin; p.mat = mat; p.n_seg = n_seg; p.zero_run = zrun;
    p.seed = seed; p.hash = hash;
    if (face >= 0) {
      p.status = kLeaked;
      p.face = face;
    } else {
      p.status = face == -3 ? kBadXS : kStuck;
    }
    finish(p, a, L);
    if (queue) push_free(Q, ctl, s, B.cap);
    return 2;
  }
  __stcs(B.x + s, widen(x) + widen(xl)); __stcs(B.y + s, widen(y) + widen(yl));
  __stcs(B.z + s, widen(z) + widen(zl));
  __stcs(B.u + s, widen(u)); __stcs(B.v + s, widen(v)); __stcs(B.w + s, widen(w));
  __stcs((unsigned long long*)(B.seed + s), (unsigned long long)seed);
  __stcs((unsigned long long*)(B.hash + s), (unsigned long long)hash);
  // the changed fields of the record's third sector only: re-reading the
  // weight, tag and collision count to write the sector whole put a
  // dependent load before the stores of every visit (164M against 200M
  // histories/s on the 2M-tet lattice)
  __stcs(B.fin + s, fin); __stcs(B.mat + s, mat); __stcs(B.n_seg + s, n_seg);
  __stcs(B.zero_run + s, zrun);
  if (r == 1) B.n_coll[s] = B.n_coll[s] + 1;
  __stcs(B.elem + s, elem);
  if (slot >= 0) {
    const double4_32a c = B.cs[s];
    B.sigt[s] = slot == 0 ? c.x : slot == 1 ? c.y : slot == 2 ? c.z : c.w;
    if (kEig) {
      const double4_32a n = B.cn[s];
      B.nuf[s] = slot == 0 ? n.x : slot == 1 ? n.y : slot == 2 ? n.z : n.w;
    }
  }
  if (kEig) B.ktl[s] = B.ktl[s] + wgt * widen(kacc);
  if (queue) {
    if (r == 1) push(Q.coll, &ctl->n_coll, s);
    else if (r == 3) push(Q.xs[nxt], &ctl->n_xs[nxt], s);
    else push(Q.adv[nxt], &ctl->n_adv[nxt], s);
  }
  return r;
}

// Mixed-precision segment walk (mixed_visit), each lane walking the
// particles of its warp's queue chunks one visit at a time.
template <bool kEig>
__global__ void __launch_bounds__(256, 3) k_ev_advance_mixed(DevMesh M, RunArgs a, Bank B, EventQueues Q,
                                                             EventCtl* ctl, int par) {
  MC_COUNTERS(L);
  const int n = *(volatile int*)&ctl->n_adv[par];
  const int nxt = par ^ 1;
  const float tol = a.tol;
  const bool hashing = a.traces != nullptr;  // the event hash is only reported in traces
  for (;;) {
    const int i = take_chunk(&ctl->adv_head) + (int)(threadIdx.x & 31);
    if (__shfl_sync(0xffffffffu, i, 0) >= n) break;
    if (i >= n) continue;
    const int s = Q.adv[par][i];
    mixed_visit<kEig>(M, a, B, Q, ctl, nxt, s, a.max_seg, tol, hashing, true, L);
  }
  flush(L, a.counters, a.leak_w);
}

template <bool kEig>
__global__ void __launch_bounds__(256) k_ev_collide(DevMesh M, DevXS X, RunArgs a, Bank B,
                                                    EventQueues Q, EventCtl* ctl, int par) {
  MC_COUNTERS(L);
  const int n = *(volatile int*)&ctl->n_coll;
  const int nxt = par ^ 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int s = Q.coll[i];
    // only the fields a collision reads; the rest when the history ends here
    Particle p;
    p.E = B.E[s]; p.wgt = B.wgt[s]; p.sigt = B.sigt[s];
    p.u = B.u[s]; p.v = B.v[s]; p.w = B.w[s];
    p.seed = B.seed[s];
    p.elem = B.elem[s]; p.mat = B.mat[s]; p.tag = B.tag[s];
    p.status = kAlive;
    // fission sites start at the collision point; eigenvalue runs also
    // need the history's id, site count and nu*Sigma_f
    const bool eig = kEig;
    p.id = eig ? B.id[s] : 0;
    p.n_prog = eig ? B.n_prog[s] : 0;
    p.nuf = eig ? B.nuf[s] : 0.0;
    if (X.nusf) {
      p.x = B.x[s]; p.y = B.y[s]; p.z = B.z[s];
    }
    score_collision(X, a.ts, tally_of(a, p.tag), p);
    collide<kEig>(X, p, a.two_d, a.eig);
    if (p.status != kAlive) {
      const int status = p.status;
      const double E = p.E;
      const uint64_t seed = p.seed;
      const int n_prog = p.n_prog;
      load(B, s, p, eig);
      p.status = status;
      p.E = E;
      p.seed = seed;
      p.n_prog = n_prog;
      finish(p, a, L);
      push_free(Q, ctl, s, B.cap);
      continue;
    }
    B.u[s] = p.u; B.v[s] = p.v; B.w[s] = p.w;
    B.E[s] = p.E; B.seed[s] = p.seed; B.mat[s] = p.mat;
    B.cm[s] = p.cm; B.fin[s] = p.fin;
    if (eig) B.n_prog[s] = p.n_prog;
    push(Q.xs[nxt], &ctl->n_xs[nxt], s);
  }
  flush(L, a.counters, a.leak_w);
}

// New histories into free slots: the i-th free slot of the ring takes
// history next_hist + i, as far as histories below the birth limit remain.
__global__ void __launch_bounds__(256) k_ev_refill(DevMesh M, DevXS X, DevSource S, RunArgs a,
                                                   Bank B, EventQueues Q, EventCtl* ctl, int par) {
  MC_COUNTERS(L);
  const long long base = *(volatile long long*)&ctl->next_hist;
  const unsigned long long head = *(volatile unsigned long long*)&ctl->free_head;
  const long long n = births_now(ctl, a.n);
  const int nxt = par ^ 1;
  for (long long i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int s = Q.free_slots[(head + (unsigned long long)i) % (unsigned long long)B.cap];
    Particle p;
    birth(M, X, S, a, a.first + base + i, p);
    if (p.status != kAlive) {
      finish(p, a, L);
      continue;  // slot stays empty for the rest of the run
    }
    store(B, s, p, a.eig.on);
    push(Q.xs[nxt], &ctl->n_xs[nxt], s);
  }
  flush(L, a.counters, a.leak_w);
}

// End of an iteration: consumed queues emptied, births committed (the same
// count the refill computed: no slot is freed between the two launches).
__global__ void k_ev_reset(EventCtl* ctl, int par, int64_t n) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const long long b = births_now(ctl, n);
    ctl->next_hist += b;
    ctl->free_head += (unsigned long long)b;
    ctl->n_xs[par] = 0;
    ctl->n_adv[par] = 0;
    ctl->n_coll = 0;
    ctl->adv_head = 0;
  }
}

// Tail of a batch: every particle still queued runs to completion in one
// launch, one thread per particle, with cross sections and collisions inline.
// Tail of the mixed walk with the default tally (fixed-source or
// k-eigenvalue): the event loop's compact visit without a segment budget,
// with the collision and cross-section events it stops at handled here,
// until the history ends.
template <bool kEig>
__device__ __forceinline__ void mixed_tail(const DevMesh& M, const DevXS& X, const RunArgs& a, const Bank& B,
                                           const EventQueues& Q, EventCtl* ctl, int s, bool need_xs,
                                           LocalCounters& L) {
  const float tol = a.tol;
  const bool hashing = a.traces != nullptr;
  int r = need_xs ? 3 : 0;
  for (;;) {
    if (r == 1 || r == 3) {
      Particle p;
      load(B, s, p, kEig);
      if (r == 1) {
        collide<kEig>(X, p, a.two_d, a.eig);
        if (p.status != kAlive) {
          finish(p, a, L);
          return;
        }
      }
      // only the current material: a lone thread's lookups run one after
      // another, and the walk asks for another material when it enters one
      if (!refresh_xs(M, X, 0, true, kEig, p, L)) {
        finish(p, a, L);
        return;
      }
      store(B, s, p, kEig);
      B.cinv[s] = make_float4(p.cm.x >= 0 ? 1.0f / narrow(p.cs0) : 0.0f, p.cm.y >= 0 ? 1.0f / narrow(p.cs1) : 0.0f,
                              p.cm.z >= 0 ? 1.0f / narrow(p.cs2) : 0.0f, p.cm.w >= 0 ? 1.0f / narrow(p.cs3) : 0.0f);
    }
    r = mixed_visit<kEig>(M, a, B, Q, ctl, 0, s, 0, tol, hashing, false, L);
    if (r == 2) return;
  }
}

template <int kPrec, bool kEig>
__global__ void __launch_bounds__(256) k_ev_finish(DevMesh M, DevXS X, RunArgs a, Bank B,
                                                   EventQueues Q, EventCtl* ctl, int par) {
  MC_COUNTERS(L);
  const int nx = *(volatile int*)&ctl->n_xs[par];
  const int na = *(volatile int*)&ctl->n_adv[par];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nx + na; i += gridDim.x * blockDim.x) {
    const int s = (i < nx) ? Q.xs[par][i] : Q.adv[par][i - nx];
    if (kPrec == MC_PREC_MIXED && !a.ts.general && !a.ts.rays) {
      mixed_tail<kEig>(M, X, a, B, Q, ctl, s, i < nx, L);
      continue;
    }
    Particle p;
    load(B, s, p, kEig);
    unsigned long long nxs = 0, nfb = 0;
    if (kPrec == MC_PREC_FP64 && !a.ts.rays) {
      // the compact FP64 segment: records loaded a step ahead (a tail
      // history is one long chain of dependent loads); cross-section
      // events are evaluated inline for the material entered
      float sigt32 = narrow(p.sigt);
      float uf = narrow(p.u), vf = narrow(p.v), wf = narrow(p.w);
      float4 O01, O23, D;
      int4 nb4;
      load_oct(M, p.elem, O01, O23, D, nb4);
      int mnext = p.mat < 0 ? __ldg(M.tmat + p.elem) : 0;
      double* const tal = tally_of(a, p.tag);
      while (p.status == kAlive) {
        const int r = segment_fp64c<kEig>(M, X, p, uf, vf, wf, O01, O23, D, nb4, mnext, tal, a.ts, sigt32, nxs);
        if (r == 3) {
          const int mat = mnext;  // a material with no cached Sigma_t at this energy
          double nf = 0.0;
          const double sg = kEig ? macro_total_nuf(X, mat, p.E, xs_bucket32(X, p.E), nf) : macro_total(X, mat, p.E);
          ++nxs;
          if (!(sg > 0.0) || sg != sg) {
            p.status = kBadXS;
            break;
          }
          p.sigt = sg;
          if (kEig) p.nuf = nf;
          xs_cache_put<kEig>(p, mat, sg, nf);
          p.mat = mat;
          sigt32 = narrow(sg);
          continue;
        }
        if (r == 1) {
          score_collision(X, a.ts, tal, p);
          collide<kEig>(X, p, a.two_d, a.eig);
          mnext = __ldg(M.tmat + p.elem);  // collide empties the cache: the element's material again
        }
        if (r == 1 || r == 5) {
          uf = narrow(p.u);
          vf = narrow(p.v);
          wf = narrow(p.w);
        }
      }
    } else if (kPrec == MC_PREC_FP64) {
      float sigt32 = narrow(p.sigt);
      float uf = narrow(p.u), vf = narrow(p.v), wf = narrow(p.w);
      while (p.status == kAlive) {
        const int r = segment_fp64g<true, true, true, kEig>(M, X, p, uf, vf, wf, tally_of(a, p.tag), a.ts, sigt32, nxs);
        if (r == 1) {
          score_collision(X, a.ts, tally_of(a, p.tag), p);
          collide<kEig>(X, p, a.two_d, a.eig);
        }
        if (r == 1 || r == 5) {
          uf = narrow(p.u);
          vf = narrow(p.v);
          wf = narrow(p.w);
        }
      }
    } else {
      Geo32 g;
      geo_load(p, g);
      float inv_sig = (p.mat >= 0) ? (float)(1.0 / p.sigt) : 0.0f;
      while (p.status == kAlive) {
        const int r = segment_mixed<true, true, kEig>(M, X, p, g, tally_of(a, p.tag), a.ts, inv_sig, a.tol, nxs, nfb);
        if (r == 1) {
          geo_store(g, p);
          score_collision(X, a.ts, tally_of(a, p.tag), p);
          collide<kEig>(X, p, a.two_d, a.eig);
          geo_load(p, g);
        }
      }
      geo_store(g, p);
    }
    L.add(kCntXS, nxs);
    L.add(kCntFallback, nfb);
    finish(p, a, L);
  }
  flush(L, a.counters, a.leak_w);
}

__global__ void __launch_bounds__(256) k_sample(DevXS X, DevSource S, int64_t first, int64_t n,
                                                uint64_t master, mc_site* out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    mc_site o;
    sample_source(X, S, skip_ahead((uint64_t)(first + i + 1) * kPrnStride), master, o);
    out[i] = o;
  }
}

// Counting sort of the advance queue by a coarse element key, so the warps
// of the walk start in nearby elements (better L1/L2 reuse of tet records).
__global__ void k_sort_copy(const int* __restrict__ q, int* __restrict__ tmp, const EventCtl* ctl, int par) {
  const int n = *(volatile const int*)&ctl->n_adv[par];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) tmp[i] = q[i];
}

__global__ void k_sort_count(const int* __restrict__ tmp, const int* __restrict__ elem, int* cnt, int shift,
                             const EventCtl* ctl, int par) {
  const int n = *(volatile const int*)&ctl->n_adv[par];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    atomicAdd(cnt + (elem[tmp[i]] >> shift), 1);
}

// Exclusive scan of nb counters in one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_sort_scan(int* cnt, int nb) {
  __shared__ int part[1024];
  const int per = (nb + 1023) / 1024;
  const int b0 = threadIdx.x * per;
  int sum = 0;
  for (int i = b0; i < b0 + per && i < nb; ++i) sum += cnt[i];
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = threadIdx.x ? part[threadIdx.x - 1] : 0;
  for (int i = b0; i < b0 + per && i < nb; ++i) {
    const int c = cnt[i];
    cnt[i] = run;
    run += c;
  }
}

__global__ void k_sort_scatter(const int* __restrict__ tmp, const int* __restrict__ elem, int* cnt, int* q,
                               int shift, const EventCtl* ctl, int par) {
  const int n = *(volatile const int*)&ctl->n_adv[par];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int s = tmp[i];
    q[atomicAdd(cnt + (elem[s] >> shift), 1)] = s;
  }
}

__global__ void k_accumulate(double* __restrict__ batch, double* __restrict__ sum,
                             double* __restrict__ sumsq, int64_t n, double inv_w) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double v = batch[i] * inv_w;
    sum[i] += v;
    sumsq[i] += v * v;
    batch[i] = 0.0;
  }
}

}  // namespace

cudaError_t launch_history(const DevMesh& M, const DevXS& X, const DevSource& S, const RunArgs& a,
                           int block, int grid, cudaStream_t st) {
  if (a.eig.on) {
    if (a.precision == MC_PREC_MIXED) k_history<MC_PREC_MIXED, true><<<grid, block, 0, st>>>(M, X, S, a);
    else k_history<MC_PREC_FP64, true><<<grid, block, 0, st>>>(M, X, S, a);
  } else {
    if (a.precision == MC_PREC_MIXED) k_history<MC_PREC_MIXED, false><<<grid, block, 0, st>>>(M, X, S, a);
    else k_history<MC_PREC_FP64, false><<<grid, block, 0, st>>>(M, X, S, a);
  }
  return cudaGetLastError();
}

cudaError_t launch_event_init(const DevMesh& M, const DevXS& X, const DevSource& S,
                              const RunArgs& a, const Bank& B, const EventQueues& Q,
                              EventCtl* ctl, int block, int grid, cudaStream_t st, int64_t birth_limit) {
  cudaError_t e = cudaMemsetAsync(ctl, 0, sizeof(EventCtl), st);
  if (e != cudaSuccess) return e;
  k_ev_init<<<grid, block, 0, st>>>(M, X, S, a, B, Q, ctl, birth_limit);
  return cudaGetLastError();
}

cudaError_t launch_event_iteration(const DevMesh& M, const DevXS& X, const DevSource& S,
                                   const RunArgs& a, const Bank& B, const EventQueues& Q,
                                   EventCtl* ctl, int par, int block, int grid, cudaStream_t st,
                                   int* n_launch, cudaEvent_t adv0, cudaEvent_t adv1) {
  if (a.eig.on) k_ev_xs<true><<<grid, block, 0, st>>>(M, X, a, B, Q, ctl, par);
  else k_ev_xs<false><<<grid, block, 0, st>>>(M, X, a, B, Q, ctl, par);
  if (a.sort_shift >= 0) {
    cudaMemsetAsync(a.sort_cnt, 0, sizeof(int) * (size_t)(a.sort_buckets + 1), st);
    k_sort_copy<<<grid, block, 0, st>>>(Q.adv[par], a.sort_tmp, ctl, par);
    k_sort_count<<<grid, block, 0, st>>>(a.sort_tmp, B.elem, a.sort_cnt, a.sort_shift, ctl, par);
    k_sort_scan<<<1, 1024, 0, st>>>(a.sort_cnt, a.sort_buckets);
    k_sort_scatter<<<grid, block, 0, st>>>(a.sort_tmp, B.elem, a.sort_cnt, Q.adv[par], a.sort_shift, ctl, par);
    if (n_launch) *n_launch += 4;
  }
  if (adv0) cudaEventRecord(adv0, st);
  if (a.eig.on) {
    // k-eigenvalue generations: the walks with the keff score (no lane
    // refill, no ray recording; the compact mixed walk for the default tally)
    if (a.precision == MC_PREC_MIXED && !a.ts.general)
      k_ev_advance_mixed<true><<<grid, block, 0, st>>>(M, a, B, Q, ctl, par);
    else if (a.precision == MC_PREC_MIXED)
      k_ev_advance_static<MC_PREC_MIXED, false, true><<<grid, block, 0, st>>>(M, X, a, B, Q, ctl, par);
    else
      k_ev_advance_fp64<true, 4><<<grid, block < 128 ? block : 128, 0, st>>>(M, X, a, B, Q, ctl, par);
  } else if (a.precision == MC_PREC_MIXED) {
    // the compact walk scores the default tally and records no rays
    if (a.refill || a.ts.general || a.ts.rays) k_ev_advance<MC_PREC_MIXED><<<grid, block, 0, st>>>(M, X, a, B, Q, ctl, par);
    else k_ev_advance_mixed<false><<<grid, block, 0, st>>>(M, a, B, Q, ctl, par);
  } else {
    if (a.refill) k_ev_advance<MC_PREC_FP64><<<grid, block, 0, st>>>(M, X, a, B, Q, ctl, par);
    else if (a.ts.rays) k_ev_advance_static<MC_PREC_FP64, true, false><<<grid, block, 0, st>>>(M, X, a, B, Q, ctl, par);
    else if (a.walk_blocks == 4)
      k_ev_advance_fp64<false, 4><<<grid, block < 128 ? block : 128, 0, st>>>(M, X, a, B, Q, ctl, par);
    else k_ev_advance_fp64<false, 5><<<grid, block < 128 ? block : 128, 0, st>>>(M, X, a, B, Q, ctl, par);
  }
  if (adv1) cudaEventRecord(adv1, st);
  if (a.eig.on) k_ev_collide<true><<<grid, block, 0, st>>>(M, X, a, B, Q, ctl, par);
  else k_ev_collide<false><<<grid, block, 0, st>>>(M, X, a, B, Q, ctl, par);
  k_ev_refill<<<grid, block, 0, st>>>(M, X, S, a, B, Q, ctl, par);
  k_ev_reset<<<1, 32, 0, st>>>(ctl, par, a.n);
  if (n_launch) *n_launch += 5;
  return cudaGetLastError();
}

cudaError_t launch_event_finish(const DevMesh& M, const DevXS& X, const DevSource& S,
                                const RunArgs& a, const Bank& B, const EventQueues& Q,
                                EventCtl* ctl, int par, int block, int grid, cudaStream_t st) {
  (void)S;
  if (a.eig.on) {
    if (a.precision == MC_PREC_MIXED) k_ev_finish<MC_PREC_MIXED, true><<<grid, block, 0, st>>>(M, X, a, B, Q, ctl, par);
    else k_ev_finish<MC_PREC_FP64, true><<<grid, block, 0, st>>>(M, X, a, B, Q, ctl, par);
  } else {
    if (a.precision == MC_PREC_MIXED) k_ev_finish<MC_PREC_MIXED, false><<<grid, block, 0, st>>>(M, X, a, B, Q, ctl, par);
    else k_ev_finish<MC_PREC_FP64, false><<<grid, block, 0, st>>>(M, X, a, B, Q, ctl, par);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Persistent form: one launch runs many batches, of one or more problems.
// Every lane loops on its own (no barrier, no warp-wide operation):
//   1. fold work first, when batches share tally slots (fold_in_run): a
//      chunk of a batch whose histories have all ended is added to its
//      problem's SUM/SUM_SQ and cleared in the batch's slot; the lane that
//      folds a batch's last chunk passes the slot on to the batch n_slots
//      later (with a slot per batch, k_persist_fold_rest folds them all
//      after the run);
//   2. else it takes the next history index of the run (one atomic), finds
//      its batch, waits (folding meanwhile) until the batch's tally slot is
//      the batch's turn, and tracks the whole history with the batch's
//      problem: the same birth, walk and collision functions as the history
//      and event forms, so FP64 histories are bit for bit the same;
//   3. the lane that ends a batch's last history puts the batch on the
//      ready list.
// A wait for a slot polls at most wait_limit times, about a microsecond
// apart, then sets the run's error flag and every lane leaves.  A lane with
// nothing left to do helps fold for a short while and leaves; folds not done
// when the kernel ends are finished by k_persist_fold_rest.

__device__ __forceinline__ unsigned long long vld(const unsigned long long* p) {
  return *(const volatile unsigned long long*)p;
}
__device__ __forceinline__ int vld(const int* p) { return *(const volatile int*)p; }

__device__ __forceinline__ void persist_fold_chunk(const PersistArgs& a, const PersistProblem& P, const PersistJob& J,
                                                   int ch) {
  const int64_t e0 = (int64_t)ch * a.chunk;
  const int64_t e1 = e0 + a.chunk < P.n_tally ? e0 + a.chunk : P.n_tally;
  double* slot = P.slots + (int64_t)(J.order % P.n_slots) * P.n_tally;
  for (int64_t e = e0; e < e1; ++e) {
    const double v = __ldcg(slot + e);  // scored by atomics at L2: read past L1
    if (v != 0.0) {
      const double b = v * J.inv_n;
      atomicAdd(P.sum + e, b);
      atomicAdd(P.sumsq + e, b * b);
      __stcg(slot + e, 0.0);
    }
  }
}

// Claims and folds one chunk of a ready batch; false when none is left.
__device__ bool persist_fold(const PersistArgs& a, const PersistProblem* sp, unsigned long long* scan_lo) {
  PersistCtl* c = a.ctl;
  const unsigned long long ready = vld(&c->ready);
  if (vld(&c->claimed) >= ready) return false;
  for (unsigned long long k = vld(scan_lo); k < ready; ++k) {
    const int j = vld(a.ready_list + k);
    if (j < 0) continue;  // reserved, not yet written
    const PersistJob J = a.jobs[j];
    const PersistProblem& P = sp[J.prob];
    if (vld(a.chunk_next + j) >= P.n_chunks) {
      atomicCAS(scan_lo, k, k + 1);  // every chunk of this entry is taken: later scans start past it
      continue;
    }
    const int ch = atomicAdd(a.chunk_next + j, 1);
    if (ch >= P.n_chunks) continue;
    if (ch == P.n_chunks - 1) atomicAdd(&c->claimed, 1ULL);
    persist_fold_chunk(a, P, J, ch);
    __threadfence();
    if (atomicAdd(a.chunk_done + j, 1) == P.n_chunks - 1) {
      // the batch's slot is folded and clear: the batch n_slots later may score into it
      __threadfence();
      atomicExch(a.slot_turn + a.slot_base[J.prob] + J.order % P.n_slots, J.order + P.n_slots);
      atomicAdd(&c->folded, 1ULL);
    }
    return true;
  }
  return false;
}

__device__ __forceinline__ int persist_job_of(const PersistArgs& a, unsigned long long h) {
  int lo = 0, hi = a.n_jobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if ((int64_t)h < a.jobs[mid].end) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

__device__ __forceinline__ void persist_set_error(const PersistArgs& a, int job, long long polls) {
  if (atomicCAS(&a.ctl->error, 0, 1) == 0) {
    a.ctl->err_job = job;
    a.ctl->err_polls = polls;
  }
}

template <int kPrec>
__global__ void __launch_bounds__(128) k_persist(PersistArgs a) {
  MC_COUNTERS(L);
  __shared__ PersistProblem sp[kMaxPersistProblems];
  {
    const int words = (int)(sizeof(PersistProblem) / sizeof(int)) * a.n_probs;
    const int* src = (const int*)a.probs;
    int* dst = (int*)sp;
    for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  PersistCtl* c = a.ctl;
  unsigned long long* scan_lo = &c->scan_lo;
  unsigned long long nxs = 0, nfb = 0;
  for (;;) {
    if (vld(&c->error)) break;
    if (a.fold_in_run && persist_fold(a, sp, scan_lo)) continue;
    const unsigned long long h = atomicAdd(&c->next, 1ULL);
    if (h >= a.total) break;
    const int j = persist_job_of(a, h);
    const PersistJob J = a.jobs[j];
    const PersistProblem& P = sp[J.prob];
    // wait until the batch's tally slot is this batch's turn, folding meanwhile
    const int* turn = a.slot_turn + a.slot_base[J.prob] + J.order % P.n_slots;
    long long polls = 0;
    bool gave_up = false;
    while (vld(turn) < J.order) {
      if (vld(&c->error)) {
        gave_up = true;
        break;
      }
      if (persist_fold(a, sp, scan_lo)) continue;
      if (++polls > a.wait_limit) {
        persist_set_error(a, j, polls);
        gave_up = true;
        break;
      }
      __nanosleep(1000);
    }
    if (gave_up) break;
    __threadfence();  // the slot's clearing is visible before this history scores into it
    double* tally = P.slots + (int64_t)(J.order % P.n_slots) * P.n_tally;
    // birth: history index J.first + (h - J.start) of the problem, as the
    // history and event forms number it
    const int64_t idx = J.first + ((int64_t)h - J.start);
    const Skip k = skip_ahead((uint64_t)(idx + 1) * kPrnStride);
    mc_site o;
    if (kPrec == MC_PREC_MIXED) sample_source32(P.X, P.S, k, J.seed, o);
    else sample_source(P.X, P.S, k, J.seed, o);
    if (P.two_d) {
      o.z = P.z2d;
      planar_dir(o.u, o.v, o.w);
    }
    Particle p;
    start(P.M, o, idx, k, J.seed, p);
    p.tag = 0;
    if (kPrec == MC_PREC_FP64) {
      // the walk on the float-certified planes with cross sections inline:
      // whole histories per lane touch the mesh in no order, and the compact
      // segment's look-ahead loads and L1 prefetches cost more there than
      // they hide (10M histories of the 41M-tet core: 2.6 s against 3.7 s)
      float sigt32 = 0.0f;
      float uf = narrow(p.u), vf = narrow(p.v), wf = narrow(p.w);
      while (p.status == kAlive) {
        const int r = segment_fp64g<true, false, true, false>(P.M, P.X, p, uf, vf, wf, tally, P.ts, sigt32, nxs);
        if (r == 1) {
          score_collision(P.X, P.ts, tally, p);
          collide<false>(P.X, p, P.two_d, EigArgs{});
        }
        if (r == 1 || r == 5) {
          uf = narrow(p.u);
          vf = narrow(p.v);
          wf = narrow(p.w);
        }
      }
    } else if (kPrec == MC_PREC_MIXED) {
      Geo32 g;
      geo_load(p, g);
      float inv_sig = 0.0f;
      while (p.status == kAlive) {
        const int r = segment_mixed<true, false, false>(P.M, P.X, p, g, tally, P.ts, inv_sig, P.tol, nxs, nfb);
        if (r == 1) {
          geo_store(g, p);
          score_collision(P.X, P.ts, tally, p);
          collide<false>(P.X, p, P.two_d, EigArgs{});
          geo_load(p, g);
        }
      }
      geo_store(g, p);
    }
    // end of the history: closing hash word, counters, trace
    p.hash = fnv(p.hash, (uint64_t)(16 + p.status));
    L.add(kCntSeg, (unsigned long long)p.n_seg);
    L.add(kCntColl, (unsigned long long)p.n_coll);
    L.add(kCntHist, 1);
    switch (p.status) {
      case kLeaked: L.add(kCntLeak, 1); L.add_leak(p.wgt); break;
      case kAbsorbed: L.add(kCntAbsorb, 1); break;
      case kCutoff: L.add(kCntCutoff, 1); break;
      case kStuck: L.add(kCntStuck, 1); break;
      case kLost: L.add(kCntLost, 1); break;
      default: L.add(kCntBadXS, 1); break;
    }
    if (a.traces) {
      mc_trace t;
      t.id = p.id;
      t.hash = p.hash;
      t.status = p.status;
      t.n_seg = p.n_seg;
      t.n_coll = p.n_coll;
      t.elem = p.elem;
      t.face = p.face;
      t.pad = 0;
      t.E = p.E;
      t.x = p.x;
      t.y = p.y;
      t.z = p.z;
      a.traces[h] = t;
    }
    __threadfence();  // this history's scores land before the batch can be folded
    if (atomicSub(a.live + j, 1) == 1) {
      // the batch's last history: put it on the ready list
      const unsigned long long pos = atomicAdd(&c->ready, 1ULL);
      atomicExch(a.ready_list + pos, j);
    }
  }
  // nothing left to take: help fold for a while (the tail's last histories
  // may still add ready batches), then leave; k_persist_fold_rest folds
  // whatever is left when the kernel ends
  for (int idle = 0;
       a.fold_in_run && idle < 2000 && !vld(&c->error) && vld(&c->folded) < (unsigned long long)a.n_jobs;) {
    if (persist_fold(a, sp, scan_lo)) {
      idle = 0;
      continue;
    }
    ++idle;
    __nanosleep(1000);
  }
  L.add(kCntXS, nxs);
  L.add(kCntFallback, nfb);
  flush(L, a.counters, a.leak_w);
}

// Folds the chunks of ready batches that no lane of k_persist claimed.
__global__ void k_persist_fold_rest(PersistArgs a) {
  const PersistCtl* c = a.ctl;
  const int nr = (int)c->ready;
  for (int k = 0; k < nr; ++k) {
    const int j = a.ready_list[k];
    const PersistJob J = a.jobs[j];
    const PersistProblem& P = a.probs[J.prob];
    const int from = a.chunk_next[j] < P.n_chunks ? a.chunk_next[j] : P.n_chunks;
    for (int ch = from + blockIdx.x; ch < P.n_chunks; ch += gridDim.x) {
      const int64_t e0 = (int64_t)ch * a.chunk;
      const int64_t e1 = e0 + a.chunk < P.n_tally ? e0 + a.chunk : P.n_tally;
      double* slot = P.slots + (int64_t)(J.order % P.n_slots) * P.n_tally;
      for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        const double v = slot[e];
        if (v != 0.0) {
          const double b = v * J.inv_n;
          atomicAdd(P.sum + e, b);
          atomicAdd(P.sumsq + e, b * b);
          slot[e] = 0.0;
        }
      }
    }
  }
}

cudaError_t launch_persistent(const PersistArgs& a, int precision, int block, int grid, cudaStream_t st) {
  if (precision == MC_PREC_MIXED) k_persist<MC_PREC_MIXED><<<grid, block, 0, st>>>(a);
  else k_persist<MC_PREC_FP64><<<grid, block, 0, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_persist_fold_rest<<<1216, 256, 0, st>>>(a);
  return cudaGetLastError();
}

int persistent_blocks_per_sm(int precision, int block) {
  int n = 0;
  if (precision == MC_PREC_MIXED)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persist<MC_PREC_MIXED>, block, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persist<MC_PREC_FP64>, block, 0);
  return n > 0 ? n : 1;
}

// Loads the kernels of the fixed-source event form (no ray recording) on the
// current device: under lazy module loading a kernel's code is put on the
// device at its first launch or attribute query, and the no-allocation run
// must not be the call that does it.
cudaError_t preload_event_kernels() {
  cudaFuncAttributes fa;
  const void* fns[] = {
      (const void*)k_ev_init,
      (const void*)k_ev_xs<false>,
      (const void*)k_ev_advance<MC_PREC_MIXED>,
      (const void*)k_ev_advance<MC_PREC_FP64>,
      (const void*)k_ev_advance_mixed<false>,
      (const void*)k_ev_advance_fp64<false, 5>,
      (const void*)k_ev_advance_fp64<false, 4>,
      (const void*)k_ev_collide<false>,
      (const void*)k_ev_refill,
      (const void*)k_ev_reset,
      (const void*)k_ev_finish<MC_PREC_MIXED, false>,
      (const void*)k_ev_finish<MC_PREC_FP64, false>,
  };
  for (const void* f : fns) {
    const cudaError_t e = cudaFuncGetAttributes(&fa, f);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_sample(const DevXS& X, const DevSource& S, int64_t first, int64_t n,
                          uint64_t master, mc_site* out, cudaStream_t st) {
  k_sample<<<1216, 256, 0, st>>>(X, S, first, n, master, out);
  return cudaGetLastError();
}

cudaError_t launch_accumulate(double* batch, double* sum, double* sumsq, int64_t n, double inv_w,
                              cudaStream_t st) {
  k_accumulate<<<1216, 256, 0, st>>>(batch, sum, sumsq, n, inv_w);
  return cudaGetLastError();
}

}  // namespace mc
