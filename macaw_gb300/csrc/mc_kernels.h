// mc_kernels.h -- launchers for the tracking kernels (host-callable).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/macaw_gb300.h"
#include "mc_device.cuh"

namespace mc {

// Batches of one pipelined mc_run in flight at once (one tally slot each).
constexpr int kPipeSlots = 32;                      // batches in flight at most
constexpr size_t kSlotBudget = (size_t)8 << 30;     // bytes of batch tallies at most

// Device counters, one 64-bit slot each.
enum Counter : int {
  kCntSeg = 0,
  kCntColl,
  kCntLeak,
  kCntAbsorb,
  kCntCutoff,
  kCntStuck,
  kCntLost,
  kCntBadXS,
  kCntXS,
  kCntFallback,
  kCntHist,
  kCntSegWalk,  // segments walked by the advance kernels
  kNumCounters
};

// Particle bank: one 192-byte record (six 32-byte sectors) per slot, plus
// the element index in an array of its own.  A walk visits particles in
// element order, so their slots are scattered: in separate arrays every
// field a visit touches costs a sector of its own, here the fields a walk
// visit moves share four sectors.
//   sector 0: x y z u          sector 1: v w seed hash
//   sector 2: wgt fin mat n_seg zero_run tag n_coll
//   sector 3: cross-section cache keys, float 1/Sigma_t of the cached values
//   sector 4: E sigt id         sector 5: cross-section cache values
// (the mixed walk reads sectors 0-3 and writes 0-1 and the fields of 2 it
// changed, the FP64 walk reads 0-5 and writes 0-2 and Sigma_t in 4).  The
// element array (4 bytes a slot) stays in L2; the queue ordering reads it
// for every queued particle.
// k-eigenvalue fields sit in arrays of their own.  RecField<T> addresses
// one field of every record: B.x[s] is slot s's x, B.x + s its address.
constexpr int64_t kBankRec = 192;

template <class T>
struct RecField {
  unsigned char* base;  // the field in slot 0
  __host__ __device__ __forceinline__ T& operator[](int64_t s) const {
    return *reinterpret_cast<T*>(base + s * kBankRec);
  }
  __host__ __device__ __forceinline__ T* operator+(int64_t s) const {
    return reinterpret_cast<T*>(base + s * kBankRec);
  }
};

struct Bank {
  RecField<double> x, y, z, u, v, w, E, wgt, sigt;
  RecField<uint64_t> seed, hash;
  RecField<int64_t> id;
  RecField<int> mat, n_seg, n_coll, zero_run, fin, tag;
  int* elem;                 // element index, one array
  RecField<int4> cm;         // cross-section cache keys
  RecField<double4_32a> cs;  // cross-section cache values
  RecField<float4> cinv;     // float 1/Sigma_t of the cached values (mixed-precision walk)
  // k-eigenvalue runs only (null otherwise): nu*Sigma_f of the current
  // material and of the cached ones, track-length keff sum, sites banked
  double *nuf, *ktl;
  double4_32a* cn;
  int* n_prog;
  int64_t cap;
};

// One slot's record, the layout above (the walks address its fields
// through RecField, never through this type).
struct BankRecord {
  double x, y, z, u;                                  // sector 0
  double v, w;                                        // sector 1
  uint64_t seed, hash;
  double wgt;                                         // sector 2
  int fin, mat, n_seg, zero_run, tag, n_coll;
  int4 cm;                                            // sector 3
  float4 cinv;
  double E, sigt;                                     // sector 4
  int64_t id, unused;
  double4_32a cs;                                     // sector 5
};
static_assert(sizeof(BankRecord) == (size_t)kBankRec, "bank record is six 32-byte sectors");
static_assert(offsetof(BankRecord, wgt) == 64 && offsetof(BankRecord, cm) == 96 &&
                  offsetof(BankRecord, E) == 128 && offsetof(BankRecord, cs) == 160,
              "bank record sectors");

// The bank whose records start at rec (cap * kBankRec bytes, 256-byte
// aligned) with its element array elem (cap ints); the k-eigenvalue
// arrays are left null.
inline Bank bank_at(void* rec, int* elem, int64_t cap) {
  unsigned char* r = static_cast<unsigned char*>(rec);
#define MC_REC(f) {r + offsetof(BankRecord, f)}
  Bank B{};
  B.x = MC_REC(x); B.y = MC_REC(y); B.z = MC_REC(z); B.u = MC_REC(u);
  B.v = MC_REC(v); B.w = MC_REC(w); B.seed = MC_REC(seed); B.hash = MC_REC(hash);
  B.wgt = MC_REC(wgt); B.fin = MC_REC(fin); B.mat = MC_REC(mat); B.n_seg = MC_REC(n_seg);
  B.zero_run = MC_REC(zero_run); B.tag = MC_REC(tag); B.n_coll = MC_REC(n_coll);
  B.cm = MC_REC(cm); B.cinv = MC_REC(cinv);
  B.E = MC_REC(E); B.sigt = MC_REC(sigt); B.id = MC_REC(id);
  B.cs = MC_REC(cs);
#undef MC_REC
  B.elem = elem;
  B.cap = r ? cap : 0;
  return B;
}

// True when the bank's records are set (checked on the host before any
// launch that uses the bank).
inline bool bank_complete(const Bank& B) { return B.x.base != nullptr && B.elem != nullptr && B.cap > 0; }

// Event-loop control block (device memory).
struct EventCtl {
  int n_xs[2], n_adv[2], n_coll;   // queue lengths, double-buffered by iteration parity
  int adv_head;                     // advance queue entries taken so far this iteration
  unsigned long long free_head, free_tail;  // ring of free bank slots (monotonic counters)
  long long next_hist;              // next history (relative to the run) to be born
  long long birth_limit;            // histories at or past this index wait (pipelined batches)
};

struct EventQueues {
  int* xs[2];
  int* adv[2];
  int* coll;
  int* free_slots;  // ring of bank-capacity entries
};

// One entry of the birth sequence: a batch of a pipelined run, or a serving
// request.  Histories [start, end) of the sequence are its histories
// 0..end-start-1, with particle ids first_id+1... and master seed `seed`,
// born from `src` (or the context source) and scored into tally `slot`.
struct DevRequest {
  int64_t start, end;
  int64_t first_id;
  uint64_t seed;
  int slot;
  int has_src;
  DevSource src;
};

struct RunArgs {
  int64_t first, n;
  uint64_t master;
  double* tally;                // scores of even batches
  double* tally2;               // tally slot 1 (== tally for a single batch); slots k >= 1 are
                                // tally2 + (k-1)*n_tally
  int64_t n_tally;              // values per tally slot: elements x energy bins x scores
  TallySpec ts;                 // what the tally scores
  const DevRequest* req;        // device: birth-sequence entries sorted by start, or null
  int n_req;
  int* live;                    // event mode: in-flight counters per tally slot, or null
  mc_trace* traces;
  unsigned long long* counters;
  double* leak_w;
  const mc_site* sites;  // device copy of caller-supplied sites, or null
  int n_mat;
  int precision;
  float tol;    // mixed form: exit ambiguity tolerance (cm)
  int max_seg;  // event mode: segments per advance launch (<= 0: until event)
  int refill;   // event mode: lanes take further queued particles within one launch
  int two_d;    // 2-D problem: planar directions, births at z = z2d
  double z2d;
  EigArgs eig;       // k-eigenvalue generation (eig.on = 0: fixed source)
  int sort_shift;    // event mode: advance queue ordered by elem >> sort_shift (-1: unordered)
  int sort_buckets;  // (n_tet >> sort_shift) + 1
  int* sort_tmp;     // bank-capacity scratch for the ordering
  int* sort_cnt;     // sort_buckets + 1 counters
  int walk_blocks;   // FP64 walk compiled for 4 or 5 resident blocks per SM (0: 5)
};

// Loads the fixed-source event-form kernels onto the current device.
cudaError_t preload_event_kernels();

// ---- persistent run of many batches of one or more problems ------------
constexpr int kMaxPersistProblems = 8;

// One problem of a persistent run: its device tables, tally definition and
// the tally slots its batches score into in turn (slot k % n_slots for the
// problem's k-th batch), folded into its SUM/SUM_SQ.
struct PersistProblem {
  DevMesh M;
  DevXS X;
  DevSource S;
  TallySpec ts;
  int64_t n_tally;
  double* slots;   // n_slots x n_tally
  double* sum;
  double* sumsq;
  int n_slots;
  int two_d;
  double z2d;
  float tol;
  int n_chunks;    // fold chunks of one tally
};

// One batch: global history indices [start, end) of the run; history
// index first + (h - start) of its problem (particle id one more).
struct PersistJob {
  int64_t start, end;
  int64_t first;
  uint64_t seed;
  double inv_n;    // 1 / histories of the batch (SUM is a sum of batch / weight)
  int prob;
  int order;       // index of the batch among its problem's batches
};

struct PersistCtl {
  unsigned long long next;          // next history index to take
  unsigned long long ready;         // batches whose histories have all ended (entries in ready list)
  unsigned long long claimed;       // batches whose fold chunks have all been claimed
  unsigned long long folded;        // batches folded into SUM/SUM_SQ
  unsigned long long scan_lo;       // ready-list entries below this have every fold chunk claimed
  int error;                        // 1: a wait gave up (err_job: the batch it waited on)
  int err_job;
  long long err_polls;
};

struct PersistArgs {
  const PersistProblem* probs;
  int n_probs;
  int n_jobs;
  const PersistJob* jobs;
  unsigned long long total;    // histories of all batches
  int* live;                   // per batch: histories not ended
  int* chunk_next;             // per batch: fold chunks claimed
  int* chunk_done;             // per batch: fold chunks done
  int* ready_list;             // batches in the order they became ready (-1: not yet written)
  int* slot_turn;              // per problem slot: order of the batch allowed to score into it
  const int* slot_base;        // per problem: its first entry in slot_turn
  int chunk;                   // tally values per fold chunk
  PersistCtl* ctl;
  mc_trace* traces;            // per history of the run (global index), or null
  unsigned long long* counters;
  double* leak_w;
  long long wait_limit;        // polls a lane makes for a slot or for fold work before giving up
  int fold_in_run;             // 1: some problem has fewer slots than batches, so lanes fold
                               // ready batches during the run to free their slots; 0: every
                               // batch has a slot of its own and k_persist_fold_rest folds all
};

cudaError_t launch_persistent(const PersistArgs& a, int precision, int block, int grid, cudaStream_t st);
// Blocks of `block` threads of the persistent kernel resident per SM.
int persistent_blocks_per_sm(int precision, int block);

cudaError_t launch_history(const DevMesh& M, const DevXS& X, const DevSource& S, const RunArgs& a,
                           int block, int grid, cudaStream_t st);

// Event mode, one call per phase; grids are persistent (grid-stride over the
// device-side queue lengths), so the launch shapes never depend on counts.
cudaError_t launch_event_init(const DevMesh& M, const DevXS& X, const DevSource& S, const RunArgs& a,
                              const Bank& B, const EventQueues& Q, EventCtl* ctl, int block,
                              int grid, cudaStream_t st, int64_t birth_limit);
cudaError_t launch_event_iteration(const DevMesh& M, const DevXS& X, const DevSource& S,
                                   const RunArgs& a, const Bank& B, const EventQueues& Q,
                                   EventCtl* ctl, int parity, int block, int grid,
                                   cudaStream_t st, int* n_launch, cudaEvent_t adv0 = nullptr,
                                   cudaEvent_t adv1 = nullptr);
cudaError_t launch_event_finish(const DevMesh& M, const DevXS& X, const DevSource& S,
                                const RunArgs& a, const Bank& B, const EventQueues& Q,
                                EventCtl* ctl, int parity, int block, int grid, cudaStream_t st);

cudaError_t launch_sample(const DevXS& X, const DevSource& S, int64_t first, int64_t n,
                          uint64_t master, mc_site* out, cudaStream_t st);

cudaError_t launch_accumulate(double* batch, double* sum, double* sumsq, int64_t n, double inv_w,
                              cudaStream_t st);

// k-eigenvalue bank processing (mc_eigen.cu).
// Fixed-order sum of v[0..n): tile b of 1024 values (zero-padded) is summed
// by a pairwise tree (v[t] += v[t+s], s = 512, 256, ..., 1) into part[b];
// the caller adds the ceil(n/1024) partials in index order.
constexpr int kReduceTile = 1024;

// Threads per block of the tail kernel: the histories left are long
// latency chains whose steps diverge, so a warp carries only a few of them
// (one in the mixed form, four in the FP64 form, where fewer, busier warps
// share each SM's FP64 pipe better); measured on the 2M-tet lattice, single
// 1e6-history calls ran 134.6M (mixed) and 50.1M (FP64) histories/s
// against 116.5M and 47.0M with 32.
inline int tail_block(int precision) { return precision == MC_PREC_MIXED ? 1 : 4; }

// Default hand-over to the tail kernel: bank/16 particles left for the
// mixed form of fixed-source runs, whose tail is a pure walk (single 1e6
// calls on the lattice: 150.3M against 134.4M histories/s at bank/64);
// bank/64 otherwise (FP64: no difference; k-eigenvalue generations, whose
// tail histories collide about five times each, ran 27.6 against 31.2 ms
// per mixed generation).
inline int64_t tail_divisor(const RunArgs& a) { return (a.precision == MC_PREC_MIXED && !a.eig.on) ? 16 : 64; }
cudaError_t launch_tile_sums(const double* v, int64_t n, double* part, cudaStream_t st);
// Exclusive prefix sum of n counts into off[0..n] (off[n] = total);
// tmp holds scan_tmp_size(n) entries.
int64_t scan_tmp_size(int64_t n);
cudaError_t launch_scan(const int* cnt, int64_t n, int64_t* off, int64_t* tmp, cudaStream_t st);
// Fission bank in (parent id, progeny) order: site k goes to
// off[parent - 1 - first] + progeny (off: scan of the n_hist histories'
// site counts).
cudaError_t launch_bank_sort(const mc_fission_site* in, int64_t m, const int64_t* off, int64_t first,
                             int64_t n_hist, mc_fission_site* out, cudaStream_t st);
// Resampling counts of the sorted bank (synchronize_bank): site i is kept
// copies + (xi_i < p) times, xi_i the (i+1)-th draw from state seed0.
cudaError_t launch_bank_counts(int64_t m, uint64_t seed0, int copies, double p, int* cnt, cudaStream_t st);
// Writes the resampled sites to src[0..n): site i fills [pos[i], pos[i+1])
// below n; then, if pos[m] < n, src[pos[m] + j] = sorted[max(0, m - need + j)]
// for j < need = n - pos[m].
cudaError_t launch_bank_fill(const mc_fission_site* sorted, int64_t m, const int64_t* pos, int64_t n,
                             mc_site* src, cudaStream_t st);

}  // namespace mc
