/*
 * macaw_gb300.h -- C ABI of the GB300 particle tracker.
 *
 * The hot path MaCaw runs through MOOSE's ray tracing module and OpenMC
 * (source birth, tet-to-tet walk, cross-section lookup, distance sampling,
 * collision, element track-length tallies) is exposed here as batch-level
 * calls with plain pointers and sizes.  Every call returns 0 on success or
 * a non-zero MC_ERR_* code; mc_last_error() then holds a message.  A context
 * is bound to one CUDA device and one stream, and its calls are serialised
 * by an internal mutex.  Device-side failures (lost or stuck particles, bad
 * cross sections) never trap: they are counted in mc_stats and reported as
 * status codes in per-history traces.
 *
 * Each entry point names the reference interface it stands in for, by file
 * and line in idaholab/macaw.
 */
#ifndef MACAW_GB300_H
#define MACAW_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MC_OK 0
#define MC_ERR_ARG 1     /* invalid argument (paramError / mooseError) */
#define MC_ERR_STATE 2   /* call out of order (missing mesh, data, source) */
#define MC_ERR_CUDA 3    /* CUDA runtime failure */
#define MC_ERR_DEVICE 4  /* device-side status word reported a failure */
#define MC_ERR_NOMEM 5   /* device or host allocation failed */

/* boundary condition types: MOOSE KillRayBC / ReflectRayBC as used in
 * test/tests/study/openmc_study.i:49-54 */
#define MC_BC_VACUUM 0
#define MC_BC_REFLECT 1

/* precision forms */
#define MC_PREC_FP64 0   /* plain FP64, per-history traces bit-exact to the oracle */
#define MC_PREC_MIXED 1  /* FP32 walk/XS, FP64 near faces/edges and for tallies */

/* execution forms */
#define MC_MODE_HISTORY 0    /* one thread per history, persistent grid */
#define MC_MODE_EVENT 1      /* event queues: birth, xs, advance, collide */

/* source kinds */
#define MC_SRC_POINT 0
#define MC_SRC_BOX 1
#define MC_SRC_CYLINDERS 2
#define MC_SRC_WATT 0
#define MC_SRC_MONO 1

/* tally estimators and scores (OpenMCTally `estimator` and `scores`) */
#define MC_EST_TRACKLENGTH 1
#define MC_EST_COLLISION 2
#define MC_SCORE_FLUX 0
#define MC_SCORE_TOTAL 1
#define MC_SCORE_SCATTER 2
#define MC_SCORE_ABSORPTION 3
#define MC_MAX_SCORES 4
#define MC_MAX_ENERGY_BINS 4096

/* tally readback kinds */
#define MC_TALLY_BATCH 0   /* raw sum of wgt*track length of the current batch */
#define MC_TALLY_SUM 1     /* OpenMC results SUM: sum over batches of batch/weight */
#define MC_TALLY_SUM_SQ 2  /* OpenMC results SUM_SQ */

/* history end states (mc_trace.status) */
#define MC_ST_LEAKED 1
#define MC_ST_ABSORBED 2
#define MC_ST_CUTOFF 3
#define MC_ST_STUCK 4
#define MC_ST_LOST 5
#define MC_ST_BADXS 6

typedef struct mc_ctx mc_ctx;

/* Fixed source (the settings.xml <source> that OpenMCStudy::defineRays
 * samples per history; src/userobjects/OpenMCStudy.C:317-360). */
typedef struct {
  int32_t space;  /* MC_SRC_POINT | MC_SRC_BOX | MC_SRC_CYLINDERS */
  int32_t energy; /* MC_SRC_WATT | MC_SRC_MONO */
  double point[3];
  double box_lo[3];
  double box_hi[3];
  int32_t n_cyl;
  int32_t pad;
  const double* cyl_xy; /* 2*n_cyl cylinder axis positions (x, y) */
  double cyl_r, cyl_z0, cyl_z1;
  double watt_a, watt_b; /* eV, 1/eV */
  double mono_E;         /* eV */
} mc_source_desc;

/* One source site: the ray MaCaw defines per history (start point,
 * direction, aux energy and weight; src/userobjects/OpenMCStudy.C:335-360).
 * The tracking stream is seeded from the history index, as for sites the
 * library samples itself. */
typedef struct {
  double x, y, z;
  double u, v, w;
  double E;
  double wgt;
} mc_site;

/* One fission site (OpenMC SourceSite as create_fission_sites fills it):
 * collision point, isotropic direction, prompt energy, weight 1, the id of
 * the history that banked it and its index among that history's sites --
 * the key OpenMC's sort_fission_bank orders the bank by. */
typedef struct {
  double x, y, z;
  double u, v, w;
  double E;
  double wgt;
  int64_t parent;
  int32_t progeny;
  int32_t pad;
} mc_fission_site;

/* One batch of histories (OpenMCStudy::generateRays + execute +
 * postExecuteStudy for a fixed-source batch;
 * src/userobjects/OpenMCStudy.C:218-242,366-402). */
typedef struct {
  int64_t first_history;   /* 0-based global index of the first history; id = index + 1 */
  int64_t n_histories;
  int64_t bank_size;       /* particles in flight (event mode); 0 = all */
  uint64_t seed;           /* master seed */
  int32_t precision;       /* MC_PREC_* */
  int32_t mode;            /* MC_MODE_* */
  int32_t block_size;      /* threads per block; 0 = default */
  int32_t max_seg_per_advance; /* event mode: segments per advance launch; 0 = until event */
  int32_t record_traces;   /* 1: fill one mc_trace per history */
  int32_t accumulate;      /* 1: fold this batch into SUM/SUM_SQ and clear the batch tally */
  int32_t sort_queue;      /* event mode: 0 off; s > 0 orders the advance queue by element id >> (s-1)
                              (coarsened to at most 65536 buckets) before each walk launch */
  int32_t profile;         /* 1: time every advance launch with CUDA events (mc_stats.ms_advance) */
  int32_t refill;          /* event mode: 1 lets an advance lane take the next queued particle when
                              its particle reaches an event; 0: lanes walk their warp's chunk of the
                              queue one visit at a time */
  int32_t n_batches;       /* > 1: consecutive batches of batch_sizes histories run through one
                              pipeline, each folded into SUM/SUM_SQ when it drains (needs accumulate) */
  int32_t graph;           /* event mode: 1 captures a cycle of event iterations once as a CUDA
                              graph and replays it (ignored with profile) */
  int32_t tail;            /* event mode: once every history is born and at most this many particles
                              are left, one tail kernel runs them to completion (0: max(4096, bank/16)
                              for MC_PREC_MIXED, max(4096, bank/64) for MC_PREC_FP64;
                              -1: never, the event loop runs until the bank is empty) */
  const mc_site* sites;    /* optional HOST array of n_histories source sites; NULL: sample on the device */
  const int64_t* batch_sizes; /* HOST array of n_batches sizes adding up to n_histories */
  double* const* batch_sum_out; /* optional HOST array of n_batches HOST buffers of mc_tally_size doubles:
                                   buffer b receives the SUM tally as it stands when batch b has been
                                   folded in (copied while later batches run; pinned buffers let the copy
                                   overlap); needs accumulate */
  int32_t walk_blocks;     /* event mode, MC_PREC_FP64: resident 128-thread blocks per SM the FP64
                              walk kernel is compiled for -- 5 (96 registers, 20 warps per SM) or 4
                              (118 registers, 16 warps); 0 = 5.  mc_autotune picks it per workload */
  int32_t pad;
} mc_run_desc;

/* Per-history outcome: element sequence hash, counts, end state. */
typedef struct {
  int64_t id;
  uint64_t hash;
  int32_t status;
  int32_t n_seg;
  int32_t n_coll;
  int32_t elem;
  int32_t face;
  int32_t pad;
  double E;
  double x, y, z;
} mc_trace;

typedef struct {
  int64_t n_hist, n_seg, n_coll, n_leak, n_absorb, n_cutoff, n_stuck, n_lost, n_badxs;
  int64_t n_fallback;   /* mixed form: segments re-solved in FP64 */
  int64_t n_xs;         /* macroscopic XS evaluations */
  int64_t n_launch;     /* kernels launched by the last mc_run */
  double leak_weight;
  double ms_total;      /* device time of the last mc_run (CUDA events) */
  double ms_advance;    /* device time in the segment-walk kernels */
  int64_t n_advance_launch;
  int64_t n_seg_advance; /* segments walked inside the segment-walk kernels (the rest: tail kernel) */
} mc_stats;

/* ---- context --------------------------------------------------------- */
/* Replaces: OpenMCStudy construction, openmc_init + openmc_simulation_init
 * (src/userobjects/OpenMCStudy.C:78-204). */
int mc_ctx_create(int device, mc_ctx** out);
/* Replaces: OpenMCStudy::~OpenMCStudy / openmc_finalize (OpenMCStudy.C:207-216). */
int mc_ctx_destroy(mc_ctx* ctx);
/* Replaces: mooseError / openmc_err_msg (OpenMCStudy.C:129-131). */
const char* mc_last_error(mc_ctx* ctx);
int mc_version(void);

/* ---- mesh (the libMesh mesh MOOSE traces on; one cell per element,
 * one universe per subdomain: OpenMCStudy.C:152-187) ------------------- */
/* tet_side_bid: optional 4*n_tet sideset ids (-1 interior/none); side f is
 * the face opposite local vertex f.  Builds face adjacency, outward face
 * planes and the start-point locator, and uploads them. */
int mc_mesh_upload(mc_ctx* ctx, int64_t n_vtx, const double* xyz, int64_t n_tet,
                   const int32_t* tet_vtx, const int32_t* tet_block, const int32_t* tet_side_bid);
/* Replaces: [RayBCs] ReflectRayBC / KillRayBC boundary lists
 * (test/tests/study/openmc_study.i:49-54). */
int mc_bc_set(mc_ctx* ctx, int32_t boundary_id, int32_t type);

/* ---- cross sections (OpenMC nuclide/material data the collision kernel
 * evaluates; CollisionKernel.C:143) ------------------------------------- */
int mc_nuclide_add(mc_ctx* ctx, int64_t n_pts, const double* E, const double* sig_t,
                   const double* sig_s, double awr, int32_t* out_index);
int mc_material_add(mc_ctx* ctx, int32_t material_id, int32_t n, const int32_t* nuclides,
                    const double* densities);
/* Replaces: CollisionKernel 'blocks'/'materials' params and the
 * block -> material map (src/raykernels/CollisionKernel.C:34-37,63-69,110). */
int mc_block_material_map(mc_ctx* ctx, int32_t n, const int32_t* blocks,
                          const int32_t* materials);
int mc_set_hash_bins(mc_ctx* ctx, int32_t n_bins);

/* ---- source ---------------------------------------------------------- */
int mc_source_set(mc_ctx* ctx, const mc_source_desc* src);

/* ---- run ------------------------------------------------------------- */
/* Replaces: one batch of OpenMCStudy::generateRays / execute /
 * postExecuteStudy, whose per-segment work is CollisionKernel::onSegment
 * (src/raykernels/CollisionKernel.C:98-275).  Asynchronous on the context
 * stream unless traces or accumulation need a sync; mc_sync waits. */
int mc_run(mc_ctx* ctx, const mc_run_desc* desc);
int mc_sync(mc_ctx* ctx);
/* Replaces: the loop over openmc::initialize_history in
 * OpenMCStudy::defineRays (src/userobjects/OpenMCStudy.C:317-360): samples
 * the source sites of histories [first, first+n) on the device and copies
 * them to the HOST array out. */
int mc_source_sample(mc_ctx* ctx, int64_t first, int64_t n, uint64_t seed, mc_site* out);
/* Work of this context goes to the given cudaStream_t (NULL: the context's
 * own stream). */
int mc_ctx_set_stream(mc_ctx* ctx, void* stream);
/* Autotuner (no counterpart in the reference, whose MPI/thread layout is set
 * by hand on the command line): picks segments per walk launch, threads per
 * block, advance-queue ordering, bank size (when base->bank_size is 0), lane
 * refill and CUDA-graph replay of the event form that give the most
 * histories/s on trials of trial_histories (>= 1024) histories of this
 * context's problem (four pipelined batches each), starting from *base;
 * writes *base with those fields replaced to *best and the rate reached to
 * *best_rate.  SUM, SUM_SQ and the batch count are restored afterwards and
 * the batch tally is left cleared. */
int mc_autotune(mc_ctx* ctx, const mc_run_desc* base, int64_t trial_histories, mc_run_desc* best,
                double* best_rate);

/* Replaces: the 2-D mode of CollisionKernel (z_coord,
 * src/raykernels/CollisionKernel.C:38,60-61,177-179,200-202) and of
 * OpenMCStudy (src/userobjects/OpenMCStudy.C:355-356).  With on = 1 every
 * source direction and every scattered direction loses its z component and
 * is renormalised in the plane (a direction along z becomes +x), and
 * histories are born at z = z_coord, so they stay in that plane.  The
 * mesh is a 2-D mesh extruded into one layer of tets around z_coord (the
 * lattice generator with nz = 1); a 2-D element's result is the sum over
 * the tets of its prism. */
int mc_set_2d(mc_ctx* ctx, int32_t on, double z_coord);

/* Segments one history may walk before it is ended as stuck (status
 * MC_ST_STUCK, counted in mc_stats.n_stuck).  No counterpart in MaCaw's own
 * sources, whose tracer (MOOSE's TraceRay) runs a ray until a kernel or a
 * boundary ends it.  0 restores the default: 4096 * ceil(cbrt(n_tet)),
 * at least 65,536 and at most 10,000,000 (a straight flight crosses of the
 * order of cbrt(n_tet) elements; the default allows 4096 such flights), so
 * a runaway walk on a small mesh is stopped early.  mc_segment_limit
 * returns the limit in force for the uploaded mesh. */
int mc_set_segment_limit(mc_ctx* ctx, int64_t max_segments);
int mc_segment_limit(mc_ctx* ctx, int64_t* out);

/* ---- k-eigenvalue runs -------------------------------------------------
 * Replaces: OpenMC's eigenvalue run mode as OpenMCStudy drives it, one
 * generation per batch (src/userobjects/OpenMCStudy.C:297-364 births from
 * the source bank; :374-402 postExecuteStudy -> finalize_generation;
 * :404-607 finalizeGeneration / synchronizeBanks) with the track-length
 * keff score of CollisionKernel.C:153-154. */

/* Fission data of a nuclide: nu*sigma_f (barn) at each point of the
 * nuclide's energy grid (n_pts values, as given to mc_nuclide_add); NULL
 * makes it non-fissionable.  A fissionable nuclide samples fission sites at
 * every collision with it (OpenMC create_fission_sites): banked in
 * eigenvalue runs, drawn and dropped in fixed-source runs. */
int mc_nuclide_set_fission(mc_ctx* ctx, int32_t nuclide, const double* nu_sig_f);

typedef struct {
  int64_t n_particles;     /* settings particles: histories per generation */
  int32_t n_batches;       /* settings batches: generations run by this call */
  int32_t n_inactive;      /* settings inactive: generations that score no tally */
  uint64_t seed;           /* master seed */
  int32_t precision;       /* MC_PREC_* */
  int32_t mode;            /* MC_MODE_* */
  int64_t bank_size;       /* event form: particles in flight; 0 = all */
  int32_t block_size;      /* 0 = default */
  int32_t max_seg_per_advance; /* event form, as mc_run_desc */
  int32_t sort_queue;      /* event form, as mc_run_desc */
  int32_t graph;           /* event form, as mc_run_desc */
  int32_t tail;            /* event form, as mc_run_desc: particles left when a generation's tail kernel
                              takes over (0: default, -1: never) */
  double keff0;            /* keff the first generation divides by (0: 1.0, OpenMC's start value) */
  double watt_a, watt_b;   /* prompt fission spectrum (0: 0.988e6 eV, 2.249e-6 /eV) */
  int64_t fission_bank_capacity; /* sites a generation may bank (0: 3 * n_particles, OpenMC's reservation) */
  const mc_site* initial_source; /* optional HOST array of n_particles sites; NULL: sampled from the
                                    source (mc_source_set) as OpenMC initialize_source does */
} mc_eigen_desc;

/* Results of one generation. */
typedef struct {
  double k_generation;     /* track-length estimate: sum of wgt*min(d,L)*nu*Sigma_f / n_particles */
  double k_collision;      /* collision estimate: sum of wgt*nu*Sigma_f/Sigma_t / n_particles */
  double k_absorption;     /* absorption estimate: sum of wgt*nu*sigma_f/sigma_a / n_particles */
  double keff;             /* running estimate after this generation (OpenMC calculate_average_keff) */
  double keff_std;         /* its standard deviation (0 until two active generations) */
  double leakage;          /* leaked weight / n_particles */
  int64_t n_sites;         /* fission sites banked */
  int64_t n_seg, n_coll;
  double ms;               /* device time of the generation, bank resampling included */
} mc_eigen_gen;

/* Runs n_batches generations of n_particles histories.  Generation g
 * (0-based) tracks histories with ids g*n_particles + 1.. (tracking stream
 * seeded from the id); the first starts from initial_source or the sampled
 * source.  After each generation the fission bank is put in (parent id,
 * progeny index) order and resampled to exactly n_particles sites
 * (synchronizeBanks, OpenMCStudy.C:430-607, with one rank); keff
 * estimators are summed over histories in a fixed order.  Active
 * generations add their tally to SUM/SUM_SQ (one batch each).  out
 * receives n_batches records.  MC_ERR_DEVICE when a generation banks no
 * site or more than the capacity. */
int mc_eigen_run(mc_ctx* ctx, const mc_eigen_desc* desc, mc_eigen_gen* out);
/* The source sites of the next generation (n_particles, after the last
 * generation's resampling). */
int mc_eigen_source_download(mc_ctx* ctx, mc_site* out, int64_t n);
/* The last generation's fission bank in sort order; *n_out = its size. */
int mc_eigen_fission_bank_download(mc_ctx* ctx, mc_fission_site* out, int64_t capacity, int64_t* n_out);

/* ---- tally definition ------------------------------------------------- */
typedef struct {
  int32_t estimator;       /* MC_EST_TRACKLENGTH or MC_EST_COLLISION */
  int32_t n_scores;        /* 1..MC_MAX_SCORES */
  int32_t scores[MC_MAX_SCORES]; /* MC_SCORE_*: track length scores flux and total; collision all four */
  int32_t n_energy_bins;   /* 0: no energy filter; else the bins between n_energy_bins+1 edges */
  int32_t pad;
  const double* energy_edges; /* HOST array of ascending edges (eV); energies outside score nothing */
} mc_tally_desc;

/* Replaces: OpenMCTally (src/userobjects/OpenMCTally.C:30-101, 103-198):
 * the estimator, scores and energy filter of the element tally (cell
 * filter: one bin per element).  Results are laid out [element][energy
 * bin][score] in every tally kind; mc_tally_size gives their number.
 *   track length, per segment: flux wgt*l, total wgt*l*Sigma_t;
 *   collision, per collision:  flux wgt/Sigma_t, total wgt, scatter
 *   wgt*Sigma_s/Sigma_t, absorption wgt*(Sigma_t-Sigma_s)/Sigma_t,
 * at the energy before the collision.  Without a call the tally is the
 * track-length flux per element.  Clears every tally and the batch count;
 * an upload of a new mesh restores the default. */
int mc_tally_configure(mc_ctx* ctx, const mc_tally_desc* desc);
int mc_tally_size(mc_ctx* ctx, int64_t* n_values);

/* ---- results --------------------------------------------------------- */
/* Replaces: OpenMCTallyAux::computeValue element readback
 * (src/auxkernels/OpenMCTallyAux.C:187-205).  n must equal mc_tally_size. */
int mc_tally_download(mc_ctx* ctx, int32_t kind, double* out, int64_t n);
int mc_tally_reset(mc_ctx* ctx);
/* Clears one tally (MC_TALLY_BATCH, MC_TALLY_SUM or MC_TALLY_SUM_SQ). */
int mc_tally_clear(mc_ctx* ctx, int32_t kind);
int mc_trace_download(mc_ctx* ctx, mc_trace* out, int64_t n);
int mc_stats_get(mc_ctx* ctx, mc_stats* out);
/* Number of completed accumulated batches (OpenMC n_realizations). */
int mc_batches_done(mc_ctx* ctx, int64_t* out);

/* ---- persistent run: many batches, of one or more problems -------------
 * Replaces: the batch loop of OpenMCStudy (generateRays / execute /
 * postExecuteStudy once per batch, src/userobjects/OpenMCStudy.C:218-242,
 * 366-402) for every batch of a run in one kernel launch; beyond the
 * reference, batches of different problems (contexts on one device) share
 * that launch.  Every lane of a persistent grid takes the next history of
 * the run, tracks it whole with its batch's problem (same arithmetic as the
 * history and event forms: FP64 histories are bit for bit those of
 * mc_run), and the lane that ends a batch's last history makes the batch
 * ready; ready batches are folded (tally / n_histories into the problem's
 * SUM and SUM_SQ, one batch each, as mc_run with accumulate) by lanes with
 * nothing else to do.  Each problem's batches take `slots` tally slots in
 * turn: a history of the problem's k-th batch waits, folding meanwhile,
 * until batch k - slots is folded; a wait that polls wait_limit times ends
 * the run with MC_ERR_DEVICE (no lane waits without a limit).  The problems
 * must be on the device already (mc_run once after the last set-up call);
 * ray recording is not done here. */
typedef struct {
  mc_ctx* ctx;             /* the batch's problem */
  int64_t first_history;   /* 0-based index of its first history (id = index + 1) */
  int64_t n_histories;     /* 1 .. 2^31 - 1 */
  uint64_t seed;           /* master seed */
} mc_job;

typedef struct {
  int32_t precision;       /* MC_PREC_* */
  int32_t block_size;      /* threads per block: a multiple of 32, at most 128 (0: 128) */
  int32_t slots;           /* tally slots per problem (0: one per batch, no waits) */
  int32_t record_traces;   /* 1: one mc_trace per history into traces, batches in the order given */
  int64_t wait_limit;      /* polls (about a microsecond apart) before a wait gives up (0: 10,000,000) */
  mc_trace* traces;        /* HOST buffer of the run's histories when record_traces */
} mc_persist_desc;

/* stats (optional) receives the run's counters; each problem's mc_stats_get
 * returns them too, and mc_batches_done counts its batches. */
int mc_run_persistent(const mc_persist_desc* desc, int32_t n_jobs, const mc_job* jobs, mc_stats* stats);

/* ---- batch run without device allocation ------------------------------
 * No counterpart in the reference: MaCaw itself never allocates device
 * memory.  mc_run obtains its particle bank, event queues and counters with
 * cudaMalloc the first time it needs them.  Callers that cannot allow a
 * device allocation at run time (an application whose memory pool owns the
 * whole GPU, a serving process that budgets HBM up front, code running where
 * an allocation would stall or fail) use mc_run_noalloc instead: it tracks
 * the same histories in the event form, but its scratch is one fixed array
 * of MC_NOALLOC_MAX_BANK particle slots (220 bytes each plus a control
 * block: about 3.60 MB) compiled into the library.  It calls no cudaMalloc,
 * cudaFree or other allocating routine.
 *
 * - The array and the event-form kernels are put on a device by
 *   mc_ctx_create (the CUDA driver loads them lazily, so this is done while
 *   the caller can still let the library take memory): every device that
 *   has had a context holds the array until the process exits.  The first
 *   mc_run_noalloc call leaves the device's free memory unchanged.
 * - bank_size must be at most MC_NOALLOC_MAX_BANK (0 means the maximum);
 *   larger values are rejected with MC_ERR_ARG.  Any number of histories
 *   is fine: the bank is refilled as histories end.
 * - tally: caller-owned DEVICE buffer of mc_tally_size doubles; scores are
 *   added to it, so clear it first.  traces: caller-owned DEVICE buffer of
 *   n_histories records when record_traces is set, else NULL.
 * - Stream: the work runs on the context's stream (mc_ctx_set_stream), with
 *   no ordering against the caller's other streams.  The caller's tally and
 *   trace buffers must be ready when the call is made: clear them on the
 *   context's stream, or synchronize before the call.  The call returns
 *   after the work has finished.
 * - The mesh, tables, block map, boundary conditions and source must already
 *   be on the device: after the last set-up call, run mc_run once (for
 *   example with n_histories = 0).  Rejected with MC_ERR_ARG, as each would
 *   need memory, events or a graph: host source sites, accumulate, profile,
 *   pipelined batches (n_batches > 1, batch_sizes, batch_sum_out),
 *   sort_queue > 0, graph, and a context with ray recording on.
 * - All calls on a device share the one array and it keeps the last call's
 *   contents (the library clears what must start at zero).  Calls whose
 *   work overlaps on the GPU race on it: run them one after another. */
#define MC_NOALLOC_MAX_BANK 16384
int mc_run_noalloc(mc_ctx* ctx, const mc_run_desc* desc, double* tally, mc_trace* traces);

/* ---- serving: continuous batching of fixed-source requests ------------
 * No counterpart in the reference (MaCaw runs one input file per process).
 * A context with its mesh and cross sections resident takes requests as
 * they arrive.  Each admitted request gets a tally slot (mc_tally_size
 * doubles, the context's tally definition) and
 * its histories join the shared particle bank, born as slots free up, so
 * requests overlap on the device without draining between them.  Request
 * particle ids are 1..n_histories under the request's seed: a request's
 * result does not depend on what else is in flight.  While serving is open,
 * mc_run in the event form is rejected on this context. */
typedef struct {
  int64_t n_histories;
  uint64_t seed;
  mc_source_desc source;  /* point or box space; Watt or mono energy */
} mc_request;
/* max_slots requests in flight (tally memory max_slots*mc_tally_size*8 bytes),
 * bank_size particles in flight, precision MC_PREC_*, max_seg segments per
 * walk launch (0: until an event). */
int mc_serve_open(mc_ctx* ctx, int32_t max_slots, int64_t bank_size, int32_t precision, int32_t max_seg);
int mc_serve_submit(mc_ctx* ctx, const mc_request* req, int64_t* ticket);
/* Admits queued requests into free slots and launches `iterations` event
 * iterations (asynchronous). */
int mc_serve_step(mc_ctx* ctx, int32_t iterations);
/* Waits for launched work; retires finished requests, writing up to
 * capacity tickets into done and their count into n_done. */
int mc_serve_poll(mc_ctx* ctx, int64_t* done, int32_t capacity, int32_t* n_done);
/* FP64 tally of a finished request (raw sums, mc_tally_size values; the
 * default definition: wgt*length per element). */
int mc_serve_result(mc_ctx* ctx, int64_t ticket, double* tally, int64_t n);
int mc_serve_status(mc_ctx* ctx, int32_t* queued, int32_t* active, int32_t* free_slots);
int mc_serve_close(mc_ctx* ctx);

/* ---- ray segments ------------------------------------------------------
 * Replaces: MOOSE RayTracingExodus output of a study's rays with their data
 * and aux data (test/tests/study/openmc_study.i [Outputs/rays]; gold
 * test/tests/study/gold/openmc_study_rays.e).  mc_rays_enable makes the
 * following runs record every segment of their first n_rays histories (in
 * birth order), up to max_segments each; mc_rays_download returns the
 * recorded segments of the last run, ray by ray in segment order. */
typedef struct {
  int64_t id;             /* particle id (1-based); the ray is id - 1 - first_history of the run */
  int32_t segment;        /* index along the ray, from 0 */
  int32_t intersections;  /* sides the ray crossed so far, this segment's included */
  int32_t elem;           /* element the segment lies in */
  int32_t pad;
  double start[3], end[3];
  double E, wgt;          /* energy and weight along the segment */
  uint64_t seed_tracking; /* tracking-stream state after the segment's draw */
} mc_ray_segment;
int mc_rays_enable(mc_ctx* ctx, int32_t n_rays, int32_t max_segments);
int mc_rays_download(mc_ctx* ctx, mc_ray_segment* out, int64_t capacity, int64_t* n_out);
/* Writes recorded segments as RayTracingExodus does: one EDGE2 element per
 * segment, consecutive segments of a ray sharing their node, element
 * variables aux_energy, aux_id, aux_n_progeny, aux_particle_type,
 * aux_seed_URR, aux_seed_source, aux_seed_tracking, aux_weight,
 * intersections and ray_id (seeds as doubles, as MaCaw stores them). */
int mc_exodus_write_rays(const char* path, const mc_ray_segment* seg, int64_t n, int64_t first_history);

/* ---- Exodus II output --------------------------------------------------
 * Replaces: MOOSE's Exodus output of a MaCaw run's element AuxVariables
 * ([Outputs] exodus = true; the reference's gold results are Exodus files,
 * test/tests/study/gold/openmc_study_rays.e).  Writes path as an Exodus II
 * file in netCDF's 64-bit-offset format: nodes, one TETRA4 element block
 * per subdomain (ascending id, elements in mesh order), side sets from
 * tet_side_bid (optional, as for mc_mesh_upload; only faces no other tet
 * shares), n_vars element variables named names[i] with
 * values[i*n_tet + elem], one time step. */
int mc_exodus_write(const char* path, const char* title, int64_t n_vtx, const double* xyz, int64_t n_tet,
                    const int32_t* tet_vtx, const int32_t* tet_block, const int32_t* tet_side_bid, int32_t n_vars,
                    const char* const* names, const double* values, double time);
/* Replaces: MOOSE FileMeshGenerator reading the mesh MaCaw traces on
 * (examples/beavrs_assembly/run_assembly.i [Mesh]).  Reads an Exodus II
 * file (netCDF classic or 64-bit offset): every element block must be
 * 4-node tetrahedra; elements are numbered in block order and take their
 * block's id; side sets set tet_side_bid (optional, 4 per tet, -1 where no
 * side set names the face).  On failure err (optional) holds the reason. */
int mc_exodus_read_sizes(const char* path, int64_t* n_vtx, int64_t* n_tet, char* err, int64_t err_len);
int mc_exodus_read(const char* path, double* xyz, int32_t* tet_vtx, int32_t* tet_block, int32_t* tet_side_bid,
                   char* err, int64_t err_len);

/* ---- input-file front end ---------------------------------------------
 * Replaces: running a MaCaw input (MooseApp::run on an .i file; src/main.C)
 * for the tracking path.  Parses the HIT blocks [Mesh] (TetCubeMeshGenerator,
 * TetLatticeMeshGenerator), [RayKernels] CollisionKernel, [RayBCs]
 * KillRayBC / ReflectRayBC, [UserObjects] OpenMCStudy, OpenMCTally and
 * SyntheticCrossSections, [AuxKernels] OpenMCTallyAux, [Executioner]
 * Transient (num_steps = batches) and [Outputs] (csv, file_base); checks
 * parameters as the objects' validParams do; runs every batch on the
 * device; writes a JSON summary into report.  mc_app_check does the
 * parsing and checks only, without a device. */
int mc_app_run(const char* input_text, int device, const char* file_base, char* report, int64_t report_len);
int mc_app_check(const char* input_text, char* report, int64_t report_len);

/* ---- synthetic problem generators (host only; no device needed) ------ */
/* Box [lo, hi] of nx x ny x nz hexes, six Kuhn tets each (split along each
 * hex's main diagonal): MOOSE's GeneratedMeshGenerator with dim = 3, as
 * test/tests/study/openmc_study.i:2-14 builds its 5 x 5 x 1 box, cut into
 * tets.  Vertex (i, j, k) sits at lo + i * (hi - lo) / n per axis (the last
 * plane at hi itself); sidesets 0..5 as MOOSE's GeneratedMesh (back,
 * bottom, right, top, left, front); every tet in block 0. */
int mc_gen_box_sizes(int32_t nx, int32_t ny, int32_t nz, int64_t* n_vtx, int64_t* n_tet);
int mc_gen_box(int32_t nx, int32_t ny, int32_t nz, const double* lo, const double* hi, double* xyz,
               int32_t* tet_vtx, int32_t* tet_block, int32_t* tet_side_bid);
/* Cube [0,L]^3 of n^3 hexes, six Kuhn tets each; sidesets 0..5 as MOOSE's
 * GeneratedMesh (back, bottom, right, top, left, front). */
int mc_gen_cube_sizes(int32_t n, int64_t* n_vtx, int64_t* n_tet);
int mc_gen_cube(int32_t n, double L, double* xyz, int32_t* tet_vtx, int32_t* tet_block,
                int32_t* tet_side_bid);
/* Square lattice of nx*ny pin cells (pitch, height, nz axial layers, n_sec
 * azimuthal sectors), rings at r_fuel / r_clad; blocks 1 fuel, 2 clad,
 * 3 moderator; outer sidesets 0..5. */
int mc_gen_lattice_sizes(int32_t nx, int32_t ny, int32_t nz, int32_t n_sec, int32_t n_fuel_rings,
                         int64_t* n_vtx, int64_t* n_tet);
int mc_gen_lattice(int32_t nx, int32_t ny, int32_t nz, int32_t n_sec, int32_t n_fuel_rings,
                   double pitch, double height, double r_fuel, double r_clad, double* xyz,
                   int32_t* tet_vtx, int32_t* tet_block, int32_t* tet_side_bid);
/* Cylindrical core: 193 assemblies of pins x pins pin cells on a 15 x 15
 * assembly grid (rows of 7, 11, 13, 13, 15 x7, 13, 13, 11, 7) centred on the
 * z axis, plus whole reflector cells whose corners lie inside radius; nz
 * axial layers over [0, height].  Blocks: fuel 1..193 (one per assembly),
 * clad 194, moderator 195, reflector 196..200 (five 72-degree sectors).
 * The square grid of cells extends past the assemblies far enough to reach
 * the radius.  Sidesets: bottom 0, top 5, radial staircase 6.  pin_xy
 * (optional, 2*n_pins) receives the pin-cell centres. */
int mc_gen_core_sizes(int32_t pins, int32_t nz, int32_t n_sec, int32_t n_fuel_rings, double pitch, double radius,
                      int64_t* n_vtx, int64_t* n_tet, int64_t* n_pins);
int mc_gen_core(int32_t pins, int32_t nz, int32_t n_sec, int32_t n_fuel_rings, double pitch, double height,
                double r_fuel, double r_clad, double radius, double* xyz, int32_t* tet_vtx, int32_t* tet_block,
                int32_t* tet_side_bid, double* pin_xy);
/* Synthetic nuclide: n_pts log-uniform energies in [E_min, E_max] eV,
 * sigma_t = a/sqrt(E) + n_peaks Lorentzians, sigma_s = f_s*sigma_t,
 * awr; all drawn from (seed, index). */
int mc_gen_nuclide(uint64_t seed, int32_t index, int64_t n_pts, double E_min, double E_max,
                   int32_t n_peaks, double* E, double* sig_t, double* sig_s, double* awr);
/* n atom densities uniform in [lo, hi] drawn from (seed, index). */
int mc_gen_densities(uint64_t seed, int32_t index, int32_t n, double lo, double hi, double* out);

#ifdef __cplusplus
}
#endif
#endif
