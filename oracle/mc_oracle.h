/*
 * mc_oracle.h -- CPU restatement of MaCaw's particle-tracking hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle that the GPU path is
 * checked against, and the timed CPU baseline.  Nothing in the product
 * (macaw_gb300/) links, loads or calls it.
 *
 * Parity pin: the random-number scheme (64-bit PCG state step, Brown
 * skip-ahead, per-history seeds future_seed(id*152917, master+stream)) is
 * checked against the per-segment seed states stored in the reference's
 * only golden file, test/tests/study/gold/openmc_study_rays.e.  The
 * geometry walk, cross-section lookup and collision physics live in the
 * reference's absent dependencies (MOOSE TraceRay, OpenMC 0.13); for them
 * parity is unpinned and the restatement follows the reference's call
 * sites and the published algorithms named beside each function.
 *
 * Compiled with -ffp-contract=off so every floating-point operation is a
 * single IEEE-754 double operation in source order.
 */
#ifndef MC_ORACLE_H
#define MC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_problem oracle_problem;

/* Source description (mirrors the fixed-source settings OpenMC reads from
 * settings.xml; OpenMCStudy::defineRays samples one site per history,
 * src/userobjects/OpenMCStudy.C:317-360). */
typedef struct {
  int32_t space;      /* 0 point, 1 box, 2 cylinders */
  int32_t energy;     /* 0 Watt, 1 mono-energetic */
  double point[3];
  double box_lo[3];
  double box_hi[3];
  int32_t n_cyl;
  int32_t pad;
  const double* cyl_xy; /* 2*n_cyl centres */
  double cyl_r, cyl_z0, cyl_z1;
  double watt_a, watt_b; /* eV, 1/eV */
  double mono_E;         /* eV */
} oracle_source;

/* Per-history outcome record; the bit-exact parity target. */
typedef struct {
  int64_t id;       /* 1-based particle id */
  uint64_t hash;    /* FNV-1a over (element, segment outcome) */
  int32_t status;   /* 1 leaked 2 absorbed 3 cutoff 4 stuck 5 lost 6 bad xs */
  int32_t n_seg;
  int32_t n_coll;
  int32_t elem;     /* last element */
  int32_t face;     /* exit face for leaked, else -1 */
  int32_t pad;
  double E;         /* last energy (eV) */
  double x, y, z;   /* last position */
} oracle_trace;

/* One recorded segment of a history (the fields of the GPU library's
 * mc_ray_segment, the per-segment output MOOSE's RayTracingExodus writes for
 * a study's rays; test/tests/study/gold/openmc_study_rays.e). */
typedef struct {
  int64_t id;             /* particle id (1-based) */
  int32_t segment;        /* index along the ray */
  int32_t intersections;  /* segments that ended on a side, this one included */
  int32_t elem;
  int32_t pad;
  double start[3], end[3];
  double E, wgt;          /* energy and weight along the segment */
  uint64_t seed_tracking; /* tracking-stream state after the segment's draw */
} oracle_ray_seg;

typedef struct {
  int64_t n_hist, n_seg, n_coll, n_leak, n_absorb, n_cutoff, n_stuck, n_lost, n_badxs;
  double leak_weight;
} oracle_stats;

/* One fission site (OpenMC SourceSite as create_fission_sites fills it). */
typedef struct {
  double x, y, z, u, v, w, E, wgt;
  int64_t parent;   /* id of the history that banked it */
  int32_t progeny;  /* its index among that history's sites */
  int32_t pad;
} oracle_fsite;

/* Results of one k-eigenvalue generation. */
typedef struct {
  double k_generation, k_collision, k_absorption, keff, keff_std, leakage;
  int64_t n_sites, n_seg, n_coll;
} oracle_gen;

oracle_problem* oracle_create(void);
void oracle_destroy(oracle_problem* p);
const char* oracle_error(oracle_problem* p);

/* Mesh: vertices, tets (4 vertex ids), subdomain id per tet and an optional
 * sideset id per tet side (-1 for none; side f is opposite local vertex f). */
int oracle_set_mesh(oracle_problem* p, int64_t n_vtx, const double* xyz, int64_t n_tet,
                    const int32_t* tet_vtx, const int32_t* tet_block, const int32_t* tet_side_bid);
/* boundary id -> 0 vacuum (KillRayBC), 1 reflective (ReflectRayBC) */
int oracle_set_bc(oracle_problem* p, int32_t bid, int32_t type);
int oracle_add_nuclide(oracle_problem* p, int64_t n_pts, const double* E, const double* sig_t,
                       const double* sig_s, double awr);
/* material_id is the OpenMC-style 1-based id; nuclides are 0-based indices */
int oracle_add_material(oracle_problem* p, int32_t material_id, int32_t n, const int32_t* nuclides,
                        const double* densities);
/* CollisionKernel blocks/materials parameters (src/raykernels/CollisionKernel.C:63-69) */
int oracle_block_map(oracle_problem* p, int32_t n, const int32_t* blocks, const int32_t* materials);
int oracle_set_source(oracle_problem* p, const oracle_source* s);
int oracle_set_hash_bins(oracle_problem* p, int32_t n_bins);
/* estimator 1 track length (scores 0 flux, 1 total), 2 collision (0 flux,
 * 1 total, 2 scatter, 3 absorption); n_energy_bins 0: no energy filter.
 * oracle_run's tally then holds oracle_tally_size values laid out
 * [element][energy bin][score]. */
int oracle_set_tally(oracle_problem* p, int32_t estimator, int32_t n_scores, const int32_t* scores,
                     int32_t n_energy_bins, const double* edges);
int64_t oracle_tally_size(const oracle_problem* p);
/* 2-D mode: planar directions, births at z = z_coord (CollisionKernel z_coord). */
int oracle_set_2d(oracle_problem* p, int32_t on, double z_coord);

/* Track histories [first, first+n) (0-based history index h, particle id
 * h+1).  tally (n_tet doubles) accumulates raw wgt*track-length sums;
 * traces (n entries) may be NULL. */
int oracle_run(oracle_problem* p, int64_t first, int64_t n, uint64_t seed, int n_threads,
               double* tally, oracle_trace* traces, oracle_stats* stats);

/* As oracle_run, with history i born from sites[8i..8i+7] (x y z u v w E
 * wgt) instead of the source; the tracking stream is still keyed by the id. */
int oracle_run_sites(oracle_problem* p, int64_t first, int64_t n, uint64_t seed, const double* sites,
                     int n_threads, double* tally, oracle_trace* traces, oracle_stats* stats);
/* Segments a history may walk before it ends as stuck (0: the default,
 * 4096 * ceil(cbrt(n_tet)) clamped to [65536, 1e7]); oracle_segment_limit
 * returns the limit in force. */
int oracle_set_segment_limit(oracle_problem* p, int64_t max_segments);
int64_t oracle_segment_limit(const oracle_problem* p);
/* Records every segment of the first n_rays histories of each following
 * run, up to max_segments each (0: off); oracle_rays returns them ray by
 * ray in segment order (*n_out: their number). */
int oracle_rays_enable(oracle_problem* p, int32_t n_rays, int32_t max_segments);
int oracle_rays(oracle_problem* p, oracle_ray_seg* out, int64_t capacity, int64_t* n_out);

/* nu*sigma_f per grid point of a nuclide (NULL: not fissionable).  A
 * fissionable nuclide samples fission sites at each collision with it:
 * banked by oracle_eigen_run, drawn and dropped by oracle_run. */
int oracle_set_fission(oracle_problem* p, int32_t nuclide, const double* nu_sig_f);

/* n_gen generations of n histories (generation g: history indices g*n..);
 * the first from init_src (n x 8 doubles: x y z u v w E wgt) or, when NULL,
 * from the source (ids 1..n, source stream).  keff0, fa, fb, cap <= 0 take
 * 1, 0.988e6 eV, 2.249e-6 /eV, 3n.  out: n_gen records; src_out (n x 8):
 * the sites of the next generation; bank_out: the last generation's sorted
 * bank (first bank_cap sites), *bank_n its size; tally_sum (optional,
 * oracle_tally_size values) accumulates batch/n over active generations. */
int oracle_eigen_run(oracle_problem* p, int64_t n, int32_t n_gen, int32_t n_inactive, uint64_t seed,
                     double keff0, double fa, double fb, int64_t cap, int n_threads, const double* init_src,
                     oracle_gen* out, double* src_out, oracle_fsite* bank_out, int64_t bank_cap,
                     int64_t* bank_n, double* tally_sum);

/* Pieces exposed for unit tests. */
double oracle_log(double x);
double oracle_quotient(double num, double den);
double oracle_prn(uint64_t* seed);
uint64_t oracle_future_seed(uint64_t n, uint64_t seed);
uint64_t oracle_init_seed(int64_t id, uint64_t master, int stream);
int oracle_xs_index(oracle_problem* p, int32_t nuclide, double E, double* f_out);
int oracle_macro_xs(oracle_problem* p, int32_t material_index, double E, double* sig_t);
int oracle_mesh_info(oracle_problem* p, const int32_t** nbr, const double** planes);
int oracle_locate(oracle_problem* p, const double* x, const double* u);

#ifdef __cplusplus
}
#endif
#endif
