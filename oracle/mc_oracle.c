/*
 * mc_oracle.c -- CPU restatement of MaCaw's particle-tracking hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU path and the timed CPU
 * baseline.  The product never links or calls this file.
 *
 * What it restates, with the reference call sites it follows:
 *  - source birth per history, in index order, ids 1-based
 *      src/userobjects/OpenMCStudy.C:317-360 (OpenMC initialize_history)
 *  - start-element location (MOOSE ClaimRays, absent), deterministic rule
 *  - element walk (MOOSE TraceRay, absent) as a plane-based tet walk
 *  - per segment: macroscopic XS (CollisionKernel.C:143), a fresh
 *    distance-to-collision sample d = -ln(xi)/Sigma_t (CollisionKernel.C:150),
 *    track-length score wgt*min(d, L) (CollisionKernel.C:153-154; the flux
 *    score per element replaces the keff score), cross if d > L
 *    (CollisionKernel.C:163-169), else collide at end-(L-d)*u
 *    (CollisionKernel.C:173-182)
 *  - collision (OpenMC event_collide, absent): nuclide, absorb/scatter,
 *    elastic target-at-rest kinematics; scatter restarts in the same
 *    element (CollisionKernel.C:204-205); absorption ends the history
 *    (CollisionKernel.C:226-230); no secondaries (CollisionKernel.C:236)
 *  - material of an element = block map id - 1 (CollisionKernel.C:110)
 *  - fission sites at collisions with fissionable nuclides (OpenMC
 *    create_fission_sites) and, in k-eigenvalue runs, the track-length,
 *    collision and absorption keff estimators (CollisionKernel.C:153-154;
 *    OpenMC event_collide, absorption), the bank sort and the resampling
 *    of OpenMCStudy::synchronizeBanks (OpenMCStudy.C:430-607)
 *
 * Parity pin: the RNG (below) is checked against the seed states in
 * test/tests/study/gold/openmc_study_rays.e.  The rest is unpinned.
 *
 * Build: cc -O2 -ffp-contract=off -fopenmp -fPIC -shared.
 */
#include "mc_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* Random numbers: OpenMC 0.13 scheme.  State step of the 64-bit PCG LCG
 * (O'Neill 2014, multiplier/increment of Knuth's MMIX), RXS-M-XS output
 * permutation, Brown (1994) arbitrary-stride skip-ahead, stride 152917 per
 * particle id, one stream per purpose (0 tracking, 2 source).            */
#define PRN_MULT 6364136223846793005ULL
#define PRN_ADD 1442695040888963407ULL
#define PRN_STRIDE 152917ULL

double oracle_prn(uint64_t* seed)
{
  uint64_t s = PRN_MULT * (*seed) + PRN_ADD;
  *seed = s;
  uint64_t w = ((s >> ((s >> 59u) + 5u)) ^ s) * 12605985483714917081ULL;
  w = (w >> 43u) ^ w;
  return (double)(w >> 11) * 0x1.0p-53;
}

uint64_t oracle_future_seed(uint64_t n, uint64_t seed)
{
  uint64_t g = PRN_MULT, c = PRN_ADD, G = 1, C = 0;
  while (n > 0) {
    if (n & 1ULL) {
      G = G * g;
      C = C * g + c;
    }
    c = (g + 1ULL) * c;
    g = g * g;
    n >>= 1;
  }
  return G * seed + C;
}

uint64_t oracle_init_seed(int64_t id, uint64_t master, int stream)
{
  return oracle_future_seed((uint64_t)id * PRN_STRIDE, master + (uint64_t)stream);
}

/* ------------------------------------------------------------------ */
/* num / den by Markstein's division sequence (P. Markstein, IBM J. Res.
 * Dev. 34(1), 1990): the correctly rounded float reciprocal of den, one
 * Newton step in double, and the quotient corrected by its residual;
 * within an ulp of the IEEE quotient.  A den whose float lies outside
 * [2^-100, 2^100] takes the IEEE division.  The device computes the same
 * sequence (mc::quotient), which needs five FP64 operations on the GPU
 * against a division's more.  It gives the walk's exit distance (in the
 * reference the MOOSE ray tracer's segment length, which onSegment reads
 * as _current_segment_length, src/raykernels/CollisionKernel.C:154,163),
 * the distance to collision, the log's atanh argument and the rejection
 * samplers' ratios. */
double oracle_quotient(double num, double den)
{
  const float df = (float)den;
  const float da = fabsf(df);
  if (!(da >= 0x1p-100f && da <= 0x1p100f)) return num / den;
  const double y0 = (double)(1.0f / df);
  const double y1 = fma(y0, fma(-den, y0, 1.0), y0);
  const double q0 = num * y1;
  return fma(fma(-den, q0, num), y1, q0);
}

/* ------------------------------------------------------------------ */
/* Natural log from the series ln(m) = 2 atanh((m-1)/(m+1)), m in
 * [sqrt(1/2), sqrt(2)), eleven odd terms, plus e*ln2 split hi/lo; the
 * Horner steps and final sums as fused multiply-adds, the atanh argument
 * by oracle_quotient -- as the device's mc::log64.                     */
double oracle_log(double x)
{
  if (!(x > 0.0)) {
    if (x == 0.0) return -INFINITY;
    return NAN;
  }
  if (x == INFINITY) return x;
  uint64_t b;
  memcpy(&b, &x, 8);
  int e = (int)((b >> 52) & 0x7ffULL);
  if (e == 0) {
    double y = x * 18014398509481984.0; /* 2^54 */
    memcpy(&b, &y, 8);
    e = (int)((b >> 52) & 0x7ffULL) - 54;
  }
  e -= 1023;
  b = (b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL;
  double m;
  memcpy(&m, &b, 8);
  if (m > 1.4142135623730951) {
    m = m * 0.5;
    e += 1;
  }
  double f = oracle_quotient(m - 1.0, m + 1.0);
  double s = f * f;
  double p = 0.043478260869565216;        /* 1/23 */
  p = fma(s, p, 0.047619047619047616);    /* 1/21 */
  p = fma(s, p, 0.05263157894736842);     /* 1/19 */
  p = fma(s, p, 0.058823529411764705);    /* 1/17 */
  p = fma(s, p, 0.06666666666666667);     /* 1/15 */
  p = fma(s, p, 0.07692307692307693);     /* 1/13 */
  p = fma(s, p, 0.09090909090909091);     /* 1/11 */
  p = fma(s, p, 0.1111111111111111);      /* 1/9 */
  p = fma(s, p, 0.14285714285714285);     /* 1/7 */
  p = fma(s, p, 0.2);                     /* 1/5 */
  p = fma(s, p, 0.3333333333333333);      /* 1/3 */
  p = s * p;
  double t = 2.0 * f;
  double r = fma(t, p, t);
  double de = (double)e;
  return fma(de, 0.6931471803691238, fma(de, 1.9082149292705877e-10, r));
}

/* ------------------------------------------------------------------ */
typedef struct {
  int64_t n_pts;
  double* E;
  double* st;
  double* ss;
  double awr;
  int32_t* hidx; /* n_bins+1 */
  double* nusf;  /* nu*sigma_f per point, or NULL: not fissionable */
} nuclide_t;

typedef struct {
  int32_t id;
  int32_t n;
  int32_t* nuc;
  double* dens;
} material_t;

struct oracle_problem {
  char err[512];
  /* mesh */
  int64_t n_vtx, n_tet;
  double* xyz;
  int32_t* tv;
  int32_t* blk;
  int32_t* side_bid; /* 4 per tet, boundary id (>=0) for boundary sides */
  int32_t* nbr;      /* 4 per tet, -1 boundary */
  double* planes;    /* 16 per tet: (nx,ny,nz,d) per side */
  int32_t* tmat;     /* material index per tet (-1 none) */
  /* locator */
  double glo[3], gh[3];
  int gn[3];
  int64_t* gstart;
  int32_t* gtets;
  /* bcs */
  int32_t bc_type[1024];
  /* data */
  int32_t n_nuc, cap_nuc;
  nuclide_t* nucs;
  int32_t n_mat, cap_mat;
  material_t* mats;
  int32_t n_map;
  int32_t* map_blocks;
  int32_t* map_mats;
  int32_t n_bins;
  double E_lo, E_hi, lE_lo, du;
  int data_ready;
  oracle_source src;
  double* src_cyl;
  /* tally definition (OpenMCTally estimator, scores, energy filter);
     results [element][energy bin][score] */
  int t_est;        /* 1 track length, 2 collision */
  int t_ns, t_nb;   /* scores, energy bins (>= 1) */
  int t_sc[4];      /* 0 flux, 1 total, 2 scatter, 3 absorption */
  double* t_edges;  /* t_nb+1 edges, or NULL: no energy filter */
  /* 2-D mode (CollisionKernel z_coord) */
  int two_d;
  double z2d;
  /* segments a history may walk before it is ended as stuck (0: the
     mesh-size default, segment_limit()) */
  int64_t seg_limit;
  /* segment recording (oracle_rays_enable): histories first..first+ray_n-1
     of the last run, ray_cap segments each */
  int32_t ray_n, ray_cap;
  oracle_ray_seg* rays;
  int32_t* ray_cnt;
};

static int fail(oracle_problem* p, const char* msg)
{
  snprintf(p->err, sizeof p->err, "%s", msg);
  return 1;
}

oracle_problem* oracle_create(void)
{
  oracle_problem* p = (oracle_problem*)calloc(1, sizeof(oracle_problem));
  p->n_bins = 8000;
  p->src.space = 0;
  p->src.energy = 0;
  p->src.watt_a = 0.988e6;
  p->src.watt_b = 2.249e-6;
  p->t_est = 1;
  p->t_ns = 1;
  p->t_nb = 1;
  return p;
}

static void free_mesh(oracle_problem* p)
{
  free(p->xyz); free(p->tv); free(p->blk); free(p->side_bid); free(p->nbr);
  free(p->planes); free(p->tmat); free(p->gstart); free(p->gtets);
  p->xyz = NULL; p->tv = NULL; p->blk = NULL; p->side_bid = NULL; p->nbr = NULL;
  p->planes = NULL; p->tmat = NULL; p->gstart = NULL; p->gtets = NULL;
}

void oracle_destroy(oracle_problem* p)
{
  if (!p) return;
  free_mesh(p);
  for (int i = 0; i < p->n_nuc; ++i) {
    free(p->nucs[i].E); free(p->nucs[i].st); free(p->nucs[i].ss); free(p->nucs[i].hidx);
    free(p->nucs[i].nusf);
  }
  free(p->nucs);
  for (int i = 0; i < p->n_mat; ++i) { free(p->mats[i].nuc); free(p->mats[i].dens); }
  free(p->mats);
  free(p->map_blocks); free(p->map_mats); free(p->src_cyl); free(p->t_edges);
  free(p->rays); free(p->ray_cnt);
  free(p);
}

const char* oracle_error(oracle_problem* p) { return p->err; }

/* ------------------------------------------------------------------ */
/* Mesh preprocessing: face adjacency by sorted vertex triples, one
 * canonical plane per distinct face (vertices in increasing global id),
 * oriented outward per tet so the two sides of an interior face carry
 * exactly negated planes.  Side f is opposite local vertex f.            */
typedef struct { int32_t a, b, c; int64_t side; } facekey;

static int cmp_face(const void* x, const void* y)
{
  const facekey* p = (const facekey*)x;
  const facekey* q = (const facekey*)y;
  if (p->a != q->a) return p->a < q->a ? -1 : 1;
  if (p->b != q->b) return p->b < q->b ? -1 : 1;
  if (p->c != q->c) return p->c < q->c ? -1 : 1;
  return p->side < q->side ? -1 : (p->side > q->side ? 1 : 0);
}

static const int FACE_VTX[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};

static void sort3(int32_t* v)
{
  int32_t t;
  if (v[0] > v[1]) { t = v[0]; v[0] = v[1]; v[1] = t; }
  if (v[1] > v[2]) { t = v[1]; v[1] = v[2]; v[2] = t; }
  if (v[0] > v[1]) { t = v[0]; v[0] = v[1]; v[1] = t; }
}

static int build_planes(oracle_problem* p)
{
  for (int64_t t = 0; t < p->n_tet; ++t) {
    for (int f = 0; f < 4; ++f) {
      int32_t v[3] = {p->tv[4 * t + FACE_VTX[f][0]], p->tv[4 * t + FACE_VTX[f][1]],
                      p->tv[4 * t + FACE_VTX[f][2]]};
      sort3(v);
      const double* A = p->xyz + 3 * (int64_t)v[0];
      const double* B = p->xyz + 3 * (int64_t)v[1];
      const double* C = p->xyz + 3 * (int64_t)v[2];
      const double* O = p->xyz + 3 * (int64_t)p->tv[4 * t + f];
      double e1x = B[0] - A[0], e1y = B[1] - A[1], e1z = B[2] - A[2];
      double e2x = C[0] - A[0], e2y = C[1] - A[1], e2z = C[2] - A[2];
      double nx = e1y * e2z - e1z * e2y;
      double ny = e1z * e2x - e1x * e2z;
      double nz = e1x * e2y - e1y * e2x;
      double len = sqrt(nx * nx + ny * ny + nz * nz);
      if (!(len > 0.0)) return fail(p, "degenerate tet face");
      nx = nx / len;
      ny = ny / len;
      nz = nz / len;
      double d = nx * A[0] + ny * A[1] + nz * A[2];
      double s = nx * O[0] + ny * O[1] + nz * O[2] - d;
      if (s == 0.0) return fail(p, "degenerate tet (zero volume)");
      if (s > 0.0) { nx = -nx; ny = -ny; nz = -nz; d = -d; }
      double* P = p->planes + 16 * t + 4 * f;
      P[0] = nx; P[1] = ny; P[2] = nz; P[3] = d;
    }
  }
  return 0;
}

static int build_adjacency(oracle_problem* p)
{
  int64_t nf = 4 * p->n_tet;
  facekey* keys = (facekey*)malloc(sizeof(facekey) * (size_t)nf);
  if (!keys) return fail(p, "out of memory");
  for (int64_t t = 0; t < p->n_tet; ++t)
    for (int f = 0; f < 4; ++f) {
      int32_t v[3] = {p->tv[4 * t + FACE_VTX[f][0]], p->tv[4 * t + FACE_VTX[f][1]],
                      p->tv[4 * t + FACE_VTX[f][2]]};
      sort3(v);
      facekey* k = keys + 4 * t + f;
      k->a = v[0]; k->b = v[1]; k->c = v[2]; k->side = 4 * t + f;
    }
  qsort(keys, (size_t)nf, sizeof(facekey), cmp_face);
  for (int64_t i = 0; i < nf; ++i) p->nbr[i] = -1;
  int64_t i = 0;
  while (i < nf) {
    int64_t j = i + 1;
    while (j < nf && keys[j].a == keys[i].a && keys[j].b == keys[i].b && keys[j].c == keys[i].c) ++j;
    if (j - i > 2) { free(keys); return fail(p, "non-manifold face shared by more than two tets"); }
    if (j - i == 2) {
      p->nbr[keys[i].side] = (int32_t)(keys[i + 1].side / 4);
      p->nbr[keys[i + 1].side] = (int32_t)(keys[i].side / 4);
    }
    i = j;
  }
  free(keys);
  return 0;
}

static int build_locator(oracle_problem* p)
{
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t v = 0; v < p->n_vtx; ++v)
    for (int k = 0; k < 3; ++k) {
      double c = p->xyz[3 * v + k];
      if (c < lo[k]) lo[k] = c;
      if (c > hi[k]) hi[k] = c;
    }
  double ext[3], vol = 1.0;
  for (int k = 0; k < 3; ++k) {
    ext[k] = hi[k] - lo[k];
    if (!(ext[k] > 0.0)) ext[k] = 1.0;
    vol *= ext[k];
  }
  double target = (double)p->n_tet / 2.0;
  if (target < 1.0) target = 1.0;
  double h = cbrt(vol / target);
  int64_t ncell = 1;
  for (int k = 0; k < 3; ++k) {
    int n = (int)(ext[k] / h);
    if (n < 1) n = 1;
    if (n > 1024) n = 1024;
    p->gn[k] = n;
    p->glo[k] = lo[k];
    p->gh[k] = ext[k] / n;
    ncell *= n;
  }
  int64_t* cnt = (int64_t*)calloc((size_t)ncell + 1, sizeof(int64_t));
  const double tol = 1e-9;
  for (int pass = 0; pass < 2; ++pass) {
    if (pass == 1) {
      int64_t acc = 0;
      for (int64_t c = 0; c < ncell; ++c) { int64_t n = cnt[c]; cnt[c] = acc; acc += n; }
      cnt[ncell] = acc;
      p->gstart = (int64_t*)malloc(sizeof(int64_t) * (size_t)(ncell + 1));
      memcpy(p->gstart, cnt, sizeof(int64_t) * (size_t)(ncell + 1));
      p->gtets = (int32_t*)malloc(sizeof(int32_t) * (size_t)(acc > 0 ? acc : 1));
    }
    for (int64_t t = 0; t < p->n_tet; ++t) {
      double blo[3] = {INFINITY, INFINITY, INFINITY}, bhi[3] = {-INFINITY, -INFINITY, -INFINITY};
      for (int a = 0; a < 4; ++a)
        for (int k = 0; k < 3; ++k) {
          double c = p->xyz[3 * (int64_t)p->tv[4 * t + a] + k];
          if (c < blo[k]) blo[k] = c;
          if (c > bhi[k]) bhi[k] = c;
        }
      int i0[3], i1[3];
      for (int k = 0; k < 3; ++k) {
        int a = (int)floor((blo[k] - tol - p->glo[k]) / p->gh[k]);
        int b = (int)floor((bhi[k] + tol - p->glo[k]) / p->gh[k]);
        if (a < 0) a = 0;
        if (b > p->gn[k] - 1) b = p->gn[k] - 1;
        i0[k] = a; i1[k] = b;
      }
      for (int z = i0[2]; z <= i1[2]; ++z)
        for (int y = i0[1]; y <= i1[1]; ++y)
          for (int x = i0[0]; x <= i1[0]; ++x) {
            int64_t c = ((int64_t)z * p->gn[1] + y) * p->gn[0] + x;
            if (pass == 0) cnt[c]++;
            else p->gtets[cnt[c]++] = (int32_t)t;
          }
    }
  }
  free(cnt);
  return 0;
}

int oracle_set_mesh(oracle_problem* p, int64_t n_vtx, const double* xyz, int64_t n_tet,
                    const int32_t* tet_vtx, const int32_t* tet_block, const int32_t* tet_side_bid)
{
  free_mesh(p);
  if (n_vtx < 4 || n_tet < 1) return fail(p, "empty mesh");
  p->n_vtx = n_vtx;
  p->n_tet = n_tet;
  p->xyz = (double*)malloc(sizeof(double) * 3 * (size_t)n_vtx);
  memcpy(p->xyz, xyz, sizeof(double) * 3 * (size_t)n_vtx);
  p->tv = (int32_t*)malloc(sizeof(int32_t) * 4 * (size_t)n_tet);
  memcpy(p->tv, tet_vtx, sizeof(int32_t) * 4 * (size_t)n_tet);
  for (int64_t i = 0; i < 4 * n_tet; ++i)
    if (p->tv[i] < 0 || p->tv[i] >= n_vtx) return fail(p, "tet vertex index out of range");
  p->blk = (int32_t*)malloc(sizeof(int32_t) * (size_t)n_tet);
  memcpy(p->blk, tet_block, sizeof(int32_t) * (size_t)n_tet);
  p->side_bid = (int32_t*)malloc(sizeof(int32_t) * 4 * (size_t)n_tet);
  for (int64_t i = 0; i < 4 * n_tet; ++i) p->side_bid[i] = tet_side_bid ? tet_side_bid[i] : -1;
  p->nbr = (int32_t*)malloc(sizeof(int32_t) * 4 * (size_t)n_tet);
  p->planes = (double*)malloc(sizeof(double) * 16 * (size_t)n_tet);
  p->tmat = (int32_t*)malloc(sizeof(int32_t) * (size_t)n_tet);
  if (build_adjacency(p)) return 1;
  if (build_planes(p)) return 1;
  if (build_locator(p)) return 1;
  return 0;
}

int oracle_set_bc(oracle_problem* p, int32_t bid, int32_t type)
{
  if (bid < 0 || bid >= 1024) return fail(p, "boundary id out of range [0,1024)");
  if (type != 0 && type != 1) return fail(p, "bc type must be 0 (vacuum) or 1 (reflect)");
  p->bc_type[bid] = type;
  return 0;
}

int oracle_add_nuclide(oracle_problem* p, int64_t n_pts, const double* E, const double* sig_t,
                       const double* sig_s, double awr)
{
  if (n_pts < 2) return fail(p, "nuclide grid needs at least 2 points");
  for (int64_t i = 0; i + 1 < n_pts; ++i)
    if (!(E[i] < E[i + 1])) return fail(p, "nuclide energy grid must be strictly increasing");
  if (!(E[0] > 0.0)) return fail(p, "nuclide energies must be positive");
  if (!isfinite(E[n_pts - 1])) return fail(p, "nuclide energies must be finite");
  for (int64_t i = 0; i < n_pts; ++i) {
    if (!isfinite(sig_t[i]) || !isfinite(sig_s[i])) return fail(p, "cross sections must be finite");
    if (!(sig_t[i] >= 0.0) || !(sig_s[i] >= 0.0) || sig_s[i] > sig_t[i])
      return fail(p, "cross sections must satisfy 0 <= sigma_s <= sigma_t");
  }
  if (!(awr > 0.0) || !isfinite(awr)) return fail(p, "atomic weight ratio must be positive");
  if (p->n_nuc == p->cap_nuc) {
    p->cap_nuc = p->cap_nuc ? 2 * p->cap_nuc : 16;
    p->nucs = (nuclide_t*)realloc(p->nucs, sizeof(nuclide_t) * (size_t)p->cap_nuc);
  }
  nuclide_t* n = p->nucs + p->n_nuc++;
  n->n_pts = n_pts;
  n->E = (double*)malloc(sizeof(double) * (size_t)n_pts);
  n->st = (double*)malloc(sizeof(double) * (size_t)n_pts);
  n->ss = (double*)malloc(sizeof(double) * (size_t)n_pts);
  memcpy(n->E, E, sizeof(double) * (size_t)n_pts);
  memcpy(n->st, sig_t, sizeof(double) * (size_t)n_pts);
  memcpy(n->ss, sig_s, sizeof(double) * (size_t)n_pts);
  n->awr = awr;
  n->hidx = NULL;
  n->nusf = NULL;
  p->data_ready = 0;
  return 0;
}

/* Fission data of a nuclide (nu*sigma_f per grid point); NULL clears. */
int oracle_set_fission(oracle_problem* p, int32_t nuclide, const double* nu_sig_f)
{
  if (nuclide < 0 || nuclide >= p->n_nuc) return fail(p, "nuclide index out of range");
  nuclide_t* n = p->nucs + nuclide;
  free(n->nusf);
  n->nusf = NULL;
  if (nu_sig_f) {
    n->nusf = (double*)malloc(sizeof(double) * (size_t)n->n_pts);
    memcpy(n->nusf, nu_sig_f, sizeof(double) * (size_t)n->n_pts);
  }
  return 0;
}

int oracle_add_material(oracle_problem* p, int32_t material_id, int32_t n, const int32_t* nuclides,
                        const double* densities)
{
  if (n < 1) return fail(p, "material needs at least one nuclide");
  for (int i = 0; i < n; ++i)
    if (nuclides[i] < 0 || nuclides[i] >= p->n_nuc) return fail(p, "material nuclide index out of range");
  if (p->n_mat == p->cap_mat) {
    p->cap_mat = p->cap_mat ? 2 * p->cap_mat : 16;
    p->mats = (material_t*)realloc(p->mats, sizeof(material_t) * (size_t)p->cap_mat);
  }
  material_t* m = p->mats + p->n_mat++;
  m->id = material_id;
  m->n = n;
  m->nuc = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  m->dens = (double*)malloc(sizeof(double) * (size_t)n);
  memcpy(m->nuc, nuclides, sizeof(int32_t) * (size_t)n);
  memcpy(m->dens, densities, sizeof(double) * (size_t)n);
  return 0;
}

int oracle_block_map(oracle_problem* p, int32_t n, const int32_t* blocks, const int32_t* materials)
{
  free(p->map_blocks); free(p->map_mats);
  p->n_map = n;
  p->map_blocks = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  p->map_mats = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
  memcpy(p->map_blocks, blocks, sizeof(int32_t) * (size_t)n);
  memcpy(p->map_mats, materials, sizeof(int32_t) * (size_t)n);
  return 0;
}

int oracle_set_source(oracle_problem* p, const oracle_source* s)
{
  p->src = *s;
  free(p->src_cyl);
  p->src_cyl = NULL;
  if (s->space == 2) {
    if (s->n_cyl < 1) return fail(p, "cylinder source needs at least one cylinder");
    p->src_cyl = (double*)malloc(sizeof(double) * 2 * (size_t)s->n_cyl);
    memcpy(p->src_cyl, s->cyl_xy, sizeof(double) * 2 * (size_t)s->n_cyl);
  }
  p->src.cyl_xy = p->src_cyl;
  return 0;
}

int oracle_set_hash_bins(oracle_problem* p, int32_t n_bins)
{
  if (n_bins < 1) return fail(p, "hash bins must be >= 1");
  p->n_bins = n_bins;
  p->data_ready = 0;
  return 0;
}

/* Tally definition: OpenMCTally's estimator, scores and energy filter
 * (src/userobjects/OpenMCTally.C:30-101), restated for the element tally. */
int oracle_set_tally(oracle_problem* p, int32_t estimator, int32_t n_scores, const int32_t* scores,
                     int32_t n_energy_bins, const double* edges)
{
  if (estimator != 1 && estimator != 2) return fail(p, "bad estimator");
  if (n_scores < 1 || n_scores > 4) return fail(p, "1 to 4 scores");
  for (int j = 0; j < n_scores; ++j) {
    if (scores[j] < 0 || scores[j] > 3) return fail(p, "bad score");
    if (estimator == 1 && scores[j] > 1) return fail(p, "track length scores flux and total");
    p->t_sc[j] = scores[j];
  }
  p->t_est = estimator;
  p->t_ns = n_scores;
  free(p->t_edges);
  p->t_edges = NULL;
  p->t_nb = 1;
  if (n_energy_bins > 0) {
    p->t_edges = (double*)malloc(sizeof(double) * (size_t)(n_energy_bins + 1));
    memcpy(p->t_edges, edges, sizeof(double) * (size_t)(n_energy_bins + 1));
    p->t_nb = n_energy_bins;
  }
  return 0;
}

int64_t oracle_tally_size(const oracle_problem* p) { return p->n_tet * p->t_nb * p->t_ns; }

/* 2-D mode: CollisionKernel.C:60-61,200-202, OpenMCStudy.C:355-356. */
int oracle_set_2d(oracle_problem* p, int32_t on, double z_coord)
{
  p->two_d = on ? 1 : 0;
  p->z2d = on ? z_coord : 0.0;
  return 0;
}

/* ------------------------------------------------------------------ */
/* Energy-grid search: logarithmic hash bins over the common energy range
 * (F. B. Brown, "New hash-based energy lookup algorithm for Monte Carlo
 * codes", 2014; OpenMC's log grid), then bisection inside the bin.      */
static int bucket_of(const oracle_problem* p, double lE)
{
  double q = (lE - p->lE_lo) / p->du;
  if (!(q >= 0.0)) return 0;
  if (q >= (double)p->n_bins) return p->n_bins - 1;
  int k = (int)q;
  if (k > p->n_bins - 1) k = p->n_bins - 1;
  return k;
}

static int prepare_data(oracle_problem* p)
{
  if (p->data_ready) return 0;
  if (p->n_nuc < 1) return fail(p, "no nuclides");
  double lo = -INFINITY, hi = INFINITY;
  for (int i = 0; i < p->n_nuc; ++i) {
    if (p->nucs[i].E[0] > lo) lo = p->nucs[i].E[0];
    if (p->nucs[i].E[p->nucs[i].n_pts - 1] < hi) hi = p->nucs[i].E[p->nucs[i].n_pts - 1];
  }
  if (!(hi > lo)) return fail(p, "nuclide energy ranges do not overlap");
  p->E_lo = lo;
  p->E_hi = hi;
  p->lE_lo = oracle_log(lo);
  p->du = (oracle_log(hi) - p->lE_lo) / (double)p->n_bins;
  for (int i = 0; i < p->n_nuc; ++i) {
    nuclide_t* n = p->nucs + i;
    free(n->hidx);
    n->hidx = (int32_t*)malloc(sizeof(int32_t) * (size_t)(p->n_bins + 1));
    /* hidx[k] = (number of grid points in bins < k) - 1, at least 0 */
    int64_t j = 0;
    for (int k = 0; k <= p->n_bins; ++k) {
      while (j < n->n_pts && bucket_of(p, oracle_log(n->E[j])) < k) ++j;
      int64_t v = j - 1;
      if (v < 0) v = 0;
      if (v > n->n_pts - 2) v = n->n_pts - 2;
      n->hidx[k] = (int32_t)v;
    }
  }
  p->data_ready = 1;
  return 0;
}

static int grid_index(const nuclide_t* n, int k, double E)
{
  int lo = n->hidx[k];
  int hi = n->hidx[k + 1] + 1;
  int last = (int)n->n_pts - 1;
  if (hi > last) hi = last;
  while (lo > 0 && E < n->E[lo]) --lo;
  while (hi < last && E >= n->E[hi]) ++hi;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (E < n->E[mid]) hi = mid;
    else lo = mid;
  }
  return lo;
}

static void micro_xs(const nuclide_t* n, int k, double E, double* st, double* ss)
{
  int i = grid_index(n, k, E);
  double f = oracle_quotient(E - n->E[i], n->E[i + 1] - n->E[i]);
  *st = fma(f, n->st[i + 1] - n->st[i], n->st[i]);
  *ss = fma(f, n->ss[i + 1] - n->ss[i], n->ss[i]);
}

static double macro_total(const oracle_problem* p, int mat, double E)
{
  const material_t* m = p->mats + mat;
  int k = bucket_of(p, oracle_log(E));
  double acc = 0.0;
  for (int j = 0; j < m->n; ++j) {
    double st, ss;
    micro_xs(p->nucs + m->nuc[j], k, E, &st, &ss);
    acc = fma(m->dens[j], st, acc);
  }
  return acc;
}

/* nu*sigma_f of a fissionable nuclide at E, interpolated on sigma_t's
 * interval with sigma_t's fraction. */
static double micro_nusf(const nuclide_t* n, int k, double E)
{
  int i = grid_index(n, k, E);
  double f = oracle_quotient(E - n->E[i], n->E[i + 1] - n->E[i]);
  return fma(f, n->nusf[i + 1] - n->nusf[i], n->nusf[i]);
}

/* nu*Sigma_f: sum over the material's fissionable nuclides of
 * N_i nu*sigma_f,i(E), in material order (OpenMC macro_xs.nu_fission). */
static double macro_nufission(const oracle_problem* p, int mat, double E)
{
  const material_t* m = p->mats + mat;
  int k = bucket_of(p, oracle_log(E));
  double acc = 0.0;
  for (int j = 0; j < m->n; ++j) {
    const nuclide_t* n = p->nucs + m->nuc[j];
    if (n->nusf) acc = fma(m->dens[j], micro_nusf(n, k, E), acc);
  }
  return acc;
}

int oracle_xs_index(oracle_problem* p, int32_t nuclide, double E, double* f_out)
{
  if (prepare_data(p)) return -1;
  const nuclide_t* n = p->nucs + nuclide;
  int k = bucket_of(p, oracle_log(E));
  int i = grid_index(n, k, E);
  if (f_out) *f_out = oracle_quotient(E - n->E[i], n->E[i + 1] - n->E[i]);
  return i;
}

int oracle_macro_xs(oracle_problem* p, int32_t material_index, double E, double* sig_t)
{
  if (prepare_data(p)) return 1;
  *sig_t = macro_total(p, material_index, E);
  return 0;
}

int oracle_mesh_info(oracle_problem* p, const int32_t** nbr, const double** planes)
{
  *nbr = p->nbr;
  *planes = p->planes;
  return 0;
}

/* ------------------------------------------------------------------ */
/* Start-element location (stands in for MOOSE ClaimRays): among tets whose
 * four half-spaces contain x within 1e-9, take the lowest id whose interior
 * the direction enters (every side with |s| <= tol has n.u < 0); if none is
 * entered, the lowest id that contains x.                                 */
int oracle_locate(oracle_problem* p, const double* x, const double* u)
{
  int ci[3];
  for (int k = 0; k < 3; ++k) {
    double q = (x[k] - p->glo[k]) / p->gh[k];
    int c = (int)floor(q);
    if (!(q >= 0.0)) c = 0;
    if (c > p->gn[k] - 1) c = p->gn[k] - 1;
    if (c < 0) c = 0;
    ci[k] = c;
  }
  int64_t cell = ((int64_t)ci[2] * p->gn[1] + ci[1]) * p->gn[0] + ci[0];
  const double tol = 1e-9;
  int best_in = -1, best_any = -1;
  for (int64_t q = p->gstart[cell]; q < p->gstart[cell + 1]; ++q) {
    int32_t t = p->gtets[q];
    const double* P = p->planes + 16 * (int64_t)t;
    int inside = 1, enters = 1;
    for (int f = 0; f < 4; ++f) {
      const double* pl = P + 4 * f;
      double s = pl[0] * x[0] + pl[1] * x[1] + pl[2] * x[2] - pl[3];
      if (s > tol) { inside = 0; break; }
      if (s >= -tol) {
        double dn = pl[0] * u[0] + pl[1] * u[1] + pl[2] * u[2];
        if (!(dn < 0.0)) enters = 0;
      }
    }
    if (!inside) continue;
    if (enters && (best_in < 0 || t < best_in)) best_in = t;
    if (best_any < 0 || t < best_any) best_any = t;
  }
  return best_in >= 0 ? best_in : best_any;
}

/* ------------------------------------------------------------------ */
/* Sampling helpers.  No sin/cos: a uniform azimuth is drawn as a point in
 * the unit disk and its doubled angle (von Neumann 1951), and the Maxwell
 * cos^2 term from a point in the unit quarter disk.                       */
static void sample_azimuth(uint64_t* s, double* c, double* sn)
{
  for (int it = 0; it < 10000; ++it) {
    double a = 2.0 * oracle_prn(s) - 1.0;
    double b = 2.0 * oracle_prn(s) - 1.0;
    double r2 = a * a + b * b;
    if (r2 > 0.0 && r2 <= 1.0) {
      const double inv = oracle_quotient(1.0, r2);
      *c = (a * a - b * b) * inv;
      *sn = (2.0 * a * b) * inv;
      return;
    }
  }
  *c = 1.0;
  *sn = 0.0;
}

static double sample_cos2_quarter(uint64_t* s)
{
  for (int it = 0; it < 10000; ++it) {
    double a = oracle_prn(s);
    double b = oracle_prn(s);
    double r2 = a * a + b * b;
    if (r2 > 0.0 && r2 <= 1.0) return oracle_quotient(a * a, r2);
  }
  return 0.5;
}

/* Watt spectrum as Maxwellian plus shift (OpenMC watt_spectrum /
 * maxwell_spectrum formulas), redrawn outside [E_lo, E_hi). */
static double sample_watt(uint64_t* s, double a, double b, double E_lo, double E_hi)
{
  for (int it = 0; it < 1000; ++it) {
    double r1 = oracle_prn(s);
    double r2 = oracle_prn(s);
    double c2 = sample_cos2_quarter(s);
    double w = -a * (oracle_log(r1) + oracle_log(r2) * c2);
    double E = w + a * a * b / 4.0 + (2.0 * oracle_prn(s) - 1.0) * sqrt(a * a * b * w);
    if (E < E_hi && E >= E_lo) return E;
  }
  return E_hi * 0.5;
}

static double pos0(double a) { return a > 0.0 ? a : 0.0; }

/* A direction without its z component, renormalised in the plane (a
 * direction along z becomes +x), as the 2-D mode sets it. */
static void planar_dir(double* u)
{
  u[2] = 0.0;
  double n2 = u[0] * u[0] + u[1] * u[1];
  if (n2 > 0.0) {
    double n = sqrt(n2);
    u[0] = u[0] / n;
    u[1] = u[1] / n;
  } else {
    u[0] = 1.0;
    u[1] = 0.0;
  }
}

static void rotate_dir(double* u, double mu, double cphi, double sphi)
{
  double u0 = u[0], v0 = u[1], w0 = u[2];
  double a = sqrt(pos0(1.0 - mu * mu));
  double b = sqrt(pos0(1.0 - w0 * w0));
  if (b > 1e-10) {
    u[0] = mu * u0 + a * (u0 * w0 * cphi - v0 * sphi) / b;
    u[1] = mu * v0 + a * (v0 * w0 * cphi + u0 * sphi) / b;
    u[2] = mu * w0 - a * b * cphi;
  } else {
    b = sqrt(1.0 - v0 * v0);
    u[0] = mu * u0 + a * (u0 * v0 * cphi + w0 * sphi) / b;
    u[1] = mu * v0 - a * b * cphi;
    u[2] = mu * w0 + a * (v0 * w0 * cphi - u0 * sphi) / b;
  }
}

/* ------------------------------------------------------------------ */
#define ST_LEAK 1
#define ST_ABSORB 2
#define ST_CUTOFF 3
#define ST_STUCK 4
#define ST_LOST 5
#define ST_BADXS 6
/* Segments a history may walk before it is ended as stuck.  A straight
 * flight crosses of the order of cbrt(n_tet) elements, so the default
 * allows 4096 such flights: 4096 * ceil(cbrt(n_tet)), at least 65,536 and
 * at most 10,000,000 (the same rule as the GPU library's default). */
static int64_t segment_limit(const oracle_problem* p)
{
  if (p->seg_limit > 0) return p->seg_limit;
  int64_t c = 1;
  while (c * c * c < p->n_tet) ++c;
  int64_t l = 4096 * c;
  if (l < 65536) l = 65536;
  if (l > 10000000) l = 10000000;
  return l;
}
#define MAX_ZERO_RUN 10000

#define FNV_OFF 14695981039346656037ULL
#define FNV_PRIME 1099511628211ULL

static int material_of_block(const oracle_problem* p, int32_t blk)
{
  for (int i = 0; i < p->n_map; ++i)
    if (p->map_blocks[i] == blk) {
      int want = p->map_mats[i];
      for (int m = 0; m < p->n_mat; ++m)
        if (p->mats[m].id == want) return m;
      return -1;
    }
  return -1;
}

/* tmat[t] = material_of_block(blk[t]) for every element, through a table
 * per distinct block id in a dense range (the common case), else directly. */
static void resolve_materials(oracle_problem* p)
{
  int32_t lo = 0, hi = -1;
  for (int64_t t = 0; t < p->n_tet; ++t) {
    if (t == 0 || p->blk[t] < lo) lo = p->blk[t];
    if (t == 0 || p->blk[t] > hi) hi = p->blk[t];
  }
  if (p->n_tet > 0 && (int64_t)hi - lo < 1000000) {
    int32_t* tab = (int32_t*)malloc(sizeof(int32_t) * (size_t)(hi - lo + 1));
    for (int32_t b = lo; b <= hi; ++b) tab[b - lo] = material_of_block(p, b);
    for (int64_t t = 0; t < p->n_tet; ++t) p->tmat[t] = tab[p->blk[t] - lo];
    free(tab);
    return;
  }
  for (int64_t t = 0; t < p->n_tet; ++t) p->tmat[t] = material_of_block(p, p->blk[t]);
}

typedef struct {
  int64_t n_seg, n_coll, n_leak, n_absorb, n_cutoff, n_stuck, n_lost, n_badxs;
  double leak_w;
} lstats;

static void birth(const oracle_problem* p, int64_t id, uint64_t* ssrc, double* x, double* u,
                  double* E)
{
  const oracle_source* S = &p->src;
  if (S->space == 0) {
    x[0] = S->point[0]; x[1] = S->point[1]; x[2] = S->point[2];
  } else if (S->space == 1) {
    for (int k = 0; k < 3; ++k) x[k] = S->box_lo[k] + oracle_prn(ssrc) * (S->box_hi[k] - S->box_lo[k]);
  } else {
    int c = (int)(oracle_prn(ssrc) * (double)S->n_cyl);
    if (c > S->n_cyl - 1) c = S->n_cyl - 1;
    double r = S->cyl_r * sqrt(oracle_prn(ssrc));
    double ct, st;
    sample_azimuth(ssrc, &ct, &st);
    x[0] = S->cyl_xy[2 * c] + r * ct;
    x[1] = S->cyl_xy[2 * c + 1] + r * st;
    x[2] = S->cyl_z0 + oracle_prn(ssrc) * (S->cyl_z1 - S->cyl_z0);
  }
  double mu = 2.0 * oracle_prn(ssrc) - 1.0;
  double cp, sp;
  sample_azimuth(ssrc, &cp, &sp);
  double sm = sqrt(pos0(1.0 - mu * mu));
  u[0] = mu;
  u[1] = sm * cp;
  u[2] = sm * sp;
  if (S->energy == 1) *E = S->mono_E;
  else *E = sample_watt(ssrc, S->watt_a, S->watt_b, p->E_lo, p->E_hi);
  (void)id;
}

/* Energy filter bin (OpenMC EnergyFilter: edges[b] <= E < edges[b+1]),
 * -1 outside. */
static int energy_bin(const oracle_problem* p, double E)
{
  if (!p->t_edges) return 0;
  if (!(E >= p->t_edges[0]) || !(E < p->t_edges[p->t_nb])) return -1;
  int lo = 0, hi = p->t_nb;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (E < p->t_edges[mid]) hi = mid; else lo = mid;
  }
  return lo;
}

/* Track-length scores of one segment; v = wgt * scored length
 * (CollisionKernel.C:153-154). */
static void score_track(const oracle_problem* p, double* tally, int elem, double E, double v, double sigt)
{
  if (p->t_est != 1) return;
  int b = energy_bin(p, E);
  if (b < 0) return;
  double* t = tally + ((int64_t)elem * p->t_nb + b) * p->t_ns;
  for (int j = 0; j < p->t_ns; ++j) t[j] += (p->t_sc[j] == 1) ? v * sigt : v;
}

/* Collision-estimator scores at a collision, before its energy change:
 * flux wgt/Sigma_t, total wgt, scatter wgt*Sigma_s/Sigma_t, absorption
 * wgt*(Sigma_t-Sigma_s)/Sigma_t, Sigma_s summed in material order. */
static void score_collision(const oracle_problem* p, double* tally, int elem, int mat, double E, double wgt,
                            double sigt)
{
  if (p->t_est != 2) return;
  int b = energy_bin(p, E);
  if (b < 0) return;
  double ss = 0.0;
  int need = 0;
  for (int j = 0; j < p->t_ns; ++j)
    if (p->t_sc[j] >= 2) need = 1;
  if (need) {
    const material_t* m = p->mats + mat;
    int k = bucket_of(p, oracle_log(E));
    for (int j = 0; j < m->n; ++j) {
      double st, sj;
      micro_xs(p->nucs + m->nuc[j], k, E, &st, &sj);
      ss = fma(m->dens[j], sj, ss);
    }
  }
  double* t = tally + ((int64_t)elem * p->t_nb + b) * p->t_ns;
  for (int j = 0; j < p->t_ns; ++j) {
    double v;
    switch (p->t_sc[j]) {
      case 0: v = wgt / sigt; break;
      case 1: v = wgt; break;
      case 2: v = wgt * ss / sigt; break;
      default: v = wgt * (sigt - ss) / sigt; break;
    }
    t[j] += v;
  }
}

/* k-eigenvalue state of one history: estimator sums and the fission
 * sites it banks, in the order it banks them. */
typedef struct {
  int on;
  double keff, fa, fb;
  double ktl, kcol, kabs;
  oracle_fsite* sites;
  int n_sites, cap_sites;
} heig;

#define WATT_A_DEFAULT 0.988e6
#define WATT_B_DEFAULT 2.249e-6

/* Fission sites of a collision with a fissionable nuclide (OpenMC
 * create_fission_sites with sample_fission_neutron; no uniform fission
 * source weighting, no delayed-neutron data): nu_t = wgt/keff *
 * nu*sigma_f/sigma_t, fraction by one draw; per site a polar cosine, an
 * azimuth, one draw against beta = 0 and a Watt energy.  Fixed-source
 * runs (e NULL or off) draw them with keff = 1 and drop them. */
static void fission_sites(const oracle_problem* p, heig* e, int64_t id, const double* x, double wgt,
                          double nf, double st, uint64_t* s)
{
  int on = e && e->on;
  double keff = on ? e->keff : 1.0;
  double fa = on ? e->fa : WATT_A_DEFAULT, fb = on ? e->fb : WATT_B_DEFAULT;
  double nu_t = wgt / keff * nf / st;
  int nu = (int)nu_t;
  if (oracle_prn(s) <= nu_t - (double)nu) ++nu;
  for (int k = 0; k < nu; ++k) {
    double mu = 2.0 * oracle_prn(s) - 1.0;
    double cp, sp;
    sample_azimuth(s, &cp, &sp);
    double sm = sqrt(pos0(1.0 - mu * mu));
    (void)oracle_prn(s);
    double E = sample_watt(s, fa, fb, p->E_lo, p->E_hi);
    if (!on) continue;
    if (e->n_sites == e->cap_sites) {
      e->cap_sites = e->cap_sites ? 2 * e->cap_sites : 4;
      e->sites = (oracle_fsite*)realloc(e->sites, sizeof(oracle_fsite) * (size_t)e->cap_sites);
    }
    oracle_fsite* o = e->sites + e->n_sites;
    o->x = x[0]; o->y = x[1]; o->z = x[2];
    o->u = mu; o->v = sm * cp; o->w = sm * sp;
    o->E = E;
    o->wgt = 1.0;
    o->parent = id;
    o->progeny = e->n_sites;
    o->pad = 0;
    e->n_sites++;
  }
}

/* One history: id h+1, born from `site` (x, y, z, u, v, w, E, wgt) when
 * given, else sampled from the source stream. */
/* Appends the segment that just ended to a recorded ray (the same fields
 * as the GPU library's mc_ray_segment). */
static void record_seg(oracle_ray_seg* rec, int32_t* rec_n, int32_t cap, int64_t id, int n_seg, int n_coll,
                       int elem, const double* s, const double* x, double E, double wgt, uint64_t seed)
{
  const int k = n_seg - 1;
  if (!rec || k >= cap) return;
  oracle_ray_seg* o = rec + k;
  o->id = id;
  o->segment = k;
  o->intersections = n_seg - n_coll;
  o->elem = elem;
  o->pad = 0;
  for (int a = 0; a < 3; ++a) { o->start[a] = s[a]; o->end[a] = x[a]; }
  o->E = E;
  o->wgt = wgt;
  o->seed_tracking = seed;
  *rec_n = k + 1;
}

static void track(const oracle_problem* p, int64_t h, uint64_t master, const double* site, heig* e,
                  double* tally, oracle_trace* tr, lstats* ls, oracle_ray_seg* rec, int32_t* rec_n)
{
  int64_t id = h + 1;
  uint64_t ssrc = oracle_init_seed(id, master, 2);
  uint64_t strk = oracle_init_seed(id, master, 0);
  double x[3], u[3], E, wgt = 1.0;
  if (site) {
    x[0] = site[0]; x[1] = site[1]; x[2] = site[2];
    u[0] = site[3]; u[1] = site[4]; u[2] = site[5];
    E = site[6];
    wgt = site[7];
  } else {
    birth(p, id, &ssrc, x, u, &E);
  }
  if (p->two_d) {
    x[2] = p->z2d;
    planar_dir(u);
  }
  const int eig = e && e->on;
  double nuf = 0.0;
  uint64_t hash = FNV_OFF;
  int status = 0, n_seg = 0, n_coll = 0, face_out = -1;
  int elem = oracle_locate(p, x, u);
  int cur_mat = -2;
  double sigt = 0.0;
  int zero_run = 0;
  const int64_t max_seg = segment_limit(p);
  const int32_t rec_cap = p->ray_cap;
  double s0[3];
  if (elem < 0) status = ST_LOST;
  while (status == 0) {
    if (n_seg >= max_seg || zero_run >= MAX_ZERO_RUN) { status = ST_STUCK; break; }
    int mat = p->tmat[elem];
    if (mat < 0) { status = ST_BADXS; break; }
    if (mat != cur_mat) {
      sigt = macro_total(p, mat, E);
      if (eig) nuf = macro_nufission(p, mat, E);
      cur_mat = mat;
      if (!(sigt > 0.0) || sigt != sigt) { status = ST_BADXS; break; }
    }
    /* exit side: smallest (d - n.x)/(n.u) over sides with n.u > 0, compared
       by cross-multiplication, ties to the lower side index.  The dot
       products and the position updates are chains of fused multiply-adds
       (C99 fma, one rounding each): the same operations the GPU's DFMA
       performs, in the same order, so both give the same bits. */
    const double* P = p->planes + 16 * (int64_t)elem;
    int bf = -1;
    double bnum = 0.0, bden = 1.0;
    for (int f = 0; f < 4; ++f) {
      const double* pl = P + 4 * f;
      double den = fma(pl[0], u[0], fma(pl[1], u[1], pl[2] * u[2]));
      if (den > 0.0) {
        double num = fma(-pl[0], x[0], fma(-pl[1], x[1], fma(-pl[2], x[2], pl[3])));
        if (bf < 0 || num * bden < bnum * den) { bf = f; bnum = num; bden = den; }
      }
    }
    if (bf < 0) { status = ST_STUCK; break; }
    double L = oracle_quotient(bnum, bden);
    if (!(L > 0.0)) L = 0.0;
    double dist = oracle_quotient(-oracle_log(oracle_prn(&strk)), sigt);
    double score = (L < dist) ? L : dist;
    score_track(p, tally, elem, E, wgt * score, sigt);
    if (eig) e->ktl = e->ktl + wgt * score * nuf; /* CollisionKernel.C:153-154 */
    ++n_seg;
    if (L == 0.0) ++zero_run; else zero_run = 0;
    s0[0] = x[0]; s0[1] = x[1]; s0[2] = x[2];
    if (dist > L) {
      hash = (hash ^ ((uint64_t)elem * 8ULL + (uint64_t)bf)) * FNV_PRIME;
      x[0] = fma(L, u[0], x[0]);
      x[1] = fma(L, u[1], x[1]);
      x[2] = fma(L, u[2], x[2]);
      record_seg(rec, rec_n, rec_cap, id, n_seg, n_coll, elem, s0, x, E, wgt, strk);
      int32_t nb = p->nbr[4 * (int64_t)elem + bf];
      if (nb >= 0) { elem = nb; continue; }
      int32_t bid = p->side_bid[4 * (int64_t)elem + bf];
      if (bid < 0) bid = 0;
      if (bid < 1024 && p->bc_type[bid] == 1) {
        const double* pl = P + 4 * bf;
        double dn = fma(u[0], pl[0], fma(u[1], pl[1], u[2] * pl[2]));
        double t2 = 2.0 * dn;
        u[0] = fma(-t2, pl[0], u[0]);
        u[1] = fma(-t2, pl[1], u[1]);
        u[2] = fma(-t2, pl[2], u[2]);
        continue;
      }
      status = ST_LEAK;
      face_out = bf;
      ls->leak_w += wgt;
      break;
    }
    /* collision inside this element */
    hash = (hash ^ ((uint64_t)elem * 8ULL + 4ULL)) * FNV_PRIME;
    double ex = fma(L, u[0], x[0]), ey = fma(L, u[1], x[1]), ez = fma(L, u[2], x[2]);
    double back = L - dist;
    x[0] = fma(-back, u[0], ex);
    x[1] = fma(-back, u[1], ey);
    x[2] = fma(-back, u[2], ez);
    ++n_coll;
    record_seg(rec, rec_n, rec_cap, id, n_seg, n_coll, elem, s0, x, E, wgt, strk);
    zero_run = 0;
    score_collision(p, tally, elem, mat, E, wgt, sigt);
    /* collision estimate of keff (OpenMC event_collide) */
    if (eig && nuf > 0.0) e->kcol = e->kcol + wgt * nuf / sigt;
    const material_t* m = p->mats + mat;
    int k = bucket_of(p, oracle_log(E));
    double cutoff = oracle_prn(&strk) * sigt;
    double acc = 0.0, st = 0.0, ss = 0.0;
    int pick = -1;
    for (int j = 0; j < m->n; ++j) {
      micro_xs(p->nucs + m->nuc[j], k, E, &st, &ss);
      acc = fma(m->dens[j], st, acc);
      if (acc >= cutoff) { pick = j; break; }
    }
    if (pick < 0) pick = m->n - 1; /* st/ss already hold the last nuclide */
    const nuclide_t* pn = p->nucs + m->nuc[pick];
    double nf = 0.0;
    if (pn->nusf) {
      nf = micro_nusf(pn, k, E);
      fission_sites(p, e, id, x, wgt, nf, st, &strk);
    }
    double sa = st - ss;
    if (oracle_prn(&strk) * st < sa) {
      /* absorption estimate of keff (OpenMC absorption) */
      if (eig && nf > 0.0) e->kabs = e->kabs + wgt * nf / sa;
      status = ST_ABSORB;
      break;
    }
    double A = pn->awr;
    double mu_cm = 2.0 * oracle_prn(&strk) - 1.0;
    double q = A * A + 2.0 * A * mu_cm + 1.0;
    double Ap1 = A + 1.0;
    double E2 = E * q / (Ap1 * Ap1);
    double cp, sp;
    sample_azimuth(&strk, &cp, &sp);
    if (!(q > 0.0) || !(E2 >= p->E_lo)) { E = E2; status = ST_CUTOFF; break; }
    double mu_lab = (1.0 + A * mu_cm) / sqrt(q);
    if (mu_lab > 1.0) mu_lab = 1.0;
    if (mu_lab < -1.0) mu_lab = -1.0;
    rotate_dir(u, mu_lab, cp, sp);
    if (p->two_d) planar_dir(u);
    E = E2;
    cur_mat = -2; /* energy changed: cross sections are recomputed */
  }
  hash = (hash ^ (uint64_t)(16 + status)) * FNV_PRIME;
  ls->n_seg += n_seg;
  ls->n_coll += n_coll;
  switch (status) {
    case ST_LEAK: ls->n_leak++; break;
    case ST_ABSORB: ls->n_absorb++; break;
    case ST_CUTOFF: ls->n_cutoff++; break;
    case ST_STUCK: ls->n_stuck++; break;
    case ST_LOST: ls->n_lost++; break;
    default: ls->n_badxs++; break;
  }
  if (tr) {
    tr->id = id;
    tr->hash = hash;
    tr->status = status;
    tr->n_seg = n_seg;
    tr->n_coll = n_coll;
    tr->elem = elem;
    tr->face = face_out;
    tr->pad = 0;
    tr->E = E;
    tr->x = x[0];
    tr->y = x[1];
    tr->z = x[2];
  }
}

/* Recorded ray of history i of a run (NULL when i is not recorded). */
static oracle_ray_seg* ray_slot(const oracle_problem* p, int64_t i, int32_t** cnt)
{
  if (!p->rays || i >= p->ray_n) { *cnt = NULL; return NULL; }
  *cnt = p->ray_cnt + i;
  return p->rays + i * (int64_t)p->ray_cap;
}

/* Histories [first, first+n): born from sites (n x 8 doubles) when given,
 * else sampled from the source. */
static int run_histories(oracle_problem* p, int64_t first, int64_t n, uint64_t seed, const double* sites,
                         int n_threads, double* tally, oracle_trace* traces, oracle_stats* stats)
{
  if (!p->planes) return fail(p, "no mesh");
  if (prepare_data(p)) return 1;
  if (p->n_mat < 1) return fail(p, "no materials");
  resolve_materials(p);
  if (p->rays) memset(p->ray_cnt, 0, sizeof(int32_t) * (size_t)p->ray_n);
  if (n_threads < 1) n_threads = 1;
  lstats tot;
  memset(&tot, 0, sizeof tot);
  int nt = n_threads;
#ifndef _OPENMP
  nt = 1;
#endif
  if (nt == 1) {
    for (int64_t i = 0; i < n; ++i) {
      int32_t* rc;
      oracle_ray_seg* rec = ray_slot(p, i, &rc);
      track(p, first + i, seed, sites ? sites + 8 * i : NULL, NULL, tally, traces ? traces + i : NULL, &tot,
            rec, rc);
    }
  } else {
#ifdef _OPENMP
    double** priv = (double**)calloc((size_t)nt, sizeof(double*));
    lstats* pl = (lstats*)calloc((size_t)nt, sizeof(lstats));
#pragma omp parallel num_threads(nt)
    {
      int tid = omp_get_thread_num();
      priv[tid] = (double*)calloc((size_t)oracle_tally_size(p), sizeof(double));
#pragma omp for schedule(dynamic, 64)
      for (int64_t i = 0; i < n; ++i) {
        int32_t* rc;
        oracle_ray_seg* rec = ray_slot(p, i, &rc);
        track(p, first + i, seed, sites ? sites + 8 * i : NULL, NULL, priv[tid], traces ? traces + i : NULL,
              pl + tid, rec, rc);
      }
    }
    for (int t = 0; t < nt; ++t) {
      if (priv[t]) {
        for (int64_t e = 0; e < oracle_tally_size(p); ++e) tally[e] += priv[t][e];
        free(priv[t]);
      }
      tot.n_seg += pl[t].n_seg; tot.n_coll += pl[t].n_coll; tot.n_leak += pl[t].n_leak;
      tot.n_absorb += pl[t].n_absorb; tot.n_cutoff += pl[t].n_cutoff; tot.n_stuck += pl[t].n_stuck;
      tot.n_lost += pl[t].n_lost; tot.n_badxs += pl[t].n_badxs; tot.leak_w += pl[t].leak_w;
    }
    free(priv);
    free(pl);
#endif
  }
  if (stats) {
    stats->n_hist = n;
    stats->n_seg = tot.n_seg;
    stats->n_coll = tot.n_coll;
    stats->n_leak = tot.n_leak;
    stats->n_absorb = tot.n_absorb;
    stats->n_cutoff = tot.n_cutoff;
    stats->n_stuck = tot.n_stuck;
    stats->n_lost = tot.n_lost;
    stats->n_badxs = tot.n_badxs;
    stats->leak_weight = tot.leak_w;
  }
  return 0;
}

int oracle_run(oracle_problem* p, int64_t first, int64_t n, uint64_t seed, int n_threads,
               double* tally, oracle_trace* traces, oracle_stats* stats)
{
  return run_histories(p, first, n, seed, NULL, n_threads, tally, traces, stats);
}

int oracle_run_sites(oracle_problem* p, int64_t first, int64_t n, uint64_t seed, const double* sites,
                     int n_threads, double* tally, oracle_trace* traces, oracle_stats* stats)
{
  if (!sites) return fail(p, "no sites");
  return run_histories(p, first, n, seed, sites, n_threads, tally, traces, stats);
}

int oracle_set_segment_limit(oracle_problem* p, int64_t max_segments)
{
  if (max_segments < 0 || max_segments > 2000000000LL) return fail(p, "segment limit out of range");
  p->seg_limit = max_segments;
  return 0;
}

int64_t oracle_segment_limit(const oracle_problem* p) { return segment_limit(p); }

int oracle_rays_enable(oracle_problem* p, int32_t n_rays, int32_t max_segments)
{
  if (n_rays < 0 || max_segments < 0 || (int64_t)n_rays * max_segments > 100000000LL)
    return fail(p, "ray recording size out of range");
  free(p->rays);
  free(p->ray_cnt);
  p->rays = NULL;
  p->ray_cnt = NULL;
  p->ray_n = 0;
  p->ray_cap = 0;
  if (n_rays == 0 || max_segments == 0) return 0;
  p->rays = (oracle_ray_seg*)calloc((size_t)n_rays * (size_t)max_segments, sizeof(oracle_ray_seg));
  p->ray_cnt = (int32_t*)calloc((size_t)n_rays, sizeof(int32_t));
  if (!p->rays || !p->ray_cnt) return fail(p, "out of memory");
  p->ray_n = n_rays;
  p->ray_cap = max_segments;
  return 0;
}

int oracle_rays(oracle_problem* p, oracle_ray_seg* out, int64_t capacity, int64_t* n_out)
{
  int64_t m = 0;
  for (int32_t r = 0; r < p->ray_n; ++r) {
    for (int32_t k = 0; k < p->ray_cnt[r]; ++k, ++m)
      if (out && m < capacity) out[m] = p->rays[(int64_t)r * p->ray_cap + k];
  }
  *n_out = m;
  return (out && m > capacity) ? fail(p, "capacity too small") : 0;
}

/* ------------------------------------------------------------------ */
/* k-eigenvalue generations (OpenMC's eigenvalue mode as OpenMCStudy runs
 * it, one generation per batch: births from the source bank,
 * src/userobjects/OpenMCStudy.C:317-360; finalize_generation with one
 * rank, :374-402; bank resampling as synchronizeBanks adapts OpenMC's
 * synchronize_bank, :430-607). */

/* Fixed-order sum: tiles of 1024 values (zero-padded), each reduced by the
 * pairwise tree t[i] += t[i+s] for s = 512, 256, ..., 1, then the tile sums
 * added in order. */
static double fixed_sum(const double* v, int64_t n)
{
  double total = 0.0;
  double t[1024];
  for (int64_t b = 0; b < n; b += 1024) {
    for (int i = 0; i < 1024; ++i) t[i] = (b + i < n) ? v[b + i] : 0.0;
    for (int s = 512; s > 0; s >>= 1)
      for (int i = 0; i < s; ++i) t[i] = t[i] + t[i + s];
    total = total + t[0];
  }
  return total;
}

static void site_from(const oracle_fsite* f, double* o)
{
  o[0] = f->x; o[1] = f->y; o[2] = f->z;
  o[3] = f->u; o[4] = f->v; o[5] = f->w;
  o[6] = f->E; o[7] = f->wgt;
}

int oracle_eigen_run(oracle_problem* p, int64_t n, int32_t n_gen, int32_t n_inactive, uint64_t seed,
                     double keff0, double fa, double fb, int64_t cap, int n_threads, const double* init_src,
                     oracle_gen* out, double* src_out, oracle_fsite* bank_out, int64_t bank_cap,
                     int64_t* bank_n, double* tally_sum)
{
  if (!p->planes) return fail(p, "no mesh");
  if (prepare_data(p)) return 1;
  if (p->n_mat < 1) return fail(p, "no materials");
  if (n < 1 || n_gen < 1 || n_inactive < 0 || n_inactive >= n_gen) return fail(p, "bad generation counts");
  int any = 0;
  for (int i = 0; i < p->n_nuc; ++i)
    if (p->nucs[i].nusf) any = 1;
  if (!any) return fail(p, "no fissionable nuclide");
  resolve_materials(p);
  if (keff0 <= 0.0) keff0 = 1.0;
  if (fa <= 0.0) fa = WATT_A_DEFAULT;
  if (fb <= 0.0) fb = WATT_B_DEFAULT;
  if (cap <= 0) cap = 3 * n;
  int nt = n_threads < 1 ? 1 : n_threads;
#ifndef _OPENMP
  nt = 1;
#endif
  const int64_t ntal = oracle_tally_size(p);
  double* src = (double*)malloc(sizeof(double) * 8 * (size_t)n);
  double* nsrc = (double*)malloc(sizeof(double) * 8 * (size_t)n);
  double* ktl = (double*)malloc(sizeof(double) * (size_t)n);
  double* kcol = (double*)malloc(sizeof(double) * (size_t)n);
  double* kabs = (double*)malloc(sizeof(double) * (size_t)n);
  heig* he = (heig*)calloc((size_t)n, sizeof(heig));
  double** priv = (double**)calloc((size_t)nt, sizeof(double*));
  lstats* pl = (lstats*)calloc((size_t)nt, sizeof(lstats));
  oracle_fsite* sorted = NULL;
  int64_t m = 0;
  int rc = 0;
  for (int t = 0; t < nt; ++t) priv[t] = (double*)calloc((size_t)ntal, sizeof(double));
  if (init_src) {
    memcpy(src, init_src, sizeof(double) * 8 * (size_t)n);
  } else {
    /* OpenMC initialize_source: site i from the source stream of id i+1 */
    for (int64_t i = 0; i < n; ++i) {
      uint64_t ss = oracle_init_seed(i + 1, seed, 2);
      double* o = src + 8 * i;
      birth(p, i + 1, &ss, o, o + 3, o + 6);
      o[7] = 1.0;
    }
  }
  double keff = keff0, k_sum0 = 0.0, k_sum1 = 0.0, keff_std = 0.0;
  int n_active = 0;
  for (int g = 0; g < n_gen && rc == 0; ++g) {
    const int active = g >= n_inactive;
    for (int t = 0; t < nt; ++t) memset(pl + t, 0, sizeof(lstats));
    for (int64_t i = 0; i < n; ++i) {
      free(he[i].sites);
      memset(he + i, 0, sizeof(heig));
      he[i].on = 1;
      he[i].keff = keff;
      he[i].fa = fa;
      he[i].fb = fb;
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
#endif
    for (int64_t i = 0; i < n; ++i) {
      int tid = 0;
#ifdef _OPENMP
      tid = omp_get_thread_num();
#endif
      track(p, (int64_t)g * n + i, seed, src + 8 * i, he + i, priv[tid], NULL, pl + tid, NULL, NULL);
    }
    lstats tot;
    memset(&tot, 0, sizeof tot);
    for (int t = 0; t < nt; ++t) {
      tot.n_seg += pl[t].n_seg;
      tot.n_coll += pl[t].n_coll;
      tot.leak_w += pl[t].leak_w;
    }
    /* the batch tally: active generations fold it (SUM += batch/n) */
    if (active && tally_sum) {
      for (int u = 1; u < nt; ++u)
        for (int64_t e = 0; e < ntal; ++e) priv[0][e] += priv[u][e];
      for (int64_t e = 0; e < ntal; ++e) tally_sum[e] += priv[0][e] * (1.0 / (double)n);
    }
    for (int t = 0; t < nt; ++t) memset(priv[t], 0, sizeof(double) * (size_t)ntal);
    /* the bank in (parent, progeny) order: histories in order, each
       history's sites in the order it banked them (sort_fission_bank) */
    m = 0;
    for (int64_t i = 0; i < n; ++i) {
      ktl[i] = he[i].ktl;
      kcol[i] = he[i].kcol;
      kabs[i] = he[i].kabs;
      m += he[i].n_sites;
    }
    if (m > cap) { rc = fail(p, "fission bank full"); break; }
    if (m == 0) { rc = fail(p, "no fission sites sampled"); break; }
    free(sorted);
    sorted = (oracle_fsite*)malloc(sizeof(oracle_fsite) * (size_t)m);
    int64_t k = 0;
    for (int64_t i = 0; i < n; ++i) {
      memcpy(sorted + k, he[i].sites, sizeof(oracle_fsite) * (size_t)he[i].n_sites);
      k += he[i].n_sites;
    }
    /* synchronize_bank, one rank: sequential draws from the generation's
       tracking-stream seed */
    uint64_t s = oracle_init_seed(g + 1, seed, 0);
    const int64_t needed = m < n ? n % m : n;
    const double p_sample = (double)needed / (double)m;
    int64_t idx = 0;
    for (int64_t i = 0; i < m; ++i) {
      if (m < n)
        for (int64_t j = 1; j <= n / m; ++j) {
          if (idx < n) site_from(sorted + i, nsrc + 8 * idx);
          ++idx;
        }
      if (oracle_prn(&s) < p_sample) {
        if (idx < n) site_from(sorted + i, nsrc + 8 * idx);
        ++idx;
      }
    }
    if (idx < n) {
      const int64_t need = n - idx;
      for (int64_t j = 0; j < need; ++j) {
        int64_t b = m - need + j;
        if (b < 0) b = 0;
        site_from(sorted + b, nsrc + 8 * (idx + j));
      }
    }
    double* sw = src;
    src = nsrc;
    nsrc = sw;
    /* calculate_generation_keff / calculate_average_keff */
    const double s_tl = fixed_sum(ktl, n), s_col = fixed_sum(kcol, n), s_abs = fixed_sum(kabs, n);
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
    if (out) {
      oracle_gen* o = out + g;
      o->k_generation = k_gen;
      o->k_collision = s_col / (double)n;
      o->k_absorption = s_abs / (double)n;
      o->keff = keff;
      o->keff_std = keff_std;
      o->leakage = tot.leak_w / (double)n;
      o->n_sites = m;
      o->n_seg = tot.n_seg;
      o->n_coll = tot.n_coll;
    }
  }
  if (rc == 0) {
    if (src_out) memcpy(src_out, src, sizeof(double) * 8 * (size_t)n);
    if (bank_n) *bank_n = m;
    if (bank_out && sorted) memcpy(bank_out, sorted, sizeof(oracle_fsite) * (size_t)(m < bank_cap ? m : bank_cap));
  }
  for (int64_t i = 0; i < n; ++i) free(he[i].sites);
  for (int t = 0; t < nt; ++t) free(priv[t]);
  free(priv); free(pl); free(he); free(ktl); free(kcol); free(kabs); free(src); free(nsrc); free(sorted);
  return rc;
}
