// mc_device.cuh -- device data views and the per-particle tracking steps.
//
// The steps restate, for a tet mesh and tabulated cross sections, what
// MaCaw does per ray segment in CollisionKernel::onSegment
// (src/raykernels/CollisionKernel.C:98-275) inside MOOSE's element walk:
//   xs      macroscopic total XS at (E, material)        CollisionKernel.C:143
//   sample  d = -ln(xi)/Sigma_t, one draw per segment      CollisionKernel.C:150
//   score   wgt*min(d, L) into the element flux tally      CollisionKernel.C:153-154
//   cross   d > L: move to the exit face, neighbour or BC  CollisionKernel.C:163-169
//   collide end-(L-d)*u, nuclide, absorb/scatter           CollisionKernel.C:173-230
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/macaw_gb300.h"
#include "mc_core.cuh"

namespace mc {

// Per-tet record of the float walk: the four outward face planes rounded to
// float and the neighbour entries, 80 bytes (three 32-byte sectors).  An
// interior entry is neighbour << 2 | the shared side's index in the
// neighbour, with kMatChange set when the neighbour's material differs; a
// boundary entry is -1-boundary_id.
struct __align__(16) Tet32 {
  float4 p[4];
  int4 nbr;
};
constexpr int kMatChange = 1 << 30;

// The mixed-precision walk's record, 64 bytes (two 32-byte sectors): each
// side's outward normal in octahedral form (two floats), the four plane
// offsets, the neighbour entries as in Tet32.  The normal is not unit: the
// walk uses oct_normal's vector as it is, and the stored offset is the
// unit plane's offset times that vector's length (computed on the host
// from the same float operations), so exit distances (d - n.x)/(n.u) are
// those of the unit plane with one float rounding per stored value.
struct __align__(64) TetOct {
  float4 oct01;  // sides 0 and 1: (a0, b0, a1, b1)
  float4 oct23;  // sides 2 and 3
  float4 d;      // plane offsets, scaled
  int4 nbr;
};

// Normal from octahedral coordinates (a, b): (a, b, 1-|a|-|b|) with the
// lower half folded back.  MC_HD: the host builds the scaled offsets from
// exactly these operations.
MC_HD void oct_normal(float a, float b, float& x, float& y, float& z) {
  z = (1.0f - fabsf(a)) - fabsf(b);
  const float t = z < 0.0f ? -z : 0.0f;
  x = a >= 0.0f ? a - t : a + t;
  y = b >= 0.0f ? b - t : b + t;
}

__device__ __forceinline__ float4 oct_plane(float a, float b, float d) {
  float x, y, z;
  oct_normal(a, b, x, y, z);
  return make_float4(x, y, z, d);
}

__device__ __forceinline__ int side_entry(const int4& n, int f) {
  return f == 0 ? n.x : f == 1 ? n.y : f == 2 ? n.z : n.w;
}

struct DevMesh {
  const double4_32a* __restrict__ planes;   // 4 per tet (nx, ny, nz, d), outward
  const Tet32* __restrict__ tet;        // float planes + neighbour entries
  const TetOct* __restrict__ teto;      // the same, normals in octahedral form (mixed walk)
  const int* __restrict__ tmat;         // material index per tet (-1: none)
  const int* __restrict__ bc_type;      // per boundary id: 0 vacuum, 1 reflect
  int n_bid;
  int max_seg;                          // segments a history may walk before it ends as stuck
  float oct_err;                        // bound on an octahedral record's unit-normal error (L1)
  int64_t n_tet;
  double glo[3], gh[3], ginv[3];  // locator origin, cell size, 1 / cell size
  int gn[3];
  const int64_t* __restrict__ gstart;
  const int* __restrict__ gtets;
  const int* __restrict__ gseed;  // per cell: a tet containing its centre, or -1
};

struct DevXS {
  const double* __restrict__ gE;        // energies of the distinct grids
  const int64_t* __restrict__ g_off;
  const int* __restrict__ g_n;
  const int* __restrict__ ghidx;        // (n_bins+1) x n_grid, bin-major
  const int* __restrict__ nuc_grid;
  const int64_t* __restrict__ nuc_off;  // into sig
  const double2* __restrict__ sig;      // (sigma_t, sigma_s) per point
  const double* __restrict__ awr;
  const int* __restrict__ mat_off;
  const int* __restrict__ mat_nuc;
  const double* __restrict__ mat_dens;
  // fission data (mc_nuclide_set_fission): nu*sigma_f per point, indexed
  // like sig; null when no nuclide is fissionable
  const double* __restrict__ nusf;
  const int* __restrict__ nuc_fiss;  // per nuclide: 1 fissionable
  const int* __restrict__ mat_fiss;  // per material: 1 holds a fissionable nuclide
  int n_nuc, n_grid, n_bins;
  double E_lo, E_hi, lE_lo, du;
};

// k-eigenvalue state of one generation (mc_eigen_run).  A fissionable
// nuclide always samples its fission sites at a collision (OpenMC
// create_fission_sites, called from sample_neutron_reaction for eigenvalue
// runs and for fixed-source runs that create fission neutrons); only with
// on = 1 are they banked and the keff estimators scored.  Per-history
// arrays are indexed by history id - 1 - first.
struct EigArgs {
  int on;
  double keff;            // the estimate site counts are divided by
  double fa, fb;          // Watt fission spectrum (eV, 1/eV)
  int64_t first;          // index of the generation's first history
  mc_fission_site* bank;  // sites of this generation in append order
  unsigned long long* n_bank;  // sites sampled (beyond cap: not stored)
  int64_t cap;
  double* ktl;            // track-length estimator, wgt*min(d,L)*nu*Sigma_f per segment
  double* kcol;           // collision estimator, wgt*nu*Sigma_f/Sigma_t per collision
  double* kabs;           // absorption estimator, wgt*nu*sigma_f/sigma_a per absorption
  int* prog;              // sites banked by the history
};

struct DevSource {
  int space, energy;
  double point[3], box_lo[3], box_hi[3];
  int n_cyl;
  const double* __restrict__ cyl_xy;
  double cyl_r, cyl_z0, cyl_z1;
  double watt_a, watt_b, mono_E;
};

struct Particle {
  double x, y, z, u, v, w, E, wgt, sigt;
  uint64_t seed, hash;
  int64_t id;
  int elem, mat, n_seg, n_coll, status, face, zero_run;
  int fin;  // side the particle entered its element through (-1: none)
  int tag;  // tally slot of the particle's batch or request
  // Sigma_t at the current energy for up to four materials, most recently
  // inserted first (an insert shifts the others down one slot and drops the
  // last); -1 marks an empty slot.  Sigma_t is a pure function of
  // (material, E), so a cached value is bit-identical to a fresh
  // evaluation whatever the slot order; every energy change empties the
  // cache.
  int4 cm;
  double cs0, cs1, cs2, cs3;
  // k-eigenvalue runs only: nu*Sigma_f of the current material at E (and
  // of the cached materials, same slots as cs), the history's track-length
  // keff sum and its count of banked fission sites
  double nuf, ktl;
  double cn0, cn1, cn2, cn3;
  int n_prog;
};

// Tally definition of a run (mc_tally_configure).  general = 0 is the
// default: the track-length flux, one value per element.
struct TallySpec {
  int general;
  int est;     // MC_EST_*
  int nb, ns;  // energy bins (>= 1) and scores per element
  int sc;      // score j (MC_SCORE_*) in bits 8j..8j+7
  int need_ss; // a score needs the macroscopic scattering cross section
  const double* __restrict__ edges;  // nb+1 ascending energy edges, or null: no energy filter
  // segment recording (mc_rays_enable): histories first .. first+ray_n-1 of
  // the run, ray_cap segments each, or rays null
  mc_ray_segment* rays;
  int64_t ray_first;
  int ray_n, ray_cap;
};

// Records the segment that just ended, from (sx, sy, sz) to (ex, ey, ez),
// when the particle's history is one of the recorded rays.  The FP64 walk
// functions take kRays = false where a launch records no rays, so that the
// walk without recording carries none of its registers.
static __device__ __noinline__ void record_ray(const TallySpec& T, const Particle& p, double sx, double sy, double sz,
                                        double ex, double ey, double ez) {
  const int64_t r = p.id - 1 - T.ray_first;
  const int k = p.n_seg - 1;
  if (r < 0 || r >= T.ray_n || k >= T.ray_cap) return;
  mc_ray_segment& o = T.rays[r * T.ray_cap + k];
  o.id = p.id;
  o.segment = k;
  o.intersections = p.n_seg - p.n_coll;
  o.elem = p.elem;
  o.pad = 0;
  o.start[0] = sx;
  o.start[1] = sy;
  o.start[2] = sz;
  o.end[0] = ex;
  o.end[1] = ey;
  o.end[2] = ez;
  o.E = p.E;
  o.wgt = p.wgt;
  o.seed_tracking = p.seed;
}

// Energy filter bin of E (OpenMC EnergyFilter: edges[b] <= E < edges[b+1]),
// -1 outside the edges.
__device__ __forceinline__ int energy_bin(const TallySpec& T, double E) {
  if (!T.edges) return 0;
  if (!(E >= __ldg(T.edges)) || !(E < __ldg(T.edges + T.nb))) return -1;
  int lo = 0, hi = T.nb;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (E < __ldg(T.edges + mid)) hi = mid;
    else lo = mid;
  }
  return lo;
}

// Track-length scores of one segment, v = wgt * scored length
// (CollisionKernel.C:153-154 scores this length).
__device__ __forceinline__ void score_track(const TallySpec& T, double* tally, int elem, double E, double v,
                                            double sigt) {
  if (!T.general) {
    atomicAdd(tally + elem, v);
    return;
  }
  if (T.est != MC_EST_TRACKLENGTH) return;
  const int b = energy_bin(T, E);
  if (b < 0) return;
  double* t = tally + ((int64_t)elem * T.nb + b) * T.ns;
  for (int j = 0; j < T.ns; ++j) atomicAdd(t + j, ((T.sc >> (8 * j)) & 0xff) == MC_SCORE_TOTAL ? v * sigt : v);
}

__device__ __forceinline__ void xs_cache_clear(Particle& p) { p.cm = make_int4(-1, -1, -1, -1); }

// Slot of material mat in a cache key set, or -1.
__device__ __forceinline__ int xs_cache_slot(const int4& cm, int mat) {
  return cm.x == mat ? 0 : cm.y == mat ? 1 : cm.z == mat ? 2 : cm.w == mat ? 3 : -1;
}

// kEig: the nu*Sigma_f values move with the Sigma_t values.
template <bool kEig = false>
__device__ __forceinline__ bool xs_cache_get(Particle& p, int mat) {
  switch (xs_cache_slot(p.cm, mat)) {
    case 0: p.sigt = p.cs0; if (kEig) p.nuf = p.cn0; return true;
    case 1: p.sigt = p.cs1; if (kEig) p.nuf = p.cn1; return true;
    case 2: p.sigt = p.cs2; if (kEig) p.nuf = p.cn2; return true;
    case 3: p.sigt = p.cs3; if (kEig) p.nuf = p.cn3; return true;
    default: return false;
  }
}

// Insert on a miss (mat is not cached).
template <bool kEig = false>
__device__ __forceinline__ void xs_cache_put(Particle& p, int mat, double s, double nf = 0.0) {
  p.cm = make_int4(mat, p.cm.x, p.cm.y, p.cm.z);
  p.cs3 = p.cs2;
  p.cs2 = p.cs1;
  p.cs1 = p.cs0;
  p.cs0 = s;
  if (kEig) {
    p.cn3 = p.cn2;
    p.cn2 = p.cn1;
    p.cn1 = p.cn0;
    p.cn0 = nf;
  }
}

// ---------------------------------------------------------------------------
// Cross sections.

// The hash bin from a float log.  grid_index's guards move from any bin to
// the right interval, so every lookup (FP64 ones too) starts from this bin:
// a bin that rounding moved by one costs one more guard step, not a
// different result, and the FP64 log stays off the narrow FP64 pipe.
__device__ __forceinline__ int xs_bucket32(const DevXS& X, double E) {
  const float q = (__logf(narrow(E)) - narrow(X.lE_lo)) / narrow(X.du);
  if (!(q >= 0.0f)) return 0;
  const int k = (int)q;
  return k > X.n_bins - 1 ? X.n_bins - 1 : k;
}

// Bisection inside the hash bin of grid g, guarded so a bin estimate that is
// off by rounding still ends on the right interval; returns the interval
// index i (E_i <= E < E_i+1) and the interpolation fraction.
// Energies and grid points are positive finite doubles, whose order is the
// order of their bit patterns as integers: the comparisons run on the
// integer pipe (exactly the same outcomes as double comparisons).
__device__ __forceinline__ int grid_index(const DevXS& X, int g, int k, double E) {
  const long long* G = reinterpret_cast<const long long*>(X.gE + __ldg(X.g_off + g));
  const long long e = __double_as_longlong(E);
  int lo = __ldg(X.ghidx + (size_t)k * X.n_grid + g);
  int hi = __ldg(X.ghidx + (size_t)(k + 1) * X.n_grid + g) + 1;
  const int last = __ldg(X.g_n + g) - 1;
  if (hi > last) hi = last;
  while (lo > 0 && e < __ldg(G + lo)) --lo;
  while (hi < last && e >= __ldg(G + hi)) ++hi;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (e < __ldg(G + mid)) hi = mid;
    else lo = mid;
  }
  return lo;
}

__device__ __forceinline__ void grid_locate(const DevXS& X, int g, int k, double E, int& i, double& f) {
  const double* G = X.gE + __ldg(X.g_off + g);
  i = grid_index(X, g, k, E);
  const double e0 = __ldg(G + i), e1 = __ldg(G + i + 1);
  f = quotient(E - e0, e1 - e0);
}

// Lookups of several nuclides at one energy: nuclides on the grid located
// last reuse its interval and fraction (identical grids give identical
// values, so this is bit-identical to a search per nuclide).
struct GridCursor {
  int g = -1, i = 0;
  double f = 0.0;
};

__device__ __forceinline__ void micro_xs(const DevXS& X, int nuc, int k, double E, GridCursor& c,
                                         double& st, double& ss) {
  const int g = __ldg(X.nuc_grid + nuc);
  if (g != c.g) {
    grid_locate(X, g, k, E, c.i, c.f);
    c.g = g;
  }
  const double2* S = X.sig + __ldg(X.nuc_off + nuc) + c.i;
  const double2 a = __ldg(S), b = __ldg(S + 1);
  st = fma(c.f, b.x - a.x, a.x);
  ss = fma(c.f, b.y - a.y, a.y);
}

// Sigma_t = sum_i N_i sigma_t,i(E), in material order (OpenMC
// Material::calculate_xs, called through event_calculate_xs).
// c: a cursor already at energy E (several materials evaluated at one
// energy share it, so nuclides of different materials on one grid are
// located once).
__device__ __forceinline__ double macro_total(const DevXS& X, int mat, double E, int k, GridCursor& c) {
  double acc = 0.0;
  const int j1 = __ldg(X.mat_off + mat + 1);
  for (int j = __ldg(X.mat_off + mat); j < j1; ++j) {
    double st, ss;
    micro_xs(X, __ldg(X.mat_nuc + j), k, E, c, st, ss);
    acc = fma(__ldg(X.mat_dens + j), st, acc);
  }
  return acc;
}

__device__ __forceinline__ double macro_total(const DevXS& X, int mat, double E, int k) {
  GridCursor c;
  return macro_total(X, mat, E, k, c);
}

__device__ __forceinline__ double macro_total(const DevXS& X, int mat, double E) {
  return macro_total(X, mat, E, xs_bucket32(X, E));
}

// nu*sigma_f of nuclide nuc at the cursor's interval (the cursor located
// nuc's grid), interpolated like sigma_t.
__device__ __forceinline__ double micro_nusf(const DevXS& X, int nuc, const GridCursor& c) {
  const double* F = X.nusf + __ldg(X.nuc_off + nuc) + c.i;
  const double a = __ldg(F), b = __ldg(F + 1);
  return fma(c.f, b - a, a);
}

// Sigma_t and nu*Sigma_f = sum over the fissionable nuclides of
// N_i nu*sigma_f,i(E), both in material order, in one pass (OpenMC
// Material::calculate_xs fills macro_xs.total and macro_xs.nu_fission).
__device__ __forceinline__ double macro_total_nuf(const DevXS& X, int mat, double E, int k, double& nuf,
                                                  GridCursor& c) {
  double acc = 0.0, nf = 0.0;
  const bool fis = X.nusf && __ldg(X.mat_fiss + mat);
  const int j1 = __ldg(X.mat_off + mat + 1);
  for (int j = __ldg(X.mat_off + mat); j < j1; ++j) {
    const int nuc = __ldg(X.mat_nuc + j);
    double st, ss;
    micro_xs(X, nuc, k, E, c, st, ss);
    const double N = __ldg(X.mat_dens + j);
    acc = fma(N, st, acc);
    if (fis && __ldg(X.nuc_fiss + nuc)) nf = fma(N, micro_nusf(X, nuc, c), nf);
  }
  nuf = nf;
  return acc;
}

__device__ __forceinline__ double macro_total_nuf(const DevXS& X, int mat, double E, int k, double& nuf) {
  GridCursor c;
  return macro_total_nuf(X, mat, E, k, nuf, c);
}

// Mixed-precision Sigma_t: the hash bin from a float log (grid_locate's
// guards correct a bin that rounding moved by one), the grid interval
// located in FP64 on the double grid, so the bracketing points are the
// FP64 ones; the fraction, the interpolation and the sum over nuclides in
// float.

// The float cursor of macro_total32: the grid located last, its interval
// and float fraction at the energy of the lookups that share it.
struct GridCursor32 {
  int g = -1, i = 0;
  float f = 0.0f;
};

template <bool kNuf = false>
__device__ __forceinline__ float macro_total32(const DevXS& X, int mat, double E, int k, GridCursor32& cur,
                                               float* nuf = nullptr) {
  float acc = 0.0f, nf = 0.0f;
  const bool fis = kNuf && X.nusf && __ldg(X.mat_fiss + mat);
  int gc = cur.g, i = cur.i;
  float f = cur.f;
  const int j1 = __ldg(X.mat_off + mat + 1);
  for (int j = __ldg(X.mat_off + mat); j < j1; ++j) {
    const int nuc = __ldg(X.mat_nuc + j);
    const int g = __ldg(X.nuc_grid + nuc);
    if (g != gc) {
      const double* G = X.gE + __ldg(X.g_off + g);
      i = grid_index(X, g, k, E);
      const double e0 = __ldg(G + i);
      f = narrow(E - e0) / narrow(__ldg(G + i + 1) - e0);
      gc = g;
    }
    const double2* S = X.sig + __ldg(X.nuc_off + nuc) + i;
    const float a = narrow(__ldg(&S[0].x)), b = narrow(__ldg(&S[1].x));
    const float N = narrow(__ldg(X.mat_dens + j));
    acc = fmaf(N, fmaf(f, b - a, a), acc);
    if (kNuf && fis && __ldg(X.nuc_fiss + nuc)) {
      const double* F = X.nusf + __ldg(X.nuc_off + nuc) + i;
      const float fa = narrow(__ldg(F)), fb = narrow(__ldg(F + 1));
      nf = fmaf(N, fmaf(f, fb - fa, fa), nf);
    }
  }
  cur.g = gc;
  cur.i = i;
  cur.f = f;
  if (kNuf) *nuf = nf;
  return acc;
}

template <bool kNuf = false>
__device__ __forceinline__ float macro_total32(const DevXS& X, int mat, double E, int k, float* nuf = nullptr) {
  GridCursor32 cur;
  return macro_total32<kNuf>(X, mat, E, k, cur, nuf);
}

// ---------------------------------------------------------------------------
// Start element (stands in for MOOSE ClaimRays): lowest-id tet containing x
// (all four half-spaces within kLocateTol) whose interior the direction
// enters; else the lowest-id containing tet; else -1.  Cell lists are in
// ascending tet id, so the first entered tet found is the answer.  Each
// candidate is first tested on the float planes: it is skipped only when a
// side proves x outside by more than the float error bound (same 12 * 2^-24
// bound as the float exit test), which the FP64 test would reject too.
__device__ __forceinline__ int locate(const DevMesh& M, double x, double y, double z, double u,
                                      double v, double w) {
  const double xs[3] = {x, y, z};
  int ci[3];
  for (int k = 0; k < 3; ++k) {
    // a multiplication instead of a division: the cell lists are padded by
    // kLocateTol, far above the few-ulp difference, so any point near a
    // cell boundary is listed in both cells and the result is the same
    const double q = (xs[k] - M.glo[k]) * M.ginv[k];
    int c = (int)floor(q);
    if (!(q >= 0.0)) c = 0;
    if (c > M.gn[k] - 1) c = M.gn[k] - 1;
    if (c < 0) c = 0;
    ci[k] = c;
  }
  const int64_t cell = ((int64_t)ci[2] * M.gn[1] + ci[1]) * M.gn[0] + ci[0];
  const float xf = (float)x, yf = (float)y, zf = (float)z;
  const float xa = fabsf(xf) + fabsf(yf) + fabsf(zf);
  // Fast path: walk from the cell's seed tet (which holds the cell centre c)
  // along the segment c -> x, one neighbour per step, on the float planes.
  // The walk only proposes a tet: it is returned when x is strictly inside
  // it by more than the float error bound and kLocateTol on every side --
  // then it is the one tet the FP64 rule below would return.  A walk that
  // meets the boundary, stalls or ends near a side falls back to the list.
  if (M.gseed) {
    int t = __ldg(M.gseed + cell);
    const float cx = (float)(M.glo[0] + (ci[0] + 0.5) * M.gh[0]);
    const float cy = (float)(M.glo[1] + (ci[1] + 0.5) * M.gh[1]);
    const float cz = (float)(M.glo[2] + (ci[2] + 0.5) * M.gh[2]);
    const float dx = xf - cx, dy = yf - cy, dz = zf - cz;
    for (int step = 0; step < 32 && t >= 0; ++step) {
      const Tet32* T = M.tet + t;
      const float4 pl[4] = {__ldg(&T->p[0]), __ldg(&T->p[1]), __ldg(&T->p[2]), __ldg(&T->p[3])};
      const int4 nb4 = __ldg(&T->nbr);
      bool in = true;
      int bf = -1;
      float tb = 3.0e38f;
#pragma unroll
      for (int f = 0; f < 4; ++f) {
        const float s32 = fmaf(pl[f].x, xf, fmaf(pl[f].y, yf, pl[f].z * zf)) - pl[f].w;
        if (!(s32 < -(1e-9f + 7.3e-7f * (fabsf(pl[f].w) + xa)))) in = false;
        const float den = fmaf(pl[f].x, dx, fmaf(pl[f].y, dy, pl[f].z * dz));
        if (den > 0.0f) {
          const float tt = (pl[f].w - fmaf(pl[f].x, cx, fmaf(pl[f].y, cy, pl[f].z * cz))) / den;
          if (tt < tb) {
            tb = tt;
            bf = f;
          }
        }
      }
      if (in) return t;
      if (bf < 0) break;
      const int nb = side_entry(nb4, bf);
      if (nb < 0) break;
      t = (nb & (kMatChange - 1)) >> 2;
    }
  }
  int best_any = -1;
  const int64_t q1 = M.gstart[cell + 1];
  for (int64_t q = M.gstart[cell]; q < q1; ++q) {
    const int t = __ldg(M.gtets + q);
    const float4* P32 = M.tet[t].p;
    bool out = false, in = true;
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      const float4 pl = __ldg(P32 + f);
      const float s32 = fmaf(pl.x, xf, fmaf(pl.y, yf, pl.z * zf)) - pl.w;
      const float m = 1e-9f + 7.3e-7f * (fabsf(pl.w) + xa);
      if (s32 > m) {
        out = true;
        break;
      }
      if (!(s32 < -m)) in = false;
    }
    if (out) continue;
    // strictly inside by more than the float error and kLocateTol on every
    // side: the FP64 test below would find it inside and entered, and no
    // other tet of a conforming mesh can contain the point
    if (in) return t;
    bool inside = true, enters = true;
    for (int f = 0; f < 4; ++f) {
      const double4_32a pl = M.planes[4 * (int64_t)t + f];
      const double s = pl.x * x + pl.y * y + pl.z * z - pl.w;
      if (s > kLocateTol) {
        inside = false;
        break;
      }
      if (s >= -kLocateTol) {
        const double dn = pl.x * u + pl.y * v + pl.z * w;
        if (!(dn < 0.0)) enters = false;
      }
    }
    if (!inside) continue;
    if (enters) return t;
    if (best_any < 0) best_any = t;
  }
  return best_any;
}

// ---------------------------------------------------------------------------
// Source site of history index h (OpenMCStudy::defineRays with OpenMC's
// initialize_history, OpenMCStudy.C:317-360): position, direction, energy
// drawn from the source stream of particle id h+1.
__device__ __forceinline__ void sample_source(const DevXS& X, const DevSource& S, const Skip& k,
                                              uint64_t master, mc_site& o) {
  uint64_t ss = stream_seed(k, master, kStreamSource);
  if (S.space == 0) {
    o.x = S.point[0];
    o.y = S.point[1];
    o.z = S.point[2];
  } else if (S.space == 1) {
    o.x = S.box_lo[0] + prn(ss) * (S.box_hi[0] - S.box_lo[0]);
    o.y = S.box_lo[1] + prn(ss) * (S.box_hi[1] - S.box_lo[1]);
    o.z = S.box_lo[2] + prn(ss) * (S.box_hi[2] - S.box_lo[2]);
  } else {
    int c = (int)(prn(ss) * (double)S.n_cyl);
    if (c > S.n_cyl - 1) c = S.n_cyl - 1;
    const double r = S.cyl_r * sqrt(prn(ss));
    double ct, st;
    sample_azimuth(ss, ct, st);
    o.x = S.cyl_xy[2 * c] + r * ct;
    o.y = S.cyl_xy[2 * c + 1] + r * st;
    o.z = S.cyl_z0 + prn(ss) * (S.cyl_z1 - S.cyl_z0);
  }
  const double mu = 2.0 * prn(ss) - 1.0;
  double cp, sp;
  sample_azimuth(ss, cp, sp);
  const double sm = sqrt(fmax0(1.0 - mu * mu));
  o.u = mu;
  o.v = sm * cp;
  o.w = sm * sp;
  o.E = (S.energy == 1) ? S.mono_E : sample_watt(ss, S.watt_a, S.watt_b, X.E_lo, X.E_hi);
  o.wgt = 1.0;
}

// Source site in float arithmetic for the mixed-precision form: the same
// source stream and the same sequence of draws as sample_source, each draw
// reduced to its 24 high bits, with float sqrt/log; the site is widened to
// double exactly.  Energies are accepted in [E_lo, E_hi) of the double
// grid bounds.
__device__ __forceinline__ float prn32(uint64_t& s) {
  s = kPrnMult * s + kPrnAdd;
  uint64_t w = ((s >> ((s >> 59u) + 5u)) ^ s) * 12605985483714917081ULL;
  w = (w >> 43u) ^ w;
  return (float)(uint32_t)(w >> 40) * 0x1.0p-24f;
}

__device__ __forceinline__ void azimuth32(uint64_t& s, float& c, float& sn) {
  for (int it = 0; it < 10000; ++it) {
    const float a = 2.0f * prn32(s) - 1.0f;
    const float b = 2.0f * prn32(s) - 1.0f;
    const float r2 = fmaf(a, a, b * b);
    if (r2 > 0.0f && r2 <= 1.0f) {
      const float inv = 1.0f / r2;
      c = (a - b) * (a + b) * inv;
      sn = 2.0f * a * b * inv;
      return;
    }
  }
  c = 1.0f;
  sn = 0.0f;
}

__device__ __forceinline__ double watt32(uint64_t& s, float a, float b, double E_lo, double E_hi) {
  const float ab4 = a * a * b * 0.25f, a2b = a * a * b;
  for (int it = 0; it < 1000; ++it) {
    const float r1 = prn32(s);
    const float r2 = prn32(s);
    float c2 = 0.5f;
    for (int j = 0; j < 10000; ++j) {
      const float p = prn32(s), q = prn32(s);
      const float rr = fmaf(p, p, q * q);
      if (rr > 0.0f && rr <= 1.0f) {
        c2 = p * p / rr;
        break;
      }
    }
    const float w = -a * (logf(r1) + logf(r2) * c2);
    const float E = w + ab4 + (2.0f * prn32(s) - 1.0f) * sqrtf(a2b * w);
    if (E > 0.0f && E < 3.0e38f) {
      const double Ed = widen(E);
      if (Ed < E_hi && Ed >= E_lo) return Ed;
    }
  }
  return E_hi * 0.5;
}

__device__ __forceinline__ void sample_source32(const DevXS& X, const DevSource& S, const Skip& k,
                                                uint64_t master, mc_site& o) {
  uint64_t ss = stream_seed(k, master, kStreamSource);
  float x, y, z;
  if (S.space == 0) {
    x = narrow(S.point[0]);
    y = narrow(S.point[1]);
    z = narrow(S.point[2]);
  } else if (S.space == 1) {
    x = fmaf(prn32(ss), narrow(S.box_hi[0]) - narrow(S.box_lo[0]), narrow(S.box_lo[0]));
    y = fmaf(prn32(ss), narrow(S.box_hi[1]) - narrow(S.box_lo[1]), narrow(S.box_lo[1]));
    z = fmaf(prn32(ss), narrow(S.box_hi[2]) - narrow(S.box_lo[2]), narrow(S.box_lo[2]));
  } else {
    int c = (int)(prn32(ss) * (float)S.n_cyl);
    if (c > S.n_cyl - 1) c = S.n_cyl - 1;
    const float r = narrow(S.cyl_r) * sqrtf(prn32(ss));
    float ct, st;
    azimuth32(ss, ct, st);
    x = fmaf(r, ct, narrow(__ldg(S.cyl_xy + 2 * c)));
    y = fmaf(r, st, narrow(__ldg(S.cyl_xy + 2 * c + 1)));
    const float z0 = narrow(S.cyl_z0);
    z = fmaf(prn32(ss), narrow(S.cyl_z1) - z0, z0);
  }
  const float mu = 2.0f * prn32(ss) - 1.0f;
  float cp, sp;
  azimuth32(ss, cp, sp);
  const float sm = sqrtf(fmaxf(0.0f, (1.0f - mu) * (1.0f + mu)));
  o.x = widen(x);
  o.y = widen(y);
  o.z = widen(z);
  o.u = widen(mu);
  o.v = widen(sm * cp);
  o.w = widen(sm * sp);
  o.E = (S.energy == 1) ? S.mono_E : watt32(ss, narrow(S.watt_a), narrow(S.watt_b), X.E_lo, X.E_hi);
  o.wgt = 1.0;
}

// A history starts at its site: tracking stream of particle id h+1, start
// element located (stands in for MOOSE ClaimRays).
__device__ __forceinline__ void start(const DevMesh& M, const mc_site& o, int64_t h, const Skip& k,
                                      uint64_t master, Particle& p) {
  p.id = h + 1;
  p.seed = stream_seed(k, master, kStreamTracking);
  p.x = o.x;
  p.y = o.y;
  p.z = o.z;
  p.u = o.u;
  p.v = o.v;
  p.w = o.w;
  p.E = o.E;
  p.wgt = o.wgt;
  p.hash = kFnvOffset;
  p.status = kAlive;
  p.n_seg = 0;
  p.n_coll = 0;
  p.face = -1;
  p.fin = -1;
  p.zero_run = 0;
  p.mat = -2;
  p.sigt = 0.0;
  p.nuf = 0.0;
  p.ktl = 0.0;
  p.n_prog = 0;
  xs_cache_clear(p);
  p.elem = locate(M, p.x, p.y, p.z, p.u, p.v, p.w);
  if (p.elem < 0) p.status = kLost;
}

// ---------------------------------------------------------------------------
// Collision-estimator scores at a collision, at the energy before it (the
// estimator OpenMCTally admits, OpenMCTally.C:86-87): flux wgt/Sigma_t,
// total wgt, scatter wgt*Sigma_s/Sigma_t, absorption
// wgt*(Sigma_t-Sigma_s)/Sigma_t; Sigma_s summed over the material's
// nuclides in material order.
__device__ __forceinline__ void score_collision(const DevXS& X, const TallySpec& T, double* tally,
                                                const Particle& p) {
  if (!T.general || T.est != MC_EST_COLLISION) return;
  const int b = energy_bin(T, p.E);
  if (b < 0) return;
  double ss = 0.0;
  if (T.need_ss) {
    const int k = xs_bucket32(X, p.E);
    GridCursor gc;
    const int j1 = __ldg(X.mat_off + p.mat + 1);
    for (int j = __ldg(X.mat_off + p.mat); j < j1; ++j) {
      double st, sj;
      micro_xs(X, __ldg(X.mat_nuc + j), k, p.E, gc, st, sj);
      ss = fma(__ldg(X.mat_dens + j), sj, ss);
    }
  }
  double* t = tally + ((int64_t)p.elem * T.nb + b) * T.ns;
  for (int j = 0; j < T.ns; ++j) {
    const int sc = (T.sc >> (8 * j)) & 0xff;
    double v;
    if (sc == MC_SCORE_FLUX) v = p.wgt / p.sigt;
    else if (sc == MC_SCORE_TOTAL) v = p.wgt;
    else if (sc == MC_SCORE_SCATTER) v = p.wgt * ss / p.sigt;
    else v = p.wgt * (p.sigt - ss) / p.sigt;
    atomicAdd(t + j, v);
  }
}

// ---------------------------------------------------------------------------
// Fission sites of a collision with fissionable nuclide nuc (OpenMC
// create_fission_sites and sample_fission_neutron, with no uniform fission
// source weighting and no delayed-neutron data): nu_t = wgt/keff *
// nu*sigma_f/sigma_t sites, its fraction by one draw; each site starts at
// the collision point with weight 1, an isotropic direction (polar cosine,
// azimuth), one draw against the delayed fraction beta = 0, and a prompt
// energy from the Watt spectrum.  Banked in eigenvalue runs; in fixed-source
// runs they are drawn and dropped (MaCaw tracks no secondaries,
// CollisionKernel.C:236).
constexpr double kWattADefault = 0.988e6;   // eV
constexpr double kWattBDefault = 2.249e-6;  // 1/eV

__device__ __forceinline__ void fission_sites(const DevXS& X, Particle& p, const EigArgs& e, bool on,
                                              double nf, double st) {
  // fixed-source runs: keff 1 and the default spectrum
  const double keff = on ? e.keff : 1.0;
  const double fa = on ? e.fa : kWattADefault, fb = on ? e.fb : kWattBDefault;
  const double nu_t = p.wgt / keff * nf / st;
  int nu = (int)nu_t;
  if (prn(p.seed) <= nu_t - (double)nu) ++nu;
  for (int k = 0; k < nu; ++k) {
    mc_fission_site o;
    o.x = p.x;
    o.y = p.y;
    o.z = p.z;
    const double mu = 2.0 * prn(p.seed) - 1.0;
    double cp, sp;
    sample_azimuth(p.seed, cp, sp);
    const double sm = sqrt(fmax0(1.0 - mu * mu));
    o.u = mu;
    o.v = sm * cp;
    o.w = sm * sp;
    (void)prn(p.seed);  // delayed or prompt: beta = 0, always prompt
    o.E = sample_watt(p.seed, fa, fb, X.E_lo, X.E_hi);
    o.wgt = 1.0;
    o.parent = p.id;
    o.progeny = p.n_prog;
    o.pad = 0;
    p.n_prog += 1;
    if (on) {
      const unsigned long long i = atomicAdd(e.n_bank, 1ull);
      if (i < (unsigned long long)e.cap) e.bank[i] = o;
    }
  }
}

// Collision at the current position (OpenMC event_collide as MaCaw calls
// it, CollisionKernel.C:185-230): nuclide by cumulative N_i sigma_t,i,
// fission sites when that nuclide is fissionable, absorption if
// xi*sigma_t < sigma_a, else elastic scattering isotropic in the
// centre-of-mass frame off a target at rest.  Absorption and energy cutoff
// end the history; secondaries are not tracked (CollisionKernel.C:236).
// Eigenvalue runs score the collision estimate of keff before the nuclide
// is drawn and the absorption estimate at an absorption (OpenMC
// event_collide, absorption).
// kEig = false: a fixed-source launch (e.on is not read).
template <bool kEig>
__device__ __forceinline__ void collide(const DevXS& X, Particle& p, bool two_d, const EigArgs& e) {
  const int mat = p.mat;
  const bool on = kEig && e.on;
  const int64_t h = p.id - 1 - e.first;
  if (on && p.nuf > 0.0) e.kcol[h] += p.wgt * p.nuf / p.sigt;
  const int k = xs_bucket32(X, p.E);
  const double cutoff = prn(p.seed) * p.sigt;
  double acc = 0.0, st = 0.0, ss = 0.0;
  const int j0 = __ldg(X.mat_off + mat), j1 = __ldg(X.mat_off + mat + 1);
  int pick = -1;
  GridCursor gc;
  for (int j = j0; j < j1; ++j) {
    micro_xs(X, __ldg(X.mat_nuc + j), k, p.E, gc, st, ss);
    acc = fma(__ldg(X.mat_dens + j), st, acc);
    if (acc >= cutoff) {
      pick = j;
      break;
    }
  }
  if (pick < 0) pick = j1 - 1;
  const int nuc = __ldg(X.mat_nuc + pick);
  double nf = 0.0;
  // the cursor holds the interval of the picked nuclide's grid
  if (X.nusf && __ldg(X.nuc_fiss + nuc)) {
    nf = micro_nusf(X, nuc, gc);
    fission_sites(X, p, e, on, nf, st);
  }
  const double sa = st - ss;
  if (prn(p.seed) * st < sa) {
    if (on && nf > 0.0) e.kabs[h] += p.wgt * nf / sa;
    p.status = kAbsorbed;
    return;
  }
  const double A = __ldg(X.awr + nuc);
  const double mu_cm = 2.0 * prn(p.seed) - 1.0;
  const double q = A * A + 2.0 * A * mu_cm + 1.0;
  const double Ap1 = A + 1.0;
  const double E2 = p.E * q / (Ap1 * Ap1);
  double cp, sp;
  sample_azimuth(p.seed, cp, sp);
  if (!(q > 0.0) || !(E2 >= X.E_lo)) {
    p.E = E2;
    p.status = kCutoff;
    return;
  }
  double mu_lab = (1.0 + A * mu_cm) / sqrt(q);
  if (mu_lab > 1.0) mu_lab = 1.0;
  if (mu_lab < -1.0) mu_lab = -1.0;
  rotate_dir(p.u, p.v, p.w, mu_lab, cp, sp);
  if (two_d) planar_dir(p.u, p.v, p.w);
  p.E = E2;
  p.mat = -2;  // energy changed: cross sections are recomputed
  p.fin = -1;
  xs_cache_clear(p);
}

// ---------------------------------------------------------------------------
// One segment of the FP64 walk.  Returns 0 when the particle crossed a face
// (or reflected) and continues, 1 when a collision was sampled inside the
// element (position already moved to the collision point), 2 when the
// history ended (leak, stuck, bad XS), 3 when the element's material has no
// cached cross section and kInlineXS is false (a cross-section event is due
// before this segment).
//
// The distance-to-collision test first compares -logf(xi) against
// L*Sigma_t in float with a margin that covers float rounding and logf's
// error bound; only when that comparison is not decisive is the FP64 log
// evaluated.  Either way the outcome and the score (L when d > L) are the
// values the FP64 arithmetic gives.
// L2 prefetch of the walk records (and, for the FP64 form, the FP64
// planes) of the neighbours of the element just entered: used by the tail
// kernel, where a few long histories walk alone and each step would
// otherwise wait a full DRAM round trip for a record nobody else touches.
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

template <bool kFP64>
__device__ __forceinline__ void prefetch_neighbours(const DevMesh& M, const int4& nb4, int fin) {
  const int e[4] = {nb4.x, nb4.y, nb4.z, nb4.w};
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    if (f == fin || e[f] < 0) continue;
    const int t = (e[f] & (kMatChange - 1)) >> 2;
    const char* r = (const char*)(M.tet + t);
    prefetch_l2(r);
    prefetch_l2(r + 64);
    if (kFP64) {
      prefetch_l2(M.planes + 4 * (int64_t)t);
      prefetch_l2(M.planes + 4 * (int64_t)t + 2);
    }
  }
}

template <bool kInlineXS, bool kRays = true, bool kEig = false>
__device__ __forceinline__ int segment_fp64(const DevMesh& M, const DevXS& X, Particle& p,
                                            double* __restrict__ tally, const TallySpec& T, float& sigt32,
                                            unsigned long long& n_xs) {
  if (p.n_seg >= M.max_seg || p.zero_run >= kMaxZeroRun) {
    p.status = kStuck;
    return 2;
  }
  // the material is looked up only when it may have changed: after birth,
  // a collision, or a crossing through a side flagged kMatChange
  if (p.mat < 0) {
    const int mat = __ldg(M.tmat + p.elem);
    if (mat < 0) {
      p.status = kBadXS;
      return 2;
    }
    if (!xs_cache_get<kEig>(p, mat)) {
      if (!kInlineXS) return 3;
      double nf = 0.0;
      const double s = kEig ? macro_total_nuf(X, mat, p.E, xs_bucket32(X, p.E), nf)
                            : macro_total(X, mat, p.E);
      ++n_xs;
      if (!(s > 0.0) || s != s) {
        p.status = kBadXS;
        return 2;
      }
      p.sigt = s;
      if (kEig) p.nuf = nf;
      xs_cache_put<kEig>(p, mat, s, nf);
    }
    p.mat = mat;
    sigt32 = narrow(p.sigt);
  }
  const double4_32a* P = M.planes + 4 * (int64_t)p.elem;
  int bf = -1;
  double bnum = 0.0, bden = 1.0;
  // The entry side is skipped: its plane is the exact negation of the exit
  // plane of the previous element, so n.u there is negative and the full
  // search would reject it anyway.
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    if (f == p.fin) continue;
    const double4_32a pl = P[f];
    const double den = fma(pl.x, p.u, fma(pl.y, p.v, pl.z * p.w));
    if (den > 0.0) {
      const double num = fma(-pl.x, p.x, fma(-pl.y, p.y, fma(-pl.z, p.z, pl.w)));
      if (bf < 0 || num * bden < bnum * den) {
        bf = f;
        bnum = num;
        bden = den;
      }
    }
  }
  if (bf < 0) {
    p.status = kStuck;
    return 2;
  }
  double L = quotient(bnum, bden);
  if (!(L > 0.0)) L = 0.0;
  const double xi = prn(p.seed);
  const float lf = -logf((float)xi);
  const float thr = (float)L * sigt32;
  bool cross;
  double dist = 0.0;
  if (lf > thr * 1.00001f + 1e-6f) {
    cross = true;
  } else {
    dist = quotient(-mc::log64(xi), p.sigt);
    cross = dist > L;
  }
  const double score = cross ? L : dist;  // (L < dist) ? L : dist
  score_track(T, tally, p.elem, p.E, p.wgt * score, p.sigt);
  if (kEig) p.ktl = p.ktl + p.wgt * score * p.nuf;  // CollisionKernel.C:153-154
  ++p.n_seg;
  if (L == 0.0) ++p.zero_run;
  else p.zero_run = 0;
  if (cross) {
    p.hash = fnv(p.hash, (uint64_t)p.elem * 8ULL + (uint64_t)bf);
    const double sx = p.x, sy = p.y, sz = p.z;
    p.x = fma(L, p.u, p.x);
    p.y = fma(L, p.v, p.y);
    p.z = fma(L, p.w, p.z);
    if (kRays && T.rays) record_ray(T, p, sx, sy, sz, p.x, p.y, p.z);
    const int nb = side_entry(M.tet[p.elem].nbr, bf);
    if (nb >= 0) {
      if (nb & kMatChange) p.mat = -2;
      p.elem = (nb & (kMatChange - 1)) >> 2;
      p.fin = nb & 3;
      return 0;
    }
    const int bid = -1 - nb;
    if (bid < M.n_bid && M.bc_type[bid] == 1) {
      const double4_32a pl = P[bf];
      const double dn = fma(p.u, pl.x, fma(p.v, pl.y, p.w * pl.z));
      const double t2 = 2.0 * dn;
      p.u = fma(-t2, pl.x, p.u);
      p.v = fma(-t2, pl.y, p.v);
      p.w = fma(-t2, pl.z, p.w);
      p.fin = -1;
      return 0;
    }
    p.status = kLeaked;
    p.face = bf;
    return 2;
  }
  p.hash = fnv(p.hash, (uint64_t)p.elem * 8ULL + 4ULL);
  const double ex = fma(L, p.u, p.x), ey = fma(L, p.v, p.y), ez = fma(L, p.w, p.z);
  const double back = L - dist;
  const double sx = p.x, sy = p.y, sz = p.z;
  p.x = fma(-back, p.u, ex);
  p.y = fma(-back, p.v, ey);
  p.z = fma(-back, p.w, ez);
  ++p.n_coll;
  if (kRays && T.rays) record_ray(T, p, sx, sy, sz, p.x, p.y, p.z);
  p.zero_run = 0;
  return 1;
}

// ---------------------------------------------------------------------------
// FP64 segment with a float-certified exit side.  Exit distances are first
// solved on the float planes with the float position; each float distance
// t32 carries a bound e on |t32 - t| derived from the float rounding of the
// planes, the position and every operation (constant 12 * 2^-24 covers the
// input roundings and the fused dot products, see below).  When the float
// intervals [t32-e, t32+e] of the nearest candidate and every other
// candidate are disjoint, and every side's n.u sign is certain, the FP64
// search of segment_fp64 would pick the same side, so only that side is
// evaluated in FP64; otherwise this falls back to segment_fp64's full
// search.  The distance-to-collision pre-test uses the float interval for L
// and a float upper bound for xi.  Results are bit-identical to
// segment_fp64.
//
// Error bounds (u = 2^-24): the float planes and position/direction are
// roundings of the FP64 values (relative u each); num32 = d - (nx*x + ny*y
// + nz*z) through two fmaf and one product and a subtraction: |num32 - num|
// <= u (2|d| + 6 sum|n_i x_i|)(1+u) <= 12u (|d| + |x|_1) since |n_i| <= 1;
// likewise |den32 - den| <= 12u |u|_1; t32 = num32/den32 rounded (0.5 ulp):
// |t - t32| <= (E_num + |t32| E_den)/(den32 - E_den) + 4.8e-7 |t32|, padded
// by 0.1%.
template <bool kInlineXS, bool kPrefetch = false, bool kRays = true, bool kEig = false>
__device__ __forceinline__ int segment_fp64g(const DevMesh& M, const DevXS& X, Particle& p,
                                             const float uf, const float vf, const float wf,
                                             double* __restrict__ tally, const TallySpec& T, float& sigt32,
                                             unsigned long long& n_xs) {
  if (p.n_seg >= M.max_seg || p.zero_run >= kMaxZeroRun) {
    p.status = kStuck;
    return 2;
  }
  // the material is looked up only when it may have changed: after birth,
  // a collision, or a crossing through a side flagged kMatChange
  if (p.mat < 0) {
    const int mat = __ldg(M.tmat + p.elem);
    if (mat < 0) {
      p.status = kBadXS;
      return 2;
    }
    if (!xs_cache_get<kEig>(p, mat)) {
      if (!kInlineXS) return 3;
      double nf = 0.0;
      const double s = kEig ? macro_total_nuf(X, mat, p.E, xs_bucket32(X, p.E), nf)
                            : macro_total(X, mat, p.E);
      ++n_xs;
      if (!(s > 0.0) || s != s) {
        p.status = kBadXS;
        return 2;
      }
      p.sigt = s;
      if (kEig) p.nuf = nf;
      xs_cache_put<kEig>(p, mat, s, nf);
    }
    p.mat = mat;
    sigt32 = narrow(p.sigt);
  }
  // float copies by integer operations (a conversion would issue on the
  // FP64 pipe, which bounds this walk); narrow() differs from a conversion
  // only below 2^-126, far inside the bounds' additive term
  const float xf = narrow(p.x), yf = narrow(p.y), zf = narrow(p.z);
  const float xa = fabsf(xf) + fabsf(yf) + fabsf(zf);
  const float Eden = 7.2e-7f * (fabsf(uf) + fabsf(vf) + fabsf(wf));
  const float4* P32 = M.tet[p.elem].p;
  const int4 nb4 = __ldg(&M.tet[p.elem].nbr);  // issued with the plane loads
  if (kPrefetch) prefetch_neighbours<true>(M, nb4, p.fin);
  bool sure = true;
  int bf = -1;
  float tb = 3.0e38f, eb = 0.0f, lo_other = 3.0e38f;
  // Branch-free over the four sides (the entry side and sides facing away
  // get t = 3e38, e = 0, which changes nothing below).  The divisions are
  // __fdividef (at most 2 ulp for the normal divisors here), inside the
  // 4.8e-7 |t| division term and the 0.1% padding of the bound.
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    const float4 pl = __ldg(P32 + f);
    const float den = fmaf(pl.x, uf, fmaf(pl.y, vf, pl.z * wf));
    const float num = pl.w - fmaf(pl.x, xf, fmaf(pl.y, yf, pl.z * zf));
    const float En = 7.2e-7f * (fabsf(pl.w) + xa);
    const bool other = f != p.fin;
    if (other && fabsf(den) <= Eden) sure = false;
    const bool cand = other && den > Eden;
    const float t = cand ? __fdividef(num, den) : 3.0e38f;
    const float e =
        cand ? (__fdividef(En + fabsf(t) * Eden, den - Eden) + 4.8e-7f * fabsf(t)) * 1.001f + 1e-30f : 0.0f;
    const bool nearer = t < tb;
    lo_other = fminf(lo_other, nearer ? tb - eb : t - e);
    bf = nearer ? f : bf;
    tb = nearer ? t : tb;
    eb = nearer ? e : eb;
  }
  if (!sure || bf < 0 || !(tb + eb < lo_other)) {
    const int r = segment_fp64<kInlineXS, kRays, kEig>(M, X, p, tally, T, sigt32, n_xs);
    return (r == 0 && p.fin < 0) ? 5 : r;  // a reflection changed the direction
  }
  const double4_32a* P = M.planes + 4 * (int64_t)p.elem;
  const double4_32a plb = P[bf];
  const double bden = fma(plb.x, p.u, fma(plb.y, p.v, plb.z * p.w));
  const double bnum = fma(-plb.x, p.x, fma(-plb.y, p.y, fma(-plb.z, p.z, plb.w)));
  double L = quotient(bnum, bden);
  // L > 0 as a sign test on the bits (bden > 0 is certified and bnum is
  // finite, so L is not NaN; -0 clamps to +0 as before)
  if ((long long)dbits(L) <= 0) L = 0.0;
  // one draw per segment: advance the state once, derive both forms
  p.seed = kPrnMult * p.seed + kPrnAdd;
  uint64_t wv = ((p.seed >> ((p.seed >> 59u) + 5u)) ^ p.seed) * 12605985483714917081ULL;
  wv = (wv >> 43u) ^ wv;
  // xi = (wv >> 11) 2^-53 < (hi32 + 1) 2^-32 <= xhi; lf is a lower bound of
  // -ln(xi): __logf's documented error is at most 2^-21.41 absolute on
  // [0.5, 2] and 3 ulp elsewhere, inside the 1e-6 relative and 1e-6
  // absolute margins
  const float xhi = fmaf((float)(uint32_t)(wv >> 32), 2.3283064365386963e-10f, 2.3283064365386963e-10f) *
                    1.00000024f;
  const float lf = -__logf(xhi) * 0.999999f - 1e-6f;
  const float thr = fmaxf(tb + eb, 0.0f) * sigt32;
  bool cross;
  double dist = 0.0;
  if (lf > thr * 1.00001f + 1e-6f) {
    cross = true;
  } else {
    const double xi = unit53(wv >> 11);
    dist = quotient(-mc::log64(xi), p.sigt);
    cross = dist > L;
  }
  const double score = cross ? L : dist;
  // weight 1 and L == 0 tested on the bits (integer pipe)
  score_track(T, tally, p.elem, p.E, dbits(p.wgt) == dbits(1.0) ? score : p.wgt * score, p.sigt);
  if (kEig) p.ktl = p.ktl + p.wgt * score * p.nuf;  // CollisionKernel.C:153-154
  ++p.n_seg;
  if (dbits(L) == 0) ++p.zero_run;
  else p.zero_run = 0;
  if (cross) {
    p.hash = fnv(p.hash, (uint64_t)p.elem * 8ULL + (uint64_t)bf);
    const double sx = p.x, sy = p.y, sz = p.z;
    p.x = fma(L, p.u, p.x);
    p.y = fma(L, p.v, p.y);
    p.z = fma(L, p.w, p.z);
    if (kRays && T.rays) record_ray(T, p, sx, sy, sz, p.x, p.y, p.z);
    const int nb = side_entry(nb4, bf);
    if (nb >= 0) {
      if (nb & kMatChange) p.mat = -2;
      p.elem = (nb & (kMatChange - 1)) >> 2;
      p.fin = nb & 3;
      return 0;
    }
    const int bid = -1 - nb;
    if (bid < M.n_bid && M.bc_type[bid] == 1) {
      const double dn = fma(p.u, plb.x, fma(p.v, plb.y, p.w * plb.z));
      const double t2 = 2.0 * dn;
      p.u = fma(-t2, plb.x, p.u);
      p.v = fma(-t2, plb.y, p.v);
      p.w = fma(-t2, plb.z, p.w);
      p.fin = -1;
      return 5;  // reflected: the caller refreshes its float direction
    }
    p.status = kLeaked;
    p.face = bf;
    return 2;
  }
  p.hash = fnv(p.hash, (uint64_t)p.elem * 8ULL + 4ULL);
  const double ex = fma(L, p.u, p.x), ey = fma(L, p.v, p.y), ez = fma(L, p.w, p.z);
  const double back = L - dist;
  const double sx = p.x, sy = p.y, sz = p.z;
  p.x = fma(-back, p.u, ex);
  p.y = fma(-back, p.v, ey);
  p.z = fma(-back, p.w, ez);
  ++p.n_coll;
  if (kRays && T.rays) record_ray(T, p, sx, sy, sz, p.x, p.y, p.z);
  p.zero_run = 0;
  return 1;
}

// ---------------------------------------------------------------------------
// The FP64 segment of the compact walk (k_ev_advance_fp64): segment_fp64g's
// arithmetic and results, bit for bit, with the element's 64-byte
// octahedral record (O01, O23, D, entries nb4 and, after a flagged side,
// the material mnext) already in registers.  The exit side is certified on
// the octahedral planes: their decoded normals m differ from the FP64 unit
// normals n by at most M.oct_err in |m/|m| - n|_1 (measured on the host
// over every plane of the mesh), which adds oct_err * (|x| + |d|) to the
// numerator bound and oct_err * |u| to the denominator bound of the float
// planes' 12 * 2^-24 (see segment_fp64g).  As soon as the exit side is
// certified and the float pretest decides that the particle crosses, the
// neighbour's record is requested and the line of its FP64 planes
// prefetched into L1, before this segment's FP64 distance, tally and
// position update; so the next segment's loads are in flight while they
// run.  Same return codes as segment_fp64g (0 crossed, 1 collision, 2
// ended, 3 XS event, 5 reflected); after the full-search fallback
// (uncertified exits) the record is reloaded.
__device__ __forceinline__ void load_oct(const DevMesh& M, int t, float4& O01, float4& O23, float4& D, int4& nb4) {
  const TetOct* T = M.teto + t;
  O01 = __ldg(&T->oct01);
  O23 = __ldg(&T->oct23);
  D = __ldg(&T->d);
  nb4 = __ldg(&T->nbr);
}

__device__ __forceinline__ void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

template <bool kEig>
__device__ __forceinline__ int segment_fp64c(const DevMesh& M, const DevXS& X, Particle& p, float& uf, float& vf,
                                             float& wf, float4& O01, float4& O23, float4& D, int4& nb4,
                                             int& mnext, double* __restrict__ tally, const TallySpec& T,
                                             float& sigt32, unsigned long long& n_xs) {
  if (p.n_seg >= M.max_seg || p.zero_run >= kMaxZeroRun) {
    p.status = kStuck;
    return 2;
  }
  if (p.mat < 0) {
    const int mat = mnext;
    if (mat < 0) {
      p.status = kBadXS;
      return 2;
    }
    if (!xs_cache_get<kEig>(p, mat)) return 3;
    p.mat = mat;
    sigt32 = narrow(p.sigt);
  }
  const float xf = narrow(p.x), yf = narrow(p.y), zf = narrow(p.z);
  const float xa = fabsf(xf) + fabsf(yf) + fabsf(zf);
  const float cb = 7.2e-7f + M.oct_err;
  const float Eden = cb * (fabsf(uf) + fabsf(vf) + fabsf(wf));
  bool sure = true;
  int bf = -1;
  float tb = 3.0e38f, eb = 0.0f, lo_other = 3.0e38f;
  auto side = [&](const float4& pl, int f) {
    const float den = fmaf(pl.x, uf, fmaf(pl.y, vf, pl.z * wf));
    const float num = pl.w - fmaf(pl.x, xf, fmaf(pl.y, yf, pl.z * zf));
    const float En = cb * (fabsf(pl.w) + xa);
    const bool other = f != p.fin;
    if (other && fabsf(den) <= Eden) sure = false;
    const bool cand = other && den > Eden;
    const float t = cand ? __fdividef(num, den) : 3.0e38f;
    const float e =
        cand ? (__fdividef(En + fabsf(t) * Eden, den - Eden) + 4.8e-7f * fabsf(t)) * 1.001f + 1e-30f : 0.0f;
    const bool nearer = t < tb;
    lo_other = fminf(lo_other, nearer ? tb - eb : t - e);
    bf = nearer ? f : bf;
    tb = nearer ? t : tb;
    eb = nearer ? e : eb;
  };
  side(oct_plane(O01.x, O01.y, D.x), 0);
  side(oct_plane(O01.z, O01.w, D.y), 1);
  side(oct_plane(O23.x, O23.y, D.z), 2);
  side(oct_plane(O23.z, O23.w, D.w), 3);
  if (!sure || bf < 0 || !(tb + eb < lo_other)) {
    const int r = segment_fp64<false, false, kEig>(M, X, p, tally, T, sigt32, n_xs);
    if (r == 0 || r == 5) {  // a new element (or a new direction): its record
      load_oct(M, p.elem, O01, O23, D, nb4);
      if (p.mat < 0) mnext = __ldg(M.tmat + p.elem);
    }
    return (r == 0 && p.fin < 0) ? 5 : r;
  }
  // one draw per segment: advance the state once, derive both forms
  p.seed = kPrnMult * p.seed + kPrnAdd;
  uint64_t wv = ((p.seed >> ((p.seed >> 59u) + 5u)) ^ p.seed) * 12605985483714917081ULL;
  wv = (wv >> 43u) ^ wv;
  const float xhi = fmaf((float)(uint32_t)(wv >> 32), 2.3283064365386963e-10f, 2.3283064365386963e-10f) *
                    1.00000024f;
  const float lf = -__logf(xhi) * 0.999999f - 1e-6f;
  const float thr = fmaxf(tb + eb, 0.0f) * sigt32;
  const bool cross_sure = lf > thr * 1.00001f + 1e-6f;
  const int nb = side_entry(nb4, bf);
  const int next = (nb & (kMatChange - 1)) >> 2;
  const double4_32a plb = M.planes[4 * (int64_t)p.elem + bf];
  if (cross_sure && nb >= 0) {
    // the neighbour's record and FP64 planes, requested ahead of this
    // segment's FP64 work
    load_oct(M, next, O01, O23, D, nb4);
    if (nb & kMatChange) mnext = __ldg(M.tmat + next);
    prefetch_l1(M.planes + 4 * (int64_t)next);
  }
  const double bden = fma(plb.x, p.u, fma(plb.y, p.v, plb.z * p.w));
  const double bnum = fma(-plb.x, p.x, fma(-plb.y, p.y, fma(-plb.z, p.z, plb.w)));
  double L = quotient(bnum, bden);
  if ((long long)dbits(L) <= 0) L = 0.0;
  bool cross = cross_sure;
  double dist = 0.0;
  if (!cross_sure) {
    const double xi = unit53(wv >> 11);
    dist = quotient(-mc::log64(xi), p.sigt);
    cross = dist > L;
    if (cross && nb >= 0) {
      load_oct(M, next, O01, O23, D, nb4);
      if (nb & kMatChange) mnext = __ldg(M.tmat + next);
    }
  }
  const double score = cross ? L : dist;
  score_track(T, tally, p.elem, p.E, dbits(p.wgt) == dbits(1.0) ? score : p.wgt * score, p.sigt);
  if (kEig) p.ktl = p.ktl + p.wgt * score * p.nuf;  // CollisionKernel.C:153-154
  ++p.n_seg;
  if (dbits(L) == 0) ++p.zero_run;
  else p.zero_run = 0;
  if (cross) {
    p.hash = fnv(p.hash, (uint64_t)p.elem * 8ULL + (uint64_t)bf);
    p.x = fma(L, p.u, p.x);
    p.y = fma(L, p.v, p.y);
    p.z = fma(L, p.w, p.z);
    if (nb >= 0) {
      if (nb & kMatChange) p.mat = -2;
      p.elem = next;
      p.fin = nb & 3;
      return 0;
    }
    const int bid = -1 - nb;
    if (bid < M.n_bid && M.bc_type[bid] == 1) {
      const double dn = fma(p.u, plb.x, fma(p.v, plb.y, p.w * plb.z));
      const double t2 = 2.0 * dn;
      p.u = fma(-t2, plb.x, p.u);
      p.v = fma(-t2, plb.y, p.v);
      p.w = fma(-t2, plb.z, p.w);
      p.fin = -1;
      return 5;  // reflected: the caller refreshes its float direction (the record is still this element's)
    }
    p.status = kLeaked;
    p.face = bf;
    return 2;
  }
  p.hash = fnv(p.hash, (uint64_t)p.elem * 8ULL + 4ULL);
  const double ex = fma(L, p.u, p.x), ey = fma(L, p.v, p.y), ez = fma(L, p.w, p.z);
  const double back = L - dist;
  p.x = fma(-back, p.u, ex);
  p.y = fma(-back, p.v, ey);
  p.z = fma(-back, p.w, ez);
  ++p.n_coll;
  p.zero_run = 0;
  return 1;
}

// ---------------------------------------------------------------------------
// Mixed-precision form.  Position and direction live in float registers for
// the walk; exits are solved on the float planes; the two nearest exit
// distances must differ by more than tol (1e-6 of the mesh bounding-box
// diagonal) and the nearest must not lie behind the particle by more than
// tol, otherwise the exit is re-solved on the FP64 planes with the position
// promoted to double (a ray passing within tol of an edge or vertex, or a
// particle that rounding left just outside its element).  Distances to
// collision are sampled in float; scores are accumulated in FP64.
struct Geo32 {
  float x, y, z, u, v, w;
};

// Conversions by integer operations (narrow, widen), off the FP64 pipe.
__device__ __forceinline__ void geo_load(const Particle& p, Geo32& g) {
  g.x = narrow(p.x); g.y = narrow(p.y); g.z = narrow(p.z);
  g.u = narrow(p.u); g.v = narrow(p.v); g.w = narrow(p.w);
}

__device__ __forceinline__ void geo_store(const Geo32& g, Particle& p) {
  p.x = widen(g.x); p.y = widen(g.y); p.z = widen(g.z);
  p.u = widen(g.u); p.v = widen(g.v); p.w = widen(g.w);
}

// FP64 re-solve of the exit side for a position and direction given in
// double (the compact walk passes its compensated position x + xl).
__device__ __forceinline__ int exit_fp64d(const DevMesh& M, int elem, int fin, double x, double y, double z,
                                          double u, double v, double w, double& L) {
  const double4_32a* P = M.planes + 4 * (int64_t)elem;
  int bf = -1;
  double bnum = 0.0, bden = 1.0;
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    if (f == fin) continue;
    const double4_32a pl = P[f];
    const double den = pl.x * u + pl.y * v + pl.z * w;
    if (den > 0.0) {
      const double num = pl.w - (pl.x * x + pl.y * y + pl.z * z);
      if (bf < 0 || num * bden < bnum * den) {
        bf = f;
        bnum = num;
        bden = den;
      }
    }
  }
  if (bf >= 0) {
    L = bnum / bden;
    if (!(L > 0.0)) L = 0.0;
  }
  return bf;
}

// The same for a float position/direction.
__device__ __forceinline__ int exit_fp64(const DevMesh& M, int elem, int fin, const Geo32& g, double& L) {
  return exit_fp64d(M, elem, fin, g.x, g.y, g.z, g.u, g.v, g.w, L);
}

template <bool kInlineXS, bool kPrefetch = false, bool kEig = false>
__device__ __forceinline__ int segment_mixed(const DevMesh& M, const DevXS& X, Particle& p,
                                             Geo32& g, double* __restrict__ tally, const TallySpec& T,
                                             float& inv_sig,
                                             float tol, unsigned long long& n_xs,
                                             unsigned long long& n_fb) {
  if (p.n_seg >= M.max_seg || p.zero_run >= kMaxZeroRun) {
    p.status = kStuck;
    return 2;
  }
  // the material is looked up only when it may have changed: after birth,
  // a collision, or a crossing through a side flagged kMatChange
  if (p.mat < 0) {
    const int mat = __ldg(M.tmat + p.elem);
    if (mat < 0) {
      p.status = kBadXS;
      return 2;
    }
    if (!xs_cache_get<kEig>(p, mat)) {
      if (!kInlineXS) return 3;
      float nf32 = 0.0f;
      const double s = widen(macro_total32<kEig>(X, mat, p.E, xs_bucket32(X, p.E), &nf32));
      ++n_xs;
      if (!(s > 0.0) || s != s) {
        p.status = kBadXS;
        return 2;
      }
      p.sigt = s;
      if (kEig) p.nuf = widen(nf32);
      xs_cache_put<kEig>(p, mat, s, widen(nf32));
    }
    p.mat = mat;
    inv_sig = (float)(1.0 / p.sigt);
  }
  const float4* P = M.tet[p.elem].p;
  const int4 nb4 = __ldg(&M.tet[p.elem].nbr);  // issued with the plane loads
  if (kPrefetch) prefetch_neighbours<false>(M, nb4, p.fin);
  int bf = -1;
  float t1 = 3.0e38f, t2 = 3.0e38f;
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    if (f == p.fin) continue;
    const float4 pl = __ldg(P + f);
    const float den = fmaf(pl.x, g.u, fmaf(pl.y, g.v, pl.z * g.w));
    if (den > 0.0f) {
      const float num = pl.w - fmaf(pl.x, g.x, fmaf(pl.y, g.y, pl.z * g.z));
      const float t = __fdividef(num, den);
      if (t < t1) {
        t2 = t1;
        t1 = t;
        bf = f;
      } else if (t < t2) {
        t2 = t;
      }
    }
  }
  float L;
  if (bf < 0 || t2 - t1 <= tol || t1 < -tol) {
    ++n_fb;
    double Ld = 0.0;
    bf = exit_fp64(M, p.elem, p.fin, g, Ld);
    if (bf < 0) {
      p.status = kStuck;
      return 2;
    }
    L = (float)Ld;
  } else {
    L = fmaxf(t1, 0.0f);
  }
  // 32 high bits of the PCG output as the uniform deviate
  p.seed = kPrnMult * p.seed + kPrnAdd;
  uint64_t wv = ((p.seed >> ((p.seed >> 59u) + 5u)) ^ p.seed) * 12605985483714917081ULL;
  wv = (wv >> 43u) ^ wv;
  const float xi = (float)(uint32_t)(wv >> 32) * 2.3283064365386963e-10f;
  const float dist = -__logf(xi) * inv_sig;
  const bool cross = dist > L;
  const float score = cross ? L : dist;
  score_track(T, tally, p.elem, p.E, p.wgt * (double)score, p.sigt);
  if (kEig) p.ktl = p.ktl + p.wgt * widen(score) * p.nuf;
  ++p.n_seg;
  if (L == 0.0f) ++p.zero_run;
  else p.zero_run = 0;
  if (cross) {
    p.hash = fnv(p.hash, (uint64_t)p.elem * 8ULL + (uint64_t)bf);
    const float sx = g.x, sy = g.y, sz = g.z;
    g.x = fmaf(L, g.u, g.x);
    g.y = fmaf(L, g.v, g.y);
    g.z = fmaf(L, g.w, g.z);
    if (T.rays) record_ray(T, p, sx, sy, sz, g.x, g.y, g.z);
    const int nb = side_entry(nb4, bf);
    if (nb >= 0) {
      if (nb & kMatChange) p.mat = -2;
      p.elem = (nb & (kMatChange - 1)) >> 2;
      p.fin = nb & 3;
      return 0;
    }
    const int bid = -1 - nb;
    if (bid < M.n_bid && M.bc_type[bid] == 1) {
      const float4 pl = __ldg(P + bf);
      const float t2r = 2.0f * fmaf(g.u, pl.x, fmaf(g.v, pl.y, g.w * pl.z));
      g.u = fmaf(-t2r, pl.x, g.u);
      g.v = fmaf(-t2r, pl.y, g.v);
      g.w = fmaf(-t2r, pl.z, g.w);
      const float nrm = rsqrtf(fmaf(g.u, g.u, fmaf(g.v, g.v, g.w * g.w)));
      g.u *= nrm;
      g.v *= nrm;
      g.w *= nrm;
      p.fin = -1;
      return 0;
    }
    p.status = kLeaked;
    p.face = bf;
    return 2;
  }
  p.hash = fnv(p.hash, (uint64_t)p.elem * 8ULL + 4ULL);
  const float sx = g.x, sy = g.y, sz = g.z;
  g.x = fmaf(dist, g.u, g.x);
  g.y = fmaf(dist, g.v, g.y);
  g.z = fmaf(dist, g.w, g.z);
  ++p.n_coll;
  if (T.rays) record_ray(T, p, sx, sy, sz, g.x, g.y, g.z);
  p.zero_run = 0;
  return 1;
}

}  // namespace mc
