// mc_host.cpp -- host preprocessing of meshes and cross-section tables.
//
// Compiled with -ffp-contract=off: the face planes computed here are the
// ones both the device walk and its bit-exact checks depend on.
#include "mc_host.h"

#include <math.h>

#include <algorithm>
#include <thread>

#include "mc_core.cuh"

namespace mc {

namespace {

const int kFaceVtx[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};

struct FaceKey {
  int32_t a, b, c;
  int64_t side;
  bool operator<(const FaceKey& o) const {
    if (a != o.a) return a < o.a;
    if (b != o.b) return b < o.b;
    if (c != o.c) return c < o.c;
    return side < o.side;
  }
};

inline void sort3(int32_t* v) {
  if (v[0] > v[1]) std::swap(v[0], v[1]);
  if (v[1] > v[2]) std::swap(v[1], v[2]);
  if (v[0] > v[1]) std::swap(v[0], v[1]);
}

template <class F>
void parallel_for(int64_t n, F&& f) {
  unsigned nt = std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  if (nt > 32) nt = 32;
  if (n < 100000) nt = 1;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t) {
    int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
    th.emplace_back([lo, hi, &f] {
      for (int64_t i = lo; i < hi; ++i) f(i);
    });
  }
  for (auto& t : th) t.join();
}

}  // namespace

std::string build_mesh_tables(int64_t n_vtx, const double* xyz, int64_t n_tet,
                              const int32_t* tet_vtx, const int32_t* tet_block,
                              const int32_t* tet_side_bid, MeshTables& M) {
  if (n_vtx < 4 || n_tet < 1) return "empty mesh";
  if (n_tet > (int64_t)1 << 28) return "too many tets (limit 2^28)";
  for (int64_t i = 0; i < 4 * n_tet; ++i)
    if (tet_vtx[i] < 0 || tet_vtx[i] >= n_vtx) return "tet vertex index out of range";
  M.n_vtx = n_vtx;
  M.n_tet = n_tet;
  M.block.assign(tet_block, tet_block + n_tet);

  // adjacency: sort sides by their sorted vertex triple
  std::vector<FaceKey> keys((size_t)(4 * n_tet));
  parallel_for(n_tet, [&](int64_t t) {
    for (int f = 0; f < 4; ++f) {
      int32_t v[3] = {tet_vtx[4 * t + kFaceVtx[f][0]], tet_vtx[4 * t + kFaceVtx[f][1]],
                      tet_vtx[4 * t + kFaceVtx[f][2]]};
      sort3(v);
      keys[4 * t + f] = FaceKey{v[0], v[1], v[2], 4 * t + f};
    }
  });
  std::sort(keys.begin(), keys.end());
  M.nbr.assign((size_t)(4 * n_tet), 0);
  std::vector<uint8_t> has_nb((size_t)(4 * n_tet), 0);
  for (size_t i = 0; i < keys.size();) {
    size_t j = i + 1;
    while (j < keys.size() && keys[j].a == keys[i].a && keys[j].b == keys[i].b &&
           keys[j].c == keys[i].c)
      ++j;
    if (j - i > 2) return "non-manifold face shared by more than two tets";
    if (j - i == 2) {
      // neighbour id and the index of the shared side within the neighbour
      M.nbr[keys[i].side] = (int32_t)((keys[i + 1].side / 4) << 2 | (keys[i + 1].side % 4));
      M.nbr[keys[i + 1].side] = (int32_t)((keys[i].side / 4) << 2 | (keys[i].side % 4));
      has_nb[keys[i].side] = has_nb[keys[i + 1].side] = 1;
    }
    i = j;
  }
  std::vector<FaceKey>().swap(keys);
  for (int64_t s = 0; s < 4 * n_tet; ++s) {
    if (has_nb[s]) continue;
    int32_t bid = tet_side_bid ? tet_side_bid[s] : -1;
    if (bid < 0) bid = 0;
    M.nbr[s] = -1 - bid;
  }

  // canonical plane per distinct face, oriented outward for each tet
  M.planes.assign((size_t)(16 * n_tet), 0.0);
  M.planes32.assign((size_t)(16 * n_tet), 0.0f);
  std::vector<uint8_t> bad((size_t)n_tet, 0);
  parallel_for(n_tet, [&](int64_t t) {
    for (int f = 0; f < 4; ++f) {
      int32_t v[3] = {tet_vtx[4 * t + kFaceVtx[f][0]], tet_vtx[4 * t + kFaceVtx[f][1]],
                      tet_vtx[4 * t + kFaceVtx[f][2]]};
      sort3(v);
      const double* A = xyz + 3 * (int64_t)v[0];
      const double* B = xyz + 3 * (int64_t)v[1];
      const double* C = xyz + 3 * (int64_t)v[2];
      const double* O = xyz + 3 * (int64_t)tet_vtx[4 * t + f];
      const double e1x = B[0] - A[0], e1y = B[1] - A[1], e1z = B[2] - A[2];
      const double e2x = C[0] - A[0], e2y = C[1] - A[1], e2z = C[2] - A[2];
      double nx = e1y * e2z - e1z * e2y;
      double ny = e1z * e2x - e1x * e2z;
      double nz = e1x * e2y - e1y * e2x;
      const double len = sqrt(nx * nx + ny * ny + nz * nz);
      if (!(len > 0.0)) {
        bad[t] = 1;
        return;
      }
      nx = nx / len;
      ny = ny / len;
      nz = nz / len;
      double d = nx * A[0] + ny * A[1] + nz * A[2];
      const double s = nx * O[0] + ny * O[1] + nz * O[2] - d;
      if (s == 0.0) {
        bad[t] = 1;
        return;
      }
      if (s > 0.0) {
        nx = -nx;
        ny = -ny;
        nz = -nz;
        d = -d;
      }
      double* P = &M.planes[16 * t + 4 * f];
      P[0] = nx;
      P[1] = ny;
      P[2] = nz;
      P[3] = d;
      float* Q = &M.planes32[16 * t + 4 * f];
      Q[0] = (float)nx;
      Q[1] = (float)ny;
      Q[2] = (float)nz;
      Q[3] = (float)d;
    }
  });
  for (int64_t t = 0; t < n_tet; ++t)
    if (bad[t]) return "degenerate tet (zero-area face or zero volume) at index " + std::to_string(t);

  // locator grid
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int64_t v = 0; v < n_vtx; ++v)
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], xyz[3 * v + k]);
      hi[k] = std::max(hi[k], xyz[3 * v + k]);
    }
  double ext[3], vol = 1.0;
  for (int k = 0; k < 3; ++k) {
    M.bbox_lo[k] = lo[k];
    M.bbox_hi[k] = hi[k];
    ext[k] = hi[k] - lo[k];
    if (!(ext[k] > 0.0)) ext[k] = 1.0;
    vol *= ext[k];
  }
  // cells sized to the mean tet bounding-box extent along each axis (so a
  // tet overlaps a few cells whatever its aspect ratio), capped at 2^24 cells
  double mext[3] = {0.0, 0.0, 0.0};
  const int64_t stride_t = std::max<int64_t>(1, n_tet / 200000);
  int64_t n_s = 0;
  for (int64_t t = 0; t < n_tet; t += stride_t, ++n_s)
    for (int k = 0; k < 3; ++k) {
      double a = INFINITY, b = -INFINITY;
      for (int v = 0; v < 4; ++v) {
        const double c = xyz[3 * (int64_t)tet_vtx[4 * t + v] + k];
        a = std::min(a, c);
        b = std::max(b, c);
      }
      mext[k] += b - a;
    }
  for (int k = 0; k < 3; ++k) mext[k] = std::max(mext[k] / (double)std::max<int64_t>(n_s, 1), ext[k] * 1e-6);
  // finest cell scale (relative to the mean extent) whose list entries stay
  // within 12 per tet and whose cell count stays within 2^25
  int64_t ncell = 1;
  double scale = 1.0;
  for (double sc : {0.35, 0.5, 0.7, 1.0}) {
    double cells = 1.0, h[3];
    for (int k = 0; k < 3; ++k) {
      h[k] = ext[k] / std::max(1.0, std::min(4096.0, floor(ext[k] / (mext[k] * sc))));
      cells *= ext[k] / h[k];
    }
    double per = 0.0;
    int64_t ns = 0;
    for (int64_t t = 0; t < n_tet; t += stride_t, ++ns) {
      double c = 1.0;
      for (int k = 0; k < 3; ++k) {
        double a = INFINITY, b = -INFINITY;
        for (int vv = 0; vv < 4; ++vv) {
          const double x = xyz[3 * (int64_t)tet_vtx[4 * t + vv] + k];
          a = std::min(a, x);
          b = std::max(b, x);
        }
        c *= floor((b - lo[k]) / h[k]) - floor((a - lo[k]) / h[k]) + 1.0;
      }
      per += c;
    }
    per /= (double)std::max<int64_t>(ns, 1);
    if ((per <= 12.0 && cells <= 33554432.0) || sc == 1.0) {
      scale = sc;
      break;
    }
  }
  for (int k = 0; k < 3; ++k) {
    int n = (int)floor(ext[k] / (mext[k] * scale));
    n = std::max(1, std::min(n, 4096));
    M.gn[k] = n;
    M.glo[k] = lo[k];
    M.gh[k] = ext[k] / n;
    ncell *= n;
  }
  (void)vol;
  std::vector<int64_t> cnt((size_t)ncell + 1, 0);
  const double tol = kLocateTol;
  auto cell_range = [&](int64_t t, int* i0, int* i1) {
    double blo[3] = {INFINITY, INFINITY, INFINITY}, bhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int a = 0; a < 4; ++a)
      for (int k = 0; k < 3; ++k) {
        const double c = xyz[3 * (int64_t)tet_vtx[4 * t + a] + k];
        blo[k] = std::min(blo[k], c);
        bhi[k] = std::max(bhi[k], c);
      }
    for (int k = 0; k < 3; ++k) {
      int a = (int)floor((blo[k] - tol - M.glo[k]) / M.gh[k]);
      int b = (int)floor((bhi[k] + tol - M.glo[k]) / M.gh[k]);
      i0[k] = std::max(a, 0);
      i1[k] = std::min(b, M.gn[k] - 1);
    }
  };
  for (int64_t t = 0; t < n_tet; ++t) {
    int i0[3], i1[3];
    cell_range(t, i0, i1);
    for (int z = i0[2]; z <= i1[2]; ++z)
      for (int y = i0[1]; y <= i1[1]; ++y)
        for (int x = i0[0]; x <= i1[0]; ++x) cnt[((int64_t)z * M.gn[1] + y) * M.gn[0] + x]++;
  }
  M.gstart.assign((size_t)ncell + 1, 0);
  for (int64_t c = 0; c < ncell; ++c) M.gstart[c + 1] = M.gstart[c] + cnt[c];
  M.gtets.assign((size_t)std::max<int64_t>(1, M.gstart[ncell]), 0);
  std::vector<int64_t> fill(M.gstart.begin(), M.gstart.end() - 1);
  for (int64_t t = 0; t < n_tet; ++t) {
    int i0[3], i1[3];
    cell_range(t, i0, i1);
    for (int z = i0[2]; z <= i1[2]; ++z)
      for (int y = i0[1]; y <= i1[1]; ++y)
        for (int x = i0[0]; x <= i1[0]; ++x)
          M.gtets[fill[((int64_t)z * M.gn[1] + y) * M.gn[0] + x]++] = (int32_t)t;
  }
  // walk seeds: the first listed tet that contains the cell centre (within
  // the locate tolerance), found on the FP64 planes
  M.gseed.assign((size_t)ncell, -1);
  parallel_for(ncell, [&](int64_t c) {
    {
      const int64_t ix = c % M.gn[0], iy = (c / M.gn[0]) % M.gn[1], iz = c / ((int64_t)M.gn[0] * M.gn[1]);
      const double p[3] = {M.glo[0] + (ix + 0.5) * M.gh[0], M.glo[1] + (iy + 0.5) * M.gh[1],
                           M.glo[2] + (iz + 0.5) * M.gh[2]};
      for (int64_t q = M.gstart[c]; q < M.gstart[c + 1]; ++q) {
        const int32_t t = M.gtets[q];
        bool in = true;
        for (int f = 0; f < 4 && in; ++f) {
          const double* pl = &M.planes[16 * (size_t)t + 4 * f];
          if (pl[0] * p[0] + pl[1] * p[1] + pl[2] * p[2] - pl[3] > tol) in = false;
        }
        if (in) {
          M.gseed[c] = t;
          break;
        }
      }
    }
  });
  return "";
}

namespace {
int bucket_of(const XSTables& X, double lE) {
  const double q = (lE - X.lE_lo) / X.du;
  if (!(q >= 0.0)) return 0;
  if (q >= (double)X.n_bins) return X.n_bins - 1;
  int k = (int)q;
  if (k > X.n_bins - 1) k = X.n_bins - 1;
  return k;
}
}  // namespace

std::string build_xs_tables(const std::vector<Nuclide>& nucs, const std::vector<Material>& mats,
                            int32_t n_bins, XSTables& X) {
  if (nucs.empty()) return "no nuclides";
  if (mats.empty()) return "no materials";
  if (n_bins < 1) return "hash bins must be >= 1";
  double lo = -INFINITY, hi = INFINITY;
  for (const auto& n : nucs) {
    lo = std::max(lo, n.E.front());
    hi = std::min(hi, n.E.back());
  }
  if (!(hi > lo)) return "nuclide energy ranges do not overlap";
  X.n_bins = n_bins;
  X.E_lo = lo;
  X.E_hi = hi;
  X.lE_lo = mc::log64(lo);
  X.du = (mc::log64(hi) - X.lE_lo) / (double)n_bins;
  const int64_t nn = (int64_t)nucs.size();
  X.nuc_grid.assign(nn, -1);
  X.nuc_off.resize(nn);
  X.awr.resize(nn);
  X.gE.clear();
  X.g_off.clear();
  X.g_n.clear();
  X.sig.clear();
  std::vector<int64_t> rep;  // a nuclide holding each grid
  for (int64_t i = 0; i < nn; ++i) {
    const Nuclide& n = nucs[i];
    int g = -1;
    for (size_t r = 0; r < rep.size() && g < 0; ++r) {
      const Nuclide& o = nucs[rep[r]];
      if (o.E.size() == n.E.size() && std::equal(o.E.begin(), o.E.end(), n.E.begin())) g = (int)r;
    }
    if (g < 0) {
      g = (int)rep.size();
      rep.push_back(i);
      X.g_off.push_back((int64_t)X.gE.size());
      X.g_n.push_back((int32_t)n.E.size());
      X.gE.insert(X.gE.end(), n.E.begin(), n.E.end());
    }
    X.nuc_grid[i] = g;
    X.awr[i] = n.awr;
    X.nuc_off[i] = (int64_t)X.sig.size() / 2;
    for (size_t j = 0; j < n.E.size(); ++j) {
      X.sig.push_back(n.st[j]);
      X.sig.push_back(n.ss[j]);
    }
  }
  X.nuc_fiss.assign(nn, 0);
  X.nusf.clear();
  bool any_fiss = false;
  for (int64_t i = 0; i < nn; ++i) {
    if (!nucs[i].nusf.empty()) {
      if (nucs[i].nusf.size() != nucs[i].E.size()) return "fission data size differs from the nuclide's grid";
      X.nuc_fiss[i] = 1;
      any_fiss = true;
    }
  }
  if (any_fiss) {
    X.nusf.assign(X.sig.size() / 2, 0.0);
    for (int64_t i = 0; i < nn; ++i)
      if (X.nuc_fiss[i]) std::copy(nucs[i].nusf.begin(), nucs[i].nusf.end(), X.nusf.begin() + X.nuc_off[i]);
  }
  const int64_t ng = (int64_t)rep.size();
  X.ghidx.assign((size_t)(n_bins + 1) * ng, 0);
  for (int64_t g = 0; g < ng; ++g) {
    const double* E = X.gE.data() + X.g_off[g];
    const int64_t np = X.g_n[g];
    // ghidx[k] = (number of grid points in bins < k) - 1, clamped to [0, n-2]
    int64_t j = 0;
    for (int k = 0; k <= n_bins; ++k) {
      while (j < np && bucket_of(X, mc::log64(E[j])) < k) ++j;
      int64_t v = std::max<int64_t>(0, std::min<int64_t>(j - 1, np - 2));
      X.ghidx[(size_t)k * ng + g] = (int32_t)v;
    }
  }
  X.mat_off.assign(mats.size() + 1, 0);
  X.mat_nuc.clear();
  X.mat_dens.clear();
  X.mat_ids.clear();
  X.mat_fiss.assign(mats.size(), 0);
  for (size_t m = 0; m < mats.size(); ++m) {
    X.mat_ids.push_back(mats[m].id);
    for (size_t j = 0; j < mats[m].nuc.size(); ++j) {
      X.mat_nuc.push_back(mats[m].nuc[j]);
      X.mat_dens.push_back(mats[m].dens[j]);
      if (X.nuc_fiss[mats[m].nuc[j]]) X.mat_fiss[m] = 1;
    }
    X.mat_off[m + 1] = (int32_t)X.mat_nuc.size();
  }
  return "";
}

}  // namespace mc
