// mc_gen.cpp -- synthetic meshes and cross-section tables.
//
// The reference's own inputs (BEAVRS meshes, ENDF data) are not available,
// so problems are generated from a seed.  Every value is produced with the
// tracker's own arithmetic (mc::exp/mc::log, IEEE sqrt and division, no
// fused multiply-add), so the same seed yields bit-identical tables on every
// host architecture.
#include <math.h>

#include <algorithm>
#include <map>
#include <utility>
#include <vector>

#include "../../include/macaw_gb300.h"
#include "mc_core.cuh"

namespace {

// Independent generator stream per (seed, purpose, index).
struct Gen {
  uint64_t s;
  Gen(uint64_t seed, uint64_t purpose, uint64_t index) {
    mc::Skip k = mc::skip_ahead((index + 1) * mc::kPrnStride);
    s = k.G * (seed + 101 * purpose + 7) + k.C;
  }
  double u() { return mc::prn(s); }
  double uniform(double lo, double hi) { return lo + u() * (hi - lo); }
  double log_uniform(double lo, double hi) {
    const double a = mc::log64(lo), b = mc::log64(hi);
    return mc::exp64(a + u() * (b - a));
  }
};

// ---------------------------------------------------------------------------
// Box of nx x ny x nz hexes, each split into the six Kuhn tets along its
// main diagonal (vertex (i,j,k) -> (i+1,j+1,k+1)): MOOSE's
// GeneratedMeshGenerator (dim = 3) with a tet split.  Every hex face is cut
// into two triangles along a diagonal that the neighbouring hex cuts the
// same way, so the tets conform.
int64_t box_vertex_index(int nx, int ny, int i, int j, int k) {
  return ((int64_t)k * (ny + 1) + j) * (nx + 1) + i;
}

// MOOSE GeneratedMesh 3D sideset ids: back=0 (z-), bottom=1 (y-), right=2
// (x+), top=3 (y+), left=4 (x-), front=5 (z+).
int box_side_id(const int* lo_hit, const int* hi_hit) {
  if (lo_hit[2]) return 0;
  if (lo_hit[1]) return 1;
  if (hi_hit[0]) return 2;
  if (hi_hit[1]) return 3;
  if (lo_hit[0]) return 4;
  if (hi_hit[2]) return 5;
  return -1;
}

const int kFaceVtx[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};

bool box_dims_ok(int32_t nx, int32_t ny, int32_t nz) {
  return nx >= 1 && ny >= 1 && nz >= 1 && nx <= 2000 && ny <= 2000 && nz <= 2000 &&
         (int64_t)6 * nx * ny * nz <= 2000000000LL;
}

}  // namespace

extern "C" int mc_gen_box_sizes(int32_t nx, int32_t ny, int32_t nz, int64_t* n_vtx, int64_t* n_tet) {
  if (!box_dims_ok(nx, ny, nz) || !n_vtx || !n_tet) return MC_ERR_ARG;
  *n_vtx = (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
  *n_tet = (int64_t)6 * nx * ny * nz;
  return MC_OK;
}

extern "C" int mc_gen_box(int32_t nx, int32_t ny, int32_t nz, const double* lo, const double* hi, double* xyz,
                          int32_t* tet_vtx, int32_t* tet_block, int32_t* tet_side_bid) {
  if (!box_dims_ok(nx, ny, nz) || !lo || !hi || !xyz || !tet_vtx || !tet_block) return MC_ERR_ARG;
  const int n[3] = {nx, ny, nz};
  double h[3];
  for (int a = 0; a < 3; ++a) {
    if (!(hi[a] > lo[a])) return MC_ERR_ARG;
    h[a] = (hi[a] - lo[a]) / n[a];
  }
  for (int k = 0; k <= nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        const int c[3] = {i, j, k};
        const int64_t v = box_vertex_index(nx, ny, i, j, k);
        // the last plane is the upper bound itself, not lo + n*h
        for (int a = 0; a < 3; ++a) xyz[3 * v + a] = (c[a] == n[a]) ? hi[a] : lo[a] + c[a] * h[a];
      }
  static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  int64_t t = 0;
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i)
        for (int p = 0; p < 6; ++p, ++t) {
          int cell[4][3] = {{i, j, k}};
          for (int s = 1; s < 4; ++s) {
            for (int a = 0; a < 3; ++a) cell[s][a] = cell[s - 1][a];
            cell[s][perms[p][s - 1]] += 1;
          }
          for (int s = 0; s < 4; ++s)
            tet_vtx[4 * t + s] = (int32_t)box_vertex_index(nx, ny, cell[s][0], cell[s][1], cell[s][2]);
          tet_block[t] = 0;
          if (tet_side_bid) {
            for (int f = 0; f < 4; ++f) {
              int lo_hit[3] = {1, 1, 1}, hi_hit[3] = {1, 1, 1};
              for (int q = 0; q < 3; ++q) {
                const int* v = cell[kFaceVtx[f][q]];
                for (int a = 0; a < 3; ++a) {
                  if (v[a] != 0) lo_hit[a] = 0;
                  if (v[a] != n[a]) hi_hit[a] = 0;
                }
              }
              tet_side_bid[4 * t + f] = box_side_id(lo_hit, hi_hit);
            }
          }
        }
  return MC_OK;
}

extern "C" int mc_gen_cube_sizes(int32_t n, int64_t* n_vtx, int64_t* n_tet) {
  if (n < 1 || n > 1000) return MC_ERR_ARG;
  return mc_gen_box_sizes(n, n, n, n_vtx, n_tet);
}

// The cube [0, L]^3 is the box with lower corner 0 (0 + i*h == i*h exactly,
// so the coordinates are those of the box generator bit for bit).
extern "C" int mc_gen_cube(int32_t n, double L, double* xyz, int32_t* tet_vtx, int32_t* tet_block,
                           int32_t* tet_side_bid) {
  if (n < 1 || n > 1000 || !(L > 0.0)) return MC_ERR_ARG;
  const double lo[3] = {0.0, 0.0, 0.0}, hi[3] = {L, L, L};
  return mc_gen_box(n, n, n, lo, hi, xyz, tet_vtx, tet_block, tet_side_bid);
}

// ---------------------------------------------------------------------------
// Pin-cell lattice.  Each square cell (pitch p) is triangulated in 2-D with
// a centre fan, n_fuel_rings rings inside r_fuel, one ring to r_clad and
// one ring out to the cell square, all on n_sec azimuthal sectors (n_sec a
// multiple of 8, so sector rays hit the cell corners).  Points on the cell
// square are placed by a per-edge formula so neighbouring cells produce
// bit-identical shared vertices.  The 2-D mesh is extruded into nz layers
// of prisms, each cut into three tets with every quad diagonal starting at
// the lower-layer vertex of the smaller 2-D id (a conforming split).
namespace {

struct Lattice2D {
  std::vector<double> x, y;
  std::vector<uint8_t> on_x0, on_x1, on_y0, on_y1;
  std::vector<int32_t> tri;  // 3 per triangle
  std::vector<int32_t> tri_block;
};

// Cell kinds of the 2-D mesh.
enum CellKind { kPinCell = 0, kFillCell = 1 };

// Cells of a square grid (pitch p, origin x0/y0), each a pin cell (fuel /
// clad / moderator blocks) or a fill cell (a fan from the centre to the
// same square points, so fill and pin cells conform).
struct CellSpec {
  int ci, cj, kind;
  int32_t fuel, clad, mod, fill;
};

int cells2d(const std::vector<CellSpec>& cells, int nx, int ny, double x0, double y0, int n_sec, int n_fr,
            double pitch, double r_fuel, double r_clad, Lattice2D& G) {
  if (n_sec < 8 || n_sec % 8 != 0 || n_fr < 1) return MC_ERR_ARG;
  if (!(r_fuel > 0.0) || !(r_clad > r_fuel) || !(pitch > 2.0 * r_clad)) return MC_ERR_ARG;
  const double twopi = 6.283185307179586;
  const int q = n_sec / 8;
  // cos/sin of the sector angles by Taylor series after reduction to
  // [-pi/4, pi/4] around the nearest multiple of pi/2 (exact at the axes).
  std::vector<double> cs(n_sec), sn(n_sec), tn(2 * q + 1);
  for (int k = 0; k < n_sec; ++k) {
    const double a = twopi * k / n_sec;
    const int quad = (k + q) / (2 * q);  // nearest multiple of pi/2
    const int oct = quad % 4;
    const double r = a - quad * (twopi / 4.0);
    double c = 0.0, s = 0.0, term_c = 1.0, term_s = r;
    for (int m = 0; m < 12; ++m) {
      c += term_c;
      s += term_s;
      term_c = -term_c * r * r / ((2.0 * m + 1.0) * (2.0 * m + 2.0));
      term_s = -term_s * r * r / ((2.0 * m + 2.0) * (2.0 * m + 3.0));
    }
    if (k % (2 * q) == 0) {
      c = 1.0;
      s = 0.0;
    }
    double C, S;
    switch (oct) {
      case 0: C = c; S = s; break;
      case 1: C = -s; S = c; break;
      case 2: C = -c; S = -s; break;
      default: C = s; S = -c; break;
    }
    cs[k] = C;
    sn[k] = S;
  }
  for (int m = 0; m <= q; ++m) {
    // tan of m/q * 45 degrees, from the sector cos/sin
    tn[q + m] = (m == q) ? 1.0 : sn[m] / cs[m];
    tn[q - m] = -tn[q + m];
  }
  std::map<std::pair<uint64_t, uint64_t>, int32_t> shared;
  auto add_pt = [&](double x, double y, bool dedup, int fx0, int fx1, int fy0, int fy1) -> int32_t {
    if (dedup) {
      auto key = std::make_pair(mc::dbits(x), mc::dbits(y));
      auto it = shared.find(key);
      if (it != shared.end()) return it->second;
      shared[key] = (int32_t)G.x.size();
    }
    G.x.push_back(x);
    G.y.push_back(y);
    G.on_x0.push_back((uint8_t)fx0);
    G.on_x1.push_back((uint8_t)fx1);
    G.on_y0.push_back((uint8_t)fy0);
    G.on_y1.push_back((uint8_t)fy1);
    return (int32_t)G.x.size() - 1;
  };
  auto tri = [&](int32_t a, int32_t b, int32_t c, int32_t blk) {
    G.tri.push_back(a);
    G.tri.push_back(b);
    G.tri.push_back(c);
    G.tri_block.push_back(blk);
  };
  const double h = pitch * 0.5;
  const int n_rings = n_fr + 1;  // fuel rings + clad ring
  std::vector<int32_t> ring((size_t)n_rings * n_sec), sq(n_sec);
  for (const CellSpec& cell : cells) {
      const int ci = cell.ci, cj = cell.cj;
      const double X0 = x0 + ci * pitch, X1 = x0 + (ci + 1) * pitch, Y0 = y0 + cj * pitch,
                   Y1 = y0 + (cj + 1) * pitch;
      const double cx = (X0 + X1) * 0.5, cy = (Y0 + Y1) * 0.5;
      const int32_t ctr = add_pt(cx, cy, false, 0, 0, 0, 0);
      for (int r = 0; r < n_rings && cell.kind == kPinCell; ++r) {
        const double rad = (r < n_fr) ? r_fuel * (r + 1) / n_fr : r_clad;
        for (int k = 0; k < n_sec; ++k) ring[(size_t)r * n_sec + k] = add_pt(cx + rad * cs[k], cy + rad * sn[k], false, 0, 0, 0, 0);
      }
      for (int k = 0; k < n_sec; ++k) {
        double x, y;
        if (k == q) { x = X1; y = Y1; }
        else if (k == 3 * q) { x = X0; y = Y1; }
        else if (k == 5 * q) { x = X0; y = Y0; }
        else if (k == 7 * q) { x = X1; y = Y0; }
        else if (k < q || k > 7 * q) { x = X1; y = cy + h * tn[q + (k < q ? k : k - n_sec)]; }
        else if (k < 3 * q) { x = cx + h * tn[q + 2 * q - k]; y = Y1; }
        else if (k < 5 * q) { x = X0; y = cy + h * tn[q + 4 * q - k]; }
        else { x = cx + h * tn[q + k - 6 * q]; y = Y0; }
        const int fx0 = (x == X0 && ci == 0), fx1 = (x == X1 && ci == nx - 1);
        const int fy0 = (y == Y0 && cj == 0), fy1 = (y == Y1 && cj == ny - 1);
        sq[k] = add_pt(x, y, true, fx0, fx1, fy0, fy1);
      }
      if (cell.kind == kFillCell) {
        for (int k = 0; k < n_sec; ++k) tri(ctr, sq[k], sq[(k + 1) % n_sec], cell.fill);
        continue;
      }
      for (int k = 0; k < n_sec; ++k) {
        const int k1 = (k + 1) % n_sec;
        tri(ctr, ring[k], ring[k1], cell.fuel);
        for (int r = 0; r + 1 < n_rings; ++r) {
          const int32_t a = ring[(size_t)r * n_sec + k], b = ring[(size_t)r * n_sec + k1];
          const int32_t c = ring[(size_t)(r + 1) * n_sec + k1], d = ring[(size_t)(r + 1) * n_sec + k];
          const int32_t blk = (r + 1 < n_fr) ? cell.fuel : cell.clad;
          tri(a, b, c, blk);
          tri(a, c, d, blk);
        }
        const int32_t a = ring[(size_t)(n_rings - 1) * n_sec + k], b = ring[(size_t)(n_rings - 1) * n_sec + k1];
        tri(a, b, sq[k1], cell.mod);
        tri(a, sq[k1], sq[k], cell.mod);
      }
    }
  return MC_OK;
}

int lattice2d(int nx, int ny, int n_sec, int n_fr, double pitch, double r_fuel, double r_clad, Lattice2D& G) {
  if (nx < 1 || ny < 1) return MC_ERR_ARG;
  std::vector<CellSpec> cells;
  for (int cj = 0; cj < ny; ++cj)
    for (int ci = 0; ci < nx; ++ci) cells.push_back(CellSpec{ci, cj, kPinCell, 1, 2, 3, 0});
  return cells2d(cells, nx, ny, 0.0, 0.0, n_sec, n_fr, pitch, r_fuel, r_clad, G);
}

// Core map of 193 assemblies: rows of 7, 11, 13, 13, 15 (x7), 13, 13, 11, 7
// centred on a 15x15 assembly grid.
const int kCoreRows[15] = {7, 11, 13, 13, 15, 15, 15, 15, 15, 15, 15, 13, 13, 11, 7};

int core2d(int pins, int n_sec, int n_fr, double pitch, double r_fuel, double r_clad, double radius, Lattice2D& G,
           std::vector<double>* pin_xy) {
  if (pins < 1 || !(radius > 0.0) || !(pitch > 0.0)) return MC_ERR_ARG;
  const int na = 15;
  // margin of reflector cells around the assembly square, out to the radius
  const double half_core = 0.5 * na * pins * pitch;
  const int m = radius > half_core ? (int)ceil((radius - half_core) / pitch) : 0;
  const int n = na * pins + 2 * m;
  if ((int64_t)n * n > ((int64_t)1 << 26)) return MC_ERR_ARG;
  const double x0 = -0.5 * n * pitch;
  std::vector<int> assembly((size_t)na * na, -1);
  int a = 0;
  for (int r = 0; r < na; ++r) {
    const int w = kCoreRows[r], c0 = (na - w) / 2;
    for (int c = c0; c < c0 + w; ++c) assembly[(size_t)r * na + c] = a++;
  }
  std::vector<CellSpec> cells;
  for (int cj = 0; cj < n; ++cj)
    for (int ci = 0; ci < n; ++ci) {
      const int ai = ci - m, aj = cj - m;
      const int as = (ai >= 0 && aj >= 0 && ai < na * pins && aj < na * pins)
                         ? assembly[(size_t)(aj / pins) * na + ai / pins]
                         : -1;
      const double cx = x0 + (ci + 0.5) * pitch, cy = x0 + (cj + 0.5) * pitch;
      if (as >= 0) {
        cells.push_back(CellSpec{ci, cj, kPinCell, 1 + as, 194, 195, 0});
        if (pin_xy) {
          pin_xy->push_back(cx);
          pin_xy->push_back(cy);
        }
        continue;
      }
      // reflector: whole cells inside the radius, five 72-degree sectors
      bool inside = true;
      for (int k = 0; k < 4; ++k) {
        const double px = x0 + (ci + (k & 1)) * pitch, py = x0 + (cj + (k >> 1)) * pitch;
        if (px * px + py * py > radius * radius) inside = false;
      }
      if (!inside) continue;
      // sector from the cell centre's quadrant and slope (no atan): 0..4
      double ang = 0.0;  // a monotone stand-in for angle / (pi/2), in [0, 4)
      const double ax = fabs(cx), ay = fabs(cy);
      const double t = ax >= ay ? (ax > 0.0 ? ay / ax : 0.0) * 0.5 : 1.0 - (ay > 0.0 ? ax / ay : 0.0) * 0.5;
      if (cx >= 0 && cy >= 0) ang = t;
      else if (cx < 0 && cy >= 0) ang = 2.0 - t;
      else if (cx < 0) ang = 2.0 + t;
      else ang = 4.0 - t;
      int sector = (int)(ang * 5.0 / 4.0);
      if (sector > 4) sector = 4;
      cells.push_back(CellSpec{ci, cj, kFillCell, 0, 0, 0, 196 + sector});
    }
  return cells2d(cells, n, n, x0, x0, n_sec, n_fr, pitch, r_fuel, r_clad, G);
}

}  // namespace

extern "C" int mc_gen_lattice_sizes(int32_t nx, int32_t ny, int32_t nz, int32_t n_sec, int32_t n_fr,
                                    int64_t* n_vtx, int64_t* n_tet) {
  Lattice2D G;
  if (nz < 1) return MC_ERR_ARG;
  int rc = lattice2d(nx, ny, n_sec, n_fr, 1.26, 0.41, 0.475, G);
  if (rc) return rc;
  *n_vtx = (int64_t)G.x.size() * (nz + 1);
  *n_tet = (int64_t)G.tri_block.size() * nz * 3;
  return MC_OK;
}

namespace {

// Extrudes the 2-D mesh into nz layers of prisms over [0, height], three
// conforming tets per prism; sidesets from the box-side flags of the 2-D
// points and the bottom/top layers (back = 0, front = 5).  With radial_id
// >= 0 the x/y box sides are not used: every face off the two z planes gets
// radial_id (only faces without a neighbour ever read it).
void extrude(const Lattice2D& G, int nz, double height, double* xyz, int32_t* tet_vtx, int32_t* tet_block,
             int32_t* tet_side_bid, int radial_id = -1) {
  const int64_t n2 = (int64_t)G.x.size();
  for (int l = 0; l <= nz; ++l) {
    const double z = (l == nz) ? height : height * l / nz;
    for (int64_t v = 0; v < n2; ++v) {
      const int64_t id = (int64_t)l * n2 + v;
      xyz[3 * id] = G.x[v];
      xyz[3 * id + 1] = G.y[v];
      xyz[3 * id + 2] = z;
    }
  }
  const int64_t nt2 = (int64_t)G.tri_block.size();
  int64_t t = 0;
  for (int l = 0; l < nz; ++l)
    for (int64_t f = 0; f < nt2; ++f) {
      int32_t v[3] = {G.tri[3 * f], G.tri[3 * f + 1], G.tri[3 * f + 2]};
      std::sort(v, v + 3);
      const int32_t a0 = (int32_t)(l * n2 + v[0]), b0 = (int32_t)(l * n2 + v[1]), c0 = (int32_t)(l * n2 + v[2]);
      const int32_t a1 = (int32_t)((l + 1) * n2 + v[0]), b1 = (int32_t)((l + 1) * n2 + v[1]),
                    c1 = (int32_t)((l + 1) * n2 + v[2]);
      const int32_t tets[3][4] = {{a0, b0, c0, c1}, {a0, b0, b1, c1}, {a0, a1, b1, c1}};
      for (int s = 0; s < 3; ++s, ++t) {
        for (int a = 0; a < 4; ++a) tet_vtx[4 * t + a] = tets[s][a];
        tet_block[t] = G.tri_block[f];
        if (tet_side_bid) {
          for (int fc = 0; fc < 4; ++fc) {
            int lo_hit[3] = {1, 1, 1}, hi_hit[3] = {1, 1, 1};
            for (int qv = 0; qv < 3; ++qv) {
              const int32_t g = tets[s][kFaceVtx[fc][qv]];
              const int64_t g2 = g % n2;
              const int64_t lay = g / n2;
              if (!G.on_x0[g2]) lo_hit[0] = 0;
              if (!G.on_x1[g2]) hi_hit[0] = 0;
              if (!G.on_y0[g2]) lo_hit[1] = 0;
              if (!G.on_y1[g2]) hi_hit[1] = 0;
              if (lay != 0) lo_hit[2] = 0;
              if (lay != nz) hi_hit[2] = 0;
            }
            if (radial_id >= 0) {
              lo_hit[0] = lo_hit[1] = hi_hit[0] = hi_hit[1] = 0;
              const int id = box_side_id(lo_hit, hi_hit);
              tet_side_bid[4 * t + fc] = id >= 0 ? id : radial_id;
            } else {
              tet_side_bid[4 * t + fc] = box_side_id(lo_hit, hi_hit);
            }
          }
        }
      }
    }
}

}  // namespace

extern "C" int mc_gen_lattice(int32_t nx, int32_t ny, int32_t nz, int32_t n_sec, int32_t n_fr,
                              double pitch, double height, double r_fuel, double r_clad,
                              double* xyz, int32_t* tet_vtx, int32_t* tet_block,
                              int32_t* tet_side_bid) {
  Lattice2D G;
  if (nz < 1 || !(height > 0.0)) return MC_ERR_ARG;
  int rc = lattice2d(nx, ny, n_sec, n_fr, pitch, r_fuel, r_clad, G);
  if (rc) return rc;
  extrude(G, nz, height, xyz, tet_vtx, tet_block, tet_side_bid);
  return MC_OK;
}

extern "C" int mc_gen_core_sizes(int32_t pins, int32_t nz, int32_t n_sec, int32_t n_fr, double pitch,
                                 double radius, int64_t* n_vtx, int64_t* n_tet, int64_t* n_pins) {
  Lattice2D G;
  std::vector<double> xy;
  if (nz < 1) return MC_ERR_ARG;
  int rc = core2d(pins, n_sec, n_fr, pitch, 0.41 * pitch / 1.26, 0.475 * pitch / 1.26, radius, G, &xy);
  if (rc) return rc;
  *n_vtx = (int64_t)G.x.size() * (nz + 1);
  *n_tet = (int64_t)G.tri_block.size() * nz * 3;
  *n_pins = (int64_t)xy.size() / 2;
  if ((int64_t)G.x.size() * (nz + 1) > ((int64_t)1 << 31) - 1) return MC_ERR_ARG;
  return MC_OK;
}

extern "C" int mc_gen_core(int32_t pins, int32_t nz, int32_t n_sec, int32_t n_fr, double pitch, double height,
                           double r_fuel, double r_clad, double radius, double* xyz, int32_t* tet_vtx,
                           int32_t* tet_block, int32_t* tet_side_bid, double* pin_xy) {
  Lattice2D G;
  std::vector<double> xy;
  if (nz < 1 || !(height > 0.0)) return MC_ERR_ARG;
  int rc = core2d(pins, n_sec, n_fr, pitch, r_fuel, r_clad, radius, G, &xy);
  if (rc) return rc;
  extrude(G, nz, height, xyz, tet_vtx, tet_block, tet_side_bid, 6);
  if (pin_xy) std::copy(xy.begin(), xy.end(), pin_xy);
  return MC_OK;
}

// ---------------------------------------------------------------------------
// Synthetic nuclide: log-uniform grid, 1/sqrt(E) background with amplitude
// U[1,10] b, n_peaks Lorentzians (centres log-U[1 eV, 100 keV], full widths
// log-U[1e-3, 1e-1] x centre, heights U[10, 1000] b), constant scatter
// fraction U[0.5, 0.99], target mass ratio U[1, 240].
extern "C" int mc_gen_nuclide(uint64_t seed, int32_t index, int64_t n_pts, double E_min,
                              double E_max, int32_t n_peaks, double* E, double* sig_t,
                              double* sig_s, double* awr) {
  if (n_pts < 2 || !(E_min > 0.0) || !(E_max > E_min) || n_peaks < 0) return MC_ERR_ARG;
  Gen g(seed, 1, (uint64_t)index);
  const double amp = g.uniform(1.0, 10.0);
  std::vector<double> ec(n_peaks), hw(n_peaks), ht(n_peaks);
  for (int p = 0; p < n_peaks; ++p) {
    ec[p] = g.log_uniform(1.0, 1.0e5);
    hw[p] = 0.5 * g.log_uniform(1.0e-3, 1.0e-1) * ec[p];
    ht[p] = g.uniform(10.0, 1000.0);
  }
  const double fs = g.uniform(0.5, 0.99);
  *awr = g.uniform(1.0, 240.0);
  const double la = mc::log64(E_min), lb = mc::log64(E_max);
  for (int64_t k = 0; k < n_pts; ++k) {
    double e;
    if (k == 0) e = E_min;
    else if (k == n_pts - 1) e = E_max;
    else e = mc::exp64(la + (lb - la) * ((double)k / (double)(n_pts - 1)));
    E[k] = e;
  }
  for (int64_t k = 1; k < n_pts; ++k)
    if (!(E[k] > E[k - 1])) return MC_ERR_ARG;
  for (int64_t k = 0; k < n_pts; ++k) {
    const double e = E[k];
    double s = amp / sqrt(e);
    for (int p = 0; p < n_peaks; ++p) {
      const double z = (e - ec[p]) / hw[p];
      s = s + ht[p] / (1.0 + z * z);
    }
    sig_t[k] = s;
    sig_s[k] = fs * s;
  }
  return MC_OK;
}

extern "C" int mc_gen_densities(uint64_t seed, int32_t index, int32_t n, double lo, double hi,
                                double* out) {
  if (n < 0 || !(hi >= lo)) return MC_ERR_ARG;
  Gen g(seed, 2, (uint64_t)index);
  for (int i = 0; i < n; ++i) out[i] = g.uniform(lo, hi);
  return MC_OK;
}
