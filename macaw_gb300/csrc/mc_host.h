// mc_host.h -- host-side data model of the tracker context.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

namespace mc {

// Face adjacency, outward planes and start-point locator of a tet mesh, in
// the layouts the kernels read.  Side f of a tet is the face opposite its
// local vertex f.
struct MeshTables {
  int64_t n_vtx = 0, n_tet = 0;
  std::vector<double> planes;   // 16 per tet: (nx, ny, nz, d) per side
  std::vector<float> planes32;  // same, rounded to float
  std::vector<int32_t> nbr;     // 4 per tet: neighbour id << 2 | shared side in the neighbour,
                                // or -1-boundary_id
  std::vector<int32_t> block;   // subdomain id per tet
  // uniform-grid locator: cells hold ascending ids of tets whose bounding
  // box (grown by the locate tolerance) overlaps the cell
  double glo[3] = {0, 0, 0}, gh[3] = {1, 1, 1};
  int32_t gn[3] = {1, 1, 1};
  std::vector<int64_t> gstart;
  std::vector<int32_t> gtets;
  // per cell: a tet containing the cell's centre (-1: none), where a
  // locate's walk to the point starts
  std::vector<int32_t> gseed;
  double bbox_lo[3] = {0, 0, 0}, bbox_hi[3] = {0, 0, 0};
};

// Builds MeshTables; returns an empty string or an error message.
std::string build_mesh_tables(int64_t n_vtx, const double* xyz, int64_t n_tet,
                              const int32_t* tet_vtx, const int32_t* tet_block,
                              const int32_t* tet_side_bid, MeshTables& out);

struct Nuclide {
  std::vector<double> E, st, ss;
  std::vector<double> nusf;  // nu*sigma_f per point; empty: not fissionable
  double awr = 1.0;
};

struct Material {
  int32_t id = 0;
  std::vector<int32_t> nuc;
  std::vector<double> dens;
};

// Flattened cross-section tables in the layouts the kernels read.  Nuclides
// whose energy grids are identical share one stored grid (and so one hash
// search and one interpolation fraction per lookup).
struct XSTables {
  std::vector<double> gE;       // energies of the distinct grids, concatenated
  std::vector<int64_t> g_off;   // first point of each grid
  std::vector<int32_t> g_n;     // points per grid
  std::vector<int32_t> ghidx;   // (n_bins+1) x n_grid, bin-major
  std::vector<int32_t> nuc_grid;  // grid of each nuclide
  std::vector<int64_t> nuc_off;   // first (sigma_t, sigma_s) pair of each nuclide
  std::vector<double> sig;        // 2 per point: (sigma_t, sigma_s), nuclides concatenated
  std::vector<double> awr;
  std::vector<double> nusf;       // 1 per point, indexed like sig pairs; empty: nothing fissionable
  std::vector<int32_t> nuc_fiss;  // per nuclide: 1 fissionable
  std::vector<int32_t> mat_fiss;  // per material: 1 holds a fissionable nuclide
  std::vector<int32_t> mat_off; // n_mat+1
  std::vector<int32_t> mat_nuc;
  std::vector<double> mat_dens;
  std::vector<int32_t> mat_ids;
  int32_t n_bins = 8000;
  double E_lo = 0, E_hi = 0, lE_lo = 0, du = 0;
};

std::string build_xs_tables(const std::vector<Nuclide>& nucs, const std::vector<Material>& mats,
                            int32_t n_bins, XSTables& out);

}  // namespace mc
