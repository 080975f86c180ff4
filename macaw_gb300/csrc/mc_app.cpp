// mc_app.cpp -- input-file front end: MaCaw's HIT blocks mapped onto the C ABI.
//
// A MaCaw input (test/tests/study/openmc_study.i, examples/*/…i) declares
// the tracking problem as MOOSE objects: a CollisionKernel in
// [RayKernels], ReflectRayBC/KillRayBC in [RayBCs], an OpenMCStudy and
// OpenMCTally in [UserObjects], an OpenMCTallyAux in [AuxKernels], and a
// Transient executioner whose steps are the batches (OpenMCStudy.C:199-203).
// This file parses that block syntax (a subset of HIT: nested [name] ... []
// blocks, key = value, quoted lists, # comments, and [a/b] path headers),
// builds the registered objects by their `type`, checks their parameters
// the way their validParams/constructors do, and drives one context through
// the batches.  OpenMC's XML inputs are replaced by the synthetic-data and
// source parameters listed with each object below.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <chrono>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/macaw_gb300.h"

namespace {

struct InputError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// ---------------------------------------------------------------------------
// HIT subset parser.
struct Block {
  std::string name, path;
  std::map<std::string, std::string> params;
  std::vector<std::string> order;  // parameter insertion order
  std::vector<Block> children;
  Block* child(const std::string& n) {
    for (auto& c : children)
      if (c.name == n) return &c;
    return nullptr;
  }
};

std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? "" : s.substr(a, b - a + 1);
}

std::string strip_comment(const std::string& line) {
  bool q1 = false, q2 = false;
  for (size_t i = 0; i < line.size(); ++i) {
    const char c = line[i];
    if (c == '\'' && !q2) q1 = !q1;
    else if (c == '"' && !q1) q2 = !q2;
    else if (c == '#' && !q1 && !q2) return line.substr(0, i);
  }
  return line;
}

std::string unquote(const std::string& v) {
  std::string t = trim(v);
  if (t.size() >= 2 && ((t.front() == '\'' && t.back() == '\'') || (t.front() == '"' && t.back() == '"')))
    return t.substr(1, t.size() - 2);
  return t;
}

Block parse_hit(const std::string& text) {
  Block root;
  root.name = "";
  std::vector<Block*> stack{&root};
  std::vector<int> depth_of;  // how many path components each open header pushed
  std::istringstream in(text);
  std::string raw;
  int lineno = 0;
  std::string pending_key, pending_val;
  bool in_quote = false;
  char quote = 0;
  while (std::getline(in, raw)) {
    ++lineno;
    std::string line = in_quote ? raw : trim(strip_comment(raw));
    if (in_quote) {  // continuation of a multi-line quoted value
      pending_val += " " + trim(raw);
      if (raw.find(quote) != std::string::npos) {
        in_quote = false;
        stack.back()->params[pending_key] = unquote(trim(pending_val));
        stack.back()->order.push_back(pending_key);
      }
      continue;
    }
    if (line.empty()) continue;
    if (line.front() == '[') {
      const size_t close = line.find(']');
      if (close == std::string::npos)
        throw InputError("line " + std::to_string(lineno) + ": unterminated block header");
      std::string hdr = trim(line.substr(1, close - 1));
      if (hdr.empty() || hdr == "../" || hdr == "..") {
        if (depth_of.empty()) throw InputError("line " + std::to_string(lineno) + ": unmatched []");
        for (int k = depth_of.back(); k > 0; --k) stack.pop_back();
        depth_of.pop_back();
        continue;
      }
      if (hdr.rfind("./", 0) == 0) hdr = hdr.substr(2);
      int pushed = 0;
      size_t pos = 0;
      while (pos <= hdr.size()) {
        size_t slash = hdr.find('/', pos);
        std::string part = hdr.substr(pos, slash == std::string::npos ? std::string::npos : slash - pos);
        if (!part.empty()) {
          Block* parent = stack.back();
          Block* c = parent->child(part);
          if (!c) {
            Block nb;
            nb.name = part;
            nb.path = parent->path.empty() ? part : parent->path + "/" + part;
            parent->children.push_back(nb);
            c = &parent->children.back();
          }
          stack.push_back(c);
          ++pushed;
        }
        if (slash == std::string::npos) break;
        pos = slash + 1;
      }
      depth_of.push_back(pushed);
      // text after the header on the same line ([block] type = X ... [])
      std::string rest = trim(line.substr(close + 1));
      if (!rest.empty()) throw InputError("line " + std::to_string(lineno) + ": put parameters on their own lines");
      continue;
    }
    const size_t eq = line.find('=');
    if (eq == std::string::npos) throw InputError("line " + std::to_string(lineno) + ": expected key = value");
    const std::string key = trim(line.substr(0, eq));
    std::string val = trim(line.substr(eq + 1));
    if (stack.size() == 1) throw InputError("line " + std::to_string(lineno) + ": parameter outside a block");
    if (!val.empty() && (val.front() == '\'' || val.front() == '"')) {
      const char q = val.front();
      if (val.size() == 1 || val.find(q, 1) == std::string::npos) {
        in_quote = true;
        quote = q;
        pending_key = key;
        pending_val = val;
        continue;
      }
    }
    stack.back()->params[key] = unquote(val);
    stack.back()->order.push_back(key);
  }
  if (in_quote) throw InputError("unterminated quoted value for '" + pending_key + "'");
  if (!depth_of.empty()) throw InputError("unterminated block (missing [])");
  return root;
}

// ---------------------------------------------------------------------------
// Parameters with the checks validParams would make.
struct Params {
  const Block* b;
  std::map<std::string, bool> used;
  explicit Params(const Block* blk) : b(blk) {}
  bool has(const std::string& k) const { return b->params.count(k) > 0; }
  std::string raw(const std::string& k) {
    used[k] = true;
    return b->params.at(k);
  }
  [[noreturn]] void error(const std::string& k, const std::string& msg) const {
    throw InputError(b->path + "/" + k + ": " + msg);
  }
  std::string str(const std::string& k, const std::string& def = "\x01") {
    if (!has(k)) {
      if (def == "\x01") error(k, "missing required parameter");
      return def;
    }
    return raw(k);
  }
  double real(const std::string& k, double def = NAN, bool required = false) {
    if (!has(k)) {
      if (required) error(k, "missing required parameter");
      return def;
    }
    const std::string v = raw(k);
    char* end = nullptr;
    const double x = strtod(v.c_str(), &end);
    if (end == v.c_str() || *end) error(k, "expected a number, got '" + v + "'");
    return x;
  }
  long long integer(const std::string& k, long long def = 0, bool required = false) {
    if (!has(k)) {
      if (required) error(k, "missing required parameter");
      return def;
    }
    const std::string v = raw(k);
    char* end = nullptr;
    const double x = strtod(v.c_str(), &end);
    if (end == v.c_str() || *end || x != floor(x)) error(k, "expected an integer, got '" + v + "'");
    return (long long)x;
  }
  bool boolean(const std::string& k, bool def) {
    if (!has(k)) return def;
    const std::string v = raw(k);
    if (v == "true" || v == "1") return true;
    if (v == "false" || v == "0") return false;
    error(k, "expected true or false");
  }
  std::vector<std::string> list(const std::string& k, bool required = false) {
    std::vector<std::string> out;
    if (!has(k)) {
      if (required) error(k, "missing required parameter");
      return out;
    }
    std::istringstream s(raw(k));
    std::string w;
    while (s >> w) out.push_back(w);
    return out;
  }
  std::vector<double> reals(const std::string& k, bool required = false) {
    std::vector<double> out;
    for (auto& w : list(k, required)) {
      char* end = nullptr;
      const double x = strtod(w.c_str(), &end);
      if (end == w.c_str() || *end) error(k, "expected numbers, got '" + w + "'");
      out.push_back(x);
    }
    return out;
  }
  std::vector<int> ints(const std::string& k, bool required = false) {
    std::vector<int> out;
    for (double x : reals(k, required)) {
      if (x != floor(x)) error(k, "expected integers");
      out.push_back((int)x);
    }
    return out;
  }
  std::string choice(const std::string& k, const std::vector<std::string>& opts, const std::string& def) {
    std::string v = has(k) ? raw(k) : def;
    for (auto& o : opts)
      if (o == v) return v;
    std::string all;
    for (auto& o : opts) all += (all.empty() ? "" : " ") + o;
    error(k, "'" + v + "' is not one of: " + all);
  }
};

// ---------------------------------------------------------------------------
// The problem being assembled.
struct Problem {
  // mesh
  std::vector<double> xyz;
  std::vector<int32_t> tv, blk, bid;
  int64_t n_vtx = 0, n_tet = 0;
  std::vector<double> cyl_xy;  // pin centres for a cylinder source (lattice meshes)
  double cyl_r = 0.0, height = 0.0, lattice_pitch = 0.0;
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  // boundaries: id -> type
  std::map<int, int> bcs;
  // block map
  std::vector<int32_t> blocks, materials;
  bool have_kernel = false;
  // data
  struct Nuc {
    std::vector<double> E, st, ss;
    std::vector<double> nusf;  // nu*sigma_f; empty: not fissionable
    double awr;
  };
  std::vector<Nuc> nucs;
  struct Mat {
    int id;
    std::vector<int32_t> nuc;
    std::vector<double> dens;
  };
  std::vector<Mat> mats;
  // study
  int64_t particles = 0, bank_size = 0;
  // OpenMC settings run_mode eigenvalue: generations = batches, the first
  // `inactive` of them score no tally
  bool eigen = false;
  int64_t inactive = 0;
  uint64_t seed = 1;
  int precision = MC_PREC_FP64, mode = MC_MODE_EVENT;
  mc_source_desc src{};
  bool have_study = false, verbose = false;
  // tallies
  struct Tally {
    int id;
    std::string filter;  // cell | universe
    int estimator;       // MC_EST_*
    std::vector<int> scores;
    std::vector<double> edges;  // energy filter edges, empty: none
  };
  std::vector<Tally> tallies;
  struct Aux {
    std::string name, variable, granularity;
    int tally_id;
    int score;       // MC_SCORE_*
    int energy_bin;  // -1: summed over the energy bins
  };
  std::vector<Aux> aux;
  int64_t batches = 1;
  std::string file_base;
  bool csv = false, exodus = false;
  bool two_d = false;
  double z2d = 0.0;
  // RayTracingExodus output: rays of the last batch, segments per ray
  bool rays = false;
  std::string rays_name;
  int32_t rays_n = 0, rays_cap = 0;
};

const std::map<std::string, int> kSideNames = {{"back", 0}, {"bottom", 1}, {"right", 2},
                                                 {"top", 3},  {"left", 4},   {"front", 5}};

using Factory = std::function<void(Params&, Problem&)>;

// --- [Mesh] generators ------------------------------------------------------
void tet_cube_mesh(Params& p, Problem& P) {
  const int n = (int)p.integer("n", 20);
  const double L = p.real("length", 20.0);
  if (n < 1) p.error("n", "must be positive");
  if (!(L > 0)) p.error("length", "must be positive");
  if (mc_gen_cube_sizes(n, &P.n_vtx, &P.n_tet)) p.error("n", "invalid size");
  P.xyz.resize(3 * P.n_vtx);
  P.tv.resize(4 * P.n_tet);
  P.blk.resize(P.n_tet);
  P.bid.resize(4 * P.n_tet);
  mc_gen_cube(n, L, P.xyz.data(), P.tv.data(), P.blk.data(), P.bid.data());
  const int block_id = (int)p.integer("block_id", 0);
  for (auto& b : P.blk) b = block_id;
  for (int k = 0; k < 3; ++k) {
    P.lo[k] = 0.0;
    P.hi[k] = L;
  }
}

void tet_lattice_mesh(Params& p, Problem& P) {
  const int nx = (int)p.integer("nx", 17), ny = (int)p.integer("ny", 17), nz = (int)p.integer("nz", 21);
  const int n_sec = (int)p.integer("sectors", 16), n_fr = (int)p.integer("fuel_rings", 2);
  const double pitch = p.real("pitch", 1.26), height = p.real("height", 50.0);
  const double r_fuel = p.real("fuel_radius", 0.41), r_clad = p.real("clad_radius", 0.475);
  if (mc_gen_lattice_sizes(nx, ny, nz, n_sec, n_fr, &P.n_vtx, &P.n_tet))
    p.error("sectors", "invalid lattice (nx, ny, nz >= 1, sectors a multiple of 8, fuel_rings >= 1)");
  P.xyz.resize(3 * P.n_vtx);
  P.tv.resize(4 * P.n_tet);
  P.blk.resize(P.n_tet);
  P.bid.resize(4 * P.n_tet);
  if (mc_gen_lattice(nx, ny, nz, n_sec, n_fr, pitch, height, r_fuel, r_clad, P.xyz.data(), P.tv.data(),
                     P.blk.data(), P.bid.data()))
    p.error("pitch", "invalid lattice geometry (need pitch > 2 clad_radius > 2 fuel_radius > 0)");
  P.cyl_xy.clear();
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      P.cyl_xy.push_back((i + 0.5) * pitch);
      P.cyl_xy.push_back((j + 0.5) * pitch);
    }
  P.cyl_r = r_fuel;
  P.height = height;
  P.lattice_pitch = pitch;
  P.lo[0] = P.lo[1] = P.lo[2] = 0.0;
  P.hi[0] = nx * pitch;
  P.hi[1] = ny * pitch;
  P.hi[2] = height;
}

// MOOSE FileMeshGenerator: a tet mesh from an Exodus II file (path relative
// to the working directory); blocks and side sets from the file.
void file_mesh(Params& p, Problem& P) {
  const std::string file = p.str("file");
  char err[512] = {0};
  if (mc_exodus_read_sizes(file.c_str(), &P.n_vtx, &P.n_tet, err, sizeof err)) p.error("file", err);
  P.xyz.resize(3 * P.n_vtx);
  P.tv.resize(4 * P.n_tet);
  P.blk.resize(P.n_tet);
  P.bid.resize(4 * P.n_tet);
  if (mc_exodus_read(file.c_str(), P.xyz.data(), P.tv.data(), P.blk.data(), P.bid.data(), err, sizeof err))
    p.error("file", err);
  for (int k = 0; k < 3; ++k) {
    P.lo[k] = INFINITY;
    P.hi[k] = -INFINITY;
  }
  for (int64_t v = 0; v < P.n_vtx; ++v)
    for (int k = 0; k < 3; ++k) {
      P.lo[k] = std::min(P.lo[k], P.xyz[3 * v + k]);
      P.hi[k] = std::max(P.hi[k], P.xyz[3 * v + k]);
    }
}

// --- [RayKernels] -------------------------------------------------------------
// CollisionKernel parameters (src/raykernels/CollisionKernel.C:24-76).
void collision_kernel(Params& p, Problem& P) {
  p.str("temperature");  // required coupled variable; synthetic tables carry no temperature
  const auto blocks = p.ints("blocks", true);
  const auto mats = p.ints("materials", true);
  if (blocks.size() != mats.size())
    p.error("blocks", "The blocks parameter must be the same size as the materials parameter.");
  // z_coord (CollisionKernel.C:38,60-61) makes the problem 2-D: the mesh is
  // then one layer of tets around that plane (e.g. TetLatticeMeshGenerator
  // with nz = 1), directions stay in the plane
  if (p.has("z_coord")) {
    P.two_d = true;
    P.z2d = p.real("z_coord", 0.0);
  }
  P.verbose = p.boolean("verbose", false) || P.verbose;
  P.blocks.assign(blocks.begin(), blocks.end());
  P.materials.assign(mats.begin(), mats.end());
  P.have_kernel = true;
}

// --- [RayBCs] -----------------------------------------------------------------
void ray_bc(Params& p, Problem& P, int type) {
  for (auto& b : p.list("boundary", true)) {
    auto it = kSideNames.find(b);
    int id;
    if (it != kSideNames.end()) id = it->second;
    else {
      char* end = nullptr;
      id = (int)strtol(b.c_str(), &end, 10);
      if (end == b.c_str() || *end || id < 0) p.error("boundary", "unknown boundary '" + b + "'");
    }
    P.bcs[id] = type;
  }
}

// --- [UserObjects] ------------------------------------------------------------
// Synthetic nuclear data in place of OpenMC's materials.xml + HDF5 library.
void synthetic_xs(Params& p, Problem& P) {
  const auto ids = p.ints("material_ids", true);
  const auto counts = p.ints("nuclides_per_material", true);
  if (ids.size() != counts.size())
    p.error("material_ids", "must have as many entries as nuclides_per_material");
  const uint64_t seed = (uint64_t)p.integer("seed", 20240611);
  const int n_pts = (int)p.integer("n_points", 10000);
  const int n_peaks = (int)p.integer("n_peaks", 20);
  const double e_min = p.real("energy_min", 1e-5), e_max = p.real("energy_max", 2e7);
  const double d_lo = p.real("density_min", 1e-4), d_hi = p.real("density_max", 5e-2);
  // constant cross sections added to every tabulated point (barn): elastic
  // scattering (sigma_s and sigma_t) and absorption (sigma_t)
  const double pot = p.real("scattering_offset", 0.0), absb = p.real("absorption_offset", 0.0);
  if (!(pot >= 0.0) || !(absb >= 0.0)) p.error("scattering_offset", "offsets must be non-negative");
  // fission data: every nuclide of the listed materials gets
  // nu*sigma_f = nu * fission_share * sigma_a at each point
  const auto fis = p.ints("fissionable_materials");
  const double nu = p.real("nu", 2.43), share = p.real("fission_share", 0.6);
  if (!(nu > 0.0) || !(share >= 0.0 && share <= 1.0)) p.error("nu", "nu must be positive, fission_share in [0, 1]");
  for (int f : fis)
    if (std::find(ids.begin(), ids.end(), f) == ids.end())
      p.error("fissionable_materials", "material " + std::to_string(f) + " is not in material_ids");
  int k = 0;
  for (size_t m = 0; m < ids.size(); ++m) {
    Problem::Mat mat;
    mat.id = ids[m];
    if (counts[m] < 1) p.error("nuclides_per_material", "must be positive");
    mat.dens.resize(counts[m]);
    if (mc_gen_densities(seed, (int)m, counts[m], d_lo, d_hi, mat.dens.data()))
      p.error("density_min", "invalid density range");
    for (int j = 0; j < counts[m]; ++j, ++k) {
      Problem::Nuc n;
      n.E.resize(n_pts);
      n.st.resize(n_pts);
      n.ss.resize(n_pts);
      if (mc_gen_nuclide(seed, k, n_pts, e_min, e_max, n_peaks, n.E.data(), n.st.data(), n.ss.data(), &n.awr))
        p.error("n_points", "invalid nuclide table parameters");
      if (pot > 0.0 || absb > 0.0)
        for (int i = 0; i < n_pts; ++i) {
          n.ss[i] = n.ss[i] + pot;
          n.st[i] = n.st[i] + (pot + absb);
        }
      if (std::find(fis.begin(), fis.end(), ids[m]) != fis.end()) {
        n.nusf.resize(n_pts);
        const double c = nu * share;
        for (int i = 0; i < n_pts; ++i) n.nusf[i] = c * (n.st[i] - n.ss[i]);
      }
      mat.nuc.push_back((int32_t)P.nucs.size());
      P.nucs.push_back(std::move(n));
    }
    P.mats.push_back(std::move(mat));
  }
}

// OpenMCStudy (src/userobjects/OpenMCStudy.C:49-76) plus the fixed-source
// settings OpenMC would read from settings.xml.
void openmc_study(Params& p, Problem& P) {
  p.boolean("suppress_openmc_output", true);
  p.boolean("has_internal_surface_tallies", false);
  P.verbose = p.boolean("verbose", true) && P.verbose;
  for (const char* k : {"execute_on", "always_cache_traces", "segments_on_cache_traces", "data_on_cache_traces",
                        "aux_data_on_cache_traces"})
    if (p.has(k)) p.raw(k);
  P.particles = p.integer("particles", 0, true);
  if (P.particles < 1) p.error("particles", "must be positive");
  P.bank_size = p.integer("bank_size", 0);
  P.seed = (uint64_t)p.integer("seed", 1);
  P.precision = p.choice("precision", {"fp64", "mixed"}, "fp64") == "mixed" ? MC_PREC_MIXED : MC_PREC_FP64;
  P.mode = p.choice("mode", {"event", "history"}, "event") == "history" ? MC_MODE_HISTORY : MC_MODE_EVENT;
  if (p.has("batches")) P.batches = p.integer("batches", 1);
  // OpenMC settings.xml run mode (OpenMCStudy.C:133-136 rejects the
  // particle, plotting and volume modes)
  P.eigen = p.choice("run_mode", {"fixed source", "fixed_source", "eigenvalue"}, "fixed_source") == "eigenvalue";
  P.inactive = p.integer("inactive", 0);
  if (P.inactive < 0) p.error("inactive", "must be non-negative");
  if (!P.eigen && P.inactive > 0) p.error("inactive", "inactive batches need run_mode = eigenvalue");
  mc_source_desc& s = P.src;
  const std::string space = p.choice("source_space", {"point", "box", "cylinders"}, "point");
  if (space == "point") {
    s.space = MC_SRC_POINT;
    auto pt = p.reals("source_point");
    if (pt.empty()) {
      for (int k = 0; k < 3; ++k) s.point[k] = 0.5 * (P.lo[k] + P.hi[k]);
    } else {
      if (pt.size() != 3) p.error("source_point", "needs three coordinates");
      for (int k = 0; k < 3; ++k) s.point[k] = pt[k];
    }
  } else if (space == "box") {
    s.space = MC_SRC_BOX;
    auto b = p.reals("source_box", true);
    if (b.size() != 6) p.error("source_box", "needs xmin ymin zmin xmax ymax zmax");
    for (int k = 0; k < 3; ++k) {
      s.box_lo[k] = b[k];
      s.box_hi[k] = b[3 + k];
    }
  } else {
    s.space = MC_SRC_CYLINDERS;
    if (P.cyl_xy.empty()) p.error("source_space", "cylinder sources need a TetLatticeMeshGenerator mesh");
    s.n_cyl = (int32_t)(P.cyl_xy.size() / 2);
    s.cyl_r = p.real("source_radius", P.cyl_r);
    s.cyl_z0 = 0.0;
    s.cyl_z1 = P.height;
  }
  const std::string en = p.choice("source_energy", {"watt", "mono"}, "watt");
  if (en == "watt") {
    s.energy = MC_SRC_WATT;
    auto w = p.reals("watt_parameters");
    s.watt_a = w.size() > 0 ? w[0] : 0.988e6;
    s.watt_b = w.size() > 1 ? w[1] : 2.249e-6;
  } else {
    s.energy = MC_SRC_MONO;
    s.mono_E = p.real("source_energy_value", 0.0, true);
  }
  P.have_study = true;
}

// Score names of the synthetic tables (no fission data: fission scores are
// rejected).
int score_of(Params& p, const char* key, const std::string& s) {
  if (s == "flux") return MC_SCORE_FLUX;
  if (s == "total") return MC_SCORE_TOTAL;
  if (s == "scatter") return MC_SCORE_SCATTER;
  if (s == "absorption") return MC_SCORE_ABSORPTION;
  p.error(key, "score '" + s + "' is not available: the synthetic tables give flux, total, scatter and "
                           "absorption");
  return -1;
}

// OpenMCTally (src/userobjects/OpenMCTally.C:30-101): estimator (COLLISION
// by default, as in the reference, or TRACKLENGTH), scores, and the filters
// cell (element bins) or universe (block bins), energy (with energy_bins)
// and particle (neutron).
void openmc_tally(Params& p, Problem& P) {
  Problem::Tally t;
  t.id = (int)p.integer("id", 0, true);
  if (p.choice("particle_type", {"neutron", "photon", "electron", "positron"}, "neutron") != "neutron")
    p.error("particle_type", "Only neutrons are currently supported.");
  const std::string est = p.choice("estimator", {"ANALOG", "TRACKLENGTH", "COLLISION"}, "COLLISION");
  if (est == "ANALOG") p.error("estimator", "the analog estimator is not available on the GPU path");
  t.estimator = est == "TRACKLENGTH" ? MC_EST_TRACKLENGTH : MC_EST_COLLISION;
  for (auto& s : p.list("scores", true)) {
    const int sc = score_of(p, "scores", s);
    if (t.estimator == MC_EST_TRACKLENGTH && sc != MC_SCORE_FLUX && sc != MC_SCORE_TOTAL)
      p.error("scores", "the tracklength estimator scores flux and total only");
    for (int o : t.scores)
      if (o == sc) p.error("scores", "repeated score '" + s + "'");
    t.scores.push_back(sc);
  }
  if (t.scores.size() > MC_MAX_SCORES) p.error("scores", "at most 4 scores");
  bool energy = false;
  for (auto& f : p.list("filters", true)) {
    if (f == "cell" || f == "universe") {
      if (!t.filter.empty()) p.error("filters", "use one of the filters 'cell' or 'universe'");
      t.filter = f;
    } else if (f == "energy") {
      energy = true;
    } else if (f != "particle") {
      p.error("filters", "unknown filter '" + f + "' (cell, universe, energy, particle)");
    }
  }
  if (t.filter.empty()) p.error("filters", "a 'cell' or 'universe' filter is needed for element results");
  if (energy) {
    if (!p.has("energy_bins"))
      p.error("energy_bins", "The energy bins parameter should be supplied if an energy filter is requested.");
    for (auto& e : p.list("energy_bins", true)) t.edges.push_back(std::stod(e));
    if (t.edges.size() < 2) p.error("energy_bins", "at least two edges");
    for (size_t b = 1; b < t.edges.size(); ++b)
      if (!(t.edges[b] > t.edges[b - 1])) p.error("energy_bins", "edges must ascend");
  }
  if (p.has("execute_on")) p.raw("execute_on");
  for (auto& o : P.tallies)
    if (o.id == t.id) p.error("id", "duplicate tally id");
  P.tallies.push_back(t);
}

// --- [AuxKernels] -------------------------------------------------------------
// OpenMCTallyAux (src/auxkernels/OpenMCTallyAux.C:26-68).
void openmc_tally_aux(Params& p, Problem& P) {
  Problem::Aux a;
  a.tally_id = (int)p.integer("tally_id", 0, true);
  a.granularity = p.choice("granularity", {"global", "universe", "cell"}, "cell");
  if (a.granularity == "global") p.error("granularity", "Global Tally retrieving currently not supported");
  a.score = score_of(p, "score", p.str("score"));
  a.energy_bin = p.has("energy_bin") ? (int)p.integer("energy_bin", 0) : -1;
  p.choice("estimator", {"ANALOG", "TRACKLENGTH", "COLLISION"}, "COLLISION");
  p.choice("particle_type", {"neutron", "photon", "electron", "positron"}, "neutron");
  a.variable = p.str("variable");
  if (p.has("execute_on")) p.raw("execute_on");
  a.name = p.b->name;
  P.aux.push_back(a);
}

std::map<std::string, Factory>& registry() {
  static std::map<std::string, Factory> r = {
      {"TetCubeMeshGenerator", tet_cube_mesh},
      {"TetLatticeMeshGenerator", tet_lattice_mesh},
      {"FileMeshGenerator", file_mesh},
      {"CollisionKernel", collision_kernel},
      {"KillRayBC", [](Params& p, Problem& P) { ray_bc(p, P, MC_BC_VACUUM); }},
      {"ReflectRayBC", [](Params& p, Problem& P) { ray_bc(p, P, MC_BC_REFLECT); }},
      {"SyntheticCrossSections", synthetic_xs},
      {"OpenMCStudy", openmc_study},
      {"OpenMCTally", openmc_tally},
      {"OpenMCTallyAux", openmc_tally_aux},
  };
  return r;
}

void build_object(const Block& b, Problem& P, const char* section) {
  auto it = b.params.find("type");
  if (it == b.params.end()) {
    // a grouping block: build its children
    for (auto& c : b.children) build_object(c, P, section);
    return;
  }
  auto f = registry().find(it->second);
  if (f == registry().end())
    throw InputError(b.path + "/type: unknown object type '" + it->second + "' in [" + section + "]");
  Params p(&b);
  p.used["type"] = true;
  f->second(p, P);
  for (auto& k : b.order)
    if (!p.used.count(k))
      throw InputError(b.path + "/" + k + ": unused parameter for " + it->second);
}

// [UserObjects] must see the mesh and data in a fixed order: data and
// tallies first, then the study (which may derive its source from the mesh).
void build_user_objects(const Block& uo, Problem& P) {
  std::vector<std::string> active;
  bool restrict = false;
  auto act = uo.params.find("active");
  if (act != uo.params.end()) {
    restrict = true;
    std::istringstream s(act->second);
    std::string w;
    while (s >> w) active.push_back(w);
  }
  auto is_active = [&](const std::string& n) {
    if (!restrict) return true;
    for (auto& a : active)
      if (a == n) return true;
    return false;
  };
  std::vector<const Block*> later;
  for (auto& c : uo.children) {
    if (!is_active(c.name)) continue;
    auto t = c.params.find("type");
    if (t != c.params.end() && t->second == "OpenMCStudy") later.push_back(&c);
    else build_object(c, P, "UserObjects");
  }
  for (auto* c : later) build_object(*c, P, "UserObjects");
}

int check(mc_ctx* ctx, int rc, const char* what) {
  if (rc) throw std::runtime_error(std::string(what) + ": " + (ctx ? mc_last_error(ctx) : "error"));
  return rc;
}

}  // namespace

// One device tally serves every OpenMCTally of an input: they must share the
// estimator and energy bins; its scores are the union of theirs in order of
// appearance.  Checks each OpenMCTallyAux against its tally (granularity,
// score, energy bin) and resolves the score's position.
struct TallyPlan {
  mc_tally_desc desc{};
  std::vector<double> edges;
  std::vector<int> scores;
  int nb = 1;
  bool general = false;
  std::vector<int> aux_score_pos;
};

TallyPlan plan_tallies(const Problem& P) {
  TallyPlan T;
  T.desc.estimator = MC_EST_TRACKLENGTH;
  T.scores = {MC_SCORE_FLUX};
  if (!P.tallies.empty()) {
    const auto& t0 = P.tallies[0];
    T.scores.clear();
    for (auto& t : P.tallies) {
      if (t.estimator != t0.estimator || t.edges != t0.edges)
        throw InputError("[UserObjects]: all OpenMCTally objects must share the estimator and energy bins on the "
                         "GPU path");
      for (int s : t.scores)
        if (std::find(T.scores.begin(), T.scores.end(), s) == T.scores.end()) T.scores.push_back(s);
    }
    if (T.scores.size() > MC_MAX_SCORES) throw InputError("[UserObjects]: at most 4 distinct scores in all");
    T.desc.estimator = t0.estimator;
    T.edges = t0.edges;
  }
  T.nb = T.edges.empty() ? 1 : (int)T.edges.size() - 1;
  T.desc.n_scores = (int32_t)T.scores.size();
  for (size_t j = 0; j < T.scores.size(); ++j) T.desc.scores[j] = T.scores[j];
  T.desc.n_energy_bins = T.edges.empty() ? 0 : T.nb;
  T.desc.energy_edges = T.edges.empty() ? nullptr : T.edges.data();
  T.general = !(T.desc.estimator == MC_EST_TRACKLENGTH && T.scores.size() == 1 && T.scores[0] == MC_SCORE_FLUX &&
                T.edges.empty());
  for (auto& a : P.aux) {
    const Problem::Tally* tt = nullptr;
    for (auto& t : P.tallies)
      if (t.id == a.tally_id) tt = &t;
    if (!tt)
      throw InputError("AuxKernels/" + a.name + "/tally_id: no OpenMCTally with id " + std::to_string(a.tally_id));
    if (a.granularity == "universe" && tt->filter != "universe")
      throw InputError("AuxKernels/" + a.name + ": Tally does not have a universe filter");
    if (a.granularity == "cell" && tt->filter != "cell")
      throw InputError("AuxKernels/" + a.name + ": Specified tally does not contain a cell filter");
    if (std::find(tt->scores.begin(), tt->scores.end(), a.score) == tt->scores.end())
      throw InputError("AuxKernels/" + a.name + "/score: The specified score does not exist in given tally");
    if (a.energy_bin >= 0 && a.energy_bin >= T.nb)
      throw InputError("AuxKernels/" + a.name + "/energy_bin: the tally has " + std::to_string(T.nb) +
                       " energy bin(s)");
    T.aux_score_pos.push_back((int)(std::find(T.scores.begin(), T.scores.end(), a.score) - T.scores.begin()));
  }
  return T;
}

// Runs a whole input: setup, `batches` batches, readback of every
// OpenMCTallyAux variable.  Writes a JSON summary into report (truncated to
// report_len) and, when [Outputs] csv = true, <file_base>_<variable>.csv.
extern "C" int mc_app_run(const char* input_text, int device, const char* file_base, char* report,
                          int64_t report_len) {
  auto put = [&](const std::string& s) {
    if (report && report_len > 0) {
      const size_t n = std::min<size_t>(s.size(), (size_t)report_len - 1);
      memcpy(report, s.data(), n);
      report[n] = 0;
    }
  };
  if (!input_text) {
    put("{\"error\": \"null input\"}");
    return MC_ERR_ARG;
  }
  mc_ctx* ctx = nullptr;
  try {
    Block root = parse_hit(input_text);
    Problem P;
    P.file_base = file_base ? file_base : "";
    Block* mesh = root.child("Mesh");
    if (!mesh) throw InputError("[Mesh]: missing");
    build_object(*mesh, P, "Mesh");
    if (P.n_tet == 0) throw InputError("[Mesh]: no mesh generator produced a mesh");
    for (const char* ignored : {"Problem", "Variables", "AuxVariables", "Postprocessors", "VectorPostprocessors"})
      (void)ignored;
    if (Block* rk = root.child("RayKernels")) build_object(*rk, P, "RayKernels");
    if (!P.have_kernel) throw InputError("[RayKernels]: a CollisionKernel is required");
    if (Block* rb = root.child("RayBCs")) build_object(*rb, P, "RayBCs");
    Block* uo = root.child("UserObjects");
    if (!uo) throw InputError("[UserObjects]: missing");
    build_user_objects(*uo, P);
    if (!P.have_study) throw InputError("[UserObjects]: an OpenMCStudy is required");
    if (P.mats.empty()) throw InputError("[UserObjects]: a SyntheticCrossSections object is required");
    if (Block* ak = root.child("AuxKernels")) build_object(*ak, P, "AuxKernels");
    if (Block* ex = root.child("Executioner")) {
      Params p(ex);
      if (p.has("type") && p.raw("type") != "Transient")
        p.error("type", "Only a Transient executioner is supported (one step per batch)");
      if (p.has("num_steps")) P.batches = p.integer("num_steps", 1);
    }
    if (P.batches < 1) throw InputError("[Executioner]/num_steps: must be positive");
    if (Block* out = root.child("Outputs")) {
      Params p(out);
      P.csv = p.boolean("csv", false);
      P.exodus = p.boolean("exodus", false);
      // [Outputs/<name>] type = RayTracingExodus (MOOSE ray_tracing module, as
      // test/tests/study/openmc_study.i uses it): the segments of the last
      // batch's first max_rays histories, up to max_segments each
      for (const Block& c : out->children) {
        Params q(&c);
        if (!q.has("type")) continue;
        if (q.raw("type") != "RayTracingExodus") q.error("type", "unknown output type (use RayTracingExodus)");
        if (q.has("study")) q.raw("study");
        q.boolean("output_data", true);
        q.boolean("output_aux_data", true);
        if (q.has("execute_on")) q.raw("execute_on");
        P.rays = true;
        P.rays_name = c.name;
        P.rays_n = (int32_t)q.integer("max_rays", 1000);
        P.rays_cap = (int32_t)q.integer("max_segments", 4096);
        if (P.rays_n < 1 || P.rays_cap < 1) q.error("max_rays", "must be positive");
        for (auto& k : c.order)
          if (!q.used.count(k)) q.error(k, "unused parameter for RayTracingExodus");
      }
      if (p.has("file_base")) P.file_base = p.raw("file_base");
    }
    TallyPlan TP = plan_tallies(P);

    // ---- device setup (OpenMCStudy constructor + initialSetup) ----
    check(nullptr, mc_ctx_create(device, &ctx), "mc_ctx_create");
    check(ctx, mc_mesh_upload(ctx, P.n_vtx, P.xyz.data(), P.n_tet, P.tv.data(), P.blk.data(), P.bid.data()),
          "mesh");
    for (auto& b : P.bcs) check(ctx, mc_bc_set(ctx, b.first, b.second), "RayBCs");
    for (auto& n : P.nucs) {
      int32_t k = 0;
      check(ctx, mc_nuclide_add(ctx, (int64_t)n.E.size(), n.E.data(), n.st.data(), n.ss.data(), n.awr, &k),
            "nuclide");
      if (!n.nusf.empty()) check(ctx, mc_nuclide_set_fission(ctx, k, n.nusf.data()), "nuclide fission data");
    }
    for (auto& m : P.mats)
      check(ctx, mc_material_add(ctx, m.id, (int32_t)m.nuc.size(), m.nuc.data(), m.dens.data()), "material");
    check(ctx, mc_block_material_map(ctx, (int32_t)P.blocks.size(), P.blocks.data(), P.materials.data()),
          "CollisionKernel");
    if (P.src.space == MC_SRC_CYLINDERS) P.src.cyl_xy = P.cyl_xy.data();
    check(ctx, mc_source_set(ctx, &P.src), "OpenMCStudy source");
    if (P.two_d) {
      if (!(P.z2d >= P.lo[2] && P.z2d <= P.hi[2]))
        throw InputError("RayKernels/z_coord: outside the mesh's z range");
      check(ctx, mc_set_2d(ctx, 1, P.z2d), "CollisionKernel z_coord");
    }
    if (TP.general) check(ctx, mc_tally_configure(ctx, &TP.desc), "OpenMCTally");
    int64_t n_tally = 0;
    check(ctx, mc_tally_size(ctx, &n_tally), "OpenMCTally");
    const int ns = TP.desc.n_scores, nb = TP.nb;

    // ---- batches (Transient steps) ----
    const auto t0 = std::chrono::steady_clock::now();
    mc_stats tot{};
    std::vector<mc_eigen_gen> gens;
    if (P.eigen) {
      // OpenMC eigenvalue mode: every batch is one generation; tallies and
      // element results come from the active ones
      if (P.inactive >= P.batches)
        throw InputError("UserObjects/OpenMCStudy/inactive: must be below the number of batches");
      bool any = false;
      for (auto& n : P.nucs) any = any || !n.nusf.empty();
      if (!any) throw InputError("UserObjects: run_mode = eigenvalue needs fissionable_materials");
      if (P.rays) throw InputError("Outputs: RayTracingExodus output is available in fixed-source runs");
      mc_eigen_desc e{};
      e.n_particles = P.particles;
      e.n_batches = (int32_t)P.batches;
      e.n_inactive = (int32_t)P.inactive;
      e.seed = P.seed;
      e.precision = P.precision;
      e.mode = P.mode;
      e.bank_size = P.bank_size;
      gens.resize((size_t)P.batches);
      check(ctx, mc_eigen_run(ctx, &e, gens.data()), "eigenvalue generations");
      for (auto& g : gens) {
        tot.n_hist += P.particles;
        tot.n_seg += g.n_seg;
        tot.n_coll += g.n_coll;
        tot.leak_weight += g.leakage * (double)P.particles;
      }
    }
    for (int64_t b = 0; b < P.batches && !P.eigen; ++b) {
      if (P.rays && b == P.batches - 1)
        check(ctx, mc_rays_enable(ctx, (int32_t)std::min<int64_t>(P.rays_n, P.particles), P.rays_cap), "rays");
      mc_run_desc d{};
      d.first_history = b * P.particles;
      d.n_histories = P.particles;
      d.bank_size = P.bank_size;
      d.seed = P.seed;
      d.precision = P.precision;
      d.mode = P.mode;
      d.accumulate = 1;
      check(ctx, mc_run(ctx, &d), "batch");
      mc_stats s;
      mc_stats_get(ctx, &s);
      tot.n_hist += s.n_hist;
      tot.n_seg += s.n_seg;
      tot.n_coll += s.n_coll;
      tot.n_leak += s.n_leak;
      tot.n_absorb += s.n_absorb;
      tot.n_stuck += s.n_stuck;
      tot.n_lost += s.n_lost;
      tot.leak_weight += s.leak_weight;
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

    // ---- AuxKernel readback ----
    std::vector<double> sum((size_t)n_tally), sq((size_t)n_tally);
    check(ctx, mc_tally_download(ctx, MC_TALLY_SUM, sum.data(), n_tally), "tally");
    check(ctx, mc_tally_download(ctx, MC_TALLY_SUM_SQ, sq.data(), n_tally), "tally");
    std::ostringstream js;
    js.precision(17);
    js << "{\"histories\": " << tot.n_hist << ", \"segments\": " << tot.n_seg << ", \"collisions\": " << tot.n_coll
       << ", \"leaked\": " << tot.n_leak << ", \"absorbed\": " << tot.n_absorb << ", \"stuck\": " << tot.n_stuck
       << ", \"lost\": " << tot.n_lost << ", \"batches\": " << P.batches << ", \"seconds\": " << secs
       << ", \"neutrons_per_s\": " << (secs > 0 ? tot.n_hist / secs : 0.0);
    if (P.eigen) {
      // OpenMCStudy::postExecuteStudy prints "Keff <keff> (<std>) Generation: <k>" per batch
      const mc_eigen_gen& L = gens.back();
      js << ", \"keff\": " << L.keff << ", \"keff_std\": " << L.keff_std << ", \"inactive\": " << P.inactive
         << ", \"generations\": [";
      for (size_t g = 0; g < gens.size(); ++g)
        js << (g ? ", " : "") << "{\"k_generation\": " << gens[g].k_generation << ", \"keff\": " << gens[g].keff
           << ", \"keff_std\": " << gens[g].keff_std << ", \"k_collision\": " << gens[g].k_collision
           << ", \"k_absorption\": " << gens[g].k_absorption << ", \"sites\": " << gens[g].n_sites << "}";
      js << "]";
      if (P.csv && !P.file_base.empty()) {
        std::ofstream f(P.file_base + "_keff.csv");
        if (!f) throw std::runtime_error("cannot write " + P.file_base + "_keff.csv");
        f.precision(17);
        f << "generation,k_generation,keff,keff_std,k_collision,k_absorption,fission_sites\n";
        for (size_t g = 0; g < gens.size(); ++g)
          f << g + 1 << "," << gens[g].k_generation << "," << gens[g].keff << "," << gens[g].keff_std << ","
            << gens[g].k_collision << "," << gens[g].k_absorption << "," << gens[g].n_sites << "\n";
      }
    }
    js << ", \"aux\": {";
    bool first = true;
    // batches whose tallies were accumulated (eigenvalue runs: the active ones)
    const double n_acc = P.eigen ? (double)(P.batches - P.inactive) : (double)P.batches;
    std::vector<std::string> ex_names;
    std::vector<double> ex_vals;  // per variable, n_tet values (per batch, as the csv)
    for (size_t ai = 0; ai < P.aux.size(); ++ai) {
      const auto& a = P.aux[ai];
      const int j = TP.aux_score_pos[ai];
      // the element's value: its score summed over the energy bins, or the one bin asked for
      // (OpenMCTallyAux.C:187-205); the relative error is kept for a single bin
      const int b0 = a.energy_bin >= 0 ? a.energy_bin : 0, b1 = a.energy_bin >= 0 ? a.energy_bin + 1 : nb;
      const bool single = b1 - b0 == 1;
      std::vector<double> cell((size_t)P.n_tet), cell_sq((size_t)P.n_tet);
      for (int64_t t = 0; t < P.n_tet; ++t)
        for (int b = b0; b < b1; ++b) {
          cell[t] += sum[((size_t)t * nb + b) * ns + j];
          cell_sq[t] += sq[((size_t)t * nb + b) * ns + j];
        }
      std::vector<double> val((size_t)P.n_tet);
      if (a.granularity == "cell") {
        val = cell;
      } else {
        std::map<int, double> per_block;
        for (int64_t t = 0; t < P.n_tet; ++t) per_block[P.blk[t]] += cell[t];
        for (int64_t t = 0; t < P.n_tet; ++t) val[t] = per_block[P.blk[t]];
      }
      double total = 0.0;
      for (double v : val) total += v;
      js << (first ? "" : ", ") << "\"" << a.variable << "\": {\"sum\": " << total << "}";
      first = false;
      if (P.exodus) {
        ex_names.push_back(a.variable);
        for (int64_t t = 0; t < P.n_tet; ++t) ex_vals.push_back(val[t] / n_acc);
      }
      if (P.csv && !P.file_base.empty()) {
        std::ofstream f(P.file_base + "_" + a.variable + ".csv");
        if (!f) throw std::runtime_error("cannot write " + P.file_base + "_" + a.variable + ".csv");
        f.precision(17);
        f << "elem,block," << a.variable << ",rel_err\n";
        const double nbat = n_acc;
        for (int64_t t = 0; t < P.n_tet; ++t) {
          double re = 0.0;
          if (a.granularity == "cell" && single && cell[t] > 0 && nbat > 1) {
            const double mean = cell[t] / nbat;
            const double var = (cell_sq[t] / nbat - mean * mean) / (nbat - 1);
            re = var > 0 ? sqrt(var) / mean : 0.0;
          }
          f << t << "," << P.blk[t] << "," << val[t] / nbat << "," << re << "\n";
        }
      }
    }
    js << "}";
    if (P.rays && !P.file_base.empty()) {
      // MOOSE names the file <file_base>_<output name>.e
      int64_t n = 0;
      mc_rays_download(ctx, nullptr, 0, &n);
      std::vector<mc_ray_segment> seg((size_t)n);
      check(ctx, mc_rays_download(ctx, seg.data(), n, &n), "rays");
      const std::string path = P.file_base + "_" + P.rays_name + ".e";
      if (n > 0 && mc_exodus_write_rays(path.c_str(), seg.data(), n, (P.batches - 1) * P.particles) != MC_OK)
        throw std::runtime_error("cannot write " + path);
      js << ", \"rays\": \"" << path << "\", \"ray_segments\": " << n;
    }
    if (P.exodus && !P.file_base.empty()) {
      // MOOSE's Exodus output of the AuxVariables at the last step
      std::vector<const char*> nm;
      for (auto& s : ex_names) nm.push_back(s.c_str());
      const std::string path = P.file_base + ".e";
      if (mc_exodus_write(path.c_str(), "macaw_gb300", P.n_vtx, P.xyz.data(), P.n_tet, P.tv.data(), P.blk.data(),
                          P.bid.data(), (int32_t)nm.size(), nm.data(), ex_vals.data(), (double)P.batches) != MC_OK)
        throw std::runtime_error("cannot write " + path);
      js << ", \"exodus\": \"" << path << "\"";
    }
    js << "}";
    put(js.str());
    mc_ctx_destroy(ctx);
    return MC_OK;
  } catch (const InputError& e) {
    if (ctx) mc_ctx_destroy(ctx);
    put(std::string("{\"error\": \"") + e.what() + "\"}");
    return MC_ERR_ARG;
  } catch (const std::exception& e) {
    if (ctx) mc_ctx_destroy(ctx);
    put(std::string("{\"error\": \"") + e.what() + "\"}");
    return MC_ERR_STATE;
  }
}

// Parses and checks an input without touching a device (used to validate
// inputs on hosts without a GPU): the same object construction and
// parameter checks as mc_app_run, returning a JSON summary of the problem.
extern "C" int mc_app_check(const char* input_text, char* report, int64_t report_len) {
  auto put = [&](const std::string& s) {
    if (report && report_len > 0) {
      const size_t n = std::min<size_t>(s.size(), (size_t)report_len - 1);
      memcpy(report, s.data(), n);
      report[n] = 0;
    }
  };
  if (!input_text) return MC_ERR_ARG;
  try {
    Block root = parse_hit(input_text);
    Problem P;
    Block* mesh = root.child("Mesh");
    if (!mesh) throw InputError("[Mesh]: missing");
    build_object(*mesh, P, "Mesh");
    if (Block* rk = root.child("RayKernels")) build_object(*rk, P, "RayKernels");
    if (!P.have_kernel) throw InputError("[RayKernels]: a CollisionKernel is required");
    if (Block* rb = root.child("RayBCs")) build_object(*rb, P, "RayBCs");
    Block* uo = root.child("UserObjects");
    if (!uo) throw InputError("[UserObjects]: missing");
    build_user_objects(*uo, P);
    if (!P.have_study) throw InputError("[UserObjects]: an OpenMCStudy is required");
    if (Block* ak = root.child("AuxKernels")) build_object(*ak, P, "AuxKernels");
    if (Block* ex = root.child("Executioner")) {
      Params p(ex);
      if (p.has("type") && p.raw("type") != "Transient")
        p.error("type", "Only a Transient executioner is supported (one step per batch)");
      if (p.has("num_steps")) P.batches = p.integer("num_steps", 1);
    }
    const TallyPlan TP = plan_tallies(P);
    std::ostringstream js;
    js << "{\"tets\": " << P.n_tet << ", \"vertices\": " << P.n_vtx << ", \"nuclides\": " << P.nucs.size()
       << ", \"materials\": " << P.mats.size() << ", \"particles\": " << P.particles << ", \"batches\": "
       << P.batches << ", \"reflective\": " << [&] {
            int n = 0;
            for (auto& b : P.bcs) n += b.second == MC_BC_REFLECT;
            return n;
          }()
       << ", \"tallies\": " << P.tallies.size() << ", \"tally_values_per_element\": " << TP.nb * TP.desc.n_scores
       << ", \"aux\": " << P.aux.size() << ", \"precision\": \""
       << (P.precision == MC_PREC_MIXED ? "mixed" : "fp64") << "\", \"run_mode\": \""
       << (P.eigen ? "eigenvalue" : "fixed source") << "\", \"inactive\": " << P.inactive
       << ", \"fissionable_nuclides\": " << [&] {
            int n = 0;
            for (auto& q : P.nucs) n += !q.nusf.empty();
            return n;
          }()
       << "}";
    put(js.str());
    return MC_OK;
  } catch (const std::exception& e) {
    put(std::string("{\"error\": \"") + e.what() + "\"}");
    return MC_ERR_ARG;
  }
}
