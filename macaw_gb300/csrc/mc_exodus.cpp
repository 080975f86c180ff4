// mc_exodus.cpp -- Exodus II files: tet meshes with element fields out,
// tet meshes in.
//
// MOOSE writes a MaCaw run's AuxVariables (the OpenMCTallyAux fields) to an
// Exodus II file ([Outputs] exodus = true).  This writes the same kind of
// file for the tracker's results: the mesh (one element block per
// subdomain, TETRA4), element variables, one time step.  Exodus II sits on
// netCDF; the file is netCDF's 64-bit-offset format, written directly from
// its published layout (big-endian header of dimensions, attributes and
// variables; fixed-size variables at their offsets; record variables
// interleaved per time step), with the Exodus II names for dimensions,
// variables and attributes.
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <ctype.h>
#include <sys/types.h>

#include <algorithm>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/macaw_gb300.h"

namespace {

enum NcType { kByte = 1, kChar = 2, kShort = 3, kInt = 4, kFloat = 5, kDouble = 6 };
const uint32_t kNcDimension = 0x0A, kNcVariable = 0x0B, kNcAttribute = 0x0C;

int type_size(int t) { return t == kDouble ? 8 : (t == kInt || t == kFloat) ? 4 : t == kShort ? 2 : 1; }

struct Buf {
  std::vector<uint8_t> b;
  void u32(uint32_t v) {
    for (int k = 3; k >= 0; --k) b.push_back((uint8_t)(v >> (8 * k)));
  }
  void u64(uint64_t v) {
    for (int k = 7; k >= 0; --k) b.push_back((uint8_t)(v >> (8 * k)));
  }
  void f64(double d) {
    uint64_t v;
    memcpy(&v, &d, 8);
    u64(v);
  }
  void f32(float f) {
    uint32_t v;
    memcpy(&v, &f, 4);
    u32(v);
  }
  void pad4() {
    while (b.size() % 4) b.push_back(0);
  }
  void name(const std::string& s) {
    u32((uint32_t)s.size());
    b.insert(b.end(), s.begin(), s.end());
    pad4();
  }
};

struct Attr {
  std::string name;
  int type;
  std::vector<uint8_t> data;  // big-endian values
  uint32_t n;
};

Attr attr_text(const std::string& name, const std::string& v) {
  Attr a{name, kChar, std::vector<uint8_t>(v.begin(), v.end()), (uint32_t)v.size()};
  return a;
}
Attr attr_int(const std::string& name, int32_t v) {
  Buf b;
  b.u32((uint32_t)v);
  return Attr{name, kInt, b.b, 1};
}
Attr attr_float(const std::string& name, float v) {
  Buf b;
  b.f32(v);
  return Attr{name, kFloat, b.b, 1};
}

struct Var {
  std::string name;
  std::vector<int> dims;  // dimension ids; a record variable has the unlimited one first
  int type;
  std::vector<Attr> attrs;
  std::vector<uint8_t> data;  // big-endian values (one record for record variables)
  bool record = false;
  uint64_t begin = 0;
};

void put_attrs(Buf& h, const std::vector<Attr>& as) {
  if (as.empty()) {
    h.u32(0);
    h.u32(0);
    return;
  }
  h.u32(kNcAttribute);
  h.u32((uint32_t)as.size());
  for (const Attr& a : as) {
    h.name(a.name);
    h.u32((uint32_t)a.type);
    h.u32(a.n);
    h.b.insert(h.b.end(), a.data.begin(), a.data.end());
    h.pad4();
  }
}

struct NcFile {
  std::vector<std::pair<std::string, uint64_t>> dims;  // length 0: the unlimited dimension
  std::vector<Attr> gatts;
  std::vector<Var> vars;
  int dim(const std::string& n, uint64_t len) {
    dims.push_back({n, len});
    return (int)dims.size() - 1;
  }
  std::vector<uint8_t> header(uint32_t numrecs) const {
    Buf h;
    h.b = {'C', 'D', 'F', 2};
    h.u32(numrecs);
    h.u32(kNcDimension);
    h.u32((uint32_t)dims.size());
    for (auto& d : dims) {
      h.name(d.first);
      h.u32((uint32_t)d.second);
    }
    put_attrs(h, gatts);
    h.u32(kNcVariable);
    h.u32((uint32_t)vars.size());
    for (const Var& v : vars) {
      h.name(v.name);
      h.u32((uint32_t)v.dims.size());
      for (int d : v.dims) h.u32((uint32_t)d);
      put_attrs(h, v.attrs);
      h.u32((uint32_t)v.type);
      uint64_t vsize = v.data.size();
      vsize = (vsize + 3) / 4 * 4;
      h.u32((uint32_t)std::min<uint64_t>(vsize, 0xffffffffu));
      h.u64(v.begin);
    }
    return h.b;
  }
};

void be_doubles(std::vector<uint8_t>& out, const double* v, size_t n, size_t stride = 1) {
  out.resize(n * 8);
  for (size_t i = 0; i < n; ++i) {
    uint64_t u;
    memcpy(&u, v + i * stride, 8);
    for (int k = 0; k < 8; ++k) out[8 * i + k] = (uint8_t)(u >> (8 * (7 - k)));
  }
}

void be_ints(std::vector<uint8_t>& out, const std::vector<int32_t>& v) {
  out.resize(v.size() * 4);
  for (size_t i = 0; i < v.size(); ++i) {
    const uint32_t u = (uint32_t)v[i];
    for (int k = 0; k < 4; ++k) out[4 * i + k] = (uint8_t)(u >> (8 * (3 - k)));
  }
}

std::vector<uint8_t> chars(const std::vector<std::string>& names, size_t len) {
  std::vector<uint8_t> out(names.size() * len, 0);
  for (size_t i = 0; i < names.size(); ++i)
    memcpy(out.data() + i * len, names[i].data(), std::min(names[i].size(), len - 1));
  return out;
}

// Lays out and writes a one-record file: fixed-size variables after the
// header, then the record variables.
int write_nc(NcFile& f, const char* path) {
  for (int pass = 0; pass < 2; ++pass) {
    uint64_t off = f.header(1).size();
    for (Var& v : f.vars)
      if (!v.record) {
        v.begin = off;
        off += (v.data.size() + 3) / 4 * 4;
      }
    for (Var& v : f.vars)
      if (v.record) {
        v.begin = off;
        off += (v.data.size() + 3) / 4 * 4;
      }
  }
  FILE* fp = fopen(path, "wb");
  if (!fp) return MC_ERR_STATE;
  const std::vector<uint8_t> h = f.header(1);
  bool ok = fwrite(h.data(), 1, h.size(), fp) == h.size();
  const uint8_t zeros[4] = {0, 0, 0, 0};
  for (int rec = 0; rec < 2 && ok; ++rec)
    for (const Var& v : f.vars) {
      if (v.record != (rec == 1)) continue;
      ok = ok && fwrite(v.data.data(), 1, v.data.size(), fp) == v.data.size();
      const size_t pad = (4 - v.data.size() % 4) % 4;
      if (pad) ok = ok && fwrite(zeros, 1, pad, fp) == pad;
    }
  ok = (fclose(fp) == 0) && ok;
  return ok ? MC_OK : MC_ERR_STATE;
}

// Exodus numbers a TETRA4's sides 1..4 as the faces (1,2,4), (2,3,4),
// (1,4,3), (1,3,2) of its nodes; side f of a tet here is the face opposite
// local vertex f.
const int kExoSideOfFace[4] = {2, 3, 1, 4};
const int kFaceOfExoSide[5] = {-1, 2, 0, 1, 3};

}  // namespace

extern "C" int mc_exodus_write(const char* path, const char* title, int64_t n_vtx, const double* xyz, int64_t n_tet,
                               const int32_t* tet_vtx, const int32_t* tet_block, const int32_t* tet_side_bid,
                               int32_t n_vars, const char* const* names, const double* values, double time) {
  if (!path || !xyz || !tet_vtx || !tet_block || n_vtx < 4 || n_tet < 1 || n_vars < 0) return MC_ERR_ARG;
  if (n_vars > 0 && (!names || !values)) return MC_ERR_ARG;
  if (n_vtx > INT32_MAX || n_tet > INT32_MAX) return MC_ERR_ARG;
  for (int64_t i = 0; i < 4 * n_tet; ++i)
    if (tet_vtx[i] < 0 || tet_vtx[i] >= n_vtx) return MC_ERR_ARG;
  // element blocks: subdomains in ascending id, elements in mesh order within each
  std::map<int32_t, std::vector<int64_t>> blocks;
  for (int64_t t = 0; t < n_tet; ++t) blocks[tet_block[t]].push_back(t);
  const size_t kLen = 33;  // len_name / len_string
  NcFile f;
  const int d_len_string = f.dim("len_string", kLen);
  const int d_len_line = f.dim("len_line", 81);
  f.dim("four", 4);
  const int d_len_name = f.dim("len_name", kLen);
  const int d_time = f.dim("time_step", 0);
  const int d_num_dim = f.dim("num_dim", 3);
  const int d_nodes = f.dim("num_nodes", (uint64_t)n_vtx);
  f.dim("num_elem", (uint64_t)n_tet);
  const int d_blk = f.dim("num_el_blk", blocks.size());
  std::vector<int> d_in_blk, d_nod_per;
  for (auto& b : blocks) {
    const size_t k = d_in_blk.size() + 1;
    d_in_blk.push_back(f.dim("num_el_in_blk" + std::to_string(k), b.second.size()));
    d_nod_per.push_back(f.dim("num_nod_per_el" + std::to_string(k), 4));
  }
  // side sets: boundary faces (no other tet shares them) with a boundary
  // id, grouped by id (ascending)
  std::map<int32_t, std::vector<std::pair<int32_t, int32_t>>> ssets;  // id -> (element, Exodus side), 1-based
  if (tet_side_bid) {
    struct Face {
      int32_t v[3];
      int64_t side;  // 4*tet + face
    };
    std::vector<Face> faces((size_t)(4 * n_tet));
    for (int64_t t = 0; t < n_tet; ++t)
      for (int fc = 0; fc < 4; ++fc) {
        Face& F = faces[(size_t)(4 * t + fc)];
        int k = 0;
        for (int a = 0; a < 4; ++a)
          if (a != fc) F.v[k++] = tet_vtx[4 * t + a];
        std::sort(F.v, F.v + 3);
        F.side = 4 * t + fc;
      }
    std::sort(faces.begin(), faces.end(), [](const Face& a, const Face& b) {
      return a.v[0] != b.v[0] ? a.v[0] < b.v[0] : a.v[1] != b.v[1] ? a.v[1] < b.v[1] : a.v[2] < b.v[2];
    });
    auto same = [](const Face& a, const Face& b) { return a.v[0] == b.v[0] && a.v[1] == b.v[1] && a.v[2] == b.v[2]; };
    // element numbers follow the block order, as readers number them
    std::vector<int64_t> exo_num((size_t)n_tet);
    int64_t e = 0;
    for (auto& b : blocks)
      for (int64_t t : b.second) exo_num[(size_t)t] = ++e;
    std::vector<int64_t> boundary;
    for (size_t i = 0; i < faces.size();) {
      size_t j = i + 1;
      while (j < faces.size() && same(faces[i], faces[j])) ++j;
      if (j == i + 1) boundary.push_back(faces[i].side);
      i = j;
    }
    std::sort(boundary.begin(), boundary.end());
    for (int64_t s : boundary) {
      const int32_t id = tet_side_bid[s];
      if (id >= 0) ssets[id].push_back({(int32_t)exo_num[(size_t)(s / 4)], kExoSideOfFace[s % 4]});
    }
  }
  std::vector<int> d_side;
  int d_nss = -1;
  if (!ssets.empty()) {
    d_nss = f.dim("num_side_sets", ssets.size());
    for (auto& s : ssets) d_side.push_back(f.dim("num_side_ss" + std::to_string(d_side.size() + 1), s.second.size()));
  }
  int d_nvar = -1;
  if (n_vars > 0) d_nvar = f.dim("num_elem_var", (uint64_t)n_vars);
  (void)d_len_string;
  (void)d_len_line;
  f.gatts = {attr_float("api_version", 5.22f), attr_float("version", 5.22f),
             attr_int("floating_point_word_size", 8), attr_int("file_size", 1),
             attr_int("maximum_name_length", 32), attr_text("title", title ? title : "macaw_gb300")};
  auto add = [&](Var v) {
    f.vars.push_back(std::move(v));
    return &f.vars.back();
  };
  {
    Var v{"time_whole", {d_time}, kDouble, {}, {}, true};
    be_doubles(v.data, &time, 1);
    add(v);
  }
  {
    std::vector<int32_t> st(blocks.size(), 1), ids;
    for (auto& b : blocks) ids.push_back(b.first);
    Var s{"eb_status", {d_blk}, kInt, {}, {}};
    be_ints(s.data, st);
    add(s);
    Var p{"eb_prop1", {d_blk}, kInt, {attr_text("name", "ID")}, {}};
    be_ints(p.data, ids);
    add(p);
    std::vector<std::string> bn;
    for (auto& b : blocks) bn.push_back("block_" + std::to_string(b.first));
    Var n{"eb_names", {d_blk, d_len_name}, kChar, {}, chars(bn, kLen)};
    add(n);
  }
  for (int k = 0; k < 3; ++k) {
    Var v{std::string("coord") + "xyz"[k], {d_nodes}, kDouble, {}, {}};
    be_doubles(v.data, xyz + k, (size_t)n_vtx, 3);
    add(v);
  }
  add(Var{"coor_names", {d_num_dim, d_len_name}, kChar, {}, chars({"x", "y", "z"}, kLen)});
  {
    size_t k = 0;
    for (auto& b : blocks) {
      std::vector<int32_t> c;
      c.reserve(b.second.size() * 4);
      for (int64_t t : b.second)
        for (int a = 0; a < 4; ++a) c.push_back(tet_vtx[4 * t + a] + 1);  // 1-based node ids
      Var v{"connect" + std::to_string(k + 1), {d_in_blk[k], d_nod_per[k]}, kInt, {attr_text("elem_type", "TETRA4")},
            {}};
      be_ints(v.data, c);
      add(v);
      ++k;
    }
  }
  if (!ssets.empty()) {
    std::vector<int32_t> ids, st(ssets.size(), 1);
    for (auto& s : ssets) ids.push_back(s.first);
    Var s{"ss_status", {d_nss}, kInt, {}, {}};
    be_ints(s.data, st);
    add(s);
    Var p{"ss_prop1", {d_nss}, kInt, {attr_text("name", "ID")}, {}};
    be_ints(p.data, ids);
    add(p);
    size_t k = 0;
    for (auto& ss : ssets) {
      std::vector<int32_t> el, sd;
      for (auto& es : ss.second) {
        el.push_back(es.first);
        sd.push_back(es.second);
      }
      Var ve{"elem_ss" + std::to_string(k + 1), {d_side[k]}, kInt, {}, {}};
      be_ints(ve.data, el);
      add(ve);
      Var vs{"side_ss" + std::to_string(k + 1), {d_side[k]}, kInt, {}, {}};
      be_ints(vs.data, sd);
      add(vs);
      ++k;
    }
  }
  if (n_vars > 0) {
    std::vector<std::string> vn;
    for (int i = 0; i < n_vars; ++i) vn.push_back(names[i] ? names[i] : "");
    add(Var{"name_elem_var", {d_nvar, d_len_name}, kChar, {}, chars(vn, kLen)});
    size_t k = 0;
    for (auto& b : blocks) {
      for (int i = 0; i < n_vars; ++i) {
        std::vector<double> vals;
        vals.reserve(b.second.size());
        for (int64_t t : b.second) vals.push_back(values[(size_t)i * (size_t)n_tet + (size_t)t]);
        Var v{"vals_elem_var" + std::to_string(i + 1) + "eb" + std::to_string(k + 1), {d_time, d_in_blk[k]},
              kDouble, {}, {}, true};
        be_doubles(v.data, vals.data(), vals.size());
        add(v);
      }
      ++k;
    }
  }
  return write_nc(f, path);
}

// Recorded ray segments as MOOSE's RayTracingExodus writes them: one EDGE2
// element per segment (block 0), the nodes of consecutive segments of a ray
// shared, one time step, and the ray's data and aux data after each
// segment as element variables, in the reference output's order.  MaCaw
// keeps its OpenMC seeds in double aux fields, so seeds are written as the
// nearest double; this tracker has no URR stream and keeps no source-stream
// state after birth, so those two are 0.
extern "C" int mc_exodus_write_rays(const char* path, const mc_ray_segment* seg, int64_t n, int64_t first_history) {
  if (!path || n < 1 || !seg || n > INT32_MAX / 2) return MC_ERR_ARG;
  std::vector<double> xyz;
  std::vector<int32_t> conn;
  int64_t prev_id = -1;
  int32_t last_node = 0;
  for (int64_t i = 0; i < n; ++i) {
    const mc_ray_segment& r = seg[i];
    if (r.id != prev_id) {  // a new ray: its first node is this segment's start
      xyz.insert(xyz.end(), r.start, r.start + 3);
      last_node = (int32_t)(xyz.size() / 3);
      prev_id = r.id;
    }
    xyz.insert(xyz.end(), r.end, r.end + 3);
    const int32_t end_node = (int32_t)(xyz.size() / 3);
    conn.push_back(last_node);
    conn.push_back(end_node);
    last_node = end_node;
  }
  const int64_t nn = (int64_t)xyz.size() / 3;
  const size_t kLen = 33;
  NcFile f;
  f.dim("len_string", kLen);
  f.dim("len_line", 81);
  f.dim("four", 4);
  const int d_time = f.dim("time_step", 0);
  const int d_len_name = f.dim("len_name", kLen);
  const int d_num_dim = f.dim("num_dim", 3);
  const int d_nodes = f.dim("num_nodes", (uint64_t)nn);
  const int d_elem = f.dim("num_elem", (uint64_t)n);
  const int d_blk = f.dim("num_el_blk", 1);
  const int d_in = f.dim("num_el_in_blk1", (uint64_t)n);
  const int d_per = f.dim("num_nod_per_el1", 2);
  const int d_nvar = f.dim("num_elem_var", 10);
  f.gatts = {attr_float("api_version", 5.22f), attr_float("version", 5.22f),
             attr_int("floating_point_word_size", 8), attr_int("file_size", 1),
             attr_int("maximum_name_length", 32), attr_text("title", "macaw_gb300 rays")};
  auto ints_of = [](const std::vector<int32_t>& v) {
    std::vector<uint8_t> b;
    be_ints(b, v);
    return b;
  };
  {
    const double t = 1.0;
    Var v{"time_whole", {d_time}, kDouble, {}, {}, true};
    be_doubles(v.data, &t, 1);
    f.vars.push_back(v);
  }
  f.vars.push_back(Var{"eb_status", {d_blk}, kInt, {}, ints_of({1})});
  f.vars.push_back(Var{"eb_prop1", {d_blk}, kInt, {attr_text("name", "ID")}, ints_of({0})});
  for (int k = 0; k < 3; ++k) {
    Var v{std::string("coord") + "xyz"[k], {d_nodes}, kDouble, {}, {}};
    be_doubles(v.data, xyz.data() + k, (size_t)nn, 3);
    f.vars.push_back(v);
  }
  f.vars.push_back(Var{"eb_names", {d_blk, d_len_name}, kChar, {}, chars({""}, kLen)});
  f.vars.push_back(Var{"coor_names", {d_num_dim, d_len_name}, kChar, {}, chars({"x", "y", "z"}, kLen)});
  {
    std::vector<int32_t> nmap((size_t)nn), emap((size_t)n);
    for (int64_t i = 0; i < nn; ++i) nmap[(size_t)i] = (int32_t)(i + 1);
    for (int64_t i = 0; i < n; ++i) emap[(size_t)i] = (int32_t)(i + 1);
    f.vars.push_back(Var{"node_num_map", {d_nodes}, kInt, {}, ints_of(nmap)});
    f.vars.push_back(Var{"connect1", {d_in, d_per}, kInt, {attr_text("elem_type", "EDGE2")}, ints_of(conn)});
    f.vars.push_back(Var{"elem_num_map", {d_elem}, kInt, {}, ints_of(emap)});
  }
  const std::vector<std::string> names = {"aux_energy",        "aux_id",         "aux_n_progeny",    "aux_particle_type",
                                          "aux_seed_URR",      "aux_seed_source", "aux_seed_tracking", "aux_weight",
                                          "intersections",     "ray_id"};
  f.vars.push_back(Var{"name_elem_var", {d_nvar, d_len_name}, kChar, {}, chars(names, kLen)});
  f.vars.push_back(Var{"elem_var_tab", {d_blk, d_nvar}, kInt, {}, ints_of(std::vector<int32_t>(10, 1))});
  for (int vi = 0; vi < 10; ++vi) {
    std::vector<double> vals((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
      const mc_ray_segment& r = seg[i];
      double v = 0.0;
      switch (vi) {
        case 0: v = r.E; break;
        case 1: v = (double)r.id; break;
        case 6: v = (double)r.seed_tracking; break;
        case 7: v = r.wgt; break;
        case 8: v = (double)r.intersections; break;
        case 9: v = (double)(r.id - 1 - first_history); break;
        default: v = 0.0; break;
      }
      vals[(size_t)i] = v;
    }
    Var v{"vals_elem_var" + std::to_string(vi + 1) + "eb1", {d_time, d_in}, kDouble, {}, {}, true};
    be_doubles(v.data, vals.data(), vals.size());
    f.vars.push_back(v);
  }
  return write_nc(f, path);
}

// ---------------------------------------------------------------------------
// Reading: the tet mesh of an Exodus II file (MOOSE FileMeshGenerator for the
// meshes MaCaw traces on).  netCDF classic and 64-bit-offset files; element
// blocks must be 4-node tetrahedra; elements are numbered in block order;
// side sets give the boundary ids of their faces.
namespace {

struct NcVar {
  std::string name;
  std::vector<uint32_t> dims;
  std::map<std::string, std::string> text_attrs;
  int type = 0;
  uint64_t vsize = 0, begin = 0;
};

struct NcReader {
  FILE* fp = nullptr;
  int version = 0;
  std::vector<std::pair<std::string, uint64_t>> dims;
  std::vector<NcVar> vars;
  uint64_t recsize = 0;
  std::string err;
  std::vector<uint8_t> h;
  size_t pos = 0;

  ~NcReader() {
    if (fp) fclose(fp);
  }
  bool need(size_t n) {
    if (pos + n <= h.size()) return true;
    // the header is read in growing chunks until it parses
    const size_t want = std::max(h.size() * 2, pos + n + 65536);
    h.resize(want);
    fseek(fp, 0, SEEK_SET);
    const size_t got = fread(h.data(), 1, want, fp);
    h.resize(got);
    return pos + n <= h.size();
  }
  uint32_t u32() {
    if (!need(4)) throw std::runtime_error("truncated netCDF header");
    const uint32_t v = ((uint32_t)h[pos] << 24) | ((uint32_t)h[pos + 1] << 16) | ((uint32_t)h[pos + 2] << 8) | h[pos + 3];
    pos += 4;
    return v;
  }
  uint64_t u64() {
    const uint64_t hi = u32();
    return (hi << 32) | u32();
  }
  std::string name() {
    const uint32_t n = u32();
    if (!need((n + 3) / 4 * 4)) throw std::runtime_error("truncated netCDF header");
    std::string s(h.begin() + (long)pos, h.begin() + (long)pos + n);
    pos += (n + 3) / 4 * 4;
    return s;
  }
  void attrs(std::map<std::string, std::string>* text) {
    const uint32_t tag = u32(), n = u32();
    if (tag == 0 && n == 0) return;
    if (tag != kNcAttribute) throw std::runtime_error("bad netCDF attribute list");
    for (uint32_t i = 0; i < n; ++i) {
      const std::string an = name();
      const uint32_t type = u32(), cnt = u32();
      const size_t bytes = ((size_t)cnt * type_size((int)type) + 3) / 4 * 4;
      if (!need(bytes)) throw std::runtime_error("truncated netCDF header");
      if (text && type == kChar) {
        std::string v(h.begin() + (long)pos, h.begin() + (long)pos + cnt);
        while (!v.empty() && v.back() == 0) v.pop_back();
        (*text)[an] = v;
      }
      pos += bytes;
    }
  }
  bool open(const char* path) {
    fp = fopen(path, "rb");
    if (!fp) {
      err = std::string("cannot open ") + path;
      return false;
    }
    try {
      if (!need(8) || h[0] != 'C' || h[1] != 'D' || h[2] != 'F' || (h[3] != 1 && h[3] != 2)) {
        err = "not a netCDF classic or 64-bit-offset file (HDF5-based netCDF-4 files are not read)";
        return false;
      }
      version = h[3];
      pos = 4;
      u32();  // numrecs
      uint32_t tag = u32(), n = u32();
      if (tag == kNcDimension)
        for (uint32_t i = 0; i < n; ++i) {
          std::string dn = name();
          dims.push_back({dn, u32()});
        }
      attrs(nullptr);
      tag = u32();
      n = u32();
      if (tag == kNcVariable)
        for (uint32_t i = 0; i < n; ++i) {
          NcVar v;
          v.name = name();
          const uint32_t nd = u32();
          for (uint32_t k = 0; k < nd; ++k) v.dims.push_back(u32());
          attrs(&v.text_attrs);
          v.type = (int)u32();
          v.vsize = u32();
          v.begin = version == 1 ? u32() : u64();
          vars.push_back(v);
        }
      int n_rec = 0;
      for (auto& v : vars)
        if (is_record(v)) {
          recsize += v.vsize;
          ++n_rec;
        }
      if (n_rec == 1)  // one record variable: its records are not padded
        for (auto& v : vars)
          if (is_record(v)) recsize = count(v) * type_size(v.type);
    } catch (const std::exception& e) {
      err = e.what();
      return false;
    }
    return true;
  }
  bool is_record(const NcVar& v) const { return !v.dims.empty() && dims[v.dims[0]].second == 0; }
  uint64_t count(const NcVar& v) const {
    uint64_t c = 1;
    for (size_t k = is_record(v) ? 1 : 0; k < v.dims.size(); ++k) c *= dims[v.dims[k]].second;
    return c;
  }
  const NcVar* var(const std::string& n) const {
    for (auto& v : vars)
      if (v.name == n) return &v;
    return nullptr;
  }
  int64_t dim(const std::string& n) const {
    for (auto& d : dims)
      if (d.first == n) return (int64_t)d.second;
    return -1;
  }
  // values of v (first record for record variables) as doubles or ints
  bool raw(const NcVar& v, std::vector<uint8_t>& out) {
    const uint64_t bytes = count(v) * type_size(v.type);
    out.resize(bytes);
    if (fseeko(fp, (off_t)v.begin, SEEK_SET) != 0 || fread(out.data(), 1, bytes, fp) != bytes) {
      err = "cannot read variable " + v.name;
      return false;
    }
    return true;
  }
  bool doubles(const NcVar& v, std::vector<double>& out) {
    std::vector<uint8_t> b;
    if (!raw(v, b)) return false;
    const size_t n = (size_t)count(v);
    out.resize(n);
    for (size_t i = 0; i < n; ++i) {
      if (v.type == kDouble) {
        uint64_t u = 0;
        for (int k = 0; k < 8; ++k) u = (u << 8) | b[8 * i + k];
        memcpy(&out[i], &u, 8);
      } else if (v.type == kFloat) {
        uint32_t u = 0;
        for (int k = 0; k < 4; ++k) u = (u << 8) | b[4 * i + k];
        float fl;
        memcpy(&fl, &u, 4);
        out[i] = fl;
      } else {
        err = v.name + ": expected floating-point values";
        return false;
      }
    }
    return true;
  }
  bool ints(const NcVar& v, std::vector<int64_t>& out) {
    std::vector<uint8_t> b;
    if (!raw(v, b)) return false;
    const size_t n = (size_t)count(v);
    out.resize(n);
    for (size_t i = 0; i < n; ++i) {
      if (v.type == kInt) {
        uint32_t u = 0;
        for (int k = 0; k < 4; ++k) u = (u << 8) | b[4 * i + k];
        out[i] = (int32_t)u;
      } else {
        err = v.name + ": expected 32-bit integers";
        return false;
      }
    }
    return true;
  }
};

void put_err(char* buf, int64_t len, const std::string& s) {
  if (buf && len > 0) {
    const size_t n = std::min<size_t>(s.size(), (size_t)len - 1);
    memcpy(buf, s.data(), n);
    buf[n] = 0;
  }
}

// The whole read; fills the arrays when they are given.
int exodus_read(const char* path, int64_t* n_vtx, int64_t* n_tet, double* xyz, int32_t* tet_vtx,
                int32_t* tet_block, int32_t* tet_side_bid, char* err, int64_t err_len) {
  NcReader r;
  if (!path || !r.open(path)) {
    put_err(err, err_len, r.err.empty() ? "null path" : r.err);
    return MC_ERR_ARG;
  }
  auto fail = [&](const std::string& m) {
    put_err(err, err_len, std::string(path) + ": " + m);
    return MC_ERR_ARG;
  };
  if (r.dim("num_dim") != 3) return fail("only 3-D meshes are read");
  const int64_t nn = r.dim("num_nodes"), nblk = r.dim("num_el_blk");
  if (nn < 4 || nblk < 1) return fail("no nodes or no element blocks");
  int64_t ne = 0;
  for (int64_t b = 1; b <= nblk; ++b) {
    const NcVar* c = r.var("connect" + std::to_string(b));
    if (!c || c->dims.size() != 2) return fail("missing connect" + std::to_string(b));
    auto it = c->text_attrs.find("elem_type");
    std::string et = it == c->text_attrs.end() ? "" : it->second;
    for (auto& ch : et) ch = (char)toupper((unsigned char)ch);
    if (r.dims[c->dims[1]].second != 4 || et.compare(0, 3, "TET") != 0)
      return fail("element block " + std::to_string(b) + " is " + (et.empty() ? "untyped" : et) +
                  ": only 4-node tetrahedra (TETRA4) are tracked");
    ne += (int64_t)r.dims[c->dims[0]].second;
  }
  if (n_vtx) *n_vtx = nn;
  if (n_tet) *n_tet = ne;
  if (!xyz) return MC_OK;
  // coordinates
  const NcVar* cx = r.var("coordx");
  if (cx) {
    for (int k = 0; k < 3; ++k) {
      const NcVar* v = r.var(std::string("coord") + "xyz"[k]);
      std::vector<double> d;
      if (!v || !r.doubles(*v, d) || (int64_t)d.size() != nn) return fail("bad coord" + std::string(1, "xyz"[k]));
      for (int64_t i = 0; i < nn; ++i) xyz[3 * i + k] = d[(size_t)i];
    }
  } else {
    const NcVar* v = r.var("coord");
    std::vector<double> d;
    if (!v || !r.doubles(*v, d) || (int64_t)d.size() != 3 * nn) return fail("no coordinates");
    for (int k = 0; k < 3; ++k)
      for (int64_t i = 0; i < nn; ++i) xyz[3 * i + k] = d[(size_t)(k * nn + i)];
  }
  // blocks
  std::vector<int64_t> ids;
  if (const NcVar* p = r.var("eb_prop1")) {
    if (!r.ints(*p, ids)) return fail(r.err);
  }
  int64_t t0 = 0;
  for (int64_t b = 1; b <= nblk; ++b) {
    std::vector<int64_t> c;
    if (!r.ints(*r.var("connect" + std::to_string(b)), c)) return fail(r.err);
    const int32_t id = (int32_t)((int64_t)ids.size() >= b ? ids[(size_t)(b - 1)] : b);
    const int64_t n = (int64_t)c.size() / 4;
    for (int64_t i = 0; i < n; ++i) {
      for (int a = 0; a < 4; ++a) {
        const int64_t node = c[(size_t)(4 * i + a)] - 1;
        if (node < 0 || node >= nn) return fail("connectivity refers to a missing node");
        tet_vtx[4 * (t0 + i) + a] = (int32_t)node;
      }
      tet_block[t0 + i] = id;
    }
    t0 += n;
  }
  // side sets
  if (tet_side_bid) {
    for (int64_t i = 0; i < 4 * ne; ++i) tet_side_bid[i] = -1;
    const int64_t nss = r.dim("num_side_sets");
    std::vector<int64_t> sids;
    if (nss > 0)
      if (const NcVar* p = r.var("ss_prop1"))
        if (!r.ints(*p, sids)) return fail(r.err);
    for (int64_t s = 1; s <= nss; ++s) {
      const NcVar* ve = r.var("elem_ss" + std::to_string(s));
      const NcVar* vs = r.var("side_ss" + std::to_string(s));
      if (!ve || !vs) continue;  // an empty side set has no variables
      std::vector<int64_t> el, sd;
      if (!r.ints(*ve, el) || !r.ints(*vs, sd) || el.size() != sd.size()) return fail("bad side set");
      const int32_t id = (int32_t)((int64_t)sids.size() >= s ? sids[(size_t)(s - 1)] : s);
      for (size_t i = 0; i < el.size(); ++i) {
        if (el[i] < 1 || el[i] > ne || sd[i] < 1 || sd[i] > 4) return fail("side set entry out of range");
        tet_side_bid[4 * (el[i] - 1) + kFaceOfExoSide[sd[i]]] = id;
      }
    }
  }
  return MC_OK;
}

}  // namespace

extern "C" int mc_exodus_read_sizes(const char* path, int64_t* n_vtx, int64_t* n_tet, char* err, int64_t err_len) {
  if (!n_vtx || !n_tet) return MC_ERR_ARG;
  return exodus_read(path, n_vtx, n_tet, nullptr, nullptr, nullptr, nullptr, err, err_len);
}

extern "C" int mc_exodus_read(const char* path, double* xyz, int32_t* tet_vtx, int32_t* tet_block,
                              int32_t* tet_side_bid, char* err, int64_t err_len) {
  if (!xyz || !tet_vtx || !tet_block) return MC_ERR_ARG;
  return exodus_read(path, nullptr, nullptr, xyz, tet_vtx, tet_block, tet_side_bid, err, err_len);
}
