// SPDX-License-Identifier: MPL-2.0
//
// ORACLE - test infrastructure only.  A command-line harness linked against
// the reference's own CPU library (deoksieze/Mitra_algo src/core, src/cpu,
// src/io compiled from the read-only reference tree by oracle/Makefile).  It
// runs the reference's public API (symmetry::prepare, make_cpu_backend()
// stage methods, point_triangle_distance2) on inputs read from a named-array
// file and writes every output to another named-array file.  The golden
// fixtures under tests/golden/ are produced with it (make_golden.py), and
// bench.py's reference arm may time it when it has been built.
//
// File format (little endian): "SYMD", then records of
//   u32 name length, name, u8 type ('d' f64, 'i' i32, 'u' u8, 'q' u64), u64
//   count, payload.
#include "symmetry/io.h"
#include "symmetry/math.h"
#include "symmetry/pipeline.h"
#include "symmetry/sampling.h"

#include <chrono>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

using namespace symmetry;

namespace {
struct Array {
  char type = 'd';
  std::vector<char> bytes;
  template <class T> std::vector<T> as() const {
    std::vector<T> v(bytes.size() / sizeof(T));
    std::memcpy(v.data(), bytes.data(), v.size() * sizeof(T));
    return v;
  }
};
using Archive = std::map<std::string, Array>;

Archive load(const std::string &path) {
  std::ifstream in(path, std::ios::binary);
  char magic[4];
  in.read(magic, 4);
  if (!in || std::memcmp(magic, "SYMD", 4) != 0)
    throw std::runtime_error("bad archive " + path);
  Archive a;
  while (true) {
    uint32_t len;
    if (!in.read(reinterpret_cast<char *>(&len), 4))
      break;
    std::string name(len, '\0');
    in.read(name.data(), len);
    Array arr;
    in.read(&arr.type, 1);
    uint64_t count;
    in.read(reinterpret_cast<char *>(&count), 8);
    size_t width = arr.type == 'd' || arr.type == 'q' ? 8 : (arr.type == 'i' ? 4 : 1);
    arr.bytes.resize(count * width);
    in.read(arr.bytes.data(), arr.bytes.size());
    a[name] = std::move(arr);
  }
  return a;
}

struct Writer {
  std::ofstream out;
  explicit Writer(const std::string &path) : out(path, std::ios::binary) {
    out.write("SYMD", 4);
  }
  void raw(const std::string &name, char type, const void *data, uint64_t count,
           size_t width) {
    uint32_t len = static_cast<uint32_t>(name.size());
    out.write(reinterpret_cast<const char *>(&len), 4);
    out.write(name.data(), len);
    out.write(&type, 1);
    out.write(reinterpret_cast<const char *>(&count), 8);
    out.write(static_cast<const char *>(data), static_cast<std::streamsize>(count * width));
  }
  void f64(const std::string &n, const std::vector<double> &v) { raw(n, 'd', v.data(), v.size(), 8); }
  void i32(const std::string &n, const std::vector<int32_t> &v) { raw(n, 'i', v.data(), v.size(), 4); }
  void u8(const std::string &n, const std::vector<uint8_t> &v) { raw(n, 'u', v.data(), v.size(), 1); }
  void u64(const std::string &n, const std::vector<uint64_t> &v) { raw(n, 'q', v.data(), v.size(), 8); }
  void text(const std::string &n, const std::string &s) { raw(n, 'u', s.data(), s.size(), 1); }
};

std::vector<double> f64(const Archive &a, const std::string &n) { return a.at(n).as<double>(); }
std::vector<int32_t> i32(const Archive &a, const std::string &n) { return a.at(n).as<int32_t>(); }
double scalar(const Archive &a, const std::string &n) { return f64(a, n).at(0); }
bool has(const Archive &a, const std::string &n) { return a.count(n) != 0; }

Options options_from(const Archive &a) {
  Options o;
  auto get = [&](const char *n, double &v) { if (has(a, n)) v = scalar(a, n); };
  get("sample_ratio", o.sample_ratio);
  get("prune", o.prune);
  get("pair_threshold", o.pair_threshold);
  get("bandwidth", o.bandwidth);
  get("verify_threshold", o.verify_threshold);
  auto geti = [&](const char *n, int &v) { if (has(a, n)) v = static_cast<int>(scalar(a, n)); };
  geti("smoothing", o.smoothing);
  geti("subdivide", o.subdivide);
  geti("max_iterations", o.max_iterations);
  geti("max_clusters", o.max_clusters);
  auto getu = [&](const char *n, std::uint64_t &v) {
    if (has(a, n)) v = a.at(n).as<uint64_t>().at(0);
  };
  getu("seed", o.seed);
  getu("max_pairs", o.max_pairs);
  getu("max_votes", o.max_votes);
  if (has(a, "patching")) o.patching = scalar(a, "patching") != 0;
  return o;
}

Mesh mesh_from(const Archive &a) {
  Mesh m;
  m.vertices.x = f64(a, "vx");
  m.vertices.y = f64(a, "vy");
  m.vertices.z = f64(a, "vz");
  m.faces.component[0] = i32(a, "f0");
  m.faces.component[1] = i32(a, "f1");
  m.faces.component[2] = i32(a, "f2");
  return m;
}

Features features_from(const Archive &a, Offset n) {
  Features f;
  f.resize(n);
  const char *lanes[9] = {"nx", "ny", "nz", "dminx", "dminy", "dminz", "dmaxx", "dmaxy", "dmaxz"};
  std::vector<double> *dst[9] = {&f.normal.x, &f.normal.y, &f.normal.z,
                                 &f.dmin.x,   &f.dmin.y,   &f.dmin.z,
                                 &f.dmax.x,   &f.dmax.y,   &f.dmax.z};
  for (int k = 0; k < 9; ++k)
    if (has(a, lanes[k])) *dst[k] = f64(a, lanes[k]);
  if (has(a, "kmin")) f.kmin = f64(a, "kmin");
  if (has(a, "kmax")) f.kmax = f64(a, "kmax");
  if (has(a, "valid")) f.valid = a.at("valid").as<uint8_t>();
  return f;
}

std::string rng_text(const std::mt19937_64 &r) {
  std::stringstream s;
  s << r;
  return s.str();
}

void write_features(Writer &w, const Features &f) {
  w.f64("nx", f.normal.x), w.f64("ny", f.normal.y), w.f64("nz", f.normal.z);
  w.f64("dminx", f.dmin.x), w.f64("dminy", f.dmin.y), w.f64("dminz", f.dmin.z);
  w.f64("dmaxx", f.dmax.x), w.f64("dmaxy", f.dmax.y), w.f64("dmaxz", f.dmax.z);
  w.f64("kmin", f.kmin), w.f64("kmax", f.kmax), w.u8("valid", f.valid);
}

void write_votes(Writer &w, const Votes &v, const std::string &p = "") {
  w.i32(p + "vote_pair", v.pairs);
  std::vector<uint8_t> kind;
  for (auto k : v.kind) kind.push_back(static_cast<uint8_t>(k));
  w.u8(p + "vote_kind", kind);
  for (int k = 0; k < 9; ++k) w.f64(p + "rot" + std::to_string(k), v.rotation.component[k]);
  w.f64(p + "tx", v.translation.x), w.f64(p + "ty", v.translation.y), w.f64(p + "tz", v.translation.z);
  w.f64(p + "pnx", v.plane_normal.x), w.f64(p + "pny", v.plane_normal.y), w.f64(p + "pnz", v.plane_normal.z);
  w.f64(p + "poff", v.plane_offset);
  for (int k = 0; k < 12; ++k) w.f64(p + "desc" + std::to_string(k), v.descriptor.component[k]);
}

Votes votes_from(const Archive &a) {
  Votes v;
  v.pairs = i32(a, "vote_pair");
  for (auto k : a.at("vote_kind").as<uint8_t>()) v.kind.push_back(static_cast<TransformKind>(k));
  for (int k = 0; k < 9; ++k) v.rotation.component[k] = f64(a, "rot" + std::to_string(k));
  v.translation.x = f64(a, "tx"), v.translation.y = f64(a, "ty"), v.translation.z = f64(a, "tz");
  v.plane_normal.x = f64(a, "pnx"), v.plane_normal.y = f64(a, "pny"), v.plane_normal.z = f64(a, "pnz");
  v.plane_offset = f64(a, "poff");
  for (int k = 0; k < 12; ++k) v.descriptor.component[k] = f64(a, "desc" + std::to_string(k));
  return v;
}

void write_clusters(Writer &w, const Clusters &c) {
  std::vector<uint8_t> refl;
  std::vector<double> rot, tr, pn, off;
  for (const auto &r : c.records) {
    refl.push_back(r.reflection);
    rot.insert(rot.end(), r.rotation.begin(), r.rotation.end());
    tr.insert(tr.end(), {r.translation.x, r.translation.y, r.translation.z});
    pn.insert(pn.end(), {r.plane_normal.x, r.plane_normal.y, r.plane_normal.z});
    off.push_back(r.plane_offset);
  }
  w.u8("cl_reflection", refl), w.f64("cl_rotation", rot), w.f64("cl_translation", tr);
  w.f64("cl_plane_normal", pn), w.f64("cl_plane_offset", off);
  w.u64("cl_vote_offsets", c.votes.offsets), w.i32("cl_vote_indices", c.votes.indices);
}

Clusters clusters_from(const Archive &a) {
  Clusters c;
  auto refl = a.at("cl_reflection").as<uint8_t>();
  auto rot = f64(a, "cl_rotation"), tr = f64(a, "cl_translation"),
       pn = f64(a, "cl_plane_normal"), off = f64(a, "cl_plane_offset");
  for (size_t i = 0; i < refl.size(); ++i) {
    ClusterRecord r{};
    r.reflection = refl[i] != 0;
    for (int k = 0; k < 9; ++k) r.rotation[k] = rot[9 * i + k];
    r.translation = {tr[3 * i], tr[3 * i + 1], tr[3 * i + 2]};
    r.plane_normal = {pn[3 * i], pn[3 * i + 1], pn[3 * i + 2]};
    r.plane_offset = off[i];
    c.append(r, {});
  }
  return c;
}

void write_verification(Writer &w, const Verification &v) {
  w.u64("ver_side_a_offsets", v.side_a.offsets), w.i32("ver_side_a", v.side_a.indices);
  w.u64("ver_side_b_offsets", v.side_b.offsets), w.i32("ver_side_b", v.side_b.indices);
  w.u64("ver_patches_a_groups", v.patches_a.groups);
  w.u64("ver_patches_a_offsets", v.patches_a.rows.offsets);
  w.i32("ver_patches_a_indices", v.patches_a.rows.indices);
  w.u64("ver_patches_b_groups", v.patches_b.groups);
  w.u64("ver_patches_b_offsets", v.patches_b.rows.offsets);
  w.i32("ver_patches_b_indices", v.patches_b.rows.indices);
  w.f64("ver_coverage", v.coverage), w.f64("ver_rms", v.rms);
}

void write_topology(Writer &w, const Prepared &p) {
  w.f64("vx", p.mesh.vertices.x), w.f64("vy", p.mesh.vertices.y), w.f64("vz", p.mesh.vertices.z);
  w.i32("f0", p.mesh.faces.component[0]), w.i32("f1", p.mesh.faces.component[1]);
  w.i32("f2", p.mesh.faces.component[2]);
  const Topology &t = p.topology;
  w.f64("vnx", t.normals.x), w.f64("vny", t.normals.y), w.f64("vnz", t.normals.z);
  w.f64("fnx", t.face_normals.x), w.f64("fny", t.face_normals.y), w.f64("fnz", t.face_normals.z);
  w.f64("weights", t.weights);
  w.u64("nbr_offsets", t.neighbors.offsets), w.i32("nbr_indices", t.neighbors.indices);
  w.u64("inc_offsets", t.incident_faces.offsets), w.i32("inc_indices", t.incident_faces.indices);
  std::vector<int32_t> edges;
  for (const auto &e : t.edges) edges.insert(edges.end(), {e.lo, e.hi, e.a, e.b, e.face0, e.face1});
  w.i32("edges", edges);
  w.f64("box_size", {p.context.box_size});
  w.f64("center", {p.context.center.x, p.context.center.y, p.context.center.z});
  w.i32("diagnostics", {p.diagnostics.rejected_faces, p.diagnostics.nonmanifold_edges,
                        p.diagnostics.orientation_conflicts});
}

double ms_since(std::chrono::steady_clock::time_point t) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
}

void run(const std::string &mode, const Archive &in, Writer &w) {
  auto cpu = make_cpu_backend();
  Options o = options_from(in);
  if (mode == "prepare") {
    write_topology(w, prepare(mesh_from(in), o));
  } else if (mode == "detect") {
    // The stages of src/core/pipeline.cpp:5-52, each timed and dumped.
    std::vector<double> times;
    auto t0 = std::chrono::steady_clock::now();
    Prepared p = prepare(mesh_from(in), o);
    times.push_back(ms_since(t0));
    write_topology(w, p);
    auto m = p.mesh.as_view();
    auto t = p.topology.as_view();
    std::mt19937_64 random(o.seed);
    t0 = std::chrono::steady_clock::now();
    Features f = cpu->curvature(m, t, o);
    times.push_back(ms_since(t0));
    write_features(w, f);
    t0 = std::chrono::steady_clock::now();
    Selection s = cpu->select(m, f.as_view(), t.weights, o, random);
    times.push_back(ms_since(t0));
    w.i32("sample", s.sample), w.i32("pruned", s.pruned);
    w.text("rng_after_select", rng_text(random));
    t0 = std::chrono::steady_clock::now();
    Pairs pairs = cpu->pairing(m, f.as_view(), view(s.pruned), p.context, o);
    times.push_back(ms_since(t0));
    w.i32("pair_a", pairs.a), w.i32("pair_b", pairs.b);
    t0 = std::chrono::steady_clock::now();
    Votes votes = cpu->transformations(m, f.as_view(), pairs.as_view(), p.context, o);
    times.push_back(ms_since(t0));
    write_votes(w, votes);
    t0 = std::chrono::steady_clock::now();
    ClusterOutput c = cpu->clustering(votes.as_view(), p.context, o, random);
    times.push_back(ms_since(t0));
    write_clusters(w, c.clusters);
    w.i32("limited_iterations", {c.limited_iterations});
    w.text("rng_after_clustering", rng_text(random));
    if (o.patching) {
      t0 = std::chrono::steady_clock::now();
      Verification v = cpu->verification(m, t, c.clusters.as_view(), p.context, o);
      times.push_back(ms_since(t0));
      write_verification(w, v);
    }
    w.f64("stage_ms", times);
  } else if (mode == "export") {
    // The reference's detect() and export_result() (src/core/pipeline.cpp:5-52,
    // src/io/export.cpp:37-189) into the directory given as text input "dir".
    const Array &d = in.at("dir");
    Result r = detect(mesh_from(in), o, *cpu);
    auto t0 = std::chrono::steady_clock::now();
    export_result(r, std::string(d.bytes.begin(), d.bytes.end()));
    w.f64("export_ms", {ms_since(t0)});
    w.i32("pairs", {int32_t(r.pairs.size())}), w.i32("votes", {int32_t(r.votes.size())});
  } else if (mode == "curvature") {
    Prepared p = prepare(mesh_from(in), o);
    write_topology(w, p);
    write_features(w, cpu->curvature(p.mesh.as_view(), p.topology.as_view(), o));
  } else if (mode == "select") {
    Mesh m;
    m.vertices.x = f64(in, "vx"), m.vertices.y = f64(in, "vy"), m.vertices.z = f64(in, "vz");
    Features f = features_from(in, m.vertices.size());
    auto weights = f64(in, "weights");
    std::mt19937_64 random(o.seed);
    Selection s = cpu->select(m.as_view(), f.as_view(), view(weights), o, random);
    w.i32("sample", s.sample), w.i32("pruned", s.pruned);
    w.text("rng_after_select", rng_text(random));
  } else if (mode == "pairing") {
    Mesh m;
    m.vertices.x = f64(in, "vx"), m.vertices.y = f64(in, "vy"), m.vertices.z = f64(in, "vz");
    Features f = features_from(in, m.vertices.size());
    auto sel = i32(in, "selected");
    ModelContext ctx{scalar(in, "box_size"), {}};
    auto t0 = std::chrono::steady_clock::now();
    Pairs p = cpu->pairing(m.as_view(), f.as_view(), view(sel), ctx, o);
    w.f64("stage_ms", {ms_since(t0)});
    w.i32("pair_a", p.a), w.i32("pair_b", p.b);
  } else if (mode == "transformations") {
    Mesh m;
    m.vertices.x = f64(in, "vx"), m.vertices.y = f64(in, "vy"), m.vertices.z = f64(in, "vz");
    Features f = features_from(in, m.vertices.size());
    Pairs pairs;
    pairs.a = i32(in, "pair_a"), pairs.b = i32(in, "pair_b");
    auto c = f64(in, "center");
    ModelContext ctx{scalar(in, "box_size"), {c[0], c[1], c[2]}};
    write_votes(w, cpu->transformations(m.as_view(), f.as_view(), pairs.as_view(), ctx, o));
  } else if (mode == "clustering") {
    Votes votes = votes_from(in);
    auto c = f64(in, "center");
    ModelContext ctx{scalar(in, "box_size"), {c[0], c[1], c[2]}};
    std::mt19937_64 random(o.seed);
    auto t0 = std::chrono::steady_clock::now();
    ClusterOutput out = cpu->clustering(votes.as_view(), ctx, o, random);
    w.f64("stage_ms", {ms_since(t0)});
    write_clusters(w, out.clusters);
    w.i32("limited_iterations", {out.limited_iterations});
    w.text("rng_after_clustering", rng_text(random));
  } else if (mode == "verification") {
    Prepared p = prepare(mesh_from(in), o);
    Clusters c = clusters_from(in);
    write_verification(w, cpu->verification(p.mesh.as_view(), p.topology.as_view(),
                                             c.as_view(), p.context, o));
  } else if (mode == "triangles") {
    auto q = f64(in, "queries");
    std::vector<double> d;
    for (size_t i = 0; i + 12 <= q.size(); i += 12)
      d.push_back(point_triangle_distance2({q[i], q[i + 1], q[i + 2]}, {q[i + 3], q[i + 4], q[i + 5]},
                                           {q[i + 6], q[i + 7], q[i + 8]}, {q[i + 9], q[i + 10], q[i + 11]}));
    w.f64("distances", d);
  } else if (mode == "rng") {
    std::mt19937_64 random(o.seed);
    w.text("rng_seeded", rng_text(random));
    std::vector<uint64_t> draws;
    for (int i = 0; i < 1000; ++i) draws.push_back(random());
    w.u64("draws", draws);
    w.text("rng_after_draws", rng_text(random));
  } else {
    throw std::runtime_error("unknown mode " + mode);
  }
}
} // namespace

int main(int argc, char **argv) {
  if (argc != 4) {
    std::cerr << "usage: ref_harness MODE IN.bin OUT.bin\n";
    return 2;
  }
  Writer w(argv[3]);
  try {
    run(argv[1], load(argv[2]), w);
  } catch (const std::invalid_argument &e) {
    w.text("error_kind", "invalid_argument"), w.text("error", e.what());
  } catch (const std::overflow_error &e) {
    w.text("error_kind", "overflow_error"), w.text("error", e.what());
  } catch (const std::exception &e) {
    w.text("error_kind", "runtime_error"), w.text("error", e.what());
  }
  return 0;
}
