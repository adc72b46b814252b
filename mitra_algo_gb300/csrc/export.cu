// SPDX-License-Identifier: MPL-2.0
// Binary result tables (sym_export_tables): the tables the reference writes
// as 17-digit text in export_result (src/io/export.cpp:37-98) -- features,
// pairs, votes, descriptors, the mesh -- written as binary column files.
// The SoA views are written as they are (one fwrite per column); only the
// derived columns are built here: each vertex's sampled / pruned flag
// (export.cpp:41-46), each vote's cluster, the last cluster listing it
// (export.cpp:55-58), and each descriptor's dimension (export.cpp:83-84).
// Host code only.
#include "common.cuh"

#include <cstdio>
#include <string>
#include <vector>

namespace sym {
namespace {

enum ColumnType : uint32_t { kInt32 = 1, kFloat64 = 2, kUInt8 = 3 };

struct Column {
  const char *name;
  uint32_t type;
  const void *data;
};

size_t type_bytes(uint32_t t) { return t == kFloat64 ? 8 : (t == kInt32 ? 4 : 1); }

struct File {
  std::FILE *f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

void write_table(const std::string &dir, const char *name, uint64_t rows,
                 const std::vector<Column> &cols) {
  for (const Column &c : cols)
    if (rows && !c.data) fail(SYM_INVALID_ARGUMENT, std::string("null column ") + c.name);
  const std::string path = dir + "/" + name;
  File out;
  out.f = std::fopen(path.c_str(), "wb");
  if (!out.f) fail(SYM_RUNTIME_ERROR, "Cannot write " + path);
  bool ok = true;
  auto put = [&](const void *p, size_t bytes) {
    if (bytes) ok = ok && std::fwrite(p, 1, bytes, out.f) == bytes;
  };
  const uint32_t ncols = uint32_t(cols.size()), zero = 0;
  put("SYMTAB01", 8);
  put(&rows, 8);
  put(&ncols, 4);
  put(&zero, 4);
  for (const Column &c : cols) {
    char label[24] = {};
    std::snprintf(label, sizeof(label), "%s", c.name);
    put(label, sizeof(label));
    put(&c.type, 4);
    put(&zero, 4);
  }
  uint64_t at = 24 + 32 * uint64_t(ncols);
  static const char pad[64] = {};
  for (const Column &c : cols) {
    const uint64_t aligned = (at + 63) / 64 * 64;
    put(pad, aligned - at);
    const uint64_t bytes = rows * type_bytes(c.type);
    put(c.data, bytes);
    at = aligned + bytes;
  }
  if (!ok || std::fflush(out.f) != 0) fail(SYM_RUNTIME_ERROR, "Output write failed");
}

void check_ids(const int32_t *ids, uint64_t n, uint64_t limit, const char *what) {
  if (n && !ids) fail(SYM_INVALID_ARGUMENT, std::string("null ") + what);
  for (uint64_t i = 0; i < n; ++i)
    if (ids[i] < 0 || uint64_t(ids[i]) >= limit)
      fail(SYM_INVALID_ARGUMENT, std::string(what) + " index out of range");
}

void export_tables(const sym_export_view &r, const std::string &dir) {
  const uint16_t probe = 1;
  if (*reinterpret_cast<const uint8_t *>(&probe) != 1)
    fail(SYM_RUNTIME_ERROR, "binary tables are little-endian");
  const uint64_t nv = r.mesh.vertices.count, nf = r.mesh.faces.count;
  if (r.features.count != nv) fail(SYM_INVALID_ARGUMENT, "SoA component lengths differ");
  check_ids(r.sample, r.sample_count, nv, "sample");
  check_ids(r.pruned, r.pruned_count, nv, "pruned");
  check_ids(r.pairs.a, r.pairs.count, nv, "pair");
  check_ids(r.pairs.b, r.pairs.count, nv, "pair");
  check_ids(r.mesh.faces.v0, nf, nv, "face");
  check_ids(r.mesh.faces.v1, nf, nv, "face");
  check_ids(r.mesh.faces.v2, nf, nv, "face");
  const sym_votes_view &v = r.votes;
  const sym_clusters_view &c = r.clusters;
  if (c.count && (!c.vote_offsets || !c.vote_indices))
    fail(SYM_INVALID_ARGUMENT, "null cluster membership");
  if (c.count && c.vote_offsets[0] != 0) fail(SYM_INVALID_ARGUMENT, "Invalid CSR offsets");
  for (uint64_t k = 0; k < c.count; ++k)
    if (c.vote_offsets[k + 1] < c.vote_offsets[k]) fail(SYM_INVALID_ARGUMENT, "Invalid CSR offsets");
  if (c.count) check_ids(c.vote_indices, c.vote_offsets[c.count], v.count, "cluster vote");

  std::vector<uint8_t> sampled(nv, 0), pruned(nv, 0);
  for (uint64_t i = 0; i < r.sample_count; ++i) sampled[r.sample[i]] = 1;
  for (uint64_t i = 0; i < r.pruned_count; ++i) pruned[r.pruned[i]] = 1;
  const sym_points_view &p = r.mesh.vertices;
  const sym_features_view &f = r.features;
  write_table(dir, "features.symt", nv,
              {{"x", kFloat64, p.x},        {"y", kFloat64, p.y},
               {"z", kFloat64, p.z},        {"kmin", kFloat64, f.kmin},
               {"kmax", kFloat64, f.kmax},  {"nx", kFloat64, f.normal.x},
               {"ny", kFloat64, f.normal.y}, {"nz", kFloat64, f.normal.z},
               {"dminx", kFloat64, f.dmin.x}, {"dminy", kFloat64, f.dmin.y},
               {"dminz", kFloat64, f.dmin.z}, {"dmaxx", kFloat64, f.dmax.x},
               {"dmaxy", kFloat64, f.dmax.y}, {"dmaxz", kFloat64, f.dmax.z},
               {"valid", kUInt8, f.valid},  {"sampled", kUInt8, sampled.data()},
               {"pruned", kUInt8, pruned.data()}});
  write_table(dir, "pairs.symt", r.pairs.count,
              {{"a", kInt32, r.pairs.a}, {"b", kInt32, r.pairs.b}});

  std::vector<int32_t> cluster(v.count, -1), dimension(v.count);
  for (uint64_t k = 0; k < c.count; ++k)
    for (uint64_t j = c.vote_offsets[k]; j < c.vote_offsets[k + 1]; ++j)
      cluster[c.vote_indices[j]] = int32_t(k);
  if (v.count && !v.kind) fail(SYM_INVALID_ARGUMENT, "null column type");
  for (uint64_t i = 0; i < v.count; ++i) dimension[i] = v.kind[i] == SYM_REFLECTION ? 4 : 12;
  static const char *rot[9] = {"r00", "r01", "r02", "r10", "r11", "r12", "r20", "r21", "r22"};
  std::vector<Column> vc{{"pair", kInt32, v.pair}, {"type", kUInt8, v.kind}};
  for (int k = 0; k < 9; ++k) vc.push_back({rot[k], kFloat64, v.rotation[k]});
  vc.push_back({"tx", kFloat64, v.translation[0]});
  vc.push_back({"ty", kFloat64, v.translation[1]});
  vc.push_back({"tz", kFloat64, v.translation[2]});
  vc.push_back({"nx", kFloat64, v.plane_normal[0]});
  vc.push_back({"ny", kFloat64, v.plane_normal[1]});
  vc.push_back({"nz", kFloat64, v.plane_normal[2]});
  vc.push_back({"d", kFloat64, v.plane_offset});
  vc.push_back({"cluster", kInt32, cluster.data()});
  write_table(dir, "votes.symt", v.count, vc);

  static const char *comp[12] = {"component0", "component1", "component2",  "component3",
                                 "component4", "component5", "component6",  "component7",
                                 "component8", "component9", "component10", "component11"};
  std::vector<Column> dc{{"dimension", kInt32, dimension.data()}};
  for (int k = 0; k < 12; ++k) dc.push_back({comp[k], kFloat64, v.descriptor[k]});
  write_table(dir, "descriptors.symt", v.count, dc);

  write_table(dir, "vertices.symt", nv, {{"x", kFloat64, p.x}, {"y", kFloat64, p.y}, {"z", kFloat64, p.z}});
  write_table(dir, "faces.symt", nf,
              {{"a", kInt32, r.mesh.faces.v0}, {"b", kInt32, r.mesh.faces.v1},
               {"c", kInt32, r.mesh.faces.v2}});
}

}  // namespace
}  // namespace sym

extern "C" sym_status sym_export_tables(const sym_export_view *result, const char *directory) {
  if (!result || !directory) {
    sym_error_text = "null argument";
    return SYM_INVALID_ARGUMENT;
  }
  try {
    sym::export_tables(*result, directory);
    return SYM_OK;
  } catch (const sym::Error &e) {
    sym_error_text = e.what();
    return e.status;
  } catch (const std::exception &e) {
    sym_error_text = e.what();
    return SYM_RUNTIME_ERROR;
  }
}
