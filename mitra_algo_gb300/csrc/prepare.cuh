// SPDX-License-Identifier: MPL-2.0
// GPU mesh preparation (prepare.cu): the reference's prepare() + topology()
// with every output in the call's workspace.
#pragma once
#include "common.cuh"

namespace sym {

struct PreparedDevice {
  uint64_t nv = 0, nf = 0, ne = 0, nbr_count = 0, rejected = 0, nonmanifold = 0, conflicts = 0;
  double *xyz = nullptr;     // 3 x nv
  int32_t *faces = nullptr;  // 3 x nf, the kept faces in input order
  double *fn = nullptr;      // 3 x nf unit face normals
  double *vn = nullptr;      // 3 x nv unit vertex normals
  double *w = nullptr;       // nv vertex weights (area / 3 per incident face)
  uint64_t *nbr_off = nullptr;
  int32_t *nbr = nullptr;
  uint64_t *inc_off = nullptr;
  int32_t *inc = nullptr;
  sym_edge *edges = nullptr;
  sym_model_context context{};
};

// Validates the options as the reference's validate_options does
// (src/core/prepare.cpp:85-100).
void validate_prepare_options(const sym_options &o);

// Uploads the mesh and prepares it; throws the reference's messages.
PreparedDevice prepare_device(Call &call, const sym_mesh_view &m, const sym_options &o);

}  // namespace sym
