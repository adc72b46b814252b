// SPDX-License-Identifier: MPL-2.0
// Pieces of the verification stage shared by the exact path
// (verification.cu) and the throughput path (verify_fast.cu).
#pragma once
#include "common.cuh"

namespace sym {

// Union-find over rows (set * nv + vertex): parent = own vertex for the
// rows whose flag is set, -1 for the others; unite_edges joins the allowed
// ends of every mesh edge within a set, always linking the larger root
// under the smaller, so a component's root is its smallest vertex.
__device__ __forceinline__ int32_t find_root(int32_t *parent, int32_t x) {
  for (int guard = 0; guard < (1 << 26); ++guard) {
    int32_t p = parent[x];
    if (p == x) return x;
    int32_t g = parent[p];
    if (g != p) parent[x] = g;  // path halving; parents only decrease
    x = p;
  }
  return -1;
}
__global__ void init_parents(const uint8_t *flags, uint64_t n, int32_t *parent, uint64_t nv);
__global__ void unite_edges(const uint64_t *nbr_off, const int32_t *nbr, uint64_t nv, uint64_t sets,
                            int32_t *parent_all, int *status);

// Linear BVH over the faces of a resident mesh, FP32 (throughput path).
struct Lbvh {
  uint64_t nv = 0, nf = 0;
  const int32_t *faces = nullptr;  // 3 x nf (the mesh's)
  float *xyz = nullptr;            // 3 x nv, FP32 copy of the vertices
  int32_t *child = nullptr;        // (nf - 1) x 2: >= 0 internal node, < 0 leaf ~face
  float *box = nullptr;            // (nf - 1) x 12: the two children's lo[3], hi[3]
  char *block = nullptr;           // owns every array above (cudaMalloc)
};

// Builds the LBVH on the device (synchronises); release with lbvh_free.
Lbvh lbvh_build(Call &call, const double *xyz, uint64_t nv, const int32_t *faces, uint64_t nf);
void lbvh_free(Lbvh &b);

}  // namespace sym
