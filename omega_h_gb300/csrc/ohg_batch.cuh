// Disjoint unions of meshes for batched passes (see ohg_batch.cu).
#pragma once
#include <vector>

#include "ohg_mesh.cuh"

namespace ohg {

// class ids of part k are stored as class_id + k * kPartStride in a union
constexpr LO kPartStride = 1 << 20;
constexpr int kMaxParts = 2047;

// The union of meshes of one dimension; every class id must lie in
// [0, kPartStride).  Cached lengths and qualities are kept when all parts
// have them.
Mesh concat_meshes(const std::vector<Mesh*>& ms);
// The K parts of a union after any number of adapt passes.  The parts share
// the union's device buffers (no copies); the union is left modified.
std::vector<Mesh> split_mesh(Mesh& u, int K);

}  // namespace ohg
