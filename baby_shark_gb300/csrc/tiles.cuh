// Active-tile lookup of a volume's internal levels: the value that the
// tree's `at` returns for a voxel outside every leaf whose 128^3 (level 1) or
// 4096^3 (level 2) node slot holds an active tile
// (internal_node/tree_node.rs:34-42, root_node/tree_node.rs:20-26).
#pragma once

#include "leaf_hash.cuh"
#include "volume_upper.cuh"

namespace bs {

struct TileLookup {
  LeafHash h1, h2;  // node origin -> index, per level
  const int* s1;    // slot states (-2: active tile)
  const float* t1;  // slot tile values
  const int* s2;
  const float* t2;
  int any;          // 0: the volume has no active tiles
};

// Value of voxel (x, y, z) from an active tile, for a voxel outside every leaf.
__device__ __forceinline__ bool tile_value(const TileLookup& T, int x, int y, int z, float& v) {
  if (!T.any) return false;
  const int n1 = T.h1.find(x & ~127, y & ~127, z & ~127);
  if (n1 >= 0) {
    const int slot = (((x >> 3) & 15) << 8) | (((y >> 3) & 15) << 4) | ((z >> 3) & 15);
    const uint64_t k = uint64_t(n1) * L1_SLOTS + slot;
    if (T.s1[k] != -2) return false;
    v = T.t1[k];
    return true;
  }
  const int n2 = T.h2.find(x & ~4095, y & ~4095, z & ~4095);
  if (n2 < 0) return false;
  const int slot = (((x >> 7) & 31) << 10) | (((y >> 7) & 31) << 5) | ((z >> 7) & 31);
  const uint64_t k = uint64_t(n2) * L2_SLOTS + slot;
  if (T.s2[k] != -2) return false;
  v = T.t2[k];
  return true;
}

}  // namespace bs
