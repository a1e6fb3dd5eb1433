// Internal-node levels of a volume (see volume_ops.cu): dense slot tables for
// the reference tree's InternalNode<4> (L1) and InternalNode<5> (L2) levels.
#pragma once

#include "bs_internal.cuh"

namespace bs {

constexpr int L1_LOG2 = 4, L1_SLOTS = 4096, L1_CHILD_SHIFT = 3;   // 16^3 leaves of 8^3
constexpr int L2_LOG2 = 5, L2_SLOTS = 32768, L2_CHILD_SHIFT = 7;  // 32^3 L1 nodes of 128^3
constexpr int L2_SHIFT = 12;                                      // L2 node = 4096^3 voxels
constexpr float FAR_F = 3.40282347e+38f;                          // f32::MAX, the reference's far()

struct Level {
  int log2 = 0, child_shift = 0, slots = 0;
  uint64_t n = 0;
  int4* d_key = nullptr;          // [n] node origin
  int* d_state = nullptr;         // [n][slots]: >= 0 child, -1 empty, -2 active tile
  float* d_tile = nullptr;        // [n][slots]
  uint8_t* d_first_neg = nullptr; // [n] first_value_sign() == Negative (after a flood fill)
  uint8_t* d_last_neg = nullptr;  // [n] last_value_sign() == Negative
  std::vector<int4> h_key;        // host copy of d_key
  Level() {}
  Level(int l, int cs) : log2(l), child_shift(cs), slots(1 << (3 * l)) {}
  void alloc(bs_ctx* ctx, uint64_t count);
  void free(bs_ctx* ctx);
  void sync_keys(bs_ctx* ctx);
};

}  // namespace bs

struct Upper;

namespace bs {

// Builds the internal levels from the leaves if the volume has none yet.
::Upper* ensure_upper(bs_ctx* ctx, bs_volume* v);
// Volume flood fill (all levels); keeps the signs CSG reads.
void flood_fill(bs_ctx* ctx, bs_volume* v);
// Rebuilds the volume's export list of active tiles from its levels.
void refresh_tiles(bs_ctx* ctx, bs_volume* v);

}  // namespace bs

struct Upper {
  bs::Level l1{bs::L1_LOG2, bs::L1_CHILD_SHIFT};
  bs::Level l2{bs::L2_LOG2, bs::L2_CHILD_SHIFT};
};
