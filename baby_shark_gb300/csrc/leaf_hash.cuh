// Open-addressing hash from a leaf origin to its index, used wherever a
// kernel needs a face neighbour (offset sweeps, dual contouring).
#pragma once

#include "bs_internal.cuh"

namespace bs {

constexpr unsigned long long HASH_EMPTY = ~0ull;

// (x, y, z) leaf origin -> 63-bit key, lexicographic in (x, y, z); origins
// are multiples of 8 within +-2^23 voxels.
__host__ __device__ __forceinline__ unsigned long long leaf_key(int x, int y, int z) {
  return (static_cast<unsigned long long>(static_cast<uint32_t>((x >> 3) + (1 << 20))) << 42) |
         (static_cast<unsigned long long>(static_cast<uint32_t>((y >> 3) + (1 << 20))) << 21) |
         static_cast<unsigned long long>(static_cast<uint32_t>((z >> 3) + (1 << 20)));
}

__device__ __forceinline__ uint32_t hash_slot(unsigned long long k, uint64_t mask) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return uint32_t(k & mask);
}

struct LeafHash {
  unsigned long long* keys = nullptr;  // [cap]
  int* vals = nullptr;                 // [cap]
  uint64_t mask = 0;                   // cap - 1 (cap is a power of two)

  // Index of the leaf at origin (x, y, z), or -1.  Probing is bounded by the capacity.
  __device__ __forceinline__ int find(int x, int y, int z) const {
    const unsigned long long k = leaf_key(x, y, z);
    uint32_t s = hash_slot(k, mask);
    for (uint64_t i = 0; i <= mask; ++i) {
      const unsigned long long c = keys[s];
      if (c == k) return vals[s];
      if (c == HASH_EMPTY) return -1;
      s = uint32_t((s + 1) & mask);
    }
    return -1;
  }
  // Inserts the key; returns the slot and sets `inserted` when this call
  // claimed it.  Returns -1 when the table is full.
  __device__ __forceinline__ int insert_key(int x, int y, int z, bool& inserted) const {
    const unsigned long long k = leaf_key(x, y, z);
    uint32_t s = hash_slot(k, mask);
    inserted = false;
    for (uint64_t i = 0; i <= mask; ++i) {
      const unsigned long long prev = atomicCAS(&keys[s], HASH_EMPTY, k);
      if (prev == HASH_EMPTY) {
        inserted = true;
        return int(s);
      }
      if (prev == k) return int(s);
      s = uint32_t((s + 1) & mask);
    }
    return -1;
  }
};

// Owns the storage of a LeafHash and fills it from leaf origins.
struct LeafHashBuf {
  DBuf<unsigned long long> keys;
  DBuf<int> vals;
  LeafHash h;
  void build(bs_ctx* ctx, const int4* origins, uint64_t n, uint64_t min_capacity);
};

}  // namespace bs
