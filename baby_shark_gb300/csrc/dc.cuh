// Shared declarations of the dual-contouring kernels (defined in dc.cu, also
// launched by the allocation-free entry point in dc_noalloc.cu).
#pragma once

#include "leaf_hash.cuh"
#include "tiles.cuh"

namespace bs {

struct DcVol {
  const int4* org;
  const float* val;
  const uint32_t* msk;
  LeafHash hash;
  TileLookup tiles;  // active tiles, read where a voxel lies outside every leaf (tiles.any == 0: none)
};

struct DcStats {
  int error;  // 1: gradient with no neighbours
};

// Launches of the kernels that read neighbour values (tiles: the volume has
// active tiles, read through the tree's `at`).
void launch_dc_edge_mask(bool tiles, const DcVol& V, uint64_t n, uint32_t* cm, uint32_t* ccnt, cudaStream_t s);
void launch_dc_edge_points(bool tiles, const DcVol& V, uint64_t n, const uint32_t* cm, const uint32_t* coff,
                           float* pts, DcStats* st, cudaStream_t s);
void launch_dc_cell_mask(bool tiles, const DcVol& V, uint64_t n, uint32_t* cellm, uint32_t* cellc, cudaStream_t s);
__global__ void k_dc_cell_points(DcVol V, uint64_t n, const uint32_t* __restrict__ cm,
                                 const uint32_t* __restrict__ coff, const float* __restrict__ pts,
                                 const uint32_t* __restrict__ cellm, const uint32_t* __restrict__ celloff,
                                 float* __restrict__ cells);
__global__ void k_dc_quads(DcVol V, uint64_t n, const uint32_t* __restrict__ cm, const uint32_t* __restrict__ cellm,
                           const uint32_t* __restrict__ celloff, const float* __restrict__ cells, float h,
                           uint64_t* __restrict__ vcount, const uint64_t* __restrict__ voff,
                           uint16_t* __restrict__ packed, float* __restrict__ tris);

}  // namespace bs
