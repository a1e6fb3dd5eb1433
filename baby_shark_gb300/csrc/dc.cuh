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

__global__ void k_dc_edge_mask(DcVol V, uint64_t n, uint32_t* __restrict__ cm, uint32_t* __restrict__ ccount);
__global__ void k_dc_edge_points(DcVol V, uint64_t n, const uint32_t* __restrict__ cm,
                                 const uint32_t* __restrict__ coff, float* __restrict__ pts, DcStats* st);
__global__ void k_dc_cell_mask(DcVol V, uint64_t n, uint32_t* __restrict__ cellm, uint32_t* __restrict__ ccount);
__global__ void k_dc_cell_points(DcVol V, uint64_t n, const uint32_t* __restrict__ cm,
                                 const uint32_t* __restrict__ coff, const float* __restrict__ pts,
                                 const uint32_t* __restrict__ cellm, const uint32_t* __restrict__ celloff,
                                 float* __restrict__ cells);
__global__ void k_dc_quads(DcVol V, uint64_t n, const uint32_t* __restrict__ cm, const uint32_t* __restrict__ cellm,
                           const uint32_t* __restrict__ celloff, const float* __restrict__ cells, float h,
                           uint64_t* __restrict__ vcount, const uint64_t* __restrict__ voff,
                           uint16_t* __restrict__ packed, float* __restrict__ tris);

}  // namespace bs
