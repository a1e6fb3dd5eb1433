// The reference's own winding-number tree on the GPU: the top-down "Area"
// SAH build of AABBTree (spatial_partitioning/aabb_tree.rs:118-199, 201-250,
// 422-514) with at most 3 triangles per leaf and depth 40, the far-field
// coefficients of compute_node_data (aabb_tree.rs:723-801), and a per-point
// traversal that sums in the order of fast_wn's recursion
// (aabb_tree.rs:662-691).  Same tree, same float32 operations, same sums:
// winding numbers equal the reference's bit for bit except where CUDA's
// atan2f and the host's differ in the last place.
#pragma once

#include <vector>

#include "bs_internal.cuh"

namespace bs {

// Node references: >= 0 an internal node (indexed by its split position - 1),
// < 0 a leaf ~p (p the position of its first triangle in leaf order).
struct RefTrees {
  DBuf<float4> rec_i;       // [n] 4 float4 per internal node: dipole xyz + far threshold, order-1 xyz + B0, B1..B4, B5..B8
  DBuf<int2> topo;          // [n] children of internal nodes
  DBuf<float4> open;        // [n] 3 float4 per internal node: both children's dipole + far threshold,
                            //     then (left ref, right ref, left leaf count, right leaf count) as int bits
  DBuf<float4> rec_l;       // [n] 4 float4 per leaf, at its first position
  DBuf<uint32_t> leaf_cnt;  // [n] triangles of the leaf starting at a position (0: none starts there)
  DBuf<float4> tri;         // [3n] triangles in leaf order
  DBuf<int> roots;          // [K] root reference of each mesh
  DBuf<float> rad_i, rad_l; // [n] node radii (compute_node_data, aabb_tree.rs:733-735)
  DBuf<int> flags;          // [n] 2 where an internal node has that id
  DBuf<uint32_t> tb;        // [K+1] first position of each mesh
  std::vector<int> h_roots;
  std::vector<float> h_beta;  // beta of the far thresholds in the records
  uint64_t nt = 0;
  int K = 0;
};

// Builds one tree per mesh over T (3 float4 per triangle, mesh m holding
// [h_tri_base[m], h_tri_base[m+1])), in triangle order as given, with the
// far thresholds of each mesh's accuracy scale h_beta[m].
void build_ref_trees(bs_ctx* ctx, const float4* T, uint64_t nt, int K, const uint32_t* h_tri_base,
                     const std::vector<float>& h_beta, RefTrees& out);

// Rewrites the far thresholds for other accuracy scales (one per mesh).
void ref_tree_set_beta(bs_ctx* ctx, RefTrees& t, const std::vector<float>& beta);

// Per-mesh parameters of the sign pass over band voxels.
struct RefSignMesh {
  int root;
  float h, beta, thresh;
};

// Signs the active voxels of K meshes (act[i] = brick << 9 | voxel; mesh m
// owns act[act_base[m], act_base[m+1]) and warps warp_base[m] ..
// warp_base[m+1] of 32 voxels each) with the winding number of their grid
// points: values[v] = +|d| when wn < thresh, else -|d|
// (mesh_to_volume.rs:245-280).  counters (device, 6 x u64, accumulated):
// warp node visits, far-field evaluations, exact solid angles, stack
// overflows, far-field evaluations and exact solid angles as the warps run
// them (a section any lane needs runs for the whole warp).
void ref_tree_sign(bs_ctx* ctx, const RefTrees& t, const uint32_t* act, const uint32_t* d_act_base,
                   const uint32_t* d_warp_base, uint64_t n_warps, int K, const RefSignMesh* d_meshes,
                   const int4* origins, float* values, unsigned long long* d_counters);

// WindingNumbers::approximate (aabb_tree.rs:654-660) at np device points of
// mesh 0's tree.
void ref_tree_points(bs_ctx* ctx, RefTrees& t, const float* d_pts, uint64_t np, float beta, float* d_out,
                     unsigned long long* d_counters);

}  // namespace bs
