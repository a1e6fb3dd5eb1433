/*
 * baby_shark_gb300 — C ABI of the GB300 (sm_103a) implementation of
 * baby_shark's implicit-modelling path: mesh -> narrow-band signed distance
 * volume (exact point–triangle distances, fast-winding-number signs),
 * volume booleans and offset, and dual-contouring extraction.
 *
 * The reference (crate baby_shark v0.3.12) is a Rust library with no FFI;
 * each entry point below replaces one public Rust method, cited as
 * file:line inside the reference crate.  A Rust wrapper binds these symbols
 * with `extern "C"` and keeps the crate's builder API on top.
 *
 * Conventions
 *  - Plain pointers and sizes only.  Arrays named h_* are host memory,
 *    d_* device memory of the context's device.
 *  - Every call returns a bs_status; results come back through out-params.
 *  - All work of a context is ordered on its CUDA stream.  Entry points that
 *    return sizes or host data synchronise that stream before returning.
 *  - One context per host thread; contexts are independent.
 *  - A volume belongs to the context that made it.  Boolean operations
 *    consume both operands, like the reference's `Volume::union(self, other)`.
 *  - Voxel storage: leaves (bricks) of 8^3 voxels whose origins are
 *    multiples of 8 in integer grid coordinates (grid point i sits at i*h).
 *    Inside a leaf, voxel (x,y,z) has index x<<6 | y<<3 | z; its active bit is
 *    bit (index & 31) of mask word (index >> 5).
 */
#ifndef BABY_SHARK_GB300_H
#define BABY_SHARK_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bs_status {
  BS_OK = 0,
  BS_ERR_INVALID_ARG = 1,  /* null pointer, bad size, unknown option */
  BS_ERR_EMPTY = 2,        /* empty mesh: the reference's convert() returns None */
  BS_ERR_OOM = 3,          /* device allocation failed */
  BS_ERR_CAPACITY = 4,     /* a grid or table bound was exceeded */
  BS_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
  BS_ERR_CUDA = 6,         /* CUDA runtime error (see bs_ctx_last_error) */
  BS_ERR_UNSUPPORTED = 7,  /* input the reference panics on (e.g. a gradient with no neighbours in DC) */
  BS_ERR_NO_DEVICE = 8     /* no CUDA device / driver */
} bs_status;

typedef struct bs_ctx bs_ctx;
typedef struct bs_volume bs_volume;

/* ---------------------------------------------------------------- context */
/* No reference counterpart: the crate runs on rayon's implicit global pool
 * and owns its trees in Box allocations; a context holds what that takes here
 * (device, stream, stream-ordered memory pool, launch shapes, counters).
 * Creates a context on `device`.  `stream` is a cudaStream_t to run on, or
 * NULL for a stream the context creates and owns. */
bs_status bs_ctx_create(int device, void* stream, bs_ctx** out);
bs_status bs_ctx_destroy(bs_ctx* ctx);
/* The cudaStream_t all work of the context is ordered on. */
void* bs_ctx_stream(bs_ctx* ctx);
bs_status bs_ctx_synchronize(bs_ctx* ctx);
/* Number of kernels this library launched on the context so far. */
uint64_t bs_ctx_kernel_launches(const bs_ctx* ctx);
/* Text of the last error on the context ("" if none). */
const char* bs_ctx_last_error(const bs_ctx* ctx);
const char* bs_status_string(bs_status s);

/* ------------------------------------------------------- diagnostics ---- */
/* These have no counterpart in the reference; they expose measurements of
 * this implementation.  Stage timing brackets every kernel launch of the
 * context with CUDA events on its stream (off by default). */
bs_status bs_ctx_set_stage_timing(bs_ctx* ctx, int enable);
/* Resolves the recorded events (synchronising them) and returns the number
 * of distinct kernel names timed so far. */
bs_status bs_ctx_stage_count(bs_ctx* ctx, int* n_stages);
/* Name (valid until the next reset), total milliseconds and launch count of stage i. */
bs_status bs_ctx_stage_info(bs_ctx* ctx, int i, const char** name, double* total_ms, uint64_t* launches);
bs_status bs_ctx_stage_reset(bs_ctx* ctx);
/* Counters of the last mesh -> volume call: [0] triangles, [1] sub-triangles,
 * [2] (brick, sub-triangle) pairs, [3] (voxel, sub-triangle) pairs,
 * [4] leaves, [5] active voxels, [6] warp-level node visits of the
 * winding-number pass, [7] warp-level far-field evaluations (low 32 bits) and
 * exact solid angles (high 32 bits).  A dual contouring call overwrites
 * [6] and [7] with its crossing and cell counts, an offset call with its
 * relaxation phases (persistent launches, one or more per sweep direction)
 * and leaf sweeps over the 8 sweep directions. */
bs_status bs_ctx_last_stats(const bs_ctx* ctx, uint64_t* out8);
/* The same counters and more: [0..7] as above, [8] which call wrote them
 * (bs_stats_kind), [9] (voxel, sub-triangle) pairs whose exact distance a
 * mesh -> volume call evaluated after culling (the rest provably could not
 * lower their voxel's minimum), [10] far-field evaluations and [11] exact
 * solid angles of the winding-number pass in 64 bits (per voxel or point on
 * the reference's tree, per warp on the library's PLOC tree), [12] which tree
 * (0 the reference's, 1 PLOC), [13] and [14] on the reference's tree the
 * far-field evaluations and solid angles as its warps execute them (a
 * section that any lane of a warp needs runs for all 32), [15] zero. */
enum bs_stats_kind {
  BS_STATS_NONE = 0,
  BS_STATS_MESH_TO_VOLUME = 1,
  BS_STATS_OFFSET = 2,
  BS_STATS_DUAL_CONTOURING = 3,
  BS_STATS_WINDING_NUMBERS = 4
};
bs_status bs_ctx_last_counters(const bs_ctx* ctx, uint64_t* out16);
/* Device memory of the context's stream-ordered pool in bytes: in use now,
 * the most in use since creation or the last reset, and reserved from the
 * device (freed blocks stay reserved for reuse).  No reference counterpart. */
bs_status bs_ctx_memory(bs_ctx* ctx, uint64_t* used, uint64_t* used_high, uint64_t* reserved);
/* Resets the high-water mark of bs_ctx_memory; with trim != 0 also returns
 * the pool's unused reserved memory to the device. */
bs_status bs_ctx_memory_reset(bs_ctx* ctx, int trim);
/* Measured FP32 FMA throughput of the context's device in TFLOP/s (a timed
 * FFMA loop over all SMs); the denominator of FP32-bound roofline fractions. */
bs_status bs_diag_fp32_peak(bs_ctx* ctx, double* tflops);
/* Checks the shared-reciprocal division of the winding-number kernels
 * (Markstein's: q0 = RN(a * RN(1/b)), one fused correction) against CUDA's
 * IEEE division on every pair of significands a, b in [1, 2) — every
 * b_stride-th divisor, every dividend; b_stride 1 covers all 2^46 pairs —
 * and returns the number of differing quotients and of pairs tested. */
bs_status bs_diag_check_division(bs_ctx* ctx, uint32_t b_stride, uint64_t* mismatches, uint64_t* tested);
/* Exact generalised winding numbers of n_points points (device float3) with
 * respect to a mesh (device arrays): the direct sum over every triangle of
 * the solid angle of aabb_tree.rs:582-615, summed in double into d_out.  A
 * validation instrument for the approximate sign pass (no reference
 * counterpart: the reference only has the tree approximation). */
bs_status bs_winding_numbers_exact(bs_ctx* ctx, const float* d_xyz, uint64_t nv, const uint32_t* d_tri,
                                   uint64_t nt, const float* d_points, uint64_t n_points, double* d_out);

/* ----------------------------------------------------- mesh -> volume ---- */
typedef struct bs_m2v_params {
  float voxel_size;    /* MeshToVolume::with_voxel_size   (mesh_to_volume.rs:40-50) */
  int32_t band_width;  /* MeshToVolume::with_narrow_band_width (mesh_to_volume.rs:28-37) */
  float wn_beta;       /* far-field accuracy scale; the reference uses 2.0 (mesh_to_volume.rs:264) */
  float wn_threshold;  /* wn < threshold => outside; the reference uses 0.2 (mesh_to_volume.rs:266) */
  int32_t wn_order;    /* far-field expansion order: 2 as the reference (aabb_tree.rs:662-691), or 3
                          (the third-order term the reference leaves undone, aabb_tree.rs:706; needs
                          wn_tree 1) */
  int32_t wn_tree;     /* 0: the reference's own tree — the top-down SAH build of AABBTree::top_down::<Area>
                          with 3 triangles per leaf (aabb_tree.rs:118-199, 422-514, 636-644), one traversal
                          per voxel summing wn(left) + wn(right) as fast_wn recurses (aabb_tree.rs:662-691):
                          signs equal the reference's bit for bit.  1: this library's PLOC tree with a
                          warp-coherent traversal (faster; signs differ only where the winding number is
                          within the far-field approximation error of the threshold).  All meshes of a
                          batch use the same value. */
} bs_m2v_params;

/* Fills `p` with the reference's defaults (voxel 1, band 0, beta 2, threshold 0.2, the reference's tree). */
void bs_m2v_params_default(bs_m2v_params* p);

/* MeshToVolume::convert (mesh_to_volume.rs:52-73) on an indexed triangle mesh
 * in HOST memory: h_xyz[3*nv] vertex positions, h_tri[3*nt] vertex indices.
 * Returns BS_ERR_EMPTY where the reference returns None (no triangles). */
bs_status bs_mesh_to_volume(bs_ctx* ctx, const float* h_xyz, uint64_t nv, const uint32_t* h_tri,
                            uint64_t nt, const bs_m2v_params* params, bs_volume** out);

/* Same as bs_mesh_to_volume with the mesh already in device memory. */
bs_status bs_mesh_to_volume_device(bs_ctx* ctx, const float* d_xyz, uint64_t nv,
                                   const uint32_t* d_tri, uint64_t nt,
                                   const bs_m2v_params* params, bs_volume** out);

/* A batch of meshes in one set of launches: n_meshes meshes whose vertices
 * (3 floats each) and triangles (3 uint32 each, indices local to the mesh's
 * own vertices) are concatenated in mesh order; vertex_counts[m] and
 * triangle_counts[m] give each mesh's share and params[m] its
 * MeshToVolume settings.  out[m] receives mesh m's volume, or NULL for a mesh
 * without triangles (convert's None).  Each volume equals what
 * bs_mesh_to_volume returns for that mesh alone.  No reference counterpart:
 * the reference converts one mesh per call. */
bs_status bs_mesh_to_volume_batch(bs_ctx* ctx, uint64_t n_meshes, const float* h_xyz, const uint64_t* vertex_counts,
                                  const uint32_t* h_tri, const uint64_t* triangle_counts,
                                  const bs_m2v_params* params, bs_volume** out);
bs_status bs_mesh_to_volume_batch_device(bs_ctx* ctx, uint64_t n_meshes, const float* d_xyz,
                                         const uint64_t* vertex_counts, const uint32_t* d_tri,
                                         const uint64_t* triangle_counts, const bs_m2v_params* params,
                                         bs_volume** out);
/* Autotuner (no reference counterpart): converts the given mesh (device
 * arrays) once per candidate — the distance pass with 64 / 128 / 256 threads
 * per brick and tiles of 8 / 16 / 32 sub-triangles per warp (256 threads take
 * tiles of 8 or 16), the sign pass with 2 / 4 / 8 warps per block, two rounds
 * — and keeps the fastest of each pass for the context's later conversions
 * (results do not depend on them).  h_choice[3]: the chosen threads per
 * brick, warps per sign block and tile; h_ms (optional, 11 floats): the best
 * distance-pass times of the shapes (64, 8), (64, 16), (64, 32), (128, 8),
 * (128, 16), (128, 32), (256, 8), (256, 16), then the sign-pass times with
 * 2, 4, 8 warps, in ms.  The brick stays 8^3: it is the reference's leaf, the
 * unit of every later boolean, offset and mesher. */
bs_status bs_autotune_mesh_to_volume(bs_ctx* ctx, const float* d_xyz, uint64_t nv, const uint32_t* d_tri, uint64_t nt,
                                     const bs_m2v_params* p, int32_t* h_choice, float* h_ms);
/* Sets the launch shapes directly (0 keeps the current value; a context
 * starts at 128 threads per brick, tiles of 32 sub-triangles and 4 sign
 * warps, and a tile left at 0 with 256 threads becomes 16). */
bs_status bs_ctx_set_launch_shape(bs_ctx* ctx, int32_t dist_threads, int32_t wn_warps, int32_t dist_tile);
/* ------------------------------------------------------------- volumes --- */
/* Volume::with_voxel_size (volume/mod.rs:17-24): an empty volume (no leaves,
 * tiles or internal nodes).  It takes part in booleans as the reference's
 * empty grid does (root_node/csg.rs:9-58): union and subtraction of it leave
 * the other operand (flood filled), intersection with it is empty. */
bs_status bs_volume_create(bs_ctx* ctx, float voxel_size, bs_volume** out);
/* Dropping a Volume (its Box<VolumeGrid>, volume/mod.rs:10-14). */
bs_status bs_volume_free(bs_volume* v);
/* Volume::voxel_size (volume/mod.rs:31-34). */
bs_status bs_volume_voxel_size(const bs_volume* v, float* out);
/* Volume's Clone impl (volume/mod.rs:114-121). */
bs_status bs_volume_clone(bs_ctx* ctx, const bs_volume* v, bs_volume** out);
/* Number of leaves and of active tiles (tiles appear only after booleans).
 * This and the two exports have no reference counterpart: they read a volume
 * out for parity checks and hosts that store it. */
bs_status bs_volume_counts(const bs_volume* v, uint64_t* n_leaves, uint64_t* n_tiles,
                           uint64_t* n_active_voxels);
/* Copies the volume to HOST memory: h_origins[3*n_leaves] (int32 leaf origins,
 * sorted by (x, y, z)), h_values[512*n_leaves], h_masks[16*n_leaves].  Any of
 * the three may be NULL.  Values of inactive voxels are those the reference
 * holds there (0 after convert, signed far values after a flood fill). */
bs_status bs_volume_export(bs_ctx* ctx, const bs_volume* v, int32_t* h_origins, float* h_values,
                           uint32_t* h_masks);
/* Active tiles: h_origins[3*n], h_sizes[n] (edge length in voxels), h_values[n]. */
bs_status bs_volume_export_tiles(bs_ctx* ctx, const bs_volume* v, int32_t* h_origins,
                                 int32_t* h_sizes, float* h_values);

/* Volume::union / subtract / intersect (volume/mod.rs:74-93): both operands are
 * flood filled, combined, and consumed; *out receives the result. */
bs_status bs_volume_union(bs_ctx* ctx, bs_volume* a, bs_volume* b, bs_volume** out);
bs_status bs_volume_subtract(bs_ctx* ctx, bs_volume* a, bs_volume* b, bs_volume** out);
bs_status bs_volume_intersect(bs_ctx* ctx, bs_volume* a, bs_volume* b, bs_volume** out);
/* Volume::offset (volume/mod.rs:95-108), in place. */
bs_status bs_volume_offset(bs_ctx* ctx, bs_volume* v, float distance);

/* ------------------------------------------------- winding numbers ---- */
typedef struct bs_wn_tree bs_wn_tree;
/* WindingNumbers::from_mesh (spatial_partitioning/aabb_tree.rs:636-644): the
 * mesh's tree with the far-field records of every node (device arrays: 3
 * floats per vertex, 3 uint32 per triangle).  order 2 is the reference's
 * expansion; 3 adds the third-order term the reference leaves undone
 * (aabb_tree.rs:706).  The tree topology is this library's (PLOC), not the
 * reference's SAH split. */
bs_status bs_winding_numbers_build(bs_ctx* ctx, const float* d_xyz, uint64_t nv, const uint32_t* d_tri, uint64_t nt,
                                   int order, bs_wn_tree** out);
/* WindingNumbers::from_mesh with a choice of tree: tree 0 is the reference's
 * own (AABBTree::top_down::<Area> with 3 triangles per leaf,
 * aabb_tree.rs:636-644; order 2 only), and bs_winding_numbers_approximate then
 * traverses it once per point, summing as fast_wn recurses
 * (aabb_tree.rs:662-691), so values equal the reference's float32 results bit
 * for bit but for last-place differences of atan2f; tree 1 is the PLOC tree
 * of bs_winding_numbers_build. */
bs_status bs_winding_numbers_build_ex(bs_ctx* ctx, const float* d_xyz, uint64_t nv, const uint32_t* d_tri,
                                      uint64_t nt, int order, int tree, bs_wn_tree** out);
/* WindingNumbers::approximate(point, accuracy_scale) (aabb_tree.rs:654-660) at
 * n_points device points (3 floats each) into d_out; beta = accuracy_scale.
 * From 2^20 points on the call traverses a Morton-sorted copy of the points
 * and returns the values in the caller's order: each warp of 32 then holds
 * nearby points and opens few nodes beyond its lanes' own cuts, so values
 * differ from those of smaller calls only within the approximation error. */
bs_status bs_winding_numbers_approximate(bs_ctx* ctx, const bs_wn_tree* tree, const float* d_points, uint64_t n_points,
                                         float beta, float* d_out);
/* Dropping the WindingNumbers tree. */
bs_status bs_winding_numbers_free(bs_wn_tree* tree);

/* ------------------------------------------------ learned far field ---- */
/* A per-mesh network that predicts the winding number at a point (no
 * reference counterpart: the reference evaluates winding numbers only at band
 * voxels, mesh_to_volume.rs:245-280).  x -> (x - centre) * scale -> 64 Fourier
 * features [sin(pi f_k . x_n), cos(pi f_k . x_n)] of 32 frequency vectors ->
 * Linear 64x64 + SiLU -> Linear 64x64 + SiLU -> Linear 64x1, BF16 tensor-core
 * kernels with FP32 accumulation.  Parameters (bs_mlp_num_params() floats):
 * W1[in][out] (4096), b1 (64), W2[in][out] (4096), b2 (64), w3 (64), b3. */
typedef struct bs_mlp bs_mlp;
int bs_mlp_num_params(void);
/* centre[3], scale > 0, h_freq[32*3], h_params[num_params] (host). */
bs_status bs_mlp_create(bs_ctx* ctx, const float* centre, float scale, const float* h_freq, const float* h_params,
                        bs_mlp** out);
bs_status bs_mlp_free(bs_mlp* net);
bs_status bs_mlp_get_params(bs_ctx* ctx, const bs_mlp* net, float* h_params);
/* Predictions at n device points into d_out (device). */
bs_status bs_mlp_predict(bs_ctx* ctx, const bs_mlp* net, const float* d_points, uint64_t n, float* d_out);
/* Adam training on mean squared error: epochs over floor(n / batch)
 * minibatches of the device arrays in their order (batch a multiple of 128),
 * cosine learning rate lr_max -> lr_min; each step is replayed from one
 * captured CUDA graph.  h_epoch_loss (optional, epochs floats): mean loss. */
bs_status bs_mlp_train(bs_ctx* ctx, bs_mlp* net, const float* d_points, const float* d_targets, uint64_t n,
                       uint32_t batch, uint32_t epochs, float lr_max, float lr_min, float* h_epoch_loss);
/* Gradient (h_grad, num_params floats) and loss of the first `batch` samples,
 * without an update (gradient checks). */
bs_status bs_mlp_gradients(bs_ctx* ctx, bs_mlp* net, const float* d_points, const float* d_targets, uint64_t n,
                           uint32_t batch, float* h_grad, float* h_loss);
/* Winding numbers of n device points into d_out: the prediction for points
 * outside the narrow band of `band` (a volume of the mesh; null: no band)
 * whose prediction is more than `margin` from `thresh`, the tree traversal
 * with accuracy scale beta (bs_winding_numbers_approximate) for every other
 * point; *n_traversed counts the latter. */
bs_status bs_mlp_classify(bs_ctx* ctx, const bs_mlp* net, const bs_wn_tree* tree, const bs_volume* band,
                          const float* d_points, uint64_t n, float thresh, float margin, float beta, float* d_out,
                          uint64_t* n_traversed);
/* d_flags[i] = 1 when the grid point nearest to device point i is an active
 * voxel of the volume (inside its narrow band), else 0. */
bs_status bs_volume_band_flags(bs_ctx* ctx, const bs_volume* v, const float* d_points, uint64_t n, uint32_t* d_flags);

/* ------------------------------------------- from_fn / VolumeBuilder ---- */
/* Volume::from_fn (volume/mod.rs:40-72) over values the caller sampled: the
 * grid points (idx_min + (i, j, k)) * voxel_size for i < dims[0], j < dims[1],
 * k < dims[2], values x-major (values[(i*dims[1] + j)*dims[2] + k]); points with
 * |value| <= (band_width + 1) * voxel_size become active voxels.  The closure
 * of from_fn is evaluated by the caller (on the host or on the device):
 * h_values is host memory, d_values device memory of the context's GPU.
 * idx_min = floor(min / voxel_size) and the last point ceil(max / voxel_size)
 * reproduce from_fn's box. */
bs_status bs_volume_from_samples(bs_ctx* ctx, float voxel_size, int64_t band_width, const int64_t* idx_min,
                                 const uint64_t* dims, const float* h_values, bs_volume** out);
bs_status bs_volume_from_samples_device(bs_ctx* ctx, float voxel_size, int64_t band_width, const int64_t* idx_min,
                                        const uint64_t* dims, const float* d_values, bs_volume** out);
/* VolumeBuilder::with_voxel_size(voxel_size).sphere(radius, origin) (volume/builder.rs:21-31). */
bs_status bs_volume_sphere(bs_ctx* ctx, float voxel_size, float radius, const float* origin3, bs_volume** out);
/* VolumeBuilder::cuboid(min, max) (volume/builder.rs:33-54). */
bs_status bs_volume_cuboid(bs_ctx* ctx, float voxel_size, const float* min3, const float* max3, bs_volume** out);
/* VolumeBuilder::iwp(min, max, cell_size), the IWP triply periodic surface
 * (volume/builder.rs:57-76); evaluated with CUDA's cosf. */
bs_status bs_volume_iwp(bs_ctx* ctx, float voxel_size, const float* min3, const float* max3, float cell_size,
                        bs_volume** out);

/* Dual contouring with the vertex of every cell placed by a quadratic error
 * function instead of the reference's particle solver: the point minimising
 * sum_i (n_i . (x - p_i))^2 over the cell's edge crossings p_i and normals n_i,
 * solved in double by a 3x3 symmetric eigen-decomposition and pseudo-inverse
 * (eigenvalues below 0.1 of the largest dropped) around the crossings' mass
 * point.  Crossings, normals, cells and quads are those of bs_dual_contour, so
 * the triangles connect the same cells.  No reference counterpart. */
bs_status bs_dual_contour_qef(bs_ctx* ctx, bs_volume* v, float voxel_size, float* h_tris, uint64_t capacity,
                              uint64_t* n_tris);

/* --------------------------------------------------- marching cubes ---- */
/* MarchingCubesMesher::with_voxel_size(..).mesh(&volume) (marching_cubes.rs:30-63,
 * 969-1011), active tiles included (the cubes on their boundary faces).  Same
 * calling convention as bs_dual_contour: capacity 0 sizes the buffer, the
 * result is cached on the volume.  Cubes, corner values and edge
 * intersections are the reference's; the tiling inside a cube is this
 * library's own face-consistent polygon fan (not the MC33 case tables), so
 * vertex positions match the reference and triangle counts match for cubes
 * without face or interior ambiguity. */
bs_status bs_marching_cubes(bs_ctx* ctx, bs_volume* v, float voxel_size, float* h_tris, uint64_t capacity,
                            uint64_t* n_tris);

/* --------------------------------------------------- dual contouring ---- */
/* DualContouringMesher::with_voxel_size(..).mesh(&volume) (dual_contouring.rs:16-91).
 * Writes up to `capacity` triangles (9 floats each, world units) to h_tris and
 * the total count to *n_tris; call with capacity 0 to size the buffer (the
 * extraction is cached on the volume, so the second call only copies).
 * Active tiles (after booleans): the reference stops with todo!()
 * (dual_contouring.rs:139, 186, 347); here the passes visit the leaves and
 * read every neighbour, cell corner and gradient voxel as the tree's `at`
 * returns it (internal_node/tree_node.rs:34-42), so a voxel of an active tile
 * carries the tile's value — a uniform tile adds no cells of its own. */
bs_status bs_dual_contour(bs_ctx* ctx, bs_volume* v, float voxel_size, float* h_tris,
                          uint64_t capacity, uint64_t* n_tris);

/* Dual contouring that allocates nothing, for callers that cannot allocate
 * device memory at call time (a host that carved all device memory up front,
 * a real-time loop that must not enter the driver's allocator, a plugin whose
 * host owns every allocation).  No counterpart in the reference: it gives the
 * triangles of bs_dual_contour on caller-owned device buffers.  Inputs, in
 * device memory of `device`: the leaves of a volume as bs_volume_export gives
 * them (d_origins int32[3*n_leaves], d_values float[512*n_leaves], d_masks
 * uint32[16*n_leaves]) and its active tiles as bs_volume_export_tiles gives
 * them (d_tile_origins int32[3*n_tiles], d_tile_sizes int32[n_tiles],
 * d_tile_values float[n_tiles]; n_tiles 0 and NULL arrays for a volume without
 * tiles).  Passing every tile of the volume gives exactly bs_dual_contour's
 * triangles; leaving tiles out gives the triangles of a volume without them.
 * Output: up to `capacity` triangles (9 floats each) in d_tris, the count in
 * *n_tris (also when the capacity is too small, which returns
 * BS_ERR_CAPACITY).  Work runs on `stream` (a cudaStream_t, NULL for the
 * legacy default stream) and the call returns after synchronising it; the
 * calling thread's current device is restored before the call returns.
 * Working memory is one static 32 MiB device array per GPU, held from module
 * load until exit; limits: 2048 leaves, 2^20 tiles in at most 256 nodes of
 * 128^3 (8^3 tiles) and 16 nodes of 4096^3 (128^3 tiles), 393216 sign-change
 * edges and 393216 vertex cells; larger inputs return BS_ERR_CAPACITY.  All
 * calls on a device share that array: calls that overlap on the GPU race and
 * must be serialised.  The first call on a device resolves the array's
 * address and must come before any stream capture; after cudaDeviceReset on
 * that device the entry point must not be used again in the process. */
bs_status bs_dual_contour_noalloc(int device, void* stream, const int32_t* d_origins, const float* d_values,
                                  const uint32_t* d_masks, uint64_t n_leaves, const int32_t* d_tile_origins,
                                  const int32_t* d_tile_sizes, const float* d_tile_values, uint64_t n_tiles,
                                  float voxel_size, float* d_tris, uint64_t capacity, uint64_t* n_tris);

/* ------------------------------------------------------- CornerTable ---- */
typedef struct bs_corner_table bs_corner_table;

/* CornerTable::builder_soup().add_faces(..).finish() (mesh/corner_table/builder.rs:292-309):
 * exactly equal points merged (algo/merge_points.rs:12-41), faces added in
 * order with non-manifold faces skipped, isolated vertices deleted and
 * non-manifold vertices split (builder.rs:168-262).  h_tris: 9 floats per
 * triangle in HOST memory. */
bs_status bs_corner_table_from_soup(bs_ctx* ctx, const float* h_tris, uint64_t n_tris, bs_corner_table** out);
/* The same on the dual-contouring output of a volume, without a host round
 * trip of the soup (VoxelRemesher with MeshingMethod::FeaturePreserving,
 * remeshing/voxel.rs:64-85). */
bs_status bs_corner_table_from_dual_contour(bs_ctx* ctx, bs_volume* v, float voxel_size, bs_corner_table** out);
/* The same on the marching-cubes output (VoxelRemesher with the default
 * MeshingMethod::Manifold, remeshing/voxel.rs:64-85). */
bs_status bs_corner_table_from_marching_cubes(bs_ctx* ctx, bs_volume* v, float voxel_size, bs_corner_table** out);
/* Faces, live vertices, vertex slots (live + deleted) and corners
 * (CornerTable::count_faces, face.rs:33; count_vertices, vertex.rs:122). */
bs_status bs_corner_table_counts(const bs_corner_table* t, uint64_t* n_faces, uint64_t* n_vertices,
                                 uint64_t* n_vertex_slots, uint64_t* n_corners);
/* Copies the tables to HOST memory (any pointer may be NULL): positions
 * [3*slots], deleted flags [slots], vertex -> corner [slots] (-1 none),
 * corner -> vertex [corners], corner -> opposite corner [corners] (-1 none). */
bs_status bs_corner_table_export(const bs_corner_table* t, float* h_positions, uint8_t* h_deleted,
                                 int32_t* h_vertex_corner, int32_t* h_corner_vertex, int32_t* h_corner_opposite);
/* Dropping the CornerTable. */
bs_status bs_corner_table_free(bs_corner_table* t);

#ifdef __cplusplus
}
#endif

#endif /* BABY_SHARK_GB300_H */
