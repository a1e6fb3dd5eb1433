// Marching-cubes surface extraction (MarchingCubesMesher::mesh,
// voxel/meshing/marching_cubes.rs:43-63, 967-1181).
//
// Kept from the reference: the cubes (one per voxel of every leaf, its eight
// corners (0,0,0) (1,0,0) (1,1,0) (0,1,0) (0,0,1) (1,0,1) (1,1,1) (0,1,1) all
// active), the corner values (|v| < 1e-6 pushed to +-1e-6), inside = negative,
// the edge intersections t = max(|a|, 1e-6) / (max(|a|, 1e-6) + max(|b|, 1e-6))
// from the lower corner, the scale by the voxel size and the removal of
// degenerate triangles.
//
// The tiling is this file's own (the reference's MC33 case tables are not
// used): every face of the cube contributes the segments of its crossing
// edges, directed from the edge where the counter-clockwise walk around the
// face (seen from outside) enters the inside to the edge where it leaves; a
// face with four crossings joins its inside corners when the bilinear saddle
// is inside (a0 a2 > a1 a3 for inside corners 0, 2).  The segments close into
// cycles oriented with the outside to the front; each cycle becomes a fan of
// triangles from its lowest-numbered edge.  Vertex positions match the
// reference bit for bit; triangle counts match wherever a cube has no
// ambiguity; interior ambiguities (MC33 tunnels) are not resolved.
//
// One warp per leaf stages the leaf and the +x, +y, +z neighbour layers in a
// 9 x 9 x 9 shared tile; a count pass, a scan and a write pass place the
// triangles of every leaf, lane and cube in a fixed order.  Active tiles
// (after booleans) are values too: a corner outside every leaf takes the
// value of the active tile holding it, and the cubes on the six boundary
// faces of every tile are meshed as the reference's tile visitor does
// (marching_cubes.rs:969-994, cubes on a tile's edges visited once per face).
#include <cub/device/device_scan.cuh>

#include "bs_internal.cuh"
#include "leaf_hash.cuh"
#include "tiles.cuh"
#include "volume_upper.cuh"

namespace bs {

namespace {

constexpr int MC_WARPS = 4;
constexpr int T9 = 9;

__constant__ int8_t c_edge[12][2] = {{0, 1}, {1, 2}, {3, 2}, {0, 3}, {4, 5}, {5, 6},
                                     {7, 6}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
__constant__ int8_t c_edge_axis[12] = {0, 1, 0, 1, 0, 1, 0, 1, 2, 2, 2, 2};
__constant__ int8_t c_face[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {3, 7, 6, 2}, {0, 4, 7, 3}, {1, 2, 6, 5}};
__constant__ int8_t c_corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
// edge between two corners, -1 if none
__constant__ int8_t c_edge_of[8][8] = {
    {-1, 0, -1, 3, 8, -1, -1, -1}, {0, -1, 1, -1, -1, 9, -1, -1},  {-1, 1, -1, 2, -1, -1, 10, -1},
    {3, -1, 2, -1, -1, -1, -1, 11}, {8, -1, -1, -1, -1, 4, -1, 7}, {-1, 9, -1, -1, 4, -1, 5, -1},
    {-1, -1, 10, -1, -1, 5, -1, 6}, {-1, -1, -1, 11, 7, -1, 6, -1}};

struct McVol {
  const int4* org;
  const float* val;
  const uint32_t* msk;
  LeafHash hash;
};

// Active tiles of the internal levels: node origin -> node index hashes and
// the slot tables (state -2 = active tile, value in tile[]).
// Value of an arbitrary voxel: its leaf decides when it has one (inactive =
// absent, Grid::at), else an active tile.
__device__ __forceinline__ float value_at(const McVol& V, const TileLookup& T, int x, int y, int z) {
  const int l = V.hash.find(x & ~7, y & ~7, z & ~7);
  if (l >= 0) {
    const int o = ((x & 7) << 6) | ((y & 7) << 3) | (z & 7);
    return ((V.msk[uint64_t(l) * 16 + (o >> 5)] >> (o & 31)) & 1u) ? V.val[uint64_t(l) * 512 + o] : INFINITY;
  }
  float v;
  return tile_value(T, x, y, z, v) ? v : INFINITY;
}

__device__ __forceinline__ int t9(int x, int y, int z) { return (x * T9 + y) * T9 + z; }

// Triangles of the cube at absolute voxel (x, y, z) whose corner i has the
// value corner(i) (+inf = not active): returns the count; writes them when
// `out` is set.  No per-cube arrays: corner values are read through the
// accessor when needed (shared memory for leaf cubes), the segment table
// `next` (edge -> next edge of its cycle) lives in 12 nibbles of a register,
// and each cycle is fanned while it is walked (triangles p0 p_i p_i+1 in
// the walk's order).
template <class Corner>
__device__ int cube_tris(Corner corner, int x, int y, int z, float h, float* out) {
  auto clamp = [](float r) { return fabsf(r) < 1e-6f ? copysignf(1e-6f, r) : r; };
  uint32_t in = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const float r = corner(i);
    if (r == INFINITY) return 0;  // a corner is not active: no cube (Cube::from_voxel)
    if (clamp(r) < 0.0f) in |= 1u << i;
  }
  if (in == 0u || in == 0xffu) return 0;
  uint64_t nxt = ~0ull;  // nibble e: the edge after e, 0xf = none
  auto set_next = [&](int e, int to) { nxt = (nxt & ~(0xfull << (4 * e))) | (uint64_t(to) << (4 * e)); };
  auto get_next = [&](int e) { return int((nxt >> (4 * e)) & 0xfull); };
#pragma unroll
  for (int f = 0; f < 6; ++f) {
    int c[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) c[s] = c_face[f][s];
    int k = 0;
#pragma unroll
    for (int s = 0; s < 4; ++s) k += ((in >> c[s]) & 1u) != ((in >> c[(s + 1) & 3]) & 1u);
    if (k == 2) {
      int entry = -1, exit = -1;
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        const int a = c[s], b = c[(s + 1) & 3];
        const bool ia = (in >> a) & 1u, ib = (in >> b) & 1u;
        if (!ia && ib) entry = c_edge_of[a][b];
        if (ia && !ib) exit = c_edge_of[a][b];
      }
      if (entry >= 0 && exit >= 0) set_next(entry, exit);  // always both on a face with two crossings
    } else if (k == 4) {
      const int p = ((in >> c[0]) & 1u) ? 0 : 1;  // corners p and p + 2 are inside
      const float prod_in = fmul(clamp(corner(c[p])), clamp(corner(c[p + 2])));
      const float prod_out = fmul(clamp(corner(c[(p + 1) & 3])), clamp(corner(c[(p + 3) & 3])));
      if (prod_in > prod_out) {
        for (int q = (p + 1) & 3, t = 0; t < 2; ++t, q = (q + 2) & 3)
          set_next(c_edge_of[c[q]][c[(q + 1) & 3]], c_edge_of[c[(q + 3) & 3]][c[q]]);
      } else {
        for (int r = p, t = 0; t < 2; ++t, r = (r + 2) & 3)
          set_next(c_edge_of[c[(r + 3) & 3]][c[r]], c_edge_of[c[r]][c[(r + 1) & 3]]);
      }
    }
  }
  // the crossing on edge e, scaled by the voxel size
  auto point = [&](int e) {
    const int a = c_edge[e][0], b = c_edge[e][1];
    const float va = fmaxf(fabsf(corner(a)), 1e-6f), vb = fmaxf(fabsf(corner(b)), 1e-6f);
    const float t = fdiv(va, fadd(va, vb));
    float qx = float(x + c_corner[a][0]), qy = float(y + c_corner[a][1]), qz = float(z + c_corner[a][2]);
    const int ax = c_edge_axis[e];
    if (ax == 0) qx = fadd(qx, t);
    else if (ax == 1) qy = fadd(qy, t);
    else qz = fadd(qz, t);
    return f3(fmul(qx, h), fmul(qy, h), fmul(qz, h));
  };
  int count = 0;
  uint32_t seen = 0;
  for (int e0 = 0; e0 < 12; ++e0) {
    if (get_next(e0) == 0xf || ((seen >> e0) & 1u)) continue;
    seen |= 1u << e0;
    const F3 a = point(e0);
    int e = get_next(e0);
    if ((seen >> e) & 1u) continue;
    seen |= 1u << e;
    F3 b = point(e);
    int n = 2;
    for (e = get_next(e); e != 0xf && !((seen >> e) & 1u) && n < 12; e = get_next(e)) {
      seen |= 1u << e;
      ++n;
      const F3 c = point(e);
      const F3 u = f3(fsub(b.x, a.x), fsub(b.y, a.y), fsub(b.z, a.z));
      const F3 w = f3(fsub(c.x, a.x), fsub(c.y, a.y), fsub(c.z, a.z));
      const float cx = fsub(fmul(u.y, w.z), fmul(u.z, w.y));
      const float cy = fsub(fmul(u.z, w.x), fmul(u.x, w.z));
      const float cz = fsub(fmul(u.x, w.y), fmul(u.y, w.x));
      if (fadd(fadd(fmul(cx, cx), fmul(cy, cy)), fmul(cz, cz)) != 0.0f) {  // Triangle3::is_degenerate
        if (out) {
          float* o = out + 9 * count;
          o[0] = a.x; o[1] = a.y; o[2] = a.z;
          o[3] = b.x; o[4] = b.y; o[5] = b.z;
          o[6] = c.x; o[7] = c.y; o[8] = c.z;
        }
        ++count;
      }
      b = c;
    }
  }
  return count;
}

__device__ __forceinline__ int leaf_cube(const float* W, int x, int y, int z, int4 org, float h, float* out) {
  return cube_tris([&](int i) { return W[t9(x + c_corner[i][0], y + c_corner[i][1], z + c_corner[i][2])]; },
                   org.x + x, org.y + y, org.z + z, h, out);
}

// One warp per leaf.  Pass 1 (tris == nullptr) stores each leaf's triangle
// count; pass 2 writes them from the leaf's scanned offset.
__global__ void __launch_bounds__(32 * MC_WARPS) k_mc(McVol V, TileLookup T, uint64_t n, float h,
                                                     uint32_t* __restrict__ leaf_count,
                                                     const uint32_t* __restrict__ leaf_off, float* __restrict__ tris) {
  __shared__ float tile[MC_WARPS][T9 * T9 * T9];
  __shared__ int snb[MC_WARPS][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint64_t leaf = blockIdx.x * uint64_t(MC_WARPS) + w;
  if (leaf >= n) return;
  float* W = tile[w];
  const int4 org = V.org[leaf];
  // the leaf: four float4 per lane (voxels 4 k4 .. 4 k4 + 3, k4 = lane + 32 j)
  // and its mask words, every load issued before the first store
  {
    const float4* lv4 = reinterpret_cast<const float4*>(V.val + leaf * 512);
    float4 in4[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) in4[j] = lv4[lane + 32 * j];
    const uint32_t mw = lane < 16 ? V.msk[leaf * 16 + lane] : 0u;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k4 = lane + 32 * j, k = 4 * k4;
      const uint32_t m = __shfl_sync(0xffffffffu, mw, k4 >> 3) >> (4 * (k4 & 7));
      const int base = t9(k >> 6, (k >> 3) & 7, k & 7);  // z, z + 1, z + 2, z + 3 follow
      W[base] = (m & 1u) ? in4[j].x : INFINITY;
      W[base + 1] = (m & 2u) ? in4[j].y : INFINITY;
      W[base + 2] = (m & 4u) ? in4[j].z : INFINITY;
      W[base + 3] = (m & 8u) ? in4[j].w : INFINITY;
    }
  }
  // neighbours +x, +y, +z, +x+y, +x+z, +y+z, +x+y+z
  if (lane < 7) {
    const int d = lane + 1;  // bit 0: x, bit 1: y, bit 2: z
    snb[w][lane] = V.hash.find(org.x + ((d & 1) ? 8 : 0), org.y + ((d & 2) ? 8 : 0), org.z + ((d & 4) ? 8 : 0));
  }
  __syncwarp();
  // the 217 halo cells: x = 8 or y = 8 or z = 8 (loop unrolled so that the
  // seven rounds' loads overlap; a neighbour's value is loaded with its mask
  // word rather than after it)
#pragma unroll
  for (int k = lane; k < 217; k += 32) {
    int x, y, z;
    if (k < 64) { x = 8; y = k >> 3; z = k & 7; }
    else if (k < 128) { x = (k - 64) >> 3; y = 8; z = (k - 64) & 7; }
    else if (k < 192) { x = (k - 128) >> 3; y = (k - 128) & 7; z = 8; }
    else if (k < 200) { x = 8; y = 8; z = k - 192; }
    else if (k < 208) { x = 8; y = k - 200; z = 8; }
    else if (k < 216) { x = k - 208; y = 8; z = 8; }
    else { x = 8; y = 8; z = 8; }
    const int d = (x == 8 ? 1 : 0) | (y == 8 ? 2 : 0) | (z == 8 ? 4 : 0);
    const int n_leaf = snb[w][d - 1];
    float val = INFINITY;
    if (n_leaf >= 0) {
      const int o = ((x & 7) << 6) | ((y & 7) << 3) | (z & 7);
      const uint32_t mword = V.msk[uint64_t(n_leaf) * 16 + (o >> 5)];
      const float vv = V.val[uint64_t(n_leaf) * 512 + o];
      if ((mword >> (o & 31)) & 1u) val = vv;
    } else {
      float tv;
      if (tile_value(T, org.x + x, org.y + y, org.z + z, tv)) val = tv;
    }
    W[t9(x, y, z)] = val;
  }
  __syncwarp();
  uint32_t mine = 0;
  for (int j = 0; j < 16; ++j) {
    const int o = 32 * j + lane;
    mine += uint32_t(leaf_cube(W, o >> 6, (o >> 3) & 7, o & 7, org, h, nullptr));
  }
  if (!tris) {
    uint32_t s = mine;
    for (int d = 16; d > 0; d >>= 1) s += __shfl_down_sync(0xffffffffu, s, d);
    if (lane == 0) leaf_count[leaf] = s;
    return;
  }
  uint32_t incl = mine;
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += t;
  }
  uint64_t at = uint64_t(leaf_off[leaf]) + (incl - mine);
  for (int j = 0; j < 16; ++j) {
    const int o = 32 * j + lane;
    at += uint64_t(leaf_cube(W, o >> 6, (o >> 3) & 7, o & 7, org, h, tris + 9 * at));
  }
}

// Cubes of the tiles' boundary faces (marching_cubes.rs:969-994): for tile
// t of size s, cube c in [cbase[t], cbase[t + 1]) is face f = r / s^2 of
// (left, right, top, bottom, front, back) at (i, j) = ((r % s^2) / s, r % s).
__global__ void k_mc_tiles(McVol V, TileLookup T, const int4* __restrict__ tiles, const uint64_t* __restrict__ cbase,
                           int n_tiles, uint64_t n_cubes, float h, uint32_t* __restrict__ count,
                           const uint64_t* __restrict__ off, float* __restrict__ tris) {
  const uint64_t c = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (c >= n_cubes) return;
  int lo = 0, hi = n_tiles - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (cbase[mid] <= c) lo = mid;
    else hi = mid - 1;
  }
  const int4 t = tiles[lo];
  const int s = t.w;
  const uint64_t r = c - cbase[lo], s2 = uint64_t(s) * s;
  const int f = int(r / s2);
  const int i = int((r % s2) / s), j = int(r % s);
  int x, y, z;
  switch (f) {
    case 0: x = 0; y = i; z = j; break;          // left
    case 1: x = s - 1; y = i; z = j; break;      // right
    case 2: x = i; y = j; z = s - 1; break;      // top
    case 3: x = i; y = j; z = 0; break;          // bottom
    case 4: x = i; y = s - 1; z = j; break;      // front
    default: x = i; y = 0; z = j; break;         // back
  }
  x += t.x;
  y += t.y;
  z += t.z;
  float raw[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) raw[k] = value_at(V, T, x + c_corner[k][0], y + c_corner[k][1], z + c_corner[k][2]);
  auto corner = [&](int k) { return raw[k]; };
  if (!tris) {
    count[c] = uint32_t(cube_tris(corner, x, y, z, h, nullptr));
  } else if (off[c + 1] > off[c]) {
    cube_tris(corner, x, y, z, h, tris + 9 * off[c]);
  }
}

__global__ void k_tile_cube_counts(const int4* __restrict__ tiles, int n, uint64_t* __restrict__ cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) cnt[i] = 6ull * uint64_t(tiles[i].w) * uint64_t(tiles[i].w);
  if (i == n) cnt[n] = 0;
}

__global__ void k_widen(const uint32_t* __restrict__ in, uint64_t n, uint64_t* __restrict__ out) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i < n) out[i] = in[i];
  if (i == n) out[n] = 0;
}

}  // namespace

// MarchingCubesMesher::with_voxel_size(voxel_size).mesh(&volume); the
// triangles stay cached on the volume until it changes.
void marching_cubes_impl(bs_ctx* ctx, bs_volume* v, float voxel_size) {
  if (v->mc_valid && v->mc_h == voxel_size) return;
  cudaStream_t s = ctx->stream;
  dfree(ctx, v->d_mc_tris);
  v->d_mc_tris = nullptr;
  v->n_mc_tris = 0;
  const uint64_t n = v->n_leaves, ntl = v->n_tiles;
  if (n == 0 && ntl == 0) {
    v->mc_valid = true;
    v->mc_h = voxel_size;
    return;
  }
  LeafHashBuf hb, h1, h2;
  hb.build(ctx, v->d_origins, n, n);
  McVol V{v->d_origins, v->d_values, v->d_masks, hb.h};
  TileLookup T{};
  T.any = 0;
  if (ntl) {
    const Upper* u = v->upper;
    if (!u) fail(BS_ERR_UNSUPPORTED, "marching cubes: tiles without internal levels");
    h1.build(ctx, u->l1.d_key, u->l1.n, u->l1.n);
    h2.build(ctx, u->l2.d_key, u->l2.n, u->l2.n);
    T = TileLookup{h1.h, h2.h, u->l1.d_state, u->l1.d_tile, u->l2.d_state, u->l2.d_tile, 1};
  }
  // leaves: count, scan, (write below)
  uint32_t nt_leaf = 0;
  DBuf<uint32_t> cnt, off;
  const unsigned grid = unsigned((n + MC_WARPS - 1) / MC_WARPS);
  if (n) {
    cnt = DBuf<uint32_t>(ctx, n + 1);
    off = DBuf<uint32_t>(ctx, n + 1);
    BS_CUDA(cudaMemsetAsync(cnt.p + n, 0, sizeof(uint32_t), s));
    BS_KERNEL(ctx, "k_mc_count", (k_mc<<<grid, 32 * MC_WARPS, 0, s>>>(V, T, n, voxel_size, cnt.p, nullptr, nullptr)));
    size_t tmp = 0;
    BS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, cnt.p, off.p, n + 1, s));
    DBuf<uint8_t> t(ctx, tmp);
    BS_CUDA(cub::DeviceScan::ExclusiveSum(t.p, tmp, cnt.p, off.p, n + 1, s));
    read_back(ctx, &nt_leaf, off.p + n, sizeof nt_leaf);
  }
  // tile boundary cubes: count, scan
  uint64_t n_cubes = 0, nt_tile = 0;
  DBuf<uint64_t> cbase, toff;
  if (ntl) {
    DBuf<uint64_t> tc(ctx, ntl + 1);
    cbase = DBuf<uint64_t>(ctx, ntl + 1);
    BS_KERNEL(ctx, "k_tile_cube_counts", (k_tile_cube_counts<<<unsigned((ntl + 256) / 256), 256, 0, s>>>(v->d_tiles, int(ntl), tc.p)));
    size_t tmp = 0;
    BS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, tc.p, cbase.p, ntl + 1, s));
    {
      DBuf<uint8_t> t(ctx, tmp);
      BS_CUDA(cub::DeviceScan::ExclusiveSum(t.p, tmp, tc.p, cbase.p, ntl + 1, s));
    }
    read_back(ctx, &n_cubes, cbase.p + ntl, sizeof n_cubes);
    if (n_cubes) {
      DBuf<uint32_t> cc(ctx, n_cubes);
      DBuf<uint64_t> c64(ctx, n_cubes + 1);
      toff = DBuf<uint64_t>(ctx, n_cubes + 1);
      BS_KERNEL(ctx, "k_mc_tiles_count", (k_mc_tiles<<<unsigned((n_cubes + 255) / 256), 256, 0, s>>>(V, T, v->d_tiles, cbase.p, int(ntl), n_cubes,
                                                                                        voxel_size, cc.p, nullptr, nullptr)));
      BS_KERNEL(ctx, "k_widen", (k_widen<<<unsigned((n_cubes + 256) / 256), 256, 0, s>>>(cc.p, n_cubes, c64.p)));
      tmp = 0;
      BS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, c64.p, toff.p, n_cubes + 1, s));
      DBuf<uint8_t> t(ctx, tmp);
      BS_CUDA(cub::DeviceScan::ExclusiveSum(t.p, tmp, c64.p, toff.p, n_cubes + 1, s));
      read_back(ctx, &nt_tile, toff.p + n_cubes, sizeof nt_tile);
    }
  }
  const uint64_t total = uint64_t(nt_leaf) + nt_tile;
  if (total) {
    v->d_mc_tris = dalloc<float>(ctx, total * 9);
    if (nt_leaf)
      BS_KERNEL(ctx, "k_mc_write", (k_mc<<<grid, 32 * MC_WARPS, 0, s>>>(V, T, n, voxel_size, nullptr, off.p, v->d_mc_tris)));
    if (nt_tile)
      BS_KERNEL(ctx, "k_mc_tiles_write", (k_mc_tiles<<<unsigned((n_cubes + 255) / 256), 256, 0, s>>>(V, T, v->d_tiles, cbase.p, int(ntl), n_cubes,
                                                                                        voxel_size, nullptr, toff.p,
                                                                                        v->d_mc_tris + 9 * uint64_t(nt_leaf))));
  }
  v->n_mc_tris = total;
  v->mc_valid = true;
  v->mc_h = voxel_size;
}

}  // namespace bs
