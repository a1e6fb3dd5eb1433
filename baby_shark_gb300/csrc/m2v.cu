// Mesh -> narrow-band signed distance volume on the GPU.
//
// Replaces MeshToVolume::convert (voxel/mesh_to_volume.rs:52-73):
//  1. subdivide every triangle until its sides are < 2 voxels
//     (mesh_to_volume.rs:75-116), one thread per input triangle;
//  2. bin sub-triangles into the 8^3 bricks their widened integer boxes
//     overlap (mesh_to_volume.rs:124-143), through a dense brick directory
//     over the mesh's brick extent: count, scan, fill;
//  3. per brick, one CTA takes the minimum exact point–triangle distance of
//     every voxel over the sub-triangles whose box contains it
//     (mesh_to_volume.rs:147-195) — the active set is the union of the boxes;
//  4. sign every active voxel with a fast winding number (order-1 + order-2
//     far field, beta = 2, threshold 0.2; mesh_to_volume.rs:245-280) over an
//     LBVH of the original triangles (Morton codes, radix sort, Karras
//     hierarchy, bottom-up coefficient refit).
// Steps 1-3 use IEEE-exact arithmetic (bs_internal.cuh) so distances and the
// active set match the reference bit for bit.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <climits>
#include <cmath>
#include <exception>
#include <memory>
#include <vector>

#include "bs_internal.cuh"
#include "ref_tree.cuh"

namespace bs {

// ------------------------------------------------------------ helpers -----
template <class T>
static void exclusive_scan(bs_ctx* ctx, const T* in, T* out, size_t n) {
  size_t tmp = 0;
  BS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, in, out, n, ctx->stream));
  DBuf<uint8_t> t(ctx, tmp);
  BS_CUDA(cub::DeviceScan::ExclusiveSum(t.p, tmp, in, out, n, ctx->stream));
}

__device__ __forceinline__ uint32_t f2ord(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float ord2f(uint32_t u) {
  uint32_t v = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
  float f;
  memcpy(&f, &v, 4);
  return f;
}

struct M2VStats {
  int vmin[3];        // conservative voxel extent of all widened boxes
  int vmax[3];
  uint32_t cmin[3];   // ordered-int bbox of triangle centroids
  uint32_t cmax[3];
  int error;          // 1: vertex index out of range, 2: sub-triangle outside directory,
                      // 3: traversal stack overflow, 4: coordinates out of int range
  int pad;
  unsigned long long n_sub;    // 64-bit totals (the scans run in 32 bit)
  unsigned long long n_pairs;  // (brick, sub-triangle) pairs
  unsigned long long n_vpairs; // (voxel, sub-triangle) pairs = sum of widened box volumes
  unsigned long long wn_visits;      // warp-level node visits of the winding-number pass
  unsigned long long wn_far;         // warp-level far-field evaluations (internal + leaf dipoles)
  unsigned long long wn_exact;       // warp-level exact solid angles
  unsigned long long n_eval;         // (voxel, sub-triangle) pairs left after culling
};

// Per-mesh parameters of a batch.  Triangles of mesh m are [tri_base,
// tri_base + n_tri) of the concatenated index array; their indices are local
// to the mesh's vertices [vtx_base, vtx_base + n_vtx).
struct MeshInfo {
  float h, inv_h, beta, thresh;
  int band, order;  // order: far-field expansion order, 2 or 3
  uint32_t tri_base, n_tri;
  uint64_t vtx_base, n_vtx;
};

// Largest m in [0, k) with base[m] <= i (segments may be empty).
template <class T>
__device__ __forceinline__ int find_seg(const T* __restrict__ base, int k, uint64_t i) {
  int lo = 0, hi = k - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (uint64_t(__ldg(base + mid)) <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Adds v to *dst once per warp when every active lane targets the same mesh.
__device__ __forceinline__ void warp_add(unsigned long long* dst, unsigned long long v, int m) {
  const unsigned mask = __activemask();
  const int leader = __ffs(mask) - 1;
  const int m0 = __shfl_sync(mask, m, leader);
  if (__all_sync(mask, m == m0)) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(mask, v, o);
    if ((threadIdx.x & 31) == leader) atomicAdd(dst, v);
  } else {
    atomicAdd(dst, v);
  }
}

// atomicMin / atomicMax of v into *dst, one atomic per warp when every active
// lane targets the same mesh (the address is then warp-uniform).
__device__ __forceinline__ bool warp_one_mesh(unsigned mask, int m) {
  return __all_sync(mask, m == __shfl_sync(mask, m, __ffs(mask) - 1));
}
template <class T>
__device__ __forceinline__ void warp_min(T* dst, T v, bool uniform, unsigned mask) {
  if (uniform) {
    const T r = __reduce_min_sync(mask, v);
    if ((threadIdx.x & 31) == __ffs(mask) - 1) atomicMin(dst, r);
  } else {
    atomicMin(dst, v);
  }
}
template <class T>
__device__ __forceinline__ void warp_max(T* dst, T v, bool uniform, unsigned mask) {
  if (uniform) {
    const T r = __reduce_max_sync(mask, v);
    if ((threadIdx.x & 31) == __ffs(mask) - 1) atomicMax(dst, r);
  } else {
    atomicMax(dst, v);
  }
}

struct SubTri {  // 64 B: vertices, cull coefficients and the widened inclusive integer box
  float4 p0;     // a.x a.y a.z b.x
  float4 p1;     // b.y b.z c.x c.y
  float4 p2;     // c.z, cull coefficients c2 and E0 (cull_coeffs), -
  int4 lo;       // box min (x, y, z), mesh
  int4 hi;       // box max
};

// ------------------------------------------- 1. triangles and subdivision --
__global__ void k_gather(const float* __restrict__ xyz, const uint32_t* __restrict__ tri, uint64_t nt,
                         const MeshInfo* __restrict__ mi, const uint32_t* __restrict__ tri_base, int K,
                         float4* __restrict__ T, uint32_t* __restrict__ nsub, M2VStats* st) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= nt) {
    if (i == nt) nsub[nt] = 0;
    return;
  }
  const int mesh = find_seg(tri_base, K, i);
  const MeshInfo M = mi[mesh];
  M2VStats* S = st + mesh;
  const float h = M.h, inv_h = M.inv_h;
  const int band = M.band;
  uint32_t ia = tri[3 * i], ib = tri[3 * i + 1], ic = tri[3 * i + 2];
  if (ia >= M.n_vtx || ib >= M.n_vtx || ic >= M.n_vtx) {
    atomicExch(&S->error, 1);
    nsub[i] = 0;
    T[3 * i] = T[3 * i + 1] = T[3 * i + 2] = make_float4(0, 0, 0, 0);
    return;
  }
  const float* X = xyz + 3 * M.vtx_base;
  F3 a = f3(X[3 * ia], X[3 * ia + 1], X[3 * ia + 2]);
  F3 b = f3(X[3 * ib], X[3 * ib + 1], X[3 * ib + 2]);
  F3 c = f3(X[3 * ic], X[3 * ic + 1], X[3 * ic + 2]);
  T[3 * i] = make_float4(a.x, a.y, a.z, 0.f);
  T[3 * i + 1] = make_float4(b.x, b.y, b.z, 0.f);
  T[3 * i + 2] = make_float4(c.x, c.y, c.z, 0.f);
  // triangle3.rs:117-124 and mesh_to_volume.rs:76-88
  F3 e0 = sub3(b, a), e1 = sub3(c, a), e2 = sub3(c, b);
  float m = fmaxf(fmaxf(dot3(e0, e0), dot3(e1, e1)), dot3(e2, e2));
  float ns = floorf(fdiv(fsqrt(m), h));
  // n^2 sub-triangles in exact integer arithmetic (k_subdivide writes exactly n^2)
  uint32_t cnt;
  if (!(ns >= 2.0f)) {
    cnt = 1;
  } else if (!(ns < 65536.0f)) {
    cnt = 0;
    atomicExch(&S->error, 4);
  } else {
    uint32_t n = uint32_t(ns);
    cnt = n * n;
  }
  nsub[i] = cnt;
  warp_add(&S->n_sub, cnt, mesh);
  F3 mn = min3(c, min3(a, b)), mx = max3(c, max3(a, b));
  float lo[3] = {mn.x, mn.y, mn.z}, hi[3] = {mx.x, mx.y, mx.z};
  const unsigned mask = __activemask();
  const bool uniform = warp_one_mesh(mask, mesh);
  for (int k = 0; k < 3; ++k) {
    float fl = floorf(fmul(lo[k], inv_h)), fh = ceilf(fmul(hi[k], inv_h));
    int vlo = 0x7fffffff, vhi = -0x7fffffff;  // identities for a lane out of range
    if (!(fabsf(fl) < 1.0e9f) || !(fabsf(fh) < 1.0e9f)) {
      atomicExch(&S->error, 4);
    } else {
      vlo = int(fl) - band - 3;
      vhi = int(fh) + band + 3;
    }
    warp_min(&S->vmin[k], vlo, uniform, mask);
    warp_max(&S->vmax[k], vhi, uniform, mask);
  }
  F3 cen = f3((a.x + b.x + c.x) * (1.0f / 3.0f), (a.y + b.y + c.y) * (1.0f / 3.0f),
              (a.z + b.z + c.z) * (1.0f / 3.0f));
  const float cc[3] = {cen.x, cen.y, cen.z};
  for (int k = 0; k < 3; ++k) {
    warp_min(&S->cmin[k], f2ord(cc[k]), uniform, mask);
    warp_max(&S->cmax[k], f2ord(cc[k]), uniform, mask);
  }
}

__device__ __forceinline__ void widened_box(F3 a, F3 b, F3 c, float inv_h, int band, int lo[3], int hi[3]) {
  F3 mn = min3(c, min3(a, b)), mx = max3(c, max3(a, b));
  lo[0] = int(floorf(fmul(mn.x, inv_h))) - band;
  lo[1] = int(floorf(fmul(mn.y, inv_h))) - band;
  lo[2] = int(floorf(fmul(mn.z, inv_h))) - band;
  hi[0] = int(ceilf(fmul(mx.x, inv_h))) + band;
  hi[1] = int(ceilf(fmul(mx.y, inv_h))) + band;
  hi[2] = int(ceilf(fmul(mx.z, inv_h))) + band;
  if (hi[0] == lo[0] || hi[1] == lo[1] || hi[2] == lo[2]) {
    for (int k = 0; k < 3; ++k) {
      lo[k] -= 1;
      hi[k] += 1;
    }
  }
}

// Cull coefficients of one sub-triangle.  In the reference's closest-point
// formula (Ericson, point_triangle_dist2) the vertex cases return a vertex
// exactly and the edge cases a parameter in [0, 1] (their denominators add
// two numbers of one sign), so there the float32 closest point leaves the
// triangle only by rounding.  The face case divides by va + vb + vc, whose
// exact value is |ab x ac|^2 and whose float32 error is at most about
// 70 u e^2 R_p^2 (u = 2^-24, e the longest edge, R_p the largest distance
// from the voxel p to a vertex: the six dot products carry 5 u e R_p each);
// the parameters then move by at most about 93 u e^2 R_p^2 / (|ab x ac|^2 / 4)
// and the point by 188 u e^3 R_p^2 / |ab x ac|^2, bounded here by
// c (d + e)^2 with c = 1024 u e^3 / |ab x ac|^2, since every vertex is within
// d + e of p for d the exact distance.  With the rounding of the vertex,
// edge and final |q - p| terms (19 u (d + e) + 16 u e + 4 u M, M a bound on
// |coordinates|) the float32 distance is at least d - eps(d), and
// eps(sqrt(lb)) <= c2 lb + E0 for c2 = 2 c and E0 = 2 c e^2 + 19 u (R + e)
// + 16 u e + 4 u M, R the widened box diagonal.  The cull test
// lb' > cur * 33/32 + 33 t^2 with t = c2 lb' + E0 (lb' the float32 sum of the
// squared box distances each scaled by 1 - 2^-20, so lb' < lb (1 - 8 u))
// implies sqrt(lb) - t > sqrt(cur) (2 t sqrt(cur) <= cur / 32 + 32 t^2), so a
// culled pair's float32 distance is above cur.  Conditions checked here:
// the perturbation is small (c R^2 <= e), d - eps(d) increases on [0, R]
// (c (R + e) <= 1/4), and the right side grows slower than lb
// (132 c (c2 R^2 + E0) <= 1/2); a sub-triangle that fails one (every
// degenerate one does) is never culled (c2 = +inf).
__device__ __forceinline__ void cull_coeffs(F3 ab, F3 ac, F3 cb, float R, float M, float& c2, float& E0) {
  const float u = 5.9604645e-8f;
  const float e2 = fmaxf(dot3(ab, ab), fmaxf(dot3(ac, ac), dot3(cb, cb)));
  const float e = sqrtf(e2);
  const F3 n = cross3(ab, ac);
  const float a2sq = dot3(n, n);
  const float c = 1024.0f * u * (e2 * e / a2sq);  // +inf or NaN for a degenerate triangle
  const float e0 = 2.0f * c * e2 + 19.0f * u * (R + e) + 16.0f * u * e + 4.0f * u * M;
  const bool ok = c * R * R <= e && c * (R + e) <= 0.25f && 132.0f * c * (2.0f * c * R * R + e0) <= 0.5f &&
                  e0 < __int_as_float(0x7f800000);
  c2 = ok ? 2.0f * c : __int_as_float(0x7f800000);
  E0 = ok ? e0 : 0.0f;
}

// A sub-triangle record: vertices, widened box, mesh, and the cull
// coefficients of the distance pass (computed once here rather than for
// every brick the box meets).
__device__ __forceinline__ void put_subtri(SubTri* S, uint64_t idx, F3 a, F3 b, F3 c, float h, float inv_h, int band,
                                           int mesh) {
  int lo[3], hi[3];
  widened_box(a, b, c, inv_h, band, lo, hi);
  // R: the widened box holds the vertices and every voxel it covers
  const float ex = float(hi[0] - lo[0]), ey = float(hi[1] - lo[1]), ez = float(hi[2] - lo[2]);
  const float R = h * (sqrtf(ex * ex + ey * ey + ez * ez) + 2.0f);
  const float gm = h * float(max(max(max(abs(lo[0]), abs(hi[0])), max(abs(lo[1]), abs(hi[1]))),
                                 max(abs(lo[2]), abs(hi[2]))) + 1);
  const float M = fmaxf(gm, fmaxf(fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fmaxf(fabsf(a.z), fabsf(b.x))),
                                  fmaxf(fmaxf(fabsf(b.y), fabsf(b.z)), fmaxf(fmaxf(fabsf(c.x), fabsf(c.y)), fabsf(c.z)))));
  float c2, e0;
  cull_coeffs(sub3(b, a), sub3(c, a), sub3(c, b), R, M, c2, e0);
  SubTri s;
  s.p0 = make_float4(a.x, a.y, a.z, b.x);
  s.p1 = make_float4(b.y, b.z, c.x, c.y);
  s.p2 = make_float4(c.z, c2, e0, 0.f);
  s.lo = make_int4(lo[0], lo[1], lo[2], mesh);
  s.hi = make_int4(hi[0], hi[1], hi[2], 0);
  S[idx] = s;
}

// mesh_to_volume.rs:75-116, same stepping and accumulation order.
__global__ void k_subdivide(const float4* __restrict__ T, const uint32_t* __restrict__ nsub,
                            const uint32_t* __restrict__ off, uint64_t nt, const MeshInfo* __restrict__ mi,
                            const uint32_t* __restrict__ tri_base, int K, SubTri* __restrict__ S) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= nt || nsub[i] == 0) return;
  const int mesh = find_seg(tri_base, K, i);
  const float h = mi[mesh].h, inv_h = mi[mesh].inv_h;
  const int band = mi[mesh].band;
  float4 ta = T[3 * i], tb = T[3 * i + 1], tc = T[3 * i + 2];
  F3 p1 = f3(ta.x, ta.y, ta.z), p2 = f3(tb.x, tb.y, tb.z), p3 = f3(tc.x, tc.y, tc.z);
  uint64_t o = off[i];
  if (nsub[i] == 1) {
    put_subtri(S, o, p1, p2, p3, h, inv_h, band, mesh);
    return;
  }
  F3 e0 = sub3(p2, p1), e1 = sub3(p3, p1), e2 = sub3(p3, p2);
  float m = fmaxf(fmaxf(dot3(e0, e0), dot3(e1, e1)), dot3(e2, e2));
  float ns = floorf(fdiv(fsqrt(m), h));
  float inv = fdiv(1.0f, ns);
  F3 s1 = scale3(sub3(p2, p1), inv);
  F3 s2 = scale3(sub3(p3, p2), inv);
  F3 a = p1;
  uint32_t n = uint32_t(ns);
  for (uint32_t r = 0; r < n; ++r) {
    F3 b = add3(a, s1);
    F3 c = add3(b, s2);
    F3 a_s = add3(a, s2), b_s = add3(b, s2), c_s = add3(c, s2);
    F3 a_prev = a;
    for (uint32_t k = 0; k < r; ++k) {
      put_subtri(S, o++, a_prev, b_s, a_s, h, inv_h, band, mesh);
      put_subtri(S, o++, a_s, b_s, c_s, h, inv_h, band, mesh);
      a_prev = a_s;
      a_s = add3(a_s, s2);
      b_s = add3(b_s, s2);
      c_s = add3(c_s, s2);
    }
    put_subtri(S, o++, a, b, c, h, inv_h, band, mesh);
    a = add3(a, s1);
  }
}

// ------------------------------------------------- 2. brick directory -----
struct Dir {
  int bx0, by0, bz0;  // brick coordinate of entry 0
  int dx, dy, dz;     // extent in bricks
};

__device__ __forceinline__ bool brick_range(const SubTri& s, const Dir& d, int lo[3], int hi[3]) {
  lo[0] = (s.lo.x >> 3) - d.bx0; hi[0] = (s.hi.x >> 3) - d.bx0;
  lo[1] = (s.lo.y >> 3) - d.by0; hi[1] = (s.hi.y >> 3) - d.by0;
  lo[2] = (s.lo.z >> 3) - d.bz0; hi[2] = (s.hi.z >> 3) - d.bz0;
  return lo[0] >= 0 && lo[1] >= 0 && lo[2] >= 0 && hi[0] < d.dx && hi[1] < d.dy && hi[2] < d.dz;
}

// Lists are grouped by the class of each (sub-triangle, brick) pair: the
// distance from the centre of the sub-triangle's widened box to the brick's
// centre in steps of 1.25 voxels, capped at LIST_CLASSES - 1.  Each brick's
// list holds class 0 first, so the distance pass meets the sub-triangles
// nearest to most of its voxels early and culls more of the rest (the result
// does not depend on the order).  Integer arithmetic: count and fill agree.
constexpr int LIST_CLASSES = 8;
__device__ __forceinline__ int pair_class(const SubTri& s, int bx, int by, int bz) {
  // twice the centre offset per axis, in voxels
  const long long dx = (long long)s.lo.x + s.hi.x - (16LL * bx + 7);
  const long long dy = (long long)s.lo.y + s.hi.y - (16LL * by + 7);
  const long long dz = (long long)s.lo.z + s.hi.z - (16LL * bz + 7);
  const long long q = 4 * (dx * dx + dy * dy + dz * dz);  // d >= 1.25 k  <=>  q >= 25 k^2
  int c = 0;
#pragma unroll
  for (int k = 1; k < LIST_CLASSES; ++k) c += q >= 25LL * k * k ? 1 : 0;
  return c;
}

__global__ void k_count_pairs(const SubTri* __restrict__ S, uint64_t ns, const Dir* __restrict__ dirs,
                              const uint64_t* __restrict__ dir_base, uint32_t* __restrict__ cnt, M2VStats* st) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= ns) return;
  SubTri s = S[i];
  const int mesh = s.lo.w;
  const Dir d = dirs[mesh];
  uint32_t* C = cnt + dir_base[mesh] * LIST_CLASSES;
  int lo[3], hi[3];
  if (!brick_range(s, d, lo, hi)) {
    atomicExch(&st[mesh].error, 2);
    return;
  }
  for (int x = lo[0]; x <= hi[0]; ++x)
    for (int y = lo[1]; y <= hi[1]; ++y)
      for (int z = lo[2]; z <= hi[2]; ++z)
        atomicAdd(&C[((uint64_t(x) * d.dy + y) * d.dz + z) * LIST_CLASSES +
                     pair_class(s, x + d.bx0, y + d.by0, z + d.bz0)], 1u);
  unsigned long long np = uint64_t(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
  unsigned long long vp = uint64_t(s.hi.x - s.lo.x + 1) * (s.hi.y - s.lo.y + 1) * (s.hi.z - s.lo.z + 1);
  warp_add(&st[mesh].n_pairs, np, mesh);
  warp_add(&st[mesh].n_vpairs, vp, mesh);
}

// flag[e] = 1 for directory entries with pairs (pair_off: scan over entries x classes)
__global__ void k_dir_flags(const uint32_t* __restrict__ pair_off, uint64_t n, uint32_t* __restrict__ flag) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i < n) flag[i] = pair_off[(i + 1) * LIST_CLASSES] != pair_off[i * LIST_CLASSES] ? 1u : 0u;
  if (i == n) flag[n] = 0u;
}

// Compacts non-empty directory entries into bricks in (mesh, x, y, z) order
// and turns cnt[] into per-(entry, class) fill cursors.
__global__ void k_dir_compact(uint32_t* __restrict__ cnt, const uint32_t* __restrict__ pair_off,
                              const uint32_t* __restrict__ bidx, uint64_t n, const Dir* __restrict__ dirs,
                              const uint64_t* __restrict__ dir_base, int K, int4* __restrict__ origins,
                              uint32_t* __restrict__ list_off) {
  uint64_t e = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (e >= n) return;
  const uint64_t e0 = e * LIST_CLASSES;
  if (pair_off[e0 + LIST_CLASSES] != pair_off[e0]) {
    const int mesh = find_seg(dir_base, K, e);
    const Dir d = dirs[mesh];
    const uint64_t l = e - dir_base[mesh];
    uint32_t b = bidx[e];
    int z = int(l % d.dz), y = int((l / d.dz) % d.dy), x = int(l / (uint64_t(d.dz) * d.dy));
    origins[b] = make_int4((x + d.bx0) * 8, (y + d.by0) * 8, (z + d.bz0) * 8, 0);
    list_off[b] = pair_off[e0];
  }
#pragma unroll
  for (int c = 0; c < LIST_CLASSES; ++c) cnt[e0 + c] = pair_off[e0 + c];
}

__global__ void k_fill_pairs(const SubTri* __restrict__ S, uint64_t ns, const Dir* __restrict__ dirs,
                             const uint64_t* __restrict__ dir_base, uint32_t* __restrict__ cursor,
                             uint32_t* __restrict__ list) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= ns) return;
  SubTri s = S[i];
  const int mesh = s.lo.w;
  const Dir d = dirs[mesh];
  uint32_t* C = cursor + dir_base[mesh] * LIST_CLASSES;
  int lo[3], hi[3];
  if (!brick_range(s, d, lo, hi)) return;
  for (int x = lo[0]; x <= hi[0]; ++x)
    for (int y = lo[1]; y <= hi[1]; ++y)
      for (int z = lo[2]; z <= hi[2]; ++z) {
        uint32_t p = atomicAdd(&C[((uint64_t(x) * d.dy + y) * d.dz + z) * LIST_CLASSES +
                                  pair_class(s, x + d.bx0, y + d.by0, z + d.bz0)], 1u);
        list[p] = uint32_t(i);
      }
}

// Per mesh: first brick (from the directory scan) and first active voxel.
__global__ void k_seg_starts(const uint32_t* __restrict__ bidx, const uint64_t* __restrict__ dir_base, int K,
                             uint32_t* __restrict__ leaf_base) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m <= K) leaf_base[m] = bidx[dir_base[m]];
}
__global__ void k_act_starts(const uint32_t* __restrict__ voff, const uint32_t* __restrict__ leaf_base, int K,
                             uint32_t* __restrict__ act_base) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m <= K) act_base[m] = voff[leaf_base[m]];
}

// ----------------------------------------------- 3. per-brick distances ----
// One CTA of 128 threads per brick.  Each warp stages DIST_BATCH sub-triangles
// of the brick's list and its lanes walk the (voxel, sub-triangle) pairs of
// (widened box of the sub-triangle) x (brick); the per-voxel minimum is kept
// in shared memory with atomicMin on the float bits (distances are >= 0, so
// unsigned order is float order; NaN distances are skipped, as `dist < cur`
// never holds for NaN in the reference).
//
// Pairs that cannot lower the voxel's minimum are culled before the exact
// point-triangle distance is evaluated: a pair is dropped when the distance
// from the voxel to the sub-triangle's bounding box, less a bound on how far
// the float32 closest point of the reference's formula can stray from the
// triangle (cull_coeffs), already exceeds the voxel's running minimum.
// The running minimum is a value some evaluated pair produced, so the
// minimum over the surviving pairs equals the minimum over all pairs, bit
// for bit, whatever the order; a voxel whose minimum is still +inf keeps all
// its pairs, so the active set is unchanged too.  Lanes take (sub-triangle,
// y, z) columns of the staged sub-triangles and test the column's eight
// voxels at once (the x part of the bound from a per-sub-triangle table, the
// y and z parts once per column, the running minima as two float4 loads);
// survivors go through a per-warp queue and are evaluated 32 at a time with
// all lanes busy (the branching closest-point formula measured
// faster here than a branch-free one with a single division).
// Threads per brick of the distance pass: 64, 128 or 256, and sub-triangles
// a warp stages at a time (the tile): 8, 16 or 32, except 32 with 256
// threads (its shared memory would pass 48 KB); bs_autotune_mesh_to_volume
// picks both per context (128 and 16 by default).
constexpr int DIST_QUEUE = 32 + 8 * 32;  // < 32 left over + one column walk of 8 steps x 32 lanes

struct __align__(16) BatchTri {
  float4 v0;   // a.x a.y a.z ab.x
  float4 v1;   // ab.y ab.z ac.x ac.y
  float4 v2;   // ac.z b.x b.y b.z
  float4 v3;   // c.x c.y c.z cb.x
  float4 v4;   // cb.y cb.z c2 1/nz (cull coefficient, see cull_coeffs)
  float4 dxa;  // (1 - 2^-20) dx^2 of the brick's voxel columns x = 0..3: distance to the bounding box in x
  float4 dxb;  //   ... x = 4..7
  float4 yz;   // bounding box lo.y lo.z hi.y hi.z
  int4 box;    // x0 y0 z0 nx: first voxel of (widened box) x (brick) and its x extent
  int4 box1;   // nz, mask of the brick x covered by the widened box, bits of E0, bits of max dx
};

constexpr float CULL_SCALE = 1.0f - 0x1p-20f;

__device__ __forceinline__ float box_d(float lo, float hi, float g) { return fmaxf(fmaxf(lo - g, g - hi), 0.0f); }

template <int THREADS, int DIST_BATCH>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS) k_brick_distance(
    const int4* __restrict__ origins, const uint32_t* __restrict__ list_off, const uint32_t* __restrict__ list,
    const SubTri* __restrict__ S, const MeshInfo* __restrict__ mi, const uint32_t* __restrict__ leaf_base, int K,
    float* __restrict__ values, uint32_t* __restrict__ masks, M2VStats* st) {
  // per-voxel running minimum of d^2, x fastest: index (y << 6) | (z << 3) | x,
  // so a (y, z) column's eight voxels are two float4 loads
  __shared__ __align__(16) uint32_t dmin[512];
  __shared__ BatchTri bt[THREADS / 32][DIST_BATCH];
  __shared__ int pre[THREADS / 32][DIST_BATCH + 1];
  __shared__ uint32_t queue[THREADS / 32][DIST_QUEUE];
  __shared__ float gtab[3][8];  // grid coordinates x * h of the brick's voxels, per axis
  __shared__ uint32_t evaluated;
  const int b = blockIdx.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int4 org = origins[b];
  const int mesh = find_seg(leaf_base, K, uint64_t(b));
  const float h = mi[mesh].h;
  for (int o = t; o < 512; o += THREADS) dmin[o] = 0x7f800000u;  // +inf
  if (t < 24) {
    const int ax = t >> 3, i = t & 7;
    gtab[ax][i] = fmul(__int2float_rn((ax == 0 ? org.x : ax == 1 ? org.y : org.z) + i), h);
  }
  if (t == 0) evaluated = 0;
  __syncthreads();
  const uint32_t beg = list_off[b], end = list_off[b + 1];
  BatchTri* W = bt[warp];
  int* P = pre[warp];
  uint32_t* Q = queue[warp];
  uint32_t n_eval = 0;

  // exact distance of one queued pair (entry = j << 9 | column-major voxel index)
  auto eval = [&](uint32_t ent) {
    const BatchTri& q = W[ent >> 9];
    const int o = int(ent & 511u);
    const F3 g = f3(gtab[0][o & 7], gtab[1][o >> 6], gtab[2][(o >> 3) & 7]);
    const float4 v0 = q.v0, v1 = q.v1, v2 = q.v2, v3 = q.v3, v4 = q.v4;
    const float d2 = point_triangle_dist2_e(f3(v0.x, v0.y, v0.z), f3(v2.y, v2.z, v2.w), f3(v3.x, v3.y, v3.z),
                                            f3(v0.w, v1.x, v1.y), f3(v1.z, v1.w, v2.x), f3(v3.w, v4.x, v4.y), g);
    if (d2 < __int_as_float(0x7f800000))  // false for NaN and +inf
      atomicMin(&dmin[o], __float_as_uint(d2));
  };

  for (uint32_t e0 = beg + warp * DIST_BATCH; e0 < end; e0 += (THREADS / 32) * DIST_BATCH) {
    // lanes 0..BATCH-1: stage one sub-triangle each and count its (y, z)
    // columns of voxels in this brick
    int cols = 0;
    if (lane < DIST_BATCH && e0 + lane < end) {
      const SubTri sb = S[list[e0 + lane]];
      const F3 a = f3(sb.p0.x, sb.p0.y, sb.p0.z), bb = f3(sb.p0.w, sb.p1.x, sb.p1.y), c = f3(sb.p1.z, sb.p1.w, sb.p2.x);
      const int x0 = max(sb.lo.x, org.x), y0 = max(sb.lo.y, org.y), z0 = max(sb.lo.z, org.z);
      const int nx = min(sb.hi.x, org.x + 7) - x0 + 1, ny = min(sb.hi.y, org.y + 7) - y0 + 1,
                nz = min(sb.hi.z, org.z + 7) - z0 + 1;
      if (nx > 0 && ny > 0 && nz > 0) {
        BatchTri& q = W[lane];
        const F3 ab = sub3(bb, a), ac = sub3(c, a), cb = sub3(c, bb);
        const float lox = fminf(fminf(a.x, bb.x), c.x), hix = fmaxf(fmaxf(a.x, bb.x), c.x);
        float dx[8], dxmax = 0.0f;
#pragma unroll
        for (int i = 0; i < 8; ++i) {  // squared box distance in x of the brick's voxel columns x = org.x + i
          const float d = box_d(lox, hix, gtab[0][i]);
          dx[i] = fmul(fmul(d, d), CULL_SCALE);
          dxmax = fmaxf(dxmax, dx[i]);
        }
        q.v0 = make_float4(a.x, a.y, a.z, ab.x);
        q.v1 = make_float4(ab.y, ab.z, ac.x, ac.y);
        q.v2 = make_float4(ac.z, bb.x, bb.y, bb.z);
        q.v3 = make_float4(c.x, c.y, c.z, cb.x);
        const float c2 = sb.p2.y, e0 = sb.p2.z;  // cull coefficients (put_subtri)
        q.v4 = make_float4(cb.y, cb.z, c2, 1.0f / float(nz));
        q.dxa = make_float4(dx[0], dx[1], dx[2], dx[3]);
        q.dxb = make_float4(dx[4], dx[5], dx[6], dx[7]);
        q.yz = make_float4(fminf(fminf(a.y, bb.y), c.y), fminf(fminf(a.z, bb.z), c.z),
                           fmaxf(fmaxf(a.y, bb.y), c.y), fmaxf(fmaxf(a.z, bb.z), c.z));
        q.box = make_int4(x0, y0, z0, nx);
        q.box1 = make_int4(nz, int(((1u << nx) - 1u) << (x0 - org.x)), __float_as_int(e0), __float_as_int(dxmax));
        cols = ny * nz;
      }
    }
    // inclusive prefix of the column counts over the batch lanes
    int inc = cols;
#pragma unroll
    for (int d = 1; d < DIST_BATCH; d <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, inc, d);
      if (lane >= d) inc += v;
    }
    if (lane < DIST_BATCH) P[lane + 1] = inc;
    if (lane == 0) P[0] = 0;
    const int total = __shfl_sync(0xffffffffu, inc, DIST_BATCH - 1);
    __syncwarp();
    int j = 0, qn = 0;
    for (int base = 0; base < total; base += 32) {
      // one lane per (sub-triangle, y, z) column: an 8-bit mask of the
      // column's voxels (x within the brick) that survive the cull test
      const int k = base + lane;
      uint32_t bits = 0, colb = 0;
      if (k < total) {
        while (k >= P[j + 1]) ++j;  // P[DIST_BATCH] = total > k
        const BatchTri& q = W[j];
        const int4 bx = q.box;
        const int4 b1 = q.box1;
        const float4 v4 = q.v4, yz = q.yz;
        const int c = k - P[j];
        // c -> (iy, iz) by reciprocal multiply: c < 64 and nz <= 8 keep the
        // product at least 0.5/8 away from the next integer
        const int iy = int((float(c) + 0.5f) * v4.w), iz = c - iy * b1.x;
        const int oy = bx.y - org.y + iy, oz = bx.z - org.z + iz;
        const float dy = box_d(yz.x, yz.z, gtab[1][oy]), dz = box_d(yz.y, yz.w, gtab[2][oz]);
        const float dyz = fadd(fmul(fmul(dy, dy), CULL_SCALE), fmul(fmul(dz, dz), CULL_SCALE));
        const float c2 = v4.z, e0 = __int_as_float(b1.z);
        const float4 dxa = q.dxa, dxb = q.dxb;
        colb = uint32_t((oy << 6) | (oz << 3));
        const float4 ca = *reinterpret_cast<const float4*>(&dmin[colb]);
        const float4 cc = *reinterpret_cast<const float4*>(&dmin[colb + 4]);
        const float dxs[8] = {dxa.x, dxa.y, dxa.z, dxa.w, dxb.x, dxb.y, dxb.z, dxb.w};
        const float cur[8] = {ca.x, ca.y, ca.z, ca.w, cc.x, cc.y, cc.z, cc.w};
        // the margin 33 t^2 with t = c2 lb + E0 grows with lb (c2, E0 >= 0 and
        // each float step is monotone), so the column's largest lb gives a
        // margin no smaller than any of its voxels' own: the test below culls
        // a subset of what the per-voxel margin would, and stays exact
        const float tcol = fmaf(c2, fadd(__int_as_float(b1.w), dyz), e0);
        const float margin = 33.0f * (tcol * tcol);
#pragma unroll
        for (int ix = 0; ix < 8; ++ix) {
          const float lb = fadd(dxs[ix], dyz);
          bits |= (lb > fmaf(cur[ix], 1.03125f, margin)) ? 0u : (1u << ix);
        }
        bits &= uint32_t(b1.y);  // the voxels of (widened box) x (brick) in this column
      }
      // survivors to the queue: warp prefix of the per-lane counts
      const int cnt = __popc(bits);
      int pos = cnt;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, pos, d);
        if (lane >= d) pos += v;
      }
      const int added = __shfl_sync(0xffffffffu, pos, 31);
      pos += qn - cnt;
      while (bits) {
        const int ix = __ffs(bits) - 1;
        bits &= bits - 1u;
        Q[pos++] = (uint32_t(j) << 9) | colb | uint32_t(ix);
      }
      qn += added;
      while (qn >= 32) {
        __syncwarp();
        qn -= 32;
        eval(Q[qn + lane]);
        n_eval += 32;
      }
      __syncwarp();
    }
    if (qn > 0) {
      if (lane < qn) eval(Q[lane]);
      n_eval += qn;
    }
    __syncwarp();
  }
  if (lane == 0 && n_eval) atomicAdd(&evaluated, n_eval);
  __syncthreads();
  if (t == 0 && evaluated) atomicAdd(&st[mesh].n_eval, (unsigned long long)evaluated);
#pragma unroll
  for (int k = 0; k < 512 / THREADS; ++k) {
    const int o = t + THREADS * k;  // (x << 6) | (y << 3) | z
    const uint32_t u = dmin[((o & 0x38) << 3) | ((o & 7) << 3) | (o >> 6)];
    const float dist = fsqrt(__uint_as_float(u));
    const bool act = dist < __int_as_float(0x7f800000);  // sqrt of a finite square can overflow to inf
    const uint32_t m = __ballot_sync(0xffffffffu, act);
    values[uint64_t(b) * 512 + o] = act ? dist : 0.0f;
    if (lane == 0) masks[uint64_t(b) * 16 + warp + (THREADS / 32) * k] = m;
  }
}

// ------------------------------------------------- active voxel list ------
__global__ void k_brick_popcount(const uint32_t* __restrict__ masks, uint64_t nb, uint32_t* __restrict__ cnt) {
  uint64_t b = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (b > nb) return;
  if (b == nb) { cnt[nb] = 0; return; }
  uint32_t c = 0;
#pragma unroll
  for (int w = 0; w < 16; ++w) c += __popc(masks[b * 16 + w]);
  cnt[b] = c;
}

// Bricks whose every candidate distance is NaN (the closest-point formula
// divides 0 by 0 on some degenerate sub-triangles) hold no active voxel; the
// reference inserts only distances below the running value
// (mesh_to_volume.rs:183-190), so it never creates their leaves.  keep[b]:
// brick b has an active voxel (keep[nb] = 0 for the scan's total).
__global__ void k_brick_keep(const uint32_t* __restrict__ cnt, uint64_t nb, uint32_t* __restrict__ keep) {
  const uint64_t b = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (b <= nb) keep[b] = (b < nb && cnt[b] > 0) ? 1u : 0u;
}
__global__ void k_brick_compact(const uint32_t* __restrict__ keep, const uint32_t* __restrict__ pos, uint64_t nb,
                                const int4* __restrict__ org, const float* __restrict__ val,
                                const uint32_t* __restrict__ msk, int4* __restrict__ org2, float* __restrict__ val2,
                                uint32_t* __restrict__ msk2) {
  const uint64_t b = blockIdx.x;
  if (b >= nb || !keep[b]) return;
  const uint64_t d = pos[b];
  if (threadIdx.x == 0) org2[d] = org[b];
  for (int k = threadIdx.x; k < 512; k += blockDim.x) val2[d * 512 + k] = val[b * 512 + k];
  if (threadIdx.x < 16) msk2[d * 16 + threadIdx.x] = msk[b * 16 + threadIdx.x];
}
__global__ void k_remap_base(uint32_t* __restrict__ base, int K, const uint32_t* __restrict__ pos) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m <= K) base[m] = pos[base[m]];
}

// One warp per brick; active voxels are listed in Morton order inside the
// brick (lane l covers Morton indices 16l .. 16l+15), so 32 consecutive
// entries form compact blocks for the warp-coherent winding-number pass.
__device__ __forceinline__ int morton9_to_offset(int m) {
  // m = z0 y0 x0 z1 y1 x1 z2 y2 x2 (bit 0 = z0): spread back to x<<6 | y<<3 | z
  const int z = (m & 1) | ((m >> 2) & 2) | ((m >> 4) & 4);
  const int y = ((m >> 1) & 1) | ((m >> 3) & 2) | ((m >> 5) & 4);
  const int x = ((m >> 2) & 1) | ((m >> 4) & 2) | ((m >> 6) & 4);
  return (x << 6) | (y << 3) | z;
}

__global__ void k_emit_active(const uint32_t* __restrict__ masks, const uint32_t* __restrict__ off, uint64_t nb,
                              uint32_t* __restrict__ act) {
  uint64_t b = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (b >= nb) return;
  const uint32_t* m = masks + b * 16;
  uint32_t bits = 0;
  for (int k = 0; k < 16; ++k) {
    const int o = morton9_to_offset(lane * 16 + k);
    if ((m[o >> 5] >> (o & 31)) & 1u) bits |= 1u << k;
  }
  const uint32_t c = __popc(bits);
  uint32_t pre = c;
#pragma unroll
  for (int s = 1; s < 32; s <<= 1) {
    uint32_t v = __shfl_up_sync(0xffffffffu, pre, s);
    if (lane >= s) pre += v;
  }
  uint32_t pos = off[b] + pre - c;
  while (bits) {
    const int k = __ffs(bits) - 1;
    bits &= bits - 1;
    act[pos++] = uint32_t(b << 9) | uint32_t(morton9_to_offset(lane * 16 + k));
  }
}

// ------------------------------------------------------ 4. LBVH + WN ------
// Internal node record: 5 float4
//   [0] dipole centre p (xyz), radius r
//   [1] order-1 coefficient a (xyz), trace(B)
//   [2] B00 B01 B02 B10   [3] B11 B12 B20 B21   [4] B22, left, right (int bits), -
// Leaf record (one triangle, sorted order): 5 float4
//   [0] centroid (xyz), radius   [1] a = area * normal (xyz), -   [2..4] vertices
// Child encoding: >= 0 internal node index, < 0 leaf ~index.
struct Sums {  // area-weighted moments of a subtree
  float ax, ay, az;           // sum area * n
  float cx, cy, cz;           // sum area * centroid
  float s;                    // sum area
  float m[9];                 // sum centroid * (area n)^T, row-major
  float lo[3], hi[3];         // bbox
};

__device__ __forceinline__ uint64_t expand21(uint64_t v) {
  v &= 0x1fffffull;
  v = (v | v << 32) & 0x1f00000000ffffull;
  v = (v | v << 16) & 0x1f0000ff0000ffull;
  v = (v | v << 8) & 0x100f00f00f00f00full;
  v = (v | v << 4) & 0x10c30c30c30c30c3ull;
  v = (v | v << 2) & 0x1249249249249249ull;
  return v;
}

__global__ void k_morton(const float4* __restrict__ T, uint64_t nt, const M2VStats* stats,
                         const uint32_t* __restrict__ tri_base, int K, uint64_t* __restrict__ keys,
                         uint32_t* __restrict__ vals) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= nt) return;
  const M2VStats* st = stats + find_seg(tri_base, K, i);
  float4 a = T[3 * i], b = T[3 * i + 1], c = T[3 * i + 2];
  float cen[3] = {(a.x + b.x + c.x) * (1.0f / 3.0f), (a.y + b.y + c.y) * (1.0f / 3.0f),
                  (a.z + b.z + c.z) * (1.0f / 3.0f)};
  uint64_t q[3];
  for (int k = 0; k < 3; ++k) {
    float lo = ord2f(st->cmin[k]), hi = ord2f(st->cmax[k]);
    float ext = hi - lo;
    float u = ext > 0.f ? (cen[k] - lo) / ext : 0.5f;
    u = fminf(fmaxf(u, 0.f), 1.f);
    q[k] = uint64_t(fminf(u * 2097152.0f, 2097151.0f));
  }
  keys[i] = (expand21(q[0]) << 2) | (expand21(q[1]) << 1) | expand21(q[2]);
  vals[i] = uint32_t(i);
}

__global__ void k_mesh_keys(const uint32_t* __restrict__ order, uint64_t nt, const uint32_t* __restrict__ tri_base,
                            int K, uint32_t* __restrict__ mk) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i < nt) mk[i] = uint32_t(find_seg(tri_base, K, order[i]));
}
// Order-3 far-field record of a node (6 float4): C_i,jk = sum over its
// triangles of n_i * integral (x - p)_j (x - p)_k dA about the dipole centre
// p (18 floats: for i = x, y, z the symmetric jk block xx xy xz yy yz zz),
// then u_k = sum_i C_i,ik and v_i = sum_j C_i,jj.
__device__ __forceinline__ void store_c3(float4* o, const float C[3][6]) {
  const float u0 = C[0][0] + C[1][1] + C[2][2];  // C_x,xx + C_y,yx + C_z,zx
  const float u1 = C[0][1] + C[1][3] + C[2][4];  // C_x,xy + C_y,yy + C_z,zy
  const float u2 = C[0][2] + C[1][4] + C[2][5];  // C_x,xz + C_y,yz + C_z,zz
  const float v0 = C[0][0] + C[0][3] + C[0][5], v1 = C[1][0] + C[1][3] + C[1][5], v2 = C[2][0] + C[2][3] + C[2][5];
  o[0] = make_float4(C[0][0], C[0][1], C[0][2], C[0][3]);
  o[1] = make_float4(C[0][4], C[0][5], C[1][0], C[1][1]);
  o[2] = make_float4(C[1][2], C[1][3], C[1][4], C[1][5]);
  o[3] = make_float4(C[2][0], C[2][1], C[2][2], C[2][3]);
  o[4] = make_float4(C[2][4], C[2][5], u0, u1);
  o[5] = make_float4(u2, v0, v1, v2);
}
__device__ __forceinline__ void load_c3(const float4* o, float C[3][6]) {
  const float4 a = o[0], b = o[1], c = o[2], d = o[3], e = o[4];
  C[0][0] = a.x; C[0][1] = a.y; C[0][2] = a.z; C[0][3] = a.w; C[0][4] = b.x; C[0][5] = b.y;
  C[1][0] = b.z; C[1][1] = b.w; C[1][2] = c.x; C[1][3] = c.y; C[1][4] = c.z; C[1][5] = c.w;
  C[2][0] = d.x; C[2][1] = d.y; C[2][2] = d.z; C[2][3] = d.w; C[2][4] = e.x; C[2][5] = e.y;
}

__global__ void k_leaves(const float4* __restrict__ T, const uint32_t* __restrict__ order, uint64_t nt,
                         float4* __restrict__ leaf, Sums* __restrict__ lsum, float4* __restrict__ leaf3) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= nt) return;
  uint32_t t = order[i];
  float4 A = T[3 * t], B = T[3 * t + 1], C = T[3 * t + 2];
  float ex = B.x - A.x, ey = B.y - A.y, ez = B.z - A.z;
  float fx = C.x - A.x, fy = C.y - A.y, fz = C.z - A.z;
  float nx = ey * fz - ez * fy, ny = ez * fx - ex * fz, nz = ex * fy - ey * fx;
  float len = sqrtf(nx * nx + ny * ny + nz * nz);
  Sums s;
  float area = 0.5f * len;
  s.ax = 0.5f * nx; s.ay = 0.5f * ny; s.az = 0.5f * nz;
  if (!(len > 0.f)) { s.ax = s.ay = s.az = 0.f; area = 0.f; }
  float cx = (A.x + B.x + C.x) * (1.0f / 3.0f), cy = (A.y + B.y + C.y) * (1.0f / 3.0f),
        cz = (A.z + B.z + C.z) * (1.0f / 3.0f);
  s.s = area;
  s.cx = area * cx; s.cy = area * cy; s.cz = area * cz;
  float cc[3] = {cx, cy, cz}, aa[3] = {s.ax, s.ay, s.az};
  for (int r = 0; r < 3; ++r)
    for (int q = 0; q < 3; ++q) s.m[3 * r + q] = cc[r] * aa[q];
  s.lo[0] = fminf(A.x, fminf(B.x, C.x)); s.hi[0] = fmaxf(A.x, fmaxf(B.x, C.x));
  s.lo[1] = fminf(A.y, fminf(B.y, C.y)); s.hi[1] = fmaxf(A.y, fmaxf(B.y, C.y));
  s.lo[2] = fminf(A.z, fminf(B.z, C.z)); s.hi[2] = fmaxf(A.z, fmaxf(B.z, C.z));
  lsum[i] = s;
  // a single triangle's dipole centre is its centroid; order-2 term vanishes.
  // Radius: the farthest vertex from the centroid (the cluster's extent),
  // rounded up by a few ulps so that it bounds the vertices.
  float da = (A.x - cx) * (A.x - cx) + (A.y - cy) * (A.y - cy) + (A.z - cz) * (A.z - cz);
  float db = (B.x - cx) * (B.x - cx) + (B.y - cy) * (B.y - cy) + (B.z - cz) * (B.z - cz);
  float dc = (C.x - cx) * (C.x - cx) + (C.y - cy) * (C.y - cy) + (C.z - cz) * (C.z - cz);
  leaf[5 * i + 0] = make_float4(cx, cy, cz, sqrtf(fmaxf(fmaxf(da, db), dc)) * 1.000001f);
  leaf[5 * i + 1] = make_float4(s.ax, s.ay, s.az, 0.f);
  leaf[5 * i + 2] = A;
  leaf[5 * i + 3] = B;
  leaf[5 * i + 4] = C;
  if (leaf3) {
    // a triangle's second moment about its centroid: (area / 12) sum_v (v - c)(v - c)^T,
    // so C_i,jk = (area n)_i / 12 * sum_v (v - c)_j (v - c)_k
    const float e[3][3] = {{A.x - cx, A.y - cy, A.z - cz}, {B.x - cx, B.y - cy, B.z - cz}, {C.x - cx, C.y - cy, C.z - cz}};
    const int J[6] = {0, 0, 0, 1, 1, 2}, Kk[6] = {0, 1, 2, 1, 2, 2};
    float S[6];
    for (int q = 0; q < 6; ++q) S[q] = (e[0][J[q]] * e[0][Kk[q]] + e[1][J[q]] * e[1][Kk[q]] + e[2][J[q]] * e[2][Kk[q]]) * (1.0f / 12.0f);
    float Cc[3][6];
    for (int q = 0; q < 6; ++q) {
      Cc[0][q] = s.ax * S[q];
      Cc[1][q] = s.ay * S[q];
      Cc[2][q] = s.az * S[q];
    }
    store_c3(leaf3 + 6 * i, Cc);
  }
}

// ---- PLOC: Meister & Bittner, "Parallel Locally-Ordered Clustering for
// Bounding Volume Hierarchy Construction" (TVCG 2018).  Clusters start as the
// triangles in Morton order; each round every cluster finds the cluster of
// its own mesh within +-PLOC_R positions whose merged bounding box has the
// smallest surface area, mutual nearest neighbours merge into a new internal
// node at the lower position, and the array is compacted.  Internal node ids
// of a mesh count down from n - 2, so its last merge, the root, is node 0.
constexpr int PLOC_R = 16;
constexpr int PLOC_T = 256;

struct Cluster {
  float lo[3], hi[3];
  int node;  // local child encoding: >= 0 internal, < 0 leaf ~index
  int mesh;
};

__device__ __forceinline__ float merged_area(const Cluster& a, const Cluster& b) {
  const float dx = fmaxf(a.hi[0], b.hi[0]) - fminf(a.lo[0], b.lo[0]);
  const float dy = fmaxf(a.hi[1], b.hi[1]) - fminf(a.lo[1], b.lo[1]);
  const float dz = fmaxf(a.hi[2], b.hi[2]) - fminf(a.lo[2], b.lo[2]);
  return dx * dy + dx * dz + dy * dz;
}

__global__ void k_ploc_init(const Sums* __restrict__ lsum, uint64_t nt, const uint32_t* __restrict__ tri_base, int K,
                            Cluster* __restrict__ cl) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= nt) return;
  const int mesh = find_seg(tri_base, K, i);
  const Sums& s = lsum[i];
  Cluster c;
  for (int k = 0; k < 3; ++k) {
    c.lo[k] = s.lo[k];
    c.hi[k] = s.hi[k];
  }
  c.node = ~int(i - tri_base[mesh]);
  c.mesh = mesh;
  cl[i] = c;
}

// Nearest neighbour of every cluster within the window (ties: lower index).
__global__ void __launch_bounds__(PLOC_T) k_ploc_nn(const Cluster* __restrict__ cl, uint32_t nc, int* __restrict__ nn) {
  __shared__ Cluster sc[PLOC_T + 2 * PLOC_R];
  const int64_t b0 = int64_t(blockIdx.x) * PLOC_T;
  for (int k = threadIdx.x; k < PLOC_T + 2 * PLOC_R; k += PLOC_T) {
    const int64_t g = b0 - PLOC_R + k;
    if (g >= 0 && g < int64_t(nc)) sc[k] = cl[g];
    else sc[k].mesh = -1;
  }
  __syncthreads();
  const int64_t i = b0 + threadIdx.x;
  if (i >= int64_t(nc)) return;
  const Cluster& me = sc[threadIdx.x + PLOC_R];
  float best = INFINITY;
  int bj = -1;
  for (int d = -PLOC_R; d <= PLOC_R; ++d) {
    if (d == 0) continue;
    const Cluster& o = sc[threadIdx.x + PLOC_R + d];
    if (o.mesh != me.mesh) continue;
    const float a = merged_area(me, o);
    if (a < best) {  // d ascends, so ties keep the lower index
      best = a;
      bj = int(i + d);
    }
  }
  nn[i] = bj;
}

// Merges mutual pairs; keep[i] says whether position i survives the round.
__global__ void k_ploc_merge(Cluster* __restrict__ cl, uint32_t nc, const int* __restrict__ nn,
                             const uint32_t* __restrict__ tri_base, const uint32_t* __restrict__ inode_base,
                             int* __restrict__ next_id, int2* __restrict__ child, int* __restrict__ parent_i,
                             int* __restrict__ parent_l, uint32_t* __restrict__ keep) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = i < nc ? nn[i] : -1;
  const bool lead = j >= 0 && nn[j] == int(i) && int(i) < j;  // this lane creates a node
  if (i == nc) keep[nc] = 0u;
  if (i < nc && !lead) keep[i] = (j >= 0 && nn[j] == int(i)) ? 0u : 1u;
  // node ids: one atomic per warp when all creating lanes belong to one mesh
  const int m = lead ? cl[i].mesh : -1;
  const unsigned warp_all = __activemask();
  const unsigned creators = __ballot_sync(warp_all, lead);
  if (!lead) return;
  const int leader = __ffs(creators) - 1;
  const int m0 = __shfl_sync(creators, m, leader);
  int slot;
  if (__all_sync(creators, m == m0)) {
    int base = 0;
    if ((threadIdx.x & 31) == leader) base = atomicAdd(&next_id[m], __popc(creators));
    base = __shfl_sync(creators, base, leader);
    slot = base + __popc(creators & ((1u << (threadIdx.x & 31)) - 1u));
  } else {
    slot = atomicAdd(&next_id[m], 1);
  }
  Cluster a = cl[i];
  const Cluster b = cl[j];
  const int n = int(tri_base[m + 1] - tri_base[m]);
  const int id = (n - 2) - slot;
  const uint64_t ib = inode_base[m], lb = tri_base[m];
  child[ib + id] = make_int2(a.node, b.node);
  if (a.node >= 0) parent_i[ib + a.node] = id;
  else parent_l[lb + ~a.node] = id;
  if (b.node >= 0) parent_i[ib + b.node] = id;
  else parent_l[lb + ~b.node] = id;
  for (int k = 0; k < 3; ++k) {
    a.lo[k] = fminf(a.lo[k], b.lo[k]);
    a.hi[k] = fmaxf(a.hi[k], b.hi[k]);
  }
  a.node = id;
  cl[i] = a;
  keep[i] = 1u;
}

__global__ void k_ploc_compact(const Cluster* __restrict__ cl, uint32_t nc, const uint32_t* __restrict__ keep,
                               const uint32_t* __restrict__ pos, Cluster* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nc && keep[i]) out[pos[i]] = cl[i];
}

// Clusters per mesh (the array is sorted by mesh), and the largest count.
__global__ void k_ploc_counts(const Cluster* __restrict__ cl, uint32_t nc, uint32_t* __restrict__ cnt,
                              uint32_t* __restrict__ max_cnt, int K) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nc) {
    const uint32_t c = atomicAdd(&cnt[cl[i].mesh], 1u) + 1u;
    atomicMax(max_cnt, c);
  }
}

// The last rounds of every mesh in one block per mesh, in shared memory (at
// most PLOC_FIN clusters per mesh): the same nearest-neighbour, merge and
// compaction steps as the global rounds, separated by block barriers.
constexpr int PLOC_FIN = 2048;
constexpr int PLOC_FIN_T = 512;

__global__ void __launch_bounds__(PLOC_FIN_T) k_ploc_finish(const Cluster* __restrict__ cl, uint32_t nc,
                                                            const uint32_t* __restrict__ tri_base,
                                                            const uint32_t* __restrict__ inode_base,
                                                            int* __restrict__ next_id, int2* __restrict__ child,
                                                            int* __restrict__ parent_i, int* __restrict__ parent_l,
                                                            int* __restrict__ err) {
  extern __shared__ unsigned char fin_smem[];
  Cluster* A = reinterpret_cast<Cluster*>(fin_smem);
  Cluster* B = A + PLOC_FIN;
  int* nn = reinterpret_cast<int*>(B + PLOC_FIN);
  int* pos = nn + PLOC_FIN;
  __shared__ int s_n, s_id;
  __shared__ int wsum[PLOC_FIN_T / 32];
  const int m = blockIdx.x;
  // this mesh's segment [s0, s1) of the sorted cluster array
  uint32_t lo = 0, hi = nc;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (cl[mid].mesh < m) lo = mid + 1;
    else hi = mid;
  }
  const uint32_t s0 = lo;
  hi = nc;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (cl[mid].mesh < m + 1) lo = mid + 1;
    else hi = mid;
  }
  const int n0 = int(lo - s0);
  if (n0 <= 1) return;
  if (n0 > PLOC_FIN) {
    if (threadIdx.x == 0) atomicExch(err, 1);
    return;
  }
  for (int k = threadIdx.x; k < n0; k += PLOC_FIN_T) A[k] = cl[s0 + k];
  if (threadIdx.x == 0) {
    s_n = n0;
    s_id = next_id[m];
  }
  __syncthreads();
  const int n_tri = int(tri_base[m + 1] - tri_base[m]);
  const uint64_t ib = inode_base[m], lb = tri_base[m];
  for (int round = 0; round < 4096 && s_n > 1; ++round) {
    const int n = s_n;
    for (int i = threadIdx.x; i < n; i += PLOC_FIN_T) {
      float best = INFINITY;
      int bj = -1;
      for (int d = -PLOC_R; d <= PLOC_R; ++d) {
        const int j = i + d;
        if (d == 0 || j < 0 || j >= n) continue;
        const float a = merged_area(A[i], A[j]);
        if (a < best) {
          best = a;
          bj = j;
        }
      }
      nn[i] = bj;
    }
    __syncthreads();
    // merge mutual pairs into B (position kept), flag survivors in pos
    for (int i = threadIdx.x; i < n; i += PLOC_FIN_T) {
      const int j = nn[i];
      int keep = 1;
      Cluster c = A[i];
      if (j >= 0 && nn[j] == i) {
        if (i > j) {
          keep = 0;
        } else {
          const Cluster b = A[j];
          const int id = (n_tri - 2) - atomicAdd(&s_id, 1);
          child[ib + id] = make_int2(c.node, b.node);
          if (c.node >= 0) parent_i[ib + c.node] = id;
          else parent_l[lb + ~c.node] = id;
          if (b.node >= 0) parent_i[ib + b.node] = id;
          else parent_l[lb + ~b.node] = id;
          for (int k = 0; k < 3; ++k) {
            c.lo[k] = fminf(c.lo[k], b.lo[k]);
            c.hi[k] = fmaxf(c.hi[k], b.hi[k]);
          }
          c.node = id;
        }
      }
      B[i] = c;
      pos[i] = keep;
    }
    __syncthreads();
    // exclusive scan of pos over n <= PLOC_FIN entries: 4 per thread
    const int t = threadIdx.x, base = 4 * t;
    int v[4], local = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[k] = (base + k < n) ? pos[base + k] : 0;
      local += v[k];
    }
    int incl = local;
    for (int d = 1; d < 32; d <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, incl, d);
      if ((t & 31) >= d) incl += u;
    }
    if ((t & 31) == 31) wsum[t >> 5] = incl;
    __syncthreads();
    int woff = 0;
    for (int w = 0; w < (t >> 5); ++w) woff += wsum[w];
    int run = woff + incl - local;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (base + k < n) {
        if (v[k]) A[run] = B[base + k];
        run += v[k];
      }
    }
    if (t == PLOC_FIN_T - 1) s_n = run;
    __syncthreads();
  }
  if (threadIdx.x == 0 && s_n != 1) atomicExch(err, 2);
}

__device__ __forceinline__ void sums_add(Sums& r, const Sums& a, const Sums& b) {
  r.ax = a.ax + b.ax; r.ay = a.ay + b.ay; r.az = a.az + b.az;
  r.cx = a.cx + b.cx; r.cy = a.cy + b.cy; r.cz = a.cz + b.cz;
  r.s = a.s + b.s;
  for (int q = 0; q < 9; ++q) r.m[q] = a.m[q] + b.m[q];
  for (int q = 0; q < 3; ++q) { r.lo[q] = fminf(a.lo[q], b.lo[q]); r.hi[q] = fmaxf(a.hi[q], b.hi[q]); }
}

// Loads a subtree sum written by another SM: bypass L1 (not coherent).
__device__ __forceinline__ Sums load_sums_cg(const Sums* p) {
  Sums r;
  const float* src = reinterpret_cast<const float*>(p);
  float* dst = reinterpret_cast<float*>(&r);
#pragma unroll
  for (int q = 0; q < int(sizeof(Sums) / 4); ++q) dst[q] = __ldcg(src + q);
  return r;
}

// Bottom-up: the second thread to reach a node combines both children.
__device__ __forceinline__ float4 ld_cg4(const float4* p) { return __ldcg(p); }

// Adds a child's order-3 coefficients, moved from its dipole centre to the
// parent's (d = child centre - parent centre):
// C_i,jk += B_child[j][i] d_k + d_j B_child[k][i] + a_i d_j d_k.
__device__ __forceinline__ void add_shifted_c3(float C[3][6], const float Cc[3][6], const float Bc[3][3],
                                               const float a[3], const float d[3]) {
  const int J[6] = {0, 0, 0, 1, 1, 2}, Kk[6] = {0, 1, 2, 1, 2, 2};
  for (int i = 0; i < 3; ++i)
    for (int q = 0; q < 6; ++q) {
      const int j = J[q], k = Kk[q];
      C[i][q] += Cc[i][q] + Bc[j][i] * d[k] + d[j] * Bc[k][i] + a[i] * d[j] * d[k];
    }
}

__global__ void k_refit(uint64_t nt, const uint32_t* __restrict__ tri_base, const uint32_t* __restrict__ inode_base,
                        int K, const int2* __restrict__ child, const int* __restrict__ parent_i,
                        const int* __restrict__ parent_l, const Sums* __restrict__ lsum, Sums* __restrict__ isum,
                        int* __restrict__ flags, float4* __restrict__ inode, const float4* __restrict__ leaf_rec,
                        float4* __restrict__ inode3, const float4* __restrict__ leaf3) {
  const uint64_t gl = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (gl >= nt) return;
  const int mesh = find_seg(tri_base, K, gl);
  const uint32_t ib = inode_base[mesh], lb = tri_base[mesh];
  const int n = int(tri_base[mesh + 1] - lb);
  int node = parent_l[gl];
  for (int guard = 0; node >= 0 && guard < n; ++guard) {
    const uint64_t gn = ib + uint64_t(node);
    __threadfence();
    if (atomicAdd(&flags[gn], 1) == 0) return;  // first arrival stops
    __threadfence();
    int2 c = child[gn];
    Sums a = c.x >= 0 ? load_sums_cg(isum + ib + c.x) : lsum[lb + ~c.x];
    Sums b = c.y >= 0 ? load_sums_cg(isum + ib + c.y) : lsum[lb + ~c.y];
    Sums r;
    sums_add(r, a, b);
    isum[gn] = r;
    float px = r.cx / r.s, py = r.cy / r.s, pz = r.cz / r.s;
    float B[9];
    float p[3] = {px, py, pz}, A[3] = {r.ax, r.ay, r.az};
    for (int rr = 0; rr < 3; ++rr)
      for (int q = 0; q < 3; ++q) B[3 * rr + q] = r.m[3 * rr + q] - p[rr] * A[q];
    float d0 = (r.lo[0] - px) * (r.lo[0] - px) + (r.lo[1] - py) * (r.lo[1] - py) + (r.lo[2] - pz) * (r.lo[2] - pz);
    float d1 = (r.hi[0] - px) * (r.hi[0] - px) + (r.hi[1] - py) * (r.hi[1] - py) + (r.hi[2] - pz) * (r.hi[2] - pz);
    // radius: the smaller of the reference's bounding-box bound (aabb_tree.rs:738-741)
    // and the sphere around p holding both children's spheres
    const float4 ca = c.x >= 0 ? ld_cg4(inode + 5 * (ib + uint64_t(c.x))) : leaf_rec[5 * (lb + uint64_t(~c.x))];
    const float4 cb = c.y >= 0 ? ld_cg4(inode + 5 * (ib + uint64_t(c.y))) : leaf_rec[5 * (lb + uint64_t(~c.y))];
    const float ea = sqrtf((ca.x - px) * (ca.x - px) + (ca.y - py) * (ca.y - py) + (ca.z - pz) * (ca.z - pz)) + ca.w;
    const float eb = sqrtf((cb.x - px) * (cb.x - px) + (cb.y - py) * (cb.y - py) + (cb.z - pz) * (cb.z - pz)) + cb.w;
    const float rad = fminf(sqrtf(fmaxf(d0, d1)), fmaxf(ea, eb) * 1.000001f);
    inode[5 * gn + 0] = make_float4(px, py, pz, rad);
    inode[5 * gn + 1] = make_float4(r.ax, r.ay, r.az, B[0] + B[4] + B[8]);
    inode[5 * gn + 2] = make_float4(B[0], B[1], B[2], B[3]);
    inode[5 * gn + 3] = make_float4(B[4], B[5], B[6], B[7]);
    inode[5 * gn + 4] = make_float4(B[8], __int_as_float(c.x), __int_as_float(c.y), 0.f);
    if (inode3) {
      float C[3][6] = {{0.f}};
      const int kids[2] = {c.x, c.y};
      for (int h = 0; h < 2; ++h) {
        const int k = kids[h];
        float Cc[3][6], Bc[3][3], a[3], d[3];
        float4 P, A1;
        if (k >= 0) {
          const float4* rec = inode + 5 * (ib + uint64_t(k));
          P = ld_cg4(rec);
          A1 = ld_cg4(rec + 1);
          const float4 b0 = ld_cg4(rec + 2), b1 = ld_cg4(rec + 3), b2 = ld_cg4(rec + 4);
          Bc[0][0] = b0.x; Bc[0][1] = b0.y; Bc[0][2] = b0.z; Bc[1][0] = b0.w; Bc[1][1] = b1.x; Bc[1][2] = b1.y;
          Bc[2][0] = b1.z; Bc[2][1] = b1.w; Bc[2][2] = b2.x;
          float4 t[5];
          for (int q = 0; q < 5; ++q) t[q] = ld_cg4(inode3 + 6 * (ib + uint64_t(k)) + q);
          load_c3(t, Cc);
        } else {
          const float4* rec = leaf_rec + 5 * (lb + uint64_t(~k));
          P = rec[0];
          A1 = rec[1];
          for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q) Bc[r][q] = 0.f;
          load_c3(leaf3 + 6 * (lb + uint64_t(~k)), Cc);
        }
        a[0] = A1.x; a[1] = A1.y; a[2] = A1.z;
        d[0] = P.x - px; d[1] = P.y - py; d[2] = P.z - pz;
        add_shifted_c3(C, Cc, Bc, a, d);
      }
      store_c3(inode3 + 6 * gn, C);
    }
    node = parent_i[gn];
  }
}

constexpr float FOUR_PI = 12.566370614359172f;
constexpr int WN_STACK = 96;

// Van Oosterom–Strackee solid angle (aabb_tree.rs:582-615), divided by 4 pi.
// Computed with the reference's operation order and no fused multiply-adds:
// for query points on a triangle's plane the numerator is then the
// reference's exact value (often exactly 0, which the reference treats as
// "on the surface"), so such voxels take the reference's sign.
__device__ __forceinline__ float tri_wn_exact(float4 A, float4 B, float4 C, F3 q) {
  F3 qa = sub3(f3(A.x, A.y, A.z), q), qb = sub3(f3(B.x, B.y, B.z), q), qc = sub3(f3(C.x, C.y, C.z), q);
  const float la = fsqrt(dot3(qa, qa)), lb = fsqrt(dot3(qb, qb)), lc = fsqrt(dot3(qc, qc));
  if (la == 0.f || lb == 0.f || lc == 0.f) return 0.f;
  qa = f3(fdiv(qa.x, la), fdiv(qa.y, la), fdiv(qa.z, la));
  qb = f3(fdiv(qb.x, lb), fdiv(qb.y, lb), fdiv(qb.z, lb));
  qc = f3(fdiv(qc.x, lc), fdiv(qc.y, lc), fdiv(qc.z, lc));
  const float num = dot3(qa, cross3(sub3(qb, qa), sub3(qc, qa)));
  if (num == 0.f) return 0.f;
  const float den = fadd(fadd(fadd(1.0f, dot3(qa, qb)), dot3(qa, qc)), dot3(qb, qc));
  return fdiv(fmul(atan2f(num, den), 2.0f), FOUR_PI);
}
// Fast form (fused arithmetic, rsqrt normalisation).  Its numerator is within
// ~1e-6 of the exact one, so whenever |num| > 1e-4 both have the same sign and
// are nonzero; closer to the triangle's plane the exact form decides.
__device__ __forceinline__ float tri_wn(float4 A, float4 B, float4 C, F3 q) {
  float ax = A.x - q.x, ay = A.y - q.y, az = A.z - q.z;
  float bx = B.x - q.x, by = B.y - q.y, bz = B.z - q.z;
  float cx = C.x - q.x, cy = C.y - q.y, cz = C.z - q.z;
  const float la2 = ax * ax + ay * ay + az * az, lb2 = bx * bx + by * by + bz * bz, lc2 = cx * cx + cy * cy + cz * cz;
  if (!(la2 > 1e-30f) || !(lb2 > 1e-30f) || !(lc2 > 1e-30f)) return tri_wn_exact(A, B, C, q);
  const float ia = rsqrtf(la2), ib = rsqrtf(lb2), ic = rsqrtf(lc2);
  ax *= ia; ay *= ia; az *= ia;
  bx *= ib; by *= ib; bz *= ib;
  cx *= ic; cy *= ic; cz *= ic;
  const float ux = bx - ax, uy = by - ay, uz = bz - az, vx = cx - ax, vy = cy - ay, vz = cz - az;
  const float num = ax * (uy * vz - uz * vy) + ay * (uz * vx - ux * vz) + az * (ux * vy - uy * vx);
  if (fabsf(num) < 1e-4f) return tri_wn_exact(A, B, C, q);
  const float den = 1.f + (ax * bx + ay * by + az * bz) + (ax * cx + ay * cy + az * cz) + (bx * cx + by * cy + bz * cz);
  return atan2f(num, den) * (2.0f / FOUR_PI);
}

// Warp-coherent traversal: the 32 lanes of a warp hold 32 consecutive active
// voxels — Morton order inside a brick, so mostly a 4x4x2 block — and walk
// the LBVH together.  A node is summed through its far field only when it is
// far (|q - p| > beta * r, aabb_tree.rs:666) for every lane; otherwise the
// warp opens it, and at a leaf every lane takes the exact solid angle.  Node
// loads are warp-uniform, control flow never diverges, and each lane's sum is
// at least as accurate as its own traversal would be.
constexpr int WN_WARPS = 4;
constexpr int WN_THREADS = 32 * WN_WARPS;

__device__ __forceinline__ void kahan(float& sum, float& comp, float w) {
  const float y = w - comp;
  const float t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

// Warps are numbered per mesh (warp_base[m] .. warp_base[m+1]) so that a warp
// never holds voxels of two meshes.
// Order-3 far-field term (1 / 8 pi) [-3 |r|^-5 (2 u.r + v.r) + 15 |r|^-7
// sum_i r_i r^T C_i r] with inv = 1 / (4 pi |r|^3) and ri2 = 1 / |r|^2.
__device__ __forceinline__ float far3(const float4* __restrict__ c3, float rx, float ry, float rz, float inv,
                                      float ri2) {
  const float4 a = __ldg(c3), b = __ldg(c3 + 1), c = __ldg(c3 + 2), d = __ldg(c3 + 3), e = __ldg(c3 + 4),
               f = __ldg(c3 + 5);
  const float xx = rx * rx, yy = ry * ry, zz = rz * rz, xy = 2.f * rx * ry, xz = 2.f * rx * rz, yz = 2.f * ry * rz;
  const float q0 = a.x * xx + a.y * xy + a.z * xz + a.w * yy + b.x * yz + b.y * zz;
  const float q1 = b.z * xx + b.w * xy + c.x * xz + c.y * yy + c.z * yz + c.w * zz;
  const float q2 = d.x * xx + d.y * xy + d.z * xz + d.w * yy + e.x * yz + e.y * zz;
  const float cubic = rx * q0 + ry * q1 + rz * q2;
  const float ur = e.z * rx + e.w * ry + f.x * rz, vr = f.y * rx + f.z * ry + f.w * rz;
  return 0.5f * inv * ri2 * (-3.0f * (2.0f * ur + vr) + 15.0f * ri2 * cubic);
}

// Traversal of one warp's 32 query points in one mesh's tree; returns each
// lane's winding number.  The 32 lanes hold nearby points (Morton order inside
// a brick for band voxels) and walk the tree together: a node is summed
// through its far field only when it is far (|q - p| > beta r,
// aabb_tree.rs:666) for every lane; otherwise the warp opens it, and at a leaf
// every lane takes the exact solid angle.  Node loads are warp-uniform, control
// flow never diverges, and each lane's sum is at least as accurate as its own
// traversal would be.  ORDER 3 adds the third-order far-field term.
template <int ORDER>
__device__ __forceinline__ float wn_traverse(F3 q, const float4* __restrict__ inode, const float4* __restrict__ leaf,
                                             const float4* __restrict__ inode3, const float4* __restrict__ leaf3, int n,
                                             float beta, M2VStats* st, int (*stk)[WN_STACK]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const float beta2 = beta * beta;
  float sum = 0.f, comp = 0.f;  // Kahan-compensated accumulation
  bool overflow = false;
  uint32_t c_exact = 0;  // node visits and far-field evaluations follow from the loop count

  // Tests one node (>= 0 internal, < 0 leaf ~index) for the whole warp and
  // sums its far field or exact solid angle; returns true when the warp has
  // to open it (an internal node that is near for some lane).
  auto visit = [&](int node) -> bool {
    if (node >= 0) {
      const float4 P = inode[5 * node];
      const float rx = P.x - q.x, ry = P.y - q.y, rz = P.z - q.z;
      const float r2 = rx * rx + ry * ry + rz * rz;
      if (!__all_sync(0xffffffffu, r2 > P.w * P.w * beta2)) return true;
      const float4 A = inode[5 * node + 1], B0 = inode[5 * node + 2], B1 = inode[5 * node + 3],
                   B2 = inode[5 * node + 4];
      // a.r / (4 pi r^3) + trace(B) / (4 pi r^3) - 3 r^T B r / (4 pi r^5)
      const float ri = rsqrtf(r2);
      const float ri2 = ri * ri;
      const float inv = ri2 * ri * (1.0f / FOUR_PI);
      const float ar = A.x * rx + A.y * ry + A.z * rz;
      const float brx = B0.x * rx + B0.y * ry + B0.z * rz;
      const float bry = B0.w * rx + B1.x * ry + B1.y * rz;
      const float brz = B1.z * rx + B1.w * ry + B2.x * rz;
      const float rbr = rx * brx + ry * bry + rz * brz;
      float wv = inv * ((ar + A.w) - 3.0f * ri2 * rbr);
      if (ORDER >= 3) wv += far3(inode3 + 6 * node, rx, ry, rz, inv, ri2);
      kahan(sum, comp, wv);
      return false;
    }
    const int li = ~node;
    const float4 P = leaf[5 * li];
    const float rx = P.x - q.x, ry = P.y - q.y, rz = P.z - q.z;
    const float r2 = rx * rx + ry * ry + rz * rz;
    float wv;
    if (__all_sync(0xffffffffu, r2 > P.w * P.w * beta2)) {
      const float4 A = leaf[5 * li + 1];
      const float ri = rsqrtf(r2);
      const float inv = ri * ri * ri * (1.0f / FOUR_PI);
      wv = (A.x * rx + A.y * ry + A.z * rz) * inv;
      if (ORDER >= 3) wv += far3(leaf3 + 6 * li, rx, ry, rz, inv, ri * ri);
    } else {
      ++c_exact;
      wv = tri_wn(leaf[5 * li + 2], leaf[5 * li + 3], leaf[5 * li + 4], q);
    }
    kahan(sum, comp, wv);
    return false;
  };

  // Each iteration opens one node: both children are tested and summed in
  // place; of the children the warp has to open, one is taken next and the
  // other pushed, so the stack holds at most one pending node per level.
  int sp = 0;
  int node = (n > 1) ? (visit(0) ? 0 : -1) : (visit(~0), -1);
  int it = 0;  // nodes opened
  for (; it < n + 2; ++it) {
    if (node < 0) {
      if (sp == 0) break;
      --sp;
      node = stk[w][sp];
      __syncwarp();
    }
    const float4 E = inode[5 * node + 4];
    const int c0 = __float_as_int(E.y), c1 = __float_as_int(E.z);
    const bool o0 = visit(c0), o1 = visit(c1);
    if (o0 && o1) {
      if (sp < WN_STACK) {
        if (lane == 0) stk[w][sp] = c1;
        ++sp;
      } else {
        overflow = true;
      }
      __syncwarp();
      node = c0;
    } else {
      node = o0 ? c0 : (o1 ? c1 : -1);
    }
  }
  if (overflow && lane == 0) atomicExch(&st->error, 3);
  // every visit either opens a node (one per iteration; a stack overflow,
  // flagged above, would drop some), takes a far field or an exact solid angle
  const uint32_t c_visit = (n > 1) ? 1u + 2u * uint32_t(it) : 1u;
  const uint32_t c_far = c_visit - c_exact - uint32_t(it);
  if (lane == 0) {
    atomicAdd(&st->wn_visits, (unsigned long long)c_visit);
    atomicAdd(&st->wn_far, (unsigned long long)c_far);
    atomicAdd(&st->wn_exact, (unsigned long long)c_exact);
  }
  return sum;
}

// Band voxel act[i] of the warp: its grid point and, after the traversal, the
// sign of its distance (mesh_to_volume.rs:264-271).
template <int ORDER>
__device__ __forceinline__ void wn_warp(const uint32_t* __restrict__ act, uint64_t i, bool valid, uint64_t last,
                                        const int4* __restrict__ origins, float* __restrict__ values,
                                        const float4* __restrict__ inode, const float4* __restrict__ leaf,
                                        const float4* __restrict__ inode3, const float4* __restrict__ leaf3, int n,
                                        float h, float beta, float thresh, M2VStats* st, int (*stk)[WN_STACK]) {
  const uint32_t v = valid ? act[i] : act[last];
  const uint32_t b = v >> 9, o = v & 511;
  const int4 org = origins[b];
  const F3 q = f3(fmul(__int2float_rn(org.x + int(o >> 6)), h), fmul(__int2float_rn(org.y + int((o >> 3) & 7)), h),
                  fmul(__int2float_rn(org.z + int(o & 7)), h));
  const float sum = wn_traverse<ORDER>(q, inode, leaf, inode3, leaf3, n, beta, st, stk);
  if (valid) {
    const float d = values[uint64_t(b) * 512 + o];
    values[uint64_t(b) * 512 + o] = (sum < thresh) ? copysignf(d, 1.0f) : copysignf(d, -1.0f);
  }
}

template <int ORDER, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) k_wn_sign(const uint32_t* __restrict__ act, uint64_t na,
                                                        const int4* __restrict__ origins, float* __restrict__ values,
                                                        const float4* __restrict__ inode,
                                                        const float4* __restrict__ leaf,
                                                        const float4* __restrict__ inode3,
                                                        const float4* __restrict__ leaf3, int n, float h, float beta,
                                                        float thresh, M2VStats* st) {
  __shared__ int stk[WARPS][WN_STACK];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint64_t i = (blockIdx.x * uint64_t(WARPS) + w) * 32 + lane;
  if ((blockIdx.x * uint64_t(WARPS) + w) * 32 >= na) return;  // whole warp out of range
  wn_warp<ORDER>(act, i, i < na, na - 1, origins, values, inode, leaf, inode3, leaf3, n, h, beta, thresh, st, stk);
}

// Batches: warps are numbered per mesh (warp_base[m] .. warp_base[m+1]) so
// that a warp never holds voxels of two meshes.
template <int ORDER>
__global__ void __launch_bounds__(WN_THREADS) k_wn_sign_batch(const uint32_t* __restrict__ act,
                                                              const uint32_t* __restrict__ act_base,
                                                              const uint32_t* __restrict__ warp_base, int K,
                                                              const MeshInfo* __restrict__ mi,
                                                              const uint32_t* __restrict__ tri_base,
                                                              const uint32_t* __restrict__ inode_base,
                                                              const int4* __restrict__ origins,
                                                              float* __restrict__ values,
                                                              const float4* __restrict__ inodes,
                                                              const float4* __restrict__ leaves,
                                                              const float4* __restrict__ inodes3,
                                                              const float4* __restrict__ leaves3, M2VStats* stats) {
  __shared__ int stk[WN_WARPS][WN_STACK];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint64_t gw = blockIdx.x * uint64_t(WN_WARPS) + w;
  if (gw >= warp_base[K]) return;  // whole warp out of range
  const int mesh = find_seg(warp_base, K, gw);
  const uint64_t a1 = act_base[mesh + 1];
  const uint64_t i = act_base[mesh] + (gw - warp_base[mesh]) * 32 + lane;
  const MeshInfo M = mi[mesh];
  const uint64_t ib = inode_base[mesh], lb = tri_base[mesh];
  if (ORDER >= 3 && M.order >= 3)
    wn_warp<3>(act, i, i < a1, a1 - 1, origins, values, inodes + 5 * ib, leaves + 5 * lb, inodes3 + 6 * ib,
               leaves3 + 6 * lb, int(M.n_tri), M.h, M.beta, M.thresh, stats + mesh, stk);
  else
    wn_warp<2>(act, i, i < a1, a1 - 1, origins, values, inodes + 5 * ib, leaves + 5 * lb, nullptr, nullptr,
               int(M.n_tri), M.h, M.beta, M.thresh, stats + mesh, stk);
}

// WindingNumbers::approximate (aabb_tree.rs:654-660) at arbitrary points: a
// warp takes 32 consecutive points of the caller's order.
template <int ORDER>
__global__ void __launch_bounds__(WN_THREADS) k_wn_points(const float* __restrict__ pts, uint64_t np,
                                                          const float4* __restrict__ inode,
                                                          const float4* __restrict__ leaf,
                                                          const float4* __restrict__ inode3,
                                                          const float4* __restrict__ leaf3, int n, float beta,
                                                          float* __restrict__ out, M2VStats* st) {
  __shared__ int stk[WN_WARPS][WN_STACK];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint64_t wbase = (blockIdx.x * uint64_t(WN_WARPS) + w) * 32;
  if (wbase >= np) return;
  const uint64_t i = wbase + lane, j = i < np ? i : np - 1;
  const F3 q = f3(pts[3 * j], pts[3 * j + 1], pts[3 * j + 2]);
  const float sum = wn_traverse<ORDER>(q, inode, leaf, inode3, leaf3, n, beta, st, stk);
  if (i < np) out[i] = sum;
}

// Large point sets in no particular order (a warp of 32 scattered points opens
// the union of 32 unrelated cuts) are traversed in Morton order: 30-bit keys
// over the cube of half-size 2 r around the root's dipole centre (points
// outside clamp to its faces, NaN to its low corner).
__device__ __forceinline__ uint32_t expand10(uint32_t v) {
  v &= 0x3ffu;
  v = (v | v << 16) & 0x030000ffu;
  v = (v | v << 8) & 0x0300f00fu;
  v = (v | v << 4) & 0x030c30c3u;
  v = (v | v << 2) & 0x09249249u;
  return v;
}

__global__ void k_point_keys(const float* __restrict__ pts, uint64_t np, const float4* __restrict__ inode,
                             uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= np) return;
  const float4 R = inode[0];
  const float inv = R.w > 0.f ? 0.25f / R.w : 0.f;
  const float c[3] = {R.x, R.y, R.z};
  uint32_t q[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float u = fminf(fmaxf((pts[3 * i + k] - c[k]) * inv + 0.5f, 0.f), 1.f);
    q[k] = uint32_t(fminf(u * 1024.0f, 1023.0f));
  }
  keys[i] = (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
  vals[i] = uint32_t(i);
}

__global__ void k_point_gather(const float* __restrict__ pts, const uint32_t* __restrict__ order, uint64_t np,
                               float* __restrict__ dst) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= np) return;
  const uint64_t k = order[i];
  dst[3 * i] = pts[3 * k];
  dst[3 * i + 1] = pts[3 * k + 1];
  dst[3 * i + 2] = pts[3 * k + 2];
}

__global__ void k_point_scatter(const float* __restrict__ v, const uint32_t* __restrict__ order, uint64_t np,
                                float* __restrict__ out) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i < np) out[order[i]] = v[i];
}

// ------------------------------------------------ exact winding numbers ---
// Direct sum over every triangle (no tree, no far field): the solid angle of
// each triangle in the reference's operation order (IEEE, unfused), the sum
// in double.  A validation instrument for the approximate traversal.
constexpr int EX_THREADS = 256, EX_TILE = 1024;

__global__ void __launch_bounds__(EX_THREADS) k_wn_exact(const float* __restrict__ xyz, uint64_t nv,
                                                         const uint32_t* __restrict__ tri, uint64_t nt,
                                                         const float* __restrict__ pts, uint64_t np,
                                                         double* __restrict__ out, int* __restrict__ err) {
  __shared__ float4 tv[EX_TILE][3];
  const uint64_t i = blockIdx.x * uint64_t(EX_THREADS) + threadIdx.x;
  const bool valid = i < np;
  const F3 q = valid ? f3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]) : f3(0.f, 0.f, 0.f);
  double sum = 0.0;
  for (uint64_t t0 = 0; t0 < nt; t0 += EX_TILE) {
    const int cnt = int((nt - t0) < uint64_t(EX_TILE) ? (nt - t0) : uint64_t(EX_TILE));
    __syncthreads();
    for (int k = threadIdx.x; k < cnt; k += EX_THREADS) {
      const uint64_t t = t0 + k;
      for (int c = 0; c < 3; ++c) {
        const uint32_t vi = tri[3 * t + c];
        if (vi >= nv) {
          atomicExch(err, 1);
          tv[k][c] = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
          tv[k][c] = make_float4(xyz[3 * vi], xyz[3 * vi + 1], xyz[3 * vi + 2], 0.f);
        }
      }
    }
    __syncthreads();
    if (valid)
      for (int k = 0; k < cnt; ++k) sum += double(tri_wn_exact(tv[k][0], tv[k][1], tv[k][2], q));
  }
  if (valid) out[i] = sum;
}

bs_status exact_winding_numbers_impl(bs_ctx* ctx, const float* d_xyz, uint64_t nv, const uint32_t* d_tri,
                                     uint64_t nt, const float* d_pts, uint64_t np, double* d_out) {
  DBuf<int> err(ctx, 1);
  BS_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), ctx->stream));
  if (np)
    BS_KERNEL(ctx, "k_wn_exact", (k_wn_exact<<<unsigned((np + EX_THREADS - 1) / EX_THREADS), EX_THREADS, 0, ctx->stream>>>(
                                     d_xyz, nv, d_tri, nt, d_pts, np, d_out, err.p)));
  int e = 0;
  read_back(ctx, &e, err.p, sizeof e);
  if (e) fail(BS_ERR_INVALID_ARG, "triangle vertex index out of range");
  return BS_OK;
}

// ------------------------------------------------------------ driver ------
static inline unsigned blocks(uint64_t n, unsigned t) { return unsigned((n + t - 1) / t); }

// One set of launches for a batch of meshes (the single-mesh call is a batch
// of one).  Every kernel covers all meshes' triangles, bricks or voxels and
// finds its mesh by a binary search of the per-mesh offsets; host syncs do
// not grow with the number of meshes.  Meshes without triangles get no
// volume (nullptr), as MeshToVolume::convert returns None for them.
struct SplitDst {
  int4* o;
  float* v;
  uint32_t* m;
};

__global__ void k_split(const uint32_t* __restrict__ leaf_base, int K, const SplitDst* __restrict__ dst,
                        const int4* __restrict__ oi, const float* __restrict__ vi, const uint32_t* __restrict__ mi_,
                        uint64_t nb) {
  const uint64_t b = blockIdx.x;
  if (b >= nb) return;
  const int mesh = find_seg(leaf_base, K, b);
  const uint64_t d = b - leaf_base[mesh];
  const SplitDst D = dst[mesh];
  reinterpret_cast<float4*>(D.v + d * 512)[threadIdx.x] = reinterpret_cast<const float4*>(vi + b * 512)[threadIdx.x];
  if (threadIdx.x < 16) D.m[d * 16 + threadIdx.x] = mi_[b * 16 + threadIdx.x];
  if (threadIdx.x == 0) D.o[d] = oi[b];
}

// One BVH per mesh over the triangles T (3 float4 per triangle, meshes in
// [tri_base[m], tri_base[m+1])), from Morton order and PLOC, with the
// far-field records of every node (and the order-3 ones when order3).
// st[m] holds each mesh's centroid bounds.
struct Event {
  cudaEvent_t e = nullptr;
  Event() { BS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming)); }
  ~Event() {
    if (e) cudaEventDestroy(e);
  }
  Event(const Event&) = delete;
  Event& operator=(const Event&) = delete;
};

// Points the context's stream at its side stream for the lifetime of the
// object (allocations, frees, launches and read-backs of the calls inside
// go there) and back afterwards, also when a call throws.
struct SideStream {
  bs_ctx* ctx;
  cudaStream_t main;
  explicit SideStream(bs_ctx* c) : ctx(c), main(c->stream) {
    if (!ctx->side) BS_CUDA(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
    ctx->stream = ctx->side;
  }
  ~SideStream() {
    // a throwing call may leave work in flight that reads buffers the
    // unwinding frees on the main stream: finish it first
    if (std::uncaught_exceptions()) cudaStreamSynchronize(ctx->side);
    ctx->stream = main;
  }
  SideStream(const SideStream&) = delete;
  SideStream& operator=(const SideStream&) = delete;
};

static void build_trees(bs_ctx* ctx, const float4* T, uint64_t nt, int K, const uint32_t* d_tb, const uint32_t* d_ib,
                        const M2VStats* st, bool order3, DBuf<float4>& leaf, DBuf<float4>& inode,
                        DBuf<float4>& leaf3, DBuf<float4>& inode3) {
  cudaStream_t s = ctx->stream;
  DBuf<uint64_t> keys(ctx, nt), keys2(ctx, nt);
  DBuf<uint32_t> vals(ctx, nt), order(ctx, nt);
  BS_KERNEL(ctx, "k_morton", (k_morton<<<blocks(nt, 256), 256, 0, s>>>(T, nt, st, d_tb, K, keys.p, vals.p)));
  {
    size_t tmp = 0;
    BS_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, keys.p, keys2.p, vals.p, order.p, int(nt), 0, 64, s));
    DBuf<uint8_t> t(ctx, tmp);
    BS_CUDA(cub::DeviceRadixSort::SortPairs(t.p, tmp, keys.p, keys2.p, vals.p, order.p, int(nt), 0, 64, s));
  }
  if (K > 1) {
    // stable second pass by mesh: every mesh keeps its full-precision Morton
    // order, so its tree is the one a call for that mesh alone builds
    int mesh_bits = 1;
    while ((1 << mesh_bits) < K) ++mesh_bits;
    DBuf<uint32_t> mk(ctx, nt), mk2(ctx, nt), order2(ctx, nt);
    BS_KERNEL(ctx, "k_mesh_keys", (k_mesh_keys<<<blocks(nt, 256), 256, 0, s>>>(order.p, nt, d_tb, K, mk.p)));
    size_t tmp = 0;
    BS_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, mk.p, mk2.p, order.p, order2.p, int(nt), 0, mesh_bits, s));
    DBuf<uint8_t> t(ctx, tmp);
    BS_CUDA(cub::DeviceRadixSort::SortPairs(t.p, tmp, mk.p, mk2.p, order.p, order2.p, int(nt), 0, mesh_bits, s));
    std::swap(order.p, order2.p);
  }
  keys.reset();
  vals.reset();
  const uint64_t n_int = nt - uint64_t(K);
  leaf = DBuf<float4>(ctx, 5 * nt);
  inode = DBuf<float4>(ctx, 5 * std::max<uint64_t>(n_int, 1));
  if (order3) {
    leaf3 = DBuf<float4>(ctx, 6 * nt);
    inode3 = DBuf<float4>(ctx, 6 * std::max<uint64_t>(n_int, 1));
  }
  DBuf<Sums> lsum(ctx, nt), isum(ctx, std::max<uint64_t>(n_int, 1));
  BS_KERNEL(ctx, "k_leaves", (k_leaves<<<blocks(nt, 256), 256, 0, s>>>(T, order.p, nt, leaf.p, lsum.p, leaf3.p)));
  {
    DBuf<int2> child(ctx, std::max<uint64_t>(n_int, 1));
    DBuf<int> parent_i(ctx, std::max<uint64_t>(n_int, 1)), parent_l(ctx, nt), flags(ctx, std::max<uint64_t>(n_int, 1));
    BS_CUDA(cudaMemsetAsync(parent_l.p, 0xff, nt * sizeof(int), s));  // single-triangle meshes: no parent
    if (n_int) {
      BS_CUDA(cudaMemsetAsync(flags.p, 0, n_int * sizeof(int), s));
      BS_CUDA(cudaMemsetAsync(parent_i.p, 0xff, n_int * sizeof(int), s));  // roots keep -1
      // topology by PLOC over the Morton-ordered triangles, one tree per mesh
      DBuf<Cluster> ca(ctx, nt), cb(ctx, nt);
      DBuf<int> nn(ctx, nt), next_id(ctx, K);
      DBuf<uint32_t> keep(ctx, nt + 1), pos(ctx, nt + 1);
      BS_CUDA(cudaMemsetAsync(next_id.p, 0, K * sizeof(int), s));
      BS_KERNEL(ctx, "k_ploc_init", (k_ploc_init<<<blocks(nt, 256), 256, 0, s>>>(lsum.p, nt, d_tb, K, ca.p)));
      uint32_t nc = uint32_t(nt);
      DBuf<uint32_t> mcnt(ctx, K + 1);
      DBuf<int> ferr(ctx, 1);
      for (int round = 0; nc > uint32_t(K); ++round) {
        if (nc <= uint32_t(PLOC_FIN) * uint32_t(K)) {
          // every mesh small enough: finish each in one block
          BS_CUDA(cudaMemsetAsync(mcnt.p, 0, (K + 1) * sizeof(uint32_t), s));
          BS_KERNEL(ctx, "k_ploc_counts", (k_ploc_counts<<<blocks(nc, 256), 256, 0, s>>>(ca.p, nc, mcnt.p, mcnt.p + K, K)));
          uint32_t mx = 0;
          read_back(ctx, &mx, mcnt.p + K, sizeof mx);
          if (mx <= uint32_t(PLOC_FIN)) {
            const size_t smem = 2 * PLOC_FIN * sizeof(Cluster) + 2 * PLOC_FIN * sizeof(int);
            BS_CUDA(cudaFuncSetAttribute(k_ploc_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
            BS_CUDA(cudaMemsetAsync(ferr.p, 0, sizeof(int), s));
            BS_KERNEL(ctx, "k_ploc_finish", (k_ploc_finish<<<unsigned(K), PLOC_FIN_T, smem, s>>>(ca.p, nc, d_tb, d_ib, next_id.p, child.p,
                                                                                     parent_i.p, parent_l.p, ferr.p)));
            int fe = 0;
            read_back(ctx, &fe, ferr.p, sizeof fe);
            if (fe) fail(BS_ERR_CAPACITY, "tree build did not converge");
            break;
          }
        }
        if (round >= 4096) fail(BS_ERR_CAPACITY, "tree build did not converge");
        BS_KERNEL(ctx, "k_ploc_nn", (k_ploc_nn<<<blocks(nc, PLOC_T), PLOC_T, 0, s>>>(ca.p, nc, nn.p)));
        BS_KERNEL(ctx, "k_ploc_merge", (k_ploc_merge<<<blocks(nc + 1, 256), 256, 0, s>>>(ca.p, nc, nn.p, d_tb, d_ib, next_id.p, child.p,
                                                                                   parent_i.p, parent_l.p, keep.p)));
        exclusive_scan(ctx, keep.p, pos.p, uint64_t(nc) + 1);
        BS_KERNEL(ctx, "k_ploc_compact", (k_ploc_compact<<<blocks(nc, 256), 256, 0, s>>>(ca.p, nc, keep.p, pos.p, cb.p)));
        std::swap(ca.p, cb.p);
        uint32_t next = 0;
        read_back(ctx, &next, pos.p + nc, sizeof next);
        if (next >= nc) fail(BS_ERR_CAPACITY, "tree build made no progress");
        nc = next;
      }
      BS_KERNEL(ctx, "k_refit", (k_refit<<<blocks(nt, 256), 256, 0, s>>>(nt, d_tb, d_ib, K, child.p, parent_i.p, parent_l.p, lsum.p, isum.p,
                                                                      flags.p, inode.p, leaf.p, inode3.p, leaf3.p)));
    }
  }
}

// A batch over one of the per-call limits: each mesh's share of the limit.
struct SplitNeeded {
  std::vector<double> share;  // indexed like the batch's meshes
};

// Throws SplitNeeded (several meshes) or BS_ERR_CAPACITY (one mesh) when the
// per-mesh quantities q exceed `limit` in total.
static void check_limit(const std::vector<uint64_t>& q, const std::vector<int>& which, size_t K_all, double limit,
                        const char* what) {
  double total = 0;
  for (uint64_t v : q) total += double(v);
  if (total < limit) return;
  if (q.size() == 1) fail(BS_ERR_CAPACITY, what);
  SplitNeeded sn;
  sn.share.assign(K_all, 0.0);
  for (size_t m = 0; m < q.size(); ++m) sn.share[size_t(which[m])] = double(q[m]) / limit;
  throw sn;
}

static std::vector<bs_volume*> batch_core(bs_ctx* ctx, const float* d_xyz, const uint32_t* d_tri,
                                          const std::vector<uint64_t>& n_vtx, const std::vector<uint64_t>& n_tri,
                                          const std::vector<bs_m2v_params>& params);

std::vector<bs_volume*> mesh_to_volume_batch_impl(bs_ctx* ctx, const float* d_xyz, const uint32_t* d_tri,
                                                  const std::vector<uint64_t>& n_vtx,
                                                  const std::vector<uint64_t>& n_tri,
                                                  const std::vector<bs_m2v_params>& params) {
  const size_t K = n_tri.size();
  if (n_vtx.size() != K || params.size() != K) fail(BS_ERR_INVALID_ARG, "batch arrays differ in length");
  try {
    return batch_core(ctx, d_xyz, d_tri, n_vtx, n_tri, params);
  } catch (const SplitNeeded& sn) {
    // pack consecutive meshes into chunks holding at most half of the limit
    // and run each chunk on its own (recursively, in case another limit bites)
    std::vector<bs_volume*> out;
    out.reserve(K);
    size_t beg = 0;
    uint64_t vtx_off = 0, tri_off = 0;
    try {
      while (beg < K) {
        size_t end = beg;
        double acc = 0.0;
        do {
          acc += sn.share[end];
          ++end;
        } while (end < K && acc + sn.share[end] <= 0.5);
        std::vector<uint64_t> v(n_vtx.begin() + beg, n_vtx.begin() + end), t(n_tri.begin() + beg, n_tri.begin() + end);
        std::vector<bs_m2v_params> p(params.begin() + beg, params.begin() + end);
        std::vector<bs_volume*> part;
        bool any = false;
        for (uint64_t x : t) any |= x != 0;
        if (any) part = mesh_to_volume_batch_impl(ctx, d_xyz + 3 * vtx_off, d_tri + 3 * tri_off, v, t, p);
        else part.assign(t.size(), nullptr);
        out.insert(out.end(), part.begin(), part.end());
        for (size_t m = beg; m < end; ++m) {
          vtx_off += n_vtx[m];
          tri_off += n_tri[m];
        }
        beg = end;
      }
    } catch (...) {
      for (bs_volume* v : out)
        if (v) volume_release(v);
      throw;
    }
    return out;
  }
}

static std::vector<bs_volume*> batch_core(bs_ctx* ctx, const float* d_xyz, const uint32_t* d_tri,
                                          const std::vector<uint64_t>& n_vtx, const std::vector<uint64_t>& n_tri,
                                          const std::vector<bs_m2v_params>& params) {
  const size_t K_all = n_tri.size();
  std::vector<bs_volume*> result(K_all, nullptr);
  // meshes with triangles, in order
  std::vector<int> which;
  std::vector<MeshInfo> mi;
  std::vector<uint32_t> tri_base(1, 0);
  uint64_t vtx_at = 0, tri_at = 0, nt = 0;
  for (size_t m = 0; m < K_all; ++m) {
    const bs_m2v_params& p = params[m];
    if (!(p.voxel_size > 0.f) || !std::isfinite(p.voxel_size)) fail(BS_ERR_INVALID_ARG, "voxel_size must be > 0");
    if (p.band_width < 0 || p.band_width > 1000000) fail(BS_ERR_INVALID_ARG, "band_width out of range");
    if (p.wn_order != 2 && p.wn_order != 3) fail(BS_ERR_INVALID_ARG, "wn_order must be 2 or 3");
    if (p.wn_tree != 0 && p.wn_tree != 1) fail(BS_ERR_INVALID_ARG, "wn_tree must be 0 or 1");
    if (p.wn_tree == 0 && p.wn_order != 2)
      fail(BS_ERR_INVALID_ARG, "the reference's tree has the order-2 far field only (order 3 needs wn_tree 1)");
    if (p.wn_tree != params[0].wn_tree) fail(BS_ERR_INVALID_ARG, "all meshes of a batch need the same wn_tree");
    if (n_tri[m]) {
      MeshInfo q{};
      q.h = p.voxel_size;
      q.inv_h = 1.0f / p.voxel_size;  // mesh_to_volume.rs:48 (reciprocal, then multiply)
      q.beta = p.wn_beta;
      q.thresh = p.wn_threshold;
      q.band = p.band_width;
      q.order = p.wn_order;
      q.tri_base = uint32_t(tri_at);
      q.n_tri = uint32_t(n_tri[m]);
      q.vtx_base = vtx_at;
      q.n_vtx = n_vtx[m];
      mi.push_back(q);
      which.push_back(int(m));
      nt += n_tri[m];
      if (nt >= (1ull << 31)) fail(BS_ERR_CAPACITY, "more than 2^31 triangles");
      tri_base.push_back(uint32_t(nt));
    }
    vtx_at += n_vtx[m];
    tri_at += n_tri[m];
  }
  const int K = int(mi.size());
  if (K == 0) fail(BS_ERR_EMPTY, "mesh has no triangles");
  cudaStream_t s = ctx->stream;

  // per-mesh tables on the device: MeshInfo[K], tri_base[K+1], inode_base[K+1]
  std::vector<uint32_t> inode_base(K + 1);
  for (int m = 0; m <= K; ++m) inode_base[m] = tri_base[m] - uint32_t(m);
  DBuf<MeshInfo> d_mi(ctx, K);
  DBuf<uint32_t> d_tb(ctx, K + 1), d_ib(ctx, K + 1);
  BS_CUDA(cudaMemcpyAsync(d_mi.p, mi.data(), K * sizeof(MeshInfo), cudaMemcpyHostToDevice, s));
  BS_CUDA(cudaMemcpyAsync(d_tb.p, tri_base.data(), (K + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
  BS_CUDA(cudaMemcpyAsync(d_ib.p, inode_base.data(), (K + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, s));

  DBuf<M2VStats> st(ctx, K);
  std::vector<M2VStats> hst(K);
  {
    M2VStats init{};
    for (int k = 0; k < 3; ++k) {
      init.vmin[k] = 0x7fffffff;
      init.vmax[k] = -0x7fffffff;
      init.cmin[k] = 0xffffffffu;
      init.cmax[k] = 0u;
    }
    std::fill(hst.begin(), hst.end(), init);
    BS_CUDA(cudaMemcpyAsync(st.p, hst.data(), K * sizeof(M2VStats), cudaMemcpyHostToDevice, s));
  }

  DBuf<float4> T(ctx, 3 * nt);
  DBuf<uint32_t> nsub(ctx, nt + 1), soff(ctx, nt + 1);
  BS_KERNEL(ctx, "k_gather", (k_gather<<<blocks(nt + 1, 256), 256, 0, s>>>(d_xyz, d_tri, nt, d_mi.p, d_tb.p, K, T.p, nsub.p, st.p)));
  // the triangles, offsets and stats the tree build reads are ready here
  Event gathered, built;
  BS_CUDA(cudaEventRecord(gathered.e, s));
  exclusive_scan(ctx, nsub.p, soff.p, nt + 1);
  uint32_t total = 0;
  read_back(ctx, hst.data(), st.p, K * sizeof(M2VStats));
  read_back(ctx, &total, soff.p + nt, sizeof(uint32_t));
  std::vector<uint64_t> q_sub(K), q_dir(K);
  std::vector<Dir> dirs(K);
  std::vector<uint64_t> dir_base(K + 1, 0);
  for (int m = 0; m < K; ++m) {
    const M2VStats& q = hst[m];
    if (q.error == 1) fail(BS_ERR_INVALID_ARG, "triangle vertex index out of range");
    if (q.error == 4) fail(BS_ERR_CAPACITY, "coordinates / voxel size exceed the int32 voxel grid");
    for (int k = 0; k < 3; ++k)  // leaf keys pack 21 bits per axis of origin / 8
      if (q.vmin[k] < -(1 << 23) + 64 || q.vmax[k] > (1 << 23) - 64)
        fail(BS_ERR_CAPACITY, "mesh extent / voxel size exceeds +-2^23 voxels per axis");
    q_sub[m] = q.n_sub;
    Dir& d = dirs[m];
    d.bx0 = q.vmin[0] >> 3; d.by0 = q.vmin[1] >> 3; d.bz0 = q.vmin[2] >> 3;
    d.dx = (q.vmax[0] >> 3) - d.bx0 + 1;
    d.dy = (q.vmax[1] >> 3) - d.by0 + 1;
    d.dz = (q.vmax[2] >> 3) - d.bz0 + 1;
    q_dir[m] = uint64_t(d.dx) * d.dy * d.dz;
    dir_base[m + 1] = dir_base[m] + q_dir[m];
  }
  // count of sub-triangles in 64 bit: nsub sums can wrap in uint32
  check_limit(q_sub, which, K_all, 4294967296.0, "more than 2^32 sub-triangles");
  check_limit(q_dir, which, K_all, 4294967294.0 / LIST_CLASSES, "brick directory exceeds 2^29 entries");
  const uint64_t ns = total;
  if (ns == 0) fail(BS_ERR_EMPTY, "no sub-triangles");
  const uint64_t D = dir_base[K];
  DBuf<Dir> d_dirs(ctx, K);
  DBuf<uint64_t> d_db(ctx, K + 1);
  BS_CUDA(cudaMemcpyAsync(d_dirs.p, dirs.data(), K * sizeof(Dir), cudaMemcpyHostToDevice, s));
  BS_CUDA(cudaMemcpyAsync(d_db.p, dir_base.data(), (K + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, s));

  DBuf<SubTri> S(ctx, ns);
  BS_KERNEL(ctx, "k_subdivide", (k_subdivide<<<blocks(nt, 128), 128, 0, s>>>(T.p, nsub.p, soff.p, nt, d_mi.p, d_tb.p, K, S.p)));
  nsub.reset();
  soff.reset();

  const uint64_t DC = D * LIST_CLASSES;
  DBuf<uint32_t> cnt(ctx, DC + 1), pair_off(ctx, DC + 1), flag(ctx, D + 1), bidx(ctx, D + 1);
  BS_CUDA(cudaMemsetAsync(cnt.p, 0, (DC + 1) * sizeof(uint32_t), s));
  BS_KERNEL(ctx, "k_count_pairs", (k_count_pairs<<<blocks(ns, 256), 256, 0, s>>>(S.p, ns, d_dirs.p, d_db.p, cnt.p, st.p)));
  exclusive_scan(ctx, cnt.p, pair_off.p, DC + 1);
  BS_KERNEL(ctx, "k_dir_flags", (k_dir_flags<<<blocks(D + 1, 256), 256, 0, s>>>(pair_off.p, D, flag.p)));
  exclusive_scan(ctx, flag.p, bidx.p, D + 1);
  DBuf<uint32_t> leaf_base(ctx, K + 1), act_base(ctx, K + 1);
  BS_KERNEL(ctx, "k_seg_starts", (k_seg_starts<<<blocks(K + 1, 128), 128, 0, s>>>(bidx.p, d_db.p, K, leaf_base.p)));
  uint32_t nb_np[2];
  read_back(ctx, &nb_np[0], bidx.p + D, sizeof(uint32_t));
  read_back(ctx, &nb_np[1], pair_off.p + DC, sizeof(uint32_t));
  read_back(ctx, hst.data(), st.p, K * sizeof(M2VStats));
  std::vector<uint64_t> q_pairs(K);
  for (int m = 0; m < K; ++m) {
    if (hst[m].error == 2) fail(BS_ERR_CAPACITY, "sub-triangle outside the brick directory");
    q_pairs[m] = hst[m].n_pairs;
  }
  check_limit(q_pairs, which, K_all, 4294967296.0, "more than 2^32 brick/sub-triangle pairs");
  uint64_t nb = nb_np[0];
  const uint64_t np = nb_np[1];
  if (nb >= (1ull << 23)) {  // active voxels are listed as brick << 9 | voxel in 32 bits
    std::vector<uint32_t> lb(K + 1);
    read_back(ctx, lb.data(), leaf_base.p, (K + 1) * sizeof(uint32_t));
    std::vector<uint64_t> q_bricks(K);
    for (int m = 0; m < K; ++m) q_bricks[m] = lb[m + 1] - lb[m];
    check_limit(q_bricks, which, K_all, 8388608.0, "more than 2^23 bricks in one call");
  }
  flag.reset();

  DBuf<int4> origins(ctx, nb);
  DBuf<float> values(ctx, nb * 512);
  DBuf<uint32_t> masks(ctx, nb * 16);
  {
    DBuf<uint32_t> list_off(ctx, nb + 1), list(ctx, np);
    BS_KERNEL(ctx, "k_dir_compact", (k_dir_compact<<<blocks(D, 256), 256, 0, s>>>(cnt.p, pair_off.p, bidx.p, D, d_dirs.p, d_db.p, K, origins.p, list_off.p)));
    BS_CUDA(cudaMemcpyAsync(list_off.p + nb, pair_off.p + DC, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    pair_off.reset();
    bidx.reset();
    BS_KERNEL(ctx, "k_fill_pairs", (k_fill_pairs<<<blocks(ns, 256), 256, 0, s>>>(S.p, ns, d_dirs.p, d_db.p, cnt.p, list.p)));
    cnt.reset();
    const int dt = ctx->tune_dist_threads, db = ctx->tune_dist_batch;
#define BS_DIST(TH, BA)                                                                                            \
  BS_KERNEL(ctx, "k_brick_distance", (k_brick_distance<TH, BA><<<unsigned(nb), TH, 0, s>>>(origins.p, list_off.p,  \
                                                                                            list.p, S.p, d_mi.p,     \
                                                                                            leaf_base.p, K, values.p, \
                                                                                            masks.p, st.p)))
    if (dt == 64 && db == 8)
      BS_DIST(64, 8);
    else if (dt == 64 && db == 32)
      BS_DIST(64, 32);
    else if (dt == 64)
      BS_DIST(64, 16);
    else if (dt == 256 && db == 8)
      BS_DIST(256, 8);
    else if (dt == 256)
      BS_DIST(256, 16);
    else if (db == 8)
      BS_DIST(128, 8);
    else if (db == 32)
      BS_DIST(128, 32);
    else
      BS_DIST(128, 16);
#undef BS_DIST
  }
  S.reset();

  // active voxels, and per mesh its first brick / voxel
  // one tree per mesh over its original triangles, built on the side stream
  // while the distance pass runs (the build's own syncs wait for it alone)
  const bool any3 = std::any_of(mi.begin(), mi.end(), [](const MeshInfo& q) { return q.order >= 3; });
  // wn_tree 0: the reference's SAH tree, traversed per voxel in its summation
  // order (ref_tree.cu); 1: this library's PLOC tree, traversed per warp
  const bool ref_tree = params[size_t(which[0])].wn_tree == 0;
  DBuf<float4> leaf, inode, leaf3, inode3;
  RefTrees rt;
  {
    SideStream side(ctx);
    BS_CUDA(cudaStreamWaitEvent(ctx->stream, gathered.e, 0));
    if (ref_tree) {
      std::vector<float> betas(K);
      for (int m = 0; m < K; ++m) betas[m] = mi[m].beta;
      build_ref_trees(ctx, T.p, nt, K, tri_base.data(), betas, rt);
    } else {
      build_trees(ctx, T.p, nt, K, d_tb.p, d_ib.p, st.p, any3, leaf, inode, leaf3, inode3);
    }
    BS_CUDA(cudaEventRecord(built.e, ctx->stream));
  }

  DBuf<uint32_t> vc(ctx, nb + 1), voff(ctx, nb + 1);
  BS_KERNEL(ctx, "k_brick_popcount", (k_brick_popcount<<<blocks(nb + 1, 256), 256, 0, s>>>(masks.p, nb, vc.p)));
  {
    DBuf<uint32_t> keep(ctx, nb + 1), kpos(ctx, nb + 1);
    BS_KERNEL(ctx, "k_brick_keep", (k_brick_keep<<<blocks(nb + 1, 256), 256, 0, s>>>(vc.p, nb, keep.p)));
    exclusive_scan(ctx, keep.p, kpos.p, nb + 1);
    uint32_t kept = 0;
    read_back(ctx, &kept, kpos.p + nb, sizeof kept);
    if (kept < nb) {
      DBuf<int4> o2(ctx, kept);
      DBuf<float> v2(ctx, uint64_t(kept) * 512);
      DBuf<uint32_t> m2(ctx, uint64_t(kept) * 16);
      BS_KERNEL(ctx, "k_brick_compact", (k_brick_compact<<<unsigned(nb), 128, 0, s>>>(keep.p, kpos.p, nb, origins.p, values.p, masks.p,
                                                                                  o2.p, v2.p, m2.p)));
      BS_KERNEL(ctx, "k_remap_base", (k_remap_base<<<blocks(K + 1, 128), 128, 0, s>>>(leaf_base.p, K, kpos.p)));
      origins = std::move(o2);
      values = std::move(v2);
      masks = std::move(m2);
      nb = kept;
      BS_KERNEL(ctx, "k_brick_popcount", (k_brick_popcount<<<blocks(nb + 1, 256), 256, 0, s>>>(masks.p, nb, vc.p)));
    }
  }
  exclusive_scan(ctx, vc.p, voff.p, nb + 1);
  BS_KERNEL(ctx, "k_act_starts", (k_act_starts<<<blocks(K + 1, 128), 128, 0, s>>>(voff.p, leaf_base.p, K, act_base.p)));
  std::vector<uint32_t> h_leaf_base(K + 1), h_act_base(K + 1);
  read_back(ctx, h_leaf_base.data(), leaf_base.p, (K + 1) * sizeof(uint32_t));
  read_back(ctx, h_act_base.data(), act_base.p, (K + 1) * sizeof(uint32_t));
  const uint64_t na = h_act_base[K];
  std::vector<uint32_t> warp_base(K + 1, 0);
  for (int m = 0; m < K; ++m) warp_base[m + 1] = warp_base[m] + (h_act_base[m + 1] - h_act_base[m] + 31) / 32;
  DBuf<uint32_t> d_wb(ctx, K + 1);
  BS_CUDA(cudaMemcpyAsync(d_wb.p, warp_base.data(), (K + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
  DBuf<uint32_t> act(ctx, std::max<uint64_t>(na, 1));
  if (nb) BS_KERNEL(ctx, "k_emit_active", (k_emit_active<<<blocks(nb * 32, 256), 256, 0, s>>>(masks.p, voff.p, nb, act.p)));
  vc.reset();
  voff.reset();

  // join the tree build; the triangles are freed after it
  BS_CUDA(cudaStreamWaitEvent(s, built.e, 0));
  T.reset();
  unsigned long long rt_cnt[6] = {0, 0, 0, 0, 0, 0};
  if (na > 0 && ref_tree) {
    std::vector<RefSignMesh> rm(K);
    for (int m = 0; m < K; ++m) rm[m] = RefSignMesh{rt.h_roots[m], mi[m].h, mi[m].beta, mi[m].thresh};
    DBuf<RefSignMesh> d_rm(ctx, K);
    DBuf<unsigned long long> d_cnt(ctx, 6);
    BS_CUDA(cudaMemcpyAsync(d_rm.p, rm.data(), K * sizeof(RefSignMesh), cudaMemcpyHostToDevice, s));
    BS_CUDA(cudaMemsetAsync(d_cnt.p, 0, 6 * sizeof(unsigned long long), s));
    ref_tree_sign(ctx, rt, act.p, act_base.p, d_wb.p, warp_base[K], K, d_rm.p, origins.p, values.p, d_cnt.p);
    read_back(ctx, rt_cnt, d_cnt.p, sizeof rt_cnt);
    if (rt_cnt[3]) fail(BS_ERR_CAPACITY, "winding-number traversal stack overflow");
  } else if (na > 0) {
    const uint64_t n_warps = warp_base[K];
#define BS_WN1(O, WP, I3, L3)                                                                                   \
  BS_KERNEL(ctx, "k_wn_sign", (k_wn_sign<O, WP><<<blocks(na, 32 * WP), 32 * WP, 0, s>>>(                      \
                                  act.p, na, origins.p, values.p, inode.p, leaf.p, I3, L3, int(nt), mi[0].h,   \
                                  mi[0].beta, mi[0].thresh, st.p)))
    const int ww = ctx->tune_wn_warps;
    if (K == 1 && mi[0].order < 3) {
      if (ww == 2)
        BS_WN1(2, 2, nullptr, nullptr);
      else if (ww == 8)
        BS_WN1(2, 8, nullptr, nullptr);
      else
        BS_WN1(2, 4, nullptr, nullptr);
    } else if (K == 1) {
      if (ww == 2)
        BS_WN1(3, 2, inode3.p, leaf3.p);
      else if (ww == 8)
        BS_WN1(3, 8, inode3.p, leaf3.p);
      else
        BS_WN1(3, 4, inode3.p, leaf3.p);
    } else if (!any3)
      BS_KERNEL(ctx, "k_wn_sign", (k_wn_sign_batch<2><<<blocks(n_warps, WN_WARPS), WN_THREADS, 0, s>>>(act.p, act_base.p, d_wb.p, K, d_mi.p, d_tb.p,
                                                                                       d_ib.p, origins.p, values.p, inode.p, leaf.p,
                                                                                       nullptr, nullptr, st.p)));
    else
      BS_KERNEL(ctx, "k_wn_sign", (k_wn_sign_batch<3><<<blocks(n_warps, WN_WARPS), WN_THREADS, 0, s>>>(act.p, act_base.p, d_wb.p, K, d_mi.p, d_tb.p,
                                                                                       d_ib.p, origins.p, values.p, inode.p, leaf.p,
                                                                                       inode3.p, leaf3.p, st.p)));
#undef BS_WN1
  }
  read_back(ctx, hst.data(), st.p, K * sizeof(M2VStats));
  uint64_t n_vp = 0, n_p = 0, visits = 0, far = 0, exact = 0, n_ev = 0;
  for (int m = 0; m < K; ++m) {
    if (hst[m].error == 3) fail(BS_ERR_CAPACITY, "winding-number traversal stack overflow");
    n_vp += hst[m].n_vpairs;
    n_ev += hst[m].n_eval;
    n_p += hst[m].n_pairs;
    visits += hst[m].wn_visits;
    far += hst[m].wn_far;
    exact += hst[m].wn_exact;
  }
  if (ref_tree) {  // per voxel rather than per warp
    visits = rt_cnt[0];
    far = rt_cnt[1];
    exact = rt_cnt[2];
  }
  ctx->last_stats[0] = nt;
  ctx->last_stats[1] = ns;
  ctx->last_stats[2] = n_p;
  ctx->last_stats[3] = n_vp;
  ctx->last_stats[4] = nb;
  ctx->last_stats[5] = na;
  ctx->last_stats[6] = visits;
  ctx->last_stats[7] = (far & 0xffffffffull) | (exact << 32);
  ctx->last_stats[8] = BS_STATS_MESH_TO_VOLUME;
  ctx->last_stats[9] = n_ev;
  ctx->last_stats[10] = far;  // full width (per voxel for the reference's tree)
  ctx->last_stats[11] = exact;
  ctx->last_stats[12] = ref_tree ? 0 : 1;
  ctx->last_stats[13] = ref_tree ? rt_cnt[4] : 0;
  ctx->last_stats[14] = ref_tree ? rt_cnt[5] : 0;

  // hand out the volumes
  std::vector<bs_volume*> vols(K, nullptr);
  try {
    for (int m = 0; m < K; ++m) {
      vols[m] = new bs_volume(ctx);
      vols[m]->h = mi[m].h;
      vols[m]->n_leaves = h_leaf_base[m + 1] - h_leaf_base[m];
      vols[m]->n_active = h_act_base[m + 1] - h_act_base[m];
    }
    if (K == 1) {
      vols[0]->d_origins = origins.release();
      vols[0]->d_values = values.release();
      vols[0]->d_masks = masks.release();
    } else {
      std::vector<SplitDst> dst(K);
      for (int m = 0; m < K; ++m) {
        const uint64_t n = std::max<uint64_t>(vols[m]->n_leaves, 1);
        vols[m]->d_origins = dalloc<int4>(ctx, n);
        vols[m]->d_values = dalloc<float>(ctx, n * 512);
        vols[m]->d_masks = dalloc<uint32_t>(ctx, n * 16);
        dst[m] = SplitDst{vols[m]->d_origins, vols[m]->d_values, vols[m]->d_masks};
      }
      DBuf<SplitDst> d_dst(ctx, K);
      BS_CUDA(cudaMemcpyAsync(d_dst.p, dst.data(), K * sizeof(SplitDst), cudaMemcpyHostToDevice, s));
      if (nb)
        BS_KERNEL(ctx, "k_split", (k_split<<<unsigned(nb), 128, 0, s>>>(leaf_base.p, K, d_dst.p, origins.p, values.p, masks.p, nb)));
      BS_CUDA(cudaStreamSynchronize(s));  // the pointer table leaves scope
    }
  } catch (...) {
    for (bs_volume* v : vols)
      if (v) volume_release(v);
    throw;
  }
  for (int m = 0; m < K; ++m) result[size_t(which[m])] = vols[m];
  return result;
}

// ---------------------------------------------------- WindingNumbers ------
// Triangles of one mesh as float4 triples, and their centroid bounds.
__global__ void k_tri_gather(const float* __restrict__ xyz, uint64_t nv, const uint32_t* __restrict__ tri, uint64_t nt,
                             float4* __restrict__ T, M2VStats* st) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= nt) return;
  const uint32_t ia = tri[3 * i], ib = tri[3 * i + 1], ic = tri[3 * i + 2];
  float4 a = make_float4(0, 0, 0, 0), b = a, c = a;
  if (ia >= nv || ib >= nv || ic >= nv) {
    atomicExch(&st->error, 1);
  } else {
    a = make_float4(xyz[3 * ia], xyz[3 * ia + 1], xyz[3 * ia + 2], 0.f);
    b = make_float4(xyz[3 * ib], xyz[3 * ib + 1], xyz[3 * ib + 2], 0.f);
    c = make_float4(xyz[3 * ic], xyz[3 * ic + 1], xyz[3 * ic + 2], 0.f);
  }
  T[3 * i] = a;
  T[3 * i + 1] = b;
  T[3 * i + 2] = c;
  const float cc[3] = {(a.x + b.x + c.x) * (1.0f / 3.0f), (a.y + b.y + c.y) * (1.0f / 3.0f),
                       (a.z + b.z + c.z) * (1.0f / 3.0f)};
  const unsigned mask = __activemask();
  for (int k = 0; k < 3; ++k) {
    warp_min(&st->cmin[k], f2ord(cc[k]), true, mask);
    warp_max(&st->cmax[k], f2ord(cc[k]), true, mask);
  }
}

}  // namespace bs

// WindingNumbers (spatial_partitioning/aabb_tree.rs:622-691): a mesh's tree
// with its far-field records, evaluated at arbitrary points.
struct bs_wn_tree {
  explicit bs_wn_tree(bs_ctx* c) : ctx(c) { ctx->refs++; }
  bs_wn_tree(const bs_wn_tree&) = delete;
  bs_wn_tree& operator=(const bs_wn_tree&) = delete;
  ~bs_wn_tree() {
    cudaSetDevice(ctx->device);
    bs::dfree(ctx, leaf);
    bs::dfree(ctx, inode);
    bs::dfree(ctx, leaf3);
    bs::dfree(ctx, inode3);
    delete ref;
    bs_ctx_release(ctx);
  }
  bs_ctx* ctx;
  uint64_t nt = 0;
  int order = 2;
  float4 *leaf = nullptr, *inode = nullptr, *leaf3 = nullptr, *inode3 = nullptr;
  bs::RefTrees* ref = nullptr;  // the reference's tree (tree kind 0)
};

namespace bs {

static bs_wn_tree* wn_tree_build(bs_ctx* ctx, const float* d_xyz, uint64_t nv, const uint32_t* d_tri, uint64_t nt,
                                 int order, int kind = 1) {
  if (nt == 0) fail(BS_ERR_EMPTY, "mesh has no triangles");
  if (nt >= (1ull << 31)) fail(BS_ERR_CAPACITY, "more than 2^31 triangles");
  if (order != 2 && order != 3) fail(BS_ERR_INVALID_ARG, "order must be 2 or 3");
  if (kind != 0 && kind != 1) fail(BS_ERR_INVALID_ARG, "tree must be 0 or 1");
  if (kind == 0 && order != 2) fail(BS_ERR_INVALID_ARG, "the reference's tree has the order-2 far field only");
  cudaStream_t s = ctx->stream;
  DBuf<float4> T(ctx, 3 * nt);
  DBuf<M2VStats> st(ctx, 1);
  M2VStats init{};
  for (int k = 0; k < 3; ++k) {
    init.cmin[k] = 0xffffffffu;
    init.cmax[k] = 0u;
  }
  BS_CUDA(cudaMemcpyAsync(st.p, &init, sizeof init, cudaMemcpyHostToDevice, s));
  BS_KERNEL(ctx, "k_tri_gather", (k_tri_gather<<<blocks(nt, 256), 256, 0, s>>>(d_xyz, nv, d_tri, nt, T.p, st.p)));
  const uint32_t tb[2] = {0, uint32_t(nt)}, ibase[2] = {0, uint32_t(nt - 1)};
  DBuf<uint32_t> d_tb(ctx, 2), d_ib(ctx, 2);
  BS_CUDA(cudaMemcpyAsync(d_tb.p, tb, sizeof tb, cudaMemcpyHostToDevice, s));
  BS_CUDA(cudaMemcpyAsync(d_ib.p, ibase, sizeof ibase, cudaMemcpyHostToDevice, s));
  DBuf<float4> leaf, inode, leaf3, inode3;
  if (kind == 0) {
    M2VStats hs;
    read_back(ctx, &hs, st.p, sizeof hs);
    if (hs.error == 1) fail(BS_ERR_INVALID_ARG, "triangle vertex index out of range");
    std::unique_ptr<RefTrees> rt(new RefTrees);
    build_ref_trees(ctx, T.p, nt, 1, tb, std::vector<float>(1, 2.0f), *rt);
    bs_wn_tree* t = new bs_wn_tree(ctx);
    t->nt = nt;
    t->order = 2;
    t->ref = rt.release();
    return t;
  }
  build_trees(ctx, T.p, nt, 1, d_tb.p, d_ib.p, st.p, order >= 3, leaf, inode, leaf3, inode3);
  M2VStats hs;
  read_back(ctx, &hs, st.p, sizeof hs);
  if (hs.error == 1) fail(BS_ERR_INVALID_ARG, "triangle vertex index out of range");
  bs_wn_tree* t = new bs_wn_tree(ctx);
  t->nt = nt;
  t->order = order;
  t->leaf = leaf.release();
  t->inode = inode.release();
  t->leaf3 = leaf3.release();
  t->inode3 = inode3.release();
  return t;
}

static void wn_tree_approximate(bs_ctx* ctx, bs_wn_tree* t, const float* d_pts, uint64_t np, float beta,
                                float* d_out) {
  if (np == 0) return;
  cudaStream_t s = ctx->stream;
  if (t->ref) {  // one traversal per point, in the caller's order
    DBuf<unsigned long long> cnt(ctx, 6);
    BS_CUDA(cudaMemsetAsync(cnt.p, 0, 6 * sizeof(unsigned long long), s));
    ref_tree_points(ctx, *t->ref, d_pts, np, beta, d_out, cnt.p);
    unsigned long long h[6];
    read_back(ctx, h, cnt.p, sizeof h);
    if (h[3]) fail(BS_ERR_CAPACITY, "winding-number traversal stack overflow");
    ctx->last_stats[6] = h[0];
    ctx->last_stats[7] = (h[1] & 0xffffffffull) | (h[2] << 32);
    ctx->last_stats[8] = BS_STATS_WINDING_NUMBERS;
    ctx->last_stats[10] = h[1];
    ctx->last_stats[11] = h[2];
    ctx->last_stats[12] = 0;
    return;
  }
  DBuf<M2VStats> st(ctx, 1);
  BS_CUDA(cudaMemsetAsync(st.p, 0, sizeof(M2VStats), s));
  // from 2^20 points on, traverse a Morton-sorted copy and scatter back
  const bool sorted = np >= (1ull << 20) && np < (1ull << 31) && t->nt >= 2;
  DBuf<uint32_t> order;
  DBuf<float> spts, sout;
  const float* q = d_pts;
  float* o = d_out;
  if (sorted) {
    DBuf<uint32_t> keys(ctx, np), keys2(ctx, np), vals(ctx, np);
    order = DBuf<uint32_t>(ctx, np);
    BS_KERNEL(ctx, "k_point_keys", (k_point_keys<<<blocks(np, 256), 256, 0, s>>>(d_pts, np, t->inode, keys.p, vals.p)));
    size_t tmp = 0;
    BS_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, keys.p, keys2.p, vals.p, order.p, int(np), 0, 30, s));
    DBuf<uint8_t> tb(ctx, tmp);
    BS_CUDA(cub::DeviceRadixSort::SortPairs(tb.p, tmp, keys.p, keys2.p, vals.p, order.p, int(np), 0, 30, s));
    spts = DBuf<float>(ctx, 3 * np);
    sout = DBuf<float>(ctx, np);
    BS_KERNEL(ctx, "k_point_gather", (k_point_gather<<<blocks(np, 256), 256, 0, s>>>(d_pts, order.p, np, spts.p)));
    q = spts.p;
    o = sout.p;
  }
  if (t->order >= 3)
    BS_KERNEL(ctx, "k_wn_points", (k_wn_points<3><<<blocks(np, WN_THREADS), WN_THREADS, 0, s>>>(q, np, t->inode, t->leaf, t->inode3,
                                                                                         t->leaf3, int(t->nt), beta, o, st.p)));
  else
    BS_KERNEL(ctx, "k_wn_points", (k_wn_points<2><<<blocks(np, WN_THREADS), WN_THREADS, 0, s>>>(q, np, t->inode, t->leaf, nullptr,
                                                                                         nullptr, int(t->nt), beta, o, st.p)));
  if (sorted)
    BS_KERNEL(ctx, "k_point_scatter", (k_point_scatter<<<blocks(np, 256), 256, 0, s>>>(sout.p, order.p, np, d_out)));
  M2VStats hs;
  read_back(ctx, &hs, st.p, sizeof hs);
  if (hs.error == 3) fail(BS_ERR_CAPACITY, "winding-number traversal stack overflow");
  ctx->last_stats[6] = hs.wn_visits;
  ctx->last_stats[7] = (hs.wn_far & 0xffffffffull) | (hs.wn_exact << 32);
  ctx->last_stats[8] = BS_STATS_WINDING_NUMBERS;
  ctx->last_stats[10] = hs.wn_far;
  ctx->last_stats[11] = hs.wn_exact;
  ctx->last_stats[12] = 1;
}

}  // namespace bs

extern "C" {

bs_status bs_winding_numbers_build(bs_ctx* ctx, const float* d_xyz, uint64_t nv, const uint32_t* d_tri, uint64_t nt,
                                   int order, bs_wn_tree** out) {
  if (!ctx || !out || (nt && (!d_xyz || !d_tri))) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  try {
    BS_CUDA(cudaSetDevice(ctx->device));
    *out = bs::wn_tree_build(ctx, d_xyz, nv, d_tri, nt, order);
    return BS_OK;
  } catch (const bs::Error& e) {
    ctx->last_error = e.msg;
    return e.status;
  } catch (const std::bad_alloc&) {
    return BS_ERR_OOM;
  }
}

bs_status bs_winding_numbers_build_ex(bs_ctx* ctx, const float* d_xyz, uint64_t nv, const uint32_t* d_tri,
                                      uint64_t nt, int order, int tree, bs_wn_tree** out) {
  if (!ctx || !out || (nt && (!d_xyz || !d_tri))) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  try {
    BS_CUDA(cudaSetDevice(ctx->device));
    *out = bs::wn_tree_build(ctx, d_xyz, nv, d_tri, nt, order, tree);
    return BS_OK;
  } catch (const bs::Error& e) {
    ctx->last_error = e.msg;
    return e.status;
  } catch (const std::bad_alloc&) {
    return BS_ERR_OOM;
  }
}

bs_status bs_winding_numbers_approximate(bs_ctx* ctx, const bs_wn_tree* t, const float* d_points, uint64_t n_points,
                                         float beta, float* d_out) {
  if (!ctx || !t || t->ctx != ctx || (n_points && (!d_points || !d_out)) || !(beta > 0.f)) return BS_ERR_INVALID_ARG;
  try {
    BS_CUDA(cudaSetDevice(ctx->device));
    // the reference tree caches its far thresholds for the last beta (stream-ordered state)
    bs::wn_tree_approximate(ctx, const_cast<bs_wn_tree*>(t), d_points, n_points, beta, d_out);
    return BS_OK;
  } catch (const bs::Error& e) {
    ctx->last_error = e.msg;
    return e.status;
  } catch (const std::bad_alloc&) {
    return BS_ERR_OOM;
  }
}

bs_status bs_winding_numbers_free(bs_wn_tree* t) {
  if (!t) return BS_ERR_INVALID_ARG;
  delete t;
  return BS_OK;
}

// Times the distance and sign passes of one mesh -> volume conversion under
// each candidate: the distance pass with 64 / 128 / 256 threads per brick
// and tiles of 8 / 16 / 32 sub-triangles per warp (8 shapes: 256 threads
// take tiles of 8 or 16), the sign pass with 2 / 4 / 8 warps per block; two
// rounds, best of each, and keeps the fastest of each pass for the context's
// later calls.  h_choice: [threads per brick, warps per sign block, tile];
// h_ms (optional, 11 floats): the 8 distance shapes in the order (64, 8),
// (64, 16), (64, 32), (128, 8), (128, 16), (128, 32), (256, 8), (256, 16),
// then the sign pass with 2, 4, 8 warps.
bs_status bs_autotune_mesh_to_volume(bs_ctx* ctx, const float* d_xyz, uint64_t nv, const uint32_t* d_tri, uint64_t nt,
                                     const bs_m2v_params* p, int32_t* h_choice, float* h_ms) {
  if (!ctx || !p || !h_choice || !d_xyz || !d_tri || !nt) return BS_ERR_INVALID_ARG;
  const bool timing0 = ctx->timing;
  const int dt0 = ctx->tune_dist_threads, ww0 = ctx->tune_wn_warps, db0 = ctx->tune_dist_batch;
  auto restore = [&] {
    ctx->timing = timing0;
    ctx->tune_dist_threads = dt0;
    ctx->tune_wn_warps = ww0;
    ctx->tune_dist_batch = db0;
  };
  try {
    BS_CUDA(cudaSetDevice(ctx->device));
    bs_ctx_resolve_stages(ctx);
    auto saved = ctx->stages;
    const int dist_cand[8][2] = {{64, 8}, {64, 16}, {64, 32}, {128, 8}, {128, 16}, {128, 32}, {256, 8}, {256, 16}};
    const int wn_cand[3] = {2, 4, 8};
    double best_d[8], best_w[3];
    for (double& b : best_d) b = 1e30;
    for (double& b : best_w) b = 1e30;
    bs::volume_release(bs::mesh_to_volume_impl(ctx, d_xyz, nv, d_tri, nt, *p));  // warm-up
    ctx->timing = true;
    for (int round = 0; round < 2; ++round) {
      for (int c = 0; c < 8; ++c) {
        ctx->tune_dist_threads = dist_cand[c][0];
        ctx->tune_dist_batch = dist_cand[c][1];
        ctx->tune_wn_warps = wn_cand[c % 3];
        ctx->stages.clear();
        bs::volume_release(bs::mesh_to_volume_impl(ctx, d_xyz, nv, d_tri, nt, *p));
        bs_ctx_resolve_stages(ctx);
        const auto d = ctx->stages.find("k_brick_distance");
        auto w = ctx->stages.find("k_wn_sign");
        if (w == ctx->stages.end()) w = ctx->stages.find("k_rt_sign");  // the reference's tree
        if (d != ctx->stages.end()) best_d[c] = std::min(best_d[c], d->second.ms);
        if (w != ctx->stages.end()) best_w[c % 3] = std::min(best_w[c % 3], w->second.ms);
      }
    }
    int bd = 4, bw = 1;
    for (int c = 0; c < 8; ++c)
      if (best_d[c] < best_d[bd]) bd = c;
    for (int c = 0; c < 3; ++c)
      if (best_w[c] < best_w[bw]) bw = c;
    ctx->stages = saved;
    ctx->timing = timing0;
    ctx->tune_dist_threads = dist_cand[bd][0];
    ctx->tune_dist_batch = dist_cand[bd][1];
    ctx->tune_wn_warps = wn_cand[bw];
    h_choice[0] = ctx->tune_dist_threads;
    h_choice[1] = ctx->tune_wn_warps;
    h_choice[2] = ctx->tune_dist_batch;
    if (h_ms) {
      for (int c = 0; c < 8; ++c) h_ms[c] = float(best_d[c]);
      for (int c = 0; c < 3; ++c) h_ms[8 + c] = float(best_w[c]);
    }
    return BS_OK;
  } catch (const bs::Error& e) {
    restore();
    ctx->last_error = e.msg;
    return e.status;
  } catch (const std::bad_alloc&) {
    restore();
    return BS_ERR_OOM;
  }
}

// Sets the launch shapes directly (0 keeps a value): threads per brick of
// the distance pass (64, 128, 256), warps per sign block (2, 4, 8) and
// sub-triangles per warp tile (8, 16, 32; not 32 with 256 threads).
bs_status bs_ctx_set_launch_shape(bs_ctx* ctx, int32_t dist_threads, int32_t wn_warps, int32_t dist_tile) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  if (dist_threads && dist_threads != 64 && dist_threads != 128 && dist_threads != 256) return BS_ERR_INVALID_ARG;
  if (wn_warps && wn_warps != 2 && wn_warps != 4 && wn_warps != 8) return BS_ERR_INVALID_ARG;
  if (dist_tile && dist_tile != 8 && dist_tile != 16 && dist_tile != 32) return BS_ERR_INVALID_ARG;
  const int th = dist_threads ? dist_threads : ctx->tune_dist_threads;
  // a tile left unset follows the threads: 256 threads take at most 16
  const int ti = dist_tile ? dist_tile : (th == 256 && ctx->tune_dist_batch == 32 ? 16 : ctx->tune_dist_batch);
  if (th == 256 && ti == 32) return BS_ERR_INVALID_ARG;
  ctx->tune_dist_threads = th;
  ctx->tune_dist_batch = ti;
  if (wn_warps) ctx->tune_wn_warps = wn_warps;
  return BS_OK;
}

}  // extern "C"

namespace bs {

bs_volume* mesh_to_volume_impl(bs_ctx* ctx, const float* d_xyz, uint64_t nv, const uint32_t* d_tri, uint64_t nt,
                               const bs_m2v_params& p) {
  if (nt == 0) fail(BS_ERR_EMPTY, "mesh has no triangles");
  return mesh_to_volume_batch_impl(ctx, d_xyz, d_tri, {nv}, {nt}, {p})[0];
}

}  // namespace bs
