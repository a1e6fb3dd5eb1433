// Volume::offset on the GPU (voxel/volume/mod.rs:95-108):
//   1. drop values with |v| > 2h (tiles included) and empty leaves;
//   2. fast sweeping (voxel/fast_sweep.rs): 8 ordered Gauss–Seidel sweeps
//      extending the distance to |d| + 2h, spawning leaves across faces;
//   3. v -= d on every active value.
//
// The reference sweeps leaves popped from a priority queue in lexicographic
// order of the sweep direction, and each leaf's voxels in the same order.  A
// leaf reads only its six face neighbours and writes only itself, so the
// result depends only on the order of face-adjacent pairs.  Processing leaves
// by diagonal plane p = sx*bx + sy*by + sz*bz (brick coordinates) keeps that
// order — a neighbour "before" in the sweep is on plane p - 1, one "after" on
// p + 1 — and all leaves of a plane run in parallel.  Inside a leaf, the same
// holds for voxels on diagonal planes ux + uy + uz.  Leaves a leaf spawns lie
// on the next plane, exactly where the reference's queue would pop them.  So
// the sweeps are bit-identical to the reference's sequential ones.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cmath>

#include "bs_internal.cuh"
#include "leaf_hash.cuh"
#include "sweep_tables.cuh"
#include "volume_upper.cuh"

namespace bs {

static inline unsigned nb_(uint64_t n, unsigned t) { return unsigned((n + t - 1) / t); }

template <class T>
static void scan_ex(bs_ctx* ctx, const T* in, T* out, size_t n) {
  size_t tmp = 0;
  BS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, in, out, n, ctx->stream));
  DBuf<uint8_t> t(ctx, tmp);
  BS_CUDA(cub::DeviceScan::ExclusiveSum(t.p, tmp, in, out, n, ctx->stream));
}

// ------------------------------------------------------------- leaf hash ---
__global__ void k_hash_insert(LeafHash h, const int4* __restrict__ org, uint64_t n, int* __restrict__ err) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int4 o = org[i];
  bool ins;
  const int s = h.insert_key(o.x, o.y, o.z, ins);
  if (s < 0) atomicExch(err, 1);
  else h.vals[s] = int(i);
}

void LeafHashBuf::build(bs_ctx* ctx, const int4* origins, uint64_t n, uint64_t min_capacity) {
  uint64_t cap = 1024;
  while (cap < 2 * std::max<uint64_t>(n, min_capacity)) cap <<= 1;
  keys = DBuf<unsigned long long>(ctx, cap);
  vals = DBuf<int>(ctx, cap);
  BS_CUDA(cudaMemsetAsync(keys.p, 0xff, cap * sizeof(unsigned long long), ctx->stream));
  BS_CUDA(cudaMemsetAsync(vals.p, 0xff, cap * sizeof(int), ctx->stream));
  h.keys = keys.p;
  h.vals = vals.p;
  h.mask = cap - 1;
  if (n) {
    DBuf<int> err(ctx, 1);
    BS_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), ctx->stream));
    BS_KERNEL(ctx, "k_hash_insert", (k_hash_insert<<<nb_(n, 256), 256, 0, ctx->stream>>>(h, origins, n, err.p)));
  }
}

// -------------------------------------------------------------- remove_if ---
// tree_node.rs remove_if(|v| v.abs() > 2h): clears the active bits, counts what remains.
__global__ void k_remove_far(const float* __restrict__ values, uint32_t* __restrict__ masks, uint64_t n, float lim,
                             uint32_t* __restrict__ keep) {
  const uint64_t b = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (b >= n) return;
  uint32_t m = 0;
  if (lane < 16) {
    m = masks[b * 16 + lane];
    uint32_t mm = m;
    while (mm) {
      const int bit = __ffs(mm) - 1;
      mm &= mm - 1;
      if (fabsf(values[b * 512 + lane * 32 + bit]) > lim) m &= ~(1u << bit);
    }
    masks[b * 16 + lane] = m;
  }
  const uint32_t any = __ballot_sync(0xffffffffu, m != 0);
  if (lane == 0) keep[b] = any ? 1u : 0u;
  if (b == n - 1 && lane == 0) keep[n] = 0u;
}

__global__ void k_gather_leaves(const uint32_t* __restrict__ keep, const uint32_t* __restrict__ pos, uint64_t n,
                                const int4* __restrict__ oi, const float* __restrict__ vi, const uint32_t* __restrict__ mi,
                                int4* __restrict__ oo, float* __restrict__ vo, uint32_t* __restrict__ mo) {
  const uint64_t b = blockIdx.x;
  if (b >= n || !keep[b]) return;
  const uint64_t d = pos[b];
  for (int t = threadIdx.x; t < 512; t += blockDim.x) vo[d * 512 + t] = vi[b * 512 + t];
  if (threadIdx.x < 16) mo[d * 16 + threadIdx.x] = mi[b * 16 + threadIdx.x];
  if (threadIdx.x == 0) oo[d] = oi[b];
}

// --------------------------------------------------------------- sweeps ----
struct SweepState {
  int4* org;
  float* val;
  uint32_t* msk;
  uint32_t* frz;  // active masks at the start of fast_sweep (fast_sweep.rs:31)
  LeafHash hash;
  int* n_leaves;  // device counter (spawned leaves are appended)
  uint64_t cap;
  int* overflow;
};

// fast_sweep.rs:509-537, operation for operation.
__device__ __forceinline__ float compute_distance(float a1, float a2, float a3, float h) {
  float t;
  if (a1 > a3) { t = a1; a1 = a3; a3 = t; }
  if (a1 > a2) { t = a1; a1 = a2; a2 = t; }
  if (a2 > a3) { t = a2; a2 = a3; a3 = t; }
  const float s1 = fadd(a1, h);
  if (fabsf(s1) <= a2) return s1;
  const float a1a2_sum = fadd(a1, a2);
  const float h_sq = fmul(h, h);
  const float two_h_sq = fadd(h_sq, h_sq);
  const float a1a2_diff = fsub(a1, a2);
  const float a1a2_diff_sq = fmul(a1a2_diff, a1a2_diff);
  const float s2 = fmul(fadd(a1a2_sum, fsqrt(fsub(two_h_sq, a1a2_diff_sq))), 0.5f);
  if (fabsf(s2) <= a3) return s2;
  const float a1a2a3_sum = fadd(a1a2_sum, a3);
  const float three_h_sq = fadd(two_h_sq, h_sq);
  const float a1a3_diff = fsub(a1, a3);
  const float a1a3_diff_sq = fmul(a1a3_diff, a1a3_diff);
  const float a2a3_diff = fsub(a2, a3);
  const float a2a3_diff_sq = fmul(a2a3_diff, a2a3_diff);
  const float r = fsub(fsub(fsub(three_h_sq, a1a2_diff_sq), a1a3_diff_sq), a2a3_diff_sq);
  return fmul(fadd(a1a2a3_sum, fsqrt(r)), 0.333333343f);  // (1.0 / 3.0) as f32
}

constexpr int SW_WARPS = 4;

struct WarpLeaf {
  float val[512];
  uint32_t msk[16];
  uint32_t frz[16];
  int nb[6];  // -x, +x, -y, +y, -z, +z
};

// Active value at local (x, y, z) of the stencil: center (shared) or a face neighbour (global).
__device__ __forceinline__ bool stencil_at(const WarpLeaf& L, const SweepState& S, int x, int y, int z, float& v) {
  int which = -1;
  if (z < 0) which = 4;
  else if (z > 7) which = 5;
  else if (y < 0) which = 2;
  else if (y > 7) which = 3;
  else if (x < 0) which = 0;
  else if (x > 7) which = 1;
  const int o = ((x & 7) << 6) | ((y & 7) << 3) | (z & 7);
  if (which < 0) {
    if (!((L.msk[o >> 5] >> (o & 31)) & 1u)) return false;
    v = L.val[o];
    return true;
  }
  const int nbi = L.nb[which];
  if (nbi < 0) return false;
  if (!((S.msk[uint64_t(nbi) * 16 + (o >> 5)] >> (o & 31)) & 1u)) return false;
  v = S.val[uint64_t(nbi) * 512 + o];
  return true;
}

// option_min_by with the |.| comparison of fast_sweep.rs:141-144 (a is the + side).
__device__ __forceinline__ bool min_by_abs(bool ha, float a, bool hb, float b, float& out) {
  if (ha && hb) {
    out = (fabsf(a) > fabsf(b)) ? b : a;
    return true;
  }
  if (ha) { out = a; return true; }
  if (hb) { out = b; return true; }
  return false;
}

// fast_sweep.rs:125-183 for one voxel of the center leaf.
__device__ __forceinline__ void sweep_voxel(WarpLeaf& L, const SweepState& S, int x, int y, int z, bool neg_sweep,
                                            float limit_abs, float h) {
  const int o = (x << 6) | (y << 3) | z;
  if ((L.frz[o >> 5] >> (o & 31)) & 1u) return;
  float xp, xn, yp, yn, zp, zn, dx, dy, dz;
  const bool hxp = stencil_at(L, S, x + 1, y, z, xp), hxn = stencil_at(L, S, x - 1, y, z, xn);
  const bool hyp = stencil_at(L, S, x, y + 1, z, yp), hyn = stencil_at(L, S, x, y - 1, z, yn);
  const bool hzp = stencil_at(L, S, x, y, z + 1, zp), hzn = stencil_at(L, S, x, y, z - 1, zn);
  const bool hx = min_by_abs(hxp, xp, hxn, xn, dx);
  const bool hy = min_by_abs(hyp, yp, hyn, yn, dy);
  const bool hz = min_by_abs(hzp, zp, hzn, zn, dz);
  if (!hx && !hy && !hz) return;
  const float first = hx ? dx : (hy ? dy : dz);
  if (bool(signbit(first)) != neg_sweep) return;
  const float d1 = hx ? dx : FAR_F, d2 = hy ? dy : FAR_F, d3 = hz ? dz : FAR_F;
  const float dn_abs = compute_distance(fabsf(d1), fabsf(d2), fabsf(d3), h);
  if (dn_abs > limit_abs) return;
  const bool act = (L.msk[o >> 5] >> (o & 31)) & 1u;
  const float d_old = act ? L.val[o] : FAR_F;
  if (dn_abs < fabsf(d_old)) {
    L.val[o] = neg_sweep ? copysignf(dn_abs, -1.0f) : copysignf(dn_abs, 1.0f);
    atomicOr(&L.msk[o >> 5], 1u << (o & 31));
  }
}

__device__ __forceinline__ void spawn(const SweepState& S, int x, int y, int z, int* dyn_next, int* dyn_next_n) {
  bool ins;
  const int slot = S.hash.insert_key(x, y, z, ins);
  if (slot < 0) {
    atomicExch(S.overflow, 1);
    return;
  }
  if (!ins) return;
  const int idx = atomicAdd(S.n_leaves, 1);
  if (uint64_t(idx) >= S.cap) {
    atomicExch(S.overflow, 1);
    return;
  }
  S.org[idx] = make_int4(x, y, z, 0);  // values, masks and frozen bits of spare leaves are zero
  S.hash.vals[slot] = idx;
  dyn_next[atomicAdd(dyn_next_n, 1)] = idx;
}

// One launch per leaf plane: static leaves [plane_off[p], plane_off[p+1]) of
// the sorted list plus the leaves spawned into this plane by the previous one.
__global__ void __launch_bounds__(32 * SW_WARPS) k_sweep_plane(SweepState S, const int* __restrict__ sorted,
                                                               const uint32_t* __restrict__ plane_off, int p, int n_planes,
                                                               const int* __restrict__ dyn_cur, const int* __restrict__ dyn_cur_n,
                                                               int* __restrict__ dyn_next, int* __restrict__ dyn_next_n,
                                                               int sx, int sy, int sz, int neg_sweep_i, float limit_abs,
                                                               float h) {
  __shared__ WarpLeaf sm[SW_WARPS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  WarpLeaf& L = sm[w];
  const uint32_t sb = p < n_planes ? plane_off[p] : 0u, se = p < n_planes ? plane_off[p + 1] : 0u;
  const int n_static = int(se - sb), n_dyn = *dyn_cur_n;
  const int total = n_static + n_dyn;
  const bool neg_sweep = neg_sweep_i != 0;
  const float lim = limit_abs;
  for (int item = blockIdx.x * SW_WARPS + w; item < total; item += gridDim.x * SW_WARPS) {
    const int leaf = item < n_static ? sorted[sb + item] : dyn_cur[item - n_static];
    const int4 org = S.org[leaf];
    for (int k = lane; k < 512; k += 32) L.val[k] = S.val[uint64_t(leaf) * 512 + k];
    if (lane < 16) {
      L.msk[lane] = S.msk[uint64_t(leaf) * 16 + lane];
      L.frz[lane] = S.frz[uint64_t(leaf) * 16 + lane];
    }
    if (lane < 6) {
      const int ax = lane >> 1, dir = (lane & 1) ? 8 : -8;
      L.nb[lane] = S.hash.find(org.x + (ax == 0 ? dir : 0), org.y + (ax == 1 ? dir : 0), org.z + (ax == 2 ? dir : 0));
    }
    __syncwarp();
    for (int q = 0; q < 22; ++q) {
      const int beg = c_plane_off[q], end = c_plane_off[q + 1];
      for (int k = beg + lane; k < end; k += 32) {
        const int u = c_plane_vox[k];
        const int ux = u >> 6, uy = (u >> 3) & 7, uz = u & 7;
        sweep_voxel(L, S, sx > 0 ? ux : 7 - ux, sy > 0 ? uy : 7 - uy, sz > 0 ? uz : 7 - uz, neg_sweep, lim, h);
      }
      __syncwarp();
    }
    for (int k = lane; k < 512; k += 32) S.val[uint64_t(leaf) * 512 + k] = L.val[k];
    if (lane < 16) S.msk[uint64_t(leaf) * 16 + lane] = L.msk[lane];
    // fast_sweep.rs:185-287: spawn the next leaf along each axis whose
    // "after" face holds a value of the sweep's sign below the limit
    const int fx = sx > 0 ? 7 : 0, fy = sy > 0 ? 7 : 0, fz = sz > 0 ? 7 : 0;
    bool hit[3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      bool any = false;
      for (int k = lane; k < 64; k += 32) {
        const int a = k >> 3, b = k & 7;
        const int o = ax == 0 ? ((fx << 6) | (a << 3) | b) : (ax == 1 ? ((a << 6) | (fy << 3) | b) : ((a << 6) | (b << 3) | fz));
        const bool act = (L.msk[o >> 5] >> (o & 31)) & 1u;
        const float v = L.val[o];
        any |= act && (bool(signbit(v)) == neg_sweep) && (fabsf(v) < lim);
      }
      hit[ax] = __any_sync(0xffffffffu, any);
    }
    if (lane == 0) {
      if (hit[0]) spawn(S, org.x + 8 * sx, org.y, org.z, dyn_next, dyn_next_n);
      if (hit[1]) spawn(S, org.x, org.y + 8 * sy, org.z, dyn_next, dyn_next_n);
      if (hit[2]) spawn(S, org.x, org.y, org.z + 8 * sz, dyn_next, dyn_next_n);
    }
    __syncwarp();
  }
}

__global__ void k_plane_keys(const int4* __restrict__ org, const int* __restrict__ n_dev, int sx, int sy, int sz,
                             int pmin, uint32_t* __restrict__ keys, int* __restrict__ idx, uint32_t* __restrict__ hist) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *n_dev) return;
  const int4 o = org[i];
  const int p = sx * (o.x >> 3) + sy * (o.y >> 3) + sz * (o.z >> 3) - pmin;
  keys[i] = uint32_t(p);
  idx[i] = i;
  atomicAdd(&hist[p], 1u);
}

__global__ void k_brick_bounds(const int4* __restrict__ org, const int* __restrict__ n_dev, int* __restrict__ bb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *n_dev) return;
  const int4 o = org[i];
  atomicMin(&bb[0], o.x >> 3); atomicMax(&bb[3], o.x >> 3);
  atomicMin(&bb[1], o.y >> 3); atomicMax(&bb[4], o.y >> 3);
  atomicMin(&bb[2], o.z >> 3); atomicMax(&bb[5], o.z >> 3);
}

__global__ void k_sub_active(float* __restrict__ val, const uint32_t* __restrict__ msk, uint64_t n, float d) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n * 512) return;
  const uint64_t b = i >> 9;
  const int o = int(i & 511);
  if ((msk[b * 16 + (o >> 5)] >> (o & 31)) & 1u) val[i] = fsub(val[i], d);
}

__global__ void k_leaf_keys(const int4* __restrict__ org, uint64_t n, unsigned long long* __restrict__ keys,
                            uint32_t* __restrict__ idx) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int4 o = org[i];
  keys[i] = leaf_key(o.x, o.y, o.z);
  idx[i] = uint32_t(i);
}

__global__ void k_permute_leaves(const uint32_t* __restrict__ perm, uint64_t n, const int4* __restrict__ oi,
                                 const float* __restrict__ vi, const uint32_t* __restrict__ mi, int4* __restrict__ oo,
                                 float* __restrict__ vo, uint32_t* __restrict__ mo) {
  const uint64_t d = blockIdx.x;
  if (d >= n) return;
  const uint64_t s = perm[d];
  for (int t = threadIdx.x; t < 512; t += blockDim.x) vo[d * 512 + t] = vi[s * 512 + t];
  if (threadIdx.x < 16) mo[d * 16 + threadIdx.x] = mi[s * 16 + threadIdx.x];
  if (threadIdx.x == 0) oo[d] = oi[s];
}

__global__ void k_count_bits(const uint32_t* __restrict__ m, uint64_t n_words, unsigned long long* out) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  unsigned long long c = i < n_words ? __popc(m[i]) : 0;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// Keeps the leaves with an active voxel, in order; returns the new count.
static uint64_t compact_nonempty(bs_ctx* ctx, bs_volume* v, float remove_above) {
  cudaStream_t s = ctx->stream;
  const uint64_t n = v->n_leaves;
  if (n == 0) return 0;
  DBuf<uint32_t> keep(ctx, n + 1), pos(ctx, n + 1);
  BS_KERNEL(ctx, "k_remove_far", (k_remove_far<<<nb_(n * 32, 256), 256, 0, s>>>(v->d_values, v->d_masks, n, remove_above, keep.p)));
  scan_ex(ctx, keep.p, pos.p, n + 1);
  uint32_t m = 0;
  read_back(ctx, &m, pos.p + n, sizeof(uint32_t));
  if (m == n) return n;
  int4* o2 = dalloc<int4>(ctx, m);
  float* v2 = dalloc<float>(ctx, uint64_t(m) * 512);
  uint32_t* m2 = dalloc<uint32_t>(ctx, uint64_t(m) * 16);
  BS_KERNEL(ctx, "k_gather_leaves", (k_gather_leaves<<<unsigned(n), 128, 0, s>>>(keep.p, pos.p, n, v->d_origins, v->d_values, v->d_masks, o2, v2, m2)));
  dfree(ctx, v->d_origins);
  dfree(ctx, v->d_values);
  dfree(ctx, v->d_masks);
  v->d_origins = o2;
  v->d_values = v2;
  v->d_masks = m2;
  v->n_leaves = m;
  return m;
}

// Runs the 8 sweeps with room for `cap` leaves.  Returns false on overflow
// (the caller retries with more room from its copy of the input).
static bool run_sweeps(bs_ctx* ctx, bs_volume* v, uint64_t cap, float h, float limit) {
  cudaStream_t s = ctx->stream;
  const uint64_t n0 = v->n_leaves;
  SweepState S;
  DBuf<int4> org(ctx, cap);
  DBuf<float> val(ctx, cap * 512);
  DBuf<uint32_t> msk(ctx, cap * 16), frz(ctx, cap * 16);
  DBuf<int> n_dev(ctx, 1), overflow(ctx, 1);
  BS_CUDA(cudaMemsetAsync(val.p, 0, cap * 512 * sizeof(float), s));
  BS_CUDA(cudaMemsetAsync(msk.p, 0, cap * 16 * sizeof(uint32_t), s));
  BS_CUDA(cudaMemsetAsync(frz.p, 0, cap * 16 * sizeof(uint32_t), s));
  if (n0) {
    BS_CUDA(cudaMemcpyAsync(org.p, v->d_origins, n0 * sizeof(int4), cudaMemcpyDeviceToDevice, s));
    BS_CUDA(cudaMemcpyAsync(val.p, v->d_values, n0 * 512 * sizeof(float), cudaMemcpyDeviceToDevice, s));
    BS_CUDA(cudaMemcpyAsync(msk.p, v->d_masks, n0 * 16 * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    BS_CUDA(cudaMemcpyAsync(frz.p, v->d_masks, n0 * 16 * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  }
  const int n0i = int(n0);
  BS_CUDA(cudaMemcpyAsync(n_dev.p, &n0i, sizeof(int), cudaMemcpyHostToDevice, s));
  BS_CUDA(cudaMemsetAsync(overflow.p, 0, sizeof(int), s));
  LeafHashBuf hb;
  hb.build(ctx, org.p, n0, cap);
  S.org = org.p;
  S.val = val.p;
  S.msk = msk.p;
  S.frz = frz.p;
  S.hash = hb.h;
  S.n_leaves = n_dev.p;
  S.cap = cap;
  S.overflow = overflow.p;
  const bool neg_sweep = signbit(limit);
  const float limit_abs = fabsf(limit);
  DBuf<int> dyn_a(ctx, cap), dyn_b(ctx, cap), cnt_a(ctx, 1), cnt_b(ctx, 1);
  DBuf<uint32_t> keys(ctx, cap), keys2(ctx, cap);
  DBuf<int> idx(ctx, cap), sorted(ctx, cap);
  DBuf<int> bb(ctx, 6);
  static const int DIRS[8][3] = {{1, 1, 1},  {-1, 1, 1},  {1, -1, 1},  {-1, -1, 1},
                                 {1, 1, -1}, {-1, 1, -1}, {1, -1, -1}, {-1, -1, -1}};
  // spawn chains reach at most the limit from the last existing plane
  const int extra_planes = int(std::ceil(limit_abs * 1.7320508f / (8.0f * h))) + 3;
  for (int d = 0; d < 8; ++d) {
    const int sx = DIRS[d][0], sy = DIRS[d][1], sz = DIRS[d][2];
    int n = 0;
    read_back(ctx, &n, n_dev.p, sizeof(int));
    if (n == 0) break;
    int init_bb[6] = {0x7fffffff, 0x7fffffff, 0x7fffffff, -0x7fffffff, -0x7fffffff, -0x7fffffff};
    BS_CUDA(cudaMemcpyAsync(bb.p, init_bb, sizeof init_bb, cudaMemcpyHostToDevice, s));
    BS_KERNEL(ctx, "k_brick_bounds", (k_brick_bounds<<<nb_(n, 256), 256, 0, s>>>(org.p, n_dev.p, bb.p)));
    int hbb[6];
    read_back(ctx, hbb, bb.p, sizeof hbb);
    const int pmin = (sx > 0 ? hbb[0] : -hbb[3]) + (sy > 0 ? hbb[1] : -hbb[4]) + (sz > 0 ? hbb[2] : -hbb[5]);
    const int pmax = (sx > 0 ? hbb[3] : -hbb[0]) + (sy > 0 ? hbb[4] : -hbb[1]) + (sz > 0 ? hbb[5] : -hbb[2]);
    const int P = pmax - pmin + 1;
    DBuf<uint32_t> hist(ctx, uint64_t(P) + 1), off(ctx, uint64_t(P) + 1);
    BS_CUDA(cudaMemsetAsync(hist.p, 0, (uint64_t(P) + 1) * sizeof(uint32_t), s));
    BS_KERNEL(ctx, "k_plane_keys", (k_plane_keys<<<nb_(n, 256), 256, 0, s>>>(org.p, n_dev.p, sx, sy, sz, pmin, keys.p, idx.p, hist.p)));
    {
      size_t tmp = 0;
      int bits = 1;
      while ((1 << bits) < P + 1 && bits < 31) ++bits;
      BS_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, keys.p, keys2.p, idx.p, sorted.p, n, 0, bits, s));
      DBuf<uint8_t> t(ctx, tmp);
      BS_CUDA(cub::DeviceRadixSort::SortPairs(t.p, tmp, keys.p, keys2.p, idx.p, sorted.p, n, 0, bits, s));
    }
    scan_ex(ctx, hist.p, off.p, uint64_t(P) + 1);
    BS_CUDA(cudaMemsetAsync(cnt_a.p, 0, sizeof(int), s));
    BS_CUDA(cudaMemsetAsync(cnt_b.p, 0, sizeof(int), s));
    int *dc = dyn_a.p, *dn = dyn_b.p, *cc = cnt_a.p, *cn = cnt_b.p;
    const unsigned grid = unsigned(std::max<uint64_t>(64, std::min<uint64_t>(4096, (uint64_t(n) / std::max(P, 1)) / SW_WARPS + 64)));
    for (int p = 0; p < P + extra_planes; ++p) {
      BS_KERNEL(ctx, "k_sweep_plane", (k_sweep_plane<<<grid, 32 * SW_WARPS, 0, s>>>(S, sorted.p, off.p, p, P, dc, cc, dn, cn, sx, sy, sz,
                                                                       neg_sweep ? 1 : 0, limit_abs, h)));
      BS_CUDA(cudaMemsetAsync(cc, 0, sizeof(int), s));
      std::swap(dc, dn);
      std::swap(cc, cn);
    }
    // any spawns left past the last planned plane: keep sweeping until none
    for (int p = P + extra_planes, guard = 0; guard < 1 << 16; ++p, ++guard) {
      int left = 0;
      read_back(ctx, &left, cc, sizeof(int));
      if (left == 0) break;
      BS_KERNEL(ctx, "k_sweep_plane", (k_sweep_plane<<<grid, 32 * SW_WARPS, 0, s>>>(S, sorted.p, off.p, p, P, dc, cc, dn, cn, sx, sy, sz,
                                                                       neg_sweep ? 1 : 0, limit_abs, h)));
      BS_CUDA(cudaMemsetAsync(cc, 0, sizeof(int), s));
      std::swap(dc, dn);
      std::swap(cc, cn);
    }
    int of = 0;
    read_back(ctx, &of, overflow.p, sizeof(int));
    if (of) return false;
  }
  int n = 0, of = 0;
  read_back(ctx, &n, n_dev.p, sizeof(int));
  read_back(ctx, &of, overflow.p, sizeof(int));
  if (of) return false;
  // adopt the swept arrays
  dfree(ctx, v->d_origins);
  dfree(ctx, v->d_values);
  dfree(ctx, v->d_masks);
  v->d_origins = org.release();
  v->d_values = val.release();
  v->d_masks = msk.release();
  v->n_leaves = uint64_t(n);
  return true;
}

void volume_offset_impl(bs_ctx* ctx, bs_volume* v, float distance) {
  cudaStream_t s = ctx->stream;
  const float h = v->h;
  // 1. remove_if(|v| > 2h) (volume/mod.rs:96): tiles all hold +-far and go
  bs_volume_free_upper(v);
  dfree(ctx, v->d_tiles);
  dfree(ctx, v->d_tile_values);
  v->d_tiles = nullptr;
  v->d_tile_values = nullptr;
  v->n_tiles = 0;
  v->dc_valid = false;
  compact_nonempty(ctx, v, h * 2.0f);  // self.voxel_size * 2.0
  // 2. fast sweeping to |d| + 2h with the sign of d (volume/mod.rs:98-102)
  volatile float hv = h;  // (|d| + h) + h in f32, as the reference
  float ext = (std::fabs(distance) + hv) + hv;
  ext = std::signbit(distance) ? -std::fabs(ext) : std::fabs(ext);
  if (v->n_leaves) {
    // the sweeps work on copies and only adopt them on success, so an
    // overflow of the spawned-leaf room just retries with twice the room
    uint64_t cap = 2 * v->n_leaves + 4096;
    bool ok = false;
    for (int attempt = 0; attempt < 6 && !ok; ++attempt, cap *= 2) ok = run_sweeps(ctx, v, cap, h, ext);
    if (!ok) fail(BS_ERR_CAPACITY, "offset: leaf capacity exhausted");
  }
  // fast_sweep.rs:63-65 remove_empty_branches: drop leaves left empty
  if (v->n_leaves) compact_nonempty(ctx, v, INFINITY);
  // 3. v -= distance on every active value (volume/mod.rs:104-105)
  const uint64_t n = v->n_leaves;
  if (n) {
    BS_KERNEL(ctx, "k_sub_active", (k_sub_active<<<nb_(n * 512, 256), 256, 0, s>>>(v->d_values, v->d_masks, n, distance)));
    // canonical leaf order: sorted by origin
    DBuf<unsigned long long> k(ctx, n), k2(ctx, n);
    DBuf<uint32_t> ix(ctx, n), perm(ctx, n);
    BS_KERNEL(ctx, "k_leaf_keys", (k_leaf_keys<<<nb_(n, 256), 256, 0, s>>>(v->d_origins, n, k.p, ix.p)));
    size_t tmp = 0;
    BS_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, k.p, k2.p, ix.p, perm.p, int(n), 0, 63, s));
    {
      DBuf<uint8_t> t(ctx, tmp);
      BS_CUDA(cub::DeviceRadixSort::SortPairs(t.p, tmp, k.p, k2.p, ix.p, perm.p, int(n), 0, 63, s));
    }
    int4* o2 = dalloc<int4>(ctx, n);
    float* v2 = dalloc<float>(ctx, n * 512);
    uint32_t* m2 = dalloc<uint32_t>(ctx, n * 16);
    BS_KERNEL(ctx, "k_permute_leaves", (k_permute_leaves<<<unsigned(n), 128, 0, s>>>(perm.p, n, v->d_origins, v->d_values, v->d_masks, o2, v2, m2)));
    dfree(ctx, v->d_origins);
    dfree(ctx, v->d_values);
    dfree(ctx, v->d_masks);
    v->d_origins = o2;
    v->d_values = v2;
    v->d_masks = m2;
  }
  DBuf<unsigned long long> cnt(ctx, 1);
  BS_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), s));
  if (n) BS_KERNEL(ctx, "k_count_bits", (k_count_bits<<<nb_(n * 16, 256), 256, 0, s>>>(v->d_masks, n * 16, cnt.p)));
  unsigned long long na = 0;
  read_back(ctx, &na, cnt.p, sizeof na);
  v->n_active = na;
}

}  // namespace bs
