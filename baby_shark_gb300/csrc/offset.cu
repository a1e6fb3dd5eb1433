// Volume::offset on the GPU (voxel/volume/mod.rs:95-108):
//   1. drop values with |v| > 2h (tiles included) and empty leaves;
//   2. fast sweeping (voxel/fast_sweep.rs): 8 ordered Gauss–Seidel sweeps
//      extending the distance to |d| + 2h, spawning leaves across faces;
//   3. v -= d on every active value.
//
// The reference sweeps leaves popped from a priority queue in lexicographic
// order of the sweep direction, and each leaf's voxels in the same order.  A
// leaf reads only its six face neighbours and writes only itself, so its
// sweep is a function of its own input, the outputs of the three neighbours
// before it in the sweep order and the inputs of the three after it; leaves
// it spawns lie after it.  The reference's result is therefore the unique
// fixed point of that dependency order.  Here every leaf is queued at once
// and one persistent kernel (k_relax_ring) keeps every resident warp taking
// the next queued leaf; a leaf is queued again whenever a face it read from a
// before-neighbour changes, until nothing is queued or being swept (no host
// round trip per wave of sweeps); a final check drops leaves that only an
// unconverged sweep asked for.  Inside a leaf the voxels go by diagonal
// planes ux + uy + uz, which keeps their order.  So the sweeps are
// bit-identical to the reference's sequential ones, in any order the queue
// happens to take them.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cmath>
#include <vector>

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
// tree_node.rs remove_if(|v| v.abs() > 2h): clears the active bits, counts
// what remains.  One warp per leaf, coalesced: mask word j covers voxels
// 32j .. 32j + 31, one per lane.
__global__ void k_remove_far(const float* __restrict__ values, uint32_t* __restrict__ masks, uint64_t n, float lim,
                             uint32_t* __restrict__ keep) {
  const uint64_t b = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (b >= n) return;
  const uint32_t mine = lane < 16 ? masks[b * 16 + lane] : 0u;
  uint32_t kept = 0, any = 0;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const uint32_t m = __shfl_sync(0xffffffffu, mine, j);
    const bool on = ((m >> lane) & 1u) && !(fabsf(values[b * 512 + j * 32 + lane]) > lim);
    const uint32_t word = __ballot_sync(0xffffffffu, on);
    if (lane == j) kept = word;
    any |= word;
  }
  if (lane < 16 && kept != mine) masks[b * 16 + lane] = kept;
  if (lane == 0) keep[b] = any ? 1u : 0u;
  if (b == n - 1 && lane == 0) keep[n] = 0u;
}

// Leaf copies: one warp per leaf, each lane moving four float4 of the leaf's
// values with all four loads issued before the stores (2 KB in flight per
// warp), streaming (evict-first) since nothing rereads them here.
constexpr int COPY_WARPS = 8;

__device__ __forceinline__ void copy_leaf(uint64_t from, uint64_t to, const int4* __restrict__ oi,
                                          const float* __restrict__ vi, const uint32_t* __restrict__ mi,
                                          int4* __restrict__ oo, float* __restrict__ vo, uint32_t* __restrict__ mo) {
  const int lane = threadIdx.x & 31;
  const float4* src = reinterpret_cast<const float4*>(vi + from * 512);
  float4* dst = reinterpret_cast<float4*>(vo + to * 512);
  const float4 r0 = __ldcs(src + lane), r1 = __ldcs(src + lane + 32), r2 = __ldcs(src + lane + 64),
               r3 = __ldcs(src + lane + 96);
  const uint32_t m = lane < 16 ? __ldcs(mi + from * 16 + lane) : 0u;
  __stcs(dst + lane, r0);
  __stcs(dst + lane + 32, r1);
  __stcs(dst + lane + 64, r2);
  __stcs(dst + lane + 96, r3);
  if (lane < 16) __stcs(mo + to * 16 + lane, m);
  if (lane == 0) oo[to] = oi[from];
}

__global__ void __launch_bounds__(32 * COPY_WARPS) k_gather_leaves(
    const uint32_t* __restrict__ keep, const uint32_t* __restrict__ pos, uint64_t n, const int4* __restrict__ oi,
    const float* __restrict__ vi, const uint32_t* __restrict__ mi, int4* __restrict__ oo, float* __restrict__ vo,
    uint32_t* __restrict__ mo) {
  const uint64_t b = blockIdx.x * uint64_t(COPY_WARPS) + (threadIdx.x >> 5);
  if (b >= n || !keep[b]) return;
  copy_leaf(b, pos[b], oi, vi, mi, oo, vo, mo);
}

// --------------------------------------------------------------- sweeps ----
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

// Sweep state for one direction.  A leaf's sweep (fast_sweep.rs:125-183 over
// its voxels) is a function of its own input, the outputs of its three
// neighbours before it in the sweep order and the inputs of its three
// neighbours after it.  Each slot keeps its input, its output, its three
// after-faces as last published (what its after-neighbours read) and its
// three before-layers of the input (what its before-neighbours read).
struct Sweep {
  int4* org;
  const float* in_val;
  const uint32_t* in_msk;
  float* out_val;
  uint32_t* out_msk;
  const uint32_t* frz;  // active masks when fast_sweep started (fast_sweep.rs:31)
  float* pub_val;       // [slot][axis][64] output after-face, 0 where inactive
  uint32_t* pub_msk;    // [slot][axis][2]
  float* inf_val;       // [slot][axis][64] input before-layer, 0 where inactive
  uint32_t* inf_msk;    // [slot][axis][2]
  int* alive;           // the slot holds a leaf of the volume
  int* spawned;         // the leaf was created during this sweep
  int* wanted;          // a before-neighbour's output asks for it
  int* dirty;           // queued for a sweep
  int* nbr;             // [slot][6] slot of the face neighbour (-x, +x, -y, +y, -z, +z) or -1
  int* linked;          // nbr of the slot is filled in
  int* busy;            // a warp is sweeping the slot (persistent relaxation)
  LeafHash hash;
  int* n_slots;
  uint64_t cap;
  int* overflow;
  int* changed;
  int sx, sy, sz, neg;
  float lim, h;
  // work queue of the persistent relaxation (null: queue into a list)
  unsigned long long* ring;  // entry: position << 32 | slot; RING_EMPTY when free
  uint32_t ring_mask;
  unsigned* qhead;           // next position to take
  unsigned* qtail;           // next position to fill
  int* pending;              // queued or being swept
  int* qerr;                 // a bounded wait gave up
  unsigned long long* n_sweeps;
};

constexpr unsigned long long RING_EMPTY = ~0ull;
constexpr int RING_SPIN = 1 << 24;  // polls before a wait gives up (with back-off, seconds)

constexpr int SW_WARPS = 4;
constexpr int PAD = 10;  // a leaf with a one-voxel halo: 10 x 10 x 10

__device__ __forceinline__ int pad_idx(int x, int y, int z) { return (x + 1) * PAD * PAD + (y + 1) * PAD + (z + 1); }

__device__ __forceinline__ bool bit(const uint32_t* m, int i) { return (m[i >> 5] >> (i & 31)) & 1u; }

// voxel (a, b) of the layer at local coordinate `fl` across axis `ax`
__device__ __forceinline__ int face_off(int ax, int fl, int i) {
  const int a = i >> 3, b = i & 7;
  return ax == 0 ? ((fl << 6) | (a << 3) | b) : (ax == 1 ? ((a << 6) | (fl << 3) | b) : ((a << 6) | (b << 3) | fl));
}
__device__ __forceinline__ int face_pad(int ax, int fl, int i) {
  const int a = i >> 3, b = i & 7;
  return ax == 0 ? pad_idx(fl, a, b) : (ax == 1 ? pad_idx(a, fl, b) : pad_idx(a, b, fl));
}

// option_min_by with the |.| comparison of fast_sweep.rs:141-144, a the + side;
// an inactive neighbour is +inf (active values are finite), so "none" stays +inf.
__device__ __forceinline__ float min_by_abs(float a, float b) { return (fabsf(a) > fabsf(b)) ? b : a; }

// fast_sweep.rs:125-183 for the voxel at padded index p of the tile W.
__device__ __forceinline__ void sweep_voxel(float* W, int p, bool neg_sweep, float limit_abs, float h) {
  const float dx = min_by_abs(W[p + PAD * PAD], W[p - PAD * PAD]);
  const float dy = min_by_abs(W[p + PAD], W[p - PAD]);
  const float dz = min_by_abs(W[p + 1], W[p - 1]);
  const bool hx = dx != INFINITY, hy = dy != INFINITY, hz = dz != INFINITY;
  if (!hx && !hy && !hz) return;
  const float first = hx ? dx : (hy ? dy : dz);
  if (bool(signbit(first)) != neg_sweep) return;
  const float d1 = hx ? dx : FAR_F, d2 = hy ? dy : FAR_F, d3 = hz ? dz : FAR_F;
  const float dn_abs = compute_distance(fabsf(d1), fabsf(d2), fabsf(d3), h);
  if (dn_abs > limit_abs) return;
  // inactive: the reference compares against FAR (f32::MAX); +inf orders the same for dn_abs <= limit
  if (dn_abs < fabsf(W[p])) W[p] = neg_sweep ? copysignf(dn_abs, -1.0f) : copysignf(dn_abs, 1.0f);
}

__device__ __forceinline__ int is_alive(const Sweep& S, int l) { return __ldcg(&S.alive[l]); }

__device__ __forceinline__ int find_alive(const Sweep& S, int x, int y, int z) {
  const int l = S.hash.find(x, y, z);
  return (l >= 0 && is_alive(S, l)) ? l : -1;
}

// Appends slot l to the work queue.  pending counts it before it can be
// taken, so pending reaches 0 only when no leaf is queued or being swept.
// A leaf is queued at most once at a time (its dirty flag), so the ring,
// larger than the slot count, never holds more entries than it has room for;
// an entry is written only into a free cell (a bounded wait for the taker of
// the cell's previous entry to clear it).
__device__ void ring_push(const Sweep& S, int l) {
  atomicAdd(S.pending, 1);
  __threadfence();
  const unsigned pos = atomicAdd(S.qtail, 1u);
  unsigned long long* cell = S.ring + (pos & S.ring_mask);
  const unsigned long long e = (uint64_t(pos) << 32) | uint32_t(l);
  for (int it = 0; it < RING_SPIN; ++it) {
    if (atomicCAS(cell, RING_EMPTY, e) == RING_EMPTY) return;
    __nanosleep(64);
  }
  atomicExch(S.qerr, 1);
}

// Queues leaf l for a sweep unless it is queued already.
__device__ __forceinline__ void mark_dirty(const Sweep& S, int l, int* list, int* cnt) {
  if (atomicExch(&S.dirty[l], 1) == 0) {
    if (S.ring)
      ring_push(S, l);
    else
      list[atomicAdd(cnt, 1)] = l;
  }
}

// Brings back a leaf dropped earlier in the offset and queues it.
__device__ __forceinline__ void revive_leaf(const Sweep& S, int idx, int* list, int* cnt) {
  S.wanted[idx] = 1;
  if (is_alive(S, idx)) return;
  S.spawned[idx] = 1;
  if (atomicExch(&S.alive[idx], 1) == 0) {
    __threadfence();
    atomicExch(S.changed, 1);
    mark_dirty(S, idx, list, cnt);
  }
}

// The leaf at (x, y, z) is asked for (fast_sweep.rs:185-287): create it, or
// bring back one dropped earlier, and queue it.  A created slot fills in its
// neighbour cache on its first sweep.
__device__ void request_leaf(const Sweep& S, int x, int y, int z, int* list, int* cnt) {
  bool ins;
  const int slot = S.hash.insert_key(x, y, z, ins);
  if (slot < 0) {
    atomicExch(S.overflow, 1);
    return;
  }
  int idx;
  if (ins) {
    idx = atomicAdd(S.n_slots, 1);
    if (uint64_t(idx) >= S.cap) {
      atomicExch(S.overflow, 1);
      return;
    }
    S.org[idx] = make_int4(x, y, z, 0);  // spare slots hold empty inputs, outputs and faces
    __threadfence();
    atomicExch(&S.hash.vals[slot], idx);
  } else {
    // the slot may be claimed by another warp right now: wait (bounded) for its index
    idx = -1;
    for (int it = 0; it < (1 << 20) && idx < 0; ++it) idx = atomicAdd(&S.hash.vals[slot], 0);
    if (idx < 0) {
      atomicExch(S.overflow, 1);
      return;
    }
  }
  revive_leaf(S, idx, list, cnt);
}

// The spawn test of fast_sweep.rs:185-287 for one value of an after-face.
__device__ __forceinline__ bool spawns(const Sweep& S, bool on, float v) {
  return on && (bool(signbit(v)) == (S.neg != 0)) && (fabsf(v) < S.lim);
}

// Per block: for the k-th voxel in diagonal-plane order of this sweep
// direction, its padded tile index (low 16 bits) and voxel index (high 16).
__device__ __forceinline__ void fill_order(const Sweep& S, uint32_t* order) {
  for (int k = threadIdx.x; k < 512; k += blockDim.x) {
    const int u = c_plane_vox[k];
    const int x = S.sx > 0 ? (u >> 6) : 7 - (u >> 6);
    const int y = S.sy > 0 ? ((u >> 3) & 7) : 7 - ((u >> 3) & 7);
    const int z = S.sz > 0 ? (u & 7) : 7 - (u & 7);
    order[k] = uint32_t(pad_idx(x, y, z)) | (uint32_t((x << 6) | (y << 3) | z) << 16);
  }
}

// One relaxation pass over the listed leaves.  Each is swept from its input
// with its neighbours' current faces; an after-face that changed queues the
// neighbour behind it, and a face that asks for a missing neighbour creates
// it.  Repeated until nothing is queued, the outputs reach the unique fixed
// point of the before/after dependency order — the result of the reference's
// sequential sweep, whose queue pops every before-neighbour first.
//
// Neighbours come from the slot's cached `nbr`.  A dropped neighbour reads as
// empty (its faces are zero).  A neighbour created after the cache was filled
// is missing from it until that neighbour's first sweep links both ways; it
// only matters as the target of a changed after-face, which falls back to the
// hash.
// Sweeps one leaf from its input with its neighbours' current faces; an
// after-face that changed queues the neighbour behind it, and a face that
// asks for a missing neighbour creates it.  Repeated until nothing is queued,
// the outputs reach the unique fixed point of the before/after dependency
// order — the result of the reference's sequential sweep, whose queue pops
// every before-neighbour first.
//
// Neighbours come from the slot's cached `nbr`.  A dropped neighbour reads as
// empty (its faces are zero).  A neighbour created after the cache was filled
// is missing from it until that neighbour's first sweep links both ways; it
// only matters as the target of a changed after-face, which falls back to the
// hash.
struct RelaxSmem {
  float tile[SW_WARPS][PAD * PAD * PAD];
  float oldf[SW_WARPS][3 * 64];
  uint32_t oldm[SW_WARPS][6];
  uint32_t frz[SW_WARPS][16];
  uint32_t order[512];
};

__device__ void relax_leaf(const Sweep& S, int leaf, RelaxSmem& sm, int* __restrict__ next,
                           int* __restrict__ n_next) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float* W = sm.tile[w];
  uint32_t* F = sm.frz[w];
  const uint32_t* order = sm.order;
  float (*oldf)[3 * 64] = sm.oldf;
  uint32_t (*oldm)[6] = sm.oldm;
  const int sdir[3] = {S.sx, S.sy, S.sz};
  int live = 0;
  if (lane == 0) {
    atomicExch(&S.dirty[leaf], 0);
    __threadfence();
    live = is_alive(S, leaf);
  }
  if (!__shfl_sync(0xffffffffu, live, 0)) return;
  const int4 org = S.org[leaf];
  int nb = -1;
  if (lane < 6) {
    if (__ldcg(&S.linked[leaf])) {
      nb = __ldcg(&S.nbr[uint64_t(leaf) * 6 + lane]);
    } else {  // first sweep of a created slot: link both ways
      const int ax = lane >> 1, step = (lane & 1) ? 8 : -8;
      nb = S.hash.find(org.x + (ax == 0 ? step : 0), org.y + (ax == 1 ? step : 0), org.z + (ax == 2 ? step : 0));
      S.nbr[uint64_t(leaf) * 6 + lane] = nb;
      if (nb >= 0) S.nbr[uint64_t(nb) * 6 + (lane ^ 1)] = leaf;
    }
  }
  // the leaf's input: each lane's four float4 (voxels 4 k4 .. 4 k4 + 3 of
  // z-line k4 / 2, k4 = lane + 32 j) and the mask words, all loads issued
  // before any store, so the leaf costs one memory latency, not sixteen
  const float4* iv4 = reinterpret_cast<const float4*>(S.in_val + uint64_t(leaf) * 512);
  const uint32_t* im = S.in_msk + uint64_t(leaf) * 16;
  {
    float4 in4[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) in4[j] = iv4[lane + 32 * j];
    const uint32_t mw_in = lane < 16 ? im[lane] : 0u;
    const uint32_t fz = lane < 16 ? S.frz[uint64_t(leaf) * 16 + lane] : 0u;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k4 = lane + 32 * j, k = 4 * k4;
      const uint32_t m = __shfl_sync(0xffffffffu, mw_in, k4 >> 3) >> (4 * (k4 & 7));
      const int base = pad_idx(k >> 6, (k >> 3) & 7, k & 7);  // z, z + 1, z + 2, z + 3 follow
      W[base] = (m & 1u) ? in4[j].x : INFINITY;
      W[base + 1] = (m & 2u) ? in4[j].y : INFINITY;
      W[base + 2] = (m & 4u) ? in4[j].z : INFINITY;
      W[base + 3] = (m & 8u) ? in4[j].w : INFINITY;
    }
    if (lane < 16) F[lane] = fz;
  }
  // this leaf's faces as published before: only this warp writes them in this pass
#pragma unroll
  for (int k = lane; k < 3 * 64; k += 32) oldf[w][k] = __ldcg(&S.pub_val[uint64_t(leaf) * 192 + k]);
  if (lane < 6) oldm[w][lane] = __ldcg(&S.pub_msk[uint64_t(leaf) * 6 + lane]);
  // halo: all twelve loads of this lane first, then the tile writes
  float hv[12];
  uint32_t hm[12];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const int n = __shfl_sync(0xffffffffu, nb, k);
    const int ax = k >> 1, side = k & 1;
    // the neighbour on the - side is before the leaf when the sweep goes +
    const bool before = (side == 0) == (sdir[ax] > 0);
    const float* fv = before ? S.pub_val : S.inf_val;
    const uint32_t* fm = before ? S.pub_msk : S.inf_msk;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      hv[2 * k + r] = INFINITY;
      hm[2 * k + r] = 0u;
      if (n >= 0) {
        hv[2 * k + r] = __ldcg(&fv[(uint64_t(n) * 3 + ax) * 64 + lane + 32 * r]);
        hm[2 * k + r] = __ldcg(&fm[(uint64_t(n) * 3 + ax) * 2 + r]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const int ax = k >> 1, side = k & 1;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int i = lane + 32 * r;
      W[face_pad(ax, side ? 8 : -1, i)] = ((hm[2 * k + r] >> lane) & 1u) ? hv[2 * k + r] : INFINITY;
    }
  }
  __syncwarp();
  for (int q = 0; q < 22; ++q) {
    const int beg = c_plane_off[q], end = c_plane_off[q + 1];
    for (int k = beg + lane; k < end; k += 32) {
      const uint32_t e = order[k];
      const int o = int(e >> 16);
      if (!bit(F, o)) sweep_voxel(W, int(e & 0xffffu), S.neg != 0, S.lim, S.h);
    }
    __syncwarp();
  }
  // outputs: the swept values where active, the input elsewhere (read again,
  // batched, from L2), and the active masks assembled from each lane's four
  {
    float4 in4[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) in4[j] = iv4[lane + 32 * j];
    float4* ov4 = reinterpret_cast<float4*>(S.out_val + uint64_t(leaf) * 512);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k4 = lane + 32 * j, k = 4 * k4;
      const int base = pad_idx(k >> 6, (k >> 3) & 7, k & 7);
      const float t0 = W[base], t1 = W[base + 1], t2 = W[base + 2], t3 = W[base + 3];
      const bool a0 = t0 != INFINITY, a1 = t1 != INFINITY, a2 = t2 != INFINITY, a3 = t3 != INFINITY;
      ov4[k4] = make_float4(a0 ? t0 : in4[j].x, a1 ? t1 : in4[j].y, a2 ? t2 : in4[j].z, a3 ? t3 : in4[j].w);
      uint32_t nib = (a0 ? 1u : 0u) | (a1 ? 2u : 0u) | (a2 ? 4u : 0u) | (a3 ? 8u : 0u);
      nib <<= 4 * (lane & 7);
      nib |= __shfl_xor_sync(0xffffffffu, nib, 1);
      nib |= __shfl_xor_sync(0xffffffffu, nib, 2);
      nib |= __shfl_xor_sync(0xffffffffu, nib, 4);
      if ((lane & 7) == 0) S.out_msk[uint64_t(leaf) * 16 + (k4 >> 3)] = nib;
    }
  }
  uint32_t flags = 0;  // bit ax: face changed, bit 3 + ax: face asks for the next leaf
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    const int fl = sdir[ax] > 0 ? 7 : 0;
    const uint64_t fb = uint64_t(leaf) * 3 + ax;
    bool diff = false, any = false;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int i = lane + 32 * r;
      const float t = W[face_pad(ax, fl, i)];
      const bool on = t != INFINITY;
      const float v = on ? t : 0.f;
      any |= spawns(S, on, v);
      const uint32_t mw = __ballot_sync(0xffffffffu, on);
      diff |= (mw != oldm[w][2 * ax + r]) || (__float_as_uint(oldf[w][ax * 64 + i]) != __float_as_uint(v));
      S.pub_val[fb * 64 + i] = v;
      if (lane == 0) S.pub_msk[fb * 2 + r] = mw;
    }
    if (__any_sync(0xffffffffu, diff)) flags |= 1u << ax;
    if (__any_sync(0xffffffffu, any)) flags |= 8u << ax;
  }
  int after3[3];
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) after3[ax] = __shfl_sync(0xffffffffu, nb, 2 * ax + (sdir[ax] > 0 ? 1 : 0));
  __threadfence();
  __syncwarp();
  if (lane == 0) {
    S.linked[leaf] = 1;
    for (int ax = 0; ax < 3; ++ax) {
      const bool chg = (flags >> ax) & 1u, spw = (flags >> (3 + ax)) & 1u;
      if (!chg && !spw) continue;
      const int x = org.x + (ax == 0 ? 8 * sdir[0] : 0), y = org.y + (ax == 1 ? 8 * sdir[1] : 0),
                z = org.z + (ax == 2 ? 8 * sdir[2] : 0);
      int after = after3[ax];
      if (after < 0) after = S.hash.find(x, y, z);  // created after the cache was filled
      if (chg && after >= 0) mark_dirty(S, after, next, n_next);
      if (spw) {
        if (after < 0) request_leaf(S, x, y, z, next, n_next);
        else revive_leaf(S, after, next, n_next);
      }
    }
  }
  __syncwarp();
}

// The queue of a persistent relaxation: the listed leaves, positions 0..n-1.
__global__ void k_ring_start(Sweep S, const int* __restrict__ list, const int* __restrict__ n_list) {
  const int n = *n_list;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) S.ring[i] = (uint64_t(i) << 32) | uint32_t(list[i]);
  if (i == 0) {
    *S.qhead = 0u;
    *S.qtail = unsigned(n);
    *S.pending = n;
  }
}

// Persistent relaxation: every warp takes the next queued leaf, sweeps it
// (queueing the leaves it changes) and takes another, until no leaf is
// queued or being swept.  Waits are bounded; a wait that gives up sets qerr
// and ends the warp (the offset then fails).
__global__ void __launch_bounds__(32 * SW_WARPS, 8) k_relax_ring(Sweep S) {
  __shared__ RelaxSmem sm;
  fill_order(S, sm.order);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  unsigned long long swept = 0;
  for (;;) {
    int leaf = -1;
    if (lane == 0) {
      const unsigned pos = atomicAdd(S.qhead, 1u);
      unsigned long long* cell = S.ring + (pos & S.ring_mask);
      int it = 0;
      for (; it < RING_SPIN; ++it) {
        const unsigned long long e = atomicAdd(cell, 0ull);
        if (e != RING_EMPTY && unsigned(e >> 32) == pos) {
          atomicExch(cell, RING_EMPTY);
          leaf = int(uint32_t(e));
          break;
        }
        if ((it & 7) == 0 && atomicAdd(S.pending, 0) == 0) break;  // nothing left anywhere
        __nanosleep(it < 64 ? 32 : 256);
      }
      if (it == RING_SPIN) atomicExch(S.qerr, 1);
      __threadfence();
    }
    leaf = __shfl_sync(0xffffffffu, leaf, 0);
    if (leaf < 0) break;
    // a leaf queued again while it is being swept waits for that sweep
    int got = 0;
    if (lane == 0) {
      for (int it = 0; it < RING_SPIN && !got; ++it) {
        got = atomicCAS(&S.busy[leaf], 0, 1) == 0;
        if (!got) __nanosleep(64);
      }
      if (!got) atomicExch(S.qerr, 1);
      __threadfence();
    }
    if (__shfl_sync(0xffffffffu, got, 0)) {
      relax_leaf(S, leaf, sm, nullptr, nullptr);
      ++swept;
    }
    if (lane == 0) {
      __threadfence();  // this sweep's writes and pushes before it stops counting
      if (got) atomicExch(&S.busy[leaf], 0);
      atomicSub(S.pending, 1);
    }
  }
  if (lane == 0 && swept) atomicAdd(S.n_sweeps, swept);
}

// Neighbour cache of the leaves present when the offset starts.
__global__ void k_link(Sweep S, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * 6) return;
  const int l = i / 6, k = i - 6 * l;
  const int4 o = S.org[l];
  const int ax = k >> 1, step = (k & 1) ? 8 : -8;
  S.nbr[i] = S.hash.find(o.x + (ax == 0 ? step : 0), o.y + (ax == 1 ? step : 0), o.z + (ax == 2 ? step : 0));
  if (k == 0) S.linked[l] = 1;
}

// Start of a sweep: after-faces published from the input, the input's
// before-layers stored, every live leaf queued.  A live leaf's output is
// written whole by its first sweep (every live leaf is queued, and a leaf
// stops being live only through k_spawn_drop, which clears its output), so
// only a slot that is not live gets its (empty) output here: its input is
// empty too (a dropped leaf's output was cleared, spare slots start empty).
__global__ void __launch_bounds__(128) k_sweep_init(Sweep S, int n, int* list, int* n_list) {
  __shared__ __align__(16) float tile[4][512];
  __shared__ uint32_t tmask[4][16];
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
  const int l = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (l >= n) return;
  const bool live = S.alive[l] != 0;
  if (!live) {
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k = lane; k < 128; k += 32) reinterpret_cast<float4*>(S.out_val + uint64_t(l) * 512)[k] = z;
    if (lane < 16) S.out_msk[uint64_t(l) * 16 + lane] = 0u;
  } else {  // the input, staged with coalesced loads (faces are strided)
    const float4* iv4 = reinterpret_cast<const float4*>(S.in_val + uint64_t(l) * 512);
#pragma unroll
    for (int j = 0; j < 4; ++j) reinterpret_cast<float4*>(tile[wi])[lane + 32 * j] = iv4[lane + 32 * j];
    if (lane < 16) tmask[wi][lane] = S.in_msk[uint64_t(l) * 16 + lane];
    __syncwarp();
  }
  const float* iv = tile[wi];
  const uint32_t* im = tmask[wi];
  const int sdir[3] = {S.sx, S.sy, S.sz};
  for (int ax = 0; ax < 3; ++ax) {
    for (int side = 0; side < 2; ++side) {
      // side 0: the after-face (published output), side 1: the before-layer;
      // a slot that is not live has an empty input, so empty faces
      const int fl = (sdir[ax] > 0) == (side == 0) ? 7 : 0;
      float* fv = side == 0 ? S.pub_val : S.inf_val;
      uint32_t* fm = side == 0 ? S.pub_msk : S.inf_msk;
      for (int r = 0; r < 2; ++r) {
        const int i = lane + 32 * r;
        const int o = face_off(ax, fl, i);
        const bool on = live && bit(im, o);
        fv[(uint64_t(l) * 3 + ax) * 64 + i] = on ? iv[o] : 0.f;
        const uint32_t mw = __ballot_sync(0xffffffffu, on);
        if (lane == 0) fm[(uint64_t(l) * 3 + ax) * 2 + r] = mw;
      }
    }
  }
  if (lane == 0) {
    S.spawned[l] = 0;
    S.dirty[l] = 0;
    if (live) {
      S.dirty[l] = 1;
      list[atomicAdd(n_list, 1)] = l;
    }
  }
}

// Check after the passes converged, step 1: forget who asked for whom.
__global__ void k_spawn_clear(Sweep S, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) S.wanted[i] = 0;
}

// Step 2: every live leaf asks for the leaves its final output calls for.
__global__ void __launch_bounds__(128) k_spawn_mark(Sweep S, int n, int* list, int* n_list) {
  const int lane = threadIdx.x & 31;
  const int l = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (l >= n || !S.alive[l]) return;
  const int sdir[3] = {S.sx, S.sy, S.sz};
  const int4 org = S.org[l];
  const float* ov = S.out_val + uint64_t(l) * 512;
  const uint32_t* om = S.out_msk + uint64_t(l) * 16;
  for (int ax = 0; ax < 3; ++ax) {
    const int fl = sdir[ax] > 0 ? 7 : 0;
    bool any = false;
    for (int r = 0; r < 2; ++r) {
      const int o = face_off(ax, fl, lane + 32 * r);
      any |= spawns(S, bit(om, o), ov[o]);
    }
    if (__any_sync(0xffffffffu, any) && lane == 0)
      request_leaf(S, org.x + (ax == 0 ? 8 * sdir[0] : 0), org.y + (ax == 1 ? 8 * sdir[1] : 0),
                   org.z + (ax == 2 ? 8 * sdir[2] : 0), list, n_list);
  }
}

// Step 3: a leaf created in this sweep that nobody asks for any more is
// dropped (a request that an earlier, unconverged pass made); the leaves
// behind its after-faces are queued again.
__global__ void __launch_bounds__(128) k_spawn_drop(Sweep S, int n, int* list, int* n_list) {
  const int lane = threadIdx.x & 31;
  const int l = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (l >= n || !S.spawned[l] || !S.alive[l] || S.wanted[l]) return;
  for (int k = lane; k < 512; k += 32) S.out_val[uint64_t(l) * 512 + k] = 0.f;
  if (lane < 16) S.out_msk[uint64_t(l) * 16 + lane] = 0u;
  for (int k = lane; k < 3 * 64; k += 32) S.pub_val[uint64_t(l) * 192 + k] = 0.f;
  if (lane < 6) S.pub_msk[uint64_t(l) * 6 + lane] = 0u;
  __threadfence();
  __syncwarp();
  if (lane == 0) {
    atomicExch(&S.alive[l], 0);
    atomicExch(S.changed, 1);
    const int4 org = S.org[l];
    const int sdir[3] = {S.sx, S.sy, S.sz};
    for (int ax = 0; ax < 3; ++ax) {
      const int a = find_alive(S, org.x + (ax == 0 ? 8 * sdir[0] : 0), org.y + (ax == 1 ? 8 * sdir[1] : 0),
                               org.z + (ax == 2 ? 8 * sdir[2] : 0));
      if (a >= 0) mark_dirty(S, a, list, n_list);
    }
  }
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

__global__ void __launch_bounds__(32 * COPY_WARPS) k_permute_leaves(
    const uint32_t* __restrict__ perm, uint64_t n, const int4* __restrict__ oi, const float* __restrict__ vi,
    const uint32_t* __restrict__ mi, int4* __restrict__ oo, float* __restrict__ vo, uint32_t* __restrict__ mo) {
  const uint64_t d = blockIdx.x * uint64_t(COPY_WARPS) + (threadIdx.x >> 5);
  if (d >= n) return;
  copy_leaf(perm[d], d, oi, vi, mi, oo, vo, mo);
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
  BS_KERNEL(ctx, "k_gather_leaves", (k_gather_leaves<<<nb_(n, COPY_WARPS), 32 * COPY_WARPS, 0, s>>>(keep.p, pos.p, n, v->d_origins, v->d_values, v->d_masks, o2, v2, m2)));
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
  DBuf<int4> org(ctx, cap);
  DBuf<float> val_a(ctx, cap * 512), val_b(ctx, cap * 512), pub_val(ctx, cap * 192), inf_val(ctx, cap * 192);
  DBuf<uint32_t> msk_a(ctx, cap * 16), msk_b(ctx, cap * 16), frz(ctx, cap * 16), pub_msk(ctx, cap * 6),
      inf_msk(ctx, cap * 6);
  DBuf<int> flags(ctx, cap * 6), list(ctx, cap), ctl(ctx, 16), nbr(ctx, cap * 6);
  // every spare slot is an empty leaf: zero inputs, outputs, faces and flags
  BS_CUDA(cudaMemsetAsync(val_a.p, 0, cap * 512 * sizeof(float), s));
  BS_CUDA(cudaMemsetAsync(val_b.p, 0, cap * 512 * sizeof(float), s));
  BS_CUDA(cudaMemsetAsync(msk_a.p, 0, cap * 16 * sizeof(uint32_t), s));
  BS_CUDA(cudaMemsetAsync(msk_b.p, 0, cap * 16 * sizeof(uint32_t), s));
  BS_CUDA(cudaMemsetAsync(frz.p, 0, cap * 16 * sizeof(uint32_t), s));
  BS_CUDA(cudaMemsetAsync(pub_val.p, 0, cap * 192 * sizeof(float), s));
  BS_CUDA(cudaMemsetAsync(pub_msk.p, 0, cap * 6 * sizeof(uint32_t), s));
  BS_CUDA(cudaMemsetAsync(inf_val.p, 0, cap * 192 * sizeof(float), s));
  BS_CUDA(cudaMemsetAsync(inf_msk.p, 0, cap * 6 * sizeof(uint32_t), s));
  BS_CUDA(cudaMemsetAsync(flags.p, 0, cap * 6 * sizeof(int), s));
  BS_CUDA(cudaMemsetAsync(ctl.p, 0, 16 * sizeof(int), s));
  int* alive = flags.p;
  BS_CUDA(cudaMemcpyAsync(org.p, v->d_origins, n0 * sizeof(int4), cudaMemcpyDeviceToDevice, s));
  BS_CUDA(cudaMemcpyAsync(val_a.p, v->d_values, n0 * 512 * sizeof(float), cudaMemcpyDeviceToDevice, s));
  BS_CUDA(cudaMemcpyAsync(msk_a.p, v->d_masks, n0 * 16 * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  BS_CUDA(cudaMemcpyAsync(frz.p, v->d_masks, n0 * 16 * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  {
    std::vector<int> ones(n0, 1);
    BS_CUDA(cudaMemcpyAsync(alive, ones.data(), n0 * sizeof(int), cudaMemcpyHostToDevice, s));
    const int n0i = int(n0);
    BS_CUDA(cudaMemcpyAsync(ctl.p + 3, &n0i, sizeof(int), cudaMemcpyHostToDevice, s));
    BS_CUDA(cudaStreamSynchronize(s));  // `ones` leaves scope
  }
  LeafHashBuf hb;
  hb.build(ctx, org.p, n0, cap);
  // ctl: [0] length of `list` (leaves to queue), [3] used slots, [4] overflow, [5] changed,
  //      [8] ring head, [9] ring tail, [10] pending, [11] a wait gave up
  int* cnt = ctl.p;
  Sweep S;
  S.org = org.p;
  S.frz = frz.p;
  S.pub_val = pub_val.p;
  S.pub_msk = pub_msk.p;
  S.inf_val = inf_val.p;
  S.inf_msk = inf_msk.p;
  S.alive = alive;
  S.spawned = flags.p + cap;
  S.wanted = flags.p + 2 * cap;
  S.dirty = flags.p + 3 * cap;
  S.linked = flags.p + 4 * cap;
  S.busy = flags.p + 5 * cap;
  S.nbr = nbr.p;
  S.hash = hb.h;
  S.n_slots = ctl.p + 3;
  S.cap = cap;
  S.overflow = ctl.p + 4;
  S.changed = ctl.p + 5;
  S.neg = signbit(limit) ? 1 : 0;
  S.lim = fabsf(limit);
  S.h = h;
  S.ring = nullptr;
  // persistent relaxation: one resident grid per phase, its queue in a ring
  // with room for every slot and four claims per resident warp
  int occ = 0, n_sm = 0;
  BS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_relax_ring, 32 * SW_WARPS, 0));
  BS_CUDA(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, ctx->device));
  const unsigned ring_grid = unsigned(std::max(1, occ) * std::max(1, n_sm));
  uint64_t rsize = 1024;
  while (rsize < cap + 4ull * ring_grid * SW_WARPS) rsize <<= 1;
  DBuf<unsigned long long> ring_buf(ctx, rsize), sweeps(ctx, 1);
  BS_CUDA(cudaMemsetAsync(ring_buf.p, 0xff, rsize * sizeof(unsigned long long), s));
  BS_CUDA(cudaMemsetAsync(sweeps.p, 0, sizeof(unsigned long long), s));
  Sweep SR = S;  // the same state, queueing into the ring
  SR.ring = ring_buf.p;
  SR.ring_mask = uint32_t(rsize - 1);
  SR.qhead = reinterpret_cast<unsigned*>(ctl.p + 8);
  SR.qtail = reinterpret_cast<unsigned*>(ctl.p + 9);
  SR.pending = ctl.p + 10;
  SR.qerr = ctl.p + 11;
  SR.n_sweeps = sweeps.p;
  BS_KERNEL(ctx, "k_link", (k_link<<<nb_(n0 * 6, 256), 256, 0, s>>>(S, int(n0))));
  float* vals[2] = {val_a.p, val_b.p};
  uint32_t* msks[2] = {msk_a.p, msk_b.p};
  int cur = 0;
  uint64_t total_passes = 0, total_sweeps = 0;
  static const int DIRS[8][3] = {{1, 1, 1},  {-1, 1, 1},  {1, -1, 1},  {-1, -1, 1},
                                 {1, 1, -1}, {-1, 1, -1}, {1, -1, -1}, {-1, -1, -1}};
  for (int d = 0; d < 8; ++d) {
    S.sx = DIRS[d][0];
    S.sy = DIRS[d][1];
    S.sz = DIRS[d][2];
    S.in_val = vals[cur];
    S.in_msk = msks[cur];
    S.out_val = vals[cur ^ 1];
    S.out_msk = msks[cur ^ 1];
    int n = 0;
    BS_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int), s));
    read_back(ctx, &n, S.n_slots, sizeof(int));
    BS_KERNEL(ctx, "k_sweep_init", (k_sweep_init<<<nb_(uint64_t(n) * 32, 128), 128, 0, s>>>(S, n, list.p, cnt)));
    int pass = 0;
    {
      const Sweep SD = [&] {
        Sweep t = SR;
        t.sx = S.sx;
        t.sy = S.sy;
        t.sz = S.sz;
        t.in_val = S.in_val;
        t.in_msk = S.in_msk;
        t.out_val = S.out_val;
        t.out_msk = S.out_msk;
        return t;
      }();
      for (;;) {
        // the queued leaves (list, cnt[0]) into the ring, then one
        // persistent relaxation until nothing is queued
        BS_KERNEL(ctx, "k_ring_start", (k_ring_start<<<nb_(cap, 256), 256, 0, s>>>(SD, list.p, cnt)));
        BS_KERNEL(ctx, "k_relax_ring", (k_relax_ring<<<ring_grid, 32 * SW_WARPS, 0, s>>>(SD)));
        ++pass;
        int qe = 0;
        read_back(ctx, &qe, SR.qerr, sizeof(int));
        if (qe) fail(BS_ERR_TIMEOUT, "offset: a wait of the persistent relaxation gave up");
        read_back(ctx, &n, S.n_slots, sizeof(int));
        if (uint64_t(n) > cap) return false;
        BS_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int), s));
        BS_CUDA(cudaMemsetAsync(S.changed, 0, sizeof(int), s));
        BS_KERNEL(ctx, "k_spawn_clear", (k_spawn_clear<<<nb_(uint64_t(n), 256), 256, 0, s>>>(S, n)));
        BS_KERNEL(ctx, "k_spawn_mark", (k_spawn_mark<<<nb_(uint64_t(n) * 32, 128), 128, 0, s>>>(S, n, list.p, cnt)));
        BS_KERNEL(ctx, "k_spawn_drop", (k_spawn_drop<<<nb_(uint64_t(n) * 32, 128), 128, 0, s>>>(S, n, list.p, cnt)));
        int ch = 0;
        read_back(ctx, &ch, S.changed, sizeof(int));
        if (!ch) break;
        if (pass >= (1 << 16)) fail(BS_ERR_TIMEOUT, "offset: sweep relaxation did not converge");
      }
    }
    total_passes += uint64_t(pass);
    int of = 0;
    read_back(ctx, &of, S.overflow, sizeof(int));
    if (of) return false;
    cur ^= 1;
  }
  int n = 0;
  read_back(ctx, &n, S.n_slots, sizeof(int));
  {
    unsigned long long sw = 0;
    read_back(ctx, &sw, sweeps.p, sizeof sw);
    total_sweeps = sw;
  }
  ctx->last_stats[6] = total_passes;
  ctx->last_stats[7] = total_sweeps;
  ctx->last_stats[8] = BS_STATS_OFFSET;
  // adopt the swept arrays (dead and empty slots go with the next compaction)
  dfree(ctx, v->d_origins);
  dfree(ctx, v->d_values);
  dfree(ctx, v->d_masks);
  v->d_origins = org.release();
  v->d_values = cur == 0 ? val_a.release() : val_b.release();
  v->d_masks = cur == 0 ? msk_a.release() : msk_b.release();
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
  v->mc_valid = false;
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
    BS_KERNEL(ctx, "k_permute_leaves", (k_permute_leaves<<<nb_(n, COPY_WARPS), 32 * COPY_WARPS, 0, s>>>(perm.p, n, v->d_origins, v->d_values, v->d_masks, o2, v2, m2)));
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
