// Volume booleans on the GPU: flood fill and CSG with the reference tree's
// tile semantics (voxel/volume/mod.rs:74-93).
//
// A volume is leaves (8^3 bricks) plus two internal levels stored as dense
// slot tables, one table per node:
//   L1: 16^3 slots per 128^3-voxel node, a slot holds a leaf      (InternalNode<4>)
//   L2: 32^3 slots per 4096^3-voxel node, a slot holds an L1 node (InternalNode<5>)
//   root: the sorted list of L2 node origins                     (RootNode, BTreeMap)
// Slot state: >= 0 child index, -1 empty, -2 active tile; plus one float per
// slot (the tile half of the reference's child union).  Flood fill and the
// per-slot CSG decisions run as kernels over all slots and leaves; only the
// root level (a handful of keys) is decided on the host.
//
// Reference behaviour kept on purpose (it changes results):
//  * an internal node's last_value_sign() reads its last child's FIRST value
//    (internal_node/flood_fill.rs:103-109);
//  * flood fill writes signed far values into empty slots without activating
//    them (internal_node/flood_fill.rs:64-69); CSG reads those signs;
//  * leaf CSG ORs the active masks for all three operations (leaf_node/csg.rs:17-39);
//  * the root fills z-gaps between two "inside" children with all-inside
//    nodes (root_node/flood_fill.rs:8-42).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cmath>
#include <map>

#include "bs_internal.cuh"
#include "volume_upper.cuh"

namespace bs {

template <class T>
static void scan_excl(bs_ctx* ctx, const T* in, T* out, size_t n) {
  size_t tmp = 0;
  BS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, in, out, n, ctx->stream));
  DBuf<uint8_t> t(ctx, tmp);
  BS_CUDA(cub::DeviceScan::ExclusiveSum(t.p, tmp, in, out, n, ctx->stream));
}

static inline unsigned nblk(uint64_t n, unsigned t) { return unsigned((n + t - 1) / t); }

// ------------------------------------------------------ building levels ---
// key of the node (at `shift`) containing voxel (x, y, z): lexicographic (x, y, z)
__device__ __forceinline__ uint64_t pack_key(int x, int y, int z, int shift) {
  return (uint64_t(uint32_t((x >> shift) + (1 << 20))) << 42) | (uint64_t(uint32_t((y >> shift) + (1 << 20))) << 21) |
         uint64_t(uint32_t((z >> shift) + (1 << 20)));
}

__global__ void k_child_keys(const int4* __restrict__ org, uint64_t n, int shift, uint64_t* __restrict__ keys,
                             uint32_t* __restrict__ vals) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  int4 o = org[i];
  keys[i] = pack_key(o.x, o.y, o.z, shift);
  vals[i] = uint32_t(i);
}

__global__ void k_new_group(const uint64_t* __restrict__ k, uint64_t n, uint32_t* __restrict__ flag) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i < n) flag[i] = (i == 0 || k[i] != k[i - 1]) ? 1u : 0u;
  if (i == n) flag[n] = 0u;
}

// state[node][slot] = child; node keys written by the group's first child
__global__ void k_assign_children(const uint32_t* __restrict__ child_sorted, const uint32_t* __restrict__ flag,
                                  const uint32_t* __restrict__ gidx, uint64_t n, const int4* __restrict__ child_org,
                                  int log2, int child_shift, int* __restrict__ state, int4* __restrict__ key) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  uint32_t c = child_sorted[i];
  uint32_t g = gidx[i] + flag[i] - 1;  // exclusive scan + own flag = group index
  int4 o = child_org[c];
  const int m = (1 << log2) - 1;
  int slot = (((o.x >> child_shift) & m) << (2 * log2)) | (((o.y >> child_shift) & m) << log2) | ((o.z >> child_shift) & m);
  state[uint64_t(g) * (1u << (3 * log2)) + slot] = int(c);
  if (flag[i]) {
    const int s = log2 + child_shift;
    key[g] = make_int4((o.x >> s) << s, (o.y >> s) << s, (o.z >> s) << s, 0);
  }
}

__global__ void k_fill_f(float* p, uint64_t n, float v) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i < n) p[i] = v;
}

// Groups `n` children (origins) into parent nodes of level `lv`.
static void build_level(bs_ctx* ctx, const int4* child_org, uint64_t n, Level& lv) {
  cudaStream_t s = ctx->stream;
  lv.free(ctx);
  if (n == 0) return;
  DBuf<uint64_t> k(ctx, n), k2(ctx, n);
  DBuf<uint32_t> v(ctx, n), v2(ctx, n), flag(ctx, n + 1), gidx(ctx, n + 1);
  BS_KERNEL(ctx, "k_child_keys", (k_child_keys<<<nblk(n, 256), 256, 0, s>>>(child_org, n, lv.log2 + lv.child_shift, k.p, v.p)));
  size_t tmp = 0;
  BS_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, k.p, k2.p, v.p, v2.p, int(n), 0, 63, s));
  {
    DBuf<uint8_t> t(ctx, tmp);
    BS_CUDA(cub::DeviceRadixSort::SortPairs(t.p, tmp, k.p, k2.p, v.p, v2.p, int(n), 0, 63, s));
  }
  BS_KERNEL(ctx, "k_new_group", (k_new_group<<<nblk(n + 1, 256), 256, 0, s>>>(k2.p, n, flag.p)));
  scan_excl(ctx, flag.p, gidx.p, n + 1);
  uint32_t ng = 0;
  read_back(ctx, &ng, gidx.p + n, sizeof(uint32_t));
  lv.alloc(ctx, ng);
  BS_CUDA(cudaMemsetAsync(lv.d_state, 0xff, ng * uint64_t(lv.slots) * sizeof(int), s));
  BS_KERNEL(ctx, "k_fill_f", (k_fill_f<<<nblk(ng * uint64_t(lv.slots), 256), 256, 0, s>>>(lv.d_tile, ng * uint64_t(lv.slots), 0.0f)));
  BS_KERNEL(ctx, "k_assign_children", (k_assign_children<<<nblk(n, 256), 256, 0, s>>>(v2.p, flag.p, gidx.p, n, child_org, lv.log2,
                                                                          lv.child_shift, lv.d_state, lv.d_key)));
  lv.sync_keys(ctx);
}

void Level::alloc(bs_ctx* ctx, uint64_t count) {
  n = count;
  d_key = dalloc<int4>(ctx, count);
  d_state = dalloc<int>(ctx, count * uint64_t(slots));
  d_tile = dalloc<float>(ctx, count * uint64_t(slots));
  d_first_neg = dalloc<uint8_t>(ctx, count);
  d_last_neg = dalloc<uint8_t>(ctx, count);
}
void Level::free(bs_ctx* ctx) {
  dfree(ctx, d_key);
  dfree(ctx, d_state);
  dfree(ctx, d_tile);
  dfree(ctx, d_first_neg);
  dfree(ctx, d_last_neg);
  d_key = nullptr;
  d_state = nullptr;
  d_tile = nullptr;
  d_first_neg = d_last_neg = nullptr;
  n = 0;
  h_key.clear();
}
void Level::sync_keys(bs_ctx* ctx) {
  h_key.resize(n);
  if (n) {
    BS_CUDA(cudaMemcpyAsync(h_key.data(), d_key, n * sizeof(int4), cudaMemcpyDeviceToHost, ctx->stream));
    BS_CUDA(cudaStreamSynchronize(ctx->stream));
  }
}

Upper* ensure_upper(bs_ctx* ctx, bs_volume* v) {
  if (v->upper) return v->upper;
  Upper* u = new Upper();
  try {
    build_level(ctx, v->d_origins, v->n_leaves, u->l1);
    build_level(ctx, u->l1.d_key, u->l1.n, u->l2);
  } catch (...) {
    u->l1.free(ctx);
    u->l2.free(ctx);
    delete u;
    throw;
  }
  v->upper = u;
  return u;
}

}  // namespace bs

void bs_volume_free_upper(bs_volume* v) {
  if (!v->upper) return;
  v->upper->l1.free(v->ctx);
  v->upper->l2.free(v->ctx);
  delete v->upper;
  v->upper = nullptr;
}

namespace bs {

// ------------------------------------------------------------ flood fill ---
__device__ __forceinline__ bool mask_on(const uint32_t* m, int i) { return (m[i >> 5] >> (i & 31)) & 1u; }
__device__ __forceinline__ float signed_far(bool neg) { return neg ? -FAR_F : FAR_F; }

// leaf_node/flood_fill.rs:12-50.  One warp per leaf.  Scanning a z-line
// (x, y), the reference carries the sign of the last active voxel it has met:
// starting from the leaf's first active voxel, then the active voxels
// (xx, 0, 0) for xx <= x, then (x, yy, 0) for yy <= y, then along the line,
// and an inactive voxel takes the carried sign (+-far).  Here the leaf's
// values stay in registers (four float4 per lane, coalesced), the active and
// sign bits of its 512 voxels go to shared memory as two 16-word masks, and
// lane l carries the sign along lines l and l + 32 with bit operations on
// those masks only; the fill bits of each line go back through shared memory
// and the leaf is written whole.  Full and empty leaves are left as they are.
constexpr int FF_WARPS = 8;
__global__ void __launch_bounds__(32 * FF_WARPS) k_ff_leaf(float* __restrict__ values, const uint32_t* __restrict__ masks,
                                                           uint64_t n, uint8_t* __restrict__ first_neg,
                                                           uint8_t* __restrict__ last_neg) {
  __shared__ uint32_t sact[FF_WARPS][16], sneg[FF_WARPS][16];
  __shared__ uint8_t sfill[FF_WARPS][64];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint64_t b = blockIdx.x * uint64_t(FF_WARPS) + w;
  if (b >= n) return;
  const uint32_t mw = lane < 16 ? masks[b * 16 + lane] : 0u;
  const bool full = __all_sync(0xffffffffu, lane >= 16 || mw == 0xffffffffu);
  const uint32_t nonzero = __ballot_sync(0xffffffffu, mw != 0u);
  float4* g4 = reinterpret_cast<float4*>(values + b * 512);
  if (full || nonzero == 0u) {
    if (lane == 0) {
      first_neg[b] = signbit(values[b * 512]) ? 1 : 0;
      last_neg[b] = signbit(values[b * 512 + 511]) ? 1 : 0;
    }
    return;
  }
  // float4 k = lane + 32 j holds voxels 4k .. 4k + 3: word k >> 3, bits 4 (k & 7) + i
  float4 r[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) r[j] = g4[lane + 32 * j];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    uint32_t nib = (signbit(r[j].x) ? 1u : 0u) | (signbit(r[j].y) ? 2u : 0u) | (signbit(r[j].z) ? 4u : 0u) |
                   (signbit(r[j].w) ? 8u : 0u);
    nib <<= 4 * (lane & 7);
    nib |= __shfl_xor_sync(0xffffffffu, nib, 1);
    nib |= __shfl_xor_sync(0xffffffffu, nib, 2);
    nib |= __shfl_xor_sync(0xffffffffu, nib, 4);
    if ((lane & 7) == 0) sneg[w][(lane >> 3) + 4 * j] = nib;
  }
  if (lane < 16) sact[w][lane] = mw;
  __syncwarp();
  const uint32_t* A = sact[w];
  const uint32_t* Ng = sneg[w];
  const int fw = __ffs(nonzero) - 1;
  const int first = fw * 32 + __ffs(__shfl_sync(0xffffffffu, mw, fw)) - 1;
  const uint32_t s0 = (Ng[first >> 5] >> (first & 31)) & 1u;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int line = lane + 32 * h, x = line >> 3, y = line & 7;
    uint32_t c = s0;
    for (int xx = 0; xx <= x; ++xx)  // voxel (xx, 0, 0): word 2 xx, bit 0
      if (A[2 * xx] & 1u) c = Ng[2 * xx] & 1u;
    for (int yy = 0; yy <= y; ++yy) {  // voxel (x, yy, 0): word 2 x + yy / 4, bit 8 (yy % 4)
      const int wd = 2 * x + (yy >> 2), bt = 8 * (yy & 3);
      if ((A[wd] >> bt) & 1u) c = (Ng[wd] >> bt) & 1u;
    }
    const int sh = 8 * (line & 3);
    const uint32_t a8 = (A[line >> 2] >> sh) & 0xffu, n8 = (Ng[line >> 2] >> sh) & 0xffu;
    uint32_t fill = 0;
#pragma unroll
    for (int z = 0; z < 8; ++z) {
      if ((a8 >> z) & 1u)
        c = (n8 >> z) & 1u;
      else
        fill |= c << z;
    }
    sfill[w][line] = uint8_t(fill);
  }
  __syncwarp();
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int k = lane + 32 * j;
    const uint32_t act4 = (A[k >> 3] >> (4 * (k & 7))) & 0xfu;
    const uint32_t fill4 = (uint32_t(sfill[w][k >> 1]) >> (4 * (k & 1))) & 0xfu;  // voxels 4k.. of line k / 2
    float4 t = r[j];
    if (!(act4 & 1u)) t.x = signed_far(fill4 & 1u);
    if (!(act4 & 2u)) t.y = signed_far(fill4 & 2u);
    if (!(act4 & 4u)) t.z = signed_far(fill4 & 4u);
    if (!(act4 & 8u)) t.w = signed_far(fill4 & 8u);
    g4[k] = t;
    if (k == 0) first_neg[b] = signbit(t.x) ? 1 : 0;
    if (k == 127) last_neg[b] = signbit(t.w) ? 1 : 0;
  }
}

// internal_node/flood_fill.rs:17-117 for one node per CTA, one thread per z-line.
template <int LOG2>
__global__ void k_ff_internal(int* __restrict__ state, float* __restrict__ tile, uint64_t n,
                              const uint8_t* __restrict__ cfirst, const uint8_t* __restrict__ clast,
                              uint8_t* __restrict__ first_neg, uint8_t* __restrict__ last_neg) {
  constexpr int DIM = 1 << LOG2, S = DIM * DIM * DIM;
  const uint64_t node = blockIdx.x;
  if (node >= n) return;
  int* st = state + node * S;
  float* tl = tile + node * S;
  __shared__ int s_first_tile, s_first_branch, s_any_none;
  if (threadIdx.x == 0) {
    s_first_tile = S;
    s_first_branch = S;
    s_any_none = 0;
  }
  __syncthreads();
  for (int o = threadIdx.x; o < S; o += blockDim.x) {
    const int q = st[o];
    if (q == -2) atomicMin(&s_first_tile, o);
    else if (q >= 0) atomicMin(&s_first_branch, o);
    if (q != -2) s_any_none = 1;  // value_mask not full
  }
  __syncthreads();
  const int fv = s_first_tile, fb = s_first_branch;
  if (s_any_none && (fv < S || fb < S)) {
    bool i0;
    if (fv < S && (fb >= S || fv <= fb)) i0 = signbit(tl[fv]);
    else i0 = cfirst[st[fb]] != 0;
    // carry sign of a present slot: tile -> its sign, branch -> child's last value sign
    auto carry = [&](int o, bool& c) {
      const int q = st[o];
      if (q >= 0) c = clast[q] != 0;
      else if (q == -2) c = signbit(tl[o]);
    };
    for (int line = threadIdx.x; line < DIM * DIM; line += blockDim.x) {
      const int x = line / DIM, y = line % DIM;
      bool c = i0;
      for (int xx = 0; xx <= x; ++xx) carry(xx * DIM * DIM, c);
      for (int yy = 0; yy <= y; ++yy) carry(x * DIM * DIM + yy * DIM, c);
      for (int z = 0; z < DIM; ++z) {
        const int o = x * DIM * DIM + y * DIM + z;
        if (st[o] == -1)
          tl[o] = signed_far(c);
        else
          carry(o, c);
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int q0 = st[0], ql = st[S - 1];
    first_neg[node] = q0 >= 0 ? cfirst[q0] : (signbit(tl[0]) ? 1 : 0);
    // the reference's last_value_sign() reads the last child's FIRST value
    last_neg[node] = ql >= 0 ? cfirst[ql] : (signbit(tl[S - 1]) ? 1 : 0);
  }
}

__global__ void k_append_l2_fill(int* __restrict__ state, float* __restrict__ tile, uint64_t from, uint64_t to,
                                 uint8_t* first_neg, uint8_t* last_neg) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  const uint64_t n = (to - from) * L2_SLOTS;
  if (i < n) {
    state[from * L2_SLOTS + i] = -1;
    tile[from * L2_SLOTS + i] = -FAR_F;  // fill_with_sign(Negative) on an empty node
  }
  if (i < to - from) {
    first_neg[from + i] = 1;
    last_neg[from + i] = 1;
  }
}

// Grows the L2 level to hold `extra` more nodes (existing contents kept).
static void grow_l2(bs_ctx* ctx, Level& l2, const std::vector<int4>& extra_keys) {
  const uint64_t n0 = l2.n, n1 = n0 + extra_keys.size();
  Level g;
  g.log2 = l2.log2;
  g.child_shift = l2.child_shift;
  g.slots = l2.slots;
  g.alloc(ctx, n1);
  cudaStream_t s = ctx->stream;
  if (n0) {
    BS_CUDA(cudaMemcpyAsync(g.d_key, l2.d_key, n0 * sizeof(int4), cudaMemcpyDeviceToDevice, s));
    BS_CUDA(cudaMemcpyAsync(g.d_state, l2.d_state, n0 * L2_SLOTS * sizeof(int), cudaMemcpyDeviceToDevice, s));
    BS_CUDA(cudaMemcpyAsync(g.d_tile, l2.d_tile, n0 * L2_SLOTS * sizeof(float), cudaMemcpyDeviceToDevice, s));
    BS_CUDA(cudaMemcpyAsync(g.d_first_neg, l2.d_first_neg, n0, cudaMemcpyDeviceToDevice, s));
    BS_CUDA(cudaMemcpyAsync(g.d_last_neg, l2.d_last_neg, n0, cudaMemcpyDeviceToDevice, s));
  }
  BS_CUDA(cudaMemcpyAsync(g.d_key + n0, extra_keys.data(), extra_keys.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
  BS_KERNEL(ctx, "k_append_l2_fill", (k_append_l2_fill<<<nblk((n1 - n0) * L2_SLOTS, 256), 256, 0, s>>>(g.d_state, g.d_tile, n0, n1,
                                                                                            g.d_first_neg, g.d_last_neg)));
  g.h_key = l2.h_key;
  g.h_key.insert(g.h_key.end(), extra_keys.begin(), extra_keys.end());
  BS_CUDA(cudaStreamSynchronize(s));  // extra_keys is host memory owned by the caller
  l2.free(ctx);
  l2 = std::move(g);
  g.d_key = nullptr;
  g.d_state = nullptr;
  g.d_tile = nullptr;
  g.d_first_neg = g.d_last_neg = nullptr;
}

static bool key_less(const int4& a, const int4& b) {
  if (a.x != b.x) return a.x < b.x;
  if (a.y != b.y) return a.y < b.y;
  return a.z < b.z;
}

// Volume flood fill (root_node/flood_fill.rs:8-42 and below): leaves, L1,
// L2 on the GPU, then the root's z-gap filling on the host.
void flood_fill(bs_ctx* ctx, bs_volume* v) {
  Upper* u = ensure_upper(ctx, v);
  cudaStream_t s = ctx->stream;
  DBuf<uint8_t> lf(ctx, v->n_leaves), ll(ctx, v->n_leaves);
  if (v->n_leaves)
    BS_KERNEL(ctx, "k_ff_leaf", (k_ff_leaf<<<nblk(v->n_leaves, FF_WARPS), 32 * FF_WARPS, 0, s>>>(v->d_values, v->d_masks, v->n_leaves, lf.p, ll.p)));
  if (u->l1.n)
    BS_KERNEL(ctx, "k_ff_internal_l1", (k_ff_internal<L1_LOG2><<<unsigned(u->l1.n), 256, 0, s>>>(u->l1.d_state, u->l1.d_tile, u->l1.n, lf.p, ll.p,
                                                                                    u->l1.d_first_neg, u->l1.d_last_neg)));
  if (u->l2.n)
    BS_KERNEL(ctx, "k_ff_internal_l2", (k_ff_internal<L2_LOG2><<<unsigned(u->l2.n), 1024, 0, s>>>(u->l2.d_state, u->l2.d_tile, u->l2.n,
                                                                                     u->l1.d_first_neg, u->l1.d_last_neg,
                                                                                     u->l2.d_first_neg, u->l2.d_last_neg)));
  // root: z-gaps between consecutive inside children on one (x, y) column
  const uint64_t n2 = u->l2.n;
  if (n2 < 2) return;
  std::vector<uint8_t> fneg(n2), lneg(n2);
  read_back(ctx, fneg.data(), u->l2.d_first_neg, n2);
  read_back(ctx, lneg.data(), u->l2.d_last_neg, n2);
  std::vector<int> order(n2);
  for (uint64_t i = 0; i < n2; ++i) order[i] = int(i);
  std::sort(order.begin(), order.end(), [&](int a, int b) { return key_less(u->l2.h_key[a], u->l2.h_key[b]); });
  std::vector<int4> extra;
  const int R = 1 << L2_SHIFT;
  for (uint64_t k = 0; k + 1 < n2; ++k) {
    const int4 a = u->l2.h_key[order[k]], b = u->l2.h_key[order[k + 1]];
    if (a.x != b.x || a.y != b.y || b.z == a.z + R) continue;
    if (!lneg[order[k]] || !fneg[order[k + 1]]) continue;
    for (int z = a.z + R; z < b.z; z += R) extra.push_back(make_int4(a.x, a.y, z, 0));
  }
  if (!extra.empty()) grow_l2(ctx, u->l2, extra);
}

// ------------------------------------------------------------------ CSG ----
enum : int { A_KEEP = 0, A_TAKE_B = 1, A_MERGE = 2, A_INSIDE = 3, A_NONE = 4, A_NEG_TILE = 5 };
enum : int { OP_UNION = 0, OP_SUBTRACT = 1, OP_INTERSECT = 2 };

// Per-slot decision of internal_node/csg.rs:68-162.  `flip` is set when the
// taken child must have its signs flipped (subtract).
__device__ __forceinline__ int csg_decide(int op, int sa, float ta, int sb, float tb, bool& flip) {
  flip = false;
  const bool a_br = sa >= 0, b_br = sb >= 0;
  const bool a_in = !a_br && signbit(ta), a_out = !a_br && !signbit(ta);
  const bool b_in = !b_br && signbit(tb), b_out = !b_br && !signbit(tb);
  if (op == OP_UNION) {
    if (a_in) return A_KEEP;
    if (b_in) return A_INSIDE;
    if (a_out) return b_br ? A_TAKE_B : A_KEEP;
    if (a_br && b_br) return A_MERGE;
    return A_KEEP;
  }
  if (op == OP_SUBTRACT) {
    if (a_out || b_out) return A_KEEP;
    if (b_in) return A_NONE;
    if (a_in) {
      if (b_br) {
        flip = true;
        return A_TAKE_B;
      }
      return sa == -2 ? A_NEG_TILE : A_KEEP;
    }
    if (a_br && b_br) return A_MERGE;
    return A_KEEP;
  }
  // intersect
  if (a_out || b_in) return A_KEEP;
  if (b_out) return A_NONE;
  if (a_in) return b_br ? A_TAKE_B : A_KEEP;
  if (a_br && b_br) return A_MERGE;
  return A_KEEP;
}

// A request for an output child: type 0 copy from A, 1 copy from B, 2 merge A+B; -1 none.
struct Req {
  int type, a, b, flip;
};

// Resolves one output node's slots.  plan: (type, a, b, flip) of this output node.
template <int LOG2>
__global__ void k_csg_slots(int op, const Req* __restrict__ plan, uint64_t n_out, const int* __restrict__ sa_,
                            const float* __restrict__ ta_, const int* __restrict__ sb_, const float* __restrict__ tb_,
                            int* __restrict__ out_state, float* __restrict__ out_tile, Req* __restrict__ child_req,
                            uint32_t* __restrict__ child_flag) {
  constexpr int S = 1 << (3 * LOG2);
  const uint64_t e = blockIdx.y;
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_out || o >= S) return;
  const Req p = plan[e];
  const uint64_t ia = uint64_t(p.a) * S + o, ib = uint64_t(p.b) * S + o, io = e * S + o;
  int st = -1;
  float tv = 0.f;
  Req cr{-1, 0, 0, 0};
  if (p.type == 0) {  // node copied from A
    st = sa_[ia];
    tv = ta_[ia];
    if (st >= 0) cr = Req{0, st, 0, 0};
  } else if (p.type == 1) {  // node taken from B (signs flipped when p.flip)
    st = sb_[ib];
    tv = tb_[ib];
    if (st >= 0) cr = Req{1, 0, st, p.flip};
    else if (st == -2 && p.flip) tv = -tv;
  } else {  // merged pair
    const int sa = sa_[ia], sb = sb_[ib];
    const float ta = ta_[ia], tb = tb_[ib];
    bool flip;
    const int act = csg_decide(op, sa, ta, sb, tb, flip);
    st = sa;
    tv = ta;
    switch (act) {
      case A_KEEP:
        if (sa >= 0) cr = Req{0, sa, 0, 0};
        break;
      case A_TAKE_B:
        cr = Req{1, 0, sb, flip ? 1 : 0};
        break;
      case A_MERGE:
        cr = Req{2, sa, sb, 0};
        break;
      case A_INSIDE:
        st = -2;
        tv = -FAR_F;
        break;
      case A_NONE:
        st = -1;
        break;
      case A_NEG_TILE:
        st = -2;
        tv = -ta;
        break;
    }
  }
  if (cr.type >= 0) st = 0;  // placeholder; rewritten with the output child index
  out_state[io] = st;
  out_tile[io] = tv;
  child_req[io] = cr;
  child_flag[io] = cr.type >= 0 ? 1u : 0u;
}

__global__ void k_compact_reqs(const Req* __restrict__ req, const uint32_t* __restrict__ flag,
                               const uint32_t* __restrict__ pos, uint64_t n, int* __restrict__ out_state,
                               Req* __restrict__ out_req) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n || !flag[i]) return;
  out_state[i] = int(pos[i]);
  out_req[pos[i]] = req[i];
}

// Node keys of the output level: from A for copies and merges, B for takes.
__global__ void k_req_keys(const Req* __restrict__ req, uint64_t n, const int4* __restrict__ ka,
                           const int4* __restrict__ kb, int4* __restrict__ out) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const Req r = req[i];
  out[i] = r.type == 1 ? kb[r.b] : ka[r.a];
}

// partial_min / partial_max of voxel/utils.rs:38-62 (ties and NaN take b)
__device__ __forceinline__ float csg_value(int op, float a, float b) {
  if (op == OP_UNION) return (a < b) ? a : b;
  if (op == OP_SUBTRACT) return (a > -b) ? a : -b;
  return (a > b) ? a : b;
}

// Output leaves: copy, copy with flipped signs, or combine (leaf_node/csg.rs:17-45).
__global__ void __launch_bounds__(128) k_csg_leaves(int op, const Req* __restrict__ req, uint64_t n,
                                                    const int4* __restrict__ oa, const float* __restrict__ va,
                                                    const uint32_t* __restrict__ ma, const int4* __restrict__ ob,
                                                    const float* __restrict__ vb, const uint32_t* __restrict__ mb,
                                                    int4* __restrict__ oo, float* __restrict__ vo,
                                                    uint32_t* __restrict__ mo) {
  const uint64_t l = blockIdx.x;
  if (l >= n) return;
  const Req r = req[l];
  const int t = threadIdx.x;
  if (t == 0) oo[l] = r.type == 1 ? ob[r.b] : oa[r.a];
  if (t < 16) {
    uint32_t m = 0;
    if (r.type == 0) m = ma[uint64_t(r.a) * 16 + t];
    else if (r.type == 1) m = mb[uint64_t(r.b) * 16 + t];
    else m = ma[uint64_t(r.a) * 16 + t] | mb[uint64_t(r.b) * 16 + t];
    mo[l * 16 + t] = m;
  }
  // one float4 of the leaf per thread
  float4 x;
  if (r.type == 0) {
    x = reinterpret_cast<const float4*>(va + uint64_t(r.a) * 512)[t];
  } else if (r.type == 1) {
    x = reinterpret_cast<const float4*>(vb + uint64_t(r.b) * 512)[t];
    if (r.flip) x = make_float4(-x.x, -x.y, -x.z, -x.w);
  } else {
    const float4 a = reinterpret_cast<const float4*>(va + uint64_t(r.a) * 512)[t];
    const float4 b = reinterpret_cast<const float4*>(vb + uint64_t(r.b) * 512)[t];
    x = make_float4(csg_value(op, a.x, b.x), csg_value(op, a.y, b.y), csg_value(op, a.z, b.z), csg_value(op, a.w, b.w));
  }
  reinterpret_cast<float4*>(vo + l * 512)[t] = x;
}

__global__ void k_count_active(const uint32_t* __restrict__ m, uint64_t n, unsigned long long* out) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  unsigned long long c = 0;
  if (i < n * 16) c = __popc(m[i]);
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// Active tiles of one level -> (origin, size) / value lists.
template <int LOG2>
__global__ void k_tile_flags(const int* __restrict__ state, uint64_t n, uint32_t* __restrict__ flag) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i < n) flag[i] = state[i] == -2 ? 1u : 0u;
  if (i == n) flag[n] = 0u;
}
template <int LOG2>
__global__ void k_tile_emit(const int* __restrict__ state, const float* __restrict__ tile, const int4* __restrict__ key,
                            uint64_t n, int child_shift, const uint32_t* __restrict__ pos, uint64_t base,
                            int4* __restrict__ out_t, float* __restrict__ out_v) {
  constexpr int S = 1 << (3 * LOG2), M = (1 << LOG2) - 1;
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n || state[i] != -2) return;
  const uint64_t node = i / S;
  const int o = int(i % S);
  const int4 k = key[node];
  const int x = (o >> (2 * LOG2)) & M, y = (o >> LOG2) & M, z = o & M;
  out_t[base + pos[i]] = make_int4(k.x + (x << child_shift), k.y + (y << child_shift), k.z + (z << child_shift),
                                   1 << child_shift);
  out_v[base + pos[i]] = tile[i];
}

static uint64_t level_tiles(bs_ctx* ctx, const Level& lv, std::vector<DBuf<uint32_t>>& keep, uint32_t** pos_out) {
  cudaStream_t s = ctx->stream;
  const uint64_t n = lv.n * uint64_t(lv.slots);
  DBuf<uint32_t> flag(ctx, n + 1), pos(ctx, n + 1);
  if (lv.log2 == L1_LOG2)
    BS_KERNEL(ctx, "k_tile_flags", (k_tile_flags<L1_LOG2><<<nblk(n + 1, 256), 256, 0, s>>>(lv.d_state, n, flag.p)));
  else
    BS_KERNEL(ctx, "k_tile_flags", (k_tile_flags<L2_LOG2><<<nblk(n + 1, 256), 256, 0, s>>>(lv.d_state, n, flag.p)));
  scan_excl(ctx, flag.p, pos.p, n + 1);
  uint32_t c = 0;
  read_back(ctx, &c, pos.p + n, sizeof(uint32_t));
  *pos_out = pos.p;
  keep.push_back(std::move(pos));
  return c;
}

// Rebuilds the export tile list (active tiles of both levels, L2 first).
void refresh_tiles(bs_ctx* ctx, bs_volume* v) {
  dfree(ctx, v->d_tiles);
  dfree(ctx, v->d_tile_values);
  v->d_tiles = nullptr;
  v->d_tile_values = nullptr;
  v->n_tiles = 0;
  Upper* u = v->upper;
  if (!u) return;
  std::vector<DBuf<uint32_t>> keep;
  uint32_t *p2 = nullptr, *p1 = nullptr;
  const uint64_t c2 = u->l2.n ? level_tiles(ctx, u->l2, keep, &p2) : 0;
  const uint64_t c1 = u->l1.n ? level_tiles(ctx, u->l1, keep, &p1) : 0;
  v->n_tiles = c1 + c2;
  if (!v->n_tiles) return;
  v->d_tiles = dalloc<int4>(ctx, v->n_tiles);
  v->d_tile_values = dalloc<float>(ctx, v->n_tiles);
  cudaStream_t s = ctx->stream;
  if (c2) {
    const uint64_t n = u->l2.n * uint64_t(L2_SLOTS);
    BS_KERNEL(ctx, "k_tile_emit", (k_tile_emit<L2_LOG2><<<nblk(n, 256), 256, 0, s>>>(u->l2.d_state, u->l2.d_tile, u->l2.d_key, n,
                                                                        L2_CHILD_SHIFT, p2, 0, v->d_tiles, v->d_tile_values)));
  }
  if (c1) {
    const uint64_t n = u->l1.n * uint64_t(L1_SLOTS);
    BS_KERNEL(ctx, "k_tile_emit", (k_tile_emit<L1_LOG2><<<nblk(n, 256), 256, 0, s>>>(u->l1.d_state, u->l1.d_tile, u->l1.d_key, n,
                                                                        L1_CHILD_SHIFT, p1, c2, v->d_tiles, v->d_tile_values)));
  }
}

// Output slots of one level and the requests for the level below.
template <int LOG2>
static uint64_t csg_level(bs_ctx* ctx, int op, const DBuf<Req>& plan, uint64_t n_out, const Level& A, const Level& B,
                          Level& out, DBuf<Req>& child_plan) {
  constexpr uint64_t S = 1ull << (3 * LOG2);
  cudaStream_t s = ctx->stream;
  out.alloc(ctx, n_out);
  if (n_out == 0) {
    child_plan = DBuf<Req>(ctx, 1);
    return 0;
  }
  const uint64_t n = n_out * S;
  DBuf<Req> req(ctx, n);
  DBuf<uint32_t> flag(ctx, n + 1), pos(ctx, n + 1);
  BS_CUDA(cudaMemsetAsync(flag.p + n, 0, sizeof(uint32_t), s));
  dim3 g(unsigned((S + 255) / 256), unsigned(n_out));
  BS_KERNEL(ctx, "k_csg_slots", (k_csg_slots<LOG2><<<g, 256, 0, s>>>(op, plan.p, n_out, A.d_state, A.d_tile, B.d_state, B.d_tile,
                                                         out.d_state, out.d_tile, req.p, flag.p)));
  scan_excl(ctx, flag.p, pos.p, n + 1);
  uint32_t nc = 0;
  read_back(ctx, &nc, pos.p + n, sizeof(uint32_t));
  child_plan = DBuf<Req>(ctx, std::max<uint64_t>(nc, 1));
  BS_KERNEL(ctx, "k_compact_reqs", (k_compact_reqs<<<nblk(n, 256), 256, 0, s>>>(req.p, flag.p, pos.p, n, out.d_state, child_plan.p)));
  BS_KERNEL(ctx, "k_req_keys", (k_req_keys<<<nblk(n_out, 256), 256, 0, s>>>(plan.p, n_out, A.d_key, B.d_key, out.d_key)));
  return nc;
}

bs_volume* volume_csg_impl(bs_ctx* ctx, bs_volume* a, bs_volume* b, int op) {
  // the reference combines the grids index by index whatever their voxel
  // sizes (volume/mod.rs:74-93) and keeps the first operand's; so does this
  flood_fill(ctx, a);
  flood_fill(ctx, b);
  Upper *ua = a->upper, *ub = b->upper;
  // ---- root level (root_node/csg.rs:9-58) on the host ----
  std::vector<Req> plan2;
  {
    std::map<std::tuple<int, int, int>, std::pair<int, int>> keys;  // sorted like RootKey
    for (uint64_t i = 0; i < ua->l2.n; ++i) {
      const int4 k = ua->l2.h_key[i];
      keys[{k.x, k.y, k.z}].first = int(i) + 1;
    }
    for (uint64_t i = 0; i < ub->l2.n; ++i) {
      const int4 k = ub->l2.h_key[i];
      keys[{k.x, k.y, k.z}].second = int(i) + 1;
    }
    for (auto& kv : keys) {
      const int ia = kv.second.first - 1, ib = kv.second.second - 1;
      if (op == OP_UNION) {
        if (ia >= 0 && ib >= 0) plan2.push_back(Req{2, ia, ib, 0});
        else if (ia >= 0) plan2.push_back(Req{0, ia, 0, 0});
        else plan2.push_back(Req{1, 0, ib, 0});
      } else if (op == OP_SUBTRACT) {
        if (ia >= 0 && ib >= 0) plan2.push_back(Req{2, ia, ib, 0});
        else if (ia >= 0) plan2.push_back(Req{0, ia, 0, 0});
      } else {
        if (ia >= 0 && ib >= 0) plan2.push_back(Req{2, ia, ib, 0});
      }
    }
  }
  bs_volume* out = new bs_volume(ctx);
  out->h = a->h;
  try {
    Upper* uo = new Upper();
    out->upper = uo;
    DBuf<Req> d_plan2(ctx, std::max<size_t>(plan2.size(), 1));
    if (!plan2.empty())
      BS_CUDA(cudaMemcpyAsync(d_plan2.p, plan2.data(), plan2.size() * sizeof(Req), cudaMemcpyHostToDevice, ctx->stream));
    DBuf<Req> plan1, plan0;
    const uint64_t n1 = csg_level<L2_LOG2>(ctx, op, d_plan2, plan2.size(), ua->l2, ub->l2, uo->l2, plan1);
    const uint64_t n0 = csg_level<L1_LOG2>(ctx, op, plan1, n1, ua->l1, ub->l1, uo->l1, plan0);
    uo->l2.sync_keys(ctx);
    uo->l1.sync_keys(ctx);
    // union never empties a merged node: a merged slot's A side was a branch,
    // which stays a branch or becomes an active inside tile
    out->n_leaves = n0;
    out->d_origins = dalloc<int4>(ctx, n0);
    out->d_values = dalloc<float>(ctx, n0 * 512);
    out->d_masks = dalloc<uint32_t>(ctx, n0 * 16);
    if (n0)
      BS_KERNEL(ctx, "k_csg_leaves", (k_csg_leaves<<<unsigned(n0), 128, 0, ctx->stream>>>(op, plan0.p, n0, a->d_origins, a->d_values,
                                                                            a->d_masks, b->d_origins, b->d_values,
                                                                            b->d_masks, out->d_origins, out->d_values,
                                                                            out->d_masks)));
    DBuf<unsigned long long> cnt(ctx, 1);
    BS_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), ctx->stream));
    if (n0)
      BS_KERNEL(ctx, "k_count_active", (k_count_active<<<nblk(n0 * 16, 256), 256, 0, ctx->stream>>>(out->d_masks, n0, cnt.p)));
    unsigned long long na = 0;
    read_back(ctx, &na, cnt.p, sizeof(na));
    out->n_active = na;
    refresh_tiles(ctx, out);
  } catch (...) {
    delete out;
    throw;
  }
  delete a;
  delete b;
  return out;
}

// ---------------------------------------------------------------- clone ----
bs_volume* volume_clone_impl(bs_ctx* ctx, const bs_volume* v) {
  bs_volume* c = new bs_volume(ctx);
  c->h = v->h;
  c->n_leaves = v->n_leaves;
  c->n_active = v->n_active;
  cudaStream_t s = ctx->stream;
  try {
    c->d_origins = dalloc<int4>(ctx, v->n_leaves);
    c->d_values = dalloc<float>(ctx, v->n_leaves * 512);
    c->d_masks = dalloc<uint32_t>(ctx, v->n_leaves * 16);
    if (v->n_leaves) {
      BS_CUDA(cudaMemcpyAsync(c->d_origins, v->d_origins, v->n_leaves * sizeof(int4), cudaMemcpyDeviceToDevice, s));
      BS_CUDA(cudaMemcpyAsync(c->d_values, v->d_values, v->n_leaves * 512 * sizeof(float), cudaMemcpyDeviceToDevice, s));
      BS_CUDA(cudaMemcpyAsync(c->d_masks, v->d_masks, v->n_leaves * 16 * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
    }
    if (v->upper) {
      Upper* u = new Upper();
      c->upper = u;
      for (int lvl = 0; lvl < 2; ++lvl) {
        const Level& src = lvl ? v->upper->l2 : v->upper->l1;
        Level& dst = lvl ? u->l2 : u->l1;
        dst.alloc(ctx, src.n);
        if (src.n) {
          BS_CUDA(cudaMemcpyAsync(dst.d_key, src.d_key, src.n * sizeof(int4), cudaMemcpyDeviceToDevice, s));
          BS_CUDA(cudaMemcpyAsync(dst.d_state, src.d_state, src.n * uint64_t(src.slots) * sizeof(int), cudaMemcpyDeviceToDevice, s));
          BS_CUDA(cudaMemcpyAsync(dst.d_tile, src.d_tile, src.n * uint64_t(src.slots) * sizeof(float), cudaMemcpyDeviceToDevice, s));
          BS_CUDA(cudaMemcpyAsync(dst.d_first_neg, src.d_first_neg, src.n, cudaMemcpyDeviceToDevice, s));
          BS_CUDA(cudaMemcpyAsync(dst.d_last_neg, src.d_last_neg, src.n, cudaMemcpyDeviceToDevice, s));
        }
        dst.h_key = src.h_key;
      }
    }
    c->n_tiles = v->n_tiles;
    if (v->n_tiles) {
      c->d_tiles = dalloc<int4>(ctx, v->n_tiles);
      c->d_tile_values = dalloc<float>(ctx, v->n_tiles);
      BS_CUDA(cudaMemcpyAsync(c->d_tiles, v->d_tiles, v->n_tiles * sizeof(int4), cudaMemcpyDeviceToDevice, s));
      BS_CUDA(cudaMemcpyAsync(c->d_tile_values, v->d_tile_values, v->n_tiles * sizeof(float), cudaMemcpyDeviceToDevice, s));
    }
  } catch (...) {
    delete c;
    throw;
  }
  return c;
}

}  // namespace bs

namespace bs {

}  // namespace bs
