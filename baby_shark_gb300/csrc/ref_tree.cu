// The reference's winding-number tree, built and traversed on the GPU.
//
// Build (AABBTree::top_down::<Area>, aabb_tree.rs:118-199, 201-250, 422-514):
// every node of more than 3 triangles and depth below 40 is split; its axes
// are tried largest extent first (stable order on ties); an axis sorts the
// node's triangles by bounding-box centre (a stable sort), puts them into 12
// buckets over the centres' bounds and takes the cheapest of the 11 bucket
// boundaries by the surface-area cost 1/8 + (n0 A0 + n1 A1) / A; the split
// stands when that cost is below the triangle count, else the next axis is
// tried, and a node no axis splits becomes a leaf.
//
// The bucket index grows with the centre coordinate, so the left child is
// exactly the set of triangles whose bucket is at most the chosen one: which
// triangles go where never depends on the order, and the passes here place
// them with atomics.  The order matters only inside a leaf (its sums run in
// it), and there it is known in closed form: a chain of stable sorts orders
// by the most recent sort key, then the one before, ... and finally by the
// input (mesh) order, and a key used twice adds nothing after its latest use.
// So each node carries the distinct axes of its sorts, most recent first
// (`prio`), and a leaf sorts its few triangles by those centre coordinates and
// then by triangle index.  Node identity: an internal node is numbered by the
// position at which it splits its range (minus one), a leaf by the position
// of its first triangle — both unique, and independent of build order.
//
// Large nodes (above SMALL triangles) are split level by level over the whole
// GPU (bucket pass with per-block shared-memory bins, a decision per node, a
// placement pass); each node of at most SMALL triangles is then finished by
// one CTA in shared memory, a warp per node and level.  Coefficients
// (compute_node_data, aabb_tree.rs:723-801) go bottom-up from the leaves, the
// second child to arrive combining a parent, in the reference's float32
// operations and order.
//
// Traversal (fast_wn, aabb_tree.rs:662-691): one query point per thread; a
// node is summed through its far field when |q - p| > beta r, a leaf
// otherwise through its triangles' exact solid angles (summed, then divided
// by 4 pi), and a branch as wn(left) + wn(right): the thread keeps the
// pending left sums on a stack of at most 40 levels so the additions happen
// in the recursion's order.
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <vector>

#include "ref_tree.cuh"

namespace bs {
namespace {

constexpr int NB = 12;                 // buckets per axis (aabb_tree.rs:437)
constexpr uint32_t MIN_LEAF = 3;       // with_min_objects_per_leaf(3) (aabb_tree.rs:640)
constexpr int MAX_DEPTH = 40;          // AABBTree's default max depth (aabb_tree.rs:69)
constexpr uint32_t SMALL = 512;        // nodes up to this many triangles are finished by one CTA
constexpr uint32_t CHUNK = 2048;       // positions per block in the passes over large nodes
constexpr int BKW = 3 * NB * 7;        // bins of a node: axis x bucket x (count, lo xyz, hi xyz)
constexpr int STACK = MAX_DEPTH;       // pending left sums of a traversal
constexpr int ST_THREADS = 256;        // CTA of the small-node kernel
constexpr int ST_WARPS = ST_THREADS / 32;
constexpr int ST_LIST = SMALL / 4 + 1; // nodes per level inside one CTA (each holds > 3 triangles)
constexpr float FOUR_PI_F = 12.566370614359172f;  // 4.0f * PI in float32 (aabb_tree.rs:600, 812)
constexpr unsigned FULL = 0xffffffffu;

// Order-preserving maps between float and uint32 (for atomic min / max).
__device__ __forceinline__ uint32_t ford(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fund(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

struct RtSeg {
  uint32_t first, count;  // positions [first, first + count)
  int parent;             // internal node id of the parent, or -1 - mesh for a root
  int side;               // 0: left child, 1: right child
  int depth;              // root = 1 (aabb_tree.rs:129)
  uint32_t prio;          // sort axes applied so far, most recent first
  uint32_t bnd[12];       // ordered: box lo xyz, box hi xyz, centre lo xyz, centre hi xyz
};

struct RtDec {
  int axis;  // -1: no axis splits (a leaf)
  int best;
  uint32_t nl;
  uint32_t prio;
};

struct RtChunk {
  uint32_t seg, begin, end;
};

struct RtBuild {  // device arrays the kernels share
  const float4* obA;  // box lo xyz, centre x
  const float4* obB;  // box hi xyz, centre y
  const float* obC;   // centre z
  uint32_t* perm;     // position -> triangle
  int2* topo;
  int* par_i;
  int* par_l;
  int* roots;
  uint32_t* leaf_cnt;
  uint32_t* leaf_prio;
  RtSeg* big_next;
  RtSeg* small;
  uint32_t* counters;  // [0] next large nodes, [1] small nodes, [2] error
  uint32_t cap_big, cap_small;
};

// Axis list after a stable sort along axis a: a first, then the earlier axes
// without a.  bits 0-1: length; bits 2k+2..2k+3: axis k.
__host__ __device__ __forceinline__ uint32_t prio_push(uint32_t p, int a) {
  const int n = int(p & 3u);
  uint32_t out = uint32_t(a) << 2;
  int m = 1;
  for (int i = 0; i < n; ++i) {
    const int b = int((p >> (2 + 2 * i)) & 3u);
    if (b != a) {
      out |= uint32_t(b) << (2 + 2 * m);
      ++m;
    }
  }
  return out | uint32_t(m);
}

// Bucket of a centre coordinate (aabb_tree.rs:447-452 with Box3::offset,
// box3.rs:185-201; `as usize` saturates, NaN -> 0).
__device__ __forceinline__ int bucket_of(float c, float cmn, float cmx) {
  float o = fsub(c, cmn);
  if (cmx > cmn) o = fdiv(o, fsub(cmx, cmn));
  const float t = fmul(12.0f, o);
  if (!(t > 0.0f)) return 0;
  if (t >= 11.0f) return NB - 1;
  return int(t);
}

// Box3::area (box3.rs:125-128).
__device__ __forceinline__ float box_area(float lx, float ly, float lz, float hx, float hy, float hz) {
  const float dx = fsub(hx, lx), dy = fsub(hy, ly), dz = fsub(hz, lz);
  return fmul(2.0f, fadd(fadd(fmul(dx, dy), fmul(dx, dz)), fmul(dy, dz)));
}

// Cost of the boundary after bucket i of one axis's bins (aabb_tree.rs:459-488).
__device__ __forceinline__ float split_cost(const uint32_t* bk, int i, float parea) {
  uint32_t c0 = 0, c1 = 0;
  uint32_t l0[3] = {FULL, FULL, FULL}, h0[3] = {0, 0, 0}, l1[3] = {FULL, FULL, FULL}, h1[3] = {0, 0, 0};
  for (int j = 0; j < NB; ++j) {
    const uint32_t* b = bk + 7 * j;
    if (j <= i) {
      c0 += b[0];
      for (int k = 0; k < 3; ++k) {
        l0[k] = min(l0[k], b[1 + k]);
        h0[k] = max(h0[k], b[4 + k]);
      }
    } else {
      c1 += b[0];
      for (int k = 0; k < 3; ++k) {
        l1[k] = min(l1[k], b[1 + k]);
        h1[k] = max(h1[k], b[4 + k]);
      }
    }
  }
  const float f0 = __uint2float_rn(c0), f1 = __uint2float_rn(c1);
  if (f0 == 0.0f || f1 == 0.0f) return __int_as_float(0x7f800000);
  const float a0 = box_area(fund(l0[0]), fund(l0[1]), fund(l0[2]), fund(h0[0]), fund(h0[1]), fund(h0[2]));
  const float a1 = box_area(fund(l1[0]), fund(l1[1]), fund(l1[2]), fund(h1[0]), fund(h1[1]), fund(h1[2]));
  return fadd(0.125f, fdiv(fadd(fmul(f0, a0), fmul(f1, a1)), parea));
}

// Axes by decreasing extent, stable (aabb_tree.rs:207-221).
__device__ __forceinline__ void axis_order(const uint32_t* bnd, int ax[3], float& parea) {
  float lo[3], hi[3], sz[3];
  for (int k = 0; k < 3; ++k) {
    lo[k] = fund(bnd[k]);
    hi[k] = fund(bnd[3 + k]);
    sz[k] = fsub(hi[k], lo[k]);
  }
  ax[0] = 0;
  ax[1] = 1;
  ax[2] = 2;
  for (int i = 1; i < 3; ++i)
    for (int j = i; j > 0 && sz[ax[j]] > sz[ax[j - 1]]; --j) {
      const int t = ax[j];
      ax[j] = ax[j - 1];
      ax[j - 1] = t;
    }
  parea = box_area(lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]);
}

// Split decision of one node from its bins (aabb_tree.rs:201-250, 422-514).
__device__ RtDec decide(const uint32_t* bnd, const uint32_t* bk, uint32_t n, uint32_t prio) {
  int ax[3];
  float parea;
  axis_order(bnd, ax, parea);
  const float leaf_cost = __uint2float_rn(n);
  for (int k = 0; k < 3; ++k) {
    const int a = ax[k];
    prio = prio_push(prio, a);
    const uint32_t* b = bk + a * NB * 7;
    int best = 0;
    float bc = split_cost(b, 0, parea);
    for (int i = 1; i < NB - 1; ++i) {
      const float c = split_cost(b, i, parea);
      if (c < bc) {
        bc = c;
        best = i;
      }
    }
    if (bc < leaf_cost) {
      uint32_t nl = 0;
      for (int j = 0; j <= best; ++j) nl += b[7 * j];
      return RtDec{a, best, nl, prio};
    }
  }
  return RtDec{-1, 0, 0, prio};
}

// Links node `ref` into its parent (or as a mesh's root).
__device__ __forceinline__ void link(const RtBuild& B, int parent, int side, int ref) {
  if (parent >= 0) reinterpret_cast<int*>(B.topo)[2 * parent + side] = ref;
  else B.roots[-1 - parent] = ref;
  if (ref >= 0) B.par_i[ref] = parent;
  else B.par_l[~ref] = parent;
}

__device__ __forceinline__ void emit_leaf(const RtBuild& B, uint32_t first, uint32_t count, uint32_t prio, int parent,
                                          int side) {
  B.leaf_cnt[first] = count;
  B.leaf_prio[first] = prio;
  link(B, parent, side, ~int(first));
}

// A new node: a leaf (at most 3 triangles or depth 40, aabb_tree.rs:164-167),
// a small node for the per-CTA kernel, or a large node for the next level.
__device__ void place(const RtBuild& B, const RtSeg& c) {
  if (c.count <= MIN_LEAF || c.depth >= MAX_DEPTH) {
    emit_leaf(B, c.first, c.count, c.prio, c.parent, c.side);
  } else if (c.count <= SMALL) {
    const uint32_t s = atomicAdd(&B.counters[1], 1u);
    if (s < B.cap_small) B.small[s] = c;
    else atomicExch(&B.counters[2], 1u);
  } else {
    const uint32_t s = atomicAdd(&B.counters[0], 1u);
    if (s < B.cap_big) B.big_next[s] = c;
    else atomicExch(&B.counters[2], 1u);
  }
}

// ------------------------------------------------------------ triangles ---
// Bounding box (triangle3.rs:309-314: min2(c, min2(a, b))) and its centre
// (box3.rs:40-42) of every triangle.
__global__ void k_rt_objects(const float4* __restrict__ T, uint64_t nt, float4* __restrict__ obA,
                             float4* __restrict__ obB, float* __restrict__ obC, uint32_t* __restrict__ perm) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= nt) return;
  const float4 a = T[3 * i], b = T[3 * i + 1], c = T[3 * i + 2];
  const F3 A = f3(a.x, a.y, a.z), Bv = f3(b.x, b.y, b.z), C = f3(c.x, c.y, c.z);
  const F3 mn = min3(C, min3(A, Bv)), mx = max3(C, max3(A, Bv));
  const F3 cen = f3(fdiv(fadd(mn.x, mx.x), 2.0f), fdiv(fadd(mn.y, mx.y), 2.0f), fdiv(fadd(mn.z, mx.z), 2.0f));
  obA[i] = make_float4(mn.x, mn.y, mn.z, cen.x);
  obB[i] = make_float4(mx.x, mx.y, mx.z, cen.y);
  obC[i] = cen.z;
  perm[i] = uint32_t(i);
}

__device__ __forceinline__ int mesh_of(const uint32_t* __restrict__ base, int K, uint64_t i) {
  int lo = 0, hi = K - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (uint64_t(base[mid]) <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Per-mesh box and centre bounds (ordered uint32) of all triangles.
__global__ void k_rt_mesh_bounds(const float4* __restrict__ obA, const float4* __restrict__ obB,
                                 const float* __restrict__ obC, uint64_t nt, const uint32_t* __restrict__ tb, int K,
                                 uint32_t* __restrict__ mb) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  const bool ok = i < nt;
  const int m = ok ? mesh_of(tb, K, i) : -1;
  float4 A = make_float4(0, 0, 0, 0), Bv = A;
  float cz = 0.f;
  if (ok) {
    A = obA[i];
    Bv = obB[i];
    cz = obC[i];
  }
  const uint32_t v[12] = {ford(A.x), ford(A.y), ford(A.z), ford(Bv.x), ford(Bv.y), ford(Bv.z),
                          ford(A.w), ford(Bv.w), ford(cz),  ford(A.w), ford(Bv.w), ford(cz)};
  const int m0 = __shfl_sync(FULL, m, 0);
  if (__all_sync(FULL, m == m0)) {
    if (m0 < 0) return;
    for (int k = 0; k < 12; ++k) {
      const bool is_min = k < 3 || (k >= 6 && k < 9);
      const uint32_t r = is_min ? __reduce_min_sync(FULL, v[k]) : __reduce_max_sync(FULL, v[k]);
      if ((threadIdx.x & 31) == 0) {
        if (is_min) atomicMin(&mb[12 * m0 + k], r);
        else atomicMax(&mb[12 * m0 + k], r);
      }
    }
  } else if (ok) {
    for (int k = 0; k < 12; ++k) {
      const bool is_min = k < 3 || (k >= 6 && k < 9);
      if (is_min) atomicMin(&mb[12 * m + k], v[k]);
      else atomicMax(&mb[12 * m + k], v[k]);
    }
  }
}

__global__ void k_rt_bounds_init(uint32_t* __restrict__ b, uint64_t n_boxes) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= 12 * n_boxes) return;
  const int k = int(i % 12);
  b[i] = (k < 3 || (k >= 6 && k < 9)) ? FULL : 0u;
}

// Roots: one node per mesh over all its triangles.
__global__ void k_rt_roots(RtBuild B, const uint32_t* __restrict__ tb, int K, const uint32_t* __restrict__ mb) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= K) return;
  RtSeg r;
  r.first = tb[m];
  r.count = tb[m + 1] - tb[m];
  r.parent = -1 - m;
  r.side = 0;
  r.depth = 1;
  r.prio = 0;
  for (int k = 0; k < 12; ++k) r.bnd[k] = mb[12 * m + k];
  if (r.count) place(B, r);
}

// ---------------------------------------------------- large-node levels ---
__global__ void k_rt_bins_init(uint32_t* __restrict__ bk, uint64_t n) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int f = int(i % 7);
  bk[i] = f == 0 ? 0u : (f <= 3 ? FULL : 0u);
}

// Bins of every large node: per block a private copy in shared memory over
// one chunk of the node's positions, then merged with global atomics.
__global__ void __launch_bounds__(256) k_rt_bins(const RtChunk* __restrict__ chunks, const RtSeg* __restrict__ segs,
                                                 const uint32_t* __restrict__ perm, const float4* __restrict__ obA,
                                                 const float4* __restrict__ obB, const float* __restrict__ obC,
                                                 uint32_t* __restrict__ bk) {
  __shared__ uint32_t sb[BKW];
  for (int j = threadIdx.x; j < BKW; j += blockDim.x) {
    const int f = j % 7;
    sb[j] = f == 0 ? 0u : (f <= 3 ? FULL : 0u);
  }
  __syncthreads();
  const RtChunk ch = chunks[blockIdx.x];
  const RtSeg& S = segs[ch.seg];
  float cmn[3], cmx[3];
  for (int k = 0; k < 3; ++k) {
    cmn[k] = fund(S.bnd[6 + k]);
    cmx[k] = fund(S.bnd[9 + k]);
  }
  for (uint32_t p = ch.begin + threadIdx.x; p < ch.end; p += blockDim.x) {
    const uint32_t o = perm[p];
    const float4 A = obA[o], Bv = obB[o];
    const float c[3] = {A.w, Bv.w, obC[o]};
    const uint32_t lo[3] = {ford(A.x), ford(A.y), ford(A.z)}, hi[3] = {ford(Bv.x), ford(Bv.y), ford(Bv.z)};
    for (int a = 0; a < 3; ++a) {
      uint32_t* e = sb + (a * NB + bucket_of(c[a], cmn[a], cmx[a])) * 7;
      atomicAdd(e, 1u);
      for (int k = 0; k < 3; ++k) {
        atomicMin(e + 1 + k, lo[k]);
        atomicMax(e + 4 + k, hi[k]);
      }
    }
  }
  __syncthreads();
  uint32_t* dst = bk + uint64_t(ch.seg) * BKW;
  for (int j = threadIdx.x; j < BKW; j += blockDim.x) {
    const int f = j % 7;
    const uint32_t v = sb[j];
    if (f == 0) {
      if (v) atomicAdd(dst + j, v);
    } else if (f <= 3) {
      if (v != FULL) atomicMin(dst + j, v);
    } else if (v) {
      atomicMax(dst + j, v);
    }
  }
}

// One thread per large node: the split (or none), and empty child bounds.
__global__ void k_rt_decide(const RtSeg* __restrict__ segs, uint32_t n, const uint32_t* __restrict__ bk,
                            RtDec* __restrict__ dec, uint32_t* __restrict__ cb, uint32_t* __restrict__ cur) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const RtSeg S = segs[s];
  dec[s] = decide(S.bnd, bk + uint64_t(s) * BKW, S.count, S.prio);
  for (int k = 0; k < 24; ++k) {
    const int f = k % 12;
    cb[24 * uint64_t(s) + k] = (f < 3 || (f >= 6 && f < 9)) ? FULL : 0u;
  }
  cur[2 * s] = 0;
  cur[2 * s + 1] = 0;
}

// Places each triangle of a split node on its side (order inside a side is
// irrelevant) and gathers both children's bounds.
__global__ void __launch_bounds__(256) k_rt_place(const RtChunk* __restrict__ chunks, const RtSeg* __restrict__ segs,
                                                  const RtDec* __restrict__ dec, const uint32_t* __restrict__ perm,
                                                  uint32_t* __restrict__ ptmp, const float4* __restrict__ obA,
                                                  const float4* __restrict__ obB, const float* __restrict__ obC,
                                                  uint32_t* __restrict__ cb, uint32_t* __restrict__ cur) {
  __shared__ uint32_t sbnd[24];
  const RtChunk ch = chunks[blockIdx.x];
  const RtDec D = dec[ch.seg];
  if (D.axis < 0) return;  // block-uniform
  const RtSeg& S = segs[ch.seg];
  if (threadIdx.x < 24) {
    const int f = threadIdx.x % 12;
    sbnd[threadIdx.x] = (f < 3 || (f >= 6 && f < 9)) ? FULL : 0u;
  }
  __syncthreads();
  const float cmn = fund(S.bnd[6 + D.axis]), cmx = fund(S.bnd[9 + D.axis]);
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  for (uint32_t base = ch.begin; base < ch.end; base += blockDim.x) {
    const uint32_t p = base + threadIdx.x;
    const bool valid = p < ch.end;
    const uint32_t o = valid ? perm[p] : 0u;
    float4 A = make_float4(0, 0, 0, 0), Bv = A;
    float cz = 0.f;
    if (valid) {
      A = obA[o];
      Bv = obB[o];
      cz = obC[o];
    }
    const float c[3] = {A.w, Bv.w, cz};
    const bool left = valid && bucket_of(c[D.axis], cmn, cmx) <= D.best;
    const bool right = valid && !left;
    const unsigned mL = __ballot_sync(FULL, left), mR = __ballot_sync(FULL, right);
    uint32_t bl = 0, br = 0;
    if (lane == 0) {
      if (mL) bl = atomicAdd(&cur[2 * ch.seg], uint32_t(__popc(mL)));
      if (mR) br = atomicAdd(&cur[2 * ch.seg + 1], uint32_t(__popc(mR)));
    }
    bl = __shfl_sync(FULL, bl, 0);
    br = __shfl_sync(FULL, br, 0);
    if (left) ptmp[S.first + bl + __popc(mL & lt)] = o;
    else if (right) ptmp[S.first + D.nl + br + __popc(mR & lt)] = o;
    const uint32_t v[12] = {ford(A.x), ford(A.y), ford(A.z), ford(Bv.x), ford(Bv.y), ford(Bv.z),
                            ford(c[0]), ford(c[1]), ford(c[2]), ford(c[0]), ford(c[1]), ford(c[2])};
    for (int side = 0; side < 2; ++side) {
      const bool mine = side ? right : left;
      if (!(side ? mR : mL)) continue;  // warp-uniform
      for (int k = 0; k < 12; ++k) {
        const bool is_min = k < 3 || (k >= 6 && k < 9);
        const uint32_t r = is_min ? __reduce_min_sync(FULL, mine ? v[k] : FULL)
                                  : __reduce_max_sync(FULL, mine ? v[k] : 0u);
        if (lane == 0) {
          if (is_min) atomicMin(&sbnd[12 * side + k], r);
          else atomicMax(&sbnd[12 * side + k], r);
        }
      }
    }
  }
  __syncthreads();
  if (threadIdx.x < 24) {
    const int f = threadIdx.x % 12;
    const uint32_t v = sbnd[threadIdx.x];
    if (f < 3 || (f >= 6 && f < 9)) {
      if (v != FULL) atomicMin(&cb[24 * uint64_t(ch.seg) + threadIdx.x], v);
    } else if (v) {
      atomicMax(&cb[24 * uint64_t(ch.seg) + threadIdx.x], v);
    }
  }
}

__global__ void k_rt_copyback(const RtChunk* __restrict__ chunks, const RtDec* __restrict__ dec,
                              const uint32_t* __restrict__ ptmp, uint32_t* __restrict__ perm) {
  const RtChunk ch = chunks[blockIdx.x];
  if (dec[ch.seg].axis < 0) return;
  for (uint32_t p = ch.begin + threadIdx.x; p < ch.end; p += blockDim.x) perm[p] = ptmp[p];
}

// One thread per large node: the node itself (a leaf, or an internal node
// numbered by its split position) and its two children.
__global__ void k_rt_children(RtBuild B, const RtSeg* __restrict__ segs, uint32_t n, const RtDec* __restrict__ dec,
                              const uint32_t* __restrict__ cb, const uint32_t* __restrict__ cur) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const RtSeg S = segs[s];
  const RtDec D = dec[s];
  if (D.axis < 0) {
    emit_leaf(B, S.first, S.count, D.prio, S.parent, S.side);
    return;
  }
  if (cur[2 * s] != D.nl || cur[2 * s + 1] != S.count - D.nl) atomicExch(&B.counters[2], 2u);
  const int id = int(S.first + D.nl) - 1;
  link(B, S.parent, S.side, id);
  for (int side = 0; side < 2; ++side) {
    RtSeg c;
    c.first = side ? S.first + D.nl : S.first;
    c.count = side ? S.count - D.nl : D.nl;
    c.parent = id;
    c.side = side;
    c.depth = S.depth + 1;
    c.prio = D.prio;
    for (int k = 0; k < 12; ++k) c.bnd[k] = cb[24 * uint64_t(s) + 12 * side + k];
    place(B, c);
  }
}

// ------------------------------------------------------- small nodes ------
struct LSeg {
  uint16_t lf, n;  // local positions [lf, lf + n)
  int parent;
  uint8_t side, depth;
  uint16_t prio;
};

// One CTA finishes the subtree of one node of at most SMALL triangles: the
// triangles' boxes and centres in shared memory, one level of nodes at a
// time, a warp per node (bounds, bins of all three axes, the decision, a
// stable in-warp partition of the local order).
__global__ void __launch_bounds__(ST_THREADS) k_rt_small(RtBuild B) {
  __shared__ float sx[9][SMALL];  // box lo xyz, box hi xyz, centre xyz
  __shared__ uint32_t oid[SMALL];
  __shared__ uint16_t pa[SMALL], pb[SMALL];
  __shared__ LSeg lst[2][ST_LIST];
  __shared__ uint32_t wb[ST_WARPS][BKW];
  __shared__ int ncnt[2];
  const RtSeg S = B.small[blockIdx.x];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t n0 = S.count;
  for (uint32_t j = threadIdx.x; j < n0; j += blockDim.x) {
    const uint32_t o = B.perm[S.first + j];
    const float4 A = B.obA[o], Bv = B.obB[o];
    oid[j] = o;
    sx[0][j] = A.x; sx[1][j] = A.y; sx[2][j] = A.z;
    sx[3][j] = Bv.x; sx[4][j] = Bv.y; sx[5][j] = Bv.z;
    sx[6][j] = A.w; sx[7][j] = Bv.w; sx[8][j] = B.obC[o];
    pa[j] = uint16_t(j);
  }
  if (threadIdx.x == 0) {
    lst[0][0] = LSeg{0, uint16_t(n0), S.parent, uint8_t(S.side), uint8_t(S.depth), uint16_t(S.prio)};
    ncnt[0] = 1;
    ncnt[1] = 0;
  }
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  int cur = 0;
  for (int level = 0; level <= MAX_DEPTH; ++level) {
    const int nseg = ncnt[cur];
    if (nseg == 0) break;
    for (int si = warp; si < nseg; si += ST_WARPS) {
      const LSeg L = lst[cur][si];
      const uint32_t lf = L.lf, n = L.n;
      // bounds of the node's boxes and centres
      uint32_t b[12];
      for (int k = 0; k < 12; ++k) b[k] = (k < 3 || (k >= 6 && k < 9)) ? FULL : 0u;
      for (uint32_t j = lane; j < n; j += 32) {
        const int i = pa[lf + j];
        for (int k = 0; k < 3; ++k) {
          b[k] = min(b[k], ford(sx[k][i]));
          b[3 + k] = max(b[3 + k], ford(sx[3 + k][i]));
          b[6 + k] = min(b[6 + k], ford(sx[6 + k][i]));
          b[9 + k] = max(b[9 + k], ford(sx[6 + k][i]));
        }
      }
      for (int k = 0; k < 12; ++k)
        b[k] = (k < 3 || (k >= 6 && k < 9)) ? __reduce_min_sync(FULL, b[k]) : __reduce_max_sync(FULL, b[k]);
      // bins of all three axes
      uint32_t* bk = wb[warp];
      for (int j = lane; j < BKW; j += 32) {
        const int f = j % 7;
        bk[j] = f == 0 ? 0u : (f <= 3 ? FULL : 0u);
      }
      __syncwarp();
      float cmn[3], cmx[3];
      for (int k = 0; k < 3; ++k) {
        cmn[k] = fund(b[6 + k]);
        cmx[k] = fund(b[9 + k]);
      }
      for (uint32_t j = lane; j < n; j += 32) {
        const int i = pa[lf + j];
        for (int a = 0; a < 3; ++a) {
          uint32_t* e = bk + (a * NB + bucket_of(sx[6 + a][i], cmn[a], cmx[a])) * 7;
          atomicAdd(e, 1u);
          for (int k = 0; k < 3; ++k) {
            atomicMin(e + 1 + k, ford(sx[k][i]));
            atomicMax(e + 4 + k, ford(sx[3 + k][i]));
          }
        }
      }
      __syncwarp();
      // decision: lanes 0..10 cost one boundary each, the scan keeps the
      // first minimum as the reference's sequential min_by does
      int ax[3];
      float parea;
      axis_order(b, ax, parea);
      const float leaf_cost = __uint2float_rn(n);
      uint32_t prio = L.prio;
      int axis = -1, best = 0;
      for (int k = 0; k < 3; ++k) {
        const int a = ax[k];
        prio = prio_push(prio, a);
        const float cst = lane < NB - 1 ? split_cost(bk + a * NB * 7, lane, parea) : 0.0f;
        float bc = __shfl_sync(FULL, cst, 0);
        int bi = 0;
        for (int i = 1; i < NB - 1; ++i) {
          const float ci = __shfl_sync(FULL, cst, i);
          if (ci < bc) {
            bc = ci;
            bi = i;
          }
        }
        if (bc < leaf_cost) {
          axis = a;
          best = bi;
          break;
        }
      }
      if (axis < 0) {
        if (lane == 0) emit_leaf(B, S.first + lf, n, prio, L.parent, L.side);
        __syncwarp();
        continue;
      }
      uint32_t nl = 0;
      for (int j = 0; j <= best; ++j) nl += bk[(axis * NB + j) * 7];
      // stable partition of the local order into pb, then back into pa
      uint32_t cl = 0, cr = 0;
      for (uint32_t base = 0; base < n; base += 32) {
        const uint32_t j = base + lane;
        const bool valid = j < n;
        const int i = valid ? pa[lf + j] : 0;
        const bool left = valid && bucket_of(sx[6 + axis][i], cmn[axis], cmx[axis]) <= best;
        const unsigned mL = __ballot_sync(FULL, left), mR = __ballot_sync(FULL, valid && !left);
        if (left) pb[lf + cl + __popc(mL & lt)] = uint16_t(i);
        else if (valid) pb[lf + nl + cr + __popc(mR & lt)] = uint16_t(i);
        cl += __popc(mL);
        cr += __popc(mR);
      }
      __syncwarp();
      for (uint32_t j = lane; j < n; j += 32) pa[lf + j] = pb[lf + j];
      __syncwarp();
      if (lane == 0) {
        if (cl != nl) atomicExch(&B.counters[2], 2u);
        const int id = int(S.first + lf + nl) - 1;
        link(B, L.parent, L.side, id);
        for (int side = 0; side < 2; ++side) {
          const uint32_t cf = side ? lf + nl : lf, cc = side ? n - nl : nl;
          const int cd = L.depth + 1;
          if (cc <= MIN_LEAF || cd >= MAX_DEPTH) {
            emit_leaf(B, S.first + cf, cc, prio, id, side);
          } else {
            const int slot = atomicAdd(&ncnt[cur ^ 1], 1);
            if (slot < ST_LIST) lst[cur ^ 1][slot] = LSeg{uint16_t(cf), uint16_t(cc), id, uint8_t(side), uint8_t(cd),
                                                          uint16_t(prio)};
            else atomicExch(&B.counters[2], 3u);
          }
        }
      }
      __syncwarp();
    }
    __syncthreads();
    if (threadIdx.x == 0) ncnt[cur] = 0;
    cur ^= 1;
    __syncthreads();
  }
  for (uint32_t j = threadIdx.x; j < n0; j += blockDim.x) B.perm[S.first + j] = oid[pa[j]];
}

// ------------------------------------------------------ leaves and data ---
// Centre coordinate of a triangle along an axis, -0 as +0 (partial_cmp
// calls them equal).
__device__ __forceinline__ float centre_key(const float4* obA, const float4* obB, const float* obC, uint32_t o,
                                            int a) {
  const float v = a == 0 ? obA[o].w : (a == 1 ? obB[o].w : obC[o]);
  return v == 0.0f ? 0.0f : v;
}
// Leaf order: the sort keys, most recent first, then the mesh order.
__device__ __forceinline__ bool leaf_less(const float4* obA, const float4* obB, const float* obC, uint32_t prio,
                                          uint32_t x, uint32_t y) {
  const int n = int(prio & 3u);
  for (int r = 0; r < n; ++r) {
    const int a = int((prio >> (2 + 2 * r)) & 3u);
    const float kx = centre_key(obA, obB, obC, x, a), ky = centre_key(obA, obB, obC, y, a);
    if (kx < ky) return true;
    if (ky < kx) return false;
  }
  return x < y;
}

constexpr uint32_t LEAF_SORT_THREAD = 32;  // larger leaves get a block each

__global__ void k_rt_leaf_sort(uint64_t nt, const uint32_t* __restrict__ leaf_cnt,
                               const uint32_t* __restrict__ leaf_prio, uint32_t* __restrict__ perm,
                               const float4* __restrict__ obA, const float4* __restrict__ obB,
                               const float* __restrict__ obC, uint32_t* __restrict__ big, uint32_t* __restrict__ n_big) {
  const uint64_t p = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (p >= nt) return;
  const uint32_t c = leaf_cnt[p];
  if (c < 2) return;
  if (c > LEAF_SORT_THREAD) {
    big[atomicAdd(n_big, 1u)] = uint32_t(p);
    return;
  }
  const uint32_t prio = leaf_prio[p];
  uint32_t v[LEAF_SORT_THREAD];
  for (uint32_t j = 0; j < c; ++j) v[j] = perm[p + j];
  for (uint32_t j = 1; j < c; ++j)
    for (uint32_t k = j; k > 0 && leaf_less(obA, obB, obC, prio, v[k], v[k - 1]); --k) {
      const uint32_t t = v[k];
      v[k] = v[k - 1];
      v[k - 1] = t;
    }
  for (uint32_t j = 0; j < c; ++j) perm[p + j] = v[j];
}

// A large leaf (many triangles with coincident centres): rank sort.
__global__ void k_rt_leaf_sort_big(const uint32_t* __restrict__ big, const uint32_t* __restrict__ leaf_cnt,
                                   const uint32_t* __restrict__ leaf_prio, uint32_t* __restrict__ perm,
                                   uint32_t* __restrict__ tmp, const float4* __restrict__ obA,
                                   const float4* __restrict__ obB, const float* __restrict__ obC) {
  const uint32_t p = big[blockIdx.x], c = leaf_cnt[p], prio = leaf_prio[p];
  for (uint32_t j = threadIdx.x; j < c; j += blockDim.x) {
    const uint32_t x = perm[p + j];
    uint32_t rank = 0;
    for (uint32_t k = 0; k < c; ++k) rank += leaf_less(obA, obB, obC, prio, perm[p + k], x) ? 1u : 0u;
    tmp[p + rank] = x;
  }
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < c; j += blockDim.x) perm[p + j] = tmp[p + j];
}

__global__ void k_rt_tri(const float4* __restrict__ T, const uint32_t* __restrict__ perm, uint64_t nt,
                         float4* __restrict__ tri) {
  const uint64_t p = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (p >= nt) return;
  const uint32_t o = perm[p];
  tri[3 * p] = T[3 * uint64_t(o)];
  tri[3 * p + 1] = T[3 * uint64_t(o) + 1];
  tri[3 * p + 2] = T[3 * uint64_t(o) + 2];
}

// InitData of a node (aabb_tree.rs:709-715) with its box: 6 float4
//   [0] awn xyz, area   [1] awc xyz, lo.x   [2] lo.y lo.z hi.x hi.y
//   [3] hi.z, o1[0..2]  [4] o1[3..6]        [5] o1[7..8], -, -
// o1 is column-major (o1[3j + i] = row i, column j).
struct Init {
  F3 awn, awc;
  float o1[9];
  float area;
  F3 lo, hi;
};
__device__ __forceinline__ void store_init(float4* d, const Init& v) {
  d[0] = make_float4(v.awn.x, v.awn.y, v.awn.z, v.area);
  d[1] = make_float4(v.awc.x, v.awc.y, v.awc.z, v.lo.x);
  d[2] = make_float4(v.lo.y, v.lo.z, v.hi.x, v.hi.y);
  d[3] = make_float4(v.hi.z, v.o1[0], v.o1[1], v.o1[2]);
  d[4] = make_float4(v.o1[3], v.o1[4], v.o1[5], v.o1[6]);
  d[5] = make_float4(v.o1[7], v.o1[8], 0.f, 0.f);
}
// Loads data another SM wrote (bypassing L1, which is not coherent).
__device__ __forceinline__ Init load_init(const float4* d) {
  float4 q[6];
  for (int k = 0; k < 6; ++k) q[k] = __ldcg(d + k);
  Init v;
  v.awn = f3(q[0].x, q[0].y, q[0].z);
  v.area = q[0].w;
  v.awc = f3(q[1].x, q[1].y, q[1].z);
  v.lo = f3(q[1].w, q[2].x, q[2].y);
  v.hi = f3(q[2].z, q[2].w, q[3].x);
  v.o1[0] = q[3].y; v.o1[1] = q[3].z; v.o1[2] = q[3].w;
  v.o1[3] = q[4].x; v.o1[4] = q[4].y; v.o1[5] = q[4].z; v.o1[6] = q[4].w;
  v.o1[7] = q[5].x; v.o1[8] = q[5].y;
  return v;
}

// NodeData of compute_node_data (aabb_tree.rs:723-747): dipole centre,
// radius to the farther box corner, order-1 = area-weighted normal, order-2
// = o1 - dipole * awn^T.
__device__ __forceinline__ void store_record(float4* r, float* rad, const Init& d, F3 dip) {
  const F3 a = sub3(d.lo, dip), b = sub3(d.hi, dip);
  const float radius = fsqrt(fmaxf(dot3(a, a), dot3(b, b)));
  *rad = radius;
  const float aw[3] = {d.awn.x, d.awn.y, d.awn.z}, dp[3] = {dip.x, dip.y, dip.z};
  float o2[9];
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) o2[3 * j + i] = fsub(d.o1[3 * j + i], fmul(dp[i], aw[j]));
  r[0] = make_float4(dip.x, dip.y, dip.z, radius);
  r[1] = make_float4(d.awn.x, d.awn.y, d.awn.z, o2[0]);
  r[2] = make_float4(o2[1], o2[2], o2[3], o2[4]);
  r[3] = make_float4(o2[5], o2[6], o2[7], o2[8]);
}

// leaf_data (aabb_tree.rs:749-777) over the leaf's triangles in order, then
// branch_data (aabb_tree.rs:779-801) up the tree: the second child to
// arrive at a parent combines it, left + right.
__global__ void k_rt_refit(uint64_t nt, const uint32_t* __restrict__ leaf_cnt, const float4* __restrict__ tri,
                           const int2* __restrict__ topo, const int* __restrict__ par_i,
                           const int* __restrict__ par_l, int* __restrict__ flags, float4* __restrict__ ld_i,
                           float4* __restrict__ ld_l, float4* __restrict__ rec_i, float4* __restrict__ rec_l,
                           float* __restrict__ rad_i, float* __restrict__ rad_l) {
  const uint64_t p = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (p >= nt) return;
  const uint32_t c = leaf_cnt[p];
  if (c == 0) return;
  Init d;
  d.awn = d.awc = f3(0.f, 0.f, 0.f);
  for (int k = 0; k < 9; ++k) d.o1[k] = 0.f;
  d.area = 0.f;
  d.lo = f3(3.40282347e+38f, 3.40282347e+38f, 3.40282347e+38f);
  d.hi = f3(-3.40282347e+38f, -3.40282347e+38f, -3.40282347e+38f);
  for (uint32_t t = 0; t < c; ++t) {
    const float4 A4 = tri[3 * (p + t)], B4 = tri[3 * (p + t) + 1], C4 = tri[3 * (p + t) + 2];
    const F3 A = f3(A4.x, A4.y, A4.z), Bv = f3(B4.x, B4.y, B4.z), C = f3(C4.x, C4.y, C4.z);
    // leaf box: the union of the triangles' boxes (aabb_tree.rs:252-258)
    const F3 mn = min3(C, min3(A, Bv)), mx = max3(C, max3(A, Bv));
    if (t == 0) {
      d.lo = mn;
      d.hi = mx;
    } else {
      d.hi = max3(d.hi, mx);
      d.lo = min3(d.lo, mn);
    }
    const F3 cr = cross3(sub3(Bv, A), sub3(C, A));
    const float n2 = dot3(cr, cr);
    if (n2 == 0.0f) continue;  // get_normal() is None (triangle3.rs:261-269)
    const float len = fsqrt(n2);
    const F3 nrm = f3(fdiv(cr.x, len), fdiv(cr.y, len), fdiv(cr.z, len));
    const float area = fmul(len, 0.5f);  // Triangle3::area (triangle3.rs:278-280)
    d.area = fadd(d.area, area);
    d.awn = add3(d.awn, f3(fmul(area, nrm.x), fmul(area, nrm.y), fmul(area, nrm.z)));
    const F3 cen = f3(fdiv(fadd(fadd(A.x, Bv.x), C.x), 3.0f), fdiv(fadd(fadd(A.y, Bv.y), C.y), 3.0f),
                      fdiv(fadd(fadd(A.z, Bv.z), C.z), 3.0f));
    const float ac[3] = {fmul(area, cen.x), fmul(area, cen.y), fmul(area, cen.z)};
    const float nn[3] = {nrm.x, nrm.y, nrm.z};
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) d.o1[3 * j + i] = fadd(d.o1[3 * j + i], fmul(ac[i], nn[j]));
    d.awc = add3(d.awc, f3(fmul(area, cen.x), fmul(area, cen.y), fmul(area, cen.z)));
  }
  F3 dip = f3(fdiv(d.awc.x, d.area), fdiv(d.awc.y, d.area), fdiv(d.awc.z, d.area));
  store_init(ld_l + 6 * p, d);
  store_record(rec_l + 4 * p, rad_l + p, d, dip);
  __threadfence();
  int par = par_l[p];
  for (int guard = 0; par >= 0 && guard <= MAX_DEPTH + 1; ++guard) {
    if (atomicAdd(&flags[par], 1) == 0) return;  // the other child finishes this parent
    __threadfence();
    const int2 ch = __ldcg(topo + par);
    const Init l = load_init(ch.x >= 0 ? ld_i + 6 * uint64_t(ch.x) : ld_l + 6 * uint64_t(~ch.x));
    const Init r = load_init(ch.y >= 0 ? ld_i + 6 * uint64_t(ch.y) : ld_l + 6 * uint64_t(~ch.y));
    Init m;
    for (int k = 0; k < 9; ++k) m.o1[k] = fadd(l.o1[k], r.o1[k]);
    m.awn = add3(l.awn, r.awn);
    m.awc = add3(l.awc, r.awc);
    m.area = fadd(l.area, r.area);
    m.lo = min3(l.lo, r.lo);
    m.hi = max3(l.hi, r.hi);
    const F3 s = add3(l.awc, r.awc);
    dip = f3(fdiv(s.x, m.area), fdiv(s.y, m.area), fdiv(s.z, m.area));
    store_init(ld_i + 6 * uint64_t(par), m);
    store_record(rec_i + 4 * uint64_t(par), rad_i + par, m, dip);
    __threadfence();
    par = __ldcg(par_i + par);
  }
}

// The far test |q - p| > beta r (aabb_tree.rs:665-666) without the square
// root: for t = RN(r * beta) >= 0 and t+ the next float above t,
// RN(sqrt(x)) > t exactly when sqrt(x) exceeds the midpoint m = (t + t+) / 2
// (sqrt(x) never equals m: m has 25 significant bits, so m^2 is no float),
// that is when x > m^2, and for a float x when x > RD(m^2).  m^2 is exact in
// double.  The record's .w holds this threshold for the call's beta.
__device__ __forceinline__ float far_tau(float radius, float beta) {
  const float t = fmul(radius, beta);
  if (t != t) return t;                                   // NaN radius: never far
  if (t < 0.0f) return -1.0f;                             // every |q - p| exceeds t
  if (t == __int_as_float(0x7f800000)) return t;          // never far
  const float tp = nextafterf(t, __int_as_float(0x7f800000));
  if (tp == __int_as_float(0x7f800000)) return 3.40282347e+38f;  // only an infinite x rounds above
  const double m = (double(t) + double(tp)) * 0.5;
  return __double2float_rd(m * m);
}

// Writes every node's far threshold for its mesh's beta into its record.
__global__ void k_rt_tau(uint64_t nt, const uint32_t* __restrict__ tb, int K, const float* __restrict__ beta,
                         const uint32_t* __restrict__ leaf_cnt, const int* __restrict__ flags,
                         const float* __restrict__ rad_i, const float* __restrict__ rad_l, float4* __restrict__ rec_i,
                         float4* __restrict__ rec_l) {
  const uint64_t p = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (p >= nt) return;
  const float b = beta[K > 1 ? mesh_of(tb, K, p) : 0];
  if (leaf_cnt[p]) rec_l[4 * p].w = far_tau(rad_l[p], b);
  if (flags[p] == 2) rec_i[4 * p].w = far_tau(rad_i[p], b);  // internal node p (both children combined)
}

// Opening record of every internal node: both children's dipole centre and
// far threshold (copied from their records) and their references and leaf
// triangle counts, so a warp opening a node reads three float4 at once.
__global__ void k_rt_open(uint64_t nt, const int* __restrict__ flags, const int2* __restrict__ topo,
                          const uint32_t* __restrict__ leaf_cnt, const float4* __restrict__ rec_i,
                          const float4* __restrict__ rec_l, float4* __restrict__ open) {
  const uint64_t p = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (p >= nt || flags[p] != 2) return;
  const int2 ch = topo[p];
  const float4 hl = ch.x >= 0 ? rec_i[4 * uint64_t(ch.x)] : rec_l[4 * uint64_t(~ch.x)];
  const float4 hr = ch.y >= 0 ? rec_i[4 * uint64_t(ch.y)] : rec_l[4 * uint64_t(~ch.y)];
  open[3 * p] = hl;
  open[3 * p + 1] = hr;
  open[3 * p + 2] = make_float4(__int_as_float(ch.x), __int_as_float(ch.y),
                                __uint_as_float(ch.x < 0 ? leaf_cnt[~ch.x] : 0u),
                                __uint_as_float(ch.y < 0 ? leaf_cnt[~ch.y] : 0u));
}

// ------------------------------------------------------------ traversal ---
// v / len for the three components of v, correctly rounded, with one
// reciprocal (mdiv) where the operands allow it.
__device__ __forceinline__ F3 div3(F3 v, float len) {
  if (mdiv_range(len) && (v.x == 0.0f || mdiv_range(v.x)) && (v.y == 0.0f || mdiv_range(v.y)) &&
      (v.z == 0.0f || mdiv_range(v.z))) {
    const float y = __frcp_rn(len);
    // a zero component keeps its sign (0 / len = 0 * (1 / len))
    return f3(v.x == 0.0f ? fmul(v.x, y) : mdiv(v.x, len, y), v.y == 0.0f ? fmul(v.y, y) : mdiv(v.y, len, y),
              v.z == 0.0f ? fmul(v.z, y) : mdiv(v.z, len, y));
  }
  return f3(fdiv(v.x, len), fdiv(v.y, len), fdiv(v.z, len));
}

// solid_angle (aabb_tree.rs:582-615): Van Oosterom–Strackee, unfused.
__device__ __forceinline__ float solid_angle(float4 A, float4 Bv, float4 C, F3 q) {
  F3 qa = sub3(f3(A.x, A.y, A.z), q), qb = sub3(f3(Bv.x, Bv.y, Bv.z), q), qc = sub3(f3(C.x, C.y, C.z), q);
  const float la = fsqrt(dot3(qa, qa)), lb = fsqrt(dot3(qb, qb)), lc = fsqrt(dot3(qc, qc));
  if (la == 0.f || lb == 0.f || lc == 0.f) return 0.f;
  qa = div3(qa, la);
  qb = div3(qb, lb);
  qc = div3(qc, lc);
  const float num = dot3(qa, cross3(sub3(qb, qa), sub3(qc, qa)));
  if (num == 0.f) return 0.f;
  const float den = fadd(fadd(fadd(1.0f, dot3(qa, qb)), dot3(qa, qc)), dot3(qb, qc));
  return fmul(atan2f(num, den), 2.0f);
}

// Far field of a node at q (aabb_tree.rs:666-671 with hessians, 803-816):
// r = p - q, the order-1 term a . r / (4 pi |r|^3) and the Frobenius product
// of the order-2 coefficients with I / (4 pi |r|^3) - 3 r r^T / (4 pi |r|^5).
// The nine quotients by 4 pi |r|^5 share one reciprocal (mdiv) when every
// component of r is 0 or within [2^-28, 2^28] and 4 pi |r|^5 within
// [2^-60, 2^60]: every dividend (3 r_i) r_j is then 0 or within [2^-60, 2^60].
// A dividend of -0 gives +0 there, which the following id - quotient turns
// into the same +0 or id that IEEE division's -0 gives.
__device__ __forceinline__ float far_field(const float4* R, float4 P, F3 q, float r2) {
  const float4 c1 = R[1], c2 = R[2], c3 = R[3];
  const float r1 = fsqrt(r2);  // |q - p| (norm, aabb_tree.rs:665; r1 of hessians, 806)
  const float r[3] = {fsub(P.x, q.x), fsub(P.y, q.y), fsub(P.z, q.z)};
  const float r3 = fmul(r2, r1);
  const float inv = fdiv(1.0f, fmul(FOUR_PI_F, r3));
  const float r5 = fmul(r3, r2);
  const float d5 = fmul(FOUR_PI_F, r5);
  const float t[3] = {fmul(3.0f, r[0]), fmul(3.0f, r[1]), fmul(3.0f, r[2])};
  const float B[9] = {c1.w, c2.x, c2.y, c2.z, c2.w, c3.x, c3.y, c3.z, c3.w};
  const float v1 = fadd(fadd(fmul(c1.x, fmul(r[0], inv)), fmul(c1.y, fmul(r[1], inv))), fmul(c1.z, fmul(r[2], inv)));
  auto comp_ok = [](float x) {
    const float ax = fabsf(x);
    return ax == 0.0f || (ax >= 0x1p-28f && ax <= 0x1p28f);
  };
  float v2 = 0.0f;
  if (mdiv_range(d5) && comp_ok(r[0]) && comp_ok(r[1]) && comp_ok(r[2])) {
    // inv is then positive and finite, so the identity's entries are inv
    // and +0, and +0 - x = -x up to the sign of a zero, which no sum here
    // can see: v2 starts at +0 and x + (+-0) is x, +0 for x = +-0
    const float y = __frcp_rn(d5);
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) {
        const float qt = mdiv(fmul(t[i], r[j]), d5, y);
        v2 = fadd(v2, fmul(B[3 * j + i], i == j ? fsub(inv, qt) : -qt));
      }
  } else {
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) {
        const float id = fmul(i == j ? 1.0f : 0.0f, inv);
        v2 = fadd(v2, fmul(B[3 * j + i], fsub(id, fdiv(fmul(t[i], r[j]), d5))));
      }
  }
  return fadd(v1, v2);
}

// Work counters, the same in every lane of a warp (computed from ballot
// masks): far-field evaluations and exact solid angles its lanes need, and
// the far-field and leaf sections the warp runs for them.
struct Counts {
  uint32_t iters = 0, far = 0, exact = 0;
  uint32_t far_sec = 0, exact_sec = 0;
  bool overflow = false;
};

// fast_wn (aabb_tree.rs:662-691) at the 32 points of a warp, each lane
// with its own cut of the tree and its own sums in the recursion's order.
// The warp walks the union of the lanes' recursions depth first.  Each step
// opens one node for the lanes that open it and tests both children for
// them: a lane takes a child's far field when it is far for it, a leaf
// child's triangles, and opens the others, so the warp descends only where
// some lane opens a child.  A lane's value for a node is therefore exactly
// its recursion's wn(node) — far field, leaf sum, or wn(left) + wn(right)
// added once both children are known.  Node records are read once per warp
// (uniform addresses); only the far-field and leaf arithmetic diverges.
// Per opened level the warp keeps the right child, the lanes opening each
// child and the lanes that opened the node (shared memory); each lane keeps
// its two child values.
struct WarpStack {
  int right[STACK];
  unsigned open_l[STACK], open_r[STACK];
  unsigned act[STACK];
};

// The lanes in `lanes` meet node `ref` (header H: dipole centre, far
// threshold; c: its leaf triangle count): far field or leaf sum into v;
// returns the lanes that open it (an internal node near for them).
__device__ __forceinline__ unsigned resolve(int ref, uint32_t c, float4 H, unsigned lanes, F3 q,
                                            const float4* __restrict__ rec_i, const float4* __restrict__ rec_l,
                                            const float4* __restrict__ tri, float& v, Counts& cnt) {
  const unsigned me = 1u << (threadIdx.x & 31);
  const float dx = fsub(q.x, H.x), dy = fsub(q.y, H.y), dz = fsub(q.z, H.z);
  const float r2 = fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz));
  const unsigned farm = __ballot_sync(FULL, r2 > H.w) & lanes;  // |q - p| > beta r
  const unsigned rest = lanes & ~farm;
  if (farm) {
    cnt.far += __popc(farm);
    ++cnt.far_sec;
    if (farm & me) v = far_field(ref >= 0 ? rec_i + 4 * ref : rec_l + 4 * (~ref), H, q, r2);
  }
  if (ref >= 0) return rest;
  if (rest) {
    cnt.exact += __popc(rest) * c;
    cnt.exact_sec += c;
    if (rest & me) {
      const uint32_t p = ~ref;
      float w = 0.0f;
      for (uint32_t k = 0; k < c; ++k)
        w = fadd(w, solid_angle(__ldg(tri + 3 * (p + k)), __ldg(tri + 3 * (p + k) + 1), __ldg(tri + 3 * (p + k) + 2), q));
      v = fdiv(w, FOUR_PI_F);  // winding_number (aabb_tree.rs:617-628)
    }
  }
  return 0u;
}

__device__ float ref_wn_warp(F3 q, unsigned valid, int root, const float4* __restrict__ rec_i,
                             const float4* __restrict__ opn, const float4* __restrict__ rec_l,
                             const uint32_t* __restrict__ leaf_cnt, const float4* __restrict__ tri, WarpStack& ws,
                             Counts& cnt) {
  const int lane = threadIdx.x & 31;
  const unsigned me = 1u << lane;
  float lval[STACK], rval[STACK];
  float v = 0.0f;
  const float4 Hroot = __ldg(root >= 0 ? rec_i + 4 * root : rec_l + 4 * (~root));
  unsigned open = resolve(root, root >= 0 ? 0u : __ldg(leaf_cnt + ~root), Hroot, valid, q, rec_i, rec_l, tri, v, cnt);
  if (!open) return v;
  const float v_root = v;  // lanes for which the root itself is far (or a leaf)
  const bool root_open = (open & me) != 0;
  int node = root, d = 0;
  uint64_t phase = 0;  // bit f: level f is descending its right child
  for (uint32_t guard = 0; guard < (1u << 30); ++guard) {
    // open `node` for the lanes in `open`
    const float4 HL = __ldg(opn + 3 * node), HR = __ldg(opn + 3 * node + 1), M = __ldg(opn + 3 * node + 2);
    const int2 ch = make_int2(__float_as_int(M.x), __float_as_int(M.y));
    float vl = 0.0f, vr = 0.0f;
    ++cnt.iters;
    const unsigned ol = resolve(ch.x, __float_as_uint(M.z), HL, open, q, rec_i, rec_l, tri, vl, cnt);
    const unsigned orr = resolve(ch.y, __float_as_uint(M.w), HR, open, q, rec_i, rec_l, tri, vr, cnt);
    if (ol | orr) {
      if (d >= STACK) {
        cnt.overflow = true;
        return 0.0f;
      }
      lval[d] = vl;
      rval[d] = vr;
      __syncwarp();  // every lane has read the entries this push may replace
      if (lane == 0) {
        ws.right[d] = ch.y;
        ws.open_l[d] = ol;
        ws.open_r[d] = orr;
        ws.act[d] = open;
      }
      __syncwarp();
      if (ol) {
        phase &= ~(1ull << d);
        node = ch.x;
        open = ol;
      } else {
        phase |= 1ull << d;
        node = ch.y;
        open = orr;
      }
      ++d;
      continue;
    }
    v = fadd(vl, vr);  // left_wn + right_wn
    // `node` is done for every lane in `open`: fold it into the pending sums
    bool next = false;
    while (d > 0) {
      const int f = d - 1;
      if (!((phase >> f) & 1ull)) {  // its left child returned
        if (ws.open_l[f] & me) lval[f] = v;
        const unsigned r = ws.open_r[f];
        if (r) {
          phase |= 1ull << f;
          node = ws.right[f];
          open = r;
          next = true;
          break;
        }
      } else if (ws.open_r[f] & me) {  // its right child returned
        rval[f] = v;
      }
      v = fadd(lval[f], rval[f]);  // left_wn + right_wn
      open = ws.act[f];
      --d;
    }
    if (!next) return root_open ? v : v_root;
  }
  cnt.overflow = true;
  return 0.0f;
}

__device__ __forceinline__ void flush_counts(const Counts& c, unsigned long long* counters) {
  const unsigned ov = __ballot_sync(FULL, c.overflow);
  if ((threadIdx.x & 31) == 0) {  // the counters are warp-uniform
    atomicAdd(counters, 1ull + 2ull * c.iters);  // node visits: the root, then two children per opening
    atomicAdd(counters + 1, (unsigned long long)c.far);
    atomicAdd(counters + 2, (unsigned long long)c.exact);
    if (ov) atomicAdd(counters + 3, 1ull);
    atomicAdd(counters + 4, (unsigned long long)c.far_sec);
    atomicAdd(counters + 5, (unsigned long long)c.exact_sec);
  }
}

constexpr int SIGN_WARPS = 4;

// One warp per 32 consecutive band voxels of one mesh (mesh_to_volume.rs:
// 245-280): warps are numbered per mesh (warp_base[m] .. warp_base[m+1]).
// WARPS per block: 2, 4 or 8 (the context's tuned launch shape).
template <int WARPS>
__global__ void __launch_bounds__(32 * WARPS) k_rt_sign(const uint32_t* __restrict__ act,
                                                             const uint32_t* __restrict__ act_base,
                                                             const uint32_t* __restrict__ warp_base, int K,
                                                             const RefSignMesh* __restrict__ meshes,
                                                             const int4* __restrict__ origins,
                                                             float* __restrict__ values,
                                                             const float4* __restrict__ rec_i,
                                                             const float4* __restrict__ opn,
                                                             const float4* __restrict__ rec_l,
                                                             const uint32_t* __restrict__ leaf_cnt,
                                                             const float4* __restrict__ tri,
                                                             unsigned long long* __restrict__ counters) {
  __shared__ WarpStack ws[WARPS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint64_t gw = blockIdx.x * uint64_t(WARPS) + w;
  if (gw >= warp_base[K]) return;  // whole warp
  const int m = K > 1 ? mesh_of(warp_base, K, gw) : 0;
  const uint64_t a1 = act_base[m + 1];
  const uint64_t i = act_base[m] + (gw - warp_base[m]) * 32 + lane;
  const bool ok = i < a1;
  const RefSignMesh M = meshes[m];
  const uint32_t v = act[ok ? i : a1 - 1];
  const uint32_t b = v >> 9, o = v & 511;
  const int4 org = origins[b];
  const F3 q = f3(fmul(__int2float_rn(org.x + int(o >> 6)), M.h), fmul(__int2float_rn(org.y + int((o >> 3) & 7)), M.h),
                  fmul(__int2float_rn(org.z + int(o & 7)), M.h));
  Counts c;
  const float wn = ref_wn_warp(q, __ballot_sync(FULL, ok), M.root, rec_i, opn, rec_l, leaf_cnt, tri, ws[w], c);
  if (ok) {
    const float d = values[uint64_t(b) * 512 + o];
    values[uint64_t(b) * 512 + o] = (wn < M.thresh) ? copysignf(d, 1.0f) : copysignf(d, -1.0f);
  }
  flush_counts(c, counters);
}

__global__ void __launch_bounds__(32 * SIGN_WARPS) k_rt_points(const float* __restrict__ pts, uint64_t np, int root,
                                                               const float4* __restrict__ rec_i,
                                                               const float4* __restrict__ opn,
                                                               const float4* __restrict__ rec_l,
                                                               const uint32_t* __restrict__ leaf_cnt,
                                                               const float4* __restrict__ tri, float* __restrict__ out,
                                                               unsigned long long* __restrict__ counters) {
  __shared__ WarpStack ws[SIGN_WARPS];
  const int w = threadIdx.x >> 5;
  const uint64_t base = (blockIdx.x * uint64_t(SIGN_WARPS) + w) * 32;
  if (base >= np) return;  // whole warp
  const uint64_t i = base + (threadIdx.x & 31);
  const bool ok = i < np;
  const uint64_t j = ok ? i : np - 1;
  const F3 q = f3(pts[3 * j], pts[3 * j + 1], pts[3 * j + 2]);
  Counts c;
  const float wn = ref_wn_warp(q, __ballot_sync(FULL, ok), root, rec_i, opn, rec_l, leaf_cnt, tri, ws[w], c);
  if (ok) out[i] = wn;
  flush_counts(c, counters);
}

inline unsigned nblk(uint64_t n, unsigned t) { return unsigned((n + t - 1) / t); }

}  // namespace

void build_ref_trees(bs_ctx* ctx, const float4* T, uint64_t nt, int K, const uint32_t* h_tb,
                     const std::vector<float>& h_beta, RefTrees& out) {
  if (nt == 0 || K <= 0) fail(BS_ERR_EMPTY, "mesh has no triangles");
  if (nt >= (1ull << 31)) fail(BS_ERR_CAPACITY, "more than 2^31 triangles");
  cudaStream_t s = ctx->stream;
  out.nt = nt;
  out.K = K;
  DBuf<float4> obA(ctx, nt), obB(ctx, nt);
  DBuf<float> obC(ctx, nt);
  DBuf<uint32_t> perm(ctx, nt), ptmp(ctx, nt), leaf_prio(ctx, nt);
  DBuf<int> par_i(ctx, nt), par_l(ctx, nt);
  out.topo = DBuf<int2>(ctx, nt);
  out.leaf_cnt = DBuf<uint32_t>(ctx, nt);
  out.roots = DBuf<int>(ctx, K);
  BS_CUDA(cudaMemsetAsync(out.leaf_cnt.p, 0, nt * sizeof(uint32_t), s));
  BS_CUDA(cudaMemsetAsync(out.topo.p, 0xff, nt * sizeof(int2), s));
  BS_KERNEL(ctx, "k_rt_objects", (k_rt_objects<<<nblk(nt, 256), 256, 0, s>>>(T, nt, obA.p, obB.p, obC.p, perm.p)));

  DBuf<uint32_t> d_tb(ctx, K + 1), mb(ctx, 12 * uint64_t(K));
  BS_CUDA(cudaMemcpyAsync(d_tb.p, h_tb, (K + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
  BS_KERNEL(ctx, "k_rt_bounds_init", (k_rt_bounds_init<<<nblk(12 * uint64_t(K), 256), 256, 0, s>>>(mb.p, K)));
  BS_KERNEL(ctx, "k_rt_mesh_bounds", (k_rt_mesh_bounds<<<nblk(nt, 256), 256, 0, s>>>(obA.p, obB.p, obC.p, nt, d_tb.p, K, mb.p)));

  const uint32_t cap_big = uint32_t(nt / SMALL + K + 1), cap_small = uint32_t(nt / 4 + K + 1);
  DBuf<RtSeg> big[2] = {DBuf<RtSeg>(ctx, cap_big), DBuf<RtSeg>(ctx, cap_big)};
  DBuf<RtSeg> small(ctx, cap_small);
  DBuf<uint32_t> counters(ctx, 4);
  BS_CUDA(cudaMemsetAsync(counters.p, 0, 4 * sizeof(uint32_t), s));
  RtBuild B;
  B.obA = obA.p;
  B.obB = obB.p;
  B.obC = obC.p;
  B.perm = perm.p;
  B.topo = out.topo.p;
  B.par_i = par_i.p;
  B.par_l = par_l.p;
  B.roots = out.roots.p;
  B.leaf_cnt = out.leaf_cnt.p;
  B.leaf_prio = leaf_prio.p;
  B.small = small.p;
  B.counters = counters.p;
  B.cap_big = cap_big;
  B.cap_small = cap_small;
  int cur = 0;
  B.big_next = big[cur].p;
  BS_KERNEL(ctx, "k_rt_roots", (k_rt_roots<<<nblk(K, 128), 128, 0, s>>>(B, d_tb.p, K, mb.p)));
  uint32_t hc[4];
  read_back(ctx, hc, counters.p, sizeof hc);
  uint32_t n_cur = hc[0];
  std::vector<RtSeg> hs;
  for (int level = 0; n_cur > 0; ++level) {
    if (level > MAX_DEPTH || hc[2]) fail(BS_ERR_CAPACITY, "reference tree build: node lists overflowed");
    hs.resize(n_cur);
    read_back(ctx, hs.data(), big[cur].p, n_cur * sizeof(RtSeg));
    std::vector<RtChunk> chunks;
    for (uint32_t k = 0; k < n_cur; ++k)
      for (uint32_t b0 = hs[k].first; b0 < hs[k].first + hs[k].count; b0 += CHUNK)
        chunks.push_back(RtChunk{k, b0, std::min(b0 + CHUNK, hs[k].first + hs[k].count)});
    const uint32_t nch = uint32_t(chunks.size());
    DBuf<RtChunk> d_ch(ctx, nch);
    BS_CUDA(cudaMemcpyAsync(d_ch.p, chunks.data(), nch * sizeof(RtChunk), cudaMemcpyHostToDevice, s));
    DBuf<uint32_t> bk(ctx, uint64_t(n_cur) * BKW), cb(ctx, 24 * uint64_t(n_cur)), cursor(ctx, 2 * uint64_t(n_cur));
    DBuf<RtDec> dec(ctx, n_cur);
    BS_KERNEL(ctx, "k_rt_bins_init", (k_rt_bins_init<<<nblk(uint64_t(n_cur) * BKW, 256), 256, 0, s>>>(bk.p, uint64_t(n_cur) * BKW)));
    BS_KERNEL(ctx, "k_rt_bins", (k_rt_bins<<<nch, 256, 0, s>>>(d_ch.p, big[cur].p, perm.p, obA.p, obB.p, obC.p, bk.p)));
    BS_KERNEL(ctx, "k_rt_decide", (k_rt_decide<<<nblk(n_cur, 128), 128, 0, s>>>(big[cur].p, n_cur, bk.p, dec.p, cb.p, cursor.p)));
    BS_KERNEL(ctx, "k_rt_place", (k_rt_place<<<nch, 256, 0, s>>>(d_ch.p, big[cur].p, dec.p, perm.p, ptmp.p, obA.p, obB.p, obC.p, cb.p, cursor.p)));
    BS_KERNEL(ctx, "k_rt_copyback", (k_rt_copyback<<<nch, 256, 0, s>>>(d_ch.p, dec.p, ptmp.p, perm.p)));
    BS_CUDA(cudaMemsetAsync(counters.p, 0, sizeof(uint32_t), s));
    B.big_next = big[cur ^ 1].p;
    BS_KERNEL(ctx, "k_rt_children", (k_rt_children<<<nblk(n_cur, 128), 128, 0, s>>>(B, big[cur].p, n_cur, dec.p, cb.p, cursor.p)));
    read_back(ctx, hc, counters.p, sizeof hc);
    n_cur = hc[0];
    cur ^= 1;
  }
  if (hc[2]) fail(BS_ERR_CAPACITY, "reference tree build: node lists overflowed");
  const uint32_t n_small = hc[1];
  if (n_small) BS_KERNEL(ctx, "k_rt_small", (k_rt_small<<<n_small, ST_THREADS, 0, s>>>(B)));
  DBuf<uint32_t> big_leaves(ctx, nt / (LEAF_SORT_THREAD + 1) + 1);
  BS_KERNEL(ctx, "k_rt_leaf_sort", (k_rt_leaf_sort<<<nblk(nt, 256), 256, 0, s>>>(nt, out.leaf_cnt.p, leaf_prio.p, perm.p, obA.p, obB.p, obC.p,
                                                                              big_leaves.p, counters.p + 3)));
  read_back(ctx, hc, counters.p, sizeof hc);
  if (hc[2] == 2) fail(BS_ERR_CUDA, "reference tree build: inconsistent partition");
  if (hc[2]) fail(BS_ERR_CAPACITY, "reference tree build: node lists overflowed");
  if (hc[3]) BS_KERNEL(ctx, "k_rt_leaf_sort_big", (k_rt_leaf_sort_big<<<hc[3], 256, 0, s>>>(big_leaves.p, out.leaf_cnt.p, leaf_prio.p, perm.p, ptmp.p,
                                                                                          obA.p, obB.p, obC.p)));
  obA.reset();
  obB.reset();
  obC.reset();
  out.tri = DBuf<float4>(ctx, 3 * nt);
  BS_KERNEL(ctx, "k_rt_tri", (k_rt_tri<<<nblk(nt, 256), 256, 0, s>>>(T, perm.p, nt, out.tri.p)));
  out.rec_i = DBuf<float4>(ctx, 4 * nt);
  out.rec_l = DBuf<float4>(ctx, 4 * nt);
  out.rad_i = DBuf<float>(ctx, nt);
  out.rad_l = DBuf<float>(ctx, nt);
  out.flags = DBuf<int>(ctx, nt);
  {
    DBuf<float4> ld_i(ctx, 6 * nt), ld_l(ctx, 6 * nt);
    BS_CUDA(cudaMemsetAsync(out.flags.p, 0, nt * sizeof(int), s));
    BS_KERNEL(ctx, "k_rt_refit", (k_rt_refit<<<nblk(nt, 128), 128, 0, s>>>(nt, out.leaf_cnt.p, out.tri.p, out.topo.p, par_i.p, par_l.p,
                                                                         out.flags.p, ld_i.p, ld_l.p, out.rec_i.p, out.rec_l.p,
                                                                         out.rad_i.p, out.rad_l.p)));
    out.h_roots.resize(K);
    read_back(ctx, out.h_roots.data(), out.roots.p, K * sizeof(int));
  }
  out.tb = std::move(d_tb);
  out.h_beta.clear();
  ref_tree_set_beta(ctx, out, h_beta);
}

void ref_tree_set_beta(bs_ctx* ctx, RefTrees& t, const std::vector<float>& beta) {
  if (int(beta.size()) != t.K) fail(BS_ERR_INVALID_ARG, "one beta per mesh");
  if (beta == t.h_beta) return;
  DBuf<float> d_beta(ctx, t.K);
  BS_CUDA(cudaMemcpyAsync(d_beta.p, beta.data(), t.K * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  BS_KERNEL(ctx, "k_rt_tau", (k_rt_tau<<<nblk(t.nt, 256), 256, 0, ctx->stream>>>(t.nt, t.tb.p, t.K, d_beta.p, t.leaf_cnt.p, t.flags.p,
                                                                             t.rad_i.p, t.rad_l.p, t.rec_i.p, t.rec_l.p)));
  if (!t.open.p) t.open = DBuf<float4>(ctx, 3 * t.nt);
  BS_KERNEL(ctx, "k_rt_open", (k_rt_open<<<nblk(t.nt, 256), 256, 0, ctx->stream>>>(t.nt, t.flags.p, t.topo.p, t.leaf_cnt.p, t.rec_i.p,
                                                                               t.rec_l.p, t.open.p)));
  t.h_beta = beta;
}

void ref_tree_sign(bs_ctx* ctx, const RefTrees& t, const uint32_t* act, const uint32_t* d_act_base,
                   const uint32_t* d_warp_base, uint64_t n_warps, int K, const RefSignMesh* d_meshes,
                   const int4* origins, float* values, unsigned long long* d_counters) {
  if (n_warps == 0) return;
#define BS_RT_SIGN(W)                                                                                        \
  BS_KERNEL(ctx, "k_rt_sign", (k_rt_sign<W><<<nblk(n_warps, W), 32 * W, 0, ctx->stream>>>(                   \
                                  act, d_act_base, d_warp_base, K, d_meshes, origins, values, t.rec_i.p, t.open.p, \
                                  t.rec_l.p, t.leaf_cnt.p, t.tri.p, d_counters)))
  if (ctx->tune_wn_warps == 2)
    BS_RT_SIGN(2);
  else if (ctx->tune_wn_warps == 8)
    BS_RT_SIGN(8);
  else
    BS_RT_SIGN(4);
#undef BS_RT_SIGN
}

void ref_tree_points(bs_ctx* ctx, RefTrees& t, const float* d_pts, uint64_t np, float beta, float* d_out,
                     unsigned long long* d_counters) {
  if (np == 0) return;
  ref_tree_set_beta(ctx, t, std::vector<float>(1, beta));
  BS_KERNEL(ctx, "k_rt_points", (k_rt_points<<<nblk(np, 32 * SIGN_WARPS), 32 * SIGN_WARPS, 0, ctx->stream>>>(
                                    d_pts, np, t.h_roots[0], t.rec_i.p, t.open.p, t.rec_l.p, t.leaf_cnt.p,
                                    t.tri.p, d_out, d_counters)));
}

}  // namespace bs
