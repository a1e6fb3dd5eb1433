// CornerTable from a triangle soup: CornerTable::builder_soup().finish()
// (mesh/corner_table/builder.rs:292-309) on top of the GPU.
//
//  * merge_points (algo/merge_points.rs:12-41) on the GPU: exactly equal
//    points (-0 == +0, NaN never equal) get one vertex, numbered in order of
//    first appearance — three stable radix sorts on the coordinate bits, a
//    group scan, and a scan over the first occurrences;
//  * the indexed build (builder.rs:168-262) on the GPU: faces in order, a
//    face that repeats a directed edge of an earlier taken face is skipped,
//    then isolated vertices are deleted and every extra corner fan of a
//    vertex gets its own copy (see corner_table_from_device_soup).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cstring>

#include "bs_internal.cuh"

struct bs_corner_table {
  std::vector<float> pos;             // [slots][3]
  std::vector<uint8_t> deleted;       // [slots]
  std::vector<int32_t> vcorner;       // [slots] -1 none
  std::vector<int32_t> cvertex;       // [corners]
  std::vector<int32_t> copp;          // [corners] -1 none
};

namespace bs {

static inline unsigned nbc(uint64_t n, unsigned t) { return unsigned((n + t - 1) / t); }

__device__ __forceinline__ uint32_t key_bits(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x7fffffffu) == 0 ? 0u : u;  // -0 == +0
}

__global__ void k_point_keys(const float* __restrict__ p, uint64_t n, int axis, uint32_t* __restrict__ key,
                             uint32_t* __restrict__ idx, int init) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const uint32_t j = init ? uint32_t(i) : idx[i];
  const float x = p[3 * uint64_t(j)], y = p[3 * uint64_t(j) + 1], z = p[3 * uint64_t(j) + 2];
  const bool nan = isnan(x) || isnan(y) || isnan(z);
  uint32_t k;
  if (nan)  // a NaN point equals nothing: make its key unique
    k = axis == 2 ? j : 0xffffffffu;
  else
    k = key_bits(axis == 0 ? x : (axis == 1 ? y : z));
  key[i] = k;
  if (init) idx[i] = j;
}

__global__ void k_group_starts(const float* __restrict__ p, const uint32_t* __restrict__ idx, uint64_t n,
                               uint32_t* __restrict__ start_sorted, uint32_t* __restrict__ is_rep) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const uint32_t j = idx[i];
  bool start = (i == 0);
  if (!start) {
    const float* a = p + 3 * uint64_t(j);
    const float* b = p + 3 * uint64_t(idx[i - 1]);
    // PartialEq on the coordinates: == on floats (NaN never equal, -0 == +0)
    start = !(a[0] == b[0] && a[1] == b[1] && a[2] == b[2]);
  }
  start_sorted[i] = start ? 1u : 0u;
  // the stable sorts started from identity order, so a group's first element
  // is its first occurrence in the soup
  is_rep[j] = start ? 1u : 0u;
}

__global__ void k_group_first(const uint32_t* __restrict__ idx, const uint32_t* __restrict__ start_sorted,
                              const uint32_t* __restrict__ gid, uint64_t n, uint32_t* __restrict__ group_rep) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i < n && start_sorted[i]) group_rep[gid[i] - 1] = idx[i];
}

__global__ void k_point_ids(const uint32_t* __restrict__ idx, const uint32_t* __restrict__ gid,
                            const uint32_t* __restrict__ group_rep, const uint32_t* __restrict__ newid, uint64_t n,
                            uint32_t* __restrict__ out_id) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  out_id[idx[i]] = newid[group_rep[gid[i] - 1]];
}

__global__ void k_unique_points(const float* __restrict__ p, const uint32_t* __restrict__ is_rep,
                                const uint32_t* __restrict__ newid, uint64_t n, float* __restrict__ out) {
  const uint64_t j = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (j >= n || !is_rep[j]) return;
  const uint32_t d = newid[j];
  out[3 * uint64_t(d)] = p[3 * j];
  out[3 * uint64_t(d) + 1] = p[3 * j + 1];
  out[3 * uint64_t(d) + 2] = p[3 * j + 2];
}

// merge_points on device points d_p[n][3]: ids[n] and the nu unique points, on the device.
static void merge_points_gpu(bs_ctx* ctx, const float* d_p, uint64_t n, DBuf<uint32_t>& ids, DBuf<float>& uniq,
                             uint32_t& nu) {
  cudaStream_t s = ctx->stream;
  nu = 0;
  if (n == 0) return;
  if (n >= (1ull << 31)) fail(BS_ERR_CAPACITY, "more than 2^31 soup points");
  DBuf<uint32_t> key(ctx, n), key2(ctx, n), idx(ctx, n), idx2(ctx, n);
  size_t tmp = 0;
  BS_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, key.p, key2.p, idx.p, idx2.p, int(n), 0, 32, s));
  DBuf<uint8_t> t(ctx, tmp);
  // LSD over (z, y, x): stable sorts give lexicographic (x, y, z), ties in original order
  for (int pass = 0; pass < 3; ++pass) {
    const int axis = 2 - pass;
    BS_KERNEL(ctx, "k_point_keys", (k_point_keys<<<nbc(n, 256), 256, 0, s>>>(d_p, n, axis, key.p, idx.p, pass == 0)));
    BS_CUDA(cub::DeviceRadixSort::SortPairs(t.p, tmp, key.p, key2.p, idx.p, idx2.p, int(n), 0, 32, s));
    std::swap(idx.p, idx2.p);
  }
  DBuf<uint32_t> start(ctx, n), gid(ctx, n), is_rep(ctx, n + 1), newid(ctx, n + 1), group_rep(ctx, n), id(ctx, n);
  BS_CUDA(cudaMemsetAsync(is_rep.p + n, 0, sizeof(uint32_t), s));
  BS_KERNEL(ctx, "k_group_starts", (k_group_starts<<<nbc(n, 256), 256, 0, s>>>(d_p, idx.p, n, start.p, is_rep.p)));
  {
    size_t t2 = 0;
    BS_CUDA(cub::DeviceScan::InclusiveSum(nullptr, t2, start.p, gid.p, n, s));
    DBuf<uint8_t> tt(ctx, t2);
    BS_CUDA(cub::DeviceScan::InclusiveSum(tt.p, t2, start.p, gid.p, n, s));
  }
  {
    size_t t3 = 0;
    BS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, t3, is_rep.p, newid.p, n + 1, s));
    DBuf<uint8_t> tt(ctx, t3);
    BS_CUDA(cub::DeviceScan::ExclusiveSum(tt.p, t3, is_rep.p, newid.p, n + 1, s));
  }
  BS_KERNEL(ctx, "k_group_first", (k_group_first<<<nbc(n, 256), 256, 0, s>>>(idx.p, start.p, gid.p, n, group_rep.p)));
  BS_KERNEL(ctx, "k_point_ids", (k_point_ids<<<nbc(n, 256), 256, 0, s>>>(idx.p, gid.p, group_rep.p, newid.p, n, id.p)));
  read_back(ctx, &nu, newid.p + n, sizeof(uint32_t));
  DBuf<float> up(ctx, uint64_t(nu) * 3);
  BS_KERNEL(ctx, "k_unique_points", (k_unique_points<<<nbc(n, 256), 256, 0, s>>>(d_p, is_rep.p, newid.p, n, up.p)));
  ids = std::move(id);
  uniq = std::move(up);
}

// ------------------------------------------------------ indexed build ----
// builder.rs:168-262 on the merged points, on the GPU.
//
// Faces are taken in order and a face is skipped when one of its directed
// edges (v2, v3), (v3, v1), (v1, v2) already belongs to an earlier taken
// face.  So a face is taken exactly when no earlier face sharing one of its
// directed edges was taken: the lexicographically first maximal independent
// set of the "shares a directed edge" graph.  The half-edges are sorted by
// key (stable, so a key's run lists faces in order); a face none of whose
// keys repeats is taken at once, the others decide in rounds — a face is
// skipped as soon as an earlier face in one of its runs is taken, and taken
// once every earlier face in its runs is skipped.  Each decision is final, so
// the result does not depend on scheduling.  Taken faces get corners
// 3r, 3r + 1, 3r + 2 (r their rank) with vertices v1, v2, v3, the
// corner_from order; the corner opposite edge (x, y) pairs with the taken
// half-edge (y, x) (for a key (x, x), only possible in a degenerate face, in
// the chain the insertion order leaves: each with the next, the last with the
// one before).  A vertex's corner is its highest (the last assigned); a
// vertex without one is deleted.  Then per vertex the fan around its corner
// stays, and every other fan, taken in order of its smallest corner, becomes
// a new vertex (numbered after all earlier vertices' new ones, in vertex
// order as the oracle's restatement numbers them).
namespace {

constexpr uint8_t F_OPEN = 0, F_TAKEN = 1, F_SKIPPED = 2;

__device__ __forceinline__ int32_t cnext_d(int32_t c) { return (c % 3 == 2) ? c - 2 : c + 1; }
__device__ __forceinline__ int32_t cprev_d(int32_t c) { return (c % 3 == 0) ? c + 2 : c - 1; }

__global__ void k_half_keys(const uint32_t* __restrict__ ids, uint64_t nf, unsigned long long* __restrict__ key,
                            uint32_t* __restrict__ half) {
  const uint64_t f = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (f >= nf) return;
  const uint32_t a = ids[3 * f], b = ids[3 * f + 1], c = ids[3 * f + 2];
  const uint32_t x[3] = {b, c, a}, y[3] = {c, a, b};  // edges of corner_from(b,c,a), (c,a,b), (a,b,c)
  for (int k = 0; k < 3; ++k) {
    key[3 * f + k] = (static_cast<unsigned long long>(x[k]) << 32) | y[k];
    half[3 * f + k] = uint32_t(3 * f + k);
  }
}

// run_head[i]: i where a run of equal keys starts, else 0 (max-scanned into run starts)
__global__ void k_half_runs(const unsigned long long* __restrict__ key, const uint32_t* __restrict__ half,
                            uint64_t n, uint32_t* __restrict__ head, uint32_t* __restrict__ pos_of,
                            uint8_t* __restrict__ shared_key) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const bool first = i == 0 || key[i] != key[i - 1];
  const bool last = i + 1 == n || key[i + 1] != key[i];
  head[i] = first ? uint32_t(i) : 0u;
  pos_of[half[i]] = uint32_t(i);
  if (!(first && last)) shared_key[half[i] / 3] = 1;  // benign race: every writer writes 1
}

struct MaxU32 {
  __device__ __forceinline__ uint32_t operator()(uint32_t a, uint32_t b) const { return a > b ? a : b; }
};

__global__ void k_face_init(const uint8_t* __restrict__ shared_key, uint64_t nf, uint8_t* __restrict__ state) {
  const uint64_t f = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (f < nf) state[f] = shared_key[f] ? F_OPEN : F_TAKEN;
}

// One round over the open faces.
__global__ void k_face_round(const uint32_t* __restrict__ half, const uint32_t* __restrict__ run_start,
                             const uint32_t* __restrict__ pos_of, uint64_t nf, uint8_t* __restrict__ state,
                             unsigned long long* __restrict__ open_left) {
  const uint64_t f = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (f >= nf) return;
  if (__ldcg(state + f) != F_OPEN) return;
  bool pending = false;
  for (int k = 0; k < 3; ++k) {
    const uint32_t i = pos_of[3 * f + k];
    for (uint32_t j = run_start[i]; j < i; ++j) {
      const uint64_t g = half[j] / 3;
      if (g == f) continue;  // a face's own repeated key never excludes it
      const uint8_t sg = __ldcg(state + g);
      if (sg == F_TAKEN) {
        state[f] = F_SKIPPED;
        return;
      }
      if (sg == F_OPEN) pending = true;
    }
  }
  if (pending) atomicAdd(open_left, 1ull);
  else state[f] = F_TAKEN;
}

__global__ void k_taken_flags(const uint8_t* __restrict__ state, uint64_t nf, uint32_t* __restrict__ flag) {
  const uint64_t f = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (f <= nf) flag[f] = (f < nf && state[f] == F_TAKEN) ? 1u : 0u;
}

__global__ void k_corner_vertices(const uint32_t* __restrict__ ids, const uint8_t* __restrict__ state,
                                  const uint32_t* __restrict__ rank, uint64_t nf, int32_t* __restrict__ cvertex,
                                  int32_t* __restrict__ vcorner) {
  const uint64_t f = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (f >= nf || state[f] != F_TAKEN) return;
  const uint64_t c0 = 3 * uint64_t(rank[f]);
  for (int k = 0; k < 3; ++k) {
    const uint32_t v = ids[3 * f + k];
    cvertex[c0 + k] = int32_t(v);
    atomicMax(vcorner + v, int32_t(c0 + k));  // the last corner assigned to the vertex
  }
}

// First position of key k in the sorted keys, or n.
__device__ __forceinline__ uint64_t lower_bound_key(const unsigned long long* __restrict__ key, uint64_t n,
                                                    unsigned long long k) {
  uint64_t lo = 0, hi = n;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (key[mid] < k) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__global__ void k_opposites(const unsigned long long* __restrict__ key, const uint32_t* __restrict__ half,
                            const uint32_t* __restrict__ pos_of, const uint8_t* __restrict__ state,
                            const uint32_t* __restrict__ rank, uint64_t nf, int32_t* __restrict__ copp) {
  const uint64_t h = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (h >= 3 * nf) return;
  const uint64_t f = h / 3;
  if (state[f] != F_TAKEN) return;
  const uint64_t n = 3 * nf;
  const unsigned long long k = key[pos_of[h]];
  const uint32_t x = uint32_t(k >> 32), y = uint32_t(k);
  const int32_t me = int32_t(3 * uint64_t(rank[f]) + h % 3);
  int32_t opp = -1;
  if (x != y) {
    const unsigned long long rk = (static_cast<unsigned long long>(y) << 32) | x;
    for (uint64_t j = lower_bound_key(key, n, rk); j < n && key[j] == rk; ++j) {
      const uint64_t g = half[j] / 3;
      if (state[g] == F_TAKEN) {
        opp = int32_t(3 * uint64_t(rank[g]) + half[j] % 3);
        break;
      }
    }
  } else {
    // a self-reversed key: the taken half-edges of this run, in insertion order
    int32_t prev = -1, next = -1;
    bool seen_me = false;
    for (uint64_t j = lower_bound_key(key, n, k); j < n && key[j] == k; ++j) {
      const uint64_t g = half[j] / 3;
      if (state[g] != F_TAKEN) continue;
      const int32_t c = int32_t(3 * uint64_t(rank[g]) + half[j] % 3);
      if (c == me) {
        seen_me = true;
        continue;
      }
      if (!seen_me) {
        prev = c;
      } else {
        next = c;
        break;
      }
    }
    opp = next >= 0 ? next : prev;  // linked to the next one, the last to the one before
  }
  copp[me] = opp;
}

__global__ void k_deleted(const int32_t* __restrict__ vcorner, uint64_t nv, uint8_t* __restrict__ deleted) {
  const uint64_t v = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (v < nv) deleted[v] = vcorner[v] < 0 ? 1 : 0;
}

// corners_around_vertex (traversal.rs:244-286) from corner c0: visit(c) for
// every corner of the fan.  Every visited corner belongs to c0's vertex: a
// corner's opposite lies across the same edge, reversed, or across the same
// degenerate edge (x, x).  The walk's state is one of the vertex's corners, so
// a walk that has not ended after deg + 1 steps is in a cycle that misses its
// start and has already visited all it ever will: guard_max = deg + 2 visits
// the same set as an unbounded walk.
template <class F>
__device__ void fan_around(const int32_t* __restrict__ copp, int32_t c0, uint32_t guard_max, F visit) {
  int32_t w = cprev_d(c0);
  const int32_t started = w;
  bool border = false;
  for (uint32_t g = 0; g < guard_max; ++g) {
    visit(cnext_d(w));
    w = cprev_d(w);
    if (copp[w] < 0) {
      border = true;
      break;
    }
    w = copp[w];
    if (w == started) break;
  }
  w = started;
  if (border && copp[w] >= 0) {
    w = copp[w];
    for (uint32_t g = 0; g < guard_max; ++g) {
      visit(cprev_d(w));
      w = cnext_d(w);
      if (copp[w] < 0) break;
      w = copp[w];
    }
  }
}

// Pass 1 per vertex (builder.rs:224-262, finish): the fan around the vertex's
// corner keeps the vertex (fan 0); then, while one of its corners is in no fan
// yet, the smallest such corner seeds a new vertex and every corner of that
// seed's fan moves to it, including corners an earlier fan had taken (a walk
// around a non-manifold vertex can cross fans).  fan[c] = the last fan that
// visited c; seed[vstart[v] + k - 1] = the corner of fan k, the new vertex's
// corner.
__global__ void k_fans(const int32_t* __restrict__ vcorner, const uint8_t* __restrict__ deleted,
                       const uint32_t* __restrict__ vstart, const int32_t* __restrict__ vlist,
                       const int32_t* __restrict__ copp, uint64_t nv, int32_t* __restrict__ fan,
                       int32_t* __restrict__ seed, uint32_t* __restrict__ extra) {
  const uint64_t v = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (v > nv) return;
  if (v == nv) {
    extra[nv] = 0;
    return;
  }
  uint32_t nfan = 0;
  if (!deleted[v]) {
    const uint32_t b = vstart[v], e = vstart[v + 1], guard = e - b + 2;
    for (uint32_t j = b; j < e; ++j) fan[vlist[j]] = -1;
    fan_around(copp, vcorner[v], guard, [&](int32_t c) { fan[c] = 0; });
    for (uint32_t j = b; j < e; ++j) {
      const int32_t ci = vlist[j];
      if (fan[ci] >= 0) continue;
      seed[b + nfan] = ci;
      ++nfan;
      fan_around(copp, ci, guard, [&](int32_t c) { fan[c] = int32_t(nfan); });
    }
  }
  extra[v] = nfan;
}

// Pass 2 per vertex: the new vertices of its extra fans (builder.rs:247,
// add_vertex at the vertex's position with the seed as its corner).
__global__ void k_split(const uint8_t* deleted, const uint32_t* __restrict__ vstart,
                        const int32_t* __restrict__ vlist, const int32_t* __restrict__ fan,
                        const int32_t* __restrict__ seed, const uint32_t* __restrict__ extra_off, uint64_t nv,
                        float* __restrict__ pos, int32_t* __restrict__ vcorner, uint8_t* del_out,
                        int32_t* __restrict__ cvertex) {
  const uint64_t v = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (v >= nv || deleted[v]) return;
  const uint32_t base = uint32_t(nv) + extra_off[v], n_extra = extra_off[v + 1] - extra_off[v];
  if (n_extra == 0) return;
  for (uint32_t j = vstart[v]; j < vstart[v + 1]; ++j) {
    const int32_t c = vlist[j];
    const int32_t k = fan[c];
    if (k > 0) cvertex[c] = int32_t(base + uint32_t(k) - 1);
  }
  for (uint32_t k = 0; k < n_extra; ++k) {
    const uint32_t nvx = base + k;
    vcorner[nvx] = seed[vstart[v] + k];
    del_out[nvx] = 0;
    pos[3 * uint64_t(nvx)] = pos[3 * v];
    pos[3 * uint64_t(nvx) + 1] = pos[3 * v + 1];
    pos[3 * uint64_t(nvx) + 2] = pos[3 * v + 2];
  }
}

__global__ void k_corner_keys(const int32_t* __restrict__ cvertex, uint64_t nc, uint32_t* __restrict__ key,
                              int32_t* __restrict__ val) {
  const uint64_t c = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (c >= nc) return;
  key[c] = uint32_t(cvertex[c]);
  val[c] = int32_t(c);
}

__global__ void k_vertex_counts(const int32_t* __restrict__ cvertex, uint64_t nc, uint32_t* __restrict__ cnt) {
  const uint64_t c = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (c < nc) atomicAdd(cnt + cvertex[c], 1u);
}

template <class T>
void scan_ex(bs_ctx* ctx, const T* in, T* out, uint64_t n) {
  size_t tmp = 0;
  BS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, in, out, n, ctx->stream));
  DBuf<uint8_t> t(ctx, tmp);
  BS_CUDA(cub::DeviceScan::ExclusiveSum(t.p, tmp, in, out, n, ctx->stream));
}

}  // namespace

bs_corner_table* corner_table_from_device_soup(bs_ctx* ctx, const float* d_pts, uint64_t n_points) {
  cudaStream_t s = ctx->stream;
  DBuf<uint32_t> ids;
  DBuf<float> uniq;
  uint32_t nu = 0;
  merge_points_gpu(ctx, d_pts, n_points, ids, uniq, nu);
  auto* t = new bs_corner_table();
  const uint64_t nf = n_points / 3, nv = nu;
  if (nf == 0) {
    t->pos.resize(uint64_t(nu) * 3);
    if (nu) BS_CUDA(cudaMemcpy(t->pos.data(), uniq.p, uint64_t(nu) * 3 * sizeof(float), cudaMemcpyDeviceToHost));
    t->deleted.assign(nu, 1);
    t->vcorner.assign(nu, -1);
    return t;
  }
  const uint64_t nh = 3 * nf;
  // faces taken or skipped (builder.rs:186-194)
  DBuf<unsigned long long> key(ctx, nh), skey(ctx, nh);
  DBuf<uint32_t> half(ctx, nh), shalf(ctx, nh);
  BS_KERNEL(ctx, "k_half_keys", (k_half_keys<<<nbc(nf, 256), 256, 0, s>>>(ids.p, nf, key.p, half.p)));
  {
    size_t tmp = 0;
    BS_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, key.p, skey.p, half.p, shalf.p, int(nh), 0, 64, s));
    DBuf<uint8_t> tb(ctx, tmp);
    BS_CUDA(cub::DeviceRadixSort::SortPairs(tb.p, tmp, key.p, skey.p, half.p, shalf.p, int(nh), 0, 64, s));
  }
  key.reset();
  half.reset();
  DBuf<uint32_t> head(ctx, nh), run_start(ctx, nh), pos_of(ctx, nh);
  DBuf<uint8_t> shared_key(ctx, nf), state(ctx, nf);
  BS_CUDA(cudaMemsetAsync(shared_key.p, 0, nf, s));
  BS_KERNEL(ctx, "k_half_runs", (k_half_runs<<<nbc(nh, 256), 256, 0, s>>>(skey.p, shalf.p, nh, head.p, pos_of.p, shared_key.p)));
  {
    size_t tmp = 0;
    BS_CUDA(cub::DeviceScan::InclusiveScan(nullptr, tmp, head.p, run_start.p, MaxU32(), nh, s));
    DBuf<uint8_t> tb(ctx, tmp);
    BS_CUDA(cub::DeviceScan::InclusiveScan(tb.p, tmp, head.p, run_start.p, MaxU32(), nh, s));
  }
  head.reset();
  BS_KERNEL(ctx, "k_face_init", (k_face_init<<<nbc(nf, 256), 256, 0, s>>>(shared_key.p, nf, state.p)));
  {
    DBuf<unsigned long long> left(ctx, 1);
    for (uint64_t round = 0;; ++round) {
      if (round > nf + 1) fail(BS_ERR_CAPACITY, "corner table: face rounds did not settle");
      BS_CUDA(cudaMemsetAsync(left.p, 0, sizeof(unsigned long long), s));
      BS_KERNEL(ctx, "k_face_round", (k_face_round<<<nbc(nf, 256), 256, 0, s>>>(shalf.p, run_start.p, pos_of.p, nf, state.p, left.p)));
      unsigned long long h = 0;
      read_back(ctx, &h, left.p, sizeof h);
      if (h == 0) break;
    }
  }
  DBuf<uint32_t> flag(ctx, nf + 1), rank(ctx, nf + 1);
  BS_KERNEL(ctx, "k_taken_flags", (k_taken_flags<<<nbc(nf + 1, 256), 256, 0, s>>>(state.p, nf, flag.p)));
  scan_ex(ctx, flag.p, rank.p, nf + 1);
  uint32_t n_taken = 0;
  read_back(ctx, &n_taken, rank.p + nf, sizeof n_taken);
  const uint64_t nc = 3 * uint64_t(n_taken);
  // corners, opposites, vertex corners (builder.rs:196-208, corner_from)
  DBuf<int32_t> cvertex(ctx, nc), copp(ctx, nc), vcorner(ctx, nv + nc);
  BS_CUDA(cudaMemsetAsync(vcorner.p, 0xff, (nv + nc) * sizeof(int32_t), s));
  if (nc) {
    BS_KERNEL(ctx, "k_corner_vertices", (k_corner_vertices<<<nbc(nf, 256), 256, 0, s>>>(ids.p, state.p, rank.p, nf, cvertex.p, vcorner.p)));
    BS_KERNEL(ctx, "k_opposites", (k_opposites<<<nbc(nh, 256), 256, 0, s>>>(skey.p, shalf.p, pos_of.p, state.p, rank.p, nf, copp.p)));
  }
  skey.reset();
  shalf.reset();
  pos_of.reset();
  run_start.reset();
  // finish (builder.rs:224-262): isolated vertices, extra fans
  DBuf<uint8_t> deleted(ctx, nv + nc);
  BS_KERNEL(ctx, "k_deleted", (k_deleted<<<nbc(nv, 256), 256, 0, s>>>(vcorner.p, nv, deleted.p)));
  DBuf<float> pos(ctx, (nv + nc) * 3);
  if (nv) BS_CUDA(cudaMemcpyAsync(pos.p, uniq.p, nv * 3 * sizeof(float), cudaMemcpyDeviceToDevice, s));
  uint32_t n_extra = 0;
  if (nc) {
    DBuf<uint32_t> vcnt(ctx, nv + 1), vstart(ctx, nv + 1), ckey(ctx, nc), ckey2(ctx, nc);
    DBuf<int32_t> cval(ctx, nc), vlist(ctx, nc), fan(ctx, nc);
    // corners of every vertex in increasing order (a stable sort by vertex)
    BS_CUDA(cudaMemsetAsync(vcnt.p, 0, (nv + 1) * sizeof(uint32_t), s));
    BS_KERNEL(ctx, "k_vertex_counts", (k_vertex_counts<<<nbc(nc, 256), 256, 0, s>>>(cvertex.p, nc, vcnt.p)));
    scan_ex(ctx, vcnt.p, vstart.p, nv + 1);
    BS_KERNEL(ctx, "k_corner_keys", (k_corner_keys<<<nbc(nc, 256), 256, 0, s>>>(cvertex.p, nc, ckey.p, cval.p)));
    {
      int bits = 1;
      while ((uint64_t(1) << bits) < nv) ++bits;
      size_t tmp = 0;
      BS_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, ckey.p, ckey2.p, cval.p, vlist.p, int(nc), 0, bits, s));
      DBuf<uint8_t> tb(ctx, tmp);
      BS_CUDA(cub::DeviceRadixSort::SortPairs(tb.p, tmp, ckey.p, ckey2.p, cval.p, vlist.p, int(nc), 0, bits, s));
    }
    DBuf<uint32_t> extra(ctx, nv + 1), extra_off(ctx, nv + 1);
    BS_KERNEL(ctx, "k_fans", (k_fans<<<nbc(nv + 1, 128), 128, 0, s>>>(vcorner.p, deleted.p, vstart.p, vlist.p, copp.p, nv, fan.p,
                                                                   cval.p, extra.p)));
    scan_ex(ctx, extra.p, extra_off.p, nv + 1);
    read_back(ctx, &n_extra, extra_off.p + nv, sizeof n_extra);
    if (n_extra)
      BS_KERNEL(ctx, "k_split", (k_split<<<nbc(nv, 128), 128, 0, s>>>(deleted.p, vstart.p, vlist.p, fan.p, cval.p, extra_off.p, nv, pos.p,
                                                                    vcorner.p, deleted.p, cvertex.p)));
  }
  const uint64_t slots = nv + n_extra;
  t->pos.resize(slots * 3);
  t->deleted.resize(slots);
  t->vcorner.resize(slots);
  t->cvertex.resize(nc);
  t->copp.resize(nc);
  if (slots) {
    BS_CUDA(cudaMemcpyAsync(t->pos.data(), pos.p, slots * 3 * sizeof(float), cudaMemcpyDeviceToHost, s));
    BS_CUDA(cudaMemcpyAsync(t->deleted.data(), deleted.p, slots, cudaMemcpyDeviceToHost, s));
    BS_CUDA(cudaMemcpyAsync(t->vcorner.data(), vcorner.p, slots * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  }
  if (nc) {
    BS_CUDA(cudaMemcpyAsync(t->cvertex.data(), cvertex.p, nc * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    BS_CUDA(cudaMemcpyAsync(t->copp.data(), copp.p, nc * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  }
  BS_CUDA(cudaStreamSynchronize(s));
  return t;
}

}  // namespace bs

extern "C" {

bs_status bs_corner_table_from_soup(bs_ctx* ctx, const float* h_tris, uint64_t n_tris, bs_corner_table** out) {
  if (!ctx || !out || (n_tris && !h_tris)) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  try {
    BS_CUDA(cudaSetDevice(ctx->device));
    bs::DBuf<float> d(ctx, n_tris * 9);
    if (n_tris) BS_CUDA(cudaMemcpyAsync(d.p, h_tris, n_tris * 9 * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    *out = bs::corner_table_from_device_soup(ctx, d.p, n_tris * 3);
    return BS_OK;
  } catch (const bs::Error& e) {
    ctx->last_error = e.msg;
    return e.status;
  } catch (const std::bad_alloc&) {
    return BS_ERR_OOM;
  }
}

bs_status bs_corner_table_from_dual_contour(bs_ctx* ctx, bs_volume* v, float voxel_size, bs_corner_table** out) {
  if (!ctx || !v || !out || v->ctx != ctx) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  try {
    BS_CUDA(cudaSetDevice(ctx->device));
    bs::dual_contour_impl(ctx, v, voxel_size);
    *out = bs::corner_table_from_device_soup(ctx, v->d_dc_tris, v->n_dc_tris * 3);
    return BS_OK;
  } catch (const bs::Error& e) {
    ctx->last_error = e.msg;
    return e.status;
  } catch (const std::bad_alloc&) {
    return BS_ERR_OOM;
  }
}

bs_status bs_corner_table_from_marching_cubes(bs_ctx* ctx, bs_volume* v, float voxel_size, bs_corner_table** out) {
  if (!ctx || !v || !out || v->ctx != ctx) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  try {
    BS_CUDA(cudaSetDevice(ctx->device));
    bs::marching_cubes_impl(ctx, v, voxel_size);
    *out = bs::corner_table_from_device_soup(ctx, v->d_mc_tris, v->n_mc_tris * 3);
    return BS_OK;
  } catch (const bs::Error& e) {
    ctx->last_error = e.msg;
    return e.status;
  } catch (const std::bad_alloc&) {
    return BS_ERR_OOM;
  }
}

bs_status bs_corner_table_counts(const bs_corner_table* t, uint64_t* n_faces, uint64_t* n_vertices,
                                 uint64_t* n_vertex_slots, uint64_t* n_corners) {
  if (!t) return BS_ERR_INVALID_ARG;
  uint64_t live = 0;
  for (uint8_t d : t->deleted) live += d == 0;
  if (n_faces) *n_faces = t->cvertex.size() / 3;
  if (n_vertices) *n_vertices = live;
  if (n_vertex_slots) *n_vertex_slots = t->deleted.size();
  if (n_corners) *n_corners = t->cvertex.size();
  return BS_OK;
}

bs_status bs_corner_table_export(const bs_corner_table* t, float* h_positions, uint8_t* h_deleted,
                                 int32_t* h_vertex_corner, int32_t* h_corner_vertex, int32_t* h_corner_opposite) {
  if (!t) return BS_ERR_INVALID_ARG;
  if (h_positions) std::memcpy(h_positions, t->pos.data(), t->pos.size() * sizeof(float));
  if (h_deleted) std::memcpy(h_deleted, t->deleted.data(), t->deleted.size());
  if (h_vertex_corner) std::memcpy(h_vertex_corner, t->vcorner.data(), t->vcorner.size() * sizeof(int32_t));
  if (h_corner_vertex) std::memcpy(h_corner_vertex, t->cvertex.data(), t->cvertex.size() * sizeof(int32_t));
  if (h_corner_opposite) std::memcpy(h_corner_opposite, t->copp.data(), t->copp.size() * sizeof(int32_t));
  return BS_OK;
}

bs_status bs_corner_table_free(bs_corner_table* t) {
  if (!t) return BS_ERR_INVALID_ARG;
  delete t;
  return BS_OK;
}

}  // extern "C"
