// CornerTable from a triangle soup: CornerTable::builder_soup().finish()
// (mesh/corner_table/builder.rs:292-309) on top of the GPU.
//
//  * merge_points (algo/merge_points.rs:12-41) on the GPU: exactly equal
//    points (-0 == +0, NaN never equal) get one vertex, numbered in order of
//    first appearance — three stable radix sorts on the coordinate bits, a
//    group scan, and a scan over the first occurrences;
//  * the indexed build (builder.rs:168-262) on the host: faces in order, a
//    face that repeats a directed edge is skipped, then isolated vertices are
//    deleted and every extra corner fan of a vertex gets its own copy.  This
//    step is order dependent by definition and touches a few bytes per face.
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

// merge_points on device points d_p[n][3]: ids[n] (host) and unique points (host).
static void merge_points_gpu(bs_ctx* ctx, const float* d_p, uint64_t n, std::vector<uint32_t>& ids,
                             std::vector<float>& uniq) {
  cudaStream_t s = ctx->stream;
  ids.assign(n, 0);
  uniq.clear();
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
  uint32_t nu = 0;
  read_back(ctx, &nu, newid.p + n, sizeof(uint32_t));
  DBuf<float> up(ctx, uint64_t(nu) * 3);
  BS_KERNEL(ctx, "k_unique_points", (k_unique_points<<<nbc(n, 256), 256, 0, s>>>(d_p, is_rep.p, newid.p, n, up.p)));
  uniq.resize(uint64_t(nu) * 3);
  BS_CUDA(cudaMemcpyAsync(ids.data(), id.p, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  if (nu) BS_CUDA(cudaMemcpyAsync(uniq.data(), up.p, uint64_t(nu) * 3 * sizeof(float), cudaMemcpyDeviceToHost, s));
  BS_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------- host indexed build ---
namespace {

struct EdgeMap {  // directed edge (a, b) -> corner, open addressing
  std::vector<uint64_t> keys;
  std::vector<int32_t> vals;
  uint64_t mask = 0;
  static constexpr uint64_t EMPTY = ~0ull;
  explicit EdgeMap(uint64_t n) {
    uint64_t cap = 64;
    while (cap < 2 * n + 16) cap <<= 1;
    keys.assign(cap, EMPTY);
    vals.assign(cap, -1);
    mask = cap - 1;
  }
  static uint64_t h(uint64_t k) {
    k ^= k >> 31;
    k *= 0x7fb5d329728ea185ull;
    k ^= k >> 27;
    k *= 0x81dadef4bc2dd44dull;
    return k ^ (k >> 33);
  }
  int32_t* find(uint32_t a, uint32_t b) {
    const uint64_t k = (uint64_t(a) << 32) | b;
    for (uint64_t s = h(k) & mask;; s = (s + 1) & mask) {
      if (keys[s] == k) return &vals[s];
      if (keys[s] == EMPTY) return nullptr;
    }
  }
  void put(uint32_t a, uint32_t b, int32_t v) {
    const uint64_t k = (uint64_t(a) << 32) | b;
    for (uint64_t s = h(k) & mask;; s = (s + 1) & mask) {
      if (keys[s] == k || keys[s] == EMPTY) {
        keys[s] = k;
        vals[s] = v;
        return;
      }
    }
  }
};

inline int32_t cnext(int32_t c) { return (c % 3 == 2) ? c - 2 : c + 1; }
inline int32_t cprev(int32_t c) { return (c % 3 == 0) ? c + 2 : c - 1; }

// traversal.rs:244-286
template <class F>
void corners_around_vertex(const bs_corner_table& t, int32_t v, F visit) {
  const size_t guard_max = t.cvertex.size() + 3;
  int32_t w = cprev(t.vcorner[v]);
  const int32_t started = w;
  bool border = false;
  for (size_t g = 0; g < guard_max; ++g) {
    visit(cnext(w));
    w = cprev(w);
    if (t.copp[w] < 0) {
      border = true;
      break;
    }
    w = t.copp[w];
    if (w == started) break;
  }
  w = started;
  if (border && t.copp[w] >= 0) {
    w = t.copp[w];
    for (size_t g = 0; g < guard_max; ++g) {
      visit(cprev(w));
      w = cnext(w);
      if (t.copp[w] < 0) break;
      w = t.copp[w];
    }
  }
}

// builder.rs:168-262 on merged points.
void indexed_build(bs_corner_table& t, const std::vector<float>& uniq, const std::vector<uint32_t>& ids) {
  const uint64_t nv = uniq.size() / 3, nf = ids.size() / 3;
  t.pos = uniq;
  t.deleted.assign(nv, 0);
  t.vcorner.assign(nv, -1);
  t.cvertex.clear();
  t.copp.clear();
  t.cvertex.reserve(nf * 3);
  t.copp.reserve(nf * 3);
  EdgeMap em(nf * 3);
  auto corner_from = [&](uint32_t a, uint32_t b, uint32_t vertex) {
    const int32_t c = int32_t(t.cvertex.size());
    t.cvertex.push_back(int32_t(vertex));
    t.copp.push_back(-1);
    if (int32_t* o = em.find(b, a)) {
      t.copp[c] = *o;
      t.copp[*o] = c;
    }
    em.put(a, b, c);
    t.vcorner[vertex] = c;
    return c;
  };
  for (uint64_t f = 0; f < nf; ++f) {
    const uint32_t a = ids[3 * f], b = ids[3 * f + 1], c = ids[3 * f + 2];
    // a face repeating a directed edge would be non-manifold: skipped (builder.rs:188-194)
    if (em.find(b, c) || em.find(c, a) || em.find(a, b)) continue;
    corner_from(b, c, a);
    corner_from(c, a, b);
    corner_from(a, b, c);
  }
  // finish(): delete isolated vertices, split non-manifold vertices
  for (uint64_t v = 0; v < nv; ++v)
    if (t.vcorner[v] < 0) t.deleted[v] = 1;
  // corners of every vertex in increasing corner order (BTreeSet)
  std::vector<uint32_t> start(nv + 1, 0);
  for (int32_t vx : t.cvertex) start[vx + 1]++;
  for (uint64_t v = 0; v < nv; ++v) start[v + 1] += start[v];
  std::vector<int32_t> corners(t.cvertex.size());
  {
    std::vector<uint32_t> fill(start.begin(), start.end() - 1);
    for (int32_t c = 0; c < int32_t(t.cvertex.size()); ++c) corners[fill[t.cvertex[c]]++] = c;
  }
  std::vector<uint8_t> seen(t.cvertex.size(), 0);
  for (uint64_t v = 0; v < nv; ++v) {
    if (t.deleted[v]) continue;
    corners_around_vertex(t, int32_t(v), [&](int32_t c) { seen[c] = 1; });
    const float px = t.pos[3 * v], py = t.pos[3 * v + 1], pz = t.pos[3 * v + 2];
    for (uint32_t k = start[v]; k < start[v + 1]; ++k) {
      const int32_t ci = corners[k];
      if (seen[ci]) continue;
      const int32_t dup = int32_t(t.vcorner.size());
      t.pos.push_back(px);
      t.pos.push_back(py);
      t.pos.push_back(pz);
      t.deleted.push_back(0);
      t.vcorner.push_back(ci);
      seen[ci] = 1;
      corners_around_vertex(t, dup, [&](int32_t c) {
        t.cvertex[c] = dup;
        seen[c] = 1;
      });
    }
  }
}

}  // namespace

bs_corner_table* corner_table_from_device_soup(bs_ctx* ctx, const float* d_pts, uint64_t n_points) {
  std::vector<uint32_t> ids;
  std::vector<float> uniq;
  merge_points_gpu(ctx, d_pts, n_points, ids, uniq);
  auto* t = new bs_corner_table();
  indexed_build(*t, uniq, ids);
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
