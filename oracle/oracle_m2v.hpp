// ORACLE — test infrastructure only (see oracle_core.hpp).
//
// Mesh -> narrow-band SDF (voxel/mesh_to_volume.rs) and the fast winding
// numbers it signs with (spatial_partitioning/aabb_tree.rs: top-down "Area"
// SAH build, order-1 + order-2 far field, exact Van Oosterom–Strackee
// solid angles at the leaves).
#pragma once

#include <algorithm>
#include <numeric>

#include "oracle_vdb.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ------------------------------------------------------------- AABB tree --
struct Box {
  V3 mn, mx;
};
inline Box box_empty() {  // Box3::empty(): min = f32::MAX, max = f32::MIN
  return Box{v3(FAR, FAR, FAR), v3(-FAR, -FAR, -FAR)};
}
inline void box_union(Box& b, const Box& o) {
  b.mx = vmax(b.mx, o.mx);
  b.mn = vmin(b.mn, o.mn);
}
inline void box_union_pt(Box& b, V3 p) {
  b.mx = vmax(b.mx, p);
  b.mn = vmin(b.mn, p);
}
inline V3 box_center(const Box& b) { return (b.mn + b.mx) / 2.0f; }
inline float box_area(const Box& b) {  // box3.rs:125-128
  V3 d = b.mx - b.mn;
  return 2.0f * (d.x * d.y + d.x * d.z + d.y * d.z);
}

struct BNode {
  bool leaf;
  size_t left, right;  // leaf: object range [left, right); branch: child ids
  Box bbox;
};

struct NodeData {  // aabb_tree.rs:701-708
  V3 order1;
  M3 order2;
  float radius;
  V3 dipole;
};

struct WindingNumbers {
  std::vector<std::pair<Tri, Box>> objects;
  std::vector<BNode> nodes;  // root is the last node
  std::vector<NodeData> data;
  size_t min_objects_per_leaf = 3;
  size_t max_depth = 40;

  // aabb_tree.rs:422-514 (Area partition strategy, 12 buckets)
  static bool area_split(std::pair<Tri, Box>* obj, size_t n, int axis, const Box& objects_bbox,
                         size_t& split_at) {
    if (n == 0) return false;
    Box cb = box_empty();
    for (size_t i = 0; i < n; ++i) box_union_pt(cb, box_center(obj[i].second));
    const int NB = 12;
    const float nbf = 12.0f;
    auto bucket_of = [&](const Box& bb) -> int {
      V3 c = box_center(bb);
      float o = c[axis] - cb.mn[axis];
      if (cb.mx[axis] > cb.mn[axis]) o /= (cb.mx[axis] - cb.mn[axis]);
      float t = nbf * o;
      size_t tmp;  // Rust `as usize`: saturating, NaN -> 0
      if (!(t > 0.0f))
        tmp = 0;
      else if (t >= 18446744073709551615.0f)
        tmp = SIZE_MAX;
      else
        tmp = size_t(t);
      return int(std::min<size_t>(tmp, NB - 1));
    };
    size_t cnt[NB] = {0};
    Box bb[NB];
    for (int k = 0; k < NB; ++k) bb[k] = box_empty();
    for (size_t i = 0; i < n; ++i) {
      int b = bucket_of(obj[i].second);
      cnt[b] += 1;
      box_union(bb[b], obj[i].second);
    }
    float costs[NB - 1];
    for (int i = 0; i < NB - 1; ++i) {
      Box b0 = box_empty(), b1 = box_empty();
      size_t c0 = 0, c1 = 0;
      for (int j = 0; j <= i; ++j) { box_union(b0, bb[j]); c0 += cnt[j]; }
      for (int j = i + 1; j < NB; ++j) { box_union(b1, bb[j]); c1 += cnt[j]; }
      float f0 = float(c0), f1 = float(c1);
      if (f0 == 0.0f || f1 == 0.0f)
        costs[i] = INFINITY;
      else
        costs[i] = 0.125f + (f0 * box_area(b0) + f1 * box_area(b1)) / box_area(objects_bbox);
    }
    int best = 0;
    for (int i = 1; i < NB - 1; ++i)
      if (costs[i] < costs[best]) best = i;
    float leaf_cost = float(n);
    if (costs[best] < leaf_cost) {
      for (size_t i = 0; i < n; ++i)
        if (bucket_of(obj[i].second) > best) { split_at = i; return true; }
      return false;
    }
    return false;
  }

  // aabb_tree.rs:201-250
  bool split(size_t first, size_t last, size_t& split_at) {
    auto* obj = objects.data() + first;
    size_t n = last - first;
    Box bbox = obj[0].second;
    for (size_t i = 0; i < n; ++i) box_union(bbox, obj[i].second);
    std::pair<float, int> ax[3] = {{bbox.mx.x - bbox.mn.x, 0},
                                   {bbox.mx.y - bbox.mn.y, 1},
                                   {bbox.mx.z - bbox.mn.z, 2}};
    std::stable_sort(ax, ax + 3, [](const std::pair<float, int>& a, const std::pair<float, int>& b) {
      return b.first < a.first;
    });
    for (int k = 0; k < 3; ++k) {
      int axis = ax[k].second;
      std::stable_sort(obj, obj + n, [axis](const std::pair<Tri, Box>& a, const std::pair<Tri, Box>& b) {
        return box_center(a.second)[axis] < box_center(b.second)[axis];
      });
      size_t s;
      if (area_split(obj, n, axis, bbox, s)) {
        split_at = s + first;
        return true;
      }
    }
    return false;
  }

  size_t leaf_node(size_t first, size_t last) {
    Box bbox = objects[first].second;
    for (size_t i = first + 1; i < last; ++i) box_union(bbox, objects[i].second);
    nodes.push_back(BNode{true, first, last, bbox});
    return nodes.size() - 1;
  }

  // aabb_tree.rs:157-199
  size_t build_node(size_t first, size_t last, size_t depth) {
    if (depth >= max_depth || last - first <= min_objects_per_leaf) return leaf_node(first, last);
    size_t s;
    if (!split(first, last, s)) return leaf_node(first, last);
    size_t l = build_node(first, s, depth + 1);
    size_t r = build_node(s, last, depth + 1);
    Box bbox = nodes[l].bbox;
    box_union(bbox, nodes[r].bbox);
    nodes.push_back(BNode{false, l, r, bbox});
    return nodes.size() - 1;
  }

  struct Init {
    V3 awn, awc;
    M3 o1;
    float area;
    V3 dipole;
  };
  // aabb_tree.rs:749-777
  Init leaf_data(const BNode& nd) const {
    Init d{v3(0, 0, 0), v3(0, 0, 0), m3_zero(), 0.0f, v3(0, 0, 0)};
    for (size_t t = nd.left; t < nd.right; ++t) {
      const Tri& tri = objects[t].first;
      V3 cr = cross(tri.b - tri.a, tri.c - tri.a);
      if (norm_sq(cr) == 0.0f) continue;
      V3 nrm = cr / norm(cr);
      float area = norm(cross(tri.b - tri.a, tri.c - tri.a)) * 0.5f;
      d.area += area;
      d.awn += area * nrm;
      V3 c = (tri.a + tri.b + tri.c) / 3.0f;
      d.o1 = d.o1 + outer(area * c, nrm);
      d.awc += area * c;
    }
    d.dipole = d.awc / d.area;
    return d;
  }
  // aabb_tree.rs:723-747, 779-801
  Init node_data(size_t idx) {
    const BNode nd = nodes[idx];
    Init d;
    if (nd.leaf) {
      d = leaf_data(nd);
    } else {
      Init l = node_data(nd.left);
      Init r = node_data(nd.right);
      d.o1 = l.o1 + r.o1;
      d.awn = l.awn + r.awn;
      d.awc = l.awc + r.awc;
      d.area = l.area + r.area;
      d.dipole = (l.awc + r.awc) / d.area;
    }
    float dmin = norm_sq(nd.bbox.mn - d.dipole);
    float dmax = norm_sq(nd.bbox.mx - d.dipole);
    float radius = std::sqrt(std::fmax(dmin, dmax));
    data[idx] = NodeData{d.awn, d.o1 - outer(d.dipole, d.awn), radius, d.dipole};
    return d;
  }

  // aabb_tree.rs:636-644
  void build(const std::vector<Tri>& tris) {
    objects.clear();
    nodes.clear();
    data.clear();
    for (const Tri& t : tris) {
      Box b;
      tri_bbox(t, b.mn, b.mx);
      objects.push_back({t, b});
    }
    if (!objects.empty()) build_node(0, objects.size(), 1);
    data.resize(nodes.size());
    if (!nodes.empty()) node_data(nodes.size() - 1);
  }

  static constexpr float PI_F = 3.14159265358979323846f;
  static constexpr float FOUR_PI = 4.0f * PI_F;

  // aabb_tree.rs:582-615
  static float solid_angle(const Tri& t, V3 q) {
    V3 qa = t.a - q, qb = t.b - q, qc = t.c - q;
    float al = norm(qa), bl = norm(qb), cl = norm(qc);
    if (al == 0.0f || bl == 0.0f || cl == 0.0f) return 0.0f;
    qa = qa / al;
    qb = qb / bl;
    qc = qc / cl;
    float num = dot(qa, cross(qb - qa, qc - qa));
    if (num == 0.0f) return 0.0f;
    float den = 1.0f + dot(qa, qb) + dot(qa, qc) + dot(qb, qc);
    return std::atan2(num, den) * 2.0f;
  }
  // aabb_tree.rs:803-816
  static void hessians(V3 dip, V3 q, V3& o1, M3& o2) {
    V3 r = dip - q;
    float r2 = norm_sq(r);
    float r1 = std::sqrt(r2);
    float r3 = r2 * r1;
    float den = FOUR_PI * r3;
    float inv = 1.0f / den;
    o1 = r * inv;
    float r5 = r3 * r2;
    M3 q3 = outer(3.0f * r, r);
    float d5 = FOUR_PI * r5;
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) {
        float id = (i == j) ? 1.0f * inv : 0.0f * inv;
        o2.m[j][i] = id - q3.m[j][i] / d5;
      }
  }
  // aabb_tree.rs:662-691 (recursion order kept: wn(node) = wn(left) + wn(right))
  float fast_wn(size_t idx, V3 p, float beta, uint64_t& n_far, uint64_t& n_leaf_tris) const {
    const NodeData& nd = data[idx];
    float dist = norm(p - nd.dipole);
    if (dist > nd.radius * beta) {
      V3 o1;
      M3 o2;
      hessians(nd.dipole, p, o1, o2);
      n_far++;
      return dot(nd.order1, o1) + mdot(nd.order2, o2);
    }
    const BNode& bn = nodes[idx];
    if (bn.leaf) {
      float wn = 0.0f;
      for (size_t t = bn.left; t < bn.right; ++t) wn += solid_angle(objects[t].first, p);
      n_leaf_tris += bn.right - bn.left;
      return wn / FOUR_PI;
    }
    float l = fast_wn(bn.left, p, beta, n_far, n_leaf_tris);
    float r = fast_wn(bn.right, p, beta, n_far, n_leaf_tris);
    return l + r;
  }
  // aabb_tree.rs:654-660
  float approximate(V3 p, float beta, uint64_t* n_far = nullptr, uint64_t* n_leaf = nullptr) const {
    if (nodes.empty()) return 0.0f;
    uint64_t f = 0, l = 0;
    float v = fast_wn(nodes.size() - 1, p, beta, f, l);
    if (n_far) *n_far += f;
    if (n_leaf) *n_leaf += l;
    return v;
  }
};

// -------------------------------------------------------- mesh to volume --
// mesh_to_volume.rs:75-116
inline void subdivide_triangle(const Tri& tri, float voxel_size, std::vector<Tri>& out) {
  float num_subs = std::floor(tri_max_side(tri) / voxel_size);
  float inv = 1.0f / num_subs;
  if (num_subs < 2.0f) {
    out.push_back(tri);
    return;
  }
  V3 s1 = (tri.b - tri.a) * inv;
  V3 s2 = (tri.c - tri.b) * inv;
  V3 a = tri.a;
  size_t n = size_t(num_subs);
  for (size_t i = 0; i < n; ++i) {
    V3 b = a + s1;
    V3 c = b + s2;
    V3 a_s = a + s2, b_s = b + s2, c_s = c + s2;
    V3 a_prev = a;
    for (size_t k = 0; k < i; ++k) {
      out.push_back(Tri{a_prev, b_s, a_s});
      out.push_back(Tri{a_s, b_s, c_s});
      a_prev = a_s;
      a_s += s2;
      b_s += s2;
      c_s += s2;
    }
    out.push_back(Tri{a, b, c});
    a += s1;
  }
}

// mesh_to_volume.rs:124-143: widened integer box of one (sub-)triangle.
inline void widened_box(const Tri& t, float inv_h, int64_t band, I3& mn, I3& mx) {
  V3 bmin, bmax;
  tri_bbox(t, bmin, bmax);
  mn = i3(int64_t(std::floor(bmin.x * inv_h)) - band, int64_t(std::floor(bmin.y * inv_h)) - band,
          int64_t(std::floor(bmin.z * inv_h)) - band);
  mx = i3(int64_t(std::ceil(bmax.x * inv_h)) + band, int64_t(std::ceil(bmax.y * inv_h)) + band,
          int64_t(std::ceil(bmax.z * inv_h)) + band);
  if (mx.x == mn.x || mx.y == mn.y || mx.z == mn.z) {
    mn = i3(mn.x - 1, mn.y - 1, mn.z - 1);
    mx = i3(mx.x + 1, mx.y + 1, mx.z + 1);
  }
}

struct MeshToVolumeStats {
  uint64_t n_subtris = 0, n_pairs = 0, n_far = 0, n_leaf_tris = 0, n_band = 0;
  uint64_t n_near_threshold = 0;  // |wn - 0.2| < 1e-3
};

// mesh_to_volume.rs:52-73, 118-196, 245-280.  The per-sub-triangle distance
// boxes are merged chunk by chunk (min is order independent, equal values are
// identical), so memory stays bounded on large meshes.
inline std::unique_ptr<Grid> mesh_to_volume(const std::vector<Tri>& tris, float voxel_size,
                                            int64_t band, MeshToVolumeStats* stats = nullptr,
                                            std::vector<float>* wn_out = nullptr) {
  const float inv_h = 1.0f / voxel_size;
  std::vector<Tri> sub;
  for (const Tri& t : tris) subdivide_triangle(t, voxel_size, sub);
  if (sub.empty()) return nullptr;

  WindingNumbers wn;
  wn.build(tris);

  auto grid = std::make_unique<Grid>();
  const size_t CH = 1 << 16;
  uint64_t pairs = 0;
  for (size_t c0 = 0; c0 < sub.size(); c0 += CH) {
    size_t c1 = std::min(sub.size(), c0 + CH);
    std::vector<std::vector<float>> dist(c1 - c0);
    std::vector<I3> mins(c1 - c0), maxs(c1 - c0);
#pragma omp parallel for schedule(dynamic, 64)
    for (long long s = (long long)c0; s < (long long)c1; ++s) {
      const Tri& t = sub[size_t(s)];
      I3 mn, mx;
      widened_box(t, inv_h, band, mn, mx);
      auto& d = dist[size_t(s) - c0];
      d.reserve(size_t((mx.x - mn.x + 1) * (mx.y - mn.y + 1) * (mx.z - mn.z + 1)));
      for (int64_t x = mn.x; x <= mx.x; ++x) {
        float xw = float(x) * voxel_size;
        for (int64_t y = mn.y; y <= mx.y; ++y) {
          float yw = float(y) * voxel_size;
          for (int64_t z = mn.z; z <= mx.z; ++z) {
            float zw = float(z) * voxel_size;
            V3 g = v3(xw, yw, zw);
            V3 cp = closest_point(t, g);
            d.push_back(norm(cp - g));
          }
        }
      }
      mins[size_t(s) - c0] = mn;
      maxs[size_t(s) - c0] = mx;
    }
    for (size_t s = 0; s < c1 - c0; ++s) {
      const I3 mn = mins[s], mx = maxs[s];
      size_t i = 0;
      for (int64_t x = mn.x; x <= mx.x; ++x)
        for (int64_t y = mn.y; y <= mx.y; ++y)
          for (int64_t z = mn.z; z <= mx.z; ++z) {
            I3 idx = i3(x, y, z);
            const float* cur = grid->at(idx);
            float cd = cur ? *cur : INFINITY;
            if (dist[s][i] < cd) grid->insert(idx, dist[s][i]);
            ++i;
          }
      pairs += i;
    }
  }

  // Signs: one fast winding number per active voxel (mesh_to_volume.rs:245-280).
  std::vector<Leaf3*> leaves;
  std::function<void(Int4&)> col4 = [&](Int4& n) {
    for (int o = 0; o < Int4::N; ++o)
      if (n.child_mask.at(o)) leaves.push_back(n.childs[o].get());
  };
  for (auto& kv : grid->root)
    for (int o = 0; o < Int5::N; ++o)
      if (kv.second->child_mask.at(o)) col4(*kv.second->childs[o]);
  uint64_t n_far = 0, n_leaf = 0, n_band = 0, n_near = 0;
  std::vector<std::vector<float>> wn_per_leaf(wn_out ? leaves.size() : 0);
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : n_far, n_leaf, n_band, n_near)
  for (long long li = 0; li < (long long)leaves.size(); ++li) {
    Leaf3& lf = *leaves[size_t(li)];
    for (int o = 0; o < Leaf3::N; ++o) {
      if (!lf.mask.at(o)) continue;
      int64_t x = lf.origin.x + (o >> 6), y = lf.origin.y + ((o >> 3) & 7), z = lf.origin.z + (o & 7);
      V3 gp = v3(float(x) * voxel_size, float(y) * voxel_size, float(z) * voxel_size);
      uint64_t f0 = 0, l0 = 0;
      float v = wn.approximate(gp, 2.0f, &f0, &l0);
      n_far += f0;
      n_leaf += l0;
      n_band += 1;
      if (std::fabs(v - 0.2f) < 1e-3f) n_near += 1;
      if (wn_out) wn_per_leaf[size_t(li)].push_back(v);
      float d = lf.values[o];
      lf.values[o] = (v < 0.2f) ? std::copysign(d, 1.0f) : std::copysign(d, -1.0f);
    }
  }
  if (wn_out) {
    wn_out->clear();
    for (auto& w : wn_per_leaf) wn_out->insert(wn_out->end(), w.begin(), w.end());
  }
  if (stats) {
    stats->n_subtris = sub.size();
    stats->n_pairs = pairs;
    stats->n_far = n_far;
    stats->n_leaf_tris = n_leaf;
    stats->n_band = n_band;
    stats->n_near_threshold = n_near;
  }
  return grid;
}

}  // namespace orc
