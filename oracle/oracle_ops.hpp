// ORACLE — test infrastructure only (see oracle_core.hpp).
//
// Volume booleans and offset: voxel/volume/mod.rs:74-108 and the fast
// sweeping eikonal solver of voxel/fast_sweep.rs (8 ordered Gauss–Seidel
// sweeps over a leaf priority queue, new leaves spawned across faces).
#pragma once

#include <queue>
#include <set>
#include <stdexcept>
#include <unordered_set>

#include "oracle_m2v.hpp"

namespace orc {

// helpers/utils.rs:5-17
inline void sort3(float& a, float& b, float& c) {
  if (a > c) std::swap(a, c);
  if (a > b) std::swap(a, b);
  if (b > c) std::swap(b, c);
}

// fast_sweep.rs:509-537
inline float compute_distance(float a1, float a2, float a3, float h) {
  sort3(a1, a2, a3);
  float s1 = a1 + h;
  if (std::fabs(s1) <= a2) return s1;
  float a1a2_sum = a1 + a2;
  float h_sq = h * h;
  float two_h_sq = h_sq + h_sq;
  float a1a2_diff = a1 - a2;
  float a1a2_diff_sq = a1a2_diff * a1a2_diff;
  float s2 = (a1a2_sum + std::sqrt(two_h_sq - a1a2_diff_sq)) * 0.5f;
  if (std::fabs(s2) <= a3) return s2;
  float a1a2a3_sum = a1a2_sum + a3;
  float three_h_sq = two_h_sq + h_sq;
  float a1a3_diff = a1 - a3;
  float a1a3_diff_sq = a1a3_diff * a1a3_diff;
  float a2a3_diff = a2 - a3;
  float a2a3_diff_sq = a2a3_diff * a2a3_diff;
  return (a1a2a3_sum + std::sqrt(three_h_sq - a1a2_diff_sq - a1a3_diff_sq - a2a3_diff_sq)) *
         (1.0f / 3.0f);
}

struct I3Hash {
  size_t operator()(const I3& p) const {
    uint64_t h = uint64_t(p.x) * 0x9E3779B97F4A7C15ull ^ uint64_t(p.y) * 0xC2B2AE3D27D4EB4Full ^
                 uint64_t(p.z) * 0x165667B19E3779F9ull;
    return size_t(h ^ (h >> 29));
  }
};

struct FastSweeping {
  float limit_abs;
  Sign sweep_sign;
  float h;
  std::map<I3, Bits<512>> frozen;  // topology of the input (clone_map to Empty)

  FastSweeping(float grid_spacing, float limit)
      : limit_abs(std::fabs(limit)), sweep_sign(sign_of(limit)), h(grid_spacing) {}

  struct Dir {
    int sx, sy, sz;
  };
  // fast_sweep.rs:30-66 (sweep order) and 589-684 (queue orderings)
  static constexpr Dir DIRS[8] = {{1, 1, 1},  {-1, 1, 1},  {1, -1, 1},  {-1, -1, 1},
                                  {1, 1, -1}, {-1, 1, -1}, {1, -1, -1}, {-1, -1, -1}};

  struct Stencil {
    std::unique_ptr<Leaf3> top, bottom, left, right, front, back, center;
    const Bits<512>* frozen;
    I3 mn, mx;
    const float* at(const I3& i) const {
      if (i.z < mn.z) return bottom->at(i);
      if (i.z >= mx.z) return top->at(i);
      if (i.y < mn.y) return front->at(i);
      if (i.y >= mx.y) return back->at(i);
      if (i.x < mn.x) return left->at(i);
      if (i.x >= mx.x) return right->at(i);
      return center->at(i);
    }
  };

  static const float* min_by_abs(const float* a, const float* b) {  // utils.rs:64-74
    if (a && b) {
      float fa = std::fabs(*a), fb = std::fabs(*b);
      bool greater = (fa > fb);  // NaN compares as Less
      return greater ? b : a;
    }
    return a ? a : b;
  }

  // fast_sweep.rs:125-183
  void sweep_voxel(const I3& idx, Stencil& st) const {
    if (st.frozen && st.frozen->at(Leaf3::offset(idx))) return;
    const float* dx = min_by_abs(st.at(i3(idx.x + 1, idx.y, idx.z)), st.at(i3(idx.x - 1, idx.y, idx.z)));
    const float* dy = min_by_abs(st.at(i3(idx.x, idx.y + 1, idx.z)), st.at(i3(idx.x, idx.y - 1, idx.z)));
    const float* dz = min_by_abs(st.at(i3(idx.x, idx.y, idx.z + 1)), st.at(i3(idx.x, idx.y, idx.z - 1)));
    const float* first = dx ? dx : (dy ? dy : dz);
    if (!first) return;
    if (sign_of(*first) != sweep_sign) return;
    float d1 = dx ? *dx : FAR, d2 = dy ? *dy : FAR, d3 = dz ? *dz : FAR;
    float dn_abs = compute_distance(std::fabs(d1), std::fabs(d2), std::fabs(d3), h);
    float dn = dn_abs;
    set_sign(dn, sweep_sign);
    if (dn_abs > limit_abs) return;
    const float* old = st.center->at(idx);
    float d_old = old ? *old : FAR;
    if (dn_abs < std::fabs(d_old)) st.center->insert(idx, dn);
  }

  bool face_has_front(const Leaf3& c, int axis, int local) const {
    for (int a = 0; a < 8; ++a)
      for (int b = 0; b < 8; ++b) {
        int x, y, z;
        if (axis == 2) { x = a; y = b; z = local; }
        else if (axis == 1) { x = a; y = local; z = b; }
        else { x = local; y = a; z = b; }
        int o = (x << 6) | (y << 3) | z;
        if (c.mask.at(o) && sign_of(c.values[o]) == sweep_sign && std::fabs(c.values[o]) < limit_abs)
          return true;
      }
    return false;
  }

  void fast_sweep(Grid& sdf) {
    frozen.clear();
    sdf.visit_leafs([&](const Leaf3& l) { frozen[l.origin] = l.mask; },
                    [&](I3, int, float) {});
    std::vector<I3> queue_init;
    sdf.visit_leafs([&](const Leaf3& l) { queue_init.push_back(l.origin); },
                    [&](I3 o, int, float) { queue_init.push_back(o); });

    std::vector<I3> items = queue_init;
    for (int d = 0; d < 8; ++d) {
      const Dir dir = DIRS[d];
      auto cmp_less = [dir](const I3& a, const I3& b) {  // a pops before b
        if (a.x != b.x) return dir.sx > 0 ? a.x < b.x : a.x > b.x;
        if (a.y != b.y) return dir.sy > 0 ? a.y < b.y : a.y > b.y;
        if (a.z != b.z) return dir.sz > 0 ? a.z < b.z : a.z > b.z;
        return false;
      };
      auto pq_cmp = [cmp_less](const I3& a, const I3& b) { return cmp_less(b, a); };
      std::priority_queue<I3, std::vector<I3>, decltype(pq_cmp)> heap(pq_cmp);
      std::unordered_set<I3, I3Hash> existing;
      for (const I3& o : items)
        if (existing.insert(o).second) heap.push(o);
      std::vector<I3> removed;
      while (!heap.empty()) {
        I3 o = heap.top();
        heap.pop();
        removed.push_back(o);
        sweep_leaf(sdf, o, dir, heap, existing);
      }
      items = removed;
    }
    sdf.remove_empty_branches();
  }

  template <class Heap>
  void sweep_leaf(Grid& sdf, const I3& o, const Dir& dir, Heap& heap,
                  std::unordered_set<I3, I3Hash>& existing) const {
    const int64_t S = 8;
    auto take = [&](I3 p) {
      auto l = sdf.take_leaf_at(p);
      return l ? std::move(l) : Leaf3::empty(p);
    };
    Stencil st;
    I3 lo = i3(o.x - S, o.y, o.z), ro = i3(o.x + S, o.y, o.z), fo = i3(o.x, o.y - S, o.z),
       bo = i3(o.x, o.y + S, o.z), to = i3(o.x, o.y, o.z + S), bto = i3(o.x, o.y, o.z - S);
    st.left = take(lo);
    st.right = take(ro);
    st.front = take(fo);
    st.back = take(bo);
    st.top = take(to);
    st.bottom = take(bto);
    st.center = sdf.take_leaf_at(o);
    if (!st.center) throw std::runtime_error("fast sweep: queued leaf missing (tile in volume)");
    auto fz = frozen.find(o);
    st.frozen = fz == frozen.end() ? nullptr : &fz->second;
    st.mn = o;
    st.mx = i3(o.x + S, o.y + S, o.z + S);
    // fast_sweep.rs:111-123 + Direction::sweeps
    for (int a = 0; a < 8; ++a) {
      int64_t x = dir.sx > 0 ? o.x + a : o.x + S - 1 - a;
      for (int b = 0; b < 8; ++b) {
        int64_t y = dir.sy > 0 ? o.y + b : o.y + S - 1 - b;
        for (int c = 0; c < 8; ++c) {
          int64_t z = dir.sz > 0 ? o.z + c : o.z + S - 1 - c;
          sweep_voxel(i3(x, y, z), st);
        }
      }
    }
    // fast_sweep.rs:185-287.  For negative directions the reference indexes
    // the face with a global coordinate; the leaf's index mask maps it to
    // local 0, which is the face used here.
    bool ins_z = face_has_front(*st.center, 2, dir.sz > 0 ? 7 : 0);
    bool ins_y = face_has_front(*st.center, 1, dir.sy > 0 ? 7 : 0);
    bool ins_x = face_has_front(*st.center, 0, dir.sx > 0 ? 7 : 0);
    auto push = [&](I3 p) {
      if (existing.insert(p).second) heap.push(p);
    };
    if (ins_x) push(i3(dir.sx > 0 ? o.x + S : o.x - S, o.y, o.z));
    if (ins_y) push(i3(o.x, dir.sy > 0 ? o.y + S : o.y - S, o.z));
    if (ins_z) push(i3(o.x, o.y, dir.sz > 0 ? o.z + S : o.z - S));
    sdf.insert_leaf_at(std::move(st.top));
    sdf.insert_leaf_at(std::move(st.bottom));
    sdf.insert_leaf_at(std::move(st.left));
    sdf.insert_leaf_at(std::move(st.right));
    sdf.insert_leaf_at(std::move(st.front));
    sdf.insert_leaf_at(std::move(st.back));
    sdf.insert_leaf_at(std::move(st.center));
  }
};

// volume/mod.rs:74-108
struct Volume {
  std::unique_ptr<Grid> grid;
  float voxel_size;
};

inline void volume_union(Volume& a, Volume&& b) {
  a.grid->flood_fill();
  b.grid->flood_fill();
  a.grid->csg_union(std::move(b.grid));
}
inline void volume_intersect(Volume& a, Volume&& b) {
  a.grid->flood_fill();
  b.grid->flood_fill();
  a.grid->csg_intersect(std::move(b.grid));
}
inline void volume_subtract(Volume& a, Volume&& b) {
  a.grid->flood_fill();
  b.grid->flood_fill();
  a.grid->csg_subtract(std::move(b.grid));
}
inline void volume_offset(Volume& v, float distance) {
  const float h = v.voxel_size;
  v.grid->remove_if([h](float x) { return std::fabs(x) > h * 2.0f; });
  float ext = std::fabs(distance) + h + h;
  set_sign(ext, sign_of(distance));
  FastSweeping fs(h, ext);
  fs.fast_sweep(*v.grid);
  v.grid->visit_values_mut([distance](float& x) { x -= distance; });
}

}  // namespace orc
