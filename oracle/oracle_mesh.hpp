// ORACLE — test infrastructure only (see oracle_core.hpp).
//
// Surface extraction and mesh assembly:
//  * dual contouring with the particle vertex solver
//    (voxel/meshing/dual_contouring.rs);
//  * a marching-cubes triangle counter used only to pin the oracle against
//    the reference's offset test (7944 vertices, voxel/volume/mod.rs:134-152);
//    it counts polygons by walking the cube faces and is exact for cubes
//    without ambiguous faces — the number of ambiguous faces met is returned;
//  * the CornerTable soup/indexed builders (mesh/corner_table/builder.rs,
//    algo/merge_points.rs).
#pragma once

#include <set>
#include <unordered_map>

#include "oracle_ops.hpp"

namespace orc {

// voxel/utils.rs:88-97
static const int CUBE_OFF[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                   {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

struct IntPoint {
  V3 point, normal;
};

// dual_contouring.rs:395-423
static const int DC_CELL_OFF[3][4][3] = {
    {{0, 0, 0}, {0, 0, -1}, {0, -1, -1}, {0, -1, 0}},
    {{0, 0, 0}, {-1, 0, 0}, {-1, 0, -1}, {0, 0, -1}},
    {{0, -1, 0}, {-1, -1, 0}, {-1, 0, 0}, {0, 0, 0}}};
static const int DC_EDGE_OFF[12][4] = {{0, 0, 0, 0}, {0, 0, 0, 1}, {0, 0, 0, 2}, {1, 0, 0, 1},
                                       {1, 0, 0, 2}, {0, 0, 1, 0}, {0, 0, 1, 1}, {0, 1, 0, 0},
                                       {0, 1, 0, 2}, {1, 0, 1, 1}, {0, 1, 1, 0}, {1, 1, 0, 2}};

// dual_contouring.rs:429-458
inline V3 find_feature_point(const std::vector<IntPoint>& pts) {
  const float threshold = 1e-6f;
  const int iters = 50;
  V3 acc = v3(0, 0, 0);
  for (const auto& p : pts) acc = acc + p.point;
  float len = float(pts.size());
  V3 c = acc / len;
  for (int i = 0; i < iters; ++i) {
    V3 force = v3(0, 0, 0);
    for (const auto& ip : pts) {
      V3 p = ip.point, n = ip.normal;
      force += (n * -1.0f) * dot(n, c - p);
    }
    float damping = 1.0f - float(i) / float(iters);
    c += (force * damping) / len;
    if (norm_sq(force) < threshold) break;
  }
  return c;
}

struct DcResult {
  std::vector<float> tris;  // 9 floats per triangle, scaled by the voxel size
  int status = 0;           // 0 ok, 1 tile met (reference: todo!), 2 gradient without neighbours
  uint64_t n_edges = 0, n_cells = 0;
};

inline uint64_t pack3(int64_t x, int64_t y, int64_t z) {
  return (uint64_t(x + (1 << 20)) << 42) | (uint64_t(y + (1 << 20)) << 21) | uint64_t(z + (1 << 20));
}

// dual_contouring.rs:23-91 (face order: leaves in tree order, voxels x-y-z).
// The reference stops at an active tile (todo!(), dual_contouring.rs:139,
// 186, 347): status 1.  With tiles_via_at the passes still visit the leaves
// only and read every neighbour through Grid::at, which returns an active
// tile's value for a voxel outside the leaves — the extension the GPU
// implements for volumes with tiles.
inline DcResult dual_contour(const Grid& g, float voxel_size, bool tiles_via_at = false) {
  DcResult res;
  bool tile = false;
  std::vector<const Leaf3*> leaves;
  g.visit_leafs([&](const Leaf3& l) { leaves.push_back(&l); },
                [&](I3, int, float) { tile = true; });
  if (tile && !tiles_via_at) { res.status = 1; return res; }
  std::unordered_map<uint64_t, IntPoint> ints[3];
  auto grad = [&](I3 p, int axis, float& out) -> bool {
    I3 pl = p, pr = p;
    pl[axis] -= 1;
    pr[axis] += 1;
    const float* vp = g.at(p);
    const float* vl = g.at(pl);
    const float* vr = g.at(pr);
    if (vp && vl && vr) { out = (*vr - *vl) * 0.5f; return true; }
    if (vp && vr) { out = *vr - *vp; return true; }
    if (vp && vl) { out = *vp - *vl; return true; }
    return false;
  };
  // edge pass, dual_contouring.rs:249-387
  for (const Leaf3* l : leaves) {
    for (int a = 0; a < 8; ++a)
      for (int b = 0; b < 8; ++b)
        for (int c = 0; c < 8; ++c) {
          I3 v1 = i3(l->origin.x + a, l->origin.y + b, l->origin.z + c);
          for (int dir = 0; dir < 3; ++dir) {
            I3 v2 = v1;
            v2[dir] += 1;
            const float* p1 = g.at(v1);
            const float* p2 = g.at(v2);
            if (!p1 || !p2) continue;
            float a1 = *p1, a2 = *p2;
            if (sign_of(a1) == sign_of(a2)) continue;
            float t = (a1 == a2) ? 0.5f : a1 / (a1 - a2);
            V3 pt = v3(float(v1.x), float(v1.y), float(v1.z));
            pt[dir] = float(v1[dir]) + t;
            float gr[2][3];
            for (int ax = 0; ax < 3; ++ax) {
              if (!grad(v1, ax, gr[0][ax]) || !grad(v2, ax, gr[1][ax])) {
                res.status = 2;
                return res;
              }
            }
            V3 nrm;
            for (int ax = 0; ax < 3; ++ax) nrm[ax] = (1.0f - t) * gr[0][ax] + t * gr[1][ax];
            nrm = nrm / norm(nrm);
            ints[dir][pack3(v1.x, v1.y, v1.z)] = IntPoint{pt, nrm};
            res.n_edges++;
          }
        }
  }
  // cell pass, dual_contouring.rs:176-247
  std::unordered_map<uint64_t, V3> cells;
  std::vector<IntPoint> pts;
  for (const Leaf3* l : leaves) {
    for (int a = 0; a < 8; ++a)
      for (int b = 0; b < 8; ++b)
        for (int c = 0; c < 8; ++c) {
          I3 o = i3(l->origin.x + a, l->origin.y + b, l->origin.z + c);
          float vals[8];
          bool ok = true;
          for (int i = 0; i < 8 && ok; ++i) {
            const float* p = g.at(i3(o.x + CUBE_OFF[i][0], o.y + CUBE_OFF[i][1], o.z + CUBE_OFF[i][2]));
            if (!p) ok = false; else vals[i] = *p;
          }
          if (!ok) continue;
          Sign s0 = sign_of(vals[0]);
          bool same = true;
          for (int i = 1; i < 8; ++i) same = same && sign_of(vals[i]) == s0;
          if (same) continue;
          pts.clear();
          for (int e = 0; e < 12; ++e) {
            I3 p = i3(o.x + DC_EDGE_OFF[e][0], o.y + DC_EDGE_OFF[e][1], o.z + DC_EDGE_OFF[e][2]);
            auto it = ints[DC_EDGE_OFF[e][3]].find(pack3(p.x, p.y, p.z));
            if (it != ints[DC_EDGE_OFF[e][3]].end()) pts.push_back(it->second);
          }
          cells[pack3(o.x, o.y, o.z)] = find_feature_point(pts);
          res.n_cells++;
        }
  }
  // triangulation, dual_contouring.rs:93-174
  std::vector<V3> verts;
  for (const Leaf3* l : leaves) {
    for (int a = 0; a < 8; ++a)
      for (int b = 0; b < 8; ++b)
        for (int c = 0; c < 8; ++c) {
          I3 v = i3(l->origin.x + a, l->origin.y + b, l->origin.z + c);
          const float* pv = l->at(v);
          if (!pv) continue;
          float v1 = *pv;
          for (int dir = 0; dir < 3; ++dir) {
            I3 v2i = v;
            v2i[dir] += 1;
            const float* p2 = g.at(v2i);
            if (!p2) continue;
            if (sign_of(v1) == sign_of(*p2)) continue;
            V3 q[4];
            bool ok = true;
            for (int k = 0; k < 4 && ok; ++k) {
              auto it = cells.find(pack3(v.x + DC_CELL_OFF[dir][k][0], v.y + DC_CELL_OFF[dir][k][1],
                                         v.z + DC_CELL_OFF[dir][k][2]));
              if (it == cells.end()) ok = false; else q[k] = it->second;
            }
            if (!ok) continue;
            V3 f[6] = {q[0], q[1], q[2], q[2], q[3], q[0]};
            if (sign_of(v1) == Sign::Neg) {
              std::swap(f[1], f[2]);
              std::swap(f[4], f[5]);
            }
            for (int k = 0; k < 6; ++k) verts.push_back(f[k]);
          }
        }
  }
  for (size_t i = 0; i + 2 < verts.size(); i += 3) {
    V3 a = verts[i] * voxel_size, b = verts[i + 1] * voxel_size, c = verts[i + 2] * voxel_size;
    if (norm_sq(cross(b - a, c - a)) == 0.0f) continue;  // Triangle3::is_degenerate
    const V3 t3[3] = {a, b, c};
    for (const V3& p : t3) {
      res.tris.push_back(p.x);
      res.tris.push_back(p.y);
      res.tris.push_back(p.z);
    }
  }
  return res;
}

// --------------------------------------------------- marching-cubes count --
struct McCount {
  uint64_t triangles = 0, ambiguous_faces = 0, cubes = 0;
};

inline void mc_count_cube(const Grid& g, const I3& vox, McCount& mc) {
  float v[8];
  for (int i = 0; i < 8; ++i) {
    const float* p = g.at(i3(vox.x + CUBE_OFF[i][0], vox.y + CUBE_OFF[i][1], vox.z + CUBE_OFF[i][2]));
    if (!p) return;
    float x = *p;
    if (std::fabs(x) < 1e-6f) x = std::copysign(1e-6f, x);  // marching_cubes.rs:1160-1181
    v[i] = x;
  }
  bool in[8];
  int nin = 0;
  for (int i = 0; i < 8; ++i) { in[i] = v[i] < 0.0f; nin += in[i]; }
  mc.cubes++;
  if (nin == 0 || nin == 8) return;
  // cube edges as corner pairs (corner numbering of CUBE_OFF)
  static const int E[12][2] = {{0, 1}, {1, 2}, {3, 2}, {0, 3}, {4, 5}, {5, 6},
                               {7, 6}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
  // faces as 4 corners in cyclic order
  static const int F[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                              {3, 2, 6, 7}, {0, 3, 7, 4}, {1, 2, 6, 5}};
  auto edge_id = [&](int a, int b) {
    for (int e = 0; e < 12; ++e)
      if ((E[e][0] == a && E[e][1] == b) || (E[e][0] == b && E[e][1] == a)) return e;
    return -1;
  };
  std::vector<int> adj[12];
  int ncross = 0;
  for (int e = 0; e < 12; ++e) ncross += in[E[e][0]] != in[E[e][1]];
  for (int f = 0; f < 6; ++f) {
    int c[4] = {F[f][0], F[f][1], F[f][2], F[f][3]};
    int ce[4];
    int k = 0;
    for (int s = 0; s < 4; ++s) {
      int a = c[s], b = c[(s + 1) & 3];
      if (in[a] != in[b]) ce[k++] = s;
    }
    if (k == 2) {
      int e0 = edge_id(c[ce[0]], c[(ce[0] + 1) & 3]);
      int e1 = edge_id(c[ce[1]], c[(ce[1] + 1) & 3]);
      adj[e0].push_back(e1);
      adj[e1].push_back(e0);
    } else if (k == 4) {
      mc.ambiguous_faces++;
      // asymptotic decider: saddle value of the bilinear face
      float a0 = v[c[0]], a1 = v[c[1]], a2 = v[c[2]], a3 = v[c[3]];
      float saddle = (a0 * a2 - a1 * a3) / (a0 + a2 - a1 - a3);
      bool c0_joins_c2 = (saddle < 0.0f) == in[c[0]];
      int e01 = edge_id(c[0], c[1]), e12 = edge_id(c[1], c[2]), e23 = edge_id(c[2], c[3]),
          e30 = edge_id(c[3], c[0]);
      if (c0_joins_c2) {
        adj[e01].push_back(e12); adj[e12].push_back(e01);
        adj[e23].push_back(e30); adj[e30].push_back(e23);
      } else {
        adj[e30].push_back(e01); adj[e01].push_back(e30);
        adj[e12].push_back(e23); adj[e23].push_back(e12);
      }
    }
  }
  // count cycles in the 2-regular crossing graph
  bool seen[12] = {false};
  int cycles = 0;
  for (int e = 0; e < 12; ++e) {
    if (in[E[e][0]] == in[E[e][1]] || seen[e]) continue;
    cycles++;
    int cur = e, prev = -1;
    while (!seen[cur]) {
      seen[cur] = true;
      int nxt = adj[cur][0] == prev ? adj[cur][1] : adj[cur][0];
      prev = cur;
      cur = nxt;
    }
  }
  mc.triangles += uint64_t(ncross - 2 * cycles);
}

// marching_cubes.rs:967-1021 (cubes of dense leaves and the boundary of tiles)
inline McCount mc_count(const Grid& g) {
  McCount mc;
  g.visit_leafs(
      [&](const Leaf3& l) {
        for (int a = 0; a < 8; ++a)
          for (int b = 0; b < 8; ++b)
            for (int c = 0; c < 8; ++c) mc_count_cube(g, i3(l.origin.x + a, l.origin.y + b, l.origin.z + c), mc);
      },
      [&](I3 o, int s, float) {
        for (int i = 0; i < s; ++i)
          for (int j = 0; j < s; ++j) {
            mc_count_cube(g, i3(o.x, o.y + i, o.z + j), mc);
            mc_count_cube(g, i3(o.x + s - 1, o.y + i, o.z + j), mc);
            mc_count_cube(g, i3(o.x + i, o.y + j, o.z + s - 1), mc);
            mc_count_cube(g, i3(o.x + i, o.y + j, o.z), mc);
            mc_count_cube(g, i3(o.x + i, o.y + s - 1, o.z + j), mc);
            mc_count_cube(g, i3(o.x + i, o.y, o.z + j), mc);
          }
      });
  return mc;
}

// ------------------------------------------------------------ CornerTable --
// mesh/corner_table/builder.rs:136-262, traversal.rs:244-298
struct CornerTableB {
  static constexpr uint32_t NONE = 0xFFFFFFFFu;
  std::vector<V3> pos;
  std::vector<uint32_t> vcorner;
  std::vector<uint8_t> vdeleted;
  std::vector<uint32_t> cvertex, copp;
  std::unordered_map<uint64_t, uint32_t> edge_map;
  std::map<uint32_t, std::set<uint32_t>> vertex_corners;
  bool failed = false;

  static uint32_t next(uint32_t c) { return (c % 3 == 2) ? c - 2 : c + 1; }
  static uint32_t prev(uint32_t c) { return (c % 3 == 0) ? c + 2 : c - 1; }
  static uint64_t ekey(uint32_t a, uint32_t b) { return (uint64_t(a) << 32) | b; }

  uint32_t add_vertex(V3 p, uint32_t corner = NONE) {
    pos.push_back(p);
    vcorner.push_back(corner);
    vdeleted.push_back(0);
    return uint32_t(pos.size() - 1);
  }
  uint32_t corner_from(uint32_t a, uint32_t b, uint32_t vertex) {
    uint32_t c = uint32_t(cvertex.size());
    cvertex.push_back(vertex);
    copp.push_back(NONE);
    auto it = edge_map.find(ekey(b, a));
    if (it != edge_map.end()) {
      copp[c] = it->second;
      copp[it->second] = c;
    }
    edge_map[ekey(a, b)] = c;
    vcorner[vertex] = c;
    return c;
  }
  bool add_face(size_t v1, size_t v2, size_t v3) {
    size_t nv = pos.size();
    if (v1 >= nv || v2 >= nv || v3 >= nv) return false;  // BuildError::InvalidVertex
    uint32_t a = uint32_t(v1), b = uint32_t(v2), c = uint32_t(v3);
    if (edge_map.count(ekey(b, c)) || edge_map.count(ekey(c, a)) || edge_map.count(ekey(a, b)))
      return true;  // non-manifold face skipped
    uint32_t c1 = corner_from(b, c, a);
    uint32_t c2 = corner_from(c, a, b);
    uint32_t c3 = corner_from(a, b, c);
    vertex_corners[a].insert(c1);
    vertex_corners[b].insert(c2);
    vertex_corners[c].insert(c3);
    return true;
  }
  template <class F>
  void corners_around_vertex(uint32_t v, F visit) const {
    uint32_t w = prev(vcorner[v]);
    uint32_t started = w;
    bool border = false;
    for (size_t guard = 0; guard < cvertex.size() + 3; ++guard) {
      visit(next(w));
      w = prev(w);
      if (copp[w] == NONE) { border = true; break; }
      w = copp[w];
      if (w == started) break;
    }
    w = started;
    if (border && copp[w] != NONE) {
      w = copp[w];
      for (size_t guard = 0; guard < cvertex.size() + 3; ++guard) {
        visit(prev(w));
        w = next(w);
        if (copp[w] == NONE) break;
        w = copp[w];
      }
    }
  }
  void finish() {
    for (size_t v = 0; v < pos.size(); ++v)
      if (vcorner[v] == NONE) vdeleted[v] = 1;
    for (auto& kv : vertex_corners) {
      uint32_t vid = kv.first;
      auto& corners = kv.second;
      if (vdeleted[vid]) continue;
      corners_around_vertex(vid, [&](uint32_t c) { corners.erase(c); });
      V3 p = pos[vid];
      while (!corners.empty()) {
        uint32_t ci = *corners.begin();
        corners.erase(corners.begin());
        uint32_t dup = add_vertex(p, ci);
        std::vector<uint32_t> around;
        corners_around_vertex(dup, [&](uint32_t c) { around.push_back(c); });
        for (uint32_t c : around) {
          cvertex[c] = dup;
          corners.erase(c);
        }
      }
    }
  }
  size_t num_faces() const { return cvertex.size() / 3; }
  size_t num_vertices() const {
    size_t n = 0;
    for (auto d : vdeleted) n += d == 0;
    return n;
  }
};

struct PosKey {
  uint32_t x, y, z;
  bool operator==(const PosKey& o) const { return x == o.x && y == o.y && z == o.z; }
};
struct PosKeyHash {
  size_t operator()(const PosKey& k) const {
    uint64_t h = uint64_t(k.x) * 0x9E3779B97F4A7C15ull ^ uint64_t(k.y) * 0xC2B2AE3D27D4EB4Full ^
                 uint64_t(k.z) * 0x165667B19E3779F9ull;
    return size_t(h ^ (h >> 31));
  }
};

// algo/merge_points.rs:12-41: exact equality (-0 == +0; NaN never merges)
inline void merge_points(const std::vector<V3>& pts, std::vector<V3>& uniq, std::vector<size_t>& idx) {
  std::unordered_map<PosKey, size_t, PosKeyHash> map;
  auto bits = [](float f) {
    if (f == 0.0f) f = 0.0f;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
  };
  uniq.clear();
  idx.clear();
  for (const V3& p : pts) {
    bool nan = std::isnan(p.x) || std::isnan(p.y) || std::isnan(p.z);
    PosKey k{bits(p.x), bits(p.y), bits(p.z)};
    if (!nan) {
      auto it = map.find(k);
      if (it != map.end()) { idx.push_back(it->second); continue; }
      map.emplace(k, uniq.size());
    }
    idx.push_back(uniq.size());
    uniq.push_back(p);
  }
}

// builder.rs:292-309
inline CornerTableB corner_table_from_soup(const std::vector<V3>& soup) {
  std::vector<V3> uniq;
  std::vector<size_t> idx;
  merge_points(soup, uniq, idx);
  CornerTableB ct;
  for (const V3& p : uniq) ct.add_vertex(p);
  for (size_t i = 0; i + 2 < idx.size(); i += 3)
    if (!ct.add_face(idx[i], idx[i + 1], idx[i + 2])) { ct.failed = true; return ct; }
  ct.finish();
  return ct;
}

}  // namespace orc
