// ORACLE — test infrastructure only (see oracle_core.hpp).
//
// Marching-cubes surface of a volume, as the GPU mesher builds it:
// the reference's cube enumeration, corner values and edge intersections
// (voxel/meshing/marching_cubes.rs:967-1181), polygons from face segments
// directed around each face's outward normal, the bilinear asymptotic
// decider on faces with four crossings, and a fan triangulation from the
// lowest edge of each cycle.  The reference's MC33 case tables are not
// restated; where the reference's tiling differs (interior ambiguities,
// diagonal choices) the triangles differ while the vertex positions and, for
// cubes without ambiguity, the triangle count agree.
#pragma once

#include <cmath>
#include <vector>

#include "oracle_mesh.hpp"

namespace orc {

namespace mcx {
// corner pairs of the 12 edges, lower corner first (axis x: 0, y: 1, z: 2)
static const int EDGE[12][2] = {{0, 1}, {1, 2}, {3, 2}, {0, 3}, {4, 5}, {5, 6},
                                {7, 6}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
static const int EDGE_AXIS[12] = {0, 1, 0, 1, 0, 1, 0, 1, 2, 2, 2, 2};
// faces, corners counter-clockwise seen from outside the cube
static const int FACE[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4},
                               {3, 7, 6, 2}, {0, 4, 7, 3}, {1, 2, 6, 5}};
inline int edge_of(int a, int b) {
  for (int e = 0; e < 12; ++e)
    if ((EDGE[e][0] == a && EDGE[e][1] == b) || (EDGE[e][0] == b && EDGE[e][1] == a)) return e;
  return -1;
}
}  // namespace mcx

// Triangles (9 floats, world units) of the cube at voxel `vox`.
inline void mc_cube_tris(const Grid& g, const I3& vox, float voxel_size, std::vector<float>& out) {
  float raw[8], v[8];
  for (int i = 0; i < 8; ++i) {
    const float* p = g.at(i3(vox.x + CUBE_OFF[i][0], vox.y + CUBE_OFF[i][1], vox.z + CUBE_OFF[i][2]));
    if (!p) return;
    raw[i] = *p;
    float x = *p;
    if (std::fabs(x) < 1e-6f) x = std::copysign(1e-6f, x);  // marching_cubes.rs:1160-1181
    v[i] = x;
  }
  bool in[8];
  int nin = 0;
  for (int i = 0; i < 8; ++i) {
    in[i] = v[i] < 0.0f;
    nin += in[i];
  }
  if (nin == 0 || nin == 8) return;
  int next[12];
  for (int e = 0; e < 12; ++e) next[e] = -1;
  for (int f = 0; f < 6; ++f) {
    const int* c = mcx::FACE[f];
    int k = 0;
    for (int s = 0; s < 4; ++s) k += in[c[s]] != in[c[(s + 1) & 3]];
    if (k == 2) {
      int entry = -1, exit = -1;
      for (int s = 0; s < 4; ++s) {
        const int a = c[s], b = c[(s + 1) & 3];
        if (!in[a] && in[b]) entry = mcx::edge_of(a, b);
        if (in[a] && !in[b]) exit = mcx::edge_of(a, b);
      }
      next[entry] = exit;
    } else if (k == 4) {
      const int p = in[c[0]] ? 0 : 1;  // corners p and p + 2 are inside
      const float prod_in = v[c[p]] * v[c[p + 2]], prod_out = v[c[(p + 1) & 3]] * v[c[(p + 3) & 3]];
      if (prod_in > prod_out) {
        // the inside corners join through the face: cut off each outside corner q
        for (int q = (p + 1) & 3, t = 0; t < 2; ++t, q = (q + 2) & 3)
          next[mcx::edge_of(c[q], c[(q + 1) & 3])] = mcx::edge_of(c[(q + 3) & 3], c[q]);
      } else {
        // cut off each inside corner r
        for (int r = p, t = 0; t < 2; ++t, r = (r + 2) & 3)
          next[mcx::edge_of(c[(r + 3) & 3], c[r])] = mcx::edge_of(c[r], c[(r + 1) & 3]);
      }
    }
  }
  // intersection points (ComputeEdgeIntersections::compute_intersection)
  V3 pt[12];
  for (int e = 0; e < 12; ++e) {
    const int a = mcx::EDGE[e][0], b = mcx::EDGE[e][1];
    if (in[a] == in[b]) continue;
    const float va = std::fmax(std::fabs(raw[a]), 1e-6f), vb = std::fmax(std::fabs(raw[b]), 1e-6f);
    const float t = va / (va + vb);
    float q[3] = {float(vox.x + CUBE_OFF[a][0]), float(vox.y + CUBE_OFF[a][1]), float(vox.z + CUBE_OFF[a][2])};
    q[mcx::EDGE_AXIS[e]] = q[mcx::EDGE_AXIS[e]] + t;
    pt[e] = v3(q[0] * voxel_size, q[1] * voxel_size, q[2] * voxel_size);
  }
  bool seen[12] = {false};
  for (int e0 = 0; e0 < 12; ++e0) {
    if (next[e0] < 0 || seen[e0]) continue;
    int poly[12], n = 0;
    for (int e = e0; !seen[e] && n < 12; e = next[e]) {
      seen[e] = true;
      poly[n++] = e;
    }
    for (int i = 1; i + 1 < n; ++i) {
      const V3 a = pt[poly[0]], b = pt[poly[i]], c = pt[poly[i + 1]];
      if (norm_sq(cross(b - a, c - a)) == 0.0f) continue;  // Triangle3::is_degenerate
      const V3 t3[3] = {a, b, c};
      for (const V3& p : t3) {
        out.push_back(p.x);
        out.push_back(p.y);
        out.push_back(p.z);
      }
    }
  }
}

// MarchingCubesMesher::mesh (marching_cubes.rs:43-63, 969-1011): every cube of
// every leaf, then the cubes on the six faces of every active tile, in the
// reference's visiting order (a cube on a tile's edge is visited once per face).
inline std::vector<float> mc_mesh(const Grid& g, float voxel_size) {
  std::vector<float> out;
  g.visit_leafs(
      [&](const Leaf3& l) {
        for (int a = 0; a < 8; ++a)
          for (int b = 0; b < 8; ++b)
            for (int c = 0; c < 8; ++c) mc_cube_tris(g, i3(l.origin.x + a, l.origin.y + b, l.origin.z + c), voxel_size, out);
      },
      [&](I3 o, int s, float) {
        for (int i = 0; i < s; ++i)
          for (int j = 0; j < s; ++j) {
            mc_cube_tris(g, i3(o.x, o.y + i, o.z + j), voxel_size, out);          // left
            mc_cube_tris(g, i3(o.x + s - 1, o.y + i, o.z + j), voxel_size, out);  // right
            mc_cube_tris(g, i3(o.x + i, o.y + j, o.z + s - 1), voxel_size, out);  // top
            mc_cube_tris(g, i3(o.x + i, o.y + j, o.z), voxel_size, out);          // bottom
            mc_cube_tris(g, i3(o.x + i, o.y + s - 1, o.z + j), voxel_size, out);  // front
            mc_cube_tris(g, i3(o.x + i, o.y, o.z + j), voxel_size, out);          // back
          }
      });
  return out;
}

}  // namespace orc
