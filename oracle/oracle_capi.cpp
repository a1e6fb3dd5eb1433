// ORACLE — test infrastructure only (see oracle_core.hpp).
//
// C entry points of the oracle for the test-suite (ctypes).  Volumes are
// exported as leaves in tree order: origin (3 x int32), 512 values, and a
// 512-bit active mask as 16 x uint32 (bit i&31 of word i>>5 = voxel i, voxel
// index x<<6 | y<<3 | z).
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <string>

#include "oracle_build.hpp"
#include "oracle_mc.hpp"
#include "oracle_mesh.hpp"

using namespace orc;

namespace {

std::vector<Tri> tris_from_indexed(const float* xyz, int64_t nv, const uint32_t* tri, int64_t nt) {
  std::vector<Tri> t;
  t.reserve(size_t(nt));
  for (int64_t i = 0; i < nt; ++i) {
    uint32_t a = tri[3 * i], b = tri[3 * i + 1], c = tri[3 * i + 2];
    if (int64_t(a) >= nv || int64_t(b) >= nv || int64_t(c) >= nv) continue;
    t.push_back(Tri{v3(xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]),
                    v3(xyz[3 * b], xyz[3 * b + 1], xyz[3 * b + 2]),
                    v3(xyz[3 * c], xyz[3 * c + 1], xyz[3 * c + 2])});
  }
  return t;
}

std::vector<const Leaf3*> leaves_of(const Grid& g) {
  std::vector<const Leaf3*> out;
  g.visit_leafs([&](const Leaf3& l) { out.push_back(&l); }, [](I3, int, float) {});
  return out;
}

// Small trees used by the ports of the reference's unit tests.
struct SmallTree {
  virtual ~SmallTree() {}
  virtual void insert(int64_t x, int64_t y, int64_t z, float v) = 0;
  virtual void flood_fill() = 0;
  virtual int sign_at(int64_t x, int64_t y, int64_t z) = 0;
  virtual int values(float* out) = 0;  // leaf kinds only
};
template <class T>
struct SmallT : SmallTree {
  std::unique_ptr<T> t = std::make_unique<T>(i3(0, 0, 0));
  void insert(int64_t x, int64_t y, int64_t z, float v) override { t->insert(i3(x, y, z), v); }
  void flood_fill() override { t->flood_fill(); }
  int sign_at(int64_t x, int64_t y, int64_t z) override { return t->sign_at(i3(x, y, z)) == Sign::Neg ? -1 : 1; }
  int values(float* out) override {
    if constexpr (T::IS_LEAF) {
      std::memcpy(out, t->values, sizeof(t->values));
      return T::N;
    } else {
      return -1;
    }
  }
};
struct SmallRoot : SmallTree {
  Root<Leaf<1>> t;
  void insert(int64_t x, int64_t y, int64_t z, float v) override { t.insert(i3(x, y, z), v); }
  void flood_fill() override { t.flood_fill(); }
  int sign_at(int64_t x, int64_t y, int64_t z) override { return t.sign_at(i3(x, y, z)) == Sign::Neg ? -1 : 1; }
  int values(float*) override { return -1; }
};

}  // namespace

extern "C" {

int orc_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// MeshToVolume::convert (mesh_to_volume.rs:52-73).  stats (optional, 6 x int64):
// sub-triangles, triangle/voxel pairs, far-field evaluations, leaf-triangle
// evaluations, band voxels, voxels with |wn - 0.2| < 1e-3.  wn_out (optional,
// one float per band voxel in export order).  Returns NULL for an empty mesh.
void* orc_mesh_to_volume(const float* xyz, int64_t nv, const uint32_t* tri, int64_t nt, float h,
                         int64_t band, int64_t* stats, float* wn_out) {
  auto tris = tris_from_indexed(xyz, nv, tri, nt);
  MeshToVolumeStats st;
  std::vector<float> wn;
  auto g = mesh_to_volume(tris, h, band, &st, wn_out ? &wn : nullptr);
  if (!g) return nullptr;
  if (stats) {
    stats[0] = int64_t(st.n_subtris);
    stats[1] = int64_t(st.n_pairs);
    stats[2] = int64_t(st.n_far);
    stats[3] = int64_t(st.n_leaf_tris);
    stats[4] = int64_t(st.n_band);
    stats[5] = int64_t(st.n_near_threshold);
  }
  if (wn_out) std::memcpy(wn_out, wn.data(), wn.size() * sizeof(float));
  return new Volume{std::move(g), h};
}

void orc_volume_free(void* v) { delete static_cast<Volume*>(v); }

// Builds an oracle volume from exported leaves (origins, all 512 values,
// masks) so that results computed elsewhere can be checked by the oracle.
void* orc_volume_from_leaves(const int32_t* origins, const float* values, const uint32_t* masks, int64_t n,
                             float voxel_size) {
  auto g = std::make_unique<Grid>();
  for (int64_t i = 0; i < n; ++i) {
    auto leaf = Leaf3::empty(i3(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]));
    std::memcpy(leaf->values, values + 512 * i, 512 * sizeof(float));
    for (int o = 0; o < 512; ++o)
      if ((masks[16 * i + (o >> 5)] >> (o & 31)) & 1u) leaf->mask.on(o);
    g->insert_leaf_at(std::move(leaf));
  }
  return new Volume{std::move(g), voxel_size};
}
// Volume::from_fn and VolumeBuilder (voxel/volume/mod.rs:40-72, volume/builder.rs:21-76)
void* orc_volume_sphere(float h, float radius, float ox, float oy, float oz) {
  return new Volume(build_sphere(h, radius, v3(ox, oy, oz)));
}
void* orc_volume_cuboid(float h, const float* mn, const float* mx) {
  return new Volume(build_cuboid(h, v3(mn[0], mn[1], mn[2]), v3(mx[0], mx[1], mx[2])));
}
void* orc_volume_iwp(float h, const float* mn, const float* mx, float cell) {
  return new Volume(build_iwp(h, v3(mn[0], mn[1], mn[2]), v3(mx[0], mx[1], mx[2]), cell));
}
void* orc_volume_from_samples(float h, int64_t band, const int64_t* idx_min, const int64_t* dims, const float* values) {
  return new Volume(from_samples(h, band, idx_min, dims, values));
}
void* orc_volume_clone(void* v) {
  auto* s = static_cast<Volume*>(v);
  return new Volume{s->grid->clone(), s->voxel_size};
}
int64_t orc_volume_num_leaves(void* v) {
  return int64_t(leaves_of(*static_cast<Volume*>(v)->grid).size());
}
void orc_volume_export(void* v, int32_t* origins, float* values, uint32_t* masks) {
  auto ls = leaves_of(*static_cast<Volume*>(v)->grid);
  for (size_t i = 0; i < ls.size(); ++i) {
    const Leaf3* l = ls[i];
    origins[3 * i] = int32_t(l->origin.x);
    origins[3 * i + 1] = int32_t(l->origin.y);
    origins[3 * i + 2] = int32_t(l->origin.z);
    if (values) std::memcpy(values + 512 * i, l->values, 512 * sizeof(float));
    if (masks) {
      for (int w = 0; w < 16; ++w) masks[16 * i + w] = 0;
      for (int o = 0; o < 512; ++o)
        if (l->mask.at(o)) masks[16 * i + (o >> 5)] |= 1u << (o & 31);
    }
  }
}
int64_t orc_volume_num_tiles(void* v) {
  int64_t n = 0;
  static_cast<Volume*>(v)->grid->visit_leafs([](const Leaf3&) {}, [&](I3, int, float) { ++n; });
  return n;
}
void orc_volume_export_tiles(void* v, int32_t* origins, int32_t* sizes, float* values) {
  int64_t n = 0;
  static_cast<Volume*>(v)->grid->visit_leafs([](const Leaf3&) {}, [&](I3 o, int s, float val) {
    origins[3 * n] = int32_t(o.x);
    origins[3 * n + 1] = int32_t(o.y);
    origins[3 * n + 2] = int32_t(o.z);
    sizes[n] = s;
    values[n] = val;
    ++n;
  });
}

// Volume::{union, subtract, intersect} consume b (volume/mod.rs:74-93).
int orc_volume_union(void* a, void* b) {
  volume_union(*static_cast<Volume*>(a), std::move(*static_cast<Volume*>(b)));
  delete static_cast<Volume*>(b);
  return 0;
}
int orc_volume_subtract(void* a, void* b) {
  volume_subtract(*static_cast<Volume*>(a), std::move(*static_cast<Volume*>(b)));
  delete static_cast<Volume*>(b);
  return 0;
}
int orc_volume_intersect(void* a, void* b) {
  volume_intersect(*static_cast<Volume*>(a), std::move(*static_cast<Volume*>(b)));
  delete static_cast<Volume*>(b);
  return 0;
}
int orc_volume_flood_fill(void* v) {
  static_cast<Volume*>(v)->grid->flood_fill();
  return 0;
}
// Volume::offset (volume/mod.rs:95-108). Returns 0, or 1 when the sweep met a tile.
int orc_volume_offset(void* v, float d) {
  try {
    volume_offset(*static_cast<Volume*>(v), d);
  } catch (const std::exception&) {
    return 1;
  }
  return 0;
}

// DualContouringMesher::mesh.  Returns the number of triangles written into
// out (9 floats each) when out_cap is large enough, else the required count.
// *status: 0 ok, 1 active tile (the reference panics), 2 gradient without
// neighbours (the reference panics).
// tiles_via_at: 0 stops at active tiles as the reference does, 1 reads them
// through Grid::at (the GPU's extension).
int64_t orc_dual_contour(void* v, float voxel_size, float* out, int64_t out_cap, int* status,
                         int64_t* n_edges, int64_t* n_cells, int tiles_via_at) {
  DcResult r = dual_contour(*static_cast<Volume*>(v)->grid, voxel_size, tiles_via_at != 0);
  if (status) *status = r.status;
  if (n_edges) *n_edges = int64_t(r.n_edges);
  if (n_cells) *n_cells = int64_t(r.n_cells);
  int64_t nt = int64_t(r.tris.size() / 9);
  if (out && out_cap >= nt) std::memcpy(out, r.tris.data(), r.tris.size() * sizeof(float));
  return nt;
}

// Triangles of a marching-cubes extraction (3 x this = MarchingCubesMesher's vertex count).
int64_t orc_mc_count(void* v, int64_t* ambiguous_faces, int64_t* cubes) {
  McCount mc = mc_count(*static_cast<Volume*>(v)->grid);
  if (ambiguous_faces) *ambiguous_faces = int64_t(mc.ambiguous_faces);
  if (cubes) *cubes = int64_t(mc.cubes);
  return int64_t(mc.triangles);
}

// Sub-triangles of MeshToVolume (mesh_to_volume.rs:75-116) with their widened
// integer boxes (124-143): returns the count, fills up to `capacity` records
// of 9 floats and 6 int64 (box min, box max).
int64_t orc_subtriangles(const float* xyz, int64_t nv, const uint32_t* tri, int64_t nt, float voxel_size,
                         int64_t band, float* out_tris, int64_t* out_boxes, int64_t capacity) {
  auto tris = tris_from_indexed(xyz, nv, tri, nt);
  std::vector<Tri> sub;
  for (const Tri& t : tris) subdivide_triangle(t, voxel_size, sub);
  const float inv_h = 1.0f / voxel_size;
  const int64_t n = int64_t(sub.size());
  for (int64_t i = 0; i < std::min(n, capacity); ++i) {
    const Tri& t = sub[size_t(i)];
    const V3 p[3] = {t.a, t.b, t.c};
    for (int k = 0; k < 3; ++k) {
      out_tris[9 * i + 3 * k] = p[k].x;
      out_tris[9 * i + 3 * k + 1] = p[k].y;
      out_tris[9 * i + 3 * k + 2] = p[k].z;
    }
    I3 mn, mx;
    widened_box(t, inv_h, band, mn, mx);
    const int64_t b[6] = {mn.x, mn.y, mn.z, mx.x, mx.y, mx.z};
    for (int k = 0; k < 6; ++k) out_boxes[6 * i + k] = b[k];
  }
  return n;
}

// Marching-cubes triangles of a volume without tiles (oracle_mc.hpp); returns
// the triangle count, copies up to `capacity` triangles.
int64_t orc_marching_cubes(void* v, float voxel_size, float* out, int64_t capacity) {
  std::vector<float> t = mc_mesh(*static_cast<Volume*>(v)->grid, voxel_size);
  const int64_t n = int64_t(t.size() / 9);
  if (out) std::memcpy(out, t.data(), size_t(std::min(n, capacity)) * 9 * sizeof(float));
  return n;
}

// CornerTable::from_triangles_soup / builder_soup().finish().
int orc_corner_table_from_soup(const float* soup, int64_t n_points, int64_t* n_faces, int64_t* n_vertices) {
  std::vector<V3> pts(static_cast<size_t>(n_points));
  for (int64_t i = 0; i < n_points; ++i) pts[size_t(i)] = v3(soup[3 * i], soup[3 * i + 1], soup[3 * i + 2]);
  CornerTableB ct = corner_table_from_soup(pts);
  if (ct.failed) return 1;
  *n_faces = int64_t(ct.num_faces());
  *n_vertices = int64_t(ct.num_vertices());
  return 0;
}

// CornerTable::from_vertex_and_face_slices.  Optional outputs (sized by the
// caller for the final corner/vertex counts): corner -> vertex, corner ->
// opposite corner (-1 none), vertex -> corner (-1 none) and deleted flags.
int orc_corner_table_from_indexed(const float* verts, int64_t nv, const int64_t* faces, int64_t n_idx,
                                  int64_t* n_faces, int64_t* n_vertices, int64_t* n_corners_total,
                                  int64_t* n_vertices_total, int32_t* corner_vertex, int32_t* corner_opp,
                                  int32_t* vertex_corner, uint8_t* vertex_deleted) {
  CornerTableB ct;
  for (int64_t i = 0; i < nv; ++i) ct.add_vertex(v3(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]));
  for (int64_t i = 0; i + 2 < n_idx; i += 3)
    if (!ct.add_face(size_t(faces[i]), size_t(faces[i + 1]), size_t(faces[i + 2]))) {
      // from_vertex_and_face_iters returns an empty table on a build error
      *n_faces = 0;
      *n_vertices = 0;
      return 1;
    }
  ct.finish();
  *n_faces = int64_t(ct.num_faces());
  *n_vertices = int64_t(ct.num_vertices());
  if (n_corners_total) *n_corners_total = int64_t(ct.cvertex.size());
  if (n_vertices_total) *n_vertices_total = int64_t(ct.pos.size());
  for (size_t c = 0; c < ct.cvertex.size(); ++c) {
    if (corner_vertex) corner_vertex[c] = int32_t(ct.cvertex[c]);
    if (corner_opp) corner_opp[c] = ct.copp[c] == CornerTableB::NONE ? -1 : int32_t(ct.copp[c]);
  }
  for (size_t v = 0; v < ct.pos.size(); ++v) {
    if (vertex_corner) vertex_corner[v] = ct.vcorner[v] == CornerTableB::NONE ? -1 : int32_t(ct.vcorner[v]);
    if (vertex_deleted) vertex_deleted[v] = ct.vdeleted[v];
  }
  return 0;
}

// WindingNumbers::from_mesh(..).approximate(p, beta) for a batch of points.
void orc_fast_wn(const float* xyz, int64_t nv, const uint32_t* tri, int64_t nt, const float* pts, int64_t np,
                 float beta, float* out, int64_t* counters) {
  auto tris = tris_from_indexed(xyz, nv, tri, nt);
  WindingNumbers wn;
  wn.build(tris);
  uint64_t nf = 0, nl = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : nf, nl)
  for (int64_t i = 0; i < np; ++i) {
    uint64_t f = 0, l = 0;
    out[i] = wn.approximate(v3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]), beta, &f, &l);
    nf += f;
    nl += l;
  }
  if (counters) {
    counters[0] = int64_t(nf);
    counters[1] = int64_t(nl);
    counters[2] = int64_t(wn.nodes.size());
  }
}

// Exact generalised winding number in FP64 by direct summation over all
// triangles (Van Oosterom–Strackee), the error reference for the far field.
void orc_exact_wn_f64(const float* xyz, int64_t nv, const uint32_t* tri, int64_t nt, const float* pts,
                      int64_t np, double* out) {
  (void)nv;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < np; ++i) {
    double qx = pts[3 * i], qy = pts[3 * i + 1], qz = pts[3 * i + 2];
    double s = 0.0;
    for (int64_t t = 0; t < nt; ++t) {
      double a[3], b[3], c[3];
      for (int k = 0; k < 3; ++k) {
        a[k] = xyz[3 * tri[3 * t] + k];
        b[k] = xyz[3 * tri[3 * t + 1] + k];
        c[k] = xyz[3 * tri[3 * t + 2] + k];
      }
      a[0] -= qx; a[1] -= qy; a[2] -= qz;
      b[0] -= qx; b[1] -= qy; b[2] -= qz;
      c[0] -= qx; c[1] -= qy; c[2] -= qz;
      double la = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
      double lb = std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
      double lc = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
      if (la == 0 || lb == 0 || lc == 0) continue;
      double det = a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) +
                   a[2] * (b[0] * c[1] - b[1] * c[0]);
      double ab = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
      double ac = a[0] * c[0] + a[1] * c[1] + a[2] * c[2];
      double bc = b[0] * c[0] + b[1] * c[1] + b[2] * c[2];
      double den = la * lb * lc + ab * lc + ac * lb + bc * la;
      s += 2.0 * std::atan2(det, den);
    }
    out[i] = s / (4.0 * M_PI);
  }
}

// ---- ports of the reference's unit tests on small trees ----
// kind 0: static_vdb!(f32, 1)   kind 1: static_vdb!(f32, 2)
// kind 2: static_vdb!(f32, 2, 1)  kind 3: dynamic_vdb!(f32, 1)
void* orc_small_new(int kind) {
  switch (kind) {
    case 0: return static_cast<SmallTree*>(new SmallT<Leaf<1>>());
    case 1: return static_cast<SmallTree*>(new SmallT<Leaf<2>>());
    case 2: return static_cast<SmallTree*>(new SmallT<Internal<2, Leaf<1>>>());
    case 3: return static_cast<SmallTree*>(new SmallRoot());
  }
  return nullptr;
}
void orc_small_free(void* t) { delete static_cast<SmallTree*>(t); }
void orc_small_insert(void* t, int64_t x, int64_t y, int64_t z, float v) { static_cast<SmallTree*>(t)->insert(x, y, z, v); }
void orc_small_flood_fill(void* t) { static_cast<SmallTree*>(t)->flood_fill(); }
int orc_small_sign_at(void* t, int64_t x, int64_t y, int64_t z) { return static_cast<SmallTree*>(t)->sign_at(x, y, z); }
int orc_small_values(void* t, float* out) { return static_cast<SmallTree*>(t)->values(out); }

// leaf_node/csg.rs tests: two fully active 2^3 leaves; op 0 union, 1 subtract, 2 intersect.
int orc_leaf1_csg(int op, const float* a, const float* b, float* out) {
  auto l1 = Leaf<1>::empty(i3(0, 0, 0));
  auto l2 = Leaf<1>::empty(i3(0, 0, 0));
  std::memcpy(l1->values, a, 8 * sizeof(float));
  std::memcpy(l2->values, b, 8 * sizeof(float));
  l1->mask.on_all();
  l2->mask.on_all();
  if (op == 0) l1->csg_union(std::move(l2));
  else if (op == 1) l1->csg_subtract(std::move(l2));
  else l1->csg_intersect(std::move(l2));
  std::memcpy(out, l1->values, 8 * sizeof(float));
  return l1->mask.is_full() ? 1 : 0;
}

// init.rs:49-86 tree geometry constants: BRANCHING, BRANCHING_TOTAL and the
// number of children per level of dynamic_vdb!(_, 5, 4, 3).
void orc_tree_constants(int64_t* out) {
  out[0] = Int5::BR; out[1] = Int5::TOTAL; out[2] = Int5::N;
  out[3] = Int4::BR; out[4] = Int4::TOTAL; out[5] = Int4::N;
  out[6] = Leaf3::BR; out[7] = Leaf3::TOTAL; out[8] = Leaf3::N;
}

}  // extern "C"
