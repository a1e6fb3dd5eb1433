// ORACLE — test infrastructure only (an analysis tool, not a checker): a CPU
// restatement of the library's winding-number tree build (Morton order of
// the triangle centroids, PLOC with a +-16 window and surface-area distance,
// mutual nearest neighbours merged; refit with area-weighted dipole centres
// and min(box bound, children's spheres) radii) and of its warp-coherent
// traversal (a node is summed through its far field only when it is far for
// all 32 lanes of the warp, otherwise opened; one-triangle leaves), used to
// rank tree designs by the node visits and evaluations a warp makes.
//
// Variants: a binned-SAH top (12 bins of the triangles' box centres on the
// largest axis, the rule of aabb_tree.rs:422-514) down to segments of at most S triangles with
// PLOC inside them (S = 1: a full binned-SAH tree), subtrees of at most
// `leafmax` triangles evaluated exactly as one leaf, and three node radii:
// the library's rule, the reference's box bound (aabb_tree.rs:738-741), or
// the farthest vertex below the node.
//
// Usage: tree_sim vertices.f32 triangles.u32 warps.f32 S leafmax radius [values.f32]
//   S: 0 = PLOC alone; radius: 0 library, 1 box bound, 2 farthest vertex.
//   warps.f32: groups of 32 query points (3 floats each).  With values.f32
//   each lane's winding number is written there: the order-2 far field of
//   aabb_tree.rs:662-671, 803-816 for the nodes the warp takes as far, the
//   solid angle of aabb_tree.rs:582-615 for the triangles it takes exactly.
#include <algorithm>
#include <cmath>
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <vector>

namespace {

std::vector<char> read_file(const char* path) {
  std::vector<char> b;
  FILE* f = fopen(path, "rb");
  if (!f) return b;
  fseek(f, 0, SEEK_END);
  const long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  b.resize(size_t(n));
  if (fread(b.data(), 1, b.size(), f) != b.size()) b.clear();
  fclose(f);
  return b;
}

uint64_t spread21(uint64_t v) {
  v &= 0x1fffffull;
  v = (v | v << 32) & 0x1f00000000ffffull;
  v = (v | v << 16) & 0x1f0000ff0000ffull;
  v = (v | v << 8) & 0x100f00f00f00f00full;
  v = (v | v << 4) & 0x10c30c30c30c30c3ull;
  v = (v | v << 2) & 0x1249249249249249ull;
  return v;
}

struct Box {
  float lo[3], hi[3];
  void add(const Box& o) {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], o.lo[k]);
      hi[k] = std::max(hi[k], o.hi[k]);
    }
  }
  float half_area() const {
    const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return dx * dy + dx * dz + dy * dz;
  }
};
Box empty_box() { return Box{{1e30f, 1e30f, 1e30f}, {-1e30f, -1e30f, -1e30f}}; }

struct Cluster {
  Box b;
  int node;  // >= 0 internal, < 0 leaf ~index
};

struct Leaf {
  float v[9], c[3], a[3], area, r;
  Box b;
};

struct Node {
  float p[3], r;
  int c0, c1, ntri;
  float a[3], B[9];  // order-1 vector and order-2 matrix about p
};

}  // namespace

int main(int argc, char** argv) {
  if (argc < 7) {
    fprintf(stderr, "usage: tree_sim vertices.f32 triangles.u32 warps.f32 S leafmax radius\n");
    return 2;
  }
  const auto vx = read_file(argv[1]), tx = read_file(argv[2]), wx = read_file(argv[3]);
  const int S = atoi(argv[4]), leafmax = atoi(argv[5]), radius = atoi(argv[6]);
  const float* X = reinterpret_cast<const float*>(vx.data());
  const uint32_t* T = reinterpret_cast<const uint32_t*>(tx.data());
  const float* W = reinterpret_cast<const float*>(wx.data());
  const int64_t nv = int64_t(vx.size() / 12), nt = int64_t(tx.size() / 12), nw = int64_t(wx.size() / 384);
  if (nt < 2 || nw < 1) return 2;
  for (int64_t i = 0; i < 3 * nt; ++i)
    if (int64_t(T[i]) >= nv) return 2;

  // leaves in Morton order of the centroids (ties keep the input order)
  float cmin[3] = {1e30f, 1e30f, 1e30f}, cmax[3] = {-1e30f, -1e30f, -1e30f};
  std::vector<float> cen(size_t(3 * nt));
  for (int64_t i = 0; i < nt; ++i)
    for (int k = 0; k < 3; ++k) {
      const float c = (X[3 * T[3 * i] + k] + X[3 * T[3 * i + 1] + k] + X[3 * T[3 * i + 2] + k]) * (1.0f / 3.0f);
      cen[3 * i + k] = c;
      cmin[k] = std::min(cmin[k], c);
      cmax[k] = std::max(cmax[k], c);
    }
  std::vector<std::pair<uint64_t, uint32_t>> key(static_cast<size_t>(nt));
  for (int64_t i = 0; i < nt; ++i) {
    uint64_t q[3];
    for (int k = 0; k < 3; ++k) {
      const float e = cmax[k] - cmin[k];
      const float u = std::min(std::max(e > 0.f ? (cen[3 * i + k] - cmin[k]) / e : 0.5f, 0.f), 1.f);
      q[k] = uint64_t(std::min(u * 2097152.0f, 2097151.0f));
    }
    key[size_t(i)] = {(spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]), uint32_t(i)};
  }
  std::stable_sort(key.begin(), key.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  std::vector<Leaf> leaf(static_cast<size_t>(nt));
  std::vector<Cluster> cl(static_cast<size_t>(nt));
  for (int64_t i = 0; i < nt; ++i) {
    Leaf& l = leaf[size_t(i)];
    const uint32_t t = key[size_t(i)].second;
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) l.v[3 * j + k] = X[3 * T[3 * t + j] + k];
    float e[3], f[3];
    for (int k = 0; k < 3; ++k) {
      e[k] = l.v[3 + k] - l.v[k];
      f[k] = l.v[6 + k] - l.v[k];
      l.c[k] = (l.v[k] + l.v[3 + k] + l.v[6 + k]) * (1.0f / 3.0f);
    }
    const float n[3] = {e[1] * f[2] - e[2] * f[1], e[2] * f[0] - e[0] * f[2], e[0] * f[1] - e[1] * f[0]};
    const float len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int k = 0; k < 3; ++k) l.a[k] = len > 0.f ? 0.5f * n[k] : 0.f;
    l.area = len > 0.f ? 0.5f * len : 0.f;
    float d2 = 0.f;
    for (int j = 0; j < 3; ++j) {
      float d = 0.f;
      for (int k = 0; k < 3; ++k) d += (l.v[3 * j + k] - l.c[k]) * (l.v[3 * j + k] - l.c[k]);
      d2 = std::max(d2, d);
    }
    l.r = std::sqrt(d2) * 1.000001f;
    l.b = empty_box();
    for (int j = 0; j < 3; ++j) l.b.add(Box{{l.v[3 * j], l.v[3 * j + 1], l.v[3 * j + 2]}, {l.v[3 * j], l.v[3 * j + 1], l.v[3 * j + 2]}});
    cl[size_t(i)] = Cluster{l.b, ~int(i)};
  }

  // topology: children are recorded before their parents
  std::vector<std::pair<int, int>> child;
  auto ploc = [&](std::vector<Cluster> c) -> int {
    const int R = 16;
    std::vector<int> nn;
    while (c.size() > 1) {
      const int n = int(c.size());
      nn.assign(size_t(n), -1);
      for (int i = 0; i < n; ++i) {
        float best = INFINITY;
        for (int d = -R; d <= R; ++d) {
          if (d == 0 || i + d < 0 || i + d >= n) continue;
          Box m = c[size_t(i)].b;
          m.add(c[size_t(i + d)].b);
          const float a = m.half_area();
          if (a < best) {
            best = a;
            nn[size_t(i)] = i + d;
          }
        }
      }
      std::vector<Cluster> next;
      next.reserve(size_t(n));
      for (int i = 0; i < n; ++i) {
        const int j = nn[size_t(i)];
        const bool mutual = j >= 0 && nn[size_t(j)] == i;
        if (mutual && i < j) {
          Cluster m = c[size_t(i)];
          m.b.add(c[size_t(j)].b);
          child.push_back({c[size_t(i)].node, c[size_t(j)].node});
          m.node = int(child.size()) - 1;
          next.push_back(m);
        } else if (!mutual) {
          next.push_back(c[size_t(i)]);
        }
      }
      if (next.size() == c.size()) exit(3);  // no mutual pair: cannot happen for a finite window
      c.swap(next);
    }
    return c[0].node;
  };
  std::function<int(std::vector<int>&)> sah = [&](std::vector<int>& idx) -> int {
    const int n = int(idx.size());
    if (n <= std::max(S, 1)) {
      std::sort(idx.begin(), idx.end());
      std::vector<Cluster> seg;
      for (int i : idx) seg.push_back(cl[size_t(i)]);
      return n == 1 ? seg[0].node : ploc(seg);
    }
    // centres of the triangles' boxes, as the reference bins them
    auto centre = [&](int i, int k) { return 0.5f * (leaf[size_t(i)].b.lo[k] + leaf[size_t(i)].b.hi[k]); };
    Box cb = empty_box();
    for (int i : idx) {
      const float c[3] = {centre(i, 0), centre(i, 1), centre(i, 2)};
      cb.add(Box{{c[0], c[1], c[2]}, {c[0], c[1], c[2]}});
    }
    int ax = 0;
    for (int k = 1; k < 3; ++k)
      if (cb.hi[k] - cb.lo[k] > cb.hi[ax] - cb.lo[ax]) ax = k;
    const int NB = 12;
    const float ext = cb.hi[ax] - cb.lo[ax];
    auto bin_of = [&](int i) {
      const int b = ext > 0.f ? int(NB * (centre(i, ax) - cb.lo[ax]) / ext) : 0;
      return std::min(std::max(b, 0), NB - 1);
    };
    Box bb[NB];
    int cnt[NB] = {0};
    for (int b = 0; b < NB; ++b) bb[b] = empty_box();
    for (int i : idx) {
      const int b = bin_of(i);
      ++cnt[b];
      bb[b].add(leaf[size_t(i)].b);
    }
    double best = 1e300;
    int split = -1;
    for (int s = 1; s < NB; ++s) {
      Box l = empty_box(), r = empty_box();
      int nl = 0, nr = 0;
      for (int b = 0; b < NB; ++b) {
        if (!cnt[b]) continue;
        (b < s ? l : r).add(bb[b]);
        (b < s ? nl : nr) += cnt[b];
      }
      if (!nl || !nr) continue;
      const double cost = double(l.half_area()) * nl + double(r.half_area()) * nr;
      if (cost < best) {
        best = cost;
        split = s;
      }
    }
    std::vector<int> li, ri;
    if (split < 0) {  // every centroid in one bin: halves of the Morton order
      std::sort(idx.begin(), idx.end());
      li.assign(idx.begin(), idx.begin() + n / 2);
      ri.assign(idx.begin() + n / 2, idx.end());
    } else {
      for (int i : idx) (bin_of(i) < split ? li : ri).push_back(i);
    }
    std::vector<int>().swap(idx);
    const int a = sah(li), b = sah(ri);
    child.push_back({a, b});
    return int(child.size()) - 1;
  };
  int root;
  if (S > 0) {
    std::vector<int> all(static_cast<size_t>(nt));
    for (int64_t i = 0; i < nt; ++i) all[size_t(i)] = int(i);
    root = sah(all);
  } else {
    root = ploc(cl);
  }

  // refit: area-weighted dipole centres and radii
  const int ni = int(child.size());
  struct Sum {
    double cx, cy, cz, s;
    Box b;
    int ntri;
    double a[3], m[9];  // sum of area * normal; sum of centroid (area * normal)^T
  };
  std::vector<Sum> sum(static_cast<size_t>(ni));
  std::vector<Node> node(static_cast<size_t>(ni));
  auto leaf_sum = [&](int i) {
    const Leaf& l = leaf[size_t(i)];
    Sum s{double(l.area) * l.c[0], double(l.area) * l.c[1], double(l.area) * l.c[2], double(l.area), l.b, 1, {}, {}};
    for (int r = 0; r < 3; ++r) {
      s.a[r] = l.a[r];
      for (int q = 0; q < 3; ++q) s.m[3 * r + q] = double(l.c[r]) * l.a[q];
    }
    return s;
  };
  auto sphere = [&](int c, float* p, float& r) {
    const float* q = c >= 0 ? node[size_t(c)].p : leaf[size_t(~c)].c;
    for (int k = 0; k < 3; ++k) p[k] = q[k];
    r = c >= 0 ? node[size_t(c)].r : leaf[size_t(~c)].r;
  };
  for (int id = 0; id < ni; ++id) {
    const Sum a = child[size_t(id)].first >= 0 ? sum[size_t(child[size_t(id)].first)] : leaf_sum(~child[size_t(id)].first);
    const Sum b = child[size_t(id)].second >= 0 ? sum[size_t(child[size_t(id)].second)] : leaf_sum(~child[size_t(id)].second);
    Sum s{a.cx + b.cx, a.cy + b.cy, a.cz + b.cz, a.s + b.s, a.b, a.ntri + b.ntri, {}, {}};
    s.b.add(b.b);
    for (int k = 0; k < 3; ++k) s.a[k] = a.a[k] + b.a[k];
    for (int k = 0; k < 9; ++k) s.m[k] = a.m[k] + b.m[k];
    sum[size_t(id)] = s;
    Node& q = node[size_t(id)];
    q.p[0] = float(s.cx / s.s);
    q.p[1] = float(s.cy / s.s);
    q.p[2] = float(s.cz / s.s);
    float d0 = 0.f, d1 = 0.f;
    for (int k = 0; k < 3; ++k) {
      d0 += (s.b.lo[k] - q.p[k]) * (s.b.lo[k] - q.p[k]);
      d1 += (s.b.hi[k] - q.p[k]) * (s.b.hi[k] - q.p[k]);
    }
    float pa[3], ra, pb[3], rb;
    sphere(child[size_t(id)].first, pa, ra);
    sphere(child[size_t(id)].second, pb, rb);
    auto dist = [&](const float* u) {
      return std::sqrt((u[0] - q.p[0]) * (u[0] - q.p[0]) + (u[1] - q.p[1]) * (u[1] - q.p[1]) +
                       (u[2] - q.p[2]) * (u[2] - q.p[2]));
    };
    const float box_bound = std::sqrt(std::max(d0, d1));
    q.r = radius == 1 ? box_bound : std::min(box_bound, std::max(dist(pa) + ra, dist(pb) + rb) * 1.000001f);
    q.c0 = child[size_t(id)].first;
    q.c1 = child[size_t(id)].second;
    q.ntri = s.ntri;
    for (int r = 0; r < 3; ++r) {
      q.a[r] = float(s.a[r]);
      for (int c = 0; c < 3; ++c) q.B[3 * r + c] = float(s.m[3 * r + c] - double(q.p[r]) * s.a[c]);
    }
  }
  if (radius == 2) {
    std::vector<int> st;
    for (int id = 0; id < ni; ++id) {
      float far2 = 0.f;
      st.assign(1, id);
      while (!st.empty()) {
        const int c = st.back();
        st.pop_back();
        if (c >= 0) {
          st.push_back(node[size_t(c)].c0);
          st.push_back(node[size_t(c)].c1);
          continue;
        }
        const Leaf& l = leaf[size_t(~c)];
        for (int j = 0; j < 3; ++j) {
          float d = 0.f;
          for (int k = 0; k < 3; ++k) d += (l.v[3 * j + k] - node[size_t(id)].p[k]) * (l.v[3 * j + k] - node[size_t(id)].p[k]);
          far2 = std::max(far2, d);
        }
      }
      node[size_t(id)].r = std::sqrt(far2) * 1.000001f;
    }
  }

  // warp-coherent traversal at accuracy scale 2
  const float beta2 = 4.0f;
  const float inv4pi = float(1.0 / (4.0 * M_PI));
  std::vector<float> value(argc > 7 ? static_cast<size_t>(32 * nw) : 0);
  auto far_field = [&](int nd, const float* x) -> float {  // order 1 + 2 about the node centre
    float p[3], r, a[3], B[9] = {0.f};
    sphere(nd, p, r);
    if (nd >= 0) {
      for (int k = 0; k < 3; ++k) a[k] = node[size_t(nd)].a[k];
      for (int k = 0; k < 9; ++k) B[k] = node[size_t(nd)].B[k];
    } else {
      for (int k = 0; k < 3; ++k) a[k] = leaf[size_t(~nd)].a[k];
    }
    const float d[3] = {p[0] - x[0], p[1] - x[1], p[2] - x[2]};
    const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const float ri = 1.0f / std::sqrt(r2), ri2 = ri * ri, inv = ri2 * ri * inv4pi;
    float rbr = 0.f;
    for (int i = 0; i < 3; ++i) rbr += d[i] * (B[3 * i] * d[0] + B[3 * i + 1] * d[1] + B[3 * i + 2] * d[2]);
    return inv * ((a[0] * d[0] + a[1] * d[1] + a[2] * d[2] + (B[0] + B[4] + B[8])) - 3.0f * ri2 * rbr);
  };
  auto solid_angle = [&](int li, const float* x) -> float {  // Van Oosterom-Strackee
    const float* v = leaf[size_t(li)].v;
    float A[3], Bv[3], Cv[3];
    for (int k = 0; k < 3; ++k) {
      A[k] = v[k] - x[k];
      Bv[k] = v[3 + k] - x[k];
      Cv[k] = v[6 + k] - x[k];
    }
    auto dot = [](const float* u, const float* w) { return u[0] * w[0] + u[1] * w[1] + u[2] * w[2]; };
    const float la = std::sqrt(dot(A, A)), lb = std::sqrt(dot(Bv, Bv)), lc = std::sqrt(dot(Cv, Cv));
    const float bc[3] = {Bv[1] * Cv[2] - Bv[2] * Cv[1], Bv[2] * Cv[0] - Bv[0] * Cv[2], Bv[0] * Cv[1] - Bv[1] * Cv[0]};
    const float num = dot(A, bc);
    const float den = la * lb * lc + dot(A, Bv) * lc + dot(Bv, Cv) * la + dot(Cv, A) * lb;
    return num == 0.f ? 0.f : 2.0f * std::atan2(num, den) * inv4pi;
  };
  double visits = 0, far = 0, exact = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : visits, far, exact)
  for (int64_t w = 0; w < nw; ++w) {
    const float* q = W + 96 * w;
    double sum[32] = {0.0};
    std::vector<int> st{root}, below;
    while (!st.empty()) {
      const int nd = st.back();
      st.pop_back();
      visits += 1;
      float p[3], r;
      sphere(nd, p, r);
      bool all_far = true;
      for (int l = 0; l < 32 && all_far; ++l) {
        const float dx = p[0] - q[3 * l], dy = p[1] - q[3 * l + 1], dz = p[2] - q[3 * l + 2];
        all_far = dx * dx + dy * dy + dz * dz > r * r * beta2;
      }
      if (all_far) {
        far += 1;
        if (!value.empty())
          for (int l = 0; l < 32; ++l) sum[l] += far_field(nd, q + 3 * l);
      } else if (nd < 0 || node[size_t(nd)].ntri <= leafmax) {
        below.assign(1, nd);
        while (!below.empty()) {  // the triangles below, exactly
          const int c = below.back();
          below.pop_back();
          if (c >= 0) {
            below.push_back(node[size_t(c)].c0);
            below.push_back(node[size_t(c)].c1);
            continue;
          }
          exact += 1;
          if (!value.empty())
            for (int l = 0; l < 32; ++l) sum[l] += solid_angle(~c, q + 3 * l);
        }
      } else {
        st.push_back(node[size_t(nd)].c1);
        st.push_back(node[size_t(nd)].c0);
      }
    }
    if (!value.empty())
      for (int l = 0; l < 32; ++l) value[size_t(32 * w + l)] = float(sum[l]);
  }
  if (!value.empty()) {
    FILE* f = fopen(argv[7], "wb");
    if (!f || fwrite(value.data(), sizeof(float), value.size(), f) != value.size()) return 4;
    fclose(f);
  }
  printf("S %d leafmax %d radius %d: warps %lld, per warp: node visits %.1f, far-field %.1f, exact %.1f, "
         "FLOP per lane %.0f\n",
         S, leafmax, radius, (long long)nw, visits / nw, far / nw, exact / nw, (31.0 * far + 70.0 * exact) / nw);
  return 0;
}
