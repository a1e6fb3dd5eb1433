// ORACLE — test infrastructure only (see oracle_core.hpp).
//
// Volume::from_fn (voxel/volume/mod.rs:40-72) and the VolumeBuilder
// primitives sphere, cuboid and iwp (voxel/volume/builder.rs:21-76), restated
// with the reference's f32 operation order.
#pragma once

#include <cmath>
#include <functional>

#include "oracle_ops.hpp"

namespace orc {

// volume/mod.rs:40-72: every grid point idx*h of the box, kept (active) where
// |f| <= (band + 1) * h.
inline Volume from_fn(float h, V3 mn, V3 mx, int64_t band, const std::function<float(const V3&)>& f) {
  auto g = std::make_unique<Grid>();
  const float nb = float(band + 1) * h;
  const int64_t x0 = int64_t(std::floor(mn.x / h)), y0 = int64_t(std::floor(mn.y / h)),
                z0 = int64_t(std::floor(mn.z / h));
  const int64_t x1 = int64_t(std::ceil(mx.x / h)), y1 = int64_t(std::ceil(mx.y / h)),
                z1 = int64_t(std::ceil(mx.z / h));
  for (int64_t x = x0; x <= x1; ++x)
    for (int64_t y = y0; y <= y1; ++y)
      for (int64_t z = z0; z <= z1; ++z) {
        const V3 p = v3(float(x) * h, float(y) * h, float(z) * h);
        const float v = f(p);
        if (std::fabs(v) > nb) continue;
        g->insert(i3(x, y, z), v);
      }
  return Volume{std::move(g), h};
}

// Box3::contains_point / squared_distance (geometry/primitives/box3.rs:96-122)
inline bool box_contains(const V3& mn, const V3& mx, const V3& p) {
  return p.x >= mn.x && p.x <= mx.x && p.y >= mn.y && p.y <= mx.y && p.z >= mn.z && p.z <= mx.z;
}
inline float box_sq_dist(const V3& mn, const V3& mx, const V3& p) {
  float sq = 0.0f;
  const float pc[3] = {p.x, p.y, p.z}, lo[3] = {mn.x, mn.y, mn.z}, hi[3] = {mx.x, mx.y, mx.z};
  for (int i = 0; i < 3; ++i) {
    if (pc[i] < lo[i]) sq += (lo[i] - pc[i]) * (lo[i] - pc[i]);
    if (pc[i] > hi[i]) sq += (pc[i] - hi[i]) * (pc[i] - hi[i]);
  }
  return sq;
}

inline V3 add_scalar(const V3& a, float s) { return v3(a.x + s, a.y + s, a.z + s); }

// builder.rs:21-31
inline Volume build_sphere(float h, float radius, V3 origin) {
  const int64_t band = 1;
  const float offset = radius + float(band) * h;
  return from_fn(h, add_scalar(origin, -offset), add_scalar(origin, offset), band,
                 [&](const V3& p) { return norm(p - origin) - radius; });
}

// builder.rs:33-54
inline Volume build_cuboid(float h, V3 mn, V3 mx) {
  const int64_t band = 1;
  const float offset = float(band) * h;
  return from_fn(h, add_scalar(mn, -offset), add_scalar(mx, offset), band, [&](const V3& p) {
    if (box_contains(mn, mx, p))
      return -std::fmin(std::fmin(std::fmin(std::fmin(std::fmin(p.x - mn.x, mx.x - p.x), p.y - mn.y), mx.y - p.y),
                                  p.z - mn.z),
                        mx.z - p.z);
    return std::sqrt(box_sq_dist(mn, mx, p));
  });
}

// builder.rs:57-76
inline Volume build_iwp(float h, V3 mn, V3 mx, float cell) {
  const float inv = 1.0f / cell;
  const V3 bmin = add_scalar(mn, -h), bmax = add_scalar(mx, h);
  return from_fn(h, bmin, bmax, 2, [&](const V3& p) {
    const float x = p.x * inv, y = p.y * inv, z = p.z * inv;
    const float cx = std::cos(x), cy = std::cos(y), cz = std::cos(z);
    const float v = -(cx + cy + cz - 0.51f * (cx * cy + cy * cz + cz * cx) - 1.0f);
    if (!box_contains(mn, mx, p)) return std::sqrt(box_sq_dist(bmin, bmax, p));
    return v * cell;
  });
}

// from_fn over caller-sampled values: values[((x - x0) * ny + (y - y0)) * nz + (z - z0)]
inline Volume from_samples(float h, int64_t band, const int64_t* idx_min, const int64_t* dims, const float* values) {
  auto g = std::make_unique<Grid>();
  const float nb = float(band + 1) * h;
  for (int64_t i = 0; i < dims[0]; ++i)
    for (int64_t j = 0; j < dims[1]; ++j)
      for (int64_t k = 0; k < dims[2]; ++k) {
        const float v = values[(i * dims[1] + j) * dims[2] + k];
        if (std::fabs(v) > nb) continue;
        g->insert(i3(idx_min[0] + i, idx_min[1] + j, idx_min[2] + k), v);
      }
  return Volume{std::move(g), h};
}

}  // namespace orc
