// Volume::from_fn (voxel/volume/mod.rs:40-72) and the VolumeBuilder
// primitives sphere, cuboid and iwp (voxel/volume/builder.rs:21-76) on the GPU.
//
// from_fn evaluates a field at every grid point idx * h of the box
// [floor(min / h), ceil(max / h)] and keeps the points with |f| <= (band+1) h
// as active voxels; the leaves of such voxels are created with 0.0 in their
// other voxels.  Here one warp takes one leaf of the leaf-aligned box: a
// first pass flags leaves with an active voxel, a scan numbers them, and a
// second pass evaluates the field again and writes values and masks.  Leaves
// come out in (x, y, z) order of their origins.
//
// The field is a device functor: the three primitives in closed form with the
// reference's f32 operation order, or values the caller sampled (the Rust
// closure of from_fn runs where the caller is; its samples are uploaded).
#include <cub/device/device_scan.cuh>

#include <cmath>

#include "bs_internal.cuh"

namespace bs {

namespace {

struct Box3i {
  long long lo[3], hi[3];  // inclusive grid-point range
};

// Box3::contains_point / squared_distance (geometry/primitives/box3.rs:96-122)
__device__ __forceinline__ bool box_contains(F3 mn, F3 mx, F3 p) {
  return p.x >= mn.x && p.x <= mx.x && p.y >= mn.y && p.y <= mx.y && p.z >= mn.z && p.z <= mx.z;
}
__device__ __forceinline__ float box_sq_dist(F3 mn, F3 mx, F3 p) {
  float sq = 0.0f;
  const float pc[3] = {p.x, p.y, p.z}, lo[3] = {mn.x, mn.y, mn.z}, hi[3] = {mx.x, mx.y, mx.z};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (pc[i] < lo[i]) {
      const float d = fsub(lo[i], pc[i]);
      sq = fadd(sq, fmul(d, d));
    }
    if (pc[i] > hi[i]) {
      const float d = fsub(pc[i], hi[i]);
      sq = fadd(sq, fmul(d, d));
    }
  }
  return sq;
}

// grid point of an index: idx.cast() * voxel_size (mod.rs:57)
__device__ __forceinline__ F3 grid_point(long long x, long long y, long long z, float h) {
  return f3(fmul(float(x), h), fmul(float(y), h), fmul(float(z), h));
}

// builder.rs:29: (p - origin).norm() - radius
struct SphereField {
  F3 origin;
  float radius, h;
  __device__ float operator()(long long x, long long y, long long z) const {
    const F3 p = grid_point(x, y, z, h);
    const float dx = fsub(p.x, origin.x), dy = fsub(p.y, origin.y), dz = fsub(p.z, origin.z);
    return fsub(fsqrt(fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz))), radius);
  }
};

// builder.rs:41-53
struct CuboidField {
  F3 mn, mx;
  float h;
  __device__ float operator()(long long x, long long y, long long z) const {
    const F3 p = grid_point(x, y, z, h);
    if (box_contains(mn, mx, p)) {
      float m = fminf(fsub(p.x, mn.x), fsub(mx.x, p.x));
      m = fminf(m, fsub(p.y, mn.y));
      m = fminf(m, fsub(mx.y, p.y));
      m = fminf(m, fsub(p.z, mn.z));
      m = fminf(m, fsub(mx.z, p.z));
      return -m;
    }
    return fsqrt(box_sq_dist(mn, mx, p));
  }
};

// builder.rs:65-75 (cosf of CUDA, which may differ from the host libm by an ulp or two)
struct IwpField {
  F3 mn, mx, bmin, bmax;
  float inv, cell, h;
  __device__ float operator()(long long x, long long y, long long z) const {
    const F3 p = grid_point(x, y, z, h);
    const float cx = cosf(fmul(p.x, inv)), cy = cosf(fmul(p.y, inv)), cz = cosf(fmul(p.z, inv));
    const float pair = fadd(fadd(fmul(cx, cy), fmul(cy, cz)), fmul(cz, cx));
    const float v = -fsub(fsub(fadd(fadd(cx, cy), cz), fmul(0.51f, pair)), 1.0f);
    if (!box_contains(mn, mx, p)) return fsqrt(box_sq_dist(bmin, bmax, p));
    return fmul(v, cell);
  }
};

// Values sampled by the caller, x-major over the grid-point box.
struct SampleField {
  const float* values;
  long long x0, y0, z0, ny, nz;
  __device__ float operator()(long long x, long long y, long long z) const {
    return values[((x - x0) * ny + (y - y0)) * nz + (z - z0)];
  }
};

struct LeafGrid {
  long long ox, oy, oz;  // origin of the first candidate leaf
  long long ny, nz;      // candidate leaves along y and z
};

constexpr int FN_WARPS = 8;

// One warp per candidate leaf; voxel o = 32 j + lane of word j.
template <class Field, bool WRITE>
__global__ void __launch_bounds__(32 * FN_WARPS) k_from_fn(Field f, Box3i box, LeafGrid lg, uint64_t n_cand, float band,
                                                           uint32_t* __restrict__ flag, const uint32_t* __restrict__ pos,
                                                           int4* __restrict__ org, float* __restrict__ val,
                                                           uint32_t* __restrict__ msk) {
  const int lane = threadIdx.x & 31;
  const uint64_t c = blockIdx.x * uint64_t(FN_WARPS) + (threadIdx.x >> 5);
  if (c >= n_cand) return;
  if (WRITE && !flag[c]) return;
  const long long iz = (long long)(c % uint64_t(lg.nz)), t = (long long)(c / uint64_t(lg.nz));
  const long long iy = t % lg.ny, ix = t / lg.ny;
  const long long bx = lg.ox + 8 * ix, by = lg.oy + 8 * iy, bz = lg.oz + 8 * iz;
  const uint64_t d = WRITE ? pos[c] : 0;
  uint32_t any = 0;
  for (int j = 0; j < 16; ++j) {
    const int o = 32 * j + lane;
    const long long x = bx + (o >> 6), y = by + ((o >> 3) & 7), z = bz + (o & 7);
    const bool inside = x >= box.lo[0] && x <= box.hi[0] && y >= box.lo[1] && y <= box.hi[1] && z >= box.lo[2] &&
                        z <= box.hi[2];
    float v = 0.0f;
    bool act = false;
    if (inside) {
      v = f(x, y, z);
      act = !(fabsf(v) > band);  // mod.rs:60-62 keeps NaN, as the reference
    }
    const uint32_t word = __ballot_sync(0xffffffffu, act);
    any |= word;
    if (WRITE) {
      val[d * 512 + o] = act ? v : 0.0f;
      if (lane == 0) msk[d * 16 + j] = word;
    }
  }
  if (lane == 0) {
    if (WRITE) org[d] = make_int4(int(bx), int(by), int(bz), 0);
    else flag[c] = any ? 1u : 0u;
  }
}

__global__ void k_count_bits_fn(const uint32_t* __restrict__ m, uint64_t n_words, unsigned long long* out) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  unsigned long long c = i < n_words ? __popc(m[i]) : 0;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

inline F3 hf3(float x, float y, float z) { return F3{x, y, z}; }

inline long long floor8(long long v) { return v >= 0 ? (v / 8) * 8 : -(((-v) + 7) / 8) * 8; }

// Host f32 arithmetic kept one rounding per operation (no contraction).
inline float h_div(float a, float b) {
  volatile float r = a / b;
  return r;
}
inline float h_add(float a, float b) {
  volatile float r = a + b;
  return r;
}
inline float h_mul(float a, float b) {
  volatile float r = a * b;
  return r;
}

Box3i index_box(const float mn[3], const float mx[3], float h) {
  Box3i b;
  for (int i = 0; i < 3; ++i) {
    const double lo = std::floor(double(h_div(mn[i], h))), hi = std::ceil(double(h_div(mx[i], h)));
    // leaf keys carry 21 bits of brick coordinate per axis
    if (!(lo >= -8388600.0 && hi <= 8388600.0)) fail(BS_ERR_CAPACITY, "from_fn: grid extent beyond +-2^23 voxels");
    b.lo[i] = (long long)lo;
    b.hi[i] = (long long)hi;
  }
  return b;
}

template <class Field>
bs_volume* build_volume(bs_ctx* ctx, const Field& f, const Box3i& box, float h, long long band_width) {
  cudaStream_t s = ctx->stream;
  const float band = h_mul(float(band_width + 1), h);
  LeafGrid lg;
  lg.ox = floor8(box.lo[0]);
  lg.oy = floor8(box.lo[1]);
  lg.oz = floor8(box.lo[2]);
  const long long nx = (floor8(box.hi[0]) - lg.ox) / 8 + 1;
  lg.ny = (floor8(box.hi[1]) - lg.oy) / 8 + 1;
  lg.nz = (floor8(box.hi[2]) - lg.oz) / 8 + 1;
  const double cand = double(nx) * double(lg.ny) * double(lg.nz);
  if (cand > double((1ull << 31) - 2)) fail(BS_ERR_CAPACITY, "from_fn: more than 2^31 candidate leaves");
  const uint64_t n_cand = uint64_t(nx) * uint64_t(lg.ny) * uint64_t(lg.nz);
  bs_volume* vol = new bs_volume(ctx);
  vol->h = h;
  try {
    DBuf<uint32_t> flag(ctx, n_cand + 1), pos(ctx, n_cand + 1);
    BS_CUDA(cudaMemsetAsync(flag.p + n_cand, 0, sizeof(uint32_t), s));
    const unsigned grid = unsigned((n_cand + FN_WARPS - 1) / FN_WARPS);
    BS_KERNEL(ctx, "k_from_fn_count", (k_from_fn<Field, false><<<grid, 32 * FN_WARPS, 0, s>>>(f, box, lg, n_cand, band, flag.p, nullptr,
                                                                                        nullptr, nullptr, nullptr)));
    size_t tmp = 0;
    BS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, flag.p, pos.p, n_cand + 1, s));
    {
      DBuf<uint8_t> t(ctx, tmp);
      BS_CUDA(cub::DeviceScan::ExclusiveSum(t.p, tmp, flag.p, pos.p, n_cand + 1, s));
    }
    uint32_t nl = 0;
    read_back(ctx, &nl, pos.p + n_cand, sizeof nl);
    vol->n_leaves = nl;
    if (nl) {
      vol->d_origins = dalloc<int4>(ctx, nl);
      vol->d_values = dalloc<float>(ctx, uint64_t(nl) * 512);
      vol->d_masks = dalloc<uint32_t>(ctx, uint64_t(nl) * 16);
      BS_KERNEL(ctx, "k_from_fn_write", (k_from_fn<Field, true><<<grid, 32 * FN_WARPS, 0, s>>>(f, box, lg, n_cand, band, flag.p, pos.p,
                                                                                         vol->d_origins, vol->d_values,
                                                                                         vol->d_masks)));
      DBuf<unsigned long long> cnt(ctx, 1);
      BS_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), s));
      BS_KERNEL(ctx, "k_count_bits_fn", (k_count_bits_fn<<<unsigned((uint64_t(nl) * 16 + 255) / 256), 256, 0, s>>>(vol->d_masks, uint64_t(nl) * 16, cnt.p)));
      unsigned long long na = 0;
      read_back(ctx, &na, cnt.p, sizeof na);
      vol->n_active = na;
    }
  } catch (...) {
    delete vol;
    throw;
  }
  return vol;
}

}  // namespace

// builder.rs:21-31
bs_volume* volume_sphere_impl(bs_ctx* ctx, float h, float radius, const float origin[3]) {
  if (!(h > 0.0f) || !(radius >= 0.0f)) fail(BS_ERR_INVALID_ARG, "sphere: voxel size and radius must be positive");
  const float offset = h_add(radius, h_mul(1.0f, h));
  float mn[3], mx[3];
  for (int i = 0; i < 3; ++i) {
    mn[i] = h_add(origin[i], -offset);
    mx[i] = h_add(origin[i], offset);
  }
  SphereField f{hf3(origin[0], origin[1], origin[2]), radius, h};
  return build_volume(ctx, f, index_box(mn, mx, h), h, 1);
}

// builder.rs:33-54
bs_volume* volume_cuboid_impl(bs_ctx* ctx, float h, const float mn[3], const float mx[3]) {
  if (!(h > 0.0f)) fail(BS_ERR_INVALID_ARG, "cuboid: voxel size must be positive");
  const float offset = h_mul(1.0f, h);
  float gmn[3], gmx[3];
  for (int i = 0; i < 3; ++i) {
    gmn[i] = h_add(mn[i], -offset);
    gmx[i] = h_add(mx[i], offset);
  }
  CuboidField f{hf3(mn[0], mn[1], mn[2]), hf3(mx[0], mx[1], mx[2]), h};
  return build_volume(ctx, f, index_box(gmn, gmx, h), h, 1);
}

// builder.rs:57-76
bs_volume* volume_iwp_impl(bs_ctx* ctx, float h, const float mn[3], const float mx[3], float cell) {
  if (!(h > 0.0f) || !(cell > 0.0f)) fail(BS_ERR_INVALID_ARG, "iwp: voxel and cell size must be positive");
  float bmn[3], bmx[3];
  for (int i = 0; i < 3; ++i) {
    bmn[i] = h_add(mn[i], -h);
    bmx[i] = h_add(mx[i], h);
  }
  IwpField f{hf3(mn[0], mn[1], mn[2]), hf3(mx[0], mx[1], mx[2]), hf3(bmn[0], bmn[1], bmn[2]), hf3(bmx[0], bmx[1], bmx[2]),
             h_div(1.0f, cell), cell, h};
  return build_volume(ctx, f, index_box(bmn, bmx, h), h, 2);
}

// mod.rs:40-72 over caller-sampled values (device pointer), x-major over
// dims[0] x dims[1] x dims[2] grid points starting at index idx_min.
bs_volume* volume_from_samples_impl(bs_ctx* ctx, float h, long long band_width, const long long idx_min[3],
                                    const unsigned long long dims[3], const float* d_values) {
  if (!(h > 0.0f) || band_width < 0) fail(BS_ERR_INVALID_ARG, "from_fn: voxel size must be positive, band >= 0");
  Box3i box;
  for (int i = 0; i < 3; ++i) {
    if (dims[i] == 0) fail(BS_ERR_EMPTY, "from_fn: empty sample grid");
    box.lo[i] = idx_min[i];
    box.hi[i] = idx_min[i] + (long long)dims[i] - 1;
    if (box.lo[i] < -8388600 || box.hi[i] > 8388600) fail(BS_ERR_CAPACITY, "from_fn: grid extent beyond +-2^23 voxels");
  }
  SampleField f{d_values, idx_min[0], idx_min[1], idx_min[2], (long long)dims[1], (long long)dims[2]};
  return build_volume(ctx, f, box, h, band_width);
}

}  // namespace bs
