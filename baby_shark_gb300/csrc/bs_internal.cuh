// Internal definitions shared by the CUDA translation units of
// libbs_gb300.so: the context (device, stream, stream-ordered memory pool,
// launch counter), the device layout of a volume, and IEEE-exact float
// helpers used where results must match the reference bit for bit.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/baby_shark_gb300.h"

// ------------------------------------------------------------- context ----
struct bs_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // second stream of the library's own (the tree build overlaps the distance
  // pass on it); created on first use, ordered against `stream` by events
  cudaStream_t side = nullptr;
  cudaMemPool_t pool = nullptr;
  uint64_t launches = 0;
  std::string last_error;
  void* h_pinned = nullptr;  // small pinned staging area for size read-backs
  size_t h_pinned_bytes = 0;
  // optional per-stage timing with CUDA events on the context stream
  bool timing = false;
  struct Pending {
    std::string name;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  struct Stage {
    double ms = 0.0;
    uint64_t launches = 0;
  };
  std::map<std::string, Stage> stages;
  // launch shapes chosen by bs_autotune_mesh_to_volume: threads per brick of
  // the distance pass (64, 128, 256) and warps per block of the sign pass
  // (2, 4, 8)
  int tune_dist_threads = 128;
  int tune_dist_batch = 32;  // sub-triangles per warp tile of the distance pass (8, 16, 32)
  int tune_wn_warps = 4;
  // counters of the last mesh -> volume, offset or dual contouring call
  // (see bs_ctx_last_counters); [8] names the call that wrote them
  uint64_t last_stats[16] = {};
  // lifetime: the caller's handle plus one reference per live volume, so a
  // volume freed after bs_ctx_destroy still finds its stream and pool
  int refs = 1;
};

// Drops one reference; the context is torn down with the last one.
void bs_ctx_release(bs_ctx* ctx);
// Folds the recorded per-kernel event pairs into ctx->stages.
extern "C" void bs_ctx_resolve_stages(bs_ctx* ctx);

namespace bs {

struct Error {
  bs_status status;
  std::string msg;
};

// Throws Error on a CUDA failure; the C-ABI wrappers catch and translate.
#define BS_CUDA(call)                                                                      \
  do {                                                                                     \
    cudaError_t e__ = (call);                                                              \
    if (e__ != cudaSuccess) {                                                              \
      throw ::bs::Error{e__ == cudaErrorMemoryAllocation ? BS_ERR_OOM : BS_ERR_CUDA,       \
                        std::string(#call) + ": " + cudaGetErrorString(e__)};              \
    }                                                                                      \
  } while (0)

#define BS_CHECK_LAUNCH(ctx)                                                               \
  do {                                                                                     \
    (ctx)->launches++;                                                                     \
    cudaError_t e__ = cudaGetLastError();                                                  \
    if (e__ != cudaSuccess)                                                                \
      throw ::bs::Error{BS_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e__)}; \
  } while (0)

inline void fail(bs_status s, const std::string& m) { throw Error{s, m}; }

// Launches one kernel (the `launch` statement), counts it, checks the launch
// error and, when stage timing is on, brackets it with CUDA events.
#define BS_KERNEL(ctx, name, launch)                                   \
  do {                                                                 \
    cudaEvent_t e0__ = nullptr;                                        \
    if ((ctx)->timing) {                                               \
      BS_CUDA(cudaEventCreate(&e0__));                                 \
      BS_CUDA(cudaEventRecord(e0__, (ctx)->stream));                   \
    }                                                                  \
    launch;                                                            \
    BS_CHECK_LAUNCH(ctx);                                              \
    if ((ctx)->timing) {                                               \
      cudaEvent_t e1__ = nullptr;                                      \
      BS_CUDA(cudaEventCreate(&e1__));                                 \
      BS_CUDA(cudaEventRecord(e1__, (ctx)->stream));                   \
      (ctx)->pending.push_back(bs_ctx::Pending{name, e0__, e1__});     \
    }                                                                  \
  } while (0)

// Stream-ordered device allocation from the context's pool.
template <class T>
T* dalloc(bs_ctx* ctx, size_t count) {
  if (count == 0) count = 1;
  void* p = nullptr;
  BS_CUDA(cudaMallocFromPoolAsync(&p, count * sizeof(T), ctx->pool, ctx->stream));
  return static_cast<T*>(p);
}
inline void dfree(bs_ctx* ctx, void* p) {
  if (p) cudaFreeAsync(p, ctx->stream);
}

// RAII device buffer for temporaries of one call.
template <class T>
struct DBuf {
  bs_ctx* ctx = nullptr;
  T* p = nullptr;
  size_t n = 0;
  DBuf() {}
  DBuf(bs_ctx* c, size_t count) : ctx(c), p(dalloc<T>(c, count)), n(count) {}
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : ctx(o.ctx), p(o.p), n(o.n) { o.p = nullptr; }
  DBuf& operator=(DBuf&& o) noexcept {
    reset();
    ctx = o.ctx; p = o.p; n = o.n; o.p = nullptr;
    return *this;
  }
  ~DBuf() { reset(); }
  void reset() {
    if (p) dfree(ctx, p);
    p = nullptr;
    n = 0;
  }
  T* release() { T* q = p; p = nullptr; n = 0; return q; }
  T* get() const { return p; }
};

// Reads `bytes` from device to host through the pinned staging area and
// waits for the stream.
void read_back(bs_ctx* ctx, void* host, const void* dev, size_t bytes);

}  // namespace bs

struct Upper;  // internal-node levels, volume_upper.cuh

// ------------------------------------------------------------- volume -----
// Leaves (8^3 bricks) sorted by origin (x, then y, then z).  Tiles are the
// active constant regions of the reference's internal nodes (128^3 and
// 4096^3 voxels); they only appear after boolean operations.
struct bs_volume {
  explicit bs_volume(bs_ctx* c) : ctx(c) { ctx->refs++; }
  bs_volume(const bs_volume&) = delete;
  bs_volume& operator=(const bs_volume&) = delete;
  bs_ctx* ctx = nullptr;
  float h = 1.0f;
  uint64_t n_leaves = 0;
  int4* d_origins = nullptr;   // [n] (x, y, z, 0)
  float* d_values = nullptr;   // [n][512]
  uint32_t* d_masks = nullptr; // [n][16]
  uint64_t n_active = 0;
  // active tiles
  uint64_t n_tiles = 0;
  int4* d_tiles = nullptr;     // [n] (x, y, z, size)
  float* d_tile_values = nullptr;
  // upper tree levels (see volume_ops.cu): kept for boolean semantics
  Upper* upper = nullptr;
  // cached dual-contouring output (world-unit triangles)
  float* d_dc_tris = nullptr;
  uint64_t n_dc_tris = 0;
  bool dc_valid = false;
  float dc_h = 0.0f;
  int dc_mode = 0;
  // cached marching-cubes output (world-unit triangles)
  float* d_mc_tris = nullptr;
  uint64_t n_mc_tris = 0;
  bool mc_valid = false;
  float mc_h = 0.0f;
  ~bs_volume();
};

namespace bs {

// ------------------------------------------------ IEEE-exact float math ---
// Each helper rounds once (round-to-nearest-even) and is never contracted
// into a fused multiply-add, matching the reference's Rust f32 arithmetic.
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

// Quotient a / b, correctly rounded, from y = RN(1/b) (computed once and
// shared by every division by b): Markstein's division (P. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Develop. 34(1), 1990): q0 = RN(a y), the remainder
// r = a - b q0 exact through a fused multiply-add, q1 = RN(q0 + r y).  Valid
// where a, b and a / b stay clear of overflow and underflow (callers keep
// |a| and |b| in [2^-60, 2^60]); each step then scales exactly with the
// operands' exponents, so it equals IEEE division everywhere in that range
// when it does on every pair of significands — bs_diag_check_division checks
// all 2^46 pairs against __fdiv_rn.  For a = -0 it returns +0 (IEEE: -0).
__device__ __forceinline__ float mdiv(float a, float b, float y) {
  const float q0 = __fmul_rn(a, y);
  return __fmaf_rn(__fmaf_rn(-b, q0, a), y, q0);
}
__device__ __forceinline__ bool mdiv_range(float x) {  // |x| in [2^-60, 2^60]
  const float ax = fabsf(x);
  return ax >= 0x1p-60f && ax <= 0x1p60f;
}

struct F3 {
  float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 add3(F3 a, F3 b) { return {fadd(a.x, b.x), fadd(a.y, b.y), fadd(a.z, b.z)}; }
__device__ __forceinline__ F3 sub3(F3 a, F3 b) { return {fsub(a.x, b.x), fsub(a.y, b.y), fsub(a.z, b.z)}; }
__device__ __forceinline__ F3 scale3(F3 a, float s) { return {fmul(a.x, s), fmul(a.y, s), fmul(a.z, s)}; }
// (x1*x2 + y1*y2) + z1*z2
__device__ __forceinline__ float dot3(F3 a, F3 b) {
  return fadd(fadd(fmul(a.x, b.x), fmul(a.y, b.y)), fmul(a.z, b.z));
}
__device__ __forceinline__ F3 cross3(F3 a, F3 b) {
  return {fsub(fmul(a.y, b.z), fmul(a.z, b.y)), fsub(fmul(a.z, b.x), fmul(a.x, b.z)),
          fsub(fmul(a.x, b.y), fmul(a.y, b.x))};
}
__device__ __forceinline__ F3 min3(F3 a, F3 b) {
  return {a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z};
}
__device__ __forceinline__ F3 max3(F3 a, F3 b) {
  return {a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z};
}

// Closest point on triangle (a, b, c) to p, Voronoi-region method of
// Ericson, "Real-Time Collision Detection" 5.1.5, with the operation order of
// triangle3.rs:317-382; returns |closest - p|^2 (before the square root of
// the reference's norm(), mesh_to_volume.rs:155).  The square root is
// monotonic and correctly rounded, so sqrt(min |.|^2) == min sqrt(|.|^2)
// bit for bit and callers take it once per voxel.
__device__ __forceinline__ float point_triangle_dist2(F3 a, F3 b, F3 c, F3 p) {
  F3 ab = sub3(b, a), ac = sub3(c, a), ap = sub3(p, a);
  float d1 = dot3(ab, ap), d2 = dot3(ac, ap);
  F3 q;
  if (d1 <= 0.0f && d2 <= 0.0f) {
    q = a;
  } else {
    F3 bp = sub3(p, b);
    float d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) {
      q = b;
    } else {
      float vc = fsub(fmul(d1, d4), fmul(d3, d2));
      if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        float v = fdiv(d1, fsub(d1, d3));
        q = add3(a, scale3(ab, v));
      } else {
        F3 cp = sub3(p, c);
        float d5 = dot3(ab, cp), d6 = dot3(ac, cp);
        if (d6 >= 0.0f && d5 <= d6) {
          q = c;
        } else {
          float vb = fsub(fmul(d5, d2), fmul(d1, d6));
          if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
            float w = fdiv(d2, fsub(d2, d6));
            q = add3(a, scale3(ac, w));
          } else {
            float va = fsub(fmul(d3, d6), fmul(d5, d4));
            float d43 = fsub(d4, d3), d56 = fsub(d5, d6);
            if (va <= 0.0f && d43 >= 0.0f && d56 >= 0.0f) {
              float w = fdiv(d43, fadd(d43, d56));
              q = add3(b, scale3(sub3(c, b), w));
            } else {
              float denom = fdiv(1.0f, fadd(fadd(va, vb), vc));
              float v = fmul(vb, denom);
              float w = fmul(vc, denom);
              q = add3(add3(a, scale3(ab, v)), scale3(ac, w));
            }
          }
        }
      }
    }
  }
  F3 d = sub3(q, p);
  return dot3(d, d);
}

// The same with the triangle's edges ab = b - a, ac = c - a, cb = c - b
// computed once by the caller (the identical roundings).
__device__ __forceinline__ float point_triangle_dist2_e(F3 a, F3 b, F3 c, F3 ab, F3 ac, F3 cb, F3 p) {
  F3 ap = sub3(p, a);
  float d1 = dot3(ab, ap), d2 = dot3(ac, ap);
  F3 q;
  if (d1 <= 0.0f && d2 <= 0.0f) {
    q = a;
  } else {
    F3 bp = sub3(p, b);
    float d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    if (d3 >= 0.0f && d4 <= d3) {
      q = b;
    } else {
      float vc = fsub(fmul(d1, d4), fmul(d3, d2));
      if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        float v = fdiv(d1, fsub(d1, d3));
        q = add3(a, scale3(ab, v));
      } else {
        F3 cp = sub3(p, c);
        float d5 = dot3(ab, cp), d6 = dot3(ac, cp);
        if (d6 >= 0.0f && d5 <= d6) {
          q = c;
        } else {
          float vb = fsub(fmul(d5, d2), fmul(d1, d6));
          if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
            float w = fdiv(d2, fsub(d2, d6));
            q = add3(a, scale3(ac, w));
          } else {
            float va = fsub(fmul(d3, d6), fmul(d5, d4));
            float d43 = fsub(d4, d3), d56 = fsub(d5, d6);
            if (va <= 0.0f && d43 >= 0.0f && d56 >= 0.0f) {
              float w = fdiv(d43, fadd(d43, d56));
              q = add3(b, scale3(cb, w));
            } else {
              float denom = fdiv(1.0f, fadd(fadd(va, vb), vc));
              float v = fmul(vb, denom);
              float w = fmul(vc, denom);
              q = add3(add3(a, scale3(ab, v)), scale3(ac, w));
            }
          }
        }
      }
    }
  }
  F3 d = sub3(q, p);
  return dot3(d, d);
}

}  // namespace bs

// Releases the upper-level (internal node) tables of a volume (volume_ops.cu).
void bs_volume_free_upper(bs_volume* v);

// Entry points implemented by the translation units (C++ linkage).
namespace bs {
bs_volume* mesh_to_volume_impl(bs_ctx* ctx, const float* d_xyz, uint64_t nv, const uint32_t* d_tri,
                               uint64_t nt, const bs_m2v_params& p);
void volume_release(bs_volume* v);
std::vector<bs_volume*> mesh_to_volume_batch_impl(bs_ctx* ctx, const float* d_xyz, const uint32_t* d_tri,
                                                  const std::vector<uint64_t>& n_vtx,
                                                  const std::vector<uint64_t>& n_tri,
                                                  const std::vector<bs_m2v_params>& params);
bs_volume* volume_clone_impl(bs_ctx* ctx, const bs_volume* v);
bs_status exact_winding_numbers_impl(bs_ctx* ctx, const float* d_xyz, uint64_t nv, const uint32_t* d_tri,
                                     uint64_t nt, const float* d_pts, uint64_t np, double* d_out);
void marching_cubes_impl(bs_ctx* ctx, bs_volume* v, float voxel_size);
bs_volume* volume_sphere_impl(bs_ctx* ctx, float h, float radius, const float origin[3]);
bs_volume* volume_cuboid_impl(bs_ctx* ctx, float h, const float mn[3], const float mx[3]);
bs_volume* volume_iwp_impl(bs_ctx* ctx, float h, const float mn[3], const float mx[3], float cell);
bs_volume* volume_from_samples_impl(bs_ctx* ctx, float h, long long band_width, const long long idx_min[3],
                                    const unsigned long long dims[3], const float* d_values);
bs_volume* volume_csg_impl(bs_ctx* ctx, bs_volume* a, bs_volume* b, int op);
void volume_offset_impl(bs_ctx* ctx, bs_volume* v, float distance);
// mode 0: the reference's particle solver; 1: the float64 QEF vertex
void dual_contour_impl(bs_ctx* ctx, bs_volume* v, float voxel_size, int mode = 0);
}  // namespace bs
