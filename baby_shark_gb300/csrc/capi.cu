// C ABI of libbs_gb300.so (include/baby_shark_gb300.h): contexts, volume
// lifetime and export, and the status/exception boundary.  Every entry point
// catches bs::Error (and std::bad_alloc) and returns a bs_status; nothing
// throws across the C boundary.
#include <cstring>
#include <iterator>
#include <new>

#include <cmath>

#include "bs_internal.cuh"

namespace bs {

void read_back(bs_ctx* ctx, void* host, const void* dev, size_t bytes) {
  if (bytes <= ctx->h_pinned_bytes) {
    BS_CUDA(cudaMemcpyAsync(ctx->h_pinned, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    BS_CUDA(cudaStreamSynchronize(ctx->stream));
    std::memcpy(host, ctx->h_pinned, bytes);
  } else {
    BS_CUDA(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    BS_CUDA(cudaStreamSynchronize(ctx->stream));
  }
}

void volume_release(bs_volume* v) { delete v; }

}  // namespace bs

bs_volume::~bs_volume() {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  bs::dfree(ctx, d_origins);
  bs::dfree(ctx, d_values);
  bs::dfree(ctx, d_masks);
  bs::dfree(ctx, d_tiles);
  bs::dfree(ctx, d_tile_values);
  bs::dfree(ctx, d_dc_tris);
  bs::dfree(ctx, d_mc_tris);
  bs_volume_free_upper(this);
  bs_ctx_release(ctx);
}

void bs_ctx_release(bs_ctx* ctx) {
  if (--ctx->refs > 0) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& p : ctx->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  if (ctx->side) {
    cudaStreamSynchronize(ctx->side);
    cudaStreamDestroy(ctx->side);
  }
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

namespace {

template <class F>
bs_status guarded(bs_ctx* ctx, F&& f) {
  try {
    if (ctx) {
      BS_CUDA(cudaSetDevice(ctx->device));
      ctx->last_error.clear();
    }
    f();
    return BS_OK;
  } catch (const bs::Error& e) {
    if (ctx) ctx->last_error = e.msg;
    return e.status;
  } catch (const std::bad_alloc&) {
    if (ctx) ctx->last_error = "host allocation failed";
    return BS_ERR_OOM;
  }
}

}  // namespace

extern "C" {

const char* bs_status_string(bs_status s) {
  switch (s) {
    case BS_OK: return "ok";
    case BS_ERR_INVALID_ARG: return "invalid argument";
    case BS_ERR_EMPTY: return "empty input";
    case BS_ERR_OOM: return "out of device memory";
    case BS_ERR_CAPACITY: return "capacity exceeded";
    case BS_ERR_TIMEOUT: return "device wait timed out";
    case BS_ERR_CUDA: return "CUDA error";
    case BS_ERR_UNSUPPORTED: return "unsupported input";
    case BS_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

bs_status bs_ctx_create(int device, void* stream, bs_ctx** out) {
  if (!out) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return BS_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) return BS_ERR_INVALID_ARG;
  bs_ctx* ctx = new (std::nothrow) bs_ctx();
  if (!ctx) return BS_ERR_OOM;
  ctx->device = device;
  bs_status st = guarded(nullptr, [&] {
    BS_CUDA(cudaSetDevice(device));
    if (stream) {
      ctx->stream = static_cast<cudaStream_t>(stream);
    } else {
      BS_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
      ctx->own_stream = true;
    }
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    BS_CUDA(cudaMemPoolCreate(&ctx->pool, &props));
    uint64_t keep = ~uint64_t(0);  // keep freed blocks cached inside this pool
    BS_CUDA(cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep));
    ctx->h_pinned_bytes = 4096;
    BS_CUDA(cudaMallocHost(&ctx->h_pinned, ctx->h_pinned_bytes));
  });
  if (st != BS_OK) {
    if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return st;
  }
  *out = ctx;
  return BS_OK;
}

bs_status bs_ctx_destroy(bs_ctx* ctx) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  bs_ctx_release(ctx);  // volumes still alive keep the context until they are freed
  return BS_OK;
}

void* bs_ctx_stream(bs_ctx* ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

bs_status bs_ctx_synchronize(bs_ctx* ctx) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  return guarded(ctx, [&] { BS_CUDA(cudaStreamSynchronize(ctx->stream)); });
}

uint64_t bs_ctx_kernel_launches(const bs_ctx* ctx) { return ctx ? ctx->launches : 0; }

const char* bs_ctx_last_error(const bs_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

bs_status bs_ctx_set_stage_timing(bs_ctx* ctx, int enable) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  ctx->timing = enable != 0;
  return BS_OK;
}

void bs_ctx_resolve_stages(bs_ctx* ctx) {
  for (auto& p : ctx->pending) {
    float ms = 0.f;
    BS_CUDA(cudaEventSynchronize(p.b));
    BS_CUDA(cudaEventElapsedTime(&ms, p.a, p.b));
    auto& st = ctx->stages[p.name];
    st.ms += ms;
    st.launches += 1;
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  ctx->pending.clear();
}

bs_status bs_ctx_stage_count(bs_ctx* ctx, int* n) {
  if (!ctx || !n) return BS_ERR_INVALID_ARG;
  return guarded(ctx, [&] {
    bs_ctx_resolve_stages(ctx);
    *n = int(ctx->stages.size());
  });
}

bs_status bs_ctx_stage_info(bs_ctx* ctx, int i, const char** name, double* total_ms, uint64_t* launches) {
  if (!ctx || i < 0 || i >= int(ctx->stages.size())) return BS_ERR_INVALID_ARG;
  auto it = ctx->stages.begin();
  std::advance(it, i);
  if (name) *name = it->first.c_str();
  if (total_ms) *total_ms = it->second.ms;
  if (launches) *launches = it->second.launches;
  return BS_OK;
}

bs_status bs_ctx_stage_reset(bs_ctx* ctx) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  return guarded(ctx, [&] {
    bs_ctx_resolve_stages(ctx);
    ctx->stages.clear();
  });
}

bs_status bs_ctx_last_stats(const bs_ctx* ctx, uint64_t* out8) {
  if (!ctx || !out8) return BS_ERR_INVALID_ARG;
  for (int k = 0; k < 8; ++k) out8[k] = ctx->last_stats[k];
  return BS_OK;
}

bs_status bs_ctx_last_counters(const bs_ctx* ctx, uint64_t* out16) {
  if (!ctx || !out16) return BS_ERR_INVALID_ARG;
  for (int k = 0; k < 16; ++k) out16[k] = ctx->last_stats[k];
  return BS_OK;
}

bs_status bs_ctx_memory(bs_ctx* ctx, uint64_t* used, uint64_t* used_high, uint64_t* reserved) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  return guarded(ctx, [&] {
    unsigned long long u = 0, hi = 0, r = 0;  // the pool attributes are 64-bit counters
    BS_CUDA(cudaMemPoolGetAttribute(ctx->pool, cudaMemPoolAttrUsedMemCurrent, &u));
    BS_CUDA(cudaMemPoolGetAttribute(ctx->pool, cudaMemPoolAttrUsedMemHigh, &hi));
    BS_CUDA(cudaMemPoolGetAttribute(ctx->pool, cudaMemPoolAttrReservedMemCurrent, &r));
    if (used) *used = u;
    if (used_high) *used_high = hi;
    if (reserved) *reserved = r;
  });
}

bs_status bs_ctx_memory_reset(bs_ctx* ctx, int trim) {
  if (!ctx) return BS_ERR_INVALID_ARG;
  return guarded(ctx, [&] {
    unsigned long long zero = 0;
    BS_CUDA(cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrUsedMemHigh, &zero));
    if (trim) {
      BS_CUDA(cudaStreamSynchronize(ctx->stream));
      BS_CUDA(cudaMemPoolTrimTo(ctx->pool, 0));
    }
  });
}

void bs_m2v_params_default(bs_m2v_params* p) {
  if (!p) return;
  p->voxel_size = 1.0f;   // MeshToVolume::default (mesh_to_volume.rs:223-236)
  p->band_width = 0;
  p->wn_beta = 2.0f;      // mesh_to_volume.rs:264
  p->wn_threshold = 0.2f; // mesh_to_volume.rs:266
  p->wn_order = 2;
  p->wn_tree = 0;         // the reference's tree and summation order
}

bs_status bs_mesh_to_volume_device(bs_ctx* ctx, const float* d_xyz, uint64_t nv, const uint32_t* d_tri,
                                   uint64_t nt, const bs_m2v_params* params, bs_volume** out) {
  if (!ctx || !params || !out || (nt && (!d_xyz || !d_tri))) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  return guarded(ctx, [&] { *out = bs::mesh_to_volume_impl(ctx, d_xyz, nv, d_tri, nt, *params); });
}

bs_status bs_mesh_to_volume(bs_ctx* ctx, const float* h_xyz, uint64_t nv, const uint32_t* h_tri, uint64_t nt,
                            const bs_m2v_params* params, bs_volume** out) {
  if (!ctx || !params || !out || (nt && (!h_xyz || !h_tri))) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  return guarded(ctx, [&] {
    if (nt == 0) bs::fail(BS_ERR_EMPTY, "mesh has no triangles");
    bs::DBuf<float> xyz(ctx, 3 * nv);
    bs::DBuf<uint32_t> tri(ctx, 3 * nt);
    BS_CUDA(cudaMemcpyAsync(xyz.p, h_xyz, 3 * nv * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    BS_CUDA(cudaMemcpyAsync(tri.p, h_tri, 3 * nt * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream));
    *out = bs::mesh_to_volume_impl(ctx, xyz.p, nv, tri.p, nt, *params);
  });
}

static bs_status batch_common(bs_ctx* ctx, uint64_t K, const float* xyz, const uint64_t* nv, const uint32_t* tri,
                              const uint64_t* nt, const bs_m2v_params* params, bs_volume** out, bool host) {
  if (!ctx || !nv || !nt || !params || !out) return BS_ERR_INVALID_ARG;
  for (uint64_t m = 0; m < K; ++m) out[m] = nullptr;
  return guarded(ctx, [&] {
    if (K == 0) bs::fail(BS_ERR_EMPTY, "no meshes");
    std::vector<uint64_t> vn(nv, nv + K), tn(nt, nt + K);
    std::vector<bs_m2v_params> ps(params, params + K);
    uint64_t V = 0, T = 0;
    for (uint64_t m = 0; m < K; ++m) {
      V += vn[m];
      T += tn[m];
    }
    if (T && (!xyz || !tri)) bs::fail(BS_ERR_INVALID_ARG, "null vertex or triangle array");
    std::vector<bs_volume*> r;
    if (host) {
      bs::DBuf<float> dx(ctx, std::max<uint64_t>(3 * V, 1));
      bs::DBuf<uint32_t> dt(ctx, std::max<uint64_t>(3 * T, 1));
      if (V) BS_CUDA(cudaMemcpyAsync(dx.p, xyz, 3 * V * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
      if (T) BS_CUDA(cudaMemcpyAsync(dt.p, tri, 3 * T * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream));
      r = bs::mesh_to_volume_batch_impl(ctx, dx.p, dt.p, vn, tn, ps);
    } else {
      r = bs::mesh_to_volume_batch_impl(ctx, xyz, tri, vn, tn, ps);
    }
    for (uint64_t m = 0; m < K; ++m) out[m] = r[m];
  });
}

bs_status bs_mesh_to_volume_batch(bs_ctx* ctx, uint64_t n_meshes, const float* h_xyz, const uint64_t* vertex_counts,
                                  const uint32_t* h_tri, const uint64_t* triangle_counts,
                                  const bs_m2v_params* params, bs_volume** out) {
  return batch_common(ctx, n_meshes, h_xyz, vertex_counts, h_tri, triangle_counts, params, out, true);
}

bs_status bs_mesh_to_volume_batch_device(bs_ctx* ctx, uint64_t n_meshes, const float* d_xyz,
                                         const uint64_t* vertex_counts, const uint32_t* d_tri,
                                         const uint64_t* triangle_counts, const bs_m2v_params* params,
                                         bs_volume** out) {
  return batch_common(ctx, n_meshes, d_xyz, vertex_counts, d_tri, triangle_counts, params, out, false);
}

bs_status bs_winding_numbers_exact(bs_ctx* ctx, const float* d_xyz, uint64_t nv, const uint32_t* d_tri,
                                   uint64_t nt, const float* d_points, uint64_t n_points, double* d_out) {
  if (!ctx || (nt && (!d_xyz || !d_tri)) || (n_points && (!d_points || !d_out))) return BS_ERR_INVALID_ARG;
  return guarded(ctx, [&] { bs::exact_winding_numbers_impl(ctx, d_xyz, nv, d_tri, nt, d_points, n_points, d_out); });
}

bs_status bs_volume_create(bs_ctx* ctx, float voxel_size, bs_volume** out) {
  if (!ctx || !out || !(voxel_size > 0.f) || !std::isfinite(voxel_size)) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  return guarded(ctx, [&] {
    bs_volume* v = new bs_volume(ctx);  // no leaves, no tiles, no internal nodes
    v->h = voxel_size;
    *out = v;
  });
}

bs_status bs_volume_free(bs_volume* v) {
  if (!v) return BS_ERR_INVALID_ARG;
  delete v;
  return BS_OK;
}

bs_status bs_volume_voxel_size(const bs_volume* v, float* out) {
  if (!v || !out) return BS_ERR_INVALID_ARG;
  *out = v->h;
  return BS_OK;
}

bs_status bs_volume_counts(const bs_volume* v, uint64_t* n_leaves, uint64_t* n_tiles, uint64_t* n_active) {
  if (!v) return BS_ERR_INVALID_ARG;
  if (n_leaves) *n_leaves = v->n_leaves;
  if (n_tiles) *n_tiles = v->n_tiles;
  if (n_active) *n_active = v->n_active;
  return BS_OK;
}

bs_status bs_volume_clone(bs_ctx* ctx, const bs_volume* v, bs_volume** out) {
  if (!ctx || !v || !out || v->ctx != ctx) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  return guarded(ctx, [&] { *out = bs::volume_clone_impl(ctx, v); });
}

bs_status bs_volume_from_samples_device(bs_ctx* ctx, float voxel_size, int64_t band_width, const int64_t* idx_min,
                                        const uint64_t* dims, const float* d_values, bs_volume** out) {
  if (!ctx || !idx_min || !dims || !d_values || !out) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  return guarded(ctx, [&] {
    const long long lo[3] = {idx_min[0], idx_min[1], idx_min[2]};
    const unsigned long long d[3] = {dims[0], dims[1], dims[2]};
    *out = bs::volume_from_samples_impl(ctx, voxel_size, band_width, lo, d, d_values);
  });
}

bs_status bs_volume_from_samples(bs_ctx* ctx, float voxel_size, int64_t band_width, const int64_t* idx_min,
                                 const uint64_t* dims, const float* h_values, bs_volume** out) {
  if (!ctx || !idx_min || !dims || !h_values || !out) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  return guarded(ctx, [&] {
    const double n = double(dims[0]) * double(dims[1]) * double(dims[2]);
    if (!(n > 0.0)) bs::fail(BS_ERR_EMPTY, "from_fn: empty sample grid");
    if (n > double(1ull << 36)) bs::fail(BS_ERR_CAPACITY, "from_fn: more than 2^36 samples");
    const uint64_t cnt = dims[0] * dims[1] * dims[2];
    bs::DBuf<float> vals(ctx, cnt);
    BS_CUDA(cudaMemcpyAsync(vals.p, h_values, cnt * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    const long long lo[3] = {idx_min[0], idx_min[1], idx_min[2]};
    const unsigned long long d[3] = {dims[0], dims[1], dims[2]};
    *out = bs::volume_from_samples_impl(ctx, voxel_size, band_width, lo, d, vals.p);
  });
}

bs_status bs_volume_sphere(bs_ctx* ctx, float voxel_size, float radius, const float* origin3, bs_volume** out) {
  if (!ctx || !origin3 || !out) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  return guarded(ctx, [&] { *out = bs::volume_sphere_impl(ctx, voxel_size, radius, origin3); });
}

bs_status bs_volume_cuboid(bs_ctx* ctx, float voxel_size, const float* min3, const float* max3, bs_volume** out) {
  if (!ctx || !min3 || !max3 || !out) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  return guarded(ctx, [&] { *out = bs::volume_cuboid_impl(ctx, voxel_size, min3, max3); });
}

bs_status bs_volume_iwp(bs_ctx* ctx, float voxel_size, const float* min3, const float* max3, float cell_size,
                        bs_volume** out) {
  if (!ctx || !min3 || !max3 || !out) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  return guarded(ctx, [&] { *out = bs::volume_iwp_impl(ctx, voxel_size, min3, max3, cell_size); });
}

bs_status bs_volume_export(bs_ctx* ctx, const bs_volume* v, int32_t* h_origins, float* h_values,
                           uint32_t* h_masks) {
  if (!ctx || !v || v->ctx != ctx) return BS_ERR_INVALID_ARG;
  return guarded(ctx, [&] {
    const uint64_t n = v->n_leaves;
    if (n == 0) return;
    if (h_origins) {
      std::vector<int4> o(n);
      BS_CUDA(cudaMemcpyAsync(o.data(), v->d_origins, n * sizeof(int4), cudaMemcpyDeviceToHost, ctx->stream));
      BS_CUDA(cudaStreamSynchronize(ctx->stream));
      for (uint64_t i = 0; i < n; ++i) {
        h_origins[3 * i] = o[i].x;
        h_origins[3 * i + 1] = o[i].y;
        h_origins[3 * i + 2] = o[i].z;
      }
    }
    if (h_values)
      BS_CUDA(cudaMemcpyAsync(h_values, v->d_values, n * 512 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    if (h_masks)
      BS_CUDA(cudaMemcpyAsync(h_masks, v->d_masks, n * 16 * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    BS_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

bs_status bs_volume_export_tiles(bs_ctx* ctx, const bs_volume* v, int32_t* h_origins, int32_t* h_sizes,
                                 float* h_values) {
  if (!ctx || !v || v->ctx != ctx) return BS_ERR_INVALID_ARG;
  return guarded(ctx, [&] {
    const uint64_t n = v->n_tiles;
    if (n == 0) return;
    std::vector<int4> t(n);
    BS_CUDA(cudaMemcpyAsync(t.data(), v->d_tiles, n * sizeof(int4), cudaMemcpyDeviceToHost, ctx->stream));
    if (h_values)
      BS_CUDA(cudaMemcpyAsync(h_values, v->d_tile_values, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    BS_CUDA(cudaStreamSynchronize(ctx->stream));
    for (uint64_t i = 0; i < n; ++i) {
      if (h_origins) {
        h_origins[3 * i] = t[i].x;
        h_origins[3 * i + 1] = t[i].y;
        h_origins[3 * i + 2] = t[i].z;
      }
      if (h_sizes) h_sizes[i] = t[i].w;
    }
  });
}

static bs_status csg(bs_ctx* ctx, bs_volume* a, bs_volume* b, bs_volume** out, int op) {
  if (!ctx || !a || !b || !out || a == b || a->ctx != ctx || b->ctx != ctx) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  return guarded(ctx, [&] { *out = bs::volume_csg_impl(ctx, a, b, op); });
}
bs_status bs_volume_union(bs_ctx* ctx, bs_volume* a, bs_volume* b, bs_volume** out) { return csg(ctx, a, b, out, 0); }
bs_status bs_volume_subtract(bs_ctx* ctx, bs_volume* a, bs_volume* b, bs_volume** out) { return csg(ctx, a, b, out, 1); }
bs_status bs_volume_intersect(bs_ctx* ctx, bs_volume* a, bs_volume* b, bs_volume** out) { return csg(ctx, a, b, out, 2); }

bs_status bs_volume_offset(bs_ctx* ctx, bs_volume* v, float distance) {
  if (!ctx || !v || v->ctx != ctx) return BS_ERR_INVALID_ARG;
  return guarded(ctx, [&] { bs::volume_offset_impl(ctx, v, distance); });
}

bs_status bs_dual_contour(bs_ctx* ctx, bs_volume* v, float voxel_size, float* h_tris, uint64_t capacity,
                          uint64_t* n_tris) {
  if (!ctx || !v || !n_tris || v->ctx != ctx || (capacity && !h_tris)) return BS_ERR_INVALID_ARG;
  return guarded(ctx, [&] {
    bs::dual_contour_impl(ctx, v, voxel_size);
    *n_tris = v->n_dc_tris;
    if (capacity >= v->n_dc_tris && v->n_dc_tris) {
      BS_CUDA(cudaMemcpyAsync(h_tris, v->d_dc_tris, v->n_dc_tris * 9 * sizeof(float), cudaMemcpyDeviceToHost,
                              ctx->stream));
      BS_CUDA(cudaStreamSynchronize(ctx->stream));
    }
  });
}

bs_status bs_dual_contour_qef(bs_ctx* ctx, bs_volume* v, float voxel_size, float* h_tris, uint64_t capacity,
                              uint64_t* n_tris) {
  if (!ctx || !v || !n_tris || v->ctx != ctx || (capacity && !h_tris)) return BS_ERR_INVALID_ARG;
  return guarded(ctx, [&] {
    bs::dual_contour_impl(ctx, v, voxel_size, 1);
    *n_tris = v->n_dc_tris;
    if (capacity >= v->n_dc_tris && v->n_dc_tris) {
      BS_CUDA(cudaMemcpyAsync(h_tris, v->d_dc_tris, v->n_dc_tris * 9 * sizeof(float), cudaMemcpyDeviceToHost,
                              ctx->stream));
      BS_CUDA(cudaStreamSynchronize(ctx->stream));
    }
  });
}

bs_status bs_marching_cubes(bs_ctx* ctx, bs_volume* v, float voxel_size, float* h_tris, uint64_t capacity,
                            uint64_t* n_tris) {
  if (!ctx || !v || !n_tris || v->ctx != ctx || (capacity && !h_tris)) return BS_ERR_INVALID_ARG;
  return guarded(ctx, [&] {
    bs::marching_cubes_impl(ctx, v, voxel_size);
    *n_tris = v->n_mc_tris;
    if (capacity >= v->n_mc_tris && v->n_mc_tris) {
      BS_CUDA(cudaMemcpyAsync(h_tris, v->d_mc_tris, v->n_mc_tris * 9 * sizeof(float), cudaMemcpyDeviceToHost,
                              ctx->stream));
      BS_CUDA(cudaStreamSynchronize(ctx->stream));
    }
  });
}

}  // extern "C"
