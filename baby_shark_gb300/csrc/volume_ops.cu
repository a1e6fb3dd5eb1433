// Volume booleans and offset (volume/mod.rs:74-108) — see the functions below.
#include "bs_internal.cuh"

void bs_volume_free_upper(bs_volume* v) { (void)v; }

namespace bs {

bs_volume* volume_clone_impl(bs_ctx* ctx, const bs_volume* v) {
  bs_volume* c = new bs_volume(ctx);
  c->h = v->h;
  c->n_leaves = v->n_leaves;
  c->n_active = v->n_active;
  try {
    c->d_origins = dalloc<int4>(ctx, v->n_leaves);
    c->d_values = dalloc<float>(ctx, v->n_leaves * 512);
    c->d_masks = dalloc<uint32_t>(ctx, v->n_leaves * 16);
    if (v->n_leaves) {
      BS_CUDA(cudaMemcpyAsync(c->d_origins, v->d_origins, v->n_leaves * sizeof(int4), cudaMemcpyDeviceToDevice, ctx->stream));
      BS_CUDA(cudaMemcpyAsync(c->d_values, v->d_values, v->n_leaves * 512 * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
      BS_CUDA(cudaMemcpyAsync(c->d_masks, v->d_masks, v->n_leaves * 16 * sizeof(uint32_t), cudaMemcpyDeviceToDevice, ctx->stream));
    }
    c->n_tiles = v->n_tiles;
    if (v->n_tiles) {
      c->d_tiles = dalloc<int4>(ctx, v->n_tiles);
      c->d_tile_values = dalloc<float>(ctx, v->n_tiles);
      BS_CUDA(cudaMemcpyAsync(c->d_tiles, v->d_tiles, v->n_tiles * sizeof(int4), cudaMemcpyDeviceToDevice, ctx->stream));
      BS_CUDA(cudaMemcpyAsync(c->d_tile_values, v->d_tile_values, v->n_tiles * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
    }
  } catch (...) {
    delete c;
    throw;
  }
  return c;
}

bs_volume* volume_csg_impl(bs_ctx*, bs_volume*, bs_volume*, int) {
  fail(BS_ERR_UNSUPPORTED, "volume booleans are not built yet");
  return nullptr;
}

void volume_offset_impl(bs_ctx*, bs_volume*, float) { fail(BS_ERR_UNSUPPORTED, "offset is not built yet"); }

void dual_contour_impl(bs_ctx*, bs_volume*, float) { fail(BS_ERR_UNSUPPORTED, "dual contouring is not built yet"); }

}  // namespace bs
