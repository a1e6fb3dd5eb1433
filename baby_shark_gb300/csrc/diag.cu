// Diagnostics without a reference counterpart: a measured FP32 peak used as
// the roofline denominator of the FP32-bound distance kernel.
#include "bs_internal.cuh"

namespace {

// 8 independent FMA chains per thread; every iteration is 8 FFMA = 16 FLOP.
__global__ void __launch_bounds__(256) k_ffma_peak(float* out, int iters, float a, float b) {
  float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f;
  float x4 = x0 + 4.f, x5 = x0 + 5.f, x6 = x0 + 6.f, x7 = x0 + 7.f;
  for (int i = 0; i < iters; ++i) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 1234.5f) out[0] = s;  // keeps the chains alive
}

}  // namespace

extern "C" bs_status bs_diag_fp32_peak(bs_ctx* ctx, double* tflops) {
  if (!ctx || !tflops) return BS_ERR_INVALID_ARG;
  try {
    BS_CUDA(cudaSetDevice(ctx->device));
    int sms = 0;
    BS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    bs::DBuf<float> out(ctx, 1);
    const int threads = 256, blocks = sms * 8, iters = 1 << 15;
    cudaEvent_t e0, e1;
    BS_CUDA(cudaEventCreate(&e0));
    BS_CUDA(cudaEventCreate(&e1));
    k_ffma_peak<<<blocks, threads, 0, ctx->stream>>>(out.p, iters / 8, 0.999f, 1e-4f);  // warm-up
    BS_CHECK_LAUNCH(ctx);
    BS_CUDA(cudaEventRecord(e0, ctx->stream));
    k_ffma_peak<<<blocks, threads, 0, ctx->stream>>>(out.p, iters, 0.999f, 1e-4f);
    BS_CHECK_LAUNCH(ctx);
    BS_CUDA(cudaEventRecord(e1, ctx->stream));
    BS_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    BS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *tflops = double(blocks) * threads * double(iters) * 16.0 / (ms * 1e-3) / 1e12;
    return BS_OK;
  } catch (const bs::Error& e) {
    ctx->last_error = e.msg;
    return e.status;
  }
}

// Every pair of significands (a, b in [1, 2)): Markstein's division with a
// shared reciprocal (bs_internal.cuh, mdiv) against CUDA's IEEE division.
__global__ void k_div_check(uint32_t b_stride, unsigned long long* bad, unsigned long long* tested) {
  const uint32_t mb = blockIdx.x * b_stride;
  if (mb >= (1u << 23)) return;
  const float b = __uint_as_float((127u << 23) | mb);
  const float y = __frcp_rn(b);
  uint32_t nbad = 0;
  for (uint32_t ma = threadIdx.x; ma < (1u << 23); ma += blockDim.x) {
    const float a = __uint_as_float((127u << 23) | ma);
    nbad += (bs::mdiv(a, b, y) != __fdiv_rn(a, b)) ? 1u : 0u;
  }
  const uint32_t w = __reduce_add_sync(0xffffffffu, nbad);
  if ((threadIdx.x & 31) == 0) {
    if (w) atomicAdd(bad, (unsigned long long)w);
    atomicAdd(tested, 32ull * ((1u << 23) / blockDim.x));
  }
}

extern "C" bs_status bs_diag_check_division(bs_ctx* ctx, uint32_t b_stride, uint64_t* mismatches, uint64_t* tested) {
  if (!ctx || !mismatches || !tested || b_stride == 0) return BS_ERR_INVALID_ARG;
  try {
    BS_CUDA(cudaSetDevice(ctx->device));
    bs::DBuf<unsigned long long> c(ctx, 2);
    BS_CUDA(cudaMemsetAsync(c.p, 0, 2 * sizeof(unsigned long long), ctx->stream));
    const unsigned nb = unsigned(((1u << 23) + b_stride - 1) / b_stride);
    k_div_check<<<nb, 256, 0, ctx->stream>>>(b_stride, c.p, c.p + 1);
    BS_CHECK_LAUNCH(ctx);
    unsigned long long h[2];
    bs::read_back(ctx, h, c.p, sizeof h);
    *mismatches = h[0];
    *tested = h[1];
    return BS_OK;
  } catch (const bs::Error& e) {
    ctx->last_error = e.msg;
    return e.status;
  }
}
