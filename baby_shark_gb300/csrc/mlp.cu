// Learned far field: a per-mesh MLP that predicts the generalised winding
// number at a point, so that queries away from the surface can skip the tree
// traversal.  No counterpart in the reference (its winding numbers are only
// evaluated at band voxels, mesh_to_volume.rs:245-280); the traversal
// (bs_winding_numbers_approximate) produces its training targets and stays
// the fallback for every point whose prediction is not confidently on one
// side of the sign threshold.
//
// Network: x -> x_n = (x - centre) * scale -> 64 Fourier features
// [sin(pi v_k), cos(pi v_k)], v_k = f_k . x_n (32 frequency vectors f_k, fixed)
// -> Linear 64x64 + SiLU -> Linear 64x64 + SiLU -> Linear 64x1.  Weights and
// activations enter the tensor cores as BF16 with FP32 accumulation
// (mma.sync m16n8k16): a warp owns 16 samples, and a layer's accumulator
// fragments are the next layer's A fragments register for register, so the
// whole forward pass and the backward pass down to the first layer run out of
// registers; only the weight-gradient reduction over samples goes through
// memory (feature-major BF16 tiles, a second tensor-core kernel with K = the
// samples).  Training step = three kernels (forward + backward, weight
// gradients, Adam), captured once in a CUDA graph and replayed per step.
#include <cuda_bf16.h>

#include <cub/device/device_scan.cuh>

#include <cmath>
#include <cstring>
#include <vector>

#include "bs_internal.cuh"
#include "leaf_hash.cuh"

namespace bs {
namespace {

constexpr int MLP_NF = 32;      // frequency vectors
constexpr int OFF_W1 = 0;       // [in][out]
constexpr int OFF_B1 = 4096;
constexpr int OFF_W2 = 4160;    // [in][out]
constexpr int OFF_B2 = 8256;
constexpr int OFF_W3 = 8320;
constexpr int OFF_B3 = 8384;
constexpr int MLP_NP = 8385;    // parameters
constexpr int SROW = 36;        // padded smem row of a bf16 64x64 matrix, in 32-bit words
constexpr int MLP_WARPS = 4;
constexpr int MLP_THREADS = 32 * MLP_WARPS;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }

// D += A (16x16, row) * B (16x8, col), BF16 in, FP32 accumulate.
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float sigmoidf_(float z) { return 1.0f / (1.0f + __expf(-z)); }

// Weights of one network as the kernels read them.
struct MlpW {
  const uint32_t* w1t;  // bf16 pairs, [out][in] (64 x 32 words)
  const uint32_t* w2t;  // [out][in]
  const uint32_t* w2;   // [in][out]
  const float* p;       // fp32 parameters (biases, last layer)
  const float* freq;    // [32][3]
  float cx, cy, cz, scale;
};

struct MlpSmem {
  uint32_t w1t[64 * SROW];
  uint32_t w2t[64 * SROW];
  uint32_t w2[64 * SROW];
  float b1[64], b2[64], w3[64], freq[96];
  float b3;
};

__device__ void load_smem(const MlpW& W, MlpSmem& S, bool with_w2) {
  for (int i = threadIdx.x; i < 64 * 32; i += blockDim.x) {
    const int r = i >> 5, c = i & 31;
    S.w1t[r * SROW + c] = W.w1t[i];
    S.w2t[r * SROW + c] = W.w2t[i];
    if (with_w2) S.w2[r * SROW + c] = W.w2[i];
  }
  for (int i = threadIdx.x; i < 64; i += blockDim.x) {
    S.b1[i] = W.p[OFF_B1 + i];
    S.b2[i] = W.p[OFF_B2 + i];
    S.w3[i] = W.p[OFF_W3 + i];
  }
  for (int i = threadIdx.x; i < 96; i += blockDim.x) S.freq[i] = W.freq[i];
  if (threadIdx.x == 0) S.b3 = W.p[OFF_B3];
}

// acc[j] (16 x 8 outputs j*8..) += A (16 x 64) * M^T where M is a padded
// [out][in] bf16 matrix in shared memory (B[k][n] = M[n][k]).
__device__ __forceinline__ void layer_mma(float (&acc)[8][4], const uint32_t (&A)[4][4], const uint32_t* M, int g,
                                          int t) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const uint32_t* row = M + (j * 8 + g) * SROW + t;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) mma16816(acc[j], A[kk], row[kk * 8], row[kk * 8 + 4]);
  }
}

// C fragments (16 x 64, fp32) -> A fragments of the next layer (bf16).
__device__ __forceinline__ void c_to_a(const float (&c)[8][4], uint32_t (&A)[4][4]) {
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    A[kk][0] = pack_bf16(c[2 * kk][0], c[2 * kk][1]);
    A[kk][1] = pack_bf16(c[2 * kk][2], c[2 * kk][3]);
    A[kk][2] = pack_bf16(c[2 * kk + 1][0], c[2 * kk + 1][1]);
    A[kk][3] = pack_bf16(c[2 * kk + 1][2], c[2 * kk + 1][3]);
  }
}

// Forward pass of the warp's 16 samples (rows g and g + 8 of this thread).
// Feature c < 32 is sin(pi v_c), c >= 32 cos(pi v_{c-32}).
struct Fwd {
  uint32_t F[4][4];   // features, A fragments
  float z1[8][4];     // layer-1 pre-activations
  float z2[8][4];     // layer-2 pre-activations
  float y[2];         // outputs of rows g, g + 8
};

__device__ __forceinline__ void forward16(const MlpW& W, const MlpSmem& S, const float* pts, uint64_t n,
                                          uint64_t row0, Fwd& f) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  float xn[2][3];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const uint64_t r = row0 + g + 8 * h;
    const bool ok = r < n;
    const float x = ok ? pts[3 * r] : W.cx, y = ok ? pts[3 * r + 1] : W.cy, z = ok ? pts[3 * r + 2] : W.cz;
    xn[h][0] = (x - W.cx) * W.scale;
    xn[h][1] = (y - W.cy) * W.scale;
    xn[h][2] = (z - W.cz) * W.scale;
  }
  // frequencies of this thread: {2t, 2t+1, 2t+8, 2t+9} + {0, 16}
  float sn[2][8], cs[2][8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int k = (q >> 2) * 16 + (q & 1) + ((q >> 1) & 1) * 8 + 2 * t;
    const float fx = S.freq[3 * k], fy = S.freq[3 * k + 1], fz = S.freq[3 * k + 2];
#pragma unroll
    for (int h = 0; h < 2; ++h) sincospif(fx * xn[h][0] + fy * xn[h][1] + fz * xn[h][2], &sn[h][q], &cs[h][q]);
  }
  // k-tile kk: features kk*16 + {2t, 2t+1} (regs 0/1) and + 8 (regs 2/3);
  // kk 0, 1 sines of frequencies kk*16 + ..., kk 2, 3 cosines
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    const int base = (kk & 1) * 4;
    const auto& v = (kk < 2) ? sn : cs;
    f.F[kk][0] = pack_bf16(v[0][base + 0], v[0][base + 1]);
    f.F[kk][1] = pack_bf16(v[1][base + 0], v[1][base + 1]);
    f.F[kk][2] = pack_bf16(v[0][base + 2], v[0][base + 3]);
    f.F[kk][3] = pack_bf16(v[1][base + 2], v[1][base + 3]);
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float b0 = S.b1[j * 8 + 2 * t], b1 = S.b1[j * 8 + 2 * t + 1];
    f.z1[j][0] = b0; f.z1[j][1] = b1; f.z1[j][2] = b0; f.z1[j][3] = b1;
  }
  layer_mma(f.z1, f.F, S.w1t, g, t);
  float h1[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j)
#pragma unroll
    for (int i = 0; i < 4; ++i) h1[j][i] = f.z1[j][i] * sigmoidf_(f.z1[j][i]);
  uint32_t A2[4][4];
  c_to_a(h1, A2);
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float b0 = S.b2[j * 8 + 2 * t], b1 = S.b2[j * 8 + 2 * t + 1];
    f.z2[j][0] = b0; f.z2[j][1] = b1; f.z2[j][2] = b0; f.z2[j][3] = b1;
  }
  layer_mma(f.z2, A2, S.w2t, g, t);
  float y0 = 0.f, y1 = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float wa = S.w3[j * 8 + 2 * t], wb = S.w3[j * 8 + 2 * t + 1];
    y0 += f.z2[j][0] * sigmoidf_(f.z2[j][0]) * wa + f.z2[j][1] * sigmoidf_(f.z2[j][1]) * wb;
    y1 += f.z2[j][2] * sigmoidf_(f.z2[j][2]) * wa + f.z2[j][3] * sigmoidf_(f.z2[j][3]) * wb;
  }
  y0 += __shfl_xor_sync(0xffffffffu, y0, 1);
  y0 += __shfl_xor_sync(0xffffffffu, y0, 2);
  y1 += __shfl_xor_sync(0xffffffffu, y1, 1);
  y1 += __shfl_xor_sync(0xffffffffu, y1, 2);
  f.y[0] = y0 + S.b3;
  f.y[1] = y1 + S.b3;
}

// Active voxels of a volume, looked up at the grid point nearest to a point.
struct BandLookup {
  LeafHash hash;
  const uint32_t* masks;
  float inv_h;
  int any;  // 0: no band
};

__device__ __forceinline__ bool in_band(const BandLookup& B, float x, float y, float z) {
  if (!B.any) return false;
  const float fx = rintf(x * B.inv_h), fy = rintf(y * B.inv_h), fz = rintf(z * B.inv_h);
  const float lim = 1073741824.0f;  // 2^30: beyond every leaf
  if (!(fabsf(fx) < lim && fabsf(fy) < lim && fabsf(fz) < lim)) return false;
  const int ix = int(fx), iy = int(fy), iz = int(fz);
  const int l = B.hash.find(ix & ~7, iy & ~7, iz & ~7);
  if (l < 0) return false;
  const int o = ((ix & 7) << 6) | ((iy & 7) << 3) | (iz & 7);
  return (B.masks[uint64_t(l) * 16 + (o >> 5)] >> (o & 31)) & 1u;
}

__global__ void k_band_flags(BandLookup B, const float* __restrict__ pts, uint64_t n, uint32_t* __restrict__ flags) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i < n) flags[i] = in_band(B, pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]) ? 1u : 0u;
}

// ------------------------------------------------------------ inference --
// out = prediction; unsure (optional) = 1 where the point lies in the band or
// the prediction is within `margin` of `thresh`.
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_predict(MlpW W, const float* __restrict__ pts, uint64_t n,
                                                             float* __restrict__ out, float thresh, float margin,
                                                             uint32_t* __restrict__ unsure, BandLookup band) {
  __shared__ MlpSmem S;
  load_smem(W, S, false);
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const uint64_t tiles = (n + 15) / 16;
  for (uint64_t tile = uint64_t(blockIdx.x) * MLP_WARPS + (threadIdx.x >> 5); tile < tiles;
       tile += uint64_t(gridDim.x) * MLP_WARPS) {
    Fwd f;
    forward16(W, S, pts, n, tile * 16, f);
    if (t == 0) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const uint64_t r = tile * 16 + g + 8 * h;
        if (r >= n) continue;
        out[r] = f.y[h];
        if (unsure)
          unsure[r] = (fabsf(f.y[h] - thresh) > margin && !in_band(band, pts[3 * r], pts[3 * r + 1], pts[3 * r + 2]))
                          ? 0u
                          : 1u;
      }
    }
  }
}

// ------------------------------------------------------------- training --
// Training state on the device.
struct MlpTrain {
  float* grad;      // [NP]
  float* m;         // Adam moments
  float* v;
  float* lr;        // per step
  float* loss;      // per epoch (sum of squared errors)
  int* step;        // steps taken
  __nv_bfloat16* ft;   // [64][B] features
  __nv_bfloat16* h1t;  // [64][B] layer-1 activations
  __nv_bfloat16* d1t;  // [64][B] layer-1 pre-activation gradients
  __nv_bfloat16* d2t;  // [64][B] layer-2 pre-activation gradients
};

// Forward + backward of one minibatch down to the layer-1 pre-activations:
// writes the feature-major tiles for the weight-gradient kernel and adds the
// last layer's gradients.  Loss = mean squared error over the minibatch.
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_fwd_bwd(MlpW W, MlpTrain T, const float* __restrict__ pts,
                                                             const float* __restrict__ tgt, uint64_t n_all,
                                                             uint32_t batch, uint32_t steps_per_epoch) {
  __shared__ MlpSmem S;
  load_smem(W, S, true);
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int step = *T.step;
  const uint64_t base = uint64_t(step % int(steps_per_epoch)) * batch;
  const float* P = pts + 3 * base;
  const float* Y = tgt + base;
  const uint64_t n = (base + batch <= n_all) ? batch : (n_all > base ? n_all - base : 0);
  const float inv_n = 1.0f / float(batch);
  const uint32_t tiles = batch / 16;
  for (uint32_t tile = blockIdx.x * MLP_WARPS + (threadIdx.x >> 5); tile < tiles; tile += gridDim.x * MLP_WARPS) {
    const uint64_t row0 = uint64_t(tile) * 16;
    Fwd f;
    forward16(W, S, P, n, row0, f);
    float dy[2], sq = 0.f;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint64_t r = row0 + g + 8 * h;
      const float e = r < n ? f.y[h] - Y[r] : 0.0f;
      dy[h] = 2.0f * e * inv_n;
      sq += (t == 0) ? e * e : 0.0f;
    }
    // last layer: dW3[c] = sum_r h2[r][c] dy[r], db3 = sum_r dy[r]
    float dz2[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int c = j * 8 + 2 * t + i;
        const float za = f.z2[j][i], zb = f.z2[j][2 + i];
        const float sa = sigmoidf_(za), sb = sigmoidf_(zb);
        float gw = za * sa * dy[0] + zb * sb * dy[1];
        gw += __shfl_xor_sync(0xffffffffu, gw, 4);
        gw += __shfl_xor_sync(0xffffffffu, gw, 8);
        gw += __shfl_xor_sync(0xffffffffu, gw, 16);
        if (g == 0) atomicAdd(&T.grad[OFF_W3 + c], gw);
        const float w = S.w3[c];
        dz2[j][i] = dy[0] * w * sa * (1.0f + za * (1.0f - sa));
        dz2[j][2 + i] = dy[1] * w * sb * (1.0f + zb * (1.0f - sb));
      }
    }
    float db3 = (t == 0) ? dy[0] + dy[1] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      db3 += __shfl_xor_sync(0xffffffffu, db3, o);
      sq += __shfl_xor_sync(0xffffffffu, sq, o);
    }
    if (lane == 0) {
      atomicAdd(&T.grad[OFF_B3], db3);
      atomicAdd(&T.loss[step / int(steps_per_epoch)], sq);
    }
    // dh1 = dz2 W2^T, dz1 = dh1 * silu'(z1)
    uint32_t D2[4][4];
    c_to_a(dz2, D2);
    float dh1[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) dh1[j][0] = dh1[j][1] = dh1[j][2] = dh1[j][3] = 0.f;
    layer_mma(dh1, D2, S.w2, g, t);
    // feature-major tiles: value of (row r, column c) at [c * batch + row0 + r]
    auto put = [&](__nv_bfloat16* dst, int c, int r, float v) {
      dst[uint64_t(c) * batch + row0 + r] = __float2bfloat16_rn(v);
    };
#pragma unroll
    for (int j = 0; j < 8; ++j) {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int c = j * 8 + 2 * t + (i & 1), r = g + 8 * (i >> 1);
        const float z = f.z1[j][i], s = sigmoidf_(z);
        put(T.h1t, c, r, z * s);
        put(T.d1t, c, r, dh1[j][i] * s * (1.0f + z * (1.0f - s)));
        put(T.d2t, c, r, dz2[j][i]);
      }
    }
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const int c = kk * 16 + 2 * t;
      const uint32_t* a = f.F[kk];
      put(T.ft, c, g, bf_lo(a[0]));
      put(T.ft, c + 1, g, bf_hi(a[0]));
      put(T.ft, c, g + 8, bf_lo(a[1]));
      put(T.ft, c + 1, g + 8, bf_hi(a[1]));
      put(T.ft, c + 8, g, bf_lo(a[2]));
      put(T.ft, c + 9, g, bf_hi(a[2]));
      put(T.ft, c + 8, g + 8, bf_lo(a[3]));
      put(T.ft, c + 9, g + 8, bf_hi(a[3]));
    }
  }
}

// Weight gradients dW = X^T D over the minibatch (blockIdx.y: 0 -> features
// and layer-1 gradients into W1, b1; 1 -> layer-1 activations and layer-2
// gradients into W2, b2).  Warp w owns input rows 16w .. 16w+15 of dW; K is
// the samples of the block's chunk.  Block (0, 0) counts the step.
constexpr uint32_t WG_CHUNK = 128;
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_wgrad(MlpTrain T, uint32_t batch) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, w = threadIdx.x >> 5;
  const bool second = blockIdx.y == 1;
  const uint16_t* X = reinterpret_cast<const uint16_t*>(second ? T.h1t : T.ft);
  const uint16_t* D = reinterpret_cast<const uint16_t*>(second ? T.d2t : T.d1t);
  const int offW = second ? OFF_W2 : OFF_W1, offB = second ? OFF_B2 : OFF_B1;
  const uint32_t n0 = blockIdx.x * WG_CHUNK;
  const uint32_t n1 = min(batch, n0 + WG_CHUNK);
  float acc[8][4];
#pragma unroll
  for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
  float bsum[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  const int in0 = 16 * w + g;
  for (uint32_t k0 = n0; k0 < n1; k0 += 16) {
    uint32_t a[4];
    a[0] = *reinterpret_cast<const uint32_t*>(X + uint64_t(in0) * batch + k0 + 2 * t);
    a[1] = *reinterpret_cast<const uint32_t*>(X + uint64_t(in0 + 8) * batch + k0 + 2 * t);
    a[2] = *reinterpret_cast<const uint32_t*>(X + uint64_t(in0) * batch + k0 + 8 + 2 * t);
    a[3] = *reinterpret_cast<const uint32_t*>(X + uint64_t(in0 + 8) * batch + k0 + 8 + 2 * t);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint16_t* dr = D + uint64_t(j * 8 + g) * batch + k0 + 2 * t;
      const uint32_t b0 = *reinterpret_cast<const uint32_t*>(dr);
      const uint32_t b1 = *reinterpret_cast<const uint32_t*>(dr + 8);
      mma16816(acc[j], a, b0, b1);
      if (w == 0) bsum[j] += (bf_lo(b0) + bf_hi(b0)) + (bf_lo(b1) + bf_hi(b1));
    }
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int out = j * 8 + 2 * t;
    atomicAdd(&T.grad[offW + in0 * 64 + out], acc[j][0]);
    atomicAdd(&T.grad[offW + in0 * 64 + out + 1], acc[j][1]);
    atomicAdd(&T.grad[offW + (in0 + 8) * 64 + out], acc[j][2]);
    atomicAdd(&T.grad[offW + (in0 + 8) * 64 + out + 1], acc[j][3]);
    if (w == 0) {
      float s = bsum[j];
      s += __shfl_xor_sync(0xffffffffu, s, 1);
      s += __shfl_xor_sync(0xffffffffu, s, 2);
      if (t == 0) atomicAdd(&T.grad[offB + j * 8 + g], s);
    }
  }
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) atomicAdd(T.step, 1);
}

// Adam (beta1 0.9, beta2 0.999, eps 1e-8) on every parameter, and a cleared
// gradient for the next step.
__global__ void k_mlp_adam(float* __restrict__ p, MlpTrain T) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int step = *T.step;  // already counted for this step
  if (i < MLP_NP) {
    const float gr = T.grad[i];
    const float m = 0.9f * T.m[i] + 0.1f * gr;
    const float v = 0.999f * T.v[i] + 0.001f * gr * gr;
    T.m[i] = m;
    T.v[i] = v;
    const float mh = m / (1.0f - powf(0.9f, float(step)));
    const float vh = v / (1.0f - powf(0.999f, float(step)));
    p[i] -= T.lr[step - 1] * mh / (sqrtf(vh) + 1e-8f);
    T.grad[i] = 0.0f;
  }
}

// BF16 copies of W1 and W2 in the layouts the kernels read (pairs along the
// reduction index): w1t, w2t [out][in], w2 [in][out].
__global__ void k_mlp_bf16(const float* __restrict__ p, uint32_t* __restrict__ w1t, uint32_t* __restrict__ w2t,
                           uint32_t* __restrict__ w2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // pair index: row r, pair c
  if (i >= 64 * 32) return;
  const int r = i >> 5, c = (i & 31) * 2;
  w1t[i] = pack_bf16(p[OFF_W1 + c * 64 + r], p[OFF_W1 + (c + 1) * 64 + r]);
  w2t[i] = pack_bf16(p[OFF_W2 + c * 64 + r], p[OFF_W2 + (c + 1) * 64 + r]);
  w2[i] = pack_bf16(p[OFF_W2 + r * 64 + c], p[OFF_W2 + r * 64 + c + 1]);
}

__global__ void k_gather3(const float* __restrict__ src, const uint32_t* __restrict__ idx, uint64_t n,
                          float* __restrict__ dst_pts, const float* __restrict__ src_t, float* __restrict__ dst_t) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = idx[i];
  dst_pts[3 * i] = src[3 * uint64_t(k)];
  dst_pts[3 * i + 1] = src[3 * uint64_t(k) + 1];
  dst_pts[3 * i + 2] = src[3 * uint64_t(k) + 2];
  if (dst_t) dst_t[i] = src_t[k];
}

__global__ void k_scatter1(const float* __restrict__ v, const uint32_t* __restrict__ idx, uint64_t n,
                           float* __restrict__ out) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i < n) out[idx[i]] = v[i];
}

__global__ void k_unsure_list(const uint32_t* __restrict__ unsure, const uint32_t* __restrict__ off, uint64_t n,
                              uint32_t* __restrict__ list) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i < n && unsure[i]) list[off[i]] = uint32_t(i);
}

unsigned grid_for(uint64_t n, unsigned t) { return unsigned(std::min<uint64_t>((n + t - 1) / t, 1u << 30)); }

void scan_u32(bs_ctx* ctx, const uint32_t* in, uint32_t* out, uint64_t n) {
  size_t tmp = 0;
  BS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, in, out, n, ctx->stream));
  DBuf<uint8_t> t(ctx, tmp);
  BS_CUDA(cub::DeviceScan::ExclusiveSum(t.p, tmp, in, out, n, ctx->stream));
}

}  // namespace
}  // namespace bs

// One network and its training state.
struct bs_mlp {
  explicit bs_mlp(bs_ctx* c) : ctx(c) { ctx->refs++; }
  bs_mlp(const bs_mlp&) = delete;
  bs_mlp& operator=(const bs_mlp&) = delete;
  ~bs_mlp() {
    cudaSetDevice(ctx->device);
    for (void* q : {(void*)p, (void*)freq, (void*)w1t, (void*)w2t, (void*)w2, (void*)grad, (void*)m, (void*)v})
      bs::dfree(ctx, q);
    bs_ctx_release(ctx);
  }
  bs_ctx* ctx;
  float centre[3] = {0, 0, 0};
  float scale = 1.0f;
  float* p = nullptr;
  float* freq = nullptr;
  uint32_t *w1t = nullptr, *w2t = nullptr, *w2 = nullptr;
  float *grad = nullptr, *m = nullptr, *v = nullptr;
  bs::MlpW weights() const {
    return bs::MlpW{w1t, w2t, w2, p, freq, centre[0], centre[1], centre[2], scale};
  }
};

namespace {
using namespace bs;

template <class F>
bs_status mlp_guard(bs_ctx* ctx, F&& f) {
  try {
    BS_CUDA(cudaSetDevice(ctx->device));
    ctx->last_error.clear();
    f();
    return BS_OK;
  } catch (const bs::Error& e) {
    ctx->last_error = e.msg;
    return e.status;
  } catch (const std::bad_alloc&) {
    ctx->last_error = "host allocation failed";
    return BS_ERR_OOM;
  }
}
}  // namespace

extern "C" {

int bs_mlp_num_params(void) { return bs::MLP_NP; }

bs_status bs_mlp_create(bs_ctx* ctx, const float* centre, float scale, const float* h_freq, const float* h_params,
                        bs_mlp** out) {
  if (!ctx || !centre || !h_freq || !h_params || !out || !(scale > 0.0f)) return BS_ERR_INVALID_ARG;
  *out = nullptr;
  return mlp_guard(ctx, [&] {
    bs_mlp* q = new bs_mlp(ctx);
    try {
      std::memcpy(q->centre, centre, sizeof q->centre);
      q->scale = scale;
      cudaStream_t s = ctx->stream;
      q->p = dalloc<float>(ctx, MLP_NP);
      q->freq = dalloc<float>(ctx, 3 * MLP_NF);
      q->w1t = dalloc<uint32_t>(ctx, 64 * 32);
      q->w2t = dalloc<uint32_t>(ctx, 64 * 32);
      q->w2 = dalloc<uint32_t>(ctx, 64 * 32);
      q->grad = dalloc<float>(ctx, MLP_NP);
      q->m = dalloc<float>(ctx, MLP_NP);
      q->v = dalloc<float>(ctx, MLP_NP);
      BS_CUDA(cudaMemcpyAsync(q->p, h_params, MLP_NP * sizeof(float), cudaMemcpyHostToDevice, s));
      BS_CUDA(cudaMemcpyAsync(q->freq, h_freq, 3 * MLP_NF * sizeof(float), cudaMemcpyHostToDevice, s));
      BS_CUDA(cudaMemsetAsync(q->grad, 0, MLP_NP * sizeof(float), s));
      BS_CUDA(cudaMemsetAsync(q->m, 0, MLP_NP * sizeof(float), s));
      BS_CUDA(cudaMemsetAsync(q->v, 0, MLP_NP * sizeof(float), s));
      BS_KERNEL(ctx, "k_mlp_bf16", (k_mlp_bf16<<<16, 128, 0, s>>>(q->p, q->w1t, q->w2t, q->w2)));
      BS_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
      delete q;
      throw;
    }
    *out = q;
  });
}

bs_status bs_mlp_free(bs_mlp* q) {
  if (!q) return BS_ERR_INVALID_ARG;  // as every other release call
  delete q;
  return BS_OK;
}

bs_status bs_mlp_get_params(bs_ctx* ctx, const bs_mlp* q, float* h_params) {
  if (!ctx || !q || !h_params) return BS_ERR_INVALID_ARG;
  return mlp_guard(ctx, [&] { read_back(ctx, h_params, q->p, MLP_NP * sizeof(float)); });
}

bs_status bs_mlp_predict(bs_ctx* ctx, const bs_mlp* q, const float* d_points, uint64_t n, float* d_out) {
  if (!ctx || !q || (n && (!d_points || !d_out))) return BS_ERR_INVALID_ARG;
  return mlp_guard(ctx, [&] {
    if (!n) return;
    const unsigned grid = grid_for((n + 15) / 16, MLP_WARPS);
    BS_KERNEL(ctx, "k_mlp_predict", (k_mlp_predict<<<std::min(grid, 152u * 16u), MLP_THREADS, 0, ctx->stream>>>(
                                         q->weights(), d_points, n, d_out, 0.f, 0.f, nullptr, BandLookup{})));
    BS_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

bs_status bs_mlp_train(bs_ctx* ctx, bs_mlp* q, const float* d_points, const float* d_targets, uint64_t n,
                       uint32_t batch, uint32_t epochs, float lr_max, float lr_min, float* h_epoch_loss) {
  if (!ctx || !q || !d_points || !d_targets || batch < WG_CHUNK || batch % WG_CHUNK || !epochs)
    return BS_ERR_INVALID_ARG;
  return mlp_guard(ctx, [&] {
    cudaStream_t s = ctx->stream;
    const uint32_t spe = uint32_t(n / batch);
    if (spe == 0) fail(BS_ERR_INVALID_ARG, "mlp training: fewer samples than one minibatch");
    const uint64_t total = uint64_t(spe) * epochs;
    // cosine learning-rate schedule, one entry per step
    std::vector<float> lr(total);
    for (uint64_t k = 0; k < total; ++k)
      lr[k] = lr_min + 0.5f * (lr_max - lr_min) * (1.0f + std::cos(3.14159265f * float(k) / float(total)));
    DBuf<float> d_lr(ctx, total), d_loss(ctx, epochs);
    DBuf<int> d_step(ctx, 1);
    DBuf<__nv_bfloat16> ft(ctx, uint64_t(64) * batch), h1t(ctx, uint64_t(64) * batch), d1t(ctx, uint64_t(64) * batch),
        d2t(ctx, uint64_t(64) * batch);
    BS_CUDA(cudaMemcpyAsync(d_lr.p, lr.data(), total * sizeof(float), cudaMemcpyHostToDevice, s));
    BS_CUDA(cudaMemsetAsync(d_loss.p, 0, epochs * sizeof(float), s));
    BS_CUDA(cudaMemsetAsync(d_step.p, 0, sizeof(int), s));
    MlpTrain T{q->grad, q->m, q->v, d_lr.p, d_loss.p, d_step.p, ft.p, h1t.p, d1t.p, d2t.p};
    const MlpW W = q->weights();
    const unsigned g1 = std::min(batch / 16 / MLP_WARPS, 152u * 8u);
    const dim3 g2(batch / WG_CHUNK, 2);
    auto one_step = [&]() {
      k_mlp_fwd_bwd<<<g1, MLP_THREADS, 0, s>>>(W, T, d_points, d_targets, n, batch, spe);
      k_mlp_wgrad<<<g2, MLP_THREADS, 0, s>>>(T, batch);
      k_mlp_adam<<<(MLP_NP + 255) / 256, 256, 0, s>>>(q->p, T);
      k_mlp_bf16<<<16, 128, 0, s>>>(q->p, q->w1t, q->w2t, q->w2);
    };
    // one step captured as a graph, replayed for every step (a stream that
    // cannot be captured, the legacy default stream, launches every step)
    BS_CUDA(cudaStreamSynchronize(s));
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      one_step();
      const cudaError_t ce = cudaStreamEndCapture(s, &graph);
      if (ce != cudaSuccess) fail(BS_ERR_CUDA, cudaGetErrorString(ce));
      const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
      if (ie != cudaSuccess) {
        cudaGraphDestroy(graph);
        fail(BS_ERR_CUDA, cudaGetErrorString(ie));
      }
    } else {
      cudaGetLastError();
    }
    cudaError_t le = cudaSuccess;
    for (uint64_t k = 0; k < total && le == cudaSuccess; ++k) {
      if (exec) {
        le = cudaGraphLaunch(exec, s);
      } else {
        one_step();
        le = cudaGetLastError();
      }
    }
    ctx->launches += 4 * total;
    const cudaError_t se = cudaStreamSynchronize(s);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (le != cudaSuccess) fail(BS_ERR_CUDA, cudaGetErrorString(le));
    if (se != cudaSuccess) fail(BS_ERR_CUDA, cudaGetErrorString(se));
    if (h_epoch_loss) {
      read_back(ctx, h_epoch_loss, d_loss.p, epochs * sizeof(float));
      for (uint32_t e = 0; e < epochs; ++e) h_epoch_loss[e] /= float(uint64_t(spe) * batch);
    }
  });
}

// Gradients of the mean squared error over the first `batch` samples (no
// parameter update): for checks against a CPU restatement.
bs_status bs_mlp_gradients(bs_ctx* ctx, bs_mlp* q, const float* d_points, const float* d_targets, uint64_t n,
                           uint32_t batch, float* h_grad, float* h_loss) {
  if (!ctx || !q || !d_points || !d_targets || !h_grad || batch < WG_CHUNK || batch % WG_CHUNK)
    return BS_ERR_INVALID_ARG;
  return mlp_guard(ctx, [&] {
    cudaStream_t s = ctx->stream;
    DBuf<float> d_loss(ctx, 1), d_lr(ctx, 1);
    DBuf<int> d_step(ctx, 1);
    DBuf<__nv_bfloat16> ft(ctx, uint64_t(64) * batch), h1t(ctx, uint64_t(64) * batch), d1t(ctx, uint64_t(64) * batch),
        d2t(ctx, uint64_t(64) * batch);
    BS_CUDA(cudaMemsetAsync(d_loss.p, 0, sizeof(float), s));
    BS_CUDA(cudaMemsetAsync(d_step.p, 0, sizeof(int), s));
    BS_CUDA(cudaMemsetAsync(q->grad, 0, MLP_NP * sizeof(float), s));
    MlpTrain T{q->grad, q->m, q->v, d_lr.p, d_loss.p, d_step.p, ft.p, h1t.p, d1t.p, d2t.p};
    const unsigned g1 = std::min(batch / 16 / MLP_WARPS, 152u * 8u);
    BS_KERNEL(ctx, "k_mlp_fwd_bwd", (k_mlp_fwd_bwd<<<g1, MLP_THREADS, 0, s>>>(q->weights(), T, d_points, d_targets, n,
                                                                             batch, 1)));
    BS_KERNEL(ctx, "k_mlp_wgrad", (k_mlp_wgrad<<<dim3(batch / WG_CHUNK, 2), MLP_THREADS, 0, s>>>(T, batch)));
    read_back(ctx, h_grad, q->grad, MLP_NP * sizeof(float));
    if (h_loss) {
      read_back(ctx, h_loss, d_loss.p, sizeof(float));
      *h_loss /= float(batch);
    }
    BS_CUDA(cudaMemsetAsync(q->grad, 0, MLP_NP * sizeof(float), s));
  });
}

// Band lookup of a volume (hash of its leaf origins built into `hb`).
static BandLookup band_of(bs_ctx* ctx, const bs_volume* v, LeafHashBuf& hb) {
  BandLookup B{};
  if (!v || !v->n_leaves) return B;
  hb.build(ctx, v->d_origins, v->n_leaves, v->n_leaves);
  B.hash = hb.h;
  B.masks = v->d_masks;
  B.inv_h = 1.0f / v->h;
  B.any = 1;
  return B;
}

// flags[i] = 1 when point i's nearest grid point is an active voxel of the
// volume (the narrow band).
bs_status bs_volume_band_flags(bs_ctx* ctx, const bs_volume* v, const float* d_points, uint64_t n, uint32_t* d_flags) {
  if (!ctx || !v || (n && (!d_points || !d_flags))) return BS_ERR_INVALID_ARG;
  return mlp_guard(ctx, [&] {
    if (!n) return;
    LeafHashBuf hb;
    const BandLookup B = band_of(ctx, v, hb);
    BS_KERNEL(ctx, "k_band_flags", (k_band_flags<<<grid_for(n, 256), 256, 0, ctx->stream>>>(B, d_points, n, d_flags)));
    BS_CUDA(cudaStreamSynchronize(ctx->stream));
  });
}

// Winding numbers of n points: the network's prediction where the point lies
// outside the band volume (if given) and the prediction lies more than
// `margin` from `thresh`; the tree traversal (accuracy scale beta) everywhere
// else.  *n_traversed: how many points went to the traversal.
bs_status bs_mlp_classify(bs_ctx* ctx, const bs_mlp* q, const bs_wn_tree* tree, const bs_volume* band,
                          const float* d_points, uint64_t n, float thresh, float margin, float beta, float* d_out,
                          uint64_t* n_traversed) {
  if (!ctx || !q || !tree || (n && (!d_points || !d_out))) return BS_ERR_INVALID_ARG;
  return mlp_guard(ctx, [&] {
    if (n_traversed) *n_traversed = 0;
    if (!n) return;
    if (n >= (1ull << 32)) fail(BS_ERR_CAPACITY, "mlp classify: more than 2^32 points in one call");
    cudaStream_t s = ctx->stream;
    LeafHashBuf hb;
    const BandLookup B = band_of(ctx, band, hb);
    DBuf<uint32_t> unsure(ctx, n + 1), off(ctx, n + 1);
    BS_CUDA(cudaMemsetAsync(unsure.p + n, 0, sizeof(uint32_t), s));
    const unsigned grid = grid_for((n + 15) / 16, MLP_WARPS);
    BS_KERNEL(ctx, "k_mlp_predict", (k_mlp_predict<<<std::min(grid, 152u * 16u), MLP_THREADS, 0, s>>>(
                                         q->weights(), d_points, n, d_out, thresh, margin, unsure.p, B)));
    scan_u32(ctx, unsure.p, off.p, n + 1);
    uint32_t nu = 0;
    read_back(ctx, &nu, off.p + n, sizeof(uint32_t));
    if (n_traversed) *n_traversed = nu;
    if (!nu) return;
    DBuf<uint32_t> list(ctx, nu);
    DBuf<float> pts(ctx, uint64_t(nu) * 3), wn(ctx, nu);
    BS_KERNEL(ctx, "k_unsure_list", (k_unsure_list<<<grid_for(n, 256), 256, 0, s>>>(unsure.p, off.p, n, list.p)));
    BS_KERNEL(ctx, "k_gather3", (k_gather3<<<grid_for(nu, 256), 256, 0, s>>>(d_points, list.p, nu, pts.p, nullptr,
                                                                            nullptr)));
    const bs_status st = bs_winding_numbers_approximate(ctx, tree, pts.p, nu, beta, wn.p);
    if (st != BS_OK) fail(st, ctx->last_error.c_str());
    BS_KERNEL(ctx, "k_scatter1", (k_scatter1<<<grid_for(nu, 256), 256, 0, s>>>(wn.p, list.p, nu, d_out)));
    BS_CUDA(cudaStreamSynchronize(s));
  });
}

}  // extern "C"
