// Dual contouring on the GPU (voxel/meshing/dual_contouring.rs:16-473).
//
// Three passes over the leaves, each counted, scanned and then written into
// compact arrays indexed through per-leaf bit masks:
//   1. edge crossings: for every active voxel and axis whose +1 neighbour is
//      active with the other sign, the crossing point and the normal from
//      interpolated central / one-sided differences (dual_contouring.rs:249-387);
//   2. cell vertices: for every cell whose 8 corners are active and not all of
//      one sign, the particle solver over its crossings (find_feature_point,
//      dual_contouring.rs:429-458, 50 damped iterations);
//   3. quads: for every sign-change edge whose 4 surrounding cells have
//      vertices, two triangles, flipped when the first end is inside, scaled
//      by the voxel size; exactly degenerate triangles are dropped
//      (dual_contouring.rs:62-79, 93-174).
// Every float operation follows the reference's order without fused
// multiply-adds, so the vertices are bit-identical to the reference's.  The
// face order is deterministic (leaves in volume order, voxels, axes); the
// reference's own order depends on thread scheduling.
#include <cub/device/device_scan.cuh>

#include "bs_internal.cuh"
#include "dc.cuh"
#include "leaf_hash.cuh"
#include "volume_upper.cuh"

namespace bs {

template <class T>
static void scan_e(bs_ctx* ctx, const T* in, T* out, size_t n) {
  size_t tmp = 0;
  BS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, in, out, n, ctx->stream));
  DBuf<uint8_t> t(ctx, tmp);
  BS_CUDA(cub::DeviceScan::ExclusiveSum(t.p, tmp, in, out, n, ctx->stream));
}

// 27 neighbour leaves around a leaf, index (dx+1)*9 + (dy+1)*3 + (dz+1).
__device__ __forceinline__ void load_neighbours(const DcVol& V, int4 org, int* nb) {
  for (int k = threadIdx.x; k < 27; k += blockDim.x) {
    const int dx = k / 9 - 1, dy = (k / 3) % 3 - 1, dz = k % 3 - 1;
    nb[k] = V.hash.find(org.x + 8 * dx, org.y + 8 * dy, org.z + 8 * dz);
  }
}

// Value at voxel (x, y, z) given relative to the leaf origin (in [-8, 16)),
// as the tree's `at` returns it: an active leaf voxel, or, for a voxel
// outside every leaf, its active tile's value.  Inactive voxels of a leaf
// have no value.
// TILES: the volume has active tiles (the kernels reading neighbour values
// come in both forms, so tile-free volumes run without the lookup).
template <bool TILES>
__device__ __forceinline__ bool at(const DcVol& V, const int* nb, int4 org, int x, int y, int z, float& v) {
  const int k = ((x >> 3) + 1) * 9 + ((y >> 3) + 1) * 3 + ((z >> 3) + 1);
  const int l = nb[k];
  if (l < 0) return TILES && tile_value(V.tiles, org.x + x, org.y + y, org.z + z, v);
  const int o = ((x & 7) << 6) | ((y & 7) << 3) | (z & 7);
  if (!((V.msk[uint64_t(l) * 16 + (o >> 5)] >> (o & 31)) & 1u)) return false;
  v = V.val[uint64_t(l) * 512 + o];
  return true;
}

// dual_contouring.rs:362-386
template <bool TILES>
__device__ __forceinline__ bool grad(const DcVol& V, const int* nb, int4 org, int x, int y, int z, int axis,
                                     float& g) {
  const int lx = axis == 0 ? 1 : 0, ly = axis == 1 ? 1 : 0, lz = axis == 2 ? 1 : 0;
  float vp, vl, vr;
  const bool hp = at<TILES>(V, nb, org, x, y, z, vp);
  const bool hl = at<TILES>(V, nb, org, x - lx, y - ly, z - lz, vl);
  const bool hr = at<TILES>(V, nb, org, x + lx, y + ly, z + lz, vr);
  if (hp && hl && hr) { g = fmul(fsub(vr, vl), 0.5f); return true; }
  if (hp && hr) { g = fsub(vr, vp); return true; }
  if (hp && hl) { g = fsub(vp, vl); return true; }
  return false;  // the reference stops with unreachable!() here
}

// Pass 1a: crossing masks.  cm[l][dir][16]
template <bool TILES>
__global__ void __launch_bounds__(128) k_dc_edge_mask(DcVol V, uint64_t n, uint32_t* __restrict__ cm,
                                                      uint32_t* __restrict__ ccount) {
  __shared__ int nb[27];
  const uint64_t l = blockIdx.x;
  if (l >= n) return;
  const int4 org = V.org[l];
  load_neighbours(V, org, nb);
  __syncthreads();
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  uint32_t cnt[3] = {0, 0, 0};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int o = t + 128 * k;
    const int x = o >> 6, y = (o >> 3) & 7, z = o & 7;
    float v1;
    const bool h1 = at<TILES>(V, nb, org, x, y, z, v1);
#pragma unroll
    for (int dir = 0; dir < 3; ++dir) {
      float v2;
      const bool cross = h1 && at<TILES>(V, nb, org, x + (dir == 0), y + (dir == 1), z + (dir == 2), v2) &&
                         (signbit(v1) != signbit(v2));
      const uint32_t m = __ballot_sync(0xffffffffu, cross);
      if (lane == 0) {
        cm[(l * 3 + dir) * 16 + w + 4 * k] = m;
        cnt[dir] += __popc(m);
      }
    }
  }
  __shared__ uint32_t sc[3];
  if (t < 3) sc[t] = 0;
  __syncthreads();
  if (lane == 0)
    for (int dir = 0; dir < 3; ++dir) atomicAdd(&sc[dir], cnt[dir]);
  __syncthreads();
  if (t < 3) ccount[l * 3 + t] = sc[t];
  if (l == n - 1 && t == 3) ccount[n * 3] = 0;
}

__device__ __forceinline__ uint32_t rank512(const uint32_t* m, int o) {
  uint32_t r = 0;
  for (int w = 0; w < (o >> 5); ++w) r += __popc(m[w]);
  return r + __popc(m[o >> 5] & ((1u << (o & 31)) - 1u));
}

// Pass 1b: crossing points and normals (dual_contouring.rs:249-313).
template <bool TILES>
__global__ void __launch_bounds__(128) k_dc_edge_points(DcVol V, uint64_t n, const uint32_t* __restrict__ cm,
                                                        const uint32_t* __restrict__ coff, float* __restrict__ pts,
                                                        DcStats* st) {
  __shared__ int nb[27];
  const uint64_t l = blockIdx.x;
  if (l >= n) return;
  const int4 org = V.org[l];
  load_neighbours(V, org, nb);
  __syncthreads();
  for (int k = threadIdx.x; k < 3 * 512; k += blockDim.x) {
    const int dir = k >> 9, o = k & 511;
    const uint32_t* m = cm + (l * 3 + dir) * 16;
    if (!((m[o >> 5] >> (o & 31)) & 1u)) continue;
    const int x = o >> 6, y = (o >> 3) & 7, z = o & 7;
    const int x2 = x + (dir == 0), y2 = y + (dir == 1), z2 = z + (dir == 2);
    float v1, v2;
    at<TILES>(V, nb, org, x, y, z, v1);
    at<TILES>(V, nb, org, x2, y2, z2, v2);
    const float t = (v1 == v2) ? 0.5f : fdiv(v1, fsub(v1, v2));
    float p[3] = {__int2float_rn(org.x + x), __int2float_rn(org.y + y), __int2float_rn(org.z + z)};
    p[dir] = fadd(p[dir], t);
    float nrm[3];
    bool ok = true;
    for (int a = 0; a < 3; ++a) {
      float g1, g2;
      ok = ok && grad<TILES>(V, nb, org, x, y, z, a, g1) && grad<TILES>(V, nb, org, x2, y2, z2, a, g2);
      if (ok) nrm[a] = fadd(fmul(fsub(1.0f, t), g1), fmul(t, g2));
    }
    if (!ok) {
      atomicExch(&st->error, 1);
      continue;
    }
    const float len = fsqrt(fadd(fadd(fmul(nrm[0], nrm[0]), fmul(nrm[1], nrm[1])), fmul(nrm[2], nrm[2])));
    const uint64_t idx = coff[l * 3 + dir] + rank512(m, o);
    float* q = pts + idx * 6;
    q[0] = p[0];
    q[1] = p[1];
    q[2] = p[2];
    q[3] = fdiv(nrm[0], len);
    q[4] = fdiv(nrm[1], len);
    q[5] = fdiv(nrm[2], len);
  }
}

// voxel/utils.rs:88-97 and dual_contouring.rs:410-423
__constant__ int8_t c_cube[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                    {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
__constant__ int8_t c_edges[12][4] = {{0, 0, 0, 0}, {0, 0, 0, 1}, {0, 0, 0, 2}, {1, 0, 0, 1},
                                      {1, 0, 0, 2}, {0, 0, 1, 0}, {0, 0, 1, 1}, {0, 1, 0, 0},
                                      {0, 1, 0, 2}, {1, 0, 1, 1}, {0, 1, 1, 0}, {1, 1, 0, 2}};
__constant__ int8_t c_cells[3][4][3] = {{{0, 0, 0}, {0, 0, -1}, {0, -1, -1}, {0, -1, 0}},
                                        {{0, 0, 0}, {-1, 0, 0}, {-1, 0, -1}, {0, 0, -1}},
                                        {{0, -1, 0}, {-1, -1, 0}, {-1, 0, 0}, {0, 0, 0}}};

// Pass 2a: cells with all 8 corners active and a sign change (dual_contouring.rs:193-217).
template <bool TILES>
__global__ void __launch_bounds__(128) k_dc_cell_mask(DcVol V, uint64_t n, uint32_t* __restrict__ cellm,
                                                      uint32_t* __restrict__ ccount) {
  __shared__ int nb[27];
  __shared__ uint32_t sc;
  const uint64_t l = blockIdx.x;
  if (l >= n) return;
  const int4 org = V.org[l];
  load_neighbours(V, org, nb);
  if (threadIdx.x == 0) sc = 0;
  __syncthreads();
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int o = t + 128 * k;
    const int x = o >> 6, y = (o >> 3) & 7, z = o & 7;
    bool ok = true, any_neg = false, any_pos = false;
    for (int c = 0; c < 8 && ok; ++c) {
      float v;
      ok = at<TILES>(V, nb, org, x + c_cube[c][0], y + c_cube[c][1], z + c_cube[c][2], v);
      if (ok) {
        if (signbit(v)) any_neg = true;
        else any_pos = true;
      }
    }
    const uint32_t m = __ballot_sync(0xffffffffu, ok && any_neg && any_pos);
    if (lane == 0) {
      cellm[l * 16 + w + 4 * k] = m;
      atomicAdd(&sc, __popc(m));
    }
  }
  __syncthreads();
  if (t == 0) ccount[l] = sc;
  if (l == n - 1 && t == 1) ccount[n] = 0;
}

// Looks up the crossing stored for edge (x, y, z, dir) of the leaf's neighbourhood.
__device__ __forceinline__ const float* edge_point(const int* nb, const uint32_t* cm, const uint32_t* coff,
                                                   const float* pts, int x, int y, int z, int dir) {
  const int k = ((x >> 3) + 1) * 9 + ((y >> 3) + 1) * 3 + ((z >> 3) + 1);
  const int l = nb[k];
  if (l < 0) return nullptr;
  const int o = ((x & 7) << 6) | ((y & 7) << 3) | (z & 7);
  const uint32_t* m = cm + (uint64_t(l) * 3 + dir) * 16;
  if (!((m[o >> 5] >> (o & 31)) & 1u)) return nullptr;
  return pts + (coff[uint64_t(l) * 3 + dir] + rank512(m, o)) * 6;
}

// Pass 2b: the particle solver (dual_contouring.rs:429-458).
__global__ void __launch_bounds__(128) k_dc_cell_points(DcVol V, uint64_t n, const uint32_t* __restrict__ cm,
                                                        const uint32_t* __restrict__ coff, const float* __restrict__ pts,
                                                        const uint32_t* __restrict__ cellm,
                                                        const uint32_t* __restrict__ celloff, float* __restrict__ cells) {
  __shared__ int nb[27];
  const uint64_t l = blockIdx.x;
  if (l >= n) return;
  const int4 org = V.org[l];
  load_neighbours(V, org, nb);
  __syncthreads();
  const uint32_t* m = cellm + l * 16;
  for (int o = threadIdx.x; o < 512; o += blockDim.x) {
    if (!((m[o >> 5] >> (o & 31)) & 1u)) continue;
    const int x = o >> 6, y = (o >> 3) & 7, z = o & 7;
    const float* ip[12];
    int np = 0;
    for (int e = 0; e < 12; ++e) {
      const float* q = edge_point(nb, cm, coff, pts, x + c_edges[e][0], y + c_edges[e][1], z + c_edges[e][2],
                                  c_edges[e][3]);
      if (q) ip[np++] = q;
    }
    const float len = __int2float_rn(np);
    float c0 = 0.f, c1 = 0.f, c2 = 0.f;
    for (int i = 0; i < np; ++i) {
      c0 = fadd(c0, ip[i][0]);
      c1 = fadd(c1, ip[i][1]);
      c2 = fadd(c2, ip[i][2]);
    }
    c0 = fdiv(c0, len);
    c1 = fdiv(c1, len);
    c2 = fdiv(c2, len);
    for (int it = 0; it < 50; ++it) {
      float f0 = 0.f, f1 = 0.f, f2 = 0.f;
      for (int i = 0; i < np; ++i) {
        const float* q = ip[i];
        const float d = fadd(fadd(fmul(q[3], fsub(c0, q[0])), fmul(q[4], fsub(c1, q[1]))), fmul(q[5], fsub(c2, q[2])));
        f0 = fadd(f0, fmul(fmul(q[3], -1.0f), d));
        f1 = fadd(f1, fmul(fmul(q[4], -1.0f), d));
        f2 = fadd(f2, fmul(fmul(q[5], -1.0f), d));
      }
      const float damping = fsub(1.0f, fdiv(__int2float_rn(it), 50.0f));
      c0 = fadd(c0, fdiv(fmul(f0, damping), len));
      c1 = fadd(c1, fdiv(fmul(f1, damping), len));
      c2 = fadd(c2, fdiv(fmul(f2, damping), len));
      if (fadd(fadd(fmul(f0, f0), fmul(f1, f1)), fmul(f2, f2)) < 1e-6f) break;
    }
    float* out = cells + (celloff[l] + rank512(m, o)) * 3;
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
  }
}

// Eigen-decomposition of a symmetric 3x3 matrix by cyclic Jacobi rotations
// (Jacobi 1846; Rutishauser's update): a is overwritten, w = eigenvalues,
// columns of V = eigenvectors.
__device__ __forceinline__ void sym3_jacobi(double a[3][3], double V[3][3], double w[3]) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) V[r][c] = r == c ? 1.0 : 0.0;
  const int P[3] = {0, 0, 1}, Q[3] = {1, 2, 2};
  for (int sweep = 0; sweep < 24; ++sweep) {
    const double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
    const double dia = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
    if (off <= 1e-30 * dia || off == 0.0) break;
    for (int k = 0; k < 3; ++k) {
      const int p = P[k], q = Q[k];
      const double apq = a[p][q];
      if (apq == 0.0) continue;
      const double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
      const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
      const double c = 1.0 / sqrt(t * t + 1.0), s = t * c, tau = s / (1.0 + c);
      a[p][p] -= t * apq;
      a[q][q] += t * apq;
      a[p][q] = a[q][p] = 0.0;
      for (int r = 0; r < 3; ++r) {
        if (r != p && r != q) {
          const double arp = a[r][p], arq = a[r][q];
          a[r][p] = a[p][r] = arp - s * (arq + tau * arp);
          a[r][q] = a[q][r] = arq + s * (arp - tau * arq);
        }
        const double vrp = V[r][p], vrq = V[r][q];
        V[r][p] = vrp - s * (vrq + tau * vrp);
        V[r][q] = vrq + s * (vrp - tau * vrq);
      }
    }
  }
  for (int k = 0; k < 3; ++k) w[k] = a[k][k];
}

// Pass 2b, QEF mode (no reference counterpart): the point minimising
// sum_i (n_i . (x - p_i))^2 over the cell's crossings p_i with normals n_i,
// taken as m + pinv(A^T A) (A^T b - A^T A m) around the crossings' mass
// point m, with eigenvalues below QEF_TRUNC of the largest dropped; all in
// double.
constexpr double QEF_TRUNC = 0.1;

__global__ void __launch_bounds__(128) k_dc_cell_qef(DcVol V, uint64_t n, const uint32_t* __restrict__ cm,
                                                     const uint32_t* __restrict__ coff, const float* __restrict__ pts,
                                                     const uint32_t* __restrict__ cellm,
                                                     const uint32_t* __restrict__ celloff, float* __restrict__ cells) {
  __shared__ int nb[27];
  const uint64_t l = blockIdx.x;
  if (l >= n) return;
  const int4 org = V.org[l];
  load_neighbours(V, org, nb);
  __syncthreads();
  const uint32_t* m = cellm + l * 16;
  for (int o = threadIdx.x; o < 512; o += blockDim.x) {
    if (!((m[o >> 5] >> (o & 31)) & 1u)) continue;
    const int x = o >> 6, y = (o >> 3) & 7, z = o & 7;
    double mp[3] = {0.0, 0.0, 0.0}, ata[3][3] = {{0.0}}, atb[3] = {0.0, 0.0, 0.0};
    int np = 0;
    for (int e = 0; e < 12; ++e) {
      const float* q = edge_point(nb, cm, coff, pts, x + c_edges[e][0], y + c_edges[e][1], z + c_edges[e][2],
                                  c_edges[e][3]);
      if (!q) continue;
      ++np;
      const double p[3] = {q[0], q[1], q[2]}, nn[3] = {q[3], q[4], q[5]};
      const double d = nn[0] * p[0] + nn[1] * p[1] + nn[2] * p[2];
      for (int r = 0; r < 3; ++r) {
        mp[r] += p[r];
        atb[r] += nn[r] * d;
        for (int c = 0; c < 3; ++c) ata[r][c] += nn[r] * nn[c];
      }
    }
    for (int r = 0; r < 3; ++r) mp[r] /= double(np);
    double rhs[3];
    for (int r = 0; r < 3; ++r) rhs[r] = atb[r] - (ata[r][0] * mp[0] + ata[r][1] * mp[1] + ata[r][2] * mp[2]);
    double a[3][3], Vm[3][3], w[3];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) a[r][c] = ata[r][c];
    sym3_jacobi(a, Vm, w);
    const double wmax = fmax(fabs(w[0]), fmax(fabs(w[1]), fabs(w[2])));
    double xs[3] = {mp[0], mp[1], mp[2]};
    for (int k = 0; k < 3; ++k) {
      if (!(fabs(w[k]) > QEF_TRUNC * wmax)) continue;
      const double proj = (Vm[0][k] * rhs[0] + Vm[1][k] * rhs[1] + Vm[2][k] * rhs[2]) / w[k];
      for (int r = 0; r < 3; ++r) xs[r] += proj * Vm[r][k];
    }
    float* out = cells + (celloff[l] + rank512(m, o)) * 3;
    out[0] = float(xs[0]);
    out[1] = float(xs[1]);
    out[2] = float(xs[2]);
  }
}

__device__ __forceinline__ const float* cell_point(const int* nb, const uint32_t* cellm, const uint32_t* celloff,
                                                   const float* cells, int x, int y, int z) {
  const int k = ((x >> 3) + 1) * 9 + ((y >> 3) + 1) * 3 + ((z >> 3) + 1);
  const int l = nb[k];
  if (l < 0) return nullptr;
  const int o = ((x & 7) << 6) | ((y & 7) << 3) | (z & 7);
  const uint32_t* m = cellm + uint64_t(l) * 16;
  if (!((m[o >> 5] >> (o & 31)) & 1u)) return nullptr;
  return cells + (celloff[l] + rank512(m, o)) * 3;
}

__device__ __forceinline__ bool degenerate(const float* a, const float* b, const float* c) {
  const float e0 = fsub(b[0], a[0]), e1 = fsub(b[1], a[1]), e2 = fsub(b[2], a[2]);
  const float f0 = fsub(c[0], a[0]), f1 = fsub(c[1], a[1]), f2 = fsub(c[2], a[2]);
  const float x = fsub(fmul(e1, f2), fmul(e2, f1)), y = fsub(fmul(e2, f0), fmul(e0, f2)),
              z = fsub(fmul(e0, f1), fmul(e1, f0));
  return fadd(fadd(fmul(x, x), fmul(y, y)), fmul(z, z)) == 0.0f;
}

// Pass 3: the two triangles of every quad around a sign-change edge
// (dual_contouring.rs:93-139), scaled by the voxel size, minus exactly
// degenerate ones (dual_contouring.rs:62-79).  Writes up to 6 triangles of
// voxel (x, y, z) to `out` (when not null) and returns how many there are.
__device__ __forceinline__ int voxel_tris(const DcVol& V, const int* nb, const uint32_t* __restrict__ cm,
                                          const uint32_t* __restrict__ cellm, const uint32_t* __restrict__ celloff,
                                          const float* __restrict__ cells, uint64_t l, int x, int y, int z, float h,
                                          float* out) {
  const int o = (x << 6) | (y << 3) | z;
  const uint32_t any = (cm[(l * 3 + 0) * 16 + (o >> 5)] | cm[(l * 3 + 1) * 16 + (o >> 5)] |
                        cm[(l * 3 + 2) * 16 + (o >> 5)]) >> (o & 31);
  if (!(any & 1u)) return 0;
  float v1 = 0.f;
  v1 = V.val[l * 512 + o];  // active: the voxel has a crossing
  int nt = 0;
  for (int dir = 0; dir < 3; ++dir) {
    if (!((cm[(l * 3 + dir) * 16 + (o >> 5)] >> (o & 31)) & 1u)) continue;
    const float* q[4];
    bool ok = true;
    for (int c = 0; c < 4 && ok; ++c) {
      q[c] = cell_point(nb, cellm, celloff, cells, x + c_cells[dir][c][0], y + c_cells[dir][c][1],
                        z + c_cells[dir][c][2]);
      ok = q[c] != nullptr;
    }
    if (!ok) continue;
    // [p0, p1, p2, p2, p3, p0], with (1,2) and (4,5) swapped when v1 < 0
    const float* f[6] = {q[0], q[1], q[2], q[2], q[3], q[0]};
    if (signbit(v1)) {
      const float* t = f[1];
      f[1] = f[2];
      f[2] = t;
      t = f[4];
      f[4] = f[5];
      f[5] = t;
    }
    for (int tt = 0; tt < 2; ++tt) {
      float a[3], b[3], c[3];
      for (int i = 0; i < 3; ++i) {
        a[i] = fmul(f[3 * tt][i], h);
        b[i] = fmul(f[3 * tt + 1][i], h);
        c[i] = fmul(f[3 * tt + 2][i], h);
      }
      if (degenerate(a, b, c)) continue;
      if (out) {
        float* d = out + nt * 9;
        for (int i = 0; i < 3; ++i) {
          d[i] = a[i];
          d[3 + i] = b[i];
          d[6 + i] = c[i];
        }
      }
      ++nt;
    }
  }
  return nt;
}

// Count pass (tris == nullptr): vcount[l] = triangles of leaf l, and the
// counts of thread t's voxels t, t + 128, t + 256, t + 384 as four 4-bit
// fields in packed[l * 128 + t] (a voxel has at most 6 triangles).  Write
// pass: the leaf's triangles from tris + voff[l], voxels in ascending index
// order; one block scan of the four counts packed in 16-bit fields of a
// 64-bit word gives every round's prefix at once.
__global__ void __launch_bounds__(128) k_dc_quads(DcVol V, uint64_t n, const uint32_t* __restrict__ cm,
                                                  const uint32_t* __restrict__ cellm, const uint32_t* __restrict__ celloff,
                                                  const float* __restrict__ cells, float h, uint64_t* __restrict__ vcount,
                                                  const uint64_t* __restrict__ voff, uint16_t* __restrict__ packed,
                                                  float* __restrict__ tris) {
  __shared__ int nb[27];
  __shared__ unsigned long long wsum[4];
  const uint64_t l = blockIdx.x;
  if (l >= n) return;
  const int4 org = V.org[l];
  load_neighbours(V, org, nb);
  __syncthreads();
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  if (!tris) {
    uint32_t pk = 0, mine = 0;
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
      const int o = t + 128 * k;
      const uint32_t c = uint32_t(voxel_tris(V, nb, cm, cellm, celloff, cells, l, o >> 6, (o >> 3) & 7, o & 7, h, nullptr));
      pk |= c << (4 * k);
      mine += c;
    }
    packed[l * 128 + t] = uint16_t(pk);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, d);
    if (lane == 0) wsum[w] = mine;
    __syncthreads();
    if (t == 0) vcount[l] = wsum[0] + wsum[1] + wsum[2] + wsum[3];
    if (l == n - 1 && t == 1) vcount[n] = 0;
    return;
  }
  const uint32_t pk = packed[l * 128 + t];
  if (__syncthreads_or(pk) == 0) return;  // no triangles in this leaf
  // counts of rounds 0..3 in 16-bit fields (a round's prefix is at most 768)
  const unsigned long long mine = (unsigned long long)(pk & 15u) | ((unsigned long long)((pk >> 4) & 15u) << 16) |
                                  ((unsigned long long)((pk >> 8) & 15u) << 32) |
                                  ((unsigned long long)(pk >> 12) << 48);
  unsigned long long inc = mine;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long v = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += v;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  unsigned long long before = 0;
  for (int i = 0; i < w; ++i) before += wsum[i];
  const unsigned long long total = wsum[0] + wsum[1] + wsum[2] + wsum[3];
  const unsigned long long excl = before + inc - mine;
  uint64_t run = voff[l];
#pragma unroll 1
  for (int k = 0; k < 4; ++k) {
    const uint32_t c = (pk >> (4 * k)) & 15u;
    if (c) {
      const int o = t + 128 * k;
      const uint64_t pos = run + ((excl >> (16 * k)) & 0xffffull);
      voxel_tris(V, nb, cm, cellm, celloff, cells, l, o >> 6, (o >> 3) & 7, o & 7, h, tris + pos * 9);
    }
    run += (total >> (16 * k)) & 0xffffull;
  }
}

// Launches of the kernels that read neighbour values, in the form for
// volumes with or without active tiles (also used by dc_noalloc.cu).
void launch_dc_edge_mask(bool tiles, const DcVol& V, uint64_t n, uint32_t* cm, uint32_t* ccnt, cudaStream_t s) {
  if (tiles)
    k_dc_edge_mask<true><<<unsigned(n), 128, 0, s>>>(V, n, cm, ccnt);
  else
    k_dc_edge_mask<false><<<unsigned(n), 128, 0, s>>>(V, n, cm, ccnt);
}
void launch_dc_edge_points(bool tiles, const DcVol& V, uint64_t n, const uint32_t* cm, const uint32_t* coff,
                           float* pts, DcStats* st, cudaStream_t s) {
  if (tiles)
    k_dc_edge_points<true><<<unsigned(n), 128, 0, s>>>(V, n, cm, coff, pts, st);
  else
    k_dc_edge_points<false><<<unsigned(n), 128, 0, s>>>(V, n, cm, coff, pts, st);
}
void launch_dc_cell_mask(bool tiles, const DcVol& V, uint64_t n, uint32_t* cellm, uint32_t* cellc, cudaStream_t s) {
  if (tiles)
    k_dc_cell_mask<true><<<unsigned(n), 128, 0, s>>>(V, n, cellm, cellc);
  else
    k_dc_cell_mask<false><<<unsigned(n), 128, 0, s>>>(V, n, cellm, cellc);
}

static bool has_active_tiles(const bs_volume* v) { return v->n_tiles != 0; }

void dual_contour_impl(bs_ctx* ctx, bs_volume* v, float voxel_size, int mode) {
  if (v->dc_valid && v->dc_h == voxel_size && v->dc_mode == mode) return;
  cudaStream_t s = ctx->stream;
  dfree(ctx, v->d_dc_tris);
  v->d_dc_tris = nullptr;
  v->n_dc_tris = 0;
  const uint64_t n = v->n_leaves;
  if (n == 0) {
    v->dc_valid = true;
    v->dc_h = voxel_size;
    v->dc_mode = mode;
    return;
  }
  LeafHashBuf hb, h1, h2;
  hb.build(ctx, v->d_origins, n, n);
  DcVol V{v->d_origins, v->d_values, v->d_masks, hb.h, TileLookup{}};
  if (has_active_tiles(v)) {
    // The reference stops at active tiles (todo!(), dual_contouring.rs:139,
    // 186, 347).  Here the passes still visit the leaves only and read every
    // neighbour, cell corner and gradient stencil voxel as the tree's `at`
    // returns it, so a voxel of an active tile has the tile's value.
    const Upper* u = v->upper;
    if (!u) fail(BS_ERR_UNSUPPORTED, "dual contouring: tiles without internal levels");
    h1.build(ctx, u->l1.d_key, u->l1.n, u->l1.n);
    h2.build(ctx, u->l2.d_key, u->l2.n, u->l2.n);
    V.tiles = TileLookup{h1.h, h2.h, u->l1.d_state, u->l1.d_tile, u->l2.d_state, u->l2.d_tile, 1};
  }
  DBuf<DcStats> st(ctx, 1);
  BS_CUDA(cudaMemsetAsync(st.p, 0, sizeof(DcStats), s));
  // 1. crossings
  DBuf<uint32_t> cm(ctx, n * 3 * 16), ccnt(ctx, n * 3 + 1), coff(ctx, n * 3 + 1);
  BS_KERNEL(ctx, "k_dc_edge_mask", launch_dc_edge_mask(V.tiles.any, V, n, cm.p, ccnt.p, s));
  scan_e(ctx, ccnt.p, coff.p, n * 3 + 1);
  uint32_t ne = 0;
  read_back(ctx, &ne, coff.p + n * 3, sizeof(uint32_t));
  DBuf<float> pts(ctx, uint64_t(ne) * 6);
  BS_KERNEL(ctx, "k_dc_edge_points", launch_dc_edge_points(V.tiles.any, V, n, cm.p, coff.p, pts.p, st.p, s));
  // 2. cells
  DBuf<uint32_t> cellm(ctx, n * 16), cellc(ctx, n + 1), celloff(ctx, n + 1);
  BS_KERNEL(ctx, "k_dc_cell_mask", launch_dc_cell_mask(V.tiles.any, V, n, cellm.p, cellc.p, s));
  scan_e(ctx, cellc.p, celloff.p, n + 1);
  uint32_t nc = 0;
  read_back(ctx, &nc, celloff.p + n, sizeof(uint32_t));
  DBuf<float> cells(ctx, uint64_t(nc) * 3);
  if (mode == 1)
    BS_KERNEL(ctx, "k_dc_cell_qef", (k_dc_cell_qef<<<unsigned(n), 128, 0, s>>>(V, n, cm.p, coff.p, pts.p, cellm.p, celloff.p, cells.p)));
  else
    BS_KERNEL(ctx, "k_dc_cell_points", (k_dc_cell_points<<<unsigned(n), 128, 0, s>>>(V, n, cm.p, coff.p, pts.p, cellm.p, celloff.p, cells.p)));
  // 3. quads
  DBuf<uint64_t> vcnt(ctx, n + 1), voff(ctx, n + 1);
  DBuf<uint16_t> packed(ctx, n * 128);
  BS_KERNEL(ctx, "k_dc_quads_count", (k_dc_quads<<<unsigned(n), 128, 0, s>>>(V, n, cm.p, cellm.p, celloff.p, cells.p, voxel_size, vcnt.p, nullptr, packed.p, nullptr)));
  scan_e(ctx, vcnt.p, voff.p, n + 1);
  uint64_t nt = 0;
  read_back(ctx, &nt, voff.p + n, sizeof(uint64_t));
  DcStats hs;
  read_back(ctx, &hs, st.p, sizeof hs);
  if (hs.error == 1)
    fail(BS_ERR_UNSUPPORTED, "dual contouring: gradient at a voxel with no active neighbour on an axis (the reference stops with unreachable!())");
  v->d_dc_tris = dalloc<float>(ctx, uint64_t(nt) * 9);
  if (nt)
    BS_KERNEL(ctx, "k_dc_quads", (k_dc_quads<<<unsigned(n), 128, 0, s>>>(V, n, cm.p, cellm.p, celloff.p, cells.p, voxel_size, nullptr, voff.p, packed.p, v->d_dc_tris)));
  v->n_dc_tris = nt;
  v->dc_valid = true;
  v->dc_h = voxel_size;
  v->dc_mode = mode;
  ctx->last_stats[6] = ne;
  ctx->last_stats[7] = nc;
  ctx->last_stats[8] = BS_STATS_DUAL_CONTOURING;
}

}  // namespace bs
