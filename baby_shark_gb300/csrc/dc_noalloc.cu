// Dual contouring for callers that cannot allocate device memory.
//
// Some hosts of this library run where cudaMalloc is off limits at call
// time: a renderer or simulation that has carved all device memory up front
// and forbids allocations in its frame loop, a real-time thread that must not
// block in the driver's allocator, or a plugin sandbox whose host owns every
// allocation.  bs_dual_contour_noalloc serves them: it takes the volume's
// leaves and the output buffer as device pointers the caller owns, and keeps
// all of its working memory in one file-scope static device array of
// DCNA_SCRATCH_BYTES, which exists on every GPU that loads the library from
// module load until process exit.  It calls no cudaMalloc, cudaFree or
// allocating library routine.
//
// The array is shared by every call on a device and keeps the previous call's
// contents; each call clears what must start empty (the leaf hash and the
// error flag).  Calls whose work overlaps on the GPU (two streams, or two host
// threads) race on the array and must be serialised by the caller.
//
// The first call on a device resolves the array's device address with
// cudaGetSymbolAddress (with that device current) and caches it; make that
// first call before any stream capture.  The cached address belongs to the
// device's primary context: after cudaDeviceReset on that device the module
// is loaded again and the address may change, so this entry point must not
// be used on that device after a reset.
//
// Active tiles (booleans leave them where a whole 8^3 or 128^3 block is
// inside or outside) are passed as exported (origin, size, value); the call
// rebuilds, in the static array, the slot tables of the internal nodes that
// hold them, so every voxel outside the leaves reads what the tree's `at`
// returns there, exactly as bs_dual_contour does.  The call leaves the
// caller's current device as it found it.
#include <cub/device/device_scan.cuh>

#include <mutex>

#include "bs_internal.cuh"
#include "dc.cuh"
#include "leaf_hash.cuh"

namespace bs {

// Declaration of the hash fill kernel in offset.cu (same definition as there).
__global__ void k_hash_insert(LeafHash h, const int4* __restrict__ org, uint64_t n, int* __restrict__ err);

}  // namespace bs

namespace {

// Limits of the static working memory (about 29 MiB in use of 32 MiB).
constexpr uint64_t DCNA_MAX_LEAVES = 2048;       // leaves of the input volume
constexpr uint64_t DCNA_MAX_CROSSINGS = 393216;  // sign-change edges
constexpr uint64_t DCNA_MAX_CELLS = 393216;      // cells that get a vertex
constexpr uint64_t DCNA_HASH_CAP = 8192;         // power of two >= 2 * DCNA_MAX_LEAVES
constexpr uint64_t DCNA_MAX_TILES = 1ull << 20;  // active tiles of the input volume
constexpr uint64_t DCNA_TILE_L1_CAP = 256;       // 128^3 nodes holding 8^3 tiles (slot tables: 8 MiB)
constexpr uint64_t DCNA_TILE_L2_CAP = 16;        // 4096^3 nodes holding 128^3 tiles (slot tables: 4 MiB)
constexpr uint64_t DCNA_SCRATCH_BYTES = 32ull << 20;

__device__ __align__(256) unsigned char g_dc_scratch[DCNA_SCRATCH_BYTES];

struct Carve {  // bump allocation inside the static array, 256-byte aligned
  unsigned char* base;
  uint64_t used = 0;
  template <class T>
  T* take(uint64_t count) {
    used = (used + 255) & ~uint64_t(255);
    T* p = reinterpret_cast<T*>(base + used);
    used += count * sizeof(T);
    if (used > DCNA_SCRATCH_BYTES) throw bs::Error{BS_ERR_CAPACITY, "no-alloc dual contouring: scratch layout exceeds its array"};
    return p;
  }
};

// Restores the calling thread's current device when the call returns.
struct DeviceGuard {
  int prev = -1;
  DeviceGuard() {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

std::mutex g_setup_mutex;
void* g_scratch_ptr[64] = {nullptr};

// Once per device, with that device current: the device address of the array.
unsigned char* scratch_for(int device) {
  if (device < 0 || device >= 64) throw bs::Error{BS_ERR_INVALID_ARG, "device index out of range"};
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[device]) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_dc_scratch);
    if (e != cudaSuccess || !ptr)
      throw bs::Error{BS_ERR_CUDA, std::string("cudaGetSymbolAddress(g_dc_scratch): ") + cudaGetErrorString(e)};
    g_scratch_ptr[device] = ptr;
  }
  return static_cast<unsigned char*>(g_scratch_ptr[device]);
}

__global__ void k_origins_to_int4(const int32_t* __restrict__ o3, uint64_t n, int4* __restrict__ o4) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i < n) o4[i] = make_int4(o3[3 * i], o3[3 * i + 1], o3[3 * i + 2], 0);
}

// Internal nodes that hold tiles: level 1 (128^3, tiles of 8^3) or level 2
// (4096^3, tiles of 128^3).  The node's index is its hash slot, so its slot
// table starts at slot * slots-per-node.
__global__ void k_tile_nodes(const int32_t* __restrict__ o3, const int32_t* __restrict__ sz, uint64_t n,
                             bs::LeafHash h1, bs::LeafHash h2, int* __restrict__ err) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int x = o3[3 * i], y = o3[3 * i + 1], z = o3[3 * i + 2], s = sz[i];
  bool ins;
  int slot;
  if (s == 8) {
    slot = h1.insert_key(x & ~127, y & ~127, z & ~127, ins);
    if (slot >= 0) h1.vals[slot] = slot;
  } else if (s == 128) {
    slot = h2.insert_key(x & ~4095, y & ~4095, z & ~4095, ins);
    if (slot >= 0) h2.vals[slot] = slot;
  } else {
    atomicExch(err, 2);  // not a tile size of this volume layout
    return;
  }
  if (slot < 0) atomicExch(err, 1);
}

// Marks each tile's slot active (-2) with its value.
__global__ void k_tile_slots(const int32_t* __restrict__ o3, const int32_t* __restrict__ sz,
                             const float* __restrict__ tv, uint64_t n, bs::LeafHash h1, bs::LeafHash h2,
                             int* __restrict__ s1, float* __restrict__ t1, int* __restrict__ s2,
                             float* __restrict__ t2) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const int x = o3[3 * i], y = o3[3 * i + 1], z = o3[3 * i + 2];
  if (sz[i] == 8) {
    const int nd = h1.find(x & ~127, y & ~127, z & ~127);
    if (nd < 0) return;
    const uint64_t k = uint64_t(nd) * bs::L1_SLOTS + ((((x >> 3) & 15) << 8) | (((y >> 3) & 15) << 4) | ((z >> 3) & 15));
    s1[k] = -2;
    t1[k] = tv[i];
  } else if (sz[i] == 128) {
    const int nd = h2.find(x & ~4095, y & ~4095, z & ~4095);
    if (nd < 0) return;
    const uint64_t k = uint64_t(nd) * bs::L2_SLOTS + ((((x >> 7) & 31) << 10) | (((y >> 7) & 31) << 5) | ((z >> 7) & 31));
    s2[k] = -2;
    t2[k] = tv[i];
  }
}

inline unsigned nblocks(uint64_t n, unsigned t) { return unsigned((n + t - 1) / t); }

template <class T>
void scan_in(cudaStream_t s, void* temp, size_t temp_bytes, const T* in, T* out, uint64_t n) {
  size_t need = 0;
  BS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, need, in, out, n, s));
  if (need > temp_bytes) throw bs::Error{BS_ERR_CAPACITY, "no-alloc dual contouring: scan workspace too small"};
  BS_CUDA(cub::DeviceScan::ExclusiveSum(temp, need, in, out, n, s));
}

template <class T>
T read1(cudaStream_t s, const T* dev) {
  T v{};
  BS_CUDA(cudaMemcpyAsync(&v, dev, sizeof(T), cudaMemcpyDeviceToHost, s));
  BS_CUDA(cudaStreamSynchronize(s));
  return v;
}

}  // namespace

extern "C" bs_status bs_dual_contour_noalloc(int device, void* stream, const int32_t* d_origins, const float* d_values,
                                             const uint32_t* d_masks, uint64_t n_leaves,
                                             const int32_t* d_tile_origins, const int32_t* d_tile_sizes,
                                             const float* d_tile_values, uint64_t n_tiles, float voxel_size,
                                             float* d_tris, uint64_t capacity, uint64_t* n_tris) {
  using namespace bs;
  if (!n_tris || (n_leaves && (!d_origins || !d_values || !d_masks)) || (capacity && !d_tris) ||
      (n_tiles && (!d_tile_origins || !d_tile_sizes || !d_tile_values)))
    return BS_ERR_INVALID_ARG;
  *n_tris = 0;
  if (n_leaves > DCNA_MAX_LEAVES || n_tiles > DCNA_MAX_TILES) return BS_ERR_CAPACITY;
  DeviceGuard restore_device;
  try {
    BS_CUDA(cudaSetDevice(device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (n_leaves == 0) return BS_OK;
    Carve c{scratch_for(device)};
    const uint64_t n = n_leaves;
    int4* org = c.take<int4>(n);
    unsigned long long* hkeys = c.take<unsigned long long>(DCNA_HASH_CAP);
    int* hvals = c.take<int>(DCNA_HASH_CAP);
    int* herr = c.take<int>(1);
    DcStats* st = c.take<DcStats>(1);
    uint32_t* cm = c.take<uint32_t>(n * 3 * 16);
    uint32_t* ccnt = c.take<uint32_t>(n * 3 + 1);
    uint32_t* coff = c.take<uint32_t>(n * 3 + 1);
    float* pts = c.take<float>(DCNA_MAX_CROSSINGS * 6);
    uint32_t* cellm = c.take<uint32_t>(n * 16);
    uint32_t* cellc = c.take<uint32_t>(n + 1);
    uint32_t* celloff = c.take<uint32_t>(n + 1);
    float* cells = c.take<float>(DCNA_MAX_CELLS * 3);
    uint64_t* vcnt = c.take<uint64_t>(n + 1);
    uint64_t* voff = c.take<uint64_t>(n + 1);
    uint16_t* packed = c.take<uint16_t>(n * 128);
    const size_t temp_bytes = 1u << 20;
    void* temp = c.take<unsigned char>(temp_bytes);
    TileLookup tiles{};
    if (n_tiles) {
      tiles.h1.keys = c.take<unsigned long long>(DCNA_TILE_L1_CAP);
      tiles.h1.vals = c.take<int>(DCNA_TILE_L1_CAP);
      tiles.h1.mask = DCNA_TILE_L1_CAP - 1;
      tiles.h2.keys = c.take<unsigned long long>(DCNA_TILE_L2_CAP);
      tiles.h2.vals = c.take<int>(DCNA_TILE_L2_CAP);
      tiles.h2.mask = DCNA_TILE_L2_CAP - 1;
      int* s1 = c.take<int>(DCNA_TILE_L1_CAP * L1_SLOTS);
      float* t1 = c.take<float>(DCNA_TILE_L1_CAP * L1_SLOTS);
      int* s2 = c.take<int>(DCNA_TILE_L2_CAP * L2_SLOTS);
      float* t2 = c.take<float>(DCNA_TILE_L2_CAP * L2_SLOTS);
      BS_CUDA(cudaMemsetAsync(tiles.h1.keys, 0xff, DCNA_TILE_L1_CAP * sizeof(unsigned long long), s));
      BS_CUDA(cudaMemsetAsync(tiles.h1.vals, 0xff, DCNA_TILE_L1_CAP * sizeof(int), s));
      BS_CUDA(cudaMemsetAsync(tiles.h2.keys, 0xff, DCNA_TILE_L2_CAP * sizeof(unsigned long long), s));
      BS_CUDA(cudaMemsetAsync(tiles.h2.vals, 0xff, DCNA_TILE_L2_CAP * sizeof(int), s));
      BS_CUDA(cudaMemsetAsync(s1, 0xff, DCNA_TILE_L1_CAP * L1_SLOTS * sizeof(int), s));
      BS_CUDA(cudaMemsetAsync(s2, 0xff, DCNA_TILE_L2_CAP * L2_SLOTS * sizeof(int), s));
      BS_CUDA(cudaMemsetAsync(herr, 0, sizeof(int), s));
      k_tile_nodes<<<nblocks(n_tiles, 256), 256, 0, s>>>(d_tile_origins, d_tile_sizes, n_tiles, tiles.h1, tiles.h2,
                                                         herr);
      BS_CUDA(cudaGetLastError());
      const int terr = read1(s, herr);
      if (terr == 2) return BS_ERR_INVALID_ARG;
      if (terr) return BS_ERR_CAPACITY;
      k_tile_slots<<<nblocks(n_tiles, 256), 256, 0, s>>>(d_tile_origins, d_tile_sizes, d_tile_values, n_tiles,
                                                         tiles.h1, tiles.h2, s1, t1, s2, t2);
      BS_CUDA(cudaGetLastError());
      tiles.s1 = s1;
      tiles.t1 = t1;
      tiles.s2 = s2;
      tiles.t2 = t2;
      tiles.any = 1;
    }
    const bool has_tiles = n_tiles != 0;
    // start empty: hash, error flags
    BS_CUDA(cudaMemsetAsync(hkeys, 0xff, DCNA_HASH_CAP * sizeof(unsigned long long), s));
    BS_CUDA(cudaMemsetAsync(hvals, 0xff, DCNA_HASH_CAP * sizeof(int), s));
    BS_CUDA(cudaMemsetAsync(herr, 0, sizeof(int), s));
    BS_CUDA(cudaMemsetAsync(st, 0, sizeof(DcStats), s));
    k_origins_to_int4<<<nblocks(n, 256), 256, 0, s>>>(d_origins, n, org);
    BS_CUDA(cudaGetLastError());
    LeafHash hash;
    hash.keys = hkeys;
    hash.vals = hvals;
    hash.mask = DCNA_HASH_CAP - 1;
    k_hash_insert<<<nblocks(n, 256), 256, 0, s>>>(hash, org, n, herr);
    BS_CUDA(cudaGetLastError());
    DcVol V{org, d_values, d_masks, hash, tiles};
    launch_dc_edge_mask(has_tiles, V, n, cm, ccnt, s);
    BS_CUDA(cudaGetLastError());
    scan_in(s, temp, temp_bytes, ccnt, coff, n * 3 + 1);
    const uint32_t ne = read1(s, coff + n * 3);
    if (ne > DCNA_MAX_CROSSINGS) return BS_ERR_CAPACITY;
    launch_dc_edge_points(has_tiles, V, n, cm, coff, pts, st, s);
    BS_CUDA(cudaGetLastError());
    launch_dc_cell_mask(has_tiles, V, n, cellm, cellc, s);
    BS_CUDA(cudaGetLastError());
    scan_in(s, temp, temp_bytes, cellc, celloff, n + 1);
    const uint32_t nc = read1(s, celloff + n);
    if (nc > DCNA_MAX_CELLS) return BS_ERR_CAPACITY;
    k_dc_cell_points<<<unsigned(n), 128, 0, s>>>(V, n, cm, coff, pts, cellm, celloff, cells);
    BS_CUDA(cudaGetLastError());
    k_dc_quads<<<unsigned(n), 128, 0, s>>>(V, n, cm, cellm, celloff, cells, voxel_size, vcnt, nullptr, packed, nullptr);
    BS_CUDA(cudaGetLastError());
    scan_in(s, temp, temp_bytes, vcnt, voff, n + 1);
    const uint64_t nt = read1(s, voff + n);
    if (read1(s, herr)) return BS_ERR_CAPACITY;
    if (read1(s, st).error == 1) return BS_ERR_UNSUPPORTED;
    *n_tris = nt;
    if (nt > capacity) return BS_ERR_CAPACITY;  // *n_tris tells the caller the size to provide
    if (nt) {
      k_dc_quads<<<unsigned(n), 128, 0, s>>>(V, n, cm, cellm, celloff, cells, voxel_size, nullptr, voff, packed, d_tris);
      BS_CUDA(cudaGetLastError());
    }
    BS_CUDA(cudaStreamSynchronize(s));
    return BS_OK;
  } catch (const bs::Error& e) {
    return e.status;
  }
}
