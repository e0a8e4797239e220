// noalloc.cu — batch-to-tile compaction that allocates nothing.
//
// Some callers cannot allocate device memory: applications that own the whole
// device heap through their own pool or arena (a database or JVM host that
// forbids foreign cudaMalloc), code that must not add allocation latency or
// synchronisation to its stream, and code paths that run where the CUDA runtime
// rejects allocations. cytom_tile_batch_noalloc serves them: it turns one edge
// batch into the tile store's sorted, deduplicated tile-CSR form using only the
// caller's input and output buffers plus the fixed scratch array below.
//
// The scratch array is a file-scope static __device__ array: every GPU that loads
// the library holds it (CYTOM_NOALLOC_SCRATCH_BYTES) until the process exits. All
// calls share it and it keeps the last call's contents, so calls that overlap on
// the GPU (other streams, other host threads) race; serialise them. Host code
// cannot use the array's name as a device address: the first call on each device,
// with that device current, looks the address up with cudaGetSymbolAddress and
// caches it. Every call ends by synchronising its stream (it reads the kept-edge
// count back), so no call can be captured in a CUDA graph.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "../../include/cytom_gpu.h"
#include "radix.cuh"

namespace cytom {

// kernels shared with the allocating path (ingest.cu)
__global__ void scan_reduce_kernel(const uint32_t* __restrict__ in, uint64_t n, uint32_t* __restrict__ sums);
__global__ void scan_down_kernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, uint64_t n,
                                 const uint32_t* __restrict__ offs, uint32_t* total_out);

namespace noalloc {

constexpr uint64_t kMax = CYTOM_NOALLOC_MAX_EDGES;
constexpr uint64_t kTile = 4096;                 // items per scan block
constexpr uint64_t kSortTile = (uint64_t)RS_T * RS_IPT_SMALL;
constexpr uint64_t kBlocks = kMax / kSortTile;   // sort tiles
// scratch layout (byte offsets, 256-aligned)
constexpr size_t kKeys0 = 0;
constexpr size_t kKeys1 = kKeys0 + kMax * 8;
constexpr size_t kW0 = kKeys1 + kMax * 8;
constexpr size_t kW1 = kW0 + kMax * 4;
constexpr size_t kKeep = kW1 + kMax * 4;
constexpr size_t kPref = kKeep + kMax * 4;
constexpr size_t kHist = kPref + kMax * 4;
constexpr size_t kOffs = kHist + 256 * kBlocks * 4;
constexpr size_t kSums = kOffs + 256 * kBlocks * 4;   // 2 x 4096 u32 block sums
constexpr size_t kFlags = kSums + 2 * 4096 * 4;        // [0] bad ids, [1] kept count
constexpr size_t kBytes = kFlags + 256;
static_assert(kBytes <= CYTOM_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the stated size");

static __device__ __align__(256) unsigned char g_scratch[CYTOM_NOALLOC_SCRATCH_BYTES];

__global__ void keys_kernel(const uint32_t* __restrict__ src, const uint32_t* __restrict__ tgt,
                            const uint32_t* __restrict__ w, uint64_t count, uint64_t n, uint32_t lvpt,
                            uint32_t lT, uint64_t* __restrict__ keys, uint32_t* __restrict__ kw,
                            unsigned int* bad) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  unsigned int nb = 0;
  const uint64_t m = (1ULL << lvpt) - 1ULL;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const uint32_t s = src[i], t = tgt[i];
    if (s >= n || t >= n) {
      ++nb;
      keys[i] = 0;
    } else {
      const uint64_t tile = (((uint64_t)s >> lvpt) << lT) | ((uint64_t)t >> lvpt);
      keys[i] = (tile << (2 * lvpt)) | (((uint64_t)s & m) << lvpt) | ((uint64_t)t & m);
    }
    kw[i] = w ? w[i] : 0u;
  }
  if (nb) atomicAdd(bad, nb);
}

// First copy of each distinct key survives with the least weight of its copies;
// fillCSR's filter (tile-manager.h:519-541) drops local (65535, 65535) when it is the
// only edge of its tile. The first thread of a run of equal keys walks the whole run:
// linear in the run's length, so the worst case (one edge repeated
// CYTOM_NOALLOC_MAX_EDGES times) is one thread making 262,144 dependent loads -- slow,
// still correct.
__global__ void keep_kernel(const uint64_t* __restrict__ K, const uint32_t* __restrict__ W, uint64_t count,
                            uint32_t lvpt, uint32_t* __restrict__ keep, uint32_t* __restrict__ wsel) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t m = (1ULL << lvpt) - 1ULL;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const uint64_t key = K[i];
    if (i > 0 && K[i - 1] == key) {
      keep[i] = 0;
      continue;
    }
    uint32_t wmin = W[i];
    for (uint64_t j = i + 1; j < count && K[j] == key; ++j) wmin = min(wmin, W[j]);
    const uint64_t tile = key >> (2 * lvpt);
    const uint32_t local = (uint32_t)((((key >> lvpt) & m) << 16) | (key & m));
    const bool corner = local == 0xFFFFFFFFu && (i == 0 || (K[i - 1] >> (2 * lvpt)) != tile);
    keep[i] = corner ? 0u : 1u;
    wsel[i] = wmin;
  }
}

__global__ void pack_kernel(const uint64_t* __restrict__ K, const uint32_t* __restrict__ keep,
                            const uint32_t* __restrict__ P, const uint32_t* __restrict__ wsel, uint64_t count,
                            uint32_t lvpt, uint32_t* __restrict__ edges, uint32_t* __restrict__ weights) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t m = (1ULL << lvpt) - 1ULL;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    if (!keep[i]) continue;
    const uint64_t key = K[i];
    edges[P[i]] = (uint32_t)((((key >> lvpt) & m) << 16) | (key & m));
    if (weights) weights[P[i]] = wsel[i];
  }
}

// tile_ptr[t] = kept edges of tiles below t: the prefix count at the first key of tile >= t.
__global__ void tile_ptr_kernel(const uint64_t* __restrict__ K, const uint32_t* __restrict__ P, uint64_t count,
                                const uint32_t* __restrict__ total, uint32_t lvpt, uint64_t ntiles,
                                unsigned long long* __restrict__ tile_ptr) {
  uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t <= ntiles; t += stride) {
    uint64_t lo = 0, hi = count;
    while (lo < hi) {
      const uint64_t mid = lo + ((hi - lo) >> 1);
      if ((K[mid] >> (2 * lvpt)) < t) lo = mid + 1;
      else hi = mid;
    }
    tile_ptr[t] = (lo < count) ? P[lo] : *total;
  }
}

static std::mutex g_mu;
static void* g_addr[64];

static cudaError_t scratch_address(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return e;
    g_addr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_addr[dev]);
  return cudaSuccess;
}

// exclusive scan of n <= kMax u32 in two levels, block sums in the scratch array
static void scan(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* sums, uint32_t* total,
                 cudaStream_t s) {
  const uint64_t nb = (n + kTile - 1) / kTile;
  if (nb <= 1) {
    scan_down_kernel<<<1, 256, 0, s>>>(in, out, n, nullptr, total);
    return;
  }
  scan_reduce_kernel<<<(unsigned)nb, 256, 0, s>>>(in, n, sums);
  scan_down_kernel<<<1, 256, 0, s>>>(sums, sums + 4096, nb, nullptr, nullptr);
  scan_down_kernel<<<(unsigned)nb, 256, 0, s>>>(in, out, n, sums + 4096, total);
}

}  // namespace noalloc
}  // namespace cytom

using namespace cytom;

extern "C" int cytom_tile_batch_noalloc(const uint32_t* src, const uint32_t* tgt, const uint32_t* w,
                                        uint64_t count, uint64_t vertices, uint64_t vertices_per_tile,
                                        unsigned long long* tile_ptr, uint32_t* edges, uint32_t* weights,
                                        uint64_t* edge_count, void* stream) {
  using namespace cytom::noalloc;
  if (count > kMax) return CYTOM_ERR_INVAL;  // beyond CYTOM_NOALLOC_MAX_EDGES
  if (!edge_count || !tile_ptr || (count && (!src || !tgt || !edges)) || (w && !weights)) return CYTOM_ERR_INVAL;
  uint64_t n = 1;
  while (n < vertices) n <<= 1;
  const uint64_t vpt = vertices_per_tile;
  if (vertices == 0 || vpt == 0 || (vpt & (vpt - 1)) || vpt > 65536 || vpt > n || n > (1ULL << 32))
    return CYTOM_ERR_INVAL;
  uint32_t lvpt = 0, lT = 0;
  while ((1ULL << lvpt) < vpt) ++lvpt;
  while ((1ULL << lT) < n / vpt) ++lT;
  const uint64_t ntiles = (n / vpt) * (n / vpt);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char* base = nullptr;
  if (scratch_address(&base) != cudaSuccess) return CYTOM_ERR_CUDA;
  uint64_t* k0 = reinterpret_cast<uint64_t*>(base + kKeys0);
  uint64_t* k1 = reinterpret_cast<uint64_t*>(base + kKeys1);
  uint32_t* w0 = reinterpret_cast<uint32_t*>(base + kW0);
  uint32_t* w1 = reinterpret_cast<uint32_t*>(base + kW1);
  uint32_t* keep = reinterpret_cast<uint32_t*>(base + kKeep);
  uint32_t* pref = reinterpret_cast<uint32_t*>(base + kPref);
  uint32_t* hist = reinterpret_cast<uint32_t*>(base + kHist);
  uint32_t* offs = reinterpret_cast<uint32_t*>(base + kOffs);
  uint32_t* sums = reinterpret_cast<uint32_t*>(base + kSums);
  uint32_t* flags = reinterpret_cast<uint32_t*>(base + kFlags);
  // the counters accumulate: clear them (the rest is fully written before it is read)
  cudaError_t e = cudaMemsetAsync(flags, 0, 256, s);
  if (e != cudaSuccess) return CYTOM_ERR_CUDA;
  const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((count + 255) / 256, 1024));
  if (count) {
    noalloc::keys_kernel<<<grid, 256, 0, s>>>(src, tgt, w, count, n, lvpt, lT, k0, w0, &flags[0]);
    // LSD radix sort of the composite keys (stable), weights ride along
    const int bits = (int)(2 * (lvpt + lT));
    const uint64_t nb = (count + kSortTile - 1) / kSortTile;
    uint64_t *kin = k0, *kout = k1;
    uint32_t *vin = w0, *vout = w1;
    for (int shift = 0; shift < bits; shift += 8) {
      radix_upsweep_kernel<RS_IPT_SMALL><<<(unsigned)nb, RS_T, 0, s>>>(kin, count, shift, hist, (uint32_t)nb);
      noalloc::scan(hist, offs, nb * 256, sums, nullptr, s);
      radix_downsweep_kernel<RS_IPT_SMALL><<<(unsigned)nb, RS_T, 0, s>>>(kin, vin, count, shift, offs, (uint32_t)nb, kout, vout);
      std::swap(kin, kout);
      std::swap(vin, vout);
    }
    noalloc::keep_kernel<<<grid, 256, 0, s>>>(kin, vin, count, lvpt, keep, vout);
    noalloc::scan(keep, pref, count, sums, &flags[1], s);
    noalloc::pack_kernel<<<grid, 256, 0, s>>>(kin, keep, pref, vout, count, lvpt, edges, w ? weights : nullptr);
    const unsigned tgrid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((ntiles + 256) / 256, 4096));
    noalloc::tile_ptr_kernel<<<tgrid, 256, 0, s>>>(kin, pref, count, &flags[1], lvpt, ntiles, tile_ptr);
  } else {
    e = cudaMemsetAsync(tile_ptr, 0, (ntiles + 1) * 8, s);
    if (e != cudaSuccess) return CYTOM_ERR_CUDA;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return CYTOM_ERR_CUDA;
  uint32_t h[2] = {0, 0};
  e = cudaMemcpyAsync(h, flags, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return CYTOM_ERR_CUDA;
  if (h[0]) return CYTOM_ERR_RANGE;
  *edge_count = h[1];
  return CYTOM_OK;
}
