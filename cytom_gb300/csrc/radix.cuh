// radix.cuh — the stable LSD radix sort's tile shape and kernels, shared by the
// allocating compaction (ingest.cu) and the allocation-free batch path (noalloc.cu).
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace cytom {

// 256 threads per tile; IPT keys per thread. Small tiles (IPT 4) give every SM many
// independent warps, which the latency-bound ranking and scatter need; large sorts use
// IPT 16 to keep the digit histogram (256 x tiles) small next to the keys.
constexpr int RS_T = 256, RS_WARPS = RS_T / 32;
constexpr int RS_IPT_SMALL = 4, RS_IPT_LARGE = 16;

// Per-tile digit counts of one 8-bit pass, digit-major: hist[digit * nb + tile].
// Stable scatter of one pass given the exclusive scan of the histogram.
template <int IPT>
__global__ void radix_upsweep_kernel(const uint64_t* __restrict__ keys, uint64_t n, int shift,
                                     uint32_t* __restrict__ hist, uint32_t nb) {
  __shared__ uint32_t cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  uint64_t base = (uint64_t)blockIdx.x * (RS_T * IPT);
  uint32_t d_reg[IPT];
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    uint64_t i = base + (uint64_t)k * RS_T + threadIdx.x;
    d_reg[k] = (i < n) ? (uint32_t)((keys[i] >> shift) & 0xFF) : 256u;
  }
  // warp-aggregated counts (skewed digits would serialise per-key shared atomics)
  const unsigned lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, d_reg[k]);
    if (d_reg[k] < 256u && (__ffs(peers) - 1) == (int)lane) atomicAdd(&cnt[d_reg[k]], (uint32_t)__popc(peers));
  }
  __syncthreads();
  hist[(uint64_t)threadIdx.x * nb + blockIdx.x] = cnt[threadIdx.x];
}

template <int IPT>
__global__ void radix_downsweep_kernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                                       uint64_t n, int shift, const uint32_t* __restrict__ offs, uint32_t nb,
                                       uint64_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out) {
  __shared__ uint32_t wcnt[RS_WARPS][256];
  __shared__ uint32_t base_d[256];
  const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  for (int d = threadIdx.x; d < RS_WARPS * 256; d += RS_T) (&wcnt[0][0])[d] = 0;
  base_d[threadIdx.x] = offs[(uint64_t)threadIdx.x * nb + blockIdx.x];
  __syncthreads();
  const uint64_t wbase = (uint64_t)blockIdx.x * (RS_T * IPT) + (uint64_t)wid * (32 * IPT);
  // every key and value is loaded before any is used
  uint64_t k_reg[IPT];
  uint32_t v_reg[IPT];
  uint32_t d_reg[IPT];
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    uint64_t i = wbase + (uint64_t)k * 32 + lane;
    k_reg[k] = (i < n) ? keys[i] : 0ULL;
    v_reg[k] = (vals && i < n) ? vals[i] : 0u;
    d_reg[k] = (i < n) ? (uint32_t)((k_reg[k] >> shift) & 0xFF) : 256u;
  }
  // phase 1: each key's rank among the warp's keys of its digit, in input order
  uint32_t r_reg[IPT];
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    const uint32_t d = d_reg[k];
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
    const int leader = __ffs(peers) - 1;
    uint32_t old = 0;
    if ((int)lane == leader && d < 256u) {
      old = wcnt[wid][d];
      wcnt[wid][d] = old + __popc(peers);
    }
    r_reg[k] = __shfl_sync(0xFFFFFFFFu, old, leader) + __popc(peers & lt);
    __syncwarp();
  }
  __syncthreads();
  // phase 2: exclusive prefix across warps per digit
  {
    uint32_t run = 0;
    const int d = threadIdx.x;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) {
      uint32_t t = wcnt[w][d];
      wcnt[w][d] = run;
      run += t;
    }
  }
  __syncthreads();
  // phase 3: scatter (stable: block offset + warp offset + rank)
#pragma unroll
  for (int k = 0; k < IPT; ++k) {
    const uint32_t d = d_reg[k];
    if (d < 256u) {
      const uint32_t pos = base_d[d] + wcnt[wid][d] + r_reg[k];
      keys_out[pos] = k_reg[k];
      if (vals) vals_out[pos] = v_reg[k];
    }
  }
}

}  // namespace cytom
