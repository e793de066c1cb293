// scan_dev.cuh - block-wide exclusive scan and the single-word decoupled
// look-back used by every single-pass scan (unique, node offsets, batched).
#pragma once

#include "gtc_internal.cuh"

namespace gtc {

// Block-wide exclusive scan of one value per thread.  Returns the prefix and
// the block total.  warp_sums holds THREADS / 32 + 1 words.
template <int THREADS>
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* warp_sums, uint32_t* total) {
  constexpr int WARPS = THREADS / 32;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const uint32_t incl = warp_inclusive_sum(v);
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = (lane < WARPS) ? warp_sums[lane] : 0u;
    const uint32_t wi = warp_inclusive_sum(w);
    if (lane < WARPS) warp_sums[lane] = wi - w;
    if (lane == WARPS - 1) warp_sums[WARPS] = wi;
  }
  __syncthreads();
  *total = warp_sums[WARPS];
  return warp_sums[warp] + incl - v;
}

// Warp 0 chains this tile to its predecessors.  Publishes the aggregate,
// looks back over a 32-tile window at a time and publishes the inclusive
// prefix.  Returns the exclusive prefix of the tile (valid in lane 0..31).
__device__ __forceinline__ uint32_t tile_lookback(uint32_t* desc, uint32_t tile, uint32_t aggregate,
                                                  uint32_t* status) {
  const int lane = threadIdx.x & 31;
  if (tile == 0) {
    if (lane == 0) st_relaxed(desc, (aggregate << 2) | FLAG_INCLUSIVE);
    return 0;
  }
  if (lane == 0) st_relaxed(desc + tile, (aggregate << 2) | FLAG_AGGREGATE);
  uint32_t excl = 0;
  int k = (int)tile - 1 - lane;
  while (true) {
    const uint32_t v = (k >= 0) ? spin_descriptor(desc + k, status) : FLAG_INCLUSIVE;
    const uint32_t incl_mask = __ballot_sync(0xffffffffu, (v & 3u) == FLAG_INCLUSIVE);
    uint32_t contrib = v >> 2;
    if (incl_mask) {
      const int first = __ffs(incl_mask) - 1;  // closest inclusive predecessor
      if (lane > first) contrib = 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) contrib += __shfl_xor_sync(0xffffffffu, contrib, o);
    excl += contrib;
    if (incl_mask) break;
    k -= 32;
  }
  if (lane == 0) st_relaxed(desc + tile, ((excl + aggregate) << 2) | FLAG_INCLUSIVE);
  return excl;
}

// Resident segment scans (scan.cu, batched.cu): a grid of co-resident blocks
// of CS_THREADS, each owning CS_WARPS consecutive segments, one per warp.
constexpr int CS_THREADS = 512;
constexpr int CS_WARPS = CS_THREADS / 32;

// Exclusive prefix of this block over the descriptors of blocks [0, t), and
// the block's own segment prefixes (s_seg: per-warp totals in, exclusive
// prefixes out).  Publishes the block total first.  Returns the prefix.
__device__ __forceinline__ uint32_t cs_block_prefix(uint32_t* desc, uint32_t* s_seg, uint32_t* s_red,
                                                    uint32_t* status) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t t = blockIdx.x;
  __syncthreads();
  if (warp == 0) {
    const uint32_t v = (lane < CS_WARPS) ? s_seg[lane] : 0u;
    const uint32_t inc = warp_inclusive_sum(v);
    if (lane < CS_WARPS) s_seg[lane] = inc - v;
    if (lane == 31) st_relaxed(desc + t, (inc << 2) | FLAG_AGGREGATE);
  }
  uint32_t acc = 0;
  for (uint32_t i = tid; i < t; i += CS_THREADS) acc += spin_descriptor(desc + i, status) >> 2;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) s_red[warp] = acc;
  __syncthreads();
  uint32_t pre = 0;
#pragma unroll
  for (int w = 0; w < CS_WARPS; ++w) pre += s_red[w];
  return pre;
}

}  // namespace gtc
