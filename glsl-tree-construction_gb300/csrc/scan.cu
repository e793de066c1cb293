// scan.cu - single-pass decoupled look-back scans: unique compaction and the
// octree node-offset scan.
//
// unique.comp:31-49 and partial_sum.comp:23-39 run on ONE GPU thread
// (unique.rs:245, partial_sum.rs:246).  Here both are one pass over the data:
// each tile of THREADS * IPT items (blocked per thread) is staged through
// shared memory with coalesced loads, reduced, chained to its predecessors by
// a warp-wide look-back over per-tile descriptors, and written back with
// coalesced stores.

#include "scan_dev.cuh"

namespace gtc {

constexpr int SCAN_THREADS = 512;
constexpr int SCAN_IPT = 9;  // odd: conflict-free blocked reads of 32-bit words
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_IPT;

// Workspace: [0] tile counter, [1..63] spare, [64..64+tiles) descriptors.
size_t scan_workspace_bytes(uint32_t n) {
  const uint32_t tiles = ceil_div(n > 0 ? n : 1, SCAN_TILE) + 1;
  return align_up((64 + (size_t)tiles) * 4, 256);
}

// --------------------------------------------------------- segment scans --
// Resident form of the two scans, used when the input is large enough to fill
// the GPU: a grid of co-resident blocks (at most what the SMs hold at once),
// each owning CS_WARPS consecutive segments of S items, one per warp.
//   1. every warp reduces its segment (coalesced row loads, many in flight);
//      the block posts its total as a descriptor;
//   2. the block adds up the totals of all lower blocks (one load per thread,
//      a single round trip: every block posts before it waits, and it waits
//      only on lower blocks, all resident);
//   3. every warp re-reads its segment (mostly from L2) and writes it with
//      warp-only scans: no block barrier, no staging in shared memory.
// The single-pass kernels above pay a chained look-back per 4.6K-item tile;
// here each block waits once.
// Inclusive scan with the node-offset rules of scan_kernel.  Rows of 128
// items (one uint4 per lane); S is a multiple of 128, so rows never straddle
// segments and in/out must be 16-byte aligned.
__global__ void __launch_bounds__(CS_THREADS) chunk_scan_kernel(const uint32_t* __restrict__ in,
                                                                uint32_t* __restrict__ out, uint32_t count_host,
                                                                const uint32_t* d_u, int node_offsets, uint32_t* ws,
                                                                uint32_t* d_o, uint32_t* status) {
  griddep_wait();
  __shared__ uint32_t s_seg[CS_WARPS];
  __shared__ uint32_t s_red[CS_WARPS];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t count = d_u ? *d_u : count_host;
  const uint32_t limit = node_offsets ? (count > 0 ? count - 1 : 0) : count;
  if (count == 0) {
    if (node_offsets && blockIdx.x == 0 && tid == 0 && d_o) *d_o = 0;
    return;
  }
  const uint32_t nseg = gridDim.x * CS_WARPS;
  const uint64_t S = (((uint64_t)count + nseg - 1) / nseg + 127) & ~(uint64_t)127;
  const uint64_t beg64 = (uint64_t)(blockIdx.x * CS_WARPS + warp) * S;
  const uint32_t beg = (uint32_t)min(beg64, (uint64_t)count);
  const uint32_t end = (uint32_t)min(beg64 + S, (uint64_t)count);
  const uint32_t full_end = beg + ((min(end, limit) > beg ? min(end, limit) - beg : 0u) & ~127u);
  const uint4* in4 = reinterpret_cast<const uint4*>(in);

  // 1. segment totals (rows tagged to stay in L2 for step 3)
  const uint64_t keep_pol = l2_keep_policy(), drop_pol = l2_drop_policy();
  uint32_t sum = 0;
  uint32_t r = beg;
  for (; r + 4 * 128 <= full_end; r += 4 * 128) {
    uint4 v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = ld_hint(in4 + (r + j * 128) / 4 + lane, keep_pol);
#pragma unroll
    for (int j = 0; j < 4; ++j) sum += v[j].x + v[j].y + v[j].z + v[j].w;
  }
  for (; r < full_end; r += 128) {
    const uint4 v = ld_hint(in4 + r / 4 + lane, keep_pol);
    sum += v.x + v.y + v.z + v.w;
  }
  for (uint32_t i = r + lane; i < end; i += 32) sum += (i < limit) ? in[i] : 0u;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) s_seg[warp] = sum;

  // 2. block prefix
  uint32_t run = cs_block_prefix(ws + 64, s_seg, s_red, status);
  run += s_seg[warp];

  // 3. rescan and write
  for (r = beg; r < end; r += 128) {
    const uint32_t i0 = r + 4 * lane;
    uint4 v;
    if (r + 128 <= full_end) {
      v = ld_hint(in4 + r / 4 + lane, drop_pol);
    } else {
      v.x = (i0 + 0 < end && i0 + 0 < limit) ? in[i0 + 0] : 0u;
      v.y = (i0 + 1 < end && i0 + 1 < limit) ? in[i0 + 1] : 0u;
      v.z = (i0 + 2 < end && i0 + 2 < limit) ? in[i0 + 2] : 0u;
      v.w = (i0 + 3 < end && i0 + 3 < limit) ? in[i0 + 3] : 0u;
    }
    v.y += v.x;
    v.z += v.y;
    v.w += v.z;
    const uint32_t inc = warp_inclusive_sum(v.w);
    const uint32_t base = run + inc - v.w;
    v.x += base;
    v.y += base;
    v.z += base;
    v.w += base;
    run += __shfl_sync(0xffffffffu, inc, 31);
    if (node_offsets && i0 == 0) v.x = 0;
    if (i0 + 4 <= end) {
      reinterpret_cast<uint4*>(out)[i0 / 4] = v;
    } else {
      if (i0 + 0 < end) out[i0 + 0] = v.x;
      if (i0 + 1 < end) out[i0 + 1] = v.y;
      if (i0 + 2 < end) out[i0 + 2] = v.z;
    }
    if (node_offsets && d_o && i0 <= count - 1 && count - 1 < i0 + 4) {
      const uint32_t j = count - 1 - i0;
      const uint32_t last = (count == 1) ? 0u : (j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w);
      *d_o = 1 + last;
    }
  }
}

// Unique, out of place (kin != kout: a segment is read twice, so no output
// may land on input not yet re-read).  Rows of 32 keys; keep = first key or
// different from its predecessor; kept keys of a row are written contiguously.
template <class K, bool HAS_VALS>
__global__ void __launch_bounds__(CS_THREADS) chunk_unique_kernel(const K* __restrict__ kin,
                                                                  const uint32_t* __restrict__ vin,
                                                                  K* __restrict__ kout, uint32_t* __restrict__ vout,
                                                                  uint32_t n, uint32_t* ws, uint32_t* d_count,
                                                                  uint32_t* status) {
  griddep_wait();
  __shared__ uint32_t s_seg[CS_WARPS];
  __shared__ uint32_t s_red[CS_WARPS];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t nseg = gridDim.x * CS_WARPS;
  const uint64_t S = (((uint64_t)n + nseg - 1) / nseg + 31) & ~(uint64_t)31;
  const uint64_t beg64 = (uint64_t)(blockIdx.x * CS_WARPS + warp) * S;
  const uint32_t beg = (uint32_t)min(beg64, (uint64_t)n);
  const uint32_t end = (uint32_t)min(beg64 + S, (uint64_t)n);
  const uint32_t full_end = beg + ((end - beg) & ~255u);
  const K first_prev = (beg > 0 && beg < end) ? kin[beg - 1] : K(0);

  // 1. kept keys per segment (keys tagged to stay in L2 for step 3)
  const uint64_t keep_pol = l2_keep_policy(), drop_pol = l2_drop_policy();
  uint32_t cnt = 0;
  {
    K carry = first_prev;
    uint32_t r = beg;
    for (; r < full_end; r += 256) {  // eight rows in flight per warp
      K k[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) k[j] = ld_hint(kin + r + 32 * j + lane, keep_pol);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        K prev = __shfl_up_sync(0xffffffffu, k[j], 1);
        if (lane == 0) prev = carry;
        const bool keep = (r + 32 * j + lane == 0) || k[j] != prev;
        cnt += __popc(__ballot_sync(0xffffffffu, keep));
        carry = __shfl_sync(0xffffffffu, k[j], 31);
      }
    }
    for (; r < end; r += 32) {
      const uint32_t i = r + lane;
      const K key = (i < end) ? kin[i] : K(0);
      K prev = __shfl_up_sync(0xffffffffu, key, 1);
      if (lane == 0) prev = carry;
      const bool keep = i < end && (i == 0 || key != prev);
      cnt += __popc(__ballot_sync(0xffffffffu, keep));
      carry = __shfl_sync(0xffffffffu, key, 31);
    }
  }
  if (lane == 0) s_seg[warp] = cnt;

  // 2. block prefix
  const uint32_t pre = cs_block_prefix(ws + 64, s_seg, s_red, status);
  uint32_t run = pre + s_seg[warp];

  // 3. rescan and write
  {
    K carry = first_prev;
    uint32_t r = beg;
    for (; r < full_end; r += 256) {
      K k[8];
      uint32_t v[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        k[j] = ld_hint(kin + r + 32 * j + lane, drop_pol);
        if (HAS_VALS) v[j] = ld_hint(vin + r + 32 * j + lane, drop_pol);
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        K prev = __shfl_up_sync(0xffffffffu, k[j], 1);
        if (lane == 0) prev = carry;
        const bool keep = (r + 32 * j + lane == 0) || k[j] != prev;
        const uint32_t bal = __ballot_sync(0xffffffffu, keep);
        if (keep) {
          const uint32_t o = run + __popc(bal & lt);
          kout[o] = k[j];
          if (HAS_VALS) vout[o] = v[j];
        }
        run += __popc(bal);
        carry = __shfl_sync(0xffffffffu, k[j], 31);
      }
    }
    for (; r < end; r += 32) {
      const uint32_t i = r + lane;
      const K key = (i < end) ? kin[i] : K(0);
      const uint32_t val = (HAS_VALS && i < end) ? vin[i] : 0u;
      K prev = __shfl_up_sync(0xffffffffu, key, 1);
      if (lane == 0) prev = carry;
      const bool keep = i < end && (i == 0 || key != prev);
      const uint32_t bal = __ballot_sync(0xffffffffu, keep);
      if (keep) {
        const uint32_t o = run + __popc(bal & lt);
        kout[o] = key;
        if (HAS_VALS) vout[o] = val;
      }
      run += __popc(bal);
      carry = __shfl_sync(0xffffffffu, key, 31);
    }
  }
  // The last warp of the last block ends at n: its running count is u.
  if (d_count && blockIdx.x == gridDim.x - 1 && warp == CS_WARPS - 1 && lane == 0) *d_count = run;
}

// Blocks of a resident grid for the segment scans (0: use the single-pass
// kernels).  Capped by the descriptor words of the workspace.
static uint32_t chunk_grid(const Launch& L, const void* kern, uint32_t n_max) {
  int occ = 0;
  if (kernel_setup(kern, CS_THREADS, 0, &occ) != cudaSuccess) {
    cudaGetLastError();
    return 0u;
  }
  const uint32_t resident = (uint32_t)occ * (uint32_t)L.num_sms;
  const uint32_t tiles = ceil_div(n_max > 0 ? n_max : 1, SCAN_TILE);  // descriptor words cleared by the launcher
  const uint32_t g = min(resident, tiles);
  // Worth it once every warp has a few rows to stream.
  return (g >= 64 && (uint64_t)n_max >= (uint64_t)g * CS_WARPS * 256) ? g : 0u;
}

// ---------------------------------------------------------------- unique --
template <class K>
struct UniqueSmem {
  K keys[SCAN_TILE];
  uint32_t vals[SCAN_TILE];
  uint32_t warp_sums[SCAN_THREADS / 32 + 1];
  uint32_t tile_id;
  uint32_t prefix;
  K halo;
};

template <class K, bool HAS_VALS>
__global__ void __launch_bounds__(SCAN_THREADS) unique_kernel(const K* kin, const uint32_t* vin, K* kout,
                                                              uint32_t* vout, uint32_t n, uint32_t* ws,
                                                              uint32_t* d_count, uint32_t* status) {
  griddep_wait();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  UniqueSmem<K>& s = *reinterpret_cast<UniqueSmem<K>*>(smem_raw);
  uint32_t* desc = ws + 64;
  const int tid = threadIdx.x;
  if (tid == 0) s.tile_id = atomicAdd(ws, 1u);
  __syncthreads();
  const uint32_t tile = s.tile_id;
  const uint32_t base = tile * SCAN_TILE;
  if (base >= n) return;  // no tile is ever launched past n by the launcher
  const uint32_t valid = min((uint32_t)SCAN_TILE, n - base);
  // Every read of this tile's input (and the halo) happens before the tile
  // publishes its aggregate, and every write happens after its look-back
  // completes, so in-place compaction (kin == kout) is safe.  A full tile
  // issues all of a thread's loads before storing any (the look-back chain
  // makes each tile's latency the cost, not the bandwidth).
  if (valid == SCAN_TILE) {
    K kr[SCAN_IPT];
    uint32_t vr[SCAN_IPT];
#pragma unroll
    for (int j = 0; j < SCAN_IPT; ++j) {
      kr[j] = kin[base + j * SCAN_THREADS + tid];
      if (HAS_VALS) vr[j] = vin[base + j * SCAN_THREADS + tid];
    }
#pragma unroll
    for (int j = 0; j < SCAN_IPT; ++j) {
      s.keys[j * SCAN_THREADS + tid] = kr[j];
      if (HAS_VALS) s.vals[j * SCAN_THREADS + tid] = vr[j];
    }
  } else {
    for (uint32_t i = tid; i < valid; i += SCAN_THREADS) {
      s.keys[i] = kin[base + i];
      if (HAS_VALS) s.vals[i] = vin[base + i];
    }
  }
  if (tid == 0) s.halo = (base > 0) ? kin[base - 1] : K(0);
  __syncthreads();
  K key[SCAN_IPT];
  uint32_t val[SCAN_IPT];
  uint32_t flags = 0, cnt = 0;
  const uint32_t first = tid * SCAN_IPT;
#pragma unroll
  for (int j = 0; j < SCAN_IPT; ++j) {
    const uint32_t i = first + j;
    if (i < valid) {
      key[j] = s.keys[i];
      if (HAS_VALS) val[j] = s.vals[i];
      const K prev = (i == 0) ? s.halo : s.keys[i - 1];
      const bool keep = (base + i == 0) || (key[j] != prev);
      flags |= (uint32_t)keep << j;
      cnt += keep;
    }
  }
  uint32_t total;
  const uint32_t excl = block_exclusive<SCAN_THREADS>(cnt, s.warp_sums, &total);
  if (tid < 32) {
    const uint32_t pre = tile_lookback(desc, tile, total, status);
    if (tid == 0) s.prefix = pre;
  }
  __syncthreads();  // also: everyone is done reading s.keys / s.vals
  uint32_t r = excl;
#pragma unroll
  for (int j = 0; j < SCAN_IPT; ++j) {
    if (flags & (1u << j)) {
      s.keys[r] = key[j];
      if (HAS_VALS) s.vals[r] = val[j];
      ++r;
    }
  }
  __syncthreads();
  const uint32_t out = s.prefix;
  for (uint32_t i = tid; i < total; i += SCAN_THREADS) {
    kout[out + i] = s.keys[i];
    if (HAS_VALS) vout[out + i] = s.vals[i];
  }
  if (tid == 0 && base + valid == n && d_count) *d_count = out + total;
}

template <class K>
cudaError_t launch_unique(const Launch& L, const K* kin, const uint32_t* vin, K* kout, uint32_t* vout, uint32_t n,
                          uint32_t* d_count, void* ws) {
  uint32_t* w = reinterpret_cast<uint32_t*>(ws);
  const uint32_t tiles = ceil_div(n, SCAN_TILE);
  cudaError_t e = L.ws_zeroed ? cudaSuccess : cudaMemsetAsync(w, 0, (64 + (size_t)tiles) * 4, L.stream);
  if (e != cudaSuccess) return e;
  if (n == 0) return d_count ? cudaMemsetAsync(d_count, 0, 4, L.stream) : cudaSuccess;
  if (kin != kout && vin != vout) {
    const void* kern = vin ? (const void*)chunk_unique_kernel<K, true> : (const void*)chunk_unique_kernel<K, false>;
    const uint32_t g = chunk_grid(L, kern, n);
    if (g) {
      if (vin)
        return launch_kernel(L, chunk_unique_kernel<K, true>, g, CS_THREADS, 0, kin, vin, kout, vout, n, w, d_count,
                             L.status);
      return launch_kernel(L, chunk_unique_kernel<K, false>, g, CS_THREADS, 0, kin, nullptr, kout, nullptr, n, w,
                           d_count, L.status);
    }
  }
  const size_t smem = sizeof(UniqueSmem<K>);
  if (vin) {
    auto kern = unique_kernel<K, true>;
    e = kernel_setup(kern, SCAN_THREADS, smem);
    if (e != cudaSuccess) return e;
    return launch_kernel(L, kern, tiles, SCAN_THREADS, smem, kin, vin, kout, vout, n, w, d_count, L.status);
  } else {
    auto kern = unique_kernel<K, false>;
    e = kernel_setup(kern, SCAN_THREADS, smem);
    if (e != cudaSuccess) return e;
    return launch_kernel(L, kern, tiles, SCAN_THREADS, smem, kin, nullptr, kout, nullptr, n, w, d_count, L.status);
  }
}
template cudaError_t launch_unique<uint32_t>(const Launch&, const uint32_t*, const uint32_t*, uint32_t*, uint32_t*,
                                             uint32_t, uint32_t*, void*);
template cudaError_t launch_unique<uint64_t>(const Launch&, const uint64_t*, const uint32_t*, uint64_t*, uint32_t*,
                                             uint32_t, uint32_t*, void*);

// ------------------------------------------------------------------ scan --
// Inclusive scan of `count` elements; element k reads in[k] when k < limit,
// else 0.  With node_offsets set: count = u = *d_u (or host), limit = u - 1,
// out[0] forced to 0 and *d_o = 1 + out[u - 1] (main.rs:127-129; D4).
struct ScanSmem {
  uint32_t vals[SCAN_TILE];
  uint32_t warp_sums[SCAN_THREADS / 32 + 1];
  uint32_t tile_id;
  uint32_t prefix;
};

__global__ void __launch_bounds__(SCAN_THREADS) scan_kernel(const uint32_t* in, uint32_t* out, uint32_t count_host,
                                                            const uint32_t* d_u, int node_offsets, uint32_t* ws,
                                                            uint32_t* d_o, uint32_t* status) {
  griddep_wait();
  __shared__ ScanSmem s;
  uint32_t* desc = ws + 64;
  const int tid = threadIdx.x;
  const uint32_t count = d_u ? *d_u : count_host;
  const uint32_t limit = node_offsets ? (count > 0 ? count - 1 : 0) : count;
  if (tid == 0) s.tile_id = atomicAdd(ws, 1u);
  __syncthreads();
  const uint32_t tile = s.tile_id;
  const uint32_t base = tile * SCAN_TILE;
  if (base >= count) {
    if (node_offsets && count == 0 && tile == 0 && tid == 0 && d_o) *d_o = 0;
    return;
  }
  const uint32_t valid = min((uint32_t)SCAN_TILE, count - base);
  if (valid == SCAN_TILE && base + SCAN_TILE <= limit) {  // all loads of a thread in flight at once
    uint32_t r[SCAN_IPT];
#pragma unroll
    for (int j = 0; j < SCAN_IPT; ++j) r[j] = in[base + j * SCAN_THREADS + tid];
#pragma unroll
    for (int j = 0; j < SCAN_IPT; ++j) s.vals[j * SCAN_THREADS + tid] = r[j];
  } else {
    for (uint32_t i = tid; i < valid; i += SCAN_THREADS) {
      const uint32_t g = base + i;
      s.vals[i] = (g < limit) ? in[g] : 0u;
    }
  }
  __syncthreads();
  uint32_t v[SCAN_IPT];
  uint32_t sum = 0;
  const uint32_t first = tid * SCAN_IPT;
#pragma unroll
  for (int j = 0; j < SCAN_IPT; ++j) {
    v[j] = (first + j < valid) ? s.vals[first + j] : 0u;
    sum += v[j];
  }
  uint32_t total;
  const uint32_t excl = block_exclusive<SCAN_THREADS>(sum, s.warp_sums, &total);
  if (tid < 32) {
    const uint32_t pre = tile_lookback(desc, tile, total, status);
    if (tid == 0) s.prefix = pre;
  }
  __syncthreads();
  uint32_t run = s.prefix + excl;
#pragma unroll
  for (int j = 0; j < SCAN_IPT; ++j) {
    run += v[j];
    if (first + j < valid) s.vals[first + j] = run;
  }
  __syncthreads();
  for (uint32_t i = tid; i < valid; i += SCAN_THREADS) {
    const uint32_t g = base + i;
    out[g] = (node_offsets && g == 0) ? 0u : s.vals[i];
  }
  if (node_offsets && tid == 0 && base + valid == count && d_o) {
    const uint32_t last = (count == 1) ? 0u : s.prefix + total;
    *d_o = 1 + last;
  }
}

static cudaError_t launch_scan(const Launch& L, const uint32_t* in, uint32_t* out, uint32_t count_host,
                               const uint32_t* d_u, uint32_t n_max, int node_offsets, uint32_t* d_o, void* ws) {
  uint32_t* w = reinterpret_cast<uint32_t*>(ws);
  const uint32_t tiles = ceil_div(n_max > 0 ? n_max : 1, SCAN_TILE);
  cudaError_t e = L.ws_zeroed ? cudaSuccess : cudaMemsetAsync(w, 0, (64 + (size_t)tiles) * 4, L.stream);
  if (e != cudaSuccess) return e;
  const bool aligned = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u) == 0;
  const uint32_t g = aligned ? chunk_grid(L, (const void*)chunk_scan_kernel, n_max) : 0u;
  if (g)
    return launch_kernel(L, chunk_scan_kernel, g, CS_THREADS, 0, in, out, count_host, d_u, node_offsets, w, d_o,
                         L.status);
  return launch_kernel(L, scan_kernel, tiles, SCAN_THREADS, 0, in, out, count_host, d_u, node_offsets, w, d_o,
                       L.status);
}

cudaError_t launch_inclusive_scan(const Launch& L, const uint32_t* in, uint32_t* out, uint32_t n, void* ws) {
  if (n == 0) return cudaSuccess;
  return launch_scan(L, in, out, n, nullptr, n, 0, nullptr, ws);
}

cudaError_t launch_inclusive_scan_dev(const Launch& L, const uint32_t* in, uint32_t* out, const uint32_t* d_count,
                                      uint32_t n_max, void* ws) {
  if (n_max == 0) return cudaSuccess;
  return launch_scan(L, in, out, 0, d_count, n_max, 0, nullptr, ws);
}

cudaError_t launch_node_offsets(const Launch& L, const uint32_t* edge, uint32_t* ps, const uint32_t* d_u,
                                uint32_t m_host, uint32_t n_max, uint32_t* d_o, void* ws) {
  // u = m + 1 entries; with d_u the count comes from the device (<= n_max).
  return launch_scan(L, edge, ps, m_host + 1, d_u, d_u ? n_max : m_host + 1, 1, d_o, ws);
}

}  // namespace gtc
