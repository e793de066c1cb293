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
  cudaError_t e = cudaMemsetAsync(w, 0, (64 + (size_t)tiles) * 4, L.stream);
  if (e != cudaSuccess) return e;
  if (n == 0) return d_count ? cudaMemsetAsync(d_count, 0, 4, L.stream) : cudaSuccess;
  const size_t smem = sizeof(UniqueSmem<K>);
  static bool attr_set[2] = {false, false};  // per instantiation: set once, outside any graph capture
  if (vin) {
    auto kern = unique_kernel<K, true>;
    if (!attr_set[1]) {
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      attr_set[1] = true;
    }
    kern<<<tiles, SCAN_THREADS, smem, L.stream>>>(kin, vin, kout, vout, n, w, d_count, L.status);
  } else {
    auto kern = unique_kernel<K, false>;
    if (!attr_set[0]) {
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      attr_set[0] = true;
    }
    kern<<<tiles, SCAN_THREADS, smem, L.stream>>>(kin, nullptr, kout, nullptr, n, w, d_count, L.status);
  }
  return cudaGetLastError();
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
  cudaError_t e = cudaMemsetAsync(w, 0, (64 + (size_t)tiles) * 4, L.stream);
  if (e != cudaSuccess) return e;
  scan_kernel<<<tiles, SCAN_THREADS, 0, L.stream>>>(in, out, count_host, d_u, node_offsets, w, d_o, L.status);
  return cudaGetLastError();
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
