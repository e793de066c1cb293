// batched.cu - many point clouds of uneven size in one stream-ordered build.
//
// No counterpart in the reference (its pipeline builds one cloud,
// main.rs:60-170).  Every cloud's outputs are defined to equal the
// single-cloud 32-bit build of that cloud alone, with cloud-local indices,
// so each cloud is checked against the oracle on its own.
//
// One launch per stage for the whole batch, every size read on the device, so
// the batch captures into one CUDA graph:
//   1. tiles:   each cloud is cut into its own tiles; tile_start[c] is the
//               first tile of cloud c (a device work list pulled by ticket);
//   2. morton:  32-bit codes, cloud-local point index payload, per-cloud
//               digit histograms of the 4 passes;
//   3. segmented onesweep, 4 passes: a tile's digit bases come from its own
//               cloud's histogram and its decoupled look-back runs only over
//               earlier tiles of the same cloud (a cloud's first tile
//               publishes an inclusive prefix at once);
//   4. unique:  compaction that restarts at every cloud start; cloud c's
//               unique codes land at [U_c, U_{c+1});
//   5. radix tree of each cloud (the window kernel of tree_window.cuh, with
//               pairs that straddle two clouds as boundaries; karras_node
//               under the per-node method) with the edge counts, and a zero
//               edge in each cloud's last slot;
//   6. one inclusive scan of all edge counts; cloud c's node offsets are the
//               scan minus its value just before U_c (the bias);
//   7. octree of each cloud (octree_warp_batch) into its node range starting
//               at O_c = (non-empty clouds before c) + bias.

#include <atomic>
#include <utility>

#include "karras.cuh"
#include "octree_dev.cuh"
#include "scan_dev.cuh"
#include "tree_window.cuh"

namespace gtc {

Launch context_launch(gtc_ctx* ctx, gtc_stream_t stream);
gtc_status context_error(gtc_ctx* ctx, gtc_status s, const char* msg, cudaError_t e);
cudaEvent_t context_stage_begin(gtc_ctx* ctx, gtc_stream_t stream);
void context_stage_end(gtc_ctx* ctx, gtc_stream_t stream, cudaEvent_t a, int stage);

namespace {

// Brackets one stage's launches with events while profiling is on.
struct Stage {
  gtc_ctx* ctx;
  gtc_stream_t s;
  int stage;
  cudaEvent_t a;
  Stage(gtc_ctx* c, gtc_stream_t st, int sg) : ctx(c), s(st), stage(sg), a(context_stage_begin(c, st)) {}
  ~Stage() { context_stage_end(ctx, s, a, stage); }
};

constexpr int BRADIX = 256;
constexpr int BPASSES = 4;  // 30-bit codes in 8-bit digits
constexpr int BM_THREADS = 512;  // Morton kernel: one block per tile
// Segmented onesweep tile shapes (threads x keys per thread), compiled as
// variants: pinned with gtc_batched_set_variant, else the autotuner's pick
// for the batch's size (gtc_autotune_batched), else variant 0.  Every tile
// division of the batch (tile list, Morton blocks, sort tiles) uses the
// chosen shape's tile.
struct BtVariant {
  int threads, kpt;
};
constexpr BtVariant kBtVariants[] = {{512, 12}, {256, 16}, {384, 16}, {512, 8}, {256, 24}};
constexpr int kBtNumVariants = sizeof(kBtVariants) / sizeof(kBtVariants[0]);
constexpr uint32_t BT_MIN_TILE = 4096;  // smallest tile of any variant: sizes the workspace
constexpr int BU_THREADS = 512;
constexpr int BU_IPT = 9;
constexpr int BU_TILE = BU_THREADS * BU_IPT;  // the scan tile of scan.cu
constexpr uint32_t MAX_CLOUDS = 1u << 20;

// Tiles per cloud and non-empty clouds, both scanned (one block).  The
// offsets must partition [0, n): off[0] = 0, non-decreasing, off[S] = n.
// Otherwise the batch is flagged bad, every later kernel returns at once and
// the outputs say zero unique codes and zero nodes.
__global__ void __launch_bounds__(1024) bt_tiles_kernel(const uint32_t* off, uint32_t S, uint32_t n, uint32_t tile,
                                                        uint32_t* tile_start, uint32_t* ne_start, uint32_t* bad,
                                                        uint32_t* uoff, uint32_t* status) {
  __shared__ uint32_t s_t[1024], s_n[1024];
  const uint32_t per = (S + 1023) / 1024;
  const uint32_t first = threadIdx.x * per, last = min(first + per, S);
  bool ok = threadIdx.x != 0 || (off[0] == 0 && off[S] == n);
  for (uint32_t c = first; c < last; ++c) ok = ok && off[c + 1] >= off[c];
  if (__syncthreads_or(!ok)) {
    if (threadIdx.x == 0) {
      *bad = 1;
      tile_start[S] = 0;
      uoff[S] = 0;
      atomicOr(status, DEV_BAD_INPUT);
    }
    return;
  }
  uint32_t t = 0, ne = 0;
  for (uint32_t c = first; c < last; ++c) {
    const uint32_t len = off[c + 1] - off[c];
    t += (len + tile - 1) / tile;
    ne += len > 0;
  }
  s_t[threadIdx.x] = t;
  s_n[threadIdx.x] = ne;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const uint32_t a = threadIdx.x >= (unsigned)o ? s_t[threadIdx.x - o] : 0u;
    const uint32_t b = threadIdx.x >= (unsigned)o ? s_n[threadIdx.x - o] : 0u;
    __syncthreads();
    s_t[threadIdx.x] += a;
    s_n[threadIdx.x] += b;
    __syncthreads();
  }
  t = threadIdx.x ? s_t[threadIdx.x - 1] : 0u;
  ne = threadIdx.x ? s_n[threadIdx.x - 1] : 0u;
  for (uint32_t c = first; c < last; ++c) {
    const uint32_t len = off[c + 1] - off[c];
    tile_start[c] = t;
    ne_start[c] = ne;
    t += (len + tile - 1) / tile;
    ne += len > 0;
  }
  if (threadIdx.x == 1023) {
    tile_start[S] = s_t[1023];
    ne_start[S] = s_n[1023];
  }
}

struct TileRange {
  uint32_t cloud, local, base, valid;
};

__device__ __forceinline__ TileRange tile_range(uint32_t t, const uint32_t* tile_start, const uint32_t* off,
                                                uint32_t S, uint32_t tile) {
  TileRange r;
  r.cloud = owner(tile_start, S, t);
  r.local = t - tile_start[r.cloud];
  r.base = off[r.cloud] + r.local * tile;
  r.valid = min(tile, off[r.cloud + 1] - r.base);
  return r;
}

// Morton codes (10 bits per axis), cloud-local payload, per-cloud digit
// histograms; also clears the look-back descriptors of all passes.
__global__ void __launch_bounds__(BM_THREADS) bt_morton_kernel(const float4* __restrict__ pts, const uint32_t* off,
                                                               uint32_t S, const uint32_t* tile_start, uint32_t tile,
                                                               float mn,
                                                               float rg, float inv_rg, uint32_t* __restrict__ keys,
                                                               uint32_t* __restrict__ idx, uint32_t* seg_hist,
                                                               uint32_t* desc, size_t desc_words) {
  __shared__ uint32_t s_hist[BPASSES * BRADIX];
  for (int i = threadIdx.x; i < BPASSES * BRADIX; i += BM_THREADS) s_hist[i] = 0;
  const size_t stride = (size_t)gridDim.x * BM_THREADS;
  for (size_t i = (size_t)blockIdx.x * BM_THREADS + threadIdx.x; i < desc_words; i += stride) desc[i] = 0;
  __syncthreads();
  if (blockIdx.x >= tile_start[S]) return;
  const TileRange r = tile_range(blockIdx.x, tile_start, off, S, tile);
  const uint32_t first = off[r.cloud];
  for (uint32_t i = threadIdx.x; i < r.valid; i += BM_THREADS) {
    const uint32_t g = r.base + i;
    const uint32_t k = encode_point<uint32_t>(__ldcs(pts + g), mn, rg, inv_rg);
    keys[g] = k;
    idx[g] = g - first;
#pragma unroll
    for (int p = 0; p < BPASSES; ++p) atomicAdd(&s_hist[p * BRADIX + ((k >> (8 * p)) & 255u)], 1u);
  }
  __syncthreads();
  uint32_t* h = seg_hist + (size_t)r.cloud * BPASSES * BRADIX;
  for (int i = threadIdx.x; i < BPASSES * BRADIX; i += BM_THREADS) {
    const uint32_t c = s_hist[i];
    if (c) atomicAdd(h + i, c);
  }
}

// Per cloud and pass: digit counts -> global digit bases, in place.
__global__ void __launch_bounds__(BRADIX) bt_seg_scan_kernel(uint32_t* seg_hist, const uint32_t* off) {
  __shared__ uint32_t s_w[BRADIX / 32];
  const uint32_t c = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int p = 0; p < BPASSES; ++p) {
    uint32_t* h = seg_hist + ((size_t)c * BPASSES + p) * BRADIX;
    const uint32_t v = h[tid];
    const uint32_t incl = warp_inclusive_sum(v);
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    uint32_t pre = 0;
    for (int w = 0; w < warp; ++w) pre += s_w[w];
    h[tid] = off[c] + pre + incl - v;
    __syncthreads();
  }
}

template <int THREADS, int KPT>
struct BtSmem {
  static constexpr int WARPS = THREADS / 32;
  static constexpr int TILE = THREADS * KPT;
  uint32_t keys[TILE];
  uint32_t vals[TILE];
  uint32_t warp_hist[WARPS][BRADIX];
  uint32_t gbase[BRADIX];
  uint32_t warp_sums[WARPS + 1];
  uint32_t tile_id;
};

// One segmented onesweep pass: the single-cloud pass of sort.cu with tiles
// confined to one cloud and digit bases from that cloud's histogram.  A
// cloud's last tile is padded with all-ones keys, which rank last in the tile
// and are never stored.  Its descriptor counts them, but no tile reads it:
// the next tile starts another cloud and does not look back.
template <int THREADS, int KPT>
__global__ void __launch_bounds__(THREADS) bt_onesweep_kernel(const uint32_t* __restrict__ kin,
                                                                 const uint32_t* __restrict__ vin,
                                                                 uint32_t* __restrict__ kout,
                                                                 uint32_t* __restrict__ vout, const uint32_t* off,
                                                                 uint32_t S, const uint32_t* tile_start, int shift,
                                                                 const uint32_t* seg_base, int pass, uint32_t* desc,
                                                                 uint32_t* tile_counter, uint32_t* status) {
  using Sm = BtSmem<THREADS, KPT>;
  constexpr int WARPS = Sm::WARPS;
  static_assert(THREADS >= BRADIX, "one thread per digit");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Sm& s = *reinterpret_cast<Sm*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t lt_mask = (1u << lane) - 1u;
  for (int i = tid; i < WARPS * BRADIX; i += THREADS) (&s.warp_hist[0][0])[i] = 0;
  if (tid == 0) s.tile_id = atomicAdd(tile_counter, 1u);
  __syncthreads();
  const uint32_t tile = s.tile_id;
  if (tile >= tile_start[S]) return;
  const TileRange r = tile_range(tile, tile_start, off, S, Sm::TILE);

  uint32_t key[KPT], val[KPT];
  const uint32_t wbase = warp * 32 * KPT + lane;
#pragma unroll
  for (int j = 0; j < KPT; ++j) {
    const uint32_t i = wbase + j * 32;
    key[j] = (i < r.valid) ? kin[r.base + i] : 0xffffffffu;
    val[j] = (i < r.valid) ? vin[r.base + i] : 0u;
  }
  uint32_t* my_hist = s.warp_hist[warp];
#pragma unroll
  for (int j = 0; j < KPT; ++j) {
    const uint32_t d = (key[j] >> shift) & 255u;
    const uint32_t d0 = __shfl_sync(0xffffffffu, d, 0);
    if (__all_sync(0xffffffffu, d == d0)) {
      if (lane == 0) atomicAdd(&my_hist[d], 32u);
    } else {
      atomicAdd(&my_hist[d], 1u);
    }
  }
  __syncthreads();
  uint32_t count = 0;
  if (tid < BRADIX) {
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
      const uint32_t c = s.warp_hist[w][tid];
      s.warp_hist[w][tid] = count;
      count += c;
    }
    st_relaxed(desc + (size_t)tile * BRADIX + tid, (count << 2) | (r.local == 0 ? FLAG_INCLUSIVE : FLAG_AGGREGATE));
  }
  // Exclusive scan of the 256 digit counts (threads past 256 add zeros).
  uint32_t total;
  const uint32_t doff = block_exclusive<THREADS>(tid < BRADIX ? count : 0u, s.warp_sums, &total);
  if (tid < BRADIX) {
#pragma unroll
    for (int w = 0; w < WARPS; ++w) s.warp_hist[w][tid] += doff;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < KPT; ++j) {
    const uint32_t d = (key[j] >> shift) & 255u;
    const uint32_t peers = warp_peers<8>(d);
    const int leader = 31 - __clz(peers);
    uint32_t b0 = 0;
    if (lane == leader) b0 = atomicAdd(&my_hist[d], (uint32_t)__popc(peers));
    b0 = __shfl_sync(0xffffffffu, b0, leader);
    const uint32_t local = b0 + __popc(peers & lt_mask);
    s.keys[local] = key[j];
    s.vals[local] = val[j];
  }
  if (tid < BRADIX) {
    uint32_t excl = 0;
    if (r.local > 0) {  // look back only over this cloud's earlier tiles
      excl = lookback_window<8, BRADIX>(desc, tile, tid, status);
      st_relaxed(desc + (size_t)tile * BRADIX + tid, ((excl + count) << 2) | FLAG_INCLUSIVE);
    }
    s.gbase[tid] = seg_base[((size_t)r.cloud * BPASSES + pass) * BRADIX + tid] + excl - doff;
  }
  __syncthreads();
  // o stays inside the cloud while every look-back completes; after one ran
  // out (DEV_TIMEOUT) a later pass may see digit counts that disagree with
  // the cloud's histogram, and the check keeps its writes in bounds.
  const uint32_t end = off[r.cloud + 1];
  for (uint32_t i = tid; i < r.valid; i += THREADS) {
    const uint32_t k = s.keys[i];
    const uint32_t o = s.gbase[(k >> shift) & 255u] + i;
    if (o >= end) continue;
    kout[o] = k;
    vout[o] = s.vals[i];
  }
}

// Unique with a restart at every cloud start (a cloud's first code is always
// kept); the thread holding a cloud's first code records U_c.  The same
// single-pass look-back compaction as scan.cu's unique.
struct BuSmem {
  uint32_t keys[BU_TILE];
  uint32_t vals[BU_TILE];
  uint32_t ws[BU_THREADS / 32 + 1];
  uint32_t tile_id, prefix, halo;
};

__global__ void __launch_bounds__(BU_THREADS) bt_unique_kernel(const uint32_t* kin, const uint32_t* vin,
                                                               uint32_t* kout, uint32_t* vout, uint32_t n,
                                                               const uint32_t* off, uint32_t S, uint32_t* uoff,
                                                               uint32_t* ws, const uint32_t* bad, uint32_t* status) {
  __shared__ BuSmem s;
  if (*bad) return;
  uint32_t* desc = ws + 64;
  const int tid = threadIdx.x;
  if (tid == 0) s.tile_id = atomicAdd(ws, 1u);
  __syncthreads();
  const uint32_t tile = s.tile_id;
  const uint32_t base = tile * BU_TILE;
  if (base >= n) return;
  const uint32_t valid = min((uint32_t)BU_TILE, n - base);
  for (uint32_t i = tid; i < valid; i += BU_THREADS) {
    s.keys[i] = kin[base + i];
    s.vals[i] = vin[base + i];
  }
  if (tid == 0) s.halo = base > 0 ? kin[base - 1] : 0u;
  __syncthreads();
  const uint32_t first = tid * BU_IPT;
  const uint32_t c0 = first < valid ? owner(off, S, base + first) : 0u;
  uint32_t c = c0;
  uint32_t key[BU_IPT], val[BU_IPT], keep_mask = 0, start_mask = 0, cnt = 0;
#pragma unroll
  for (int j = 0; j < BU_IPT; ++j) {
    const uint32_t i = first + j;
    if (i < valid) {
      const uint32_t g = base + i;
      while (g >= off[c + 1]) ++c;  // off[S] = n > g, so c stays below S
      const bool start = (g == off[c]);
      key[j] = s.keys[i];
      val[j] = s.vals[i];
      const uint32_t prev = (i == 0) ? s.halo : s.keys[i - 1];
      const bool keep = start || key[j] != prev;
      keep_mask |= (uint32_t)keep << j;
      start_mask |= (uint32_t)start << j;
      cnt += keep;
    }
  }
  uint32_t total;
  const uint32_t excl = block_exclusive<BU_THREADS>(cnt, s.ws, &total);
  if (tid < 32) {
    const uint32_t pre = tile_lookback(desc, tile, total, status);
    if (tid == 0) s.prefix = pre;
  }
  __syncthreads();
  const uint32_t out0 = s.prefix;
  if (start_mask) {
    c = c0;
    uint32_t rr = excl;
#pragma unroll
    for (int j = 0; j < BU_IPT; ++j) {
      const uint32_t i = first + j;
      if (i < valid) {
        const uint32_t g = base + i;
        while (g >= off[c + 1]) ++c;
        if (start_mask & (1u << j)) uoff[c] = out0 + rr;
        rr += (keep_mask >> j) & 1u;
      }
    }
  }
  uint32_t r = excl;
#pragma unroll
  for (int j = 0; j < BU_IPT; ++j) {
    if (keep_mask & (1u << j)) {
      s.keys[r] = key[j];
      s.vals[r] = val[j];
      ++r;
    }
  }
  __syncthreads();
  for (uint32_t i = tid; i < total; i += BU_THREADS) {
    kout[out0 + i] = s.keys[i];
    vout[out0 + i] = s.vals[i];
  }
  if (tid == 0 && base + valid == n) uoff[S] = out0 + total;
}

// The resident segment form of the same unique (scan.cu's
// chunk_unique_kernel, out of place): rows of 32 codes per warp; a warp
// tracks the cloud of its row (one binary search per segment, then a step
// per cloud start), so the cloud starts of a row come as a bit mask.
__device__ __forceinline__ uint32_t bt_row_starts(const uint32_t* off, uint32_t S, uint32_t r, uint32_t& cur) {
  uint32_t smask = (off[cur] == r) ? 1u : 0u;
  while (cur + 1 < S && off[cur + 1] < r + 32) {
    ++cur;
    smask |= 1u << (off[cur] - r);
  }
  return smask;
}

__global__ void __launch_bounds__(CS_THREADS) bt_chunk_unique_kernel(const uint32_t* __restrict__ kin,
                                                                     const uint32_t* __restrict__ vin,
                                                                     uint32_t* __restrict__ kout,
                                                                     uint32_t* __restrict__ vout, uint32_t n,
                                                                     const uint32_t* off, uint32_t S, uint32_t* uoff,
                                                                     uint32_t* ws, const uint32_t* bad,
                                                                     uint32_t* status) {
  __shared__ uint32_t s_seg[CS_WARPS];
  __shared__ uint32_t s_red[CS_WARPS];
  if (*bad) return;  // the same word for every block
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t nseg = gridDim.x * CS_WARPS;
  const uint64_t SL = (((uint64_t)n + nseg - 1) / nseg + 31) & ~(uint64_t)31;
  const uint64_t beg64 = (uint64_t)(blockIdx.x * CS_WARPS + warp) * SL;
  const uint32_t beg = (uint32_t)min(beg64, (uint64_t)n);
  const uint32_t end = (uint32_t)min(beg64 + SL, (uint64_t)n);
  const uint32_t c_beg = (beg < end) ? owner(off, S, beg) : 0u;
  const uint32_t first_prev = (beg > 0 && beg < end) ? kin[beg - 1] : 0u;

  // 1. kept codes per segment
  uint32_t cnt = 0;
  {
    uint32_t carry = first_prev, cur = c_beg;
    for (uint32_t r = beg; r < end; r += 32) {
      const uint32_t i = r + lane;
      const uint32_t key = (i < end) ? kin[i] : 0u;
      const uint32_t smask = bt_row_starts(off, S, r, cur);
      uint32_t prev = __shfl_up_sync(0xffffffffu, key, 1);
      if (lane == 0) prev = carry;
      const bool keep = i < end && (i == 0 || key != prev || ((smask >> lane) & 1u));
      cnt += __popc(__ballot_sync(0xffffffffu, keep));
      carry = __shfl_sync(0xffffffffu, key, 31);
    }
  }
  if (lane == 0) s_seg[warp] = cnt;

  // 2. block prefix
  uint32_t run = cs_block_prefix(ws + 64, s_seg, s_red, status);
  run += s_seg[warp];

  // 3. rescan and write; the lane holding a cloud's first code records U_c
  {
    uint32_t carry = first_prev, cur = c_beg;
    for (uint32_t r = beg; r < end; r += 32) {
      const uint32_t i = r + lane;
      const uint32_t key = (i < end) ? kin[i] : 0u;
      const uint32_t val = (i < end) ? vin[i] : 0u;
      const uint32_t smask = bt_row_starts(off, S, r, cur);
      uint32_t prev = __shfl_up_sync(0xffffffffu, key, 1);
      if (lane == 0) prev = carry;
      const bool start = i < end && ((smask >> lane) & 1u);
      const bool keep = i < end && (i == 0 || key != prev || start);
      const uint32_t bal = __ballot_sync(0xffffffffu, keep);
      if (keep) {
        const uint32_t o = run + __popc(bal & lt);
        kout[o] = key;
        vout[o] = val;
        if (start) uoff[owner(off, S, i)] = o;
      }
      run += __popc(bal);
      carry = __shfl_sync(0xffffffffu, key, 31);
    }
  }
  // The last warp of the last block ends at n: its running count is U.
  if (blockIdx.x == gridDim.x - 1 && warp == CS_WARPS - 1 && lane == 0) uoff[S] = run;
}

// Empty clouds own no code: their U_c is the next cloud's (one thread; runs
// from the end, so runs of empty clouds resolve).
__global__ void bt_uoff_fix_kernel(const uint32_t* off, uint32_t S, uint32_t* uoff, const uint32_t* bad) {
  if (blockIdx.x != 0 || threadIdx.x != 0 || *bad) return;
  for (int c = (int)S - 1; c >= 0; --c)
    if (off[c + 1] == off[c]) uoff[c] = uoff[c + 1];
}

// Radix tree of every cloud, one thread per unique code.
__global__ void __launch_bounds__(256) bt_tree_kernel(const uint32_t* __restrict__ codes, const uint32_t* uoff,
                                                      uint32_t S, uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr,
                                                      int32_t* left, int32_t* parent, uint32_t* edge) {
  const uint32_t U = uoff[S];
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < U; g += stride) {
    const uint32_t c = owner(uoff, S, g);
    const uint32_t U0 = uoff[c];
    const int i = (int)(g - U0);
    const int m = (int)(uoff[c + 1] - U0) - 1;
    if (i == 0 && m > 0) {
      parent[U0] = 0;
      edge[U0] = 0;
    }
    if (i < m)
      karras_node<uint32_t>(codes + U0, m, i, prefix_n + U0, hll + U0, hlr + U0, left + U0, parent + U0,
                            edge + U0);
    else
      edge[g] = 0;  // the cloud's last slot adds nothing to the scan
  }
}

// Per cloud: u, m, o and the first node slot O_c, from the global scan; and
// the cloud's (U0, U1, bias, O_c) for the octree kernel.
__global__ void bt_cloud_offsets_kernel(uint32_t* uoff, const uint32_t* ne_start, const uint32_t* ps, uint32_t S,
                                        uint32_t* node_off, uint32_t* cloud_counts, uint4* cinfo,
                                        const uint32_t* bad) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= S) return;
  if (*bad) {
    uoff[c] = 0;
    node_off[c] = 0;
    cloud_counts[3 * c + 0] = cloud_counts[3 * c + 1] = cloud_counts[3 * c + 2] = 0;
    if (c == S - 1) node_off[S] = 0;
    return;
  }
  const uint32_t U0 = uoff[c], U1 = uoff[c + 1];
  const uint32_t u = U1 - U0;
  const uint32_t bias = U0 > 0 ? ps[U0 - 1] : 0u;
  const uint32_t O = ne_start[c] + bias;
  const uint32_t o = u > 0 ? 1 + ps[U1 - 1] - bias : 0u;
  node_off[c] = O;
  cinfo[c] = make_uint4(U0, U1, bias, O);
  cloud_counts[3 * c + 0] = u;
  cloud_counts[3 * c + 1] = u > 0 ? u - 1 : 0u;
  cloud_counts[3 * c + 2] = o;
  if (c == S - 1) node_off[S] = O + o;
}

// One octree body: code g of the cloud described by ci.
// Octree of every cloud, and the cloud-local node offsets (what the
// single-cloud node-offset scan gives each cloud).  Warp slices of 32 codes:
// the slice's cloud comes from one binary search (then a step or two per
// lane), every lane writes its node offset, and the codes that own octree
// nodes are compacted, with their clouds, into a per-warp queue and run 32
// at a time through the single-cloud kernel's breadth-first warp batch
// (octree_warp_batch), each lane with its own cloud.
constexpr int BT_OCT_THREADS = 256;

__global__ void __launch_bounds__(BT_OCT_THREADS) bt_octree_kernel(const uint32_t* __restrict__ codes,
                                                                   const uint32_t* uoff, uint32_t S,
                                                                   const uint4* cinfo, const uint8_t* prefix_n,
                                                                   const uint8_t* hll, const uint8_t* hlr,
                                                                   const int32_t* left, const uint32_t* edge,
                                                                   const uint32_t* ps, uint32_t* node_offsets,
                                                                   float mn, float rg, gtc_octnode* nodes,
                                                                   uint32_t capacity, uint32_t lmask_keep,
                                                                   uint32_t* status) {
  constexpr int WARPS = BT_OCT_THREADS / 32;
  constexpr int A = KeyTraits<uint32_t>::A;
  __shared__ OctWarp s_warp[WARPS];
  __shared__ uint32_t s_cloud[WARPS][64];
  const uint32_t U = uoff[S];
  const int lane = threadIdx.x & 31;
  OctWarp& Wq = s_warp[threadIdx.x >> 5];
  uint32_t* qc = s_cloud[threadIdx.x >> 5];
  uint32_t qn = 0;  // warp-uniform
  const uint32_t warps = gridDim.x * WARPS;
  auto run_batch = [&](uint32_t cnt) {
    const bool valid = (uint32_t)lane < cnt;
    const uint32_t g = valid ? Wq.q[lane] : 0u;
    const uint32_t c = valid ? qc[lane] : 0u;
    const uint32_t rest_g = (lane + 32 < qn) ? Wq.q[lane + 32] : 0u;
    const uint32_t rest_c = (lane + 32 < qn) ? qc[lane + 32] : 0u;
    __syncwarp();
    if (lane + 32 < qn) {
      Wq.q[lane] = rest_g;
      qc[lane] = rest_c;
    }
    qn -= cnt;
    OctCloud cl{0u, 0u, 0u, 0, nodes, 0u};
    bool ok = valid;
    if (valid) {
      const uint4 ci = cinfo[c];
      cl.u0 = ci.x;
      cl.mend = ci.y - 1;
      cl.bias = ci.z;
      cl.root_level = (prefix_n[ci.x] - A) / 3;
      if (ci.w >= capacity) {
        if (g == ci.x) atomicOr(status, DEV_CAPACITY);
        ok = false;
      } else {
        cl.nodes = nodes + ci.w;
        cl.capacity = capacity - ci.w;
      }
    }
    octree_warp_batch<uint32_t, true>(Wq, ok, g, cl, codes, prefix_n, hll, hlr, left, edge, ps, mn, rg, lmask_keep,
                                      status);
  };
  for (uint32_t base = (blockIdx.x * WARPS + (threadIdx.x >> 5)) * 32; base < U; base += warps * 32) {
    const uint32_t g = base + lane;
    bool act = false;
    uint32_t c = owner(uoff, S, base);  // the same address in every lane
    if (g < U) {
      while (g >= uoff[c + 1]) ++c;
      const uint4 ci = cinfo[c];
      const uint32_t k = g - ci.x, m = ci.y - ci.x - 1;
      node_offsets[g] = (k == 0) ? 0u : ps[g] - ci.z;
      if (m == 0) {  // a cloud of one distinct key: its root alone (D18)
        if (ci.w < capacity)
          octree_root_only<uint32_t>(nodes + ci.w, capacity - ci.w, mn, rg, status);
        else
          atomicOr(status, DEV_CAPACITY);
      } else {
        act = k < m && (k == 0 || edge[g] > 0);
      }
    }
    const uint32_t bal = __ballot_sync(0xffffffffu, act);
    if (act) {
      const uint32_t pos = qn + __popc(bal & ((1u << lane) - 1u));
      Wq.q[pos] = g;
      qc[pos] = c;
    }
    qn += __popc(bal);
    __syncwarp();
    if (qn >= 32) run_batch(32u);
  }
  if (qn > 0) run_batch(qn);
}

template <int THREADS, int KPT>
cudaError_t launch_bt_pass(cudaStream_t s, uint32_t grid, const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                           uint32_t* vout, const uint32_t* off, uint32_t S, const uint32_t* tile_start, int shift,
                           const uint32_t* seg_base, int pass, uint32_t* desc, uint32_t* tile_counter,
                           uint32_t* status) {
  using Sm = BtSmem<THREADS, KPT>;
  cudaError_t e = kernel_setup(bt_onesweep_kernel<THREADS, KPT>, THREADS, sizeof(Sm));
  if (e != cudaSuccess) return e;
  bt_onesweep_kernel<THREADS, KPT><<<grid, THREADS, sizeof(Sm), s>>>(kin, vin, kout, vout, off, S, tile_start, shift,
                                                                     seg_base, pass, desc, tile_counter, status);
  return cudaGetLastError();
}

cudaError_t launch_bt_variant(int v, cudaStream_t s, uint32_t grid, const uint32_t* kin, const uint32_t* vin,
                              uint32_t* kout, uint32_t* vout, const uint32_t* off, uint32_t S,
                              const uint32_t* tile_start, int shift, const uint32_t* seg_base, int pass,
                              uint32_t* desc, uint32_t* tile_counter, uint32_t* status) {
#define GTC_BT(T, K)                                                                                               \
  return launch_bt_pass<T, K>(s, grid, kin, vin, kout, vout, off, S, tile_start, shift, seg_base, pass, desc, \
                              tile_counter, status)
  switch (v) {
    case 1: GTC_BT(256, 16);
    case 2: GTC_BT(384, 16);
    case 3: GTC_BT(512, 8);
    case 4: GTC_BT(256, 24);
    default: GTC_BT(512, 12);
  }
#undef GTC_BT
}

std::atomic<int> g_bt_pinned{-1};  // gtc_batched_set_variant

struct BatchWs {
  uint32_t* tile_start;  // [S + 1]
  uint32_t* ne_start;    // [S + 1]
  uint32_t* seg_hist;    // [S][4][256]
  uint32_t* counters;    // [0..3] pass tickets
  uint32_t* desc;        // [4][tiles_max][256]
  uint32_t* keys_alt;    // [n]
  uint32_t* idx_alt;     // [n]
  uint32_t* ps;          // [n]
  void* scan_ws;
  size_t desc_words;
  uint32_t tiles_max;
};

// A cloud of len points has ceil(len / TILE) tiles, so the batch has at most
// n / TILE + S of them; sized for the smallest tile of any variant.
size_t batch_layout(uint32_t n, uint32_t S, BatchWs* W, char* p) {
  const uint32_t tiles_max = ceil_div(n > 0 ? n : 1, BT_MIN_TILE) + S;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    char* q = p ? p + o : nullptr;
    o += align_up(bytes, 256);
    return q;
  };
  BatchWs w;
  w.tile_start = reinterpret_cast<uint32_t*>(take(((size_t)S + 1) * 4));
  w.ne_start = reinterpret_cast<uint32_t*>(take(((size_t)S + 1) * 4));
  w.seg_hist = reinterpret_cast<uint32_t*>(take((size_t)S * BPASSES * BRADIX * 4));
  w.counters = reinterpret_cast<uint32_t*>(take(256));
  w.desc_words = (size_t)BPASSES * tiles_max * BRADIX;
  w.desc = reinterpret_cast<uint32_t*>(take(w.desc_words * 4));
  w.keys_alt = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
  w.idx_alt = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
  w.ps = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
  w.scan_ws = take(scan_workspace_bytes(n));
  w.tiles_max = tiles_max;
  if (W) *W = w;
  return o;
}

}  // namespace
}  // namespace gtc

using namespace gtc;

extern "C" {

GTC_API gtc_status gtc_batched_workspace_size(uint32_t n_total, uint32_t n_clouds, size_t* bytes) {
  if (!bytes || n_clouds == 0 || n_clouds > MAX_CLOUDS || n_total >= (1u << 30)) return GTC_ERR_INVALID_ARG;
  *bytes = batch_layout(n_total, n_clouds, nullptr, nullptr);
  return GTC_OK;
}

}  // extern "C"

namespace gtc {
int batched_select_variant(uint32_t n) {
  const int pinned = g_bt_pinned.load(std::memory_order_relaxed);
  if (pinned >= 0) return pinned;
  const int t = tuned_batched_variant(n);
  return (t >= 0 && t < kBtNumVariants) ? t : 0;
}
int batched_num_variants() { return kBtNumVariants; }

// The batched build with the segmented onesweep's tile shape given.
gtc_status build_octree_batched_variant(gtc_ctx* ctx, const float* pts, const uint32_t* d_offsets,
                                        uint32_t n_clouds, uint32_t n_total, float min_coord, float range,
                                        const gtc_batch_buffers* out, void* ws, size_t ws_bytes,
                                        gtc_stream_t stream, int variant) {
  if (!ctx) return GTC_ERR_INVALID_ARG;
  if (variant < 0 || variant >= kBtNumVariants)
    return context_error(ctx, GTC_ERR_INVALID_ARG, "no such batched variant", cudaSuccess);
  const uint32_t tile = (uint32_t)(kBtVariants[variant].threads * kBtVariants[variant].kpt);
  if (!out || !d_offsets || n_clouds == 0 || n_clouds > MAX_CLOUDS)
    return context_error(ctx, GTC_ERR_INVALID_ARG, "need offsets, outputs and 1..2^20 clouds", cudaSuccess);
  if (n_total >= (1u << 30)) return context_error(ctx, GTC_ERR_INVALID_ARG, "n_total must be < 2^30", cudaSuccess);
  if (n_total > 0 && (!pts || (reinterpret_cast<uintptr_t>(pts) & 15)))
    return context_error(ctx, GTC_ERR_INVALID_ARG, "pts must be a 16-byte aligned float[n][4]", cudaSuccess);
  if (!out->keys || !out->idx || !out->prefix_n || !out->has_leaf_left || !out->has_leaf_right ||
      !out->left_child || !out->parent || !out->edge_count || !out->node_offsets || !out->nodes ||
      !out->key_offset || !out->node_offset || !out->cloud_counts)
    return context_error(ctx, GTC_ERR_INVALID_ARG, "null output buffer", cudaSuccess);
  const size_t need = batch_layout(n_total, n_clouds, nullptr, nullptr);
  if (!ws || ws_bytes < need || (reinterpret_cast<uintptr_t>(ws) & 255))
    return context_error(ctx, GTC_ERR_INVALID_ARG, "batched workspace missing, too small or not 256-byte aligned",
                         cudaSuccess);
  BatchWs W;
  batch_layout(n_total, n_clouds, &W, reinterpret_cast<char*>(ws));
  const Launch L = context_launch(ctx, stream);
  cudaStream_t s = L.stream;
  const uint32_t S = n_clouds;
  cudaError_t e;
#define BCHK(x)                                                                   \
  do {                                                                            \
    if ((e = (x)) != cudaSuccess) return context_error(ctx, GTC_ERR_CUDA, #x, e); \
  } while (0)
  if (n_total == 0) {
    BCHK(cudaMemsetAsync(out->key_offset, 0, ((size_t)S + 1) * 4, s));
    BCHK(cudaMemsetAsync(out->node_offset, 0, ((size_t)S + 1) * 4, s));
    BCHK(cudaMemsetAsync(out->cloud_counts, 0, (size_t)S * 12, s));
    return GTC_OK;
  }
  uint32_t* bad = W.counters + 8;
  {
    Stage t(ctx, stream, GTC_STAGE_MORTON);
    BCHK(cudaMemsetAsync(W.seg_hist, 0, (size_t)S * BPASSES * BRADIX * 4, s));
    BCHK(cudaMemsetAsync(W.counters, 0, 256, s));
    bt_tiles_kernel<<<1, 1024, 0, s>>>(d_offsets, S, n_total, tile, W.tile_start, W.ne_start, bad,
                                       out->key_offset, L.status);
    BCHK(cudaGetLastError());
    bt_morton_kernel<<<W.tiles_max, BM_THREADS, 0, s>>>(reinterpret_cast<const float4*>(pts), d_offsets, S,
                                                        W.tile_start, tile, min_coord, range, pow2_reciprocal(range),
                                                        W.keys_alt, W.idx_alt,
                                                        W.seg_hist, W.desc, W.desc_words);
    BCHK(cudaGetLastError());
    bt_seg_scan_kernel<<<S, BRADIX, 0, s>>>(W.seg_hist, d_offsets);
    BCHK(cudaGetLastError());
  }
  uint32_t* src_k = W.keys_alt;
  uint32_t* src_v = W.idx_alt;
  uint32_t* dst_k = out->keys;
  uint32_t* dst_v = out->idx;
  for (int p = 0; p < BPASSES; ++p) {
    Stage t(ctx, stream, GTC_STAGE_ONESWEEP);
    BCHK(launch_bt_variant(variant, s, W.tiles_max, src_k, src_v, dst_k, dst_v, d_offsets, S, W.tile_start, 8 * p,
                           W.seg_hist, p, W.desc + (size_t)p * W.tiles_max * BRADIX, W.counters + p, L.status));
    std::swap(src_k, dst_k);
    std::swap(src_v, dst_v);
  }
  // After 4 passes the sorted pairs are back in the alternate buffers.
  {
    Stage t(ctx, stream, GTC_STAGE_UNIQUE);
    const uint32_t utiles = ceil_div(n_total, BU_TILE);
    uint32_t* uws = reinterpret_cast<uint32_t*>(W.scan_ws);
    // The resident segment form once the batch fills the GPU; its
    // descriptors fit the workspace's tile count.
    int occ = 1;  // resident blocks per SM
    if (kernel_setup(bt_chunk_unique_kernel, CS_THREADS, 0, &occ) != cudaSuccess) {
      cudaGetLastError();
      occ = 1;
    }
    const uint32_t g = min((uint32_t)(occ * L.num_sms), utiles);
    if (g >= 64 && (uint64_t)n_total >= (uint64_t)g * CS_WARPS * 256) {
      BCHK(cudaMemsetAsync(uws, 0, (64 + (size_t)g) * 4, s));
      bt_chunk_unique_kernel<<<g, CS_THREADS, 0, s>>>(src_k, src_v, out->keys, out->idx, n_total, d_offsets, S,
                                                      out->key_offset, uws, bad, L.status);
    } else {
      BCHK(cudaMemsetAsync(uws, 0, (64 + (size_t)utiles) * 4, s));
      bt_unique_kernel<<<utiles, BU_THREADS, 0, s>>>(src_k, src_v, out->keys, out->idx, n_total, d_offsets, S,
                                                     out->key_offset, uws, bad, L.status);
    }
    BCHK(cudaGetLastError());
    bt_uoff_fix_kernel<<<1, 32, 0, s>>>(d_offsets, S, out->key_offset, bad);
    BCHK(cudaGetLastError());
  }
  {
    Stage t(ctx, stream, GTC_STAGE_RADIX_TREE);
    if (tree_get_method() == 1) {
      // idx_alt is free after unique: the queue of long-range splits.
      uint32_t* q_count = W.counters + 16;  // zeroed with the counters
      radix_tree_window_kernel<uint32_t, true><<<ceil_div(n_total, TW_T), TW_THREADS, 0, s>>>(
          out->keys, nullptr, 0, out->key_offset, S, out->prefix_n, out->has_leaf_left, out->has_leaf_right,
          out->left_child, out->parent, out->edge_count, nullptr, W.idx_alt, q_count);
      BCHK(cudaGetLastError());
      radix_tree_slow_kernel<uint32_t, true><<<L.num_sms * 2, 256, 0, s>>>(
          out->keys, nullptr, 0, out->key_offset, S, out->prefix_n, out->has_leaf_left, out->has_leaf_right,
          out->left_child, out->parent, out->edge_count, W.idx_alt, q_count);
    } else {
      const uint32_t grid = max(1u, min(ceil_div(n_total, 256), (uint32_t)L.num_sms * 8));
      bt_tree_kernel<<<grid, 256, 0, s>>>(out->keys, out->key_offset, S, out->prefix_n, out->has_leaf_left,
                                          out->has_leaf_right, out->left_child, out->parent, out->edge_count);
    }
    BCHK(cudaGetLastError());
  }
  {
    Stage t(ctx, stream, GTC_STAGE_PREFIX_SUM);
    BCHK(launch_inclusive_scan_dev(L, out->edge_count, W.ps, out->key_offset + S, n_total, W.scan_ws));
    // The per-cloud digit histograms are dead after the sort: their space
    // holds the per-cloud octree info.
    bt_cloud_offsets_kernel<<<ceil_div(S, 256), 256, 0, s>>>(out->key_offset, W.ne_start, W.ps, S,
                                                            out->node_offset, out->cloud_counts,
                                                            reinterpret_cast<uint4*>(W.seg_hist), bad);
    BCHK(cudaGetLastError());
  }
  {
    Stage t(ctx, stream, GTC_STAGE_OCTREE);
    int occ = 4;  // resident blocks per SM
    if (kernel_setup(bt_octree_kernel, BT_OCT_THREADS, 0, &occ) != cudaSuccess) {
      cudaGetLastError();
      occ = 4;
    }
    const uint32_t ogrid = max(1u, min(ceil_div(n_total, BT_OCT_THREADS), (uint32_t)(L.num_sms * occ)));
    bt_octree_kernel<<<ogrid, BT_OCT_THREADS, 0, s>>>(out->keys, out->key_offset, S, reinterpret_cast<const uint4*>(W.seg_hist),
                                           out->prefix_n, out->has_leaf_left, out->has_leaf_right, out->left_child,
                                           out->edge_count, W.ps, out->node_offsets, min_coord, range, out->nodes,
                                           out->nodes_capacity, leaf_mask_keep(), L.status);
    BCHK(cudaGetLastError());
  }
#undef BCHK
  return GTC_OK;
}
}  // namespace gtc

extern "C" {

GTC_API gtc_status gtc_build_octree_batched(gtc_ctx* ctx, const float* pts, const uint32_t* d_offsets,
                                            uint32_t n_clouds, uint32_t n_total, float min_coord, float range,
                                            const gtc_batch_buffers* out, void* ws, size_t ws_bytes,
                                            gtc_stream_t stream) {
  return build_octree_batched_variant(ctx, pts, d_offsets, n_clouds, n_total, min_coord, range, out, ws, ws_bytes,
                                      stream, batched_select_variant(n_total));
}

GTC_API int gtc_batched_num_variants(void) { return kBtNumVariants; }

GTC_API gtc_status gtc_batched_variant_shape(int variant, int* threads, int* keys_per_thread) {
  if (variant < 0 || variant >= kBtNumVariants) return GTC_ERR_INVALID_ARG;
  if (threads) *threads = kBtVariants[variant].threads;
  if (keys_per_thread) *keys_per_thread = kBtVariants[variant].kpt;
  return GTC_OK;
}

GTC_API gtc_status gtc_batched_set_variant(int variant) {
  if (variant < -1 || variant >= kBtNumVariants) return GTC_ERR_INVALID_ARG;
  g_bt_pinned.store(variant, std::memory_order_relaxed);
  return GTC_OK;
}

GTC_API int gtc_batched_get_variant(uint32_t n_total) { return batched_select_variant(n_total); }

}  // extern "C"
