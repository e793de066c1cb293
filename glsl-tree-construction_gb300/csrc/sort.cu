// sort.cu - global digit histogram and onesweep LSD digit-binning passes.
//
// Replaces histogram.comp:103-195 (upfront histogram) and
// new_radix_sort.comp:116-314 (one onesweep pass) driven by
// test_radix_sort (radixsort-vulkan/src/main.rs:175-800), with a u32 payload
// carried alongside the keys and 8-bit digits over [begin_bit, end_bit).
//
// One pass over a tile of TILE = THREADS * KPT keys:
//   1. tile ticket from an atomic counter (tiles start in ticket order, so a
//      tile only ever waits on tiles that are already running);
//   2. warp-striped coalesced loads (lane l of warp w holds keys
//      w*32*KPT + j*32 + l), padding past n with all-ones keys (max digit);
//   3. warp-level multisplit: 8 __ballot_sync per key give the peer mask of
//      lanes with the same digit; ranks follow original order (stable);
//   4. per-digit counts published as AGGREGATE descriptors [tile][digit];
//   5. decoupled look-back, one thread per digit, bounded spins;
//   6. scatter into shared memory in tile-local digit order, then coalesced
//      writes of each digit run to its global position.

#include <cstddef>
#include <cstdio>

#include <atomic>

#include "gtc_internal.cuh"

namespace gtc {

constexpr int RADIX = 256;
constexpr int MAX_PASSES = 8;

// ----------------------------------------------------- block-level helpers --
// Exclusive scan of one value per thread over the first 256 threads (warps
// 0..7); every thread of the block must call it.  Returns the exclusive
// prefix for threads < 256.
template <int THREADS>
__device__ __forceinline__ uint32_t scan256_exclusive(uint32_t v, uint32_t* warp_sums /*[8]*/) {
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  uint32_t incl = 0;
  if (tid < RADIX) {
    incl = warp_inclusive_sum(v);
    if (lane == 31) warp_sums[warp] = incl;
  }
  __syncthreads();
  uint32_t pre = 0;
  if (tid < RADIX) {
#pragma unroll
    for (int w = 0; w < RADIX / 32; ++w) pre += (w < warp) ? warp_sums[w] : 0u;
  }
  return pre + incl - v;
}

// ------------------------------------------------------ global histogram ---
template <class K>
__device__ __forceinline__ void hist_add(uint32_t (*s_hist)[RADIX], K k, int begin_bit, int end_bit, int passes,
                                         int db) {
#pragma unroll
  for (int p = 0; p < MAX_PASSES; ++p) {
    if (p < passes) {
      const int sh = begin_bit + db * p;
      const int bits = min(db, end_bit - sh);
      const uint32_t d = (uint32_t)(k >> sh) & ((1u << bits) - 1u);
      atomicAdd(&s_hist[p][d], 1u);
    }
  }
}

// Adds the block's shared histograms into the global counts; the last block
// to finish turns the counts into exclusive prefixes (bin offsets) and resets
// the done counter, so the workspace needs no clearing between calls.
template <int THREADS>
__device__ __forceinline__ void hist_finish(uint32_t (*s_hist)[RADIX], int passes, uint32_t* counts,
                                            uint32_t* bin_offsets, uint32_t* done, uint32_t* s_last) {
  __syncthreads();
  for (int i = threadIdx.x; i < passes * RADIX; i += THREADS) {
    const uint32_t c = (&s_hist[0][0])[i];
    if (c) atomicAdd(&counts[i], c);
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) *s_last = (atomicAdd(done, 1u) == gridDim.x - 1) ? 1u : 0u;
  __syncthreads();
  if (*s_last == 0) return;
  __threadfence();
  // The last block turns every pass's counts into offsets at once: one warp
  // per pass, eight consecutive bins per lane (one round trip for all).
  static_assert(THREADS / 32 >= MAX_PASSES, "a warp per pass");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp < passes) {
    const uint4* c4 = reinterpret_cast<const uint4*>(counts + warp * RADIX + lane * 8);
    const uint4 a = __ldcg(c4), b = __ldcg(c4 + 1);
    uint4 ea, eb;  // lane-local exclusive prefixes
    ea.x = 0;
    ea.y = a.x;
    ea.z = ea.y + a.y;
    ea.w = ea.z + a.z;
    eb.x = ea.w + a.w;
    eb.y = eb.x + b.x;
    eb.z = eb.y + b.y;
    eb.w = eb.z + b.z;
    const uint32_t tot = eb.w + b.w;
    const uint32_t base = warp_inclusive_sum(tot) - tot;
    ea.x += base;
    ea.y += base;
    ea.z += base;
    ea.w += base;
    eb.x += base;
    eb.y += base;
    eb.z += base;
    eb.w += base;
    uint4* o4 = reinterpret_cast<uint4*>(bin_offsets + warp * RADIX + lane * 8);
    o4[0] = ea;
    o4[1] = eb;
  }
  if (threadIdx.x == 0) *done = 0;
}

__device__ __forceinline__ void zero_region(uint32_t* p, size_t words) {
  // Grid-stride zeroing of a 16-byte aligned region (next sort's descriptors).
  const size_t n4 = words / 4;
  uint4* p4 = reinterpret_cast<uint4*>(p);
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) p4[i] = make_uint4(0, 0, 0, 0);
  for (size_t i = n4 * 4 + (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += stride) p[i] = 0;
}

template <class K, int THREADS>
__global__ void __launch_bounds__(THREADS) global_hist_kernel(const K* __restrict__ keys, uint32_t n, int begin_bit,
                                                              int end_bit, int passes, int db, uint32_t* counts,
                                                              uint32_t* bin_offsets, uint32_t* done,
                                                              uint32_t* zero_ptr, size_t zero_words,
                                                              const uint32_t* run_if) {
  if (run_if && *run_if == 0) return;
  __shared__ uint32_t s_hist[MAX_PASSES][RADIX];
  __shared__ uint32_t s_last;
  for (int i = threadIdx.x; i < MAX_PASSES * RADIX; i += THREADS) (&s_hist[0][0])[i] = 0;
  zero_region(zero_ptr, zero_words);
  __syncthreads();
  const size_t stride = (size_t)gridDim.x * THREADS;
  constexpr int VEC = 16 / sizeof(K);
  const bool aligned = (reinterpret_cast<uintptr_t>(keys) & 15) == 0;
  const uint32_t nvec = aligned ? n / VEC : 0;
  for (size_t v = (size_t)blockIdx.x * THREADS + threadIdx.x; v < nvec; v += stride) {
    const uint4 q = __ldcs(reinterpret_cast<const uint4*>(keys) + v);
    const K* kk = reinterpret_cast<const K*>(&q);
#pragma unroll
    for (int e = 0; e < VEC; ++e) hist_add<K>(s_hist, kk[e], begin_bit, end_bit, passes, db);
  }
  for (size_t i = (size_t)nvec * VEC + (size_t)blockIdx.x * THREADS + threadIdx.x; i < n; i += stride)
    hist_add<K>(s_hist, keys[i], begin_bit, end_bit, passes, db);
  hist_finish<THREADS>(s_hist, passes, counts, bin_offsets, done, &s_last);
}

// Digit counts of every pass over bits [LB, 3B) of a Morton code: the
// shifts and masks are compile-time constants.
template <class K, int LB>
__device__ __forceinline__ void hist_add_code(uint32_t (*s_hist)[RADIX], K k) {
  constexpr int BITS = 3 * KeyTraits<K>::B;
  constexpr int P = (BITS - LB + 7) / 8;
#pragma unroll
  for (int p = 0; p < P; ++p) {
    const int sh = LB + 8 * p;
    const uint32_t d = (uint32_t)(k >> sh) & ((1u << (BITS - sh < 8 ? BITS - sh : 8)) - 1u);
    atomicAdd(&s_hist[p][d], 1u);
  }
}

// Fused Morton encode + global histogram of all passes of the following
// sort over bits [LB, 3B) of the code: the first stage of the pipeline reads
// the points once and leaves the sort ready to run (its first pass makes
// the index payload itself).
template <class K, int THREADS, int Q, int LB>
__global__ void __launch_bounds__(THREADS, 3) morton_hist_kernel(const float4* __restrict__ pts, K* __restrict__ keys,
                                                              uint32_t n, float mn, float rg, float inv_rg,
                                                              uint32_t* counts, uint32_t* bin_offsets, uint32_t* done,
                                                              uint32_t* zero_ptr, size_t zero_words) {
  griddep_wait();
  constexpr int P = (3 * KeyTraits<K>::B - LB + 7) / 8;
  __shared__ uint32_t s_hist[P][RADIX];
  __shared__ uint32_t s_last;
  for (int i = threadIdx.x; i < P * RADIX; i += THREADS) (&s_hist[0][0])[i] = 0;
  zero_region(zero_ptr, zero_words);
  __syncthreads();
  const size_t stride = (size_t)gridDim.x * THREADS;
  size_t i = (size_t)blockIdx.x * THREADS + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {  // four points in flight per thread
    float4 p[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) p[u] = __ldcs(pts + i + u * stride);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const K k = encode_point<K, Q>(p[u], mn, rg, inv_rg);
      keys[i + u * stride] = k;
      hist_add_code<K, LB>(s_hist, k);
    }
  }
  for (; i < n; i += stride) {
    const K k = encode_point<K, Q>(__ldcs(pts + i), mn, rg, inv_rg);
    keys[i] = k;
    hist_add_code<K, LB>(s_hist, k);
  }
  hist_finish<THREADS>(s_hist, P, counts, bin_offsets, done, &s_last);
}

// --------------------------------------------------------- run fixup ----
// A stable LSD sort over bits [lb, 64) only leaves keys that agree above bit
// lb together, in their original order.  Sorting every such run stably by
// its low lb bits completes the sort of the whole key: the low digits decide
// only among keys whose high digits tie.  For point-cloud Morton codes these
// runs are short (277,486 runs of 2 to 20 keys in the 10M clustered codes
// for lb = 23, 0.66M keys in all), so three 8-bit passes over every key
// become one read of the keys and a few touches of 7% of them.
// run_fixup_kernel finds the runs of a chunk of keys per block and sorts
// them: a run of up to FX_LANE keys is sorted by one lane (all lanes at
// once), up to 31 are ranked in registers by a warp, and longer runs are
// sorted by stable 8-bit counting passes through the scratch arrays (any
// length, one warp, linear time).  Runs whose low bits are already in order
// are left as they are.
constexpr int FX_THREADS = 256;
constexpr int FX_ROWS = 8;        // rows of 32 keys loaded together

template <class K>
__device__ __forceinline__ bool fx_same(K a, K b, int lb) {
  return (a >> lb) == (b >> lb);
}

// Run starting at s, by one lane: if it holds at most FX_LANE keys, sorts it
// in registers (odd-even transposition over FX_LANE slots; swapping only on
// strictly greater low bits keeps it stable) and returns true; longer runs
// are left to the whole warp.
constexpr int FX_LANE = 8;
template <class K>
__device__ __forceinline__ bool fx_lane_run(K* keys, uint32_t* vals, uint32_t s, uint32_t n, int lb) {
  const K lmask = (K(1) << lb) - 1;
  K kk[FX_LANE + 1];
#pragma unroll
  for (int q = 0; q <= FX_LANE; ++q) kk[q] = (s + q < n) ? keys[s + q] : K(0);
  uint32_t g = 1;
#pragma unroll
  for (int q = 1; q <= FX_LANE; ++q)
    if (g == (uint32_t)q && s + q < n && fx_same(kk[q], kk[0], lb)) g = q + 1;
  if (g > (uint32_t)FX_LANE) return false;
  bool sorted = true;
#pragma unroll
  for (int q = 1; q < FX_LANE; ++q)
    if ((uint32_t)q < g && (kk[q - 1] & lmask) > (kk[q] & lmask)) sorted = false;
  if (sorted) return true;
  uint32_t vv[FX_LANE];
#pragma unroll
  for (int q = 0; q < FX_LANE; ++q) vv[q] = (uint32_t)q < g ? vals[s + q] : 0u;
#pragma unroll
  for (int round = 0; round < FX_LANE; ++round) {
#pragma unroll
    for (int q = round & 1; q + 1 < FX_LANE; q += 2) {
      if ((uint32_t)(q + 1) < g && (kk[q] & lmask) > (kk[q + 1] & lmask)) {
        const K tk = kk[q];
        kk[q] = kk[q + 1];
        kk[q + 1] = tk;
        const uint32_t tv = vv[q];
        vv[q] = vv[q + 1];
        vv[q + 1] = tv;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < FX_LANE; ++q)
    if ((uint32_t)q < g) {
      keys[s + q] = kk[q];
      vals[s + q] = vv[q];
    }
  return true;
}

// Run [s, s + g), 2 <= g <= 32, ranked by (low bits, position) in registers;
// lane l holds key s + l (loaded by the caller).
template <class K>
__device__ __forceinline__ void fx_short_run(K* keys, uint32_t* vals, uint32_t s, uint32_t g, int lb, K k) {
  const int lane = threadIdx.x & 31;
  const bool in = (uint32_t)lane < g;
  const uint32_t lo = (uint32_t)(k & ((K(1) << lb) - 1));
  const uint32_t pl = __shfl_up_sync(0xffffffffu, lo, 1);
  if (__ballot_sync(0xffffffffu, in && lane > 0 && pl > lo) == 0) return;  // already in order
  const uint32_t v = in ? vals[s + lane] : 0u;
  uint32_t rank = 0;
  for (uint32_t i = 0; i < g; ++i) {  // warp-uniform
    const uint32_t li = __shfl_sync(0xffffffffu, lo, (int)i);
    rank += (li < lo || (li == lo && i < (uint32_t)lane)) ? 1u : 0u;
  }
  __syncwarp();
  if (in) {
    keys[s + rank] = k;
    vals[s + rank] = v;
  }
}

// Run [s, s + g), g >= 32: stable counting passes over the low bits, 8 at a
// time from bit 0, alternating between the keys and the scratch arrays (an
// odd number of passes ends with a copy back).  Digits that reach above lb
// hold bits the whole run shares, so they order nothing.  cnt is this
// warp's 256 shared counters.
template <class K>
__device__ void fx_long_run(K* keys, uint32_t* vals, K* sk, uint32_t* sv, uint32_t s, uint32_t g, int lb,
                            uint32_t* cnt) {
  const int lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  const K lmask = (K(1) << lb) - 1;
  bool bad = false;
  for (uint32_t i = 1 + lane; i < g; i += 32) bad |= (keys[s + i - 1] & lmask) > (keys[s + i] & lmask);
  if (__ballot_sync(0xffffffffu, bad) == 0) return;  // already in order (runs of equal keys)
  const int npass = (lb + 7) / 8;
  for (int pass = 0; pass < npass; ++pass) {
    const bool odd = pass & 1;
    const K* ik = odd ? sk : keys;
    const uint32_t* iv = odd ? sv : vals;
    K* ok = odd ? keys : sk;
    uint32_t* ov = odd ? vals : sv;
    const int sh = 8 * pass;
    for (int b = lane; b < 256; b += 32) cnt[b] = 0;
    __syncwarp();
    for (uint32_t i = lane; i < g; i += 32) atomicAdd(&cnt[(uint32_t)(ik[s + i] >> sh) & 255u], 1u);
    __syncwarp();
    uint32_t c[8], tot = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      c[j] = cnt[lane * 8 + j];
      tot += c[j];
    }
    uint32_t base = warp_inclusive_sum(tot) - tot;
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      cnt[lane * 8 + j] = base;
      base += c[j];
    }
    __syncwarp();
    for (uint32_t r0 = 0; r0 < g; r0 += 32) {  // rounds of 32 in order: stable
      const uint32_t i = r0 + lane;
      const bool in = i < g;
      const K k = in ? ik[s + i] : K(0);
      const uint32_t v = in ? iv[s + i] : 0u;
      const uint32_t d = in ? ((uint32_t)(k >> sh) & 255u) : 256u + (uint32_t)lane;  // idle lanes: own digit
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
      const uint32_t pos = in ? cnt[d] + __popc(peers & lt) : 0u;
      __syncwarp();
      if (in && (peers >> lane) == 1u) cnt[d] += __popc(peers);  // the highest peer advances the digit
      __syncwarp();
      if (in) {
        ok[s + pos] = k;
        ov[s + pos] = v;
      }
    }
    __syncwarp();  // the pass's writes are visible to the warp's next reads
  }
  if (npass & 1) {  // the last pass wrote the scratch arrays
    for (uint32_t i = lane; i < g; i += 32) {
      keys[s + i] = sk[s + i];
      vals[s + i] = sv[s + i];
    }
    __syncwarp();
  }
}

// Finds and sorts the runs of one chunk of FX_THREADS * FX_ROWS = 2,048
// consecutive keys per block.  Each warp streams eight rows of 32 keys (a
// second, offset load for the next key, one ballot per row); a run starts
// where key i + 1 agrees with key i above lb but key i - 1 does not.  The
// block lists its starts in shared memory (at most one per two keys), then
// its lanes take one listed run each: those keys were just read by this SM,
// so the sort mostly hits L1.  A run belongs to the block holding its first
// key and may reach into later chunks.  Blocks never write outside their own
// runs, and what a block reads of a neighbour's run is the same whatever
// order that run is in at the time (its keys agree above lb), so blocks run
// in any order.
template <class K>
__global__ void __launch_bounds__(FX_THREADS, 4) run_fixup_kernel(K* keys, uint32_t* vals, K* sk, uint32_t* sv,
                                                                 uint32_t n, int lb) {
  griddep_wait();
  constexpr int WARPS = FX_THREADS / 32;
  constexpr uint32_t CHUNK = FX_THREADS * FX_ROWS;
  __shared__ uint32_t s_list[CHUNK / 2];
  __shared__ uint32_t s_tot[WARPS];
  __shared__ uint32_t s_cnt[WARPS][256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t r0 = blockIdx.x * CHUNK + (uint32_t)warp * FX_ROWS * 32;
  uint32_t st[FX_ROWS];
  uint32_t tot = 0;
  if (r0 < n) {  // warp-uniform
    K kr[FX_ROWS], kn[FX_ROWS];
#pragma unroll
    for (int j = 0; j < FX_ROWS; ++j) {
      const uint32_t i = r0 + (uint32_t)j * 32 + lane;
      const bool ok = i + 1 < n;
      kr[j] = ok ? keys[i] : K(0);
      kn[j] = ok ? keys[i + 1] : K(0);
    }
    // Does the run through r0 start before it?
    bool carry = r0 > 0 && fx_same(keys[r0 - 1], keys[r0], lb);  // warp-uniform, two broadcast loads
#pragma unroll
    for (int j = 0; j < FX_ROWS; ++j) {
      const uint32_t i = r0 + (uint32_t)j * 32 + lane;
      const uint32_t dup = __ballot_sync(0xffffffffu, i + 1 < n && fx_same(kr[j], kn[j], lb));
      st[j] = dup & ~((dup << 1) | (carry ? 1u : 0u));
      carry = (dup >> 31) != 0;
      tot += (uint32_t)__popc(st[j]);
    }
  } else {
#pragma unroll
    for (int j = 0; j < FX_ROWS; ++j) st[j] = 0;
  }
  if (lane == 0) s_tot[warp] = tot;
  __syncthreads();
  uint32_t at = 0, total = 0;
#pragma unroll
  for (int w = 0; w < WARPS; ++w) {
    const uint32_t c = s_tot[w];
    at += w < warp ? c : 0u;
    total += c;
  }
#pragma unroll
  for (int j = 0; j < FX_ROWS; ++j) {
    if ((st[j] >> lane) & 1u) s_list[at + (uint32_t)__popc(st[j] & lt)] = r0 + (uint32_t)j * 32 + lane;
    at += (uint32_t)__popc(st[j]);
  }
  __syncthreads();
  // Each lane the short run at one list entry, then the warp the longer
  // runs its lanes met, one by one.
  for (uint32_t e0 = (uint32_t)warp * 32; e0 < total; e0 += FX_THREADS) {  // warp-uniform
    const uint32_t e = e0 + lane;
    const uint32_t s0 = e < total ? s_list[e] : 0u;
    const bool longer = e < total && !fx_lane_run<K>(keys, vals, s0, n, lb);
    __syncwarp();  // the lanes' writes are visible to the warp
    uint32_t bal = __ballot_sync(0xffffffffu, longer);
    while (bal) {  // warp-uniform
      const uint32_t s = __shfl_sync(0xffffffffu, s0, __ffs(bal) - 1);
      bal &= bal - 1;
      // Keys s .. s + 31 in one load: the run's end if it holds at most 32
      // keys, and then its keys as well.
      const K kq = s + lane < n ? keys[s + lane] : K(0);
      const K ks = (K)__shfl_sync(0xffffffffu, (unsigned long long)kq, 0);
      const uint32_t b0 = __ballot_sync(0xffffffffu, s + lane >= n || !fx_same(kq, ks, lb));
      if (b0) {
        fx_short_run<K>(keys, vals, s, (uint32_t)(__ffs(b0) - 1), lb, kq);
        continue;
      }
      uint32_t g = 0;  // run length: first key past s + 31 that differs above lb
      for (uint32_t q0 = s + 32;; q0 += 32) {
        const uint32_t q = q0 + lane;
        const bool differs = q >= n || !fx_same(keys[q], ks, lb);
        const uint32_t bq = __ballot_sync(0xffffffffu, differs);
        if (bq) {
          g = q0 + (uint32_t)(__ffs(bq) - 1) - s;
          break;
        }
      }
      fx_long_run<K>(keys, vals, sk, sv, s, g, lb, s_cnt[warp]);
    }
  }
}

template <class K>
cudaError_t launch_run_fixup(const Launch& L, K* keys, uint32_t* vals, K* scratch_keys, uint32_t* scratch_vals,
                             uint32_t n, int low_bits) {
  if (n < 2) return cudaSuccess;
  if (low_bits < 1 || low_bits > 32 || low_bits >= (int)(8 * sizeof(K)))
    return cudaErrorInvalidValue;  // run ranks hold 32 low bits, and some high bits must be sorted
  const uint32_t grid = ceil_div(n, (uint32_t)(FX_THREADS * FX_ROWS));
  return launch_kernel(L, run_fixup_kernel<K>, grid, FX_THREADS, 0, keys, vals, scratch_keys, scratch_vals, n,
                       low_bits);
}
template cudaError_t launch_run_fixup<uint32_t>(const Launch&, uint32_t*, uint32_t*, uint32_t*, uint32_t*, uint32_t,
                                                int);
template cudaError_t launch_run_fixup<uint64_t>(const Launch&, uint64_t*, uint32_t*, uint64_t*, uint32_t*, uint32_t,
                                                int);

// ------------------------------------------------------------ onesweep ----
template <class K, int THREADS, int KPT>
struct OnesweepSmem {
  static constexpr int WARPS = THREADS / 32;
  static constexpr int TILE = THREADS * KPT;
  K keys[TILE];
  uint32_t vals[TILE];
  uint32_t warp_hist[WARPS][RADIX];
  uint32_t digit_offset[RADIX];
  uint32_t global_base[RADIX];
  uint32_t warp_sums[8];
  uint32_t tile_id;
};

template <class K, int THREADS, int KPT, bool HAS_VALS, int MINB, int LBW, int RANK, bool L2H = false>
__global__ void __launch_bounds__(THREADS, MINB) onesweep_kernel(const K* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                           K* __restrict__ kout, uint32_t* __restrict__ vout,
                                                           uint32_t n, int shift, uint32_t dmask,
                                                           const uint32_t* __restrict__ bin_off,
                                                           uint32_t* __restrict__ desc,
                                                           uint32_t* __restrict__ tile_counter,
                                                           uint32_t* __restrict__ status,
                                                           const uint32_t* run_if) {
  griddep_wait();
  if (run_if && *run_if == 0) return;
  using S = OnesweepSmem<K, THREADS, KPT>;
  constexpr int WARPS = S::WARPS;
  constexpr int TILE = S::TILE;
  static_assert(THREADS >= RADIX, "one thread per digit");
  static_assert(TILE <= 65536, "warp ranks are packed in 16 bits");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S& s = *reinterpret_cast<S*>(smem_raw);
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;

  for (int i = tid; i < WARPS * RADIX; i += THREADS) (&s.warp_hist[0][0])[i] = 0;
  // RANK 2: three rotating per-warp arrays of digit peer masks live in the
  // key/value staging space, which is free until the scatter; zeroed here.
  constexpr int MATCH_WORDS = 3 * WARPS * RADIX;
  if constexpr (RANK == 2) {
    static_assert(sizeof(s.keys) + sizeof(s.vals) >= MATCH_WORDS * 4, "peer masks fit in the staging space");
    static_assert(offsetof(S, vals) == sizeof(s.keys), "keys and values are contiguous");
    uint4* m4 = reinterpret_cast<uint4*>(s.keys);
    for (int i = tid; i < MATCH_WORDS / 4; i += THREADS) m4[i] = make_uint4(0, 0, 0, 0);
  }
  if (tid == 0) s.tile_id = atomicAdd(tile_counter, 1u);
  // Blocks start in about index order, so the ticket is usually close to
  // this block's index: warm L2 with that tile while the ticket is in flight
  // (a hint only; the tile actually processed is the ticket's).
  {
    const uint32_t guess = blockIdx.x * TILE;
    constexpr uint32_t KL = 128 / sizeof(K), VL = 32;  // elements per 128-byte line
    for (uint32_t e = guess + tid * KL; e < guess + TILE && e < n; e += THREADS * KL) prefetch_l2(kin + e);
    if (HAS_VALS && vin)
      for (uint32_t e = guess + tid * VL; e < guess + TILE && e < n; e += THREADS * VL) prefetch_l2(vin + e);
  }
  __syncthreads();
  const uint32_t tile = s.tile_id;
  // A ticket past the last tile has nothing to sort (tickets start at 0, so
  // only a counter advanced on purpose, gtc_debug_skip_first_tile, gets here).
  if (tile >= (n + TILE - 1) / TILE) return;
  const uint32_t tile_base = tile * TILE;

  // 2. warp-striped coalesced loads.
  K key[KPT];
  uint32_t val[KPT];
  const uint32_t wbase = tile_base + warp * 32 * KPT + lane;
  // L2H: the input is read once (evict first); the output, which the next
  // pass reads, is written evict last so that part of it is still in L2.
  uint64_t pol_in = 0, pol_out = 0;
  if (L2H) {
    pol_in = l2_drop_policy();
    pol_out = l2_keep_policy();
  }
#pragma unroll
  for (int j = 0; j < KPT; ++j) {
    const uint32_t pos = wbase + j * 32;
    // Values absent with HAS_VALS: the iota payload (the first pass of a
    // sort whose values are the input positions).
    if (L2H) {
      key[j] = (pos < n) ? ld_hint(kin + pos, pol_in) : ~K(0);
      if (HAS_VALS) val[j] = (pos < n) ? (vin ? ld_hint(vin + pos, pol_in) : pos) : 0u;
    } else {
      key[j] = (pos < n) ? kin[pos] : ~K(0);
      if (HAS_VALS) val[j] = (pos < n) ? (vin ? vin[pos] : pos) : 0u;
    }
  }

  const uint32_t lt_mask = (1u << lane) - 1u;
  uint32_t* my_hist = s.warp_hist[warp];
  uint32_t rank[KPT];  // RANK 1, 2: rank within the warp's digit run | digit << 16
  if (RANK == 0) {
    // 3. early per-warp digit counts: one shared atomic per key (one per warp
    // when all 32 lanes share the digit, the low-entropy case).
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
      const uint32_t d = (uint32_t)(key[j] >> shift) & dmask;
      const uint32_t d0 = __shfl_sync(0xffffffffu, d, 0);
      if (__all_sync(0xffffffffu, d == d0)) {
        if (lane == 0) atomicAdd(&my_hist[d], 32u);
      } else {
        atomicAdd(&my_hist[d], 1u);
      }
    }
  } else if (RANK == 2) {
    // 3''. counts and warp ranks in one sweep, the peer mask from one shared
    // atomicOr per key instead of 8 ballots: every lane sets its bit in the
    // warp's mask word of its digit, and after __syncwarp the word holds the
    // peer group.  Masks rotate over three arrays: the leader clears the
    // word of key j - 1 after the __syncwarp of key j (every lane has read
    // it by then), and that array is next written for key j + 2, after the
    // __syncwarp of key j + 1.
    uint32_t* mbase = reinterpret_cast<uint32_t*>(s.keys) + warp * RADIX;
    uint32_t prev_d = 0;
    bool prev_lead = false;
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
      uint32_t* mw = mbase + (j % 3) * (WARPS * RADIX);
      const uint32_t d = (uint32_t)(key[j] >> shift) & dmask;
      atomicOr(&mw[d], 1u << lane);
      __syncwarp();
      if (j > 0 && prev_lead) mbase[((j - 1) % 3) * (WARPS * RADIX) + prev_d] = 0;
      const uint32_t peers = mw[d];
      const int leader = 31 - __clz(peers);
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(&my_hist[d], (uint32_t)__popc(peers));
      base = __shfl_sync(0xffffffffu, base, leader);
      rank[j] = (base + __popc(peers & lt_mask)) | (d << 16);
      prev_d = d;
      prev_lead = lane == leader;
    }
  } else {
    // 3'. counts and warp ranks in one sweep: the peer group's leader adds the
    // group's size to the warp's digit counter and gets the group's base back.
    // The scatter waits until the warp offsets are known, so the counter
    // atomics of consecutive keys follow each other without stores between.
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
      const uint32_t d = (uint32_t)(key[j] >> shift) & dmask;
      const uint32_t peers = warp_peers<8>(d);
      const int leader = 31 - __clz(peers);
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(&my_hist[d], (uint32_t)__popc(peers));
      base = __shfl_sync(0xffffffffu, base, leader);
      rank[j] = (base + __popc(peers & lt_mask)) | (d << 16);
    }
  }
  __syncthreads();

  // 4. per-digit counts across warps; publish the tile aggregate; turn the
  // per-warp counts into tile-local start positions.
  uint32_t count = 0;
  if (tid < RADIX) {
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
      const uint32_t c = s.warp_hist[w][tid];
      s.warp_hist[w][tid] = count;
      count += c;
    }
    st_relaxed(desc + (size_t)tile * RADIX + tid, (count << 2) | (tile == 0 ? FLAG_INCLUSIVE : FLAG_AGGREGATE));
  }
  const uint32_t digit_off = scan256_exclusive<THREADS>(count, s.warp_sums);
  if (tid < RADIX) {
    s.digit_offset[tid] = digit_off;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) s.warp_hist[w][tid] += digit_off;
  }
  __syncthreads();

  if (RANK == 0) {
    // 5. stable ranks by warp multisplit (8 __ballot_sync give the peer mask;
    // the highest peer advances the warp's digit cursor and broadcasts the old
    // value) and the scatter into tile-local digit order.
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
      const uint32_t d = (uint32_t)(key[j] >> shift) & dmask;
      const uint32_t peers = warp_peers<8>(d);
      const int leader = 31 - __clz(peers);
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(&my_hist[d], (uint32_t)__popc(peers));
      base = __shfl_sync(0xffffffffu, base, leader);
      const uint32_t local = base + __popc(peers & lt_mask);
      s.keys[local] = key[j];
      if (HAS_VALS) s.vals[local] = val[j];
    }
  } else {
    // 5'. scatter into tile-local digit order.
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
      const uint32_t local = my_hist[rank[j] >> 16] + (rank[j] & 0xffffu);
      s.keys[local] = key[j];
      if (HAS_VALS) s.vals[local] = val[j];
    }
  }

  // 6. decoupled look-back over predecessor tiles, one thread per digit.
  if (tid < RADIX) {
    uint32_t excl = 0;
    if (tile > 0) {
      excl = lookback_window<LBW, RADIX>(desc, tile, tid, status);
      st_relaxed(desc + (size_t)tile * RADIX + tid, ((excl + count) << 2) | FLAG_INCLUSIVE);
    }
    s.global_base[tid] = bin_off[tid] + excl - digit_off;
  }
  __syncthreads();

  // 7. coalesced writes of each digit run.  o < n always holds while every
  // look-back completes; after one ran out (DEV_TIMEOUT) a later pass may see
  // digit counts that disagree with the global histogram, and the check keeps
  // its writes in bounds.
  const uint32_t valid = min((uint32_t)TILE, n - tile_base);
  for (uint32_t i = tid; i < valid; i += THREADS) {
    const K k = s.keys[i];
    const uint32_t o = s.global_base[(uint32_t)(k >> shift) & dmask] + i;
    if (o >= n) continue;
    if (L2H) {
      st_hint(kout + o, k, pol_out);
      if (HAS_VALS) st_hint(vout + o, s.vals[i], pol_out);
    } else {
      kout[o] = k;
      if (HAS_VALS) vout[o] = s.vals[i];
    }
  }
}

// ------------------------------------------- persistent TMA onesweep ------
// The same pass as onesweep_kernel, restructured so HBM never idles:
//   * persistent CTAs (a few per SM) pull tile tickets in a loop;
//   * each CTA double-buffers tiles in shared memory: while it ranks and
//     scatters tile t, a TMA bulk copy (cp.async.bulk + mbarrier) is already
//     streaming the keys and values of its next tile into the other buffer;
//   * ranking: early per-warp digit counts (one shared atomic per peer group
//     from __match_any_sync or 8 ballots), block offsets, then per key a
//     leader atomicAdd on the warp's digit cursor returns the rank base, so
//     consecutive keys carry no register dependency on each other;
//   * the tile aggregate is published before ranking and the look-back is
//     done after the tile is already scattered in shared memory, so
//     predecessors have had the longest time to publish inclusive prefixes.
// Forward progress: a CTA owns at most a current and a prefetched ticket and
// processes its tickets in increasing order; the lowest unfinished tile is
// always some CTA's current tile and only waits on finished tiles.
template <class K, int THREADS, int KPT, bool HV>
struct TmaSmem {
  static constexpr int WARPS = THREADS / 32;
  static constexpr int TILE = THREADS * KPT;
  K keys[2][TILE];
  uint32_t vals[2][HV ? TILE : 4];
  uint32_t cnt[WARPS][RADIX];
  uint32_t digit_off[RADIX];
  uint32_t gbase[RADIX];
  uint32_t warp_sums[8];
  uint32_t next_tile;
  uint32_t pending;
  uint64_t bar[2];
};

template <bool MATCH>
__device__ __forceinline__ uint32_t peer_mask(uint32_t d) {
  if (MATCH) return __match_any_sync(0xffffffffu, d);
  return warp_peers<8>(d);
}

template <class K, int THREADS, int KPT, bool HV, bool MATCH>
__global__ void __launch_bounds__(THREADS, (THREADS <= 256 ? 2 : 1)) onesweep_tma_kernel(const K* __restrict__ kin,
                                                               const uint32_t* __restrict__ vin, K* __restrict__ kout,
                                                               uint32_t* __restrict__ vout, uint32_t n, int shift,
                                                               uint32_t dmask, const uint32_t* __restrict__ bin_off,
                                                               uint32_t* __restrict__ desc,
                                                               uint32_t* __restrict__ tile_counter,
                                                               uint32_t* __restrict__ status,
                                                               const uint32_t* run_if) {
  griddep_wait();
  if (run_if && *run_if == 0) return;
  using S = TmaSmem<K, THREADS, KPT, HV>;
  constexpr int TILE = S::TILE;
  constexpr int WARPS = S::WARPS;
  static_assert(THREADS >= RADIX, "one thread per digit");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S& s = *reinterpret_cast<S*>(smem_raw);
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const uint32_t tiles = (n + TILE - 1) / TILE;
  const uint32_t full_tiles = n / TILE;  // complete tiles come by TMA, a ragged last tile by plain loads

  auto issue = [&](uint32_t t, int b) {  // thread 0 only
    constexpr uint32_t kb = TILE * sizeof(K);
    constexpr uint32_t vb = TILE * 4;
    mbar_arrive_expect_tx(&s.bar[b], kb + (HV ? vb : 0u));
    tma_load_1d(s.keys[b], kin + (size_t)t * TILE, kb, &s.bar[b]);
    if (HV) tma_load_1d(s.vals[b], vin + (size_t)t * TILE, vb, &s.bar[b]);
    s.pending |= 1u << b;
  };

  for (int i = tid; i < WARPS * RADIX; i += THREADS) (&s.cnt[0][0])[i] = 0;
  if (tid == 0) {
    mbar_init(&s.bar[0], 1);
    mbar_init(&s.bar[1], 1);
    fence_mbar_init();
    s.pending = 0;
    const uint32_t t = atomicAdd(tile_counter, 1u);
    s.next_tile = t;
    if (t < full_tiles) issue(t, 0);
  }
  __syncthreads();
  uint32_t tile = s.next_tile;
  int buf = 0;
  uint32_t parity = 0;  // bit b: phase parity to wait for on buffer b

  while (tile < tiles) {
    __syncthreads();  // every thread has read s.next_tile
    if (tid == 0) {
      const uint32_t nt = atomicAdd(tile_counter, 1u);
      s.next_tile = nt;
      if (nt < full_tiles) issue(nt, buf ^ 1);
    }
    const uint32_t base = tile * TILE;
    const uint32_t valid = min((uint32_t)TILE, n - base);
    if (tile < full_tiles) {
      bool ok = mbar_wait_bounded(&s.bar[buf], (parity >> buf) & 1u, status);
      if (__syncthreads_or(!ok)) {
        // A copy that never landed: wait (bounded) for anything still in
        // flight into this CTA's shared memory, then leave; the successors'
        // bounded look-backs report the timeout.
        if (tid == 0) {
          for (int b = 0; b < 2; ++b)
            if (s.pending & (1u << b)) mbar_wait_bounded(&s.bar[b], (parity >> b) & 1u, status);
        }
        __syncthreads();
        return;
      }
      parity ^= 1u << buf;
      if (tid == 0) s.pending &= ~(1u << buf);
    } else {
      for (uint32_t i = tid; i < valid; i += THREADS) {
        s.keys[buf][i] = kin[base + i];
        if (HV) s.vals[buf][i] = vin[base + i];
      }
      __syncthreads();
    }

    // Keys (and values) of this thread, warp-striped from the staged tile.
    K key[KPT];
    uint32_t val[KPT];
    const int sb = warp * 32 * KPT + lane;
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
      const int i = sb + j * 32;
      key[j] = (i < (int)valid) ? s.keys[buf][i] : ~K(0);
      if (HV) val[j] = s.vals[buf][i];
    }
    // A. early per-warp digit counts (shared atomics; one per warp when all
    // lanes share the digit).
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
      const uint32_t d = (uint32_t)(key[j] >> shift) & dmask;
      const uint32_t d0 = __shfl_sync(0xffffffffu, d, 0);
      if (__all_sync(0xffffffffu, d == d0)) {
        if (lane == 0) atomicAdd(&s.cnt[warp][d], 32u);
      } else {
        atomicAdd(&s.cnt[warp][d], 1u);
      }
    }
    __syncthreads();
    // B. per-digit offsets across warps, tile aggregate, tile-local digit bases.
    uint32_t count = 0;
    if (tid < RADIX) {
#pragma unroll
      for (int w = 0; w < WARPS; ++w) {
        const uint32_t c = s.cnt[w][tid];
        s.cnt[w][tid] = count;
        count += c;
      }
      st_relaxed(desc + (size_t)tile * RADIX + tid, (count << 2) | (tile == 0 ? FLAG_INCLUSIVE : FLAG_AGGREGATE));
    }
    const uint32_t doff = scan256_exclusive<THREADS>(count, s.warp_sums);
    if (tid < RADIX) {
      s.digit_off[tid] = doff;
#pragma unroll
      for (int w = 0; w < WARPS; ++w) s.cnt[w][tid] += doff;
    }
    __syncthreads();
    // C. ranks and scatter into the staged buffer (all reads of it are done).
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
      const uint32_t d = (uint32_t)(key[j] >> shift) & dmask;
      const uint32_t peers = peer_mask<MATCH>(d);
      const int leader = 31 - __clz(peers);
      uint32_t b0 = 0;
      if (lane == leader) b0 = atomicAdd(&s.cnt[warp][d], (uint32_t)__popc(peers));
      b0 = __shfl_sync(0xffffffffu, b0, leader);
      const uint32_t pos = b0 + __popc(peers & lt_mask);
      s.keys[buf][pos] = key[j];
      if (HV) s.vals[buf][pos] = val[j];
    }
    // D. decoupled look-back, one thread per digit.
    if (tid < RADIX) {
      uint32_t excl = 0;
      if (tile > 0) {
        excl = lookback_window<8, RADIX>(desc, tile, tid, status);
        st_relaxed(desc + (size_t)tile * RADIX + tid, ((excl + count) << 2) | FLAG_INCLUSIVE);
      }
      s.gbase[tid] = bin_off[tid] + excl - s.digit_off[tid];
    }
    __syncthreads();
    // E. coalesced writes of each digit run.
    for (uint32_t i = tid; i < valid; i += THREADS) {
      const K k = s.keys[buf][i];
      const uint32_t o = s.gbase[(uint32_t)(k >> shift) & dmask] + i;
      if (o >= n) continue;  // only after a timed-out look-back (see onesweep_kernel)
      kout[o] = k;
      if (HV) vout[o] = s.vals[buf][i];
    }
    for (int i = tid; i < WARPS * RADIX; i += THREADS) (&s.cnt[0][0])[i] = 0;
    fence_proxy_async_smem();  // this buffer is refilled by TMA two tiles from now
    __syncthreads();
    tile = s.next_tile;
    buf ^= 1;
  }
}

// ------------------------------------------------------------- variants ---
// Tile shapes compiled in.  kind 0: one tile per CTA (onesweep_kernel);
// kind 1: persistent TMA, __match_any_sync ranks; kind 2: persistent TMA,
// ballot ranks.  The autotuner times them per key width
// (gtc_sort_set_variant); TMA kinds need 16-byte aligned inputs and fall back
// to kind 0 shapes otherwise.
struct Variant {
  int threads;
  int kpt;
  int kind;
  int min_blocks;  // kind 0: __launch_bounds__ minimum CTAs per SM (caps registers: an
                   // explicit 1 lets the compiler spend ~116 registers and run slower)
  int rank;        // kind 0: 0 = per-key early counts, then ballot ranks; 1 = counts and ballot ranks in
                   // one sweep; 2 = counts and ranks in one sweep, peer masks from shared atomicOr
};
constexpr Variant kVariants[] = {{256, 16, 0, 3, 0}, {384, 16, 0, 2, 0}, {512, 12, 0, 2, 0}, {256, 16, 1, 1, 0},
                                 {256, 16, 2, 1, 0}, {512, 8, 2, 1, 0},  {256, 24, 2, 1, 0}, {256, 16, 0, 4, 0},
                                 {512, 8, 0, 2, 0},  {384, 12, 0, 3, 0}, {256, 16, 0, 3, 1}, {384, 16, 0, 2, 1},
                                 {512, 12, 0, 2, 1}, {256, 24, 0, 2, 1}, {256, 16, 4, 3, 0}, {512, 12, 4, 2, 1},
                                 {256, 16, 4, 3, 2}, {512, 12, 4, 2, 2}, {384, 16, 4, 2, 2}};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);
static const int g_variant[2] = {0, 2};  // [u32, u64]: measured best on GB300 without tuning
static std::atomic<int> g_pinned[2] = {{-1}, {-1}};  // gtc_sort_set_variant: overrides the tuned choice

int sort_select_variant(int key_bits, int bits, uint32_t n) {
  const int w = key_bits == 64;
  const int pinned = g_pinned[w].load(std::memory_order_relaxed);
  if (pinned >= 0) return pinned;
  const int t = tuned_variant(key_bits, bits, n);
  return (t >= 0 && t < kNumVariants) ? t : g_variant[w];
}

template <class K, int THREADS, int KPT, bool HV, int MINB, int RANK, bool L2H = false>
static cudaError_t launch_one(const Launch& L, const K* kin, const uint32_t* vin, K* kout, uint32_t* vout,
                              uint32_t n, int shift, uint32_t dmask, const uint32_t* bin_off, uint32_t* desc,
                              uint32_t* tile_counter) {
  using S = OnesweepSmem<K, THREADS, KPT>;
  auto kern = onesweep_kernel<K, THREADS, KPT, HV, MINB, 8, RANK, L2H>;
  cudaError_t e = kernel_setup(kern, THREADS, sizeof(S));
  if (e != cudaSuccess) return e;
  const uint32_t tiles = ceil_div(n, S::TILE);
  return launch_kernel(L, kern, tiles, THREADS, sizeof(S), kin, vin, kout, vout, n, shift, dmask, bin_off, desc,
                       tile_counter, L.status, L.run_if);
}

template <class K, int THREADS, int KPT, bool HV, bool MATCH>
static cudaError_t launch_tma(const Launch& L, const K* kin, const uint32_t* vin, K* kout, uint32_t* vout,
                              uint32_t n, int shift, uint32_t dmask, const uint32_t* bin_off, uint32_t* desc,
                              uint32_t* tile_counter) {
  using S = TmaSmem<K, THREADS, KPT, HV>;
  auto kern = onesweep_tma_kernel<K, THREADS, KPT, HV, MATCH>;
  int per_sm = 1;  // resident CTAs per SM
  cudaError_t e = kernel_setup(kern, THREADS, sizeof(S), &per_sm);
  if (e != cudaSuccess) return e;
  const uint32_t tiles = ceil_div(n, S::TILE);
  const uint32_t grid = min(tiles, (uint32_t)(per_sm * L.num_sms));
  return launch_kernel(L, kern, grid, THREADS, sizeof(S), kin, vin, kout, vout, n, shift, dmask, bin_off, desc,
                       tile_counter, L.status, L.run_if);
}

template <class K>
static cudaError_t launch_variant(int v, bool hv, const Launch& L, const K* kin, const uint32_t* vin, K* kout,
                                  uint32_t* vout, uint32_t n, int shift, uint32_t dmask, const uint32_t* bin_off,
                                  uint32_t* desc, uint32_t* tc) {
  // TMA bulk copies need 16-byte aligned sources; other inputs use the
  // one-tile-per-CTA kernel of the same tile width.
  const bool aligned = (reinterpret_cast<uintptr_t>(kin) & 15) == 0 && (!hv || (reinterpret_cast<uintptr_t>(vin) & 15) == 0);
  if ((kVariants[v].kind == 1 || kVariants[v].kind == 2) && (!aligned || (hv && !vin))) v = 0;
#define GTC_OS(T, P, MB, RK)                                                                                   \
  return hv ? launch_one<K, T, P, true, MB, RK>(L, kin, vin, kout, vout, n, shift, dmask, bin_off, desc, tc) \
            : launch_one<K, T, P, false, MB, RK>(L, kin, vin, kout, vout, n, shift, dmask, bin_off, desc, tc)
#define GTC_OSH(T, P, MB, RK)                                                                                  \
  return hv ? launch_one<K, T, P, true, MB, RK, true>(L, kin, vin, kout, vout, n, shift, dmask, bin_off, desc, tc) \
            : launch_one<K, T, P, false, MB, RK, true>(L, kin, vin, kout, vout, n, shift, dmask, bin_off, desc, tc)
#define GTC_TMA(T, P, M)                                                                                     \
  return hv ? launch_tma<K, T, P, true, M>(L, kin, vin, kout, vout, n, shift, dmask, bin_off, desc, tc)    \
            : launch_tma<K, T, P, false, M>(L, kin, vin, kout, vout, n, shift, dmask, bin_off, desc, tc)
  switch (v) {
    case 0: GTC_OS(256, 16, 3, 0);
    case 1: GTC_OS(384, 16, 2, 0);
    case 2: GTC_OS(512, 12, 2, 0);
    case 3: GTC_TMA(256, 16, true);
    case 4: GTC_TMA(256, 16, false);
    case 5: GTC_TMA(512, 8, false);
    case 6: GTC_TMA(256, 24, false);
    case 7: GTC_OS(256, 16, 4, 0);
    case 8: GTC_OS(512, 8, 2, 0);
    case 9: GTC_OS(384, 12, 3, 0);
    case 10: GTC_OS(256, 16, 3, 1);
    case 11: GTC_OS(384, 16, 2, 1);
    case 12: GTC_OS(512, 12, 2, 1);
    case 13: GTC_OS(256, 24, 2, 1);
    case 14: GTC_OSH(256, 16, 3, 0);
    case 15: GTC_OSH(512, 12, 2, 1);
    case 16: GTC_OSH(256, 16, 3, 2);
    case 17: GTC_OSH(512, 12, 2, 2);
    default: GTC_OSH(384, 16, 2, 2);
  }
#undef GTC_OS
#undef GTC_OSH
#undef GTC_TMA
}

// Smallest tile of any variant: sizes the descriptor array for every variant.
static int min_tile_keys() {
  int t = 1 << 30;
  for (const Variant& v : kVariants) t = t < v.threads * v.kpt ? t : v.threads * v.kpt;
  return t;
}

size_t sort_workspace_bytes(uint32_t n, int passes, int /*tile_keys*/) {
  const uint32_t tiles = ceil_div(n > 0 ? n : 1, (uint32_t)min_tile_keys());
  size_t words = 64 + 2 * (size_t)MAX_PASSES * RADIX;  // header + counts + bin offsets
  words = align_up(words, 64);
  words += (size_t)passes * tiles * RADIX;
  return align_up(words * 4, 256);
}

SortWorkspace carve_sort_workspace(void* ws, uint32_t n, int passes, int /*tile_keys*/) {
  SortWorkspace W;
  uint32_t* p = reinterpret_cast<uint32_t*>(ws);
  W.tiles = ceil_div(n > 0 ? n : 1, (uint32_t)min_tile_keys());
  W.header = p;                              // [0] done, [1..8] tile counters
  W.counts = p + 64;                         // [passes][256]
  W.bin_offsets = p + 64 + MAX_PASSES * RADIX;
  W.header_words = 64 + (size_t)MAX_PASSES * RADIX;  // header + counts zeroed per call
  const size_t desc_off = align_up(64 + 2 * (size_t)MAX_PASSES * RADIX, 64);
  W.desc = p + desc_off;
  W.desc_words = (size_t)passes * W.tiles * RADIX;
  return W;
}

template <class K>
cudaError_t launch_global_hist(const Launch& L, const K* keys, uint32_t n, int begin_bit, int end_bit,
                               const SortWorkspace& W, int passes, int db) {
  if (db < 1 || db > 8 || passes < 1 || passes > MAX_PASSES) return cudaErrorInvalidValue;
  constexpr int T = 512;
  const uint32_t want = ceil_div(n, T * 16);
  const uint32_t grid = max(1u, min(want, (uint32_t)L.num_sms * 2));
  global_hist_kernel<K, T><<<grid, T, 0, L.stream>>>(keys, n, begin_bit, end_bit, passes, db, W.counts,
                                                     W.bin_offsets, W.header, W.desc, W.desc_words, L.run_if);
  return cudaGetLastError();
}
template cudaError_t launch_global_hist<uint32_t>(const Launch&, const uint32_t*, uint32_t, int, int,
                                                  const SortWorkspace&, int, int);
template cudaError_t launch_global_hist<uint64_t>(const Launch&, const uint64_t*, uint32_t, int, int,
                                                  const SortWorkspace&, int, int);

template <class K>
cudaError_t launch_morton_hist(const Launch& L, const float4* pts, K* keys, uint32_t n, float mn, float rg,
                               const SortWorkspace& W, int begin_bit, int passes) {
  constexpr int T = 512;
  constexpr int BITS = 3 * KeyTraits<K>::B;
  if ((begin_bit != 0 && begin_bit != RUN_FIXUP_BITS) || passes != (BITS - begin_bit + 7) / 8)
    return cudaErrorInvalidValue;  // the code from bit 0, or from the run-fixup boundary
  const float inv = pow2_reciprocal(rg);
  const int form = (inv != 0.0f ? 0 : 1) + (begin_bit ? 2 : 0);
  auto kern = form == 0 ? morton_hist_kernel<K, T, 1, 0>
            : form == 1 ? morton_hist_kernel<K, T, 2, 0>
            : form == 2 ? morton_hist_kernel<K, T, 1, RUN_FIXUP_BITS>
                        : morton_hist_kernel<K, T, 2, RUN_FIXUP_BITS>;
  // One resident wave: every block loops over the points.
  int occ = 2;  // blocks per SM
  if (kernel_setup(kern, T, 0, &occ) != cudaSuccess) {
    cudaGetLastError();
    occ = 2;
  }
  const uint32_t want = ceil_div(n, T * 8);
  const uint32_t grid = max(1u, min(want, (uint32_t)(L.num_sms * occ)));
  return launch_kernel(L, kern, grid, T, 0, pts, keys, n, mn, rg, inv, W.counts, W.bin_offsets, W.header, W.desc,
                       W.desc_words);
}
template cudaError_t launch_morton_hist<uint32_t>(const Launch&, const float4*, uint32_t*, uint32_t, float, float,
                                                  const SortWorkspace&, int, int);
template cudaError_t launch_morton_hist<uint64_t>(const Launch&, const float4*, uint64_t*, uint32_t, float, float,
                                                  const SortWorkspace&, int, int);

template <class K>
cudaError_t launch_onesweep_passes(const Launch& L, K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt,
                                   uint32_t n, int begin_bit, int end_bit, const SortWorkspace& W, int passes,
                                   bool* result_in_alt, cudaEvent_t* ev, int variant, bool iota_vals, int db) {
  if (db < 1 || db > 8 || passes < 1 || passes > MAX_PASSES) return cudaErrorInvalidValue;
  const int v = (variant >= 0 && variant < kNumVariants) ? variant
                                                          : sort_select_variant(8 * sizeof(K), end_bit - begin_bit, n);
  const bool hv = vals != nullptr;
  K* src_k = keys;
  K* dst_k = keys_alt;
  uint32_t* src_v = (hv && iota_vals) ? nullptr : vals;  // the first pass makes the iota payload itself
  uint32_t* dst_v = vals_alt;
  for (int p = 0; p < passes; ++p) {
    const int shift = begin_bit + db * p;
    const int bits = min(db, end_bit - shift);
    const uint32_t dmask = (1u << bits) - 1u;
    if (ev) cudaEventRecord(ev[2 * p], L.stream);
    cudaError_t e = launch_variant<K>(v, hv, L, src_k, src_v, dst_k, dst_v, n, shift, dmask, W.bin_offsets + p * RADIX,
                                      W.desc + (size_t)p * W.tiles * RADIX, W.header + 1 + p);
    if (e != cudaSuccess) return e;
    if (ev) cudaEventRecord(ev[2 * p + 1], L.stream);
    K* tk = src_k;
    src_k = dst_k;
    dst_k = tk;
    uint32_t* tv = (p == 0 && hv && iota_vals) ? vals : src_v;
    src_v = dst_v;
    dst_v = tv;
  }
  *result_in_alt = (passes % 2) == 1;
  return cudaSuccess;
}
template cudaError_t launch_onesweep_passes<uint32_t>(const Launch&, uint32_t*, uint32_t*, uint32_t*, uint32_t*,
                                                      uint32_t, int, int, const SortWorkspace&, int, bool*,
                                                      cudaEvent_t*, int, bool, int);
template cudaError_t launch_onesweep_passes<uint64_t>(const Launch&, uint64_t*, uint32_t*, uint64_t*, uint32_t*,
                                                      uint32_t, int, int, const SortWorkspace&, int, bool*,
                                                      cudaEvent_t*, int, bool, int);

// Digit width of a sort: 8 bits, or 7 or 6 where the bit range still fits
// in MAX_PASSES passes.  Pinned per key width (gtc_sort_set_digit_bits), else
// the autotuner's pick for (key width, bits, n), else 8.
static std::atomic<int> g_pinned_db[2] = {{-1}, {-1}};

bool sort_digit_bits_ok(int bits, int db) { return db >= 6 && db <= 8 && (bits + db - 1) / db <= MAX_PASSES; }

int sort_select_digit_bits(int key_bits, int bits, uint32_t n) {
  const int pinned = g_pinned_db[key_bits == 64].load(std::memory_order_relaxed);
  if (pinned > 0 && sort_digit_bits_ok(bits, pinned)) return pinned;
  const int t = tuned_digit_bits(key_bits, bits, n);
  return (t > 0 && sort_digit_bits_ok(bits, t)) ? t : 8;
}

bool sort_set_digit_bits(int key_bits, int db) {
  if (db != -1 && (db < 6 || db > 8)) return false;
  g_pinned_db[key_bits == 64].store(db, std::memory_order_relaxed);
  return true;
}

int sort_max_passes() { return MAX_PASSES; }

int sort_num_variants() { return kNumVariants; }
int sort_get_variant(int key_bits) {
  const int w = key_bits == 64;
  const int pinned = g_pinned[w].load(std::memory_order_relaxed);
  return pinned >= 0 ? pinned : g_variant[w];
}
// v = -1 unpins (back to tuned / default selection).
bool sort_set_variant(int key_bits, int v) {
  if (v < -1 || v >= kNumVariants) return false;
  g_pinned[key_bits == 64].store(v, std::memory_order_relaxed);
  return true;
}
void sort_variant_shape(int v, int* threads, int* kpt) {
  *threads = kVariants[v].threads;
  *kpt = kVariants[v].kpt;
}

}  // namespace gtc
