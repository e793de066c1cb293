// learned.cu - learned-bucket sort of 64-bit keys with a u32 payload.
//
// No counterpart in the reference (its sort is the onesweep of
// new_radix_sort.comp); the output is defined to be exactly the stable
// onesweep result.
//
// Model: a piecewise-linear CDF with B segments (one per bucket).  The B + 1
// knots are u64 keys at quantiles of a 1% sample of a previously sorted key
// set; the B + 1 FP32 heights are trained on the GPU by the forward / backward
// / Adam kernels below (mean squared error against the sample's empirical
// CDF).  bucket(key) = floor(B * F(key)), with F clamped inside each segment
// so that F, and therefore the bucket, is monotone in the key whenever the
// heights are non-decreasing (the update projects them so).
//
// Sort (all stream-ordered, decisions on the device):
//   1. count:   the model bucket of every key, written as a u16 id, and the
//               global bucket histogram;
//   2. scan:    bucket bases; a bucket larger than the on-chip capacity sets
//               the OVERFLOW flag, non-monotone heights BAD_MODEL;
//   3. group:   two stable LSD passes over the bucket-id digits (onesweep
//               style: tile-local ranking, decoupled look-back, coalesced
//               runs of writes) carry keys and values into bucket order, equal
//               keys still in input order;
//   4. bucket sort: one CTA per bucket sorts its segment in shared memory
//               (stable passes over the 16 highest bits that vary inside the
//               bucket, then short groups by insertion) and writes the output;
//   5. check:   consecutive non-empty buckets must hold increasing key ranges
//               (ORDER flag);
//   6. fallback: with any flag set, the input is copied to the output and the
//               plain onesweep kernels (launched unconditionally, gated on the
//               flag word) sort it; otherwise they return at once.

#include <atomic>
#include <cstdio>
#include <new>

#include "gtc_internal.cuh"

namespace gtc {

Launch context_launch(gtc_ctx* ctx, gtc_stream_t stream);
gtc_status context_error(gtc_ctx* ctx, gtc_status s, const char* msg, cudaError_t e);

constexpr uint32_t LFLAG_OVERFLOW = 1u;   // a bucket exceeds the on-chip sort capacity
constexpr uint32_t LFLAG_ORDER = 2u;      // bucket key ranges out of order
constexpr uint32_t LFLAG_BAD_MODEL = 4u;  // heights not non-decreasing

constexpr int LC_THREADS = 1024;  // count kernel: one resident CTA per SM, looping over the keys
constexpr int LC_ILP = 4;          // keys per thread searched at once (independent dependency chains)
constexpr int BS_THREADS = 512;    // in-bucket sort: two CTAs per SM
constexpr int BS_CAP = 8192;       // keys per bucket sorted on chip
constexpr int BS_IPT = BS_CAP / BS_THREADS;
constexpr int kFallbackVariant = 4;  // onesweep variant of the fallback: persistent, TMA-fed
constexpr int MAX_BUCKETS = 16384;  // the count kernel's knots, heights and counters fill one CTA's shared memory

// ---------------------------------------------------------------- model ---
// Bucket line of segment s (knots k0 = kn[s], k1 = kn[s + 1], heights y0 =
// y[s], y1 = y[s + 1]): t(key) = a + c * float(key - k0) clamped to amax, with
// a = B * y0, amax = B * y1, c = B * (y1 - y0) / float(k1 - k0).  Every
// operation is one IEEE round-to-nearest step (no contraction), so the oracle
// (orc_pwl_buckets) evaluates the same function bit for bit.  For
// non-decreasing heights t is non-decreasing in the key: inside a segment
// each rounding step is monotone and c >= 0; at a knot the segment's clamp
// amax equals the next segment's start a.  bucket = floor(t) is therefore
// monotone, which makes bucket key ranges ordered by construction.
__device__ __forceinline__ int pwl_bucket(uint64_t key, uint64_t k0, uint64_t k1, float y0, float y1, int B) {
  const float fb = (float)B;
  const float dy = __fmul_rn(fb, __fsub_rn(y1, y0));
  const float c = (k1 > k0 && dy > 0.0f) ? __fdiv_rn(dy, __ull2float_rn(k1 - k0)) : 0.0f;
  const float t = fminf(__fadd_rn(__fmul_rn(fb, y0), __fmul_rn(c, __ull2float_rn(key - k0))), __fmul_rn(fb, y1));
  return min(__float2int_rz(t), B - 1);
}

// Segment of a key and its interpolation weight (the training forward pass).
__device__ __forceinline__ int model_segment(uint64_t key, const uint64_t* kn, int B, float* w) {
  int lo = 0, hi = B;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (kn[mid] <= key) lo = mid;
    else hi = mid;
  }
  const uint64_t k0 = kn[lo], k1 = kn[lo + 1];
  *w = (k1 > k0) ? __fdiv_rn((float)(key - k0), (float)(k1 - k0)) : 0.0f;
  return lo;
}

__device__ __forceinline__ uint32_t lower_bound_u64(const uint64_t* a, uint32_t n, uint64_t x) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// ------------------------------------------------------------- training ---
__global__ void sample_kernel(const uint64_t* sorted, uint32_t ns, uint32_t stride, uint64_t* sample) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < ns; j += gridDim.x * blockDim.x)
    sample[j] = sorted[(size_t)j * stride];
}

// Knots at the sample's quantiles (fixed); heights initialised to the
// uniform CDF over the key space, y = key / 2^64, i.e. equal-width buckets of
// the key range: the model before training.  Training moves the heights to
// the data's CDF.
__global__ void knots_init_kernel(const uint64_t* sample, uint32_t ns, int B, uint64_t* kn, float* y, float* m1,
                                  float* m2) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b <= B; b += gridDim.x * blockDim.x) {
    uint64_t k;
    if (b == 0) k = 0;
    else if (b == B) k = ~0ull;
    else k = sample[(uint64_t)b * ns / (uint32_t)B];
    kn[b] = k;
    y[b] = (b == B) ? 1.0f : __ull2float_rn(k) * 0x1p-64f;
    m1[b] = 0.0f;
    m2[b] = 0.0f;
  }
}

// Forward: mean squared error of F against t_j = (j + 0.5) / ns.
__global__ void loss_kernel(const uint64_t* sample, uint32_t ns, const uint64_t* kn, const float* y, int B,
                            float* loss) {
  __shared__ float s_part[32];
  float acc = 0.0f;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < ns; j += gridDim.x * blockDim.x) {
    float w;
    const int s = model_segment(sample[j], kn, B, &w);
    const float F = y[s] + (y[s + 1] - y[s]) * w;
    const float r = F - ((float)j + 0.5f) / (float)ns;
    acc += r * r;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = (threadIdx.x < blockDim.x / 32) ? s_part[threadIdx.x] : 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) atomicAdd(loss, v / (float)ns);
  }
}

// Backward: dL/dy_k = (2 / ns) * [sum over segment k of r (1 - w) + sum over
// segment k-1 of r w].  One thread per knot; the sample is sorted, so each
// segment is a contiguous index range found by binary search; sums run in
// index order (deterministic).
__global__ void grad_kernel(const uint64_t* sample, uint32_t ns, const uint64_t* kn, const float* y, int B,
                            float* grad) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k <= B; k += gridDim.x * blockDim.x) {
    float g = 0.0f;
    for (int s = k - 1; s <= k; ++s) {
      if (s < 0 || s >= B) continue;
      const uint32_t a = lower_bound_u64(sample, ns, kn[s]);
      const uint32_t e = (s + 1 == B) ? ns : lower_bound_u64(sample, ns, kn[s + 1]);
      const uint64_t k0 = kn[s], k1 = kn[s + 1];
      const float y0 = y[s], y1 = y[s + 1];
      for (uint32_t j = a; j < e; ++j) {
        const float w = (k1 > k0) ? __fdiv_rn((float)(sample[j] - k0), (float)(k1 - k0)) : 0.0f;
        const float r = y0 + (y1 - y0) * w - ((float)j + 0.5f) / (float)ns;
        g += (s == k) ? r * (1.0f - w) : r * w;
      }
    }
    grad[k] = 2.0f * g / (float)ns;
  }
}

// Adam step on the heights, then projection: y_0 = 0, y_B = 1, clamp to
// [0, 1], running maximum so the heights are non-decreasing.  One block.
__global__ void __launch_bounds__(1024) adam_kernel(float* y, const float* grad, float* m1, float* m2, int B, float lr,
                                                    int step) {
  __shared__ float s_max[1024];
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-12f;
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  const int n = B + 1;
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int first = threadIdx.x * per;
  float run = 0.0f;
  for (int i = first; i < min(first + per, n); ++i) {
    const float g = grad[i];
    const float a = b1 * m1[i] + (1.0f - b1) * g;
    const float v = b2 * m2[i] + (1.0f - b2) * g * g;
    m1[i] = a;
    m2[i] = v;
    float yi = y[i] - lr * (a / c1) / (sqrtf(v / c2) + eps);
    yi = (i == 0) ? 0.0f : (i == B ? 1.0f : fminf(fmaxf(yi, 0.0f), 1.0f));
    run = fmaxf(run, yi);
    y[i] = run;  // running max within the chunk
  }
  s_max[threadIdx.x] = run;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {  // inclusive max-scan of chunk maxima
    const float t = (threadIdx.x >= (unsigned)o) ? s_max[threadIdx.x - o] : 0.0f;
    __syncthreads();
    s_max[threadIdx.x] = fmaxf(s_max[threadIdx.x], t);
    __syncthreads();
  }
  const float before = threadIdx.x > 0 ? s_max[threadIdx.x - 1] : 0.0f;
  for (int i = first; i < min(first + per, n); ++i) y[i] = fmaxf(y[i], before);
}

// --------------------------------------------------------------- sorting --
// Per-key bucket ids are computed once (count pass) and carried as a u16
// payload through two stable LSD passes over their digits, which group the
// keys by bucket with tile-local ranking and coalesced runs of writes (the
// onesweep pass of sort.cu with a third array).  Stable passes keep equal
// keys in input order inside every bucket, so the in-bucket sort needs no
// positions to order them.
// Grouping pass tile shapes (threads x keys per thread), compiled as
// variants: pinned with gtc_learned_set_variant, else the autotuner's pick for
// n (gtc_autotune_learned), else variant 0.
struct LpVariant {
  int threads, kpt;
};
constexpr LpVariant kLpVariants[] = {{256, 16}, {512, 12}, {384, 16}, {512, 8}};
constexpr int kLpNumVariants = sizeof(kLpVariants) / sizeof(kLpVariants[0]);
constexpr int LP_MIN_TILE = 4096;  // smallest tile of any variant: sizes the descriptors
constexpr int LP_RADIX = 128;      // bucket-id digits of at most 7 bits

// 0. model preparation before a sort (one thread per segment): the interior
// knots in Eytzinger order for the count kernel's search, and the
// monotonicity check of the heights.
__global__ void learned_prepare_kernel(const uint64_t* kn, const float* y, int B, uint64_t* eytz, uint32_t* flags) {
  const int d = 31 - __clz(B);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B; i += gridDim.x * blockDim.x) {
    if (flags && !(y[i] <= y[i + 1])) atomicOr(flags, LFLAG_BAD_MODEL);
    if (i > 0) {  // node i of the perfect tree over interior knots 1..B-1
      const int L = 31 - __clz(i);
      const int rank = ((2 * (i - (1 << L)) + 1) << (d - 1 - L)) - 1;  // in-order position
      eytz[i] = kn[rank + 1];
    }
  }
}

// 1. bucket of every key (written as u16 when bids is set) and the bucket
// histogram.  One resident CTA per SM loops over the keys.  Everything the
// model needs sits in shared memory: the interior knots in Eytzinger
// (breadth-first) order, so the lanes of a warp walking down the tree read
// neighbouring words at every level; the B + 1 heights; and the counters.
// The knots are kept as two word arrays: a level compares the high words and
// reads the low word only where they are equal.  The walk also names the
// segment's end knots: in a search tree the last node where the walk turned
// right holds the largest knot <= key (kn[seg]) and the last node where it
// turned left the smallest knot > key (kn[seg + 1]); both are read back off
// the leaf index.  So a key costs no global load beyond itself (the segment
// constants from global memory were one 32-sector L1 request per warp each).
// Each thread walks LC_ILP keys at once to keep several shared-memory loads in
// flight.  The counters are 16-bit halves of 32-bit words (the heights take
// the room): a counter that wraps needs more than 65,535 keys of one bucket
// in one CTA, far above the on-chip capacity, so the CTA flags OVERFLOW (the
// sort falls back), found from the sum of its counters; without a flag word
// (the histogram entry point) it counts its keys again with global atomics.
__device__ __forceinline__ uint64_t knot_at(const uint32_t* s_hi, const uint32_t* s_lo, uint32_t node) {
  return ((uint64_t)s_hi[node] << 32) | s_lo[node];
}

// Bucket of a key whose walk ended at leaf (B <= leaf < 2B).
__device__ __forceinline__ int leaf_bucket(uint64_t key, uint32_t leaf, const uint32_t* s_hi, const uint32_t* s_lo,
                                           const float* s_y, uint64_t kmax, int B) {
  const int seg = (int)leaf - B;
  const uint32_t rn = leaf >> __ffs(leaf);   // last right turn; 0 (slot of kn[0]) when none
  const uint32_t ln = leaf >> __ffs(~leaf);  // last left turn; 0 when none (kn[B])
  const uint64_t k0 = knot_at(s_hi, s_lo, rn);
  const uint64_t k1 = ln ? knot_at(s_hi, s_lo, ln) : kmax;
  return pwl_bucket(key, k0, k1, s_y[seg], s_y[seg + 1], B);
}

__global__ void __launch_bounds__(LC_THREADS, 1) learned_count_kernel(const uint64_t* __restrict__ keys, uint32_t n,
                                                                      const uint64_t* __restrict__ eytz,
                                                                      const uint64_t* __restrict__ kn,
                                                                      const float* __restrict__ y, int B,
                                                                      uint32_t* totals, uint16_t* __restrict__ bids,
                                                                      uint32_t* flags) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t* s_hi = reinterpret_cast<uint32_t*>(smem_raw);
  uint32_t* s_lo = s_hi + B;
  float* s_y = reinterpret_cast<float*>(s_lo + B);                 // [B + 1]
  uint32_t* s_hist = reinterpret_cast<uint32_t*>(s_y + B + 1);     // [B / 2]: counters 2w, 2w + 1
  for (int i = threadIdx.x; i < B; i += LC_THREADS) {
    const uint64_t e = (i > 0) ? eytz[i] : kn[0];  // slot 0 (no tree node): the lowest knot
    s_hi[i] = (uint32_t)(e >> 32);
    s_lo[i] = (uint32_t)e;
    s_y[i] = y[i];
  }
  for (int i = threadIdx.x; i < B / 2; i += LC_THREADS) s_hist[i] = 0;
  if (threadIdx.x == 0) s_y[B] = y[B];
  const uint64_t kmax = kn[B];
  __syncthreads();
  const int levels = 31 - __clz(B);
  const uint32_t step = gridDim.x * LC_THREADS * LC_ILP;
  uint32_t mine = 0;  // keys counted by this thread
  for (uint32_t base = blockIdx.x * LC_THREADS * LC_ILP + threadIdx.x; base < n; base += step) {
    uint64_t k[LC_ILP];
    uint32_t node[LC_ILP];
#pragma unroll
    for (int j = 0; j < LC_ILP; ++j) {
      const uint32_t i = base + j * LC_THREADS;
      k[j] = (i < n) ? __ldcs(keys + i) : 0ull;
      node[j] = 1;
    }
    uint32_t kh[LC_ILP], kl[LC_ILP];
#pragma unroll
    for (int j = 0; j < LC_ILP; ++j) {
      kh[j] = (uint32_t)(k[j] >> 32);
      kl[j] = (uint32_t)k[j];
    }
    for (int l = 0; l < levels; ++l) {
#pragma unroll
      for (int j = 0; j < LC_ILP; ++j) {
        const uint32_t h = s_hi[node[j]];
        // knot <= key: high words decide unless equal
        const bool right = (h != kh[j]) ? (h < kh[j]) : (s_lo[node[j]] <= kl[j]);
        node[j] = 2 * node[j] + (right ? 1u : 0u);
      }
    }
#pragma unroll
    for (int j = 0; j < LC_ILP; ++j) {
      const uint32_t i = base + j * LC_THREADS;
      if (i < n) {
        const int b = leaf_bucket(k[j], node[j], s_hi, s_lo, s_y, kmax, B);
        atomicAdd(&s_hist[b >> 1], 1u << ((b & 1) * 16));
        if (bids) bids[i] = (uint16_t)b;
        ++mine;
      }
    }
  }
  __syncthreads();
  // Flush; a wrapped counter shows as a shortfall of the counters' sum.
  uint32_t sum = 0;
  for (int w = threadIdx.x; w < B / 2; w += LC_THREADS) {
    const uint32_t c = s_hist[w];
    sum += (c & 0xffffu) + (c >> 16);
  }
  __shared__ uint32_t s_short;  // keys counted minus the counters' sum, mod 2^32: 0 unless one wrapped
  if (threadIdx.x == 0) s_short = 0;
  __syncthreads();
  const uint32_t d = __reduce_add_sync(0xffffffffu, mine - sum);
  if ((threadIdx.x & 31) == 0) atomicAdd(&s_short, d);
  __syncthreads();
  if (!s_short) {
    for (int w = threadIdx.x; w < B / 2; w += LC_THREADS) {
      const uint32_t c = s_hist[w];
      if (c & 0xffffu) atomicAdd(totals + 2 * w, c & 0xffffu);
      if (c >> 16) atomicAdd(totals + 2 * w + 1, c >> 16);
    }
    return;
  }
  if (flags) {  // the sort: some bucket holds more than 65,535 keys, far above BS_CAP
    if (threadIdx.x == 0) atomicOr(flags, LFLAG_OVERFLOW);
    return;
  }
  // The histogram entry point: count this CTA's keys again, exactly.
  for (uint32_t base = blockIdx.x * LC_THREADS * LC_ILP + threadIdx.x; base < n; base += step) {
    for (int j = 0; j < LC_ILP; ++j) {
      const uint32_t i = base + j * LC_THREADS;
      if (i >= n) continue;
      const uint64_t key = keys[i];
      const uint32_t kh = (uint32_t)(key >> 32), kl = (uint32_t)key;
      uint32_t nd = 1;
      for (int l = 0; l < levels; ++l) {
        const uint32_t h = s_hi[nd];
        nd = 2 * nd + (((h != kh) ? (h < kh) : (s_lo[nd] <= kl)) ? 1u : 0u);
      }
      atomicAdd(totals + leaf_bucket(key, nd, s_hi, s_lo, s_y, kmax, B), 1u);
    }
  }
}

// 2. one block: bucket bases, the capacity and model checks, and the digit
// bases of the two passes (low db1 bits of the bucket id, then the rest).
__global__ void __launch_bounds__(1024) learned_scan_kernel(const uint32_t* totals, int B, int db1, const float* y,
                                                            uint32_t* base, uint32_t* off1, uint32_t* off2,
                                                            uint32_t* flags) {
  __shared__ uint32_t s_part[1024];
  const int tid = threadIdx.x;
  const int per = (B + 1023) / 1024;
  const int first = tid * per, last = min(first + per, B);
  uint32_t sum = 0;
  bool over = false, bad = false;
  for (int i = first; i < last; ++i) {
    const uint32_t t = totals[i];
    sum += t;
    over |= t > (uint32_t)BS_CAP;
    bad |= y[i] > y[i + 1];
  }
  if (over) atomicOr(flags, LFLAG_OVERFLOW);
  if (bad) atomicOr(flags, LFLAG_BAD_MODEL);
  s_part[tid] = sum;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const uint32_t t = (tid >= o) ? s_part[tid - o] : 0u;
    __syncthreads();
    s_part[tid] += t;
    __syncthreads();
  }
  uint32_t run = tid > 0 ? s_part[tid - 1] : 0u;
  for (int i = first; i < last; ++i) {
    base[i] = run;
    run += totals[i];
  }
  __syncthreads();
  const int r1 = 1 << db1;
  if (tid < r1) {
    uint32_t c = 0;
    for (int b = tid; b < B; b += r1) c += totals[b];
    s_part[tid] = c;
  }
  __syncthreads();
  if (tid < r1) {
    uint32_t pre = 0;
    for (int d = 0; d < tid; ++d) pre += s_part[d];
    off1[tid] = pre;
  }
  if (tid < (B >> db1)) off2[tid] = base[tid << db1];
}

// 3. one stable pass over the bucket-id digit (bid >> shift) & mask.  FIRST:
// the caller's keys and values (values absent: the index) in, bucket ids
// carried out; otherwise the ids are read and dropped.
template <int THREADS, int KPT>
struct LpSmem {
  static constexpr int WARPS = THREADS / 32;
  static constexpr int TILE = THREADS * KPT;
  uint64_t keys[TILE];
  uint32_t vals[TILE];
  uint16_t bids[TILE];
  uint32_t warp_hist[WARPS][LP_RADIX];
  uint32_t gbase[LP_RADIX];
  uint32_t warp_sums[LP_RADIX / 32];
  uint32_t tile_id;
};

template <bool FIRST, int THREADS, int KPT>
__global__ void __launch_bounds__(THREADS) learned_pass_kernel(
    const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin, const uint16_t* __restrict__ bin,
    uint64_t* __restrict__ kout, uint32_t* __restrict__ vout, uint16_t* __restrict__ bout, uint32_t n, int shift,
    uint32_t mask, const uint32_t* __restrict__ bin_off, uint32_t* __restrict__ desc, uint32_t* tile_counter,
    uint32_t* status, const uint32_t* flags) {
  if (*flags & (LFLAG_OVERFLOW | LFLAG_BAD_MODEL)) return;
  using Sm = LpSmem<THREADS, KPT>;
  constexpr int WARPS = Sm::WARPS;
  constexpr int TILE = Sm::TILE;
  static_assert(THREADS >= LP_RADIX, "one thread per digit");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Sm& s = *reinterpret_cast<Sm*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t lt_mask = (1u << lane) - 1u;
  for (int i = tid; i < WARPS * LP_RADIX; i += THREADS) (&s.warp_hist[0][0])[i] = 0;
  if (tid == 0) s.tile_id = atomicAdd(tile_counter, 1u);
  __syncthreads();
  const uint32_t tile = s.tile_id;
  const uint32_t tbase = tile * TILE;

  uint64_t key[KPT];
  uint32_t val[KPT], bd[KPT];
  const uint32_t wbase = tbase + warp * 32 * KPT + lane;
#pragma unroll
  for (int j = 0; j < KPT; ++j) {
    const uint32_t pos = wbase + j * 32;
    const bool ok = pos < n;
    key[j] = ok ? kin[pos] : ~0ull;
    val[j] = ok ? ((FIRST && !vin) ? pos : vin[pos]) : 0u;
    bd[j] = ok ? (uint32_t)bin[pos] : 0xffffu;  // padding ranks last
  }
  uint32_t* my_hist = s.warp_hist[warp];
#pragma unroll
  for (int j = 0; j < KPT; ++j) {
    const uint32_t d = (bd[j] >> shift) & mask;
    const uint32_t d0 = __shfl_sync(0xffffffffu, d, 0);
    if (__all_sync(0xffffffffu, d == d0)) {
      if (lane == 0) atomicAdd(&my_hist[d], 32u);
    } else {
      atomicAdd(&my_hist[d], 1u);
    }
  }
  __syncthreads();
  uint32_t count = 0;
  if (tid < LP_RADIX) {
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
      const uint32_t c = s.warp_hist[w][tid];
      s.warp_hist[w][tid] = count;
      count += c;
    }
    st_relaxed(desc + (size_t)tile * LP_RADIX + tid, (count << 2) | (tile == 0 ? FLAG_INCLUSIVE : FLAG_AGGREGATE));
  }
  uint32_t incl = 0;
  if (tid < LP_RADIX) {
    incl = warp_inclusive_sum(count);
    if (lane == 31) s.warp_sums[warp] = incl;
  }
  __syncthreads();
  uint32_t doff = 0;
  if (tid < LP_RADIX) {
    for (int w = 0; w < LP_RADIX / 32; ++w) doff += (w < warp) ? s.warp_sums[w] : 0u;
    doff += incl - count;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) s.warp_hist[w][tid] += doff;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < KPT; ++j) {
    const uint32_t d = (bd[j] >> shift) & mask;
    const uint32_t peers = warp_peers<7>(d);
    const int leader = 31 - __clz(peers);
    uint32_t b0 = 0;
    if (lane == leader) b0 = atomicAdd(&my_hist[d], (uint32_t)__popc(peers));
    b0 = __shfl_sync(0xffffffffu, b0, leader);
    const uint32_t local = b0 + __popc(peers & lt_mask);
    s.keys[local] = key[j];
    s.vals[local] = val[j];
    s.bids[local] = (uint16_t)bd[j];
  }
  if (tid < LP_RADIX) {
    uint32_t excl = 0;
    if (tile > 0) {
      excl = lookback_window<8, LP_RADIX>(desc, tile, tid, status);
      st_relaxed(desc + (size_t)tile * LP_RADIX + tid, ((excl + count) << 2) | FLAG_INCLUSIVE);
    }
    s.gbase[tid] = bin_off[tid] + excl - doff;
  }
  __syncthreads();
  // o < n while every look-back completes; after one ran out (DEV_TIMEOUT)
  // the second pass may read ids that disagree with the bucket histogram,
  // and the check keeps its writes in bounds.
  const uint32_t valid = min((uint32_t)TILE, n - tbase);
  for (uint32_t i = tid; i < valid; i += THREADS) {
    const uint32_t b = s.bids[i];
    const uint32_t o = s.gbase[(b >> shift) & mask] + i;
    if (o >= n) continue;
    kout[o] = s.keys[i];
    vout[o] = s.vals[i];
    if (FIRST) bout[o] = (uint16_t)b;
  }
}

// 4. in-bucket sort.  One CTA per bucket (two CTAs per SM); the bucket's
// keys arrive grouped and in input order.  Only positions move: idx holds
// each key's offset inside the bucket, and the counting passes read a 32-bit
// sort word per key in shared memory (the 24 highest bits that vary inside
// the bucket), so a pass extracts its digit with one byte select.  The full
// keys stay in global memory (read twice at the start, then cached); the
// output gathers keys and values by the final order.
constexpr int BS_WARPS = BS_THREADS / 32;
constexpr int BS_SORT_BITS = 24;  // bits sorted by counting passes below the highest varying bit
constexpr int BS_RUN_LIMIT = 64;  // longest run of equal sorted bits finished by insertion

struct BucketSmem {
  uint32_t sk[BS_CAP];          // sort words: key bits [lo, lo + 24)
  uint16_t idx[2][BS_CAP];      // positions; the destination array doubles as the ranking's peer masks
  uint32_t cnt[BS_WARPS][128];  // per-warp digit counters / offsets, two 16-bit halves per word
  uint32_t warp_sums[8];
  uint64_t red[2 * BS_WARPS];
  uint32_t skip, big;
};
static_assert(sizeof(uint16_t) * BS_CAP >= sizeof(uint32_t) * 256 * BS_WARPS, "peer masks fit in an index array");

__device__ __forceinline__ uint32_t half16(uint32_t word, uint32_t d) { return (word >> ((d & 1u) * 16u)) & 0xffffu; }

// One stable 8-bit counting pass of idx[cur] into idx[cur ^ 1] (cur flips).
// The digit of the key at offset x is byte `shift / 8` of sk[x], or, with
// gkeys, (gkeys[x] >> shift) & 255 (the rare full passes beyond the sort
// word).  Warp w owns positions [w * 32 * ipt, (w + 1) * 32 * ipt) in
// (j, lane) order.  One sweep gives counts and ranks: every lane sets its bit
// in the warp's peer-mask word of its digit (shared atomicOr, the words kept
// in the destination index array, which is free until the scatter), and the
// highest lane of each peer group adds the group's size to the warp's 16-bit
// digit counter, gets the group's base back and clears the mask word.  The
// block then turns the counters into offsets (digit-major, warp-minor; 16-bit
// halves never carry: every count and offset is below BS_CAP) and a second
// sweep scatters the indices.  A digit shared by every key makes the pass the
// identity: skipped.  Called by every thread of the block.
template <int IPT>
__device__ __forceinline__ void bucket_pass(BucketSmem& s, uint32_t cnt, int ipt, int shift, int& cur,
                                            const uint64_t* gkeys) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const uint32_t wrun = (uint32_t)warp * 32u * (uint32_t)ipt;
  uint32_t* row = s.cnt[warp];
  uint32_t* mw = reinterpret_cast<uint32_t*>(s.idx[cur ^ 1]) + warp * 256;
  for (int i = lane; i < 128; i += 32) row[i] = 0;
  for (int i = lane; i < 256; i += 32) mw[i] = 0;
  __syncwarp();
  const uint32_t sel = 0x4440u + (uint32_t)(shift >> 3);  // byte select of the sort word
  // Per key: rank within the warp's digit run (< 32 * BS_IPT = 512: 9 bits) |
  // digit << 9 | moving index << 17 (< BS_CAP: 13 bits); ~0: no key.
  static_assert(32 * IPT <= 512 && BS_CAP <= 8192, "rank, digit and index pack into 30 bits");
  uint32_t rk[IPT];
#pragma unroll
  for (int j = 0; j < IPT; ++j) {
    rk[j] = 0xffffffffu;
    if (j < ipt && wrun + j * 32 < cnt) {  // warp-uniform
      const uint32_t pos = wrun + j * 32 + lane;
      const bool valid = pos < cnt;
      const uint32_t x = valid ? s.idx[cur][pos] : 0u;
      uint32_t d = 0;
      if (valid) d = gkeys ? (uint32_t)(gkeys[x] >> shift) & 255u : __byte_perm(s.sk[x], 0u, sel);
      if (valid) atomicOr(&mw[d], 1u << lane);
      __syncwarp();
      const uint32_t peers = valid ? mw[d] : 0u;
      __syncwarp();  // every lane has read its mask word before the leaders clear them
      const int leader = valid ? 31 - __clz(peers) : lane;
      uint32_t b0 = 0;
      if (valid && lane == leader) {
        b0 = atomicAdd(&row[d >> 1], (uint32_t)__popc(peers) << ((d & 1u) * 16u));
        mw[d] = 0;
      }
      b0 = half16(__shfl_sync(0xffffffffu, b0, leader), d);
      if (valid) rk[j] = (b0 + __popc(peers & lt_mask)) | (d << 9) | (x << 17);
      __syncwarp();  // the words are clear before the next key's atomicOr
    }
  }
  if (tid == 0) s.skip = 0;
  __syncthreads();
  // Offsets.  Thread t owns the digit pair q = t & 127 (one counter word) for
  // the four warps of quarter t >> 7; quarter sums meet in scratch space of
  // the destination index array, which the scatter overwrites afterwards.
  static_assert(BS_THREADS == 512 && BS_WARPS == 16, "four quarters of four warps");
  const int q = tid & 127, quarter = tid >> 7;
  uint32_t mine[4];
  uint32_t part = 0;
#pragma unroll
  for (int w = 0; w < 4; ++w) {
    mine[w] = part;
    part += s.cnt[quarter * 4 + w][q];
  }
  uint32_t* scratch = reinterpret_cast<uint32_t*>(s.idx[cur ^ 1]);
  scratch[quarter * 128 + q] = part;
  __syncthreads();
  uint32_t t0 = 0, t1 = 0, t2 = 0, pair = 0, incl = 0, lo = 0;
  if (tid < 128) {
    t0 = scratch[q];
    t1 = scratch[128 + q];
    t2 = scratch[256 + q];
    const uint32_t tot = t0 + t1 + t2 + scratch[384 + q];
    lo = tot & 0xffffu;
    const uint32_t hi = tot >> 16;
    if (lo == cnt || hi == cnt) s.skip = 1;
    pair = lo + hi;
    incl = warp_inclusive_sum(pair);
    if (lane == 31) s.warp_sums[warp] = incl;
  }
  __syncthreads();
  if (tid < 128) {
    uint32_t pre = 0;
#pragma unroll
    for (int w = 0; w < 4; ++w) pre += (w < warp) ? s.warp_sums[w] : 0u;
    const uint32_t e = pre + incl - pair;  // base of digit 2q
    const uint32_t base = e | ((e + lo) << 16);
    scratch[q] = base;
    scratch[128 + q] = base + t0;
    scratch[256 + q] = base + t0 + t1;
    scratch[384 + q] = base + t0 + t1 + t2;
  }
  __syncthreads();
  if (s.skip) return;  // block-uniform: every key has the same digit
  {
    const uint32_t qoff = scratch[quarter * 128 + q];
#pragma unroll
    for (int w = 0; w < 4; ++w) s.cnt[quarter * 4 + w][q] = qoff + mine[w];
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < IPT; ++j) {
    if (rk[j] != 0xffffffffu) {
      const uint32_t d = (rk[j] >> 9) & 255u;
      s.idx[cur ^ 1][half16(row[d >> 1], d) + (rk[j] & 511u)] = (uint16_t)(rk[j] >> 17);
    }
  }
  __syncthreads();
  cur ^= 1;
}

// The passes and the run fixup of one bucket (see bucket_sort_kernel), the
// pass loops unrolled for IPT keys per thread.  Returns the index array
// holding the final order.
template <int IPT>
__device__ __forceinline__ int bucket_sort_body(BucketSmem& s, uint32_t cnt, int ipt, int vbits,
                                                const uint64_t* keys) {
  const int tid = threadIdx.x;
  int cur = 0;
  const int np = (min(vbits, BS_SORT_BITS) + 7) / 8;
  for (int p = 0; p < np; ++p) bucket_pass<IPT>(s, cnt, ipt, 8 * p, cur, nullptr);
  if (vbits > BS_SORT_BITS) {
    uint16_t* ix = s.idx[cur];
    // Run starts of a contiguous chunk of ipt positions per thread, found from
    // one batch of independent reads: w[k] is the word at position
    // q0 + k - 1 (the chunk and both neighbours), and bit k of eq says that
    // w[k] equals w[k - 1].  Reads that fall inside another thread's run
    // while it is being reordered still see a word of that run: equal.
    const uint32_t q0 = (uint32_t)tid * (uint32_t)ipt;
    uint32_t starts = 0;
    if (q0 < cnt) {
      const uint32_t len = min((uint32_t)ipt, cnt - q0);
      uint32_t w[IPT + 2];
#pragma unroll
      for (int k = 0; k < IPT + 2; ++k) {
        const uint32_t p = q0 + (uint32_t)k - 1u;  // wraps past 0 for k = 0 of the first chunk
        // sort words are below 2^24: the sentinels equal neither them nor each other
        w[k] = ((uint32_t)k <= len + 1u && p < cnt) ? s.sk[ix[p]] : 0x1000000u + (uint32_t)k;
      }
      uint32_t eq = 0;
#pragma unroll
      for (int k = 1; k < IPT + 2; ++k) eq |= (w[k] == w[k - 1] ? 1u : 0u) << k;
      // position q0 + j starts a run: it equals the next (bit j + 2), not the previous (bit j + 1)
      starts = (eq >> 2) & ~(eq >> 1) & ((1u << len) - 1u);
    }
    while (starts) {
      const uint32_t i = q0 + (uint32_t)(__ffs(starts) - 1);
      starts &= starts - 1u;
      const uint32_t h = s.sk[ix[i]];
      uint32_t e = i + 1;
      while (e < cnt && e - i <= (uint32_t)BS_RUN_LIMIT && s.sk[ix[e]] == h) ++e;
      if (e - i > (uint32_t)BS_RUN_LIMIT) {
        s.big = 1;
        continue;
      }
      for (uint32_t a = i + 1; a < e; ++a) {  // stable: only strictly greater keys move up
        const uint16_t x = ix[a];
        const uint64_t kx = keys[x];
        uint32_t c = a;
        while (c > i && keys[ix[c - 1]] > kx) {
          ix[c] = ix[c - 1];
          --c;
        }
        ix[c] = x;
      }
    }
    __syncthreads();
    if (s.big) {  // block-uniform: start over with full passes over every varying bit
      for (uint32_t i = tid; i < cnt; i += BS_THREADS) s.idx[0][i] = (uint16_t)i;
      cur = 0;
      __syncthreads();
      for (int p = 0; p < (vbits + 7) / 8; ++p) bucket_pass<IPT>(s, cnt, ipt, 8 * p, cur, keys);
    }
  }
  return cur;
}

// One CTA per bucket.  Stable counting passes over the sort word (the 24
// bits below the highest bit that varies inside the bucket; all varying bits
// when there are at most 24), then every run of keys equal in those bits
// (short: measured on the learned workload's keys, the longest runs hold a
// few dozen keys) is finished by a stable insertion sort on the full key.  A
// longer run sends the bucket through full passes over all its varying bits
// instead.
__global__ void __launch_bounds__(BS_THREADS, 2) bucket_sort_kernel(
    const uint64_t* __restrict__ ukeys, const uint32_t* __restrict__ uvals, const uint32_t* base,
    const uint32_t* totals, uint64_t* __restrict__ out_keys, uint32_t* __restrict__ out_vals, uint64_t* bmin,
    uint64_t* bmax, uint32_t* flags) {
  if (*flags & (LFLAG_OVERFLOW | LFLAG_BAD_MODEL)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  BucketSmem& s = *reinterpret_cast<BucketSmem*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int b = blockIdx.x;
  const uint32_t cnt = totals[b];
  const uint32_t off = base[b];
  if (cnt == 0) {
    if (tid == 0) {
      bmin[b] = ~0ull;
      bmax[b] = 0;
    }
    return;
  }
  if (cnt > (uint32_t)BS_CAP) {  // the scan has flagged it already
    if (tid == 0) atomicOr(flags, LFLAG_OVERFLOW);
    return;
  }
  const uint64_t* keys = ukeys + off;
  // The values are read once, gathered by the final order: request their
  // lines into L2 now, so that the gather at the end does not wait on DRAM.
  for (uint32_t i = tid * 32; i < cnt; i += BS_THREADS * 32) prefetch_l2(uvals + off + i);
  if (tid == 0) prefetch_l2(uvals + off + cnt - 1);
  uint64_t mn = ~0ull, mx = 0;
  for (uint32_t i = tid; i < cnt; i += BS_THREADS) {
    const uint64_t k = keys[i];
    mn = min(mn, k);
    mx = max(mx, k);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if (lane == 0) {
    s.red[warp] = mn;
    s.red[BS_WARPS + warp] = mx;
  }
  if (tid == 0) s.big = 0;
  __syncthreads();
  mn = s.red[0];
  mx = s.red[BS_WARPS];
#pragma unroll
  for (int w = 1; w < BS_WARPS; ++w) {
    mn = min(mn, s.red[w]);
    mx = max(mx, s.red[BS_WARPS + w]);
  }
  const int vbits = (mn == mx) ? 0 : 64 - __clzll((long long)(mn ^ mx));
  const int lo = vbits > BS_SORT_BITS ? vbits - BS_SORT_BITS : 0;
  for (uint32_t i = tid; i < cnt; i += BS_THREADS) {  // second read: cached
    s.sk[i] = (uint32_t)(keys[i] >> lo) & 0xffffffu;
    s.idx[0][i] = (uint16_t)i;
  }
  __syncthreads();
  const int ipt = (int)((cnt + BS_THREADS - 1) / BS_THREADS);
  // passes unrolled for the bucket's keys per thread: 8, 12 or 16
  const int cur = ipt <= 8    ? bucket_sort_body<8>(s, cnt, ipt, vbits, keys)
                  : ipt <= 12 ? bucket_sort_body<12>(s, cnt, ipt, vbits, keys)
                              : bucket_sort_body<BS_IPT>(s, cnt, ipt, vbits, keys);
  for (uint32_t i = tid; i < cnt; i += BS_THREADS) {
    const uint16_t x = s.idx[cur][i];
    out_keys[off + i] = keys[x];
    out_vals[off + i] = uvals[off + x];
  }
  if (tid == 0) {
    bmin[b] = mn;
    bmax[b] = mx;
  }
}

// Consecutive non-empty buckets must hold strictly increasing key ranges.
__global__ void learned_order_check_kernel(const uint32_t* totals, const uint64_t* bmin, const uint64_t* bmax, int B,
                                           uint32_t* flags) {
  if (*flags) return;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
    if (totals[b] == 0) continue;
    int nb = b + 1;
    while (nb < B && totals[nb] == 0) ++nb;
    if (nb < B && bmax[b] >= bmin[nb]) atomicOr(flags, LFLAG_ORDER);
  }
}

// Fallback preparation: with any flag set, copy the input to the output.
__global__ void cond_copy_kernel(const uint64_t* keys, const uint32_t* vals, uint64_t* keys_out, uint32_t* vals_out,
                                 uint32_t n, const uint32_t* flags) {
  if (*flags == 0) return;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    keys_out[i] = keys[i];
    vals_out[i] = vals ? vals[i] : (uint32_t)i;
  }
}

// ------------------------------------------------------------ host side --
struct LearnedWorkspace {
  uint32_t* totals;   // [B]
  uint32_t* base;     // [B]
  uint64_t* bmin;     // [B]
  uint64_t* bmax;     // [B]
  uint32_t* misc;     // [1], [2]: pass tile tickets
  uint32_t* off1;     // [128] digit bases of pass 1
  uint32_t* off2;     // [128] digit bases of pass 2
  uint16_t* bid;      // [n] bucket ids
  uint16_t* bid2;     // [n] bucket ids after pass 1
  uint64_t* tkeys;    // [n] after pass 1 (and the fallback's alternate buffer)
  uint32_t* tvals;    // [n]
  uint64_t* ukeys;    // [n] grouped by bucket
  uint32_t* uvals;    // [n]
  uint32_t* desc;     // [2][pass tiles][128]
  size_t desc_words;  // per pass
  void* sort_ws;      // onesweep fallback workspace
};

static size_t learned_ws_layout(uint32_t n, int B, LearnedWorkspace* W, char* p) {
  const uint32_t ptiles = ceil_div(n > 0 ? n : 1, LP_MIN_TILE);
  size_t o = 0;
  auto take = [&](size_t bytes) {
    char* q = p ? p + o : nullptr;
    o += align_up(bytes, 256);
    return q;
  };
  LearnedWorkspace w;
  w.totals = reinterpret_cast<uint32_t*>(take((size_t)B * 4));
  w.base = reinterpret_cast<uint32_t*>(take((size_t)B * 4));
  w.bmin = reinterpret_cast<uint64_t*>(take((size_t)B * 8));
  w.bmax = reinterpret_cast<uint64_t*>(take((size_t)B * 8));
  w.misc = reinterpret_cast<uint32_t*>(take(256));
  w.off1 = reinterpret_cast<uint32_t*>(take(LP_RADIX * 4));
  w.off2 = reinterpret_cast<uint32_t*>(take(LP_RADIX * 4));
  w.bid = reinterpret_cast<uint16_t*>(take((size_t)n * 2));
  w.bid2 = reinterpret_cast<uint16_t*>(take((size_t)n * 2));
  w.tkeys = reinterpret_cast<uint64_t*>(take((size_t)n * 8));
  w.tvals = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
  w.ukeys = reinterpret_cast<uint64_t*>(take((size_t)n * 8));
  w.uvals = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
  w.desc_words = (size_t)ptiles * LP_RADIX;
  w.desc = reinterpret_cast<uint32_t*>(take(2 * w.desc_words * 4));
  w.sort_ws = take(sort_workspace_bytes(n, 8, 0));
  if (W) *W = w;
  return o;
}

size_t learned_workspace_bytes(uint32_t n) { return learned_ws_layout(n, MAX_BUCKETS, nullptr, nullptr); }

}  // namespace gtc

using namespace gtc;

struct gtc_learned_model {
  int B = 0;
  uint64_t* knots = nullptr;   // [B + 1]
  float* heights = nullptr;    // [B + 1]
  uint64_t* eytz = nullptr;    // [B]: interior knots in Eytzinger order (derived before each sort)
  float* m1 = nullptr;         // Adam moments [B + 1]
  float* m2 = nullptr;
  float* grad = nullptr;       // [B + 1]
  float* loss = nullptr;       // [1]
  uint64_t* sample = nullptr;  // training sample
  uint32_t sample_cap = 0;
  uint32_t ns = 0;             // sample size of the last training call
};

namespace {
gtc_status cuda_fail(gtc_ctx* ctx, const char* what, cudaError_t e) {
  return context_error(ctx, e == cudaErrorMemoryAllocation ? GTC_ERR_OOM : GTC_ERR_CUDA, what, e);
}
#define LTRY(ctx, expr)                                  \
  do {                                                   \
    cudaError_t _e = (expr);                             \
    if (_e != cudaSuccess) return cuda_fail(ctx, #expr, _e); \
  } while (0)

// Count kernel: Eytzinger knots (two word arrays of B), the B + 1 heights and
// B 16-bit counters: 14 B + 4 bytes, 229,380 at 2^14 buckets.
size_t count_smem_bytes(int B) { return (size_t)B * 14 + 4; }

// Derives the sort-time model arrays from the knots and heights.
gtc_status prepare_model(gtc_ctx* ctx, const gtc_learned_model* m, uint32_t* d_flags, cudaStream_t s) {
  learned_prepare_kernel<<<ceil_div(m->B, 256), 256, 0, s>>>(m->knots, m->heights, m->B, m->eytz, d_flags);
  LTRY(ctx, cudaGetLastError());
  return GTC_OK;
}

// The count kernel over the keys: one resident CTA per SM.
gtc_status launch_count(gtc_ctx* ctx, const gtc_learned_model* m, const uint64_t* keys, uint32_t n, uint32_t* totals,
                        uint16_t* bids, uint32_t* d_flags, cudaStream_t s) {
  const int B = m->B;
  LTRY(ctx, kernel_setup(learned_count_kernel, LC_THREADS, count_smem_bytes(MAX_BUCKETS)));
  const Launch L = context_launch(ctx, reinterpret_cast<gtc_stream_t>(s));
  const uint32_t grid = max(1u, min((uint32_t)L.num_sms, ceil_div(n, LC_THREADS * LC_ILP)));
  learned_count_kernel<<<grid, LC_THREADS, count_smem_bytes(B), s>>>(keys, n, m->eytz, m->knots, m->heights, B,
                                                                     totals, bids, d_flags);
  LTRY(ctx, cudaGetLastError());
  return GTC_OK;
}

// One grouping pass with the tile shape of variant v.
template <bool FIRST, int THREADS, int KPT>
cudaError_t launch_lp_shape(cudaStream_t s, uint32_t n, const uint64_t* kin, const uint32_t* vin, const uint16_t* bin,
                            uint64_t* kout, uint32_t* vout, uint16_t* bout, int shift, uint32_t mask,
                            const uint32_t* off, uint32_t* desc, uint32_t* tc, uint32_t* status,
                            const uint32_t* flags) {
  using Sm = LpSmem<THREADS, KPT>;
  cudaError_t e = kernel_setup(learned_pass_kernel<FIRST, THREADS, KPT>, THREADS, sizeof(Sm));
  if (e != cudaSuccess) return e;
  learned_pass_kernel<FIRST, THREADS, KPT><<<ceil_div(n, (uint32_t)Sm::TILE), THREADS, sizeof(Sm), s>>>(
      kin, vin, bin, kout, vout, bout, n, shift, mask, off, desc, tc, status, flags);
  return cudaGetLastError();
}

template <bool FIRST>
cudaError_t launch_lp(int v, cudaStream_t s, uint32_t n, const uint64_t* kin, const uint32_t* vin,
                      const uint16_t* bin, uint64_t* kout, uint32_t* vout, uint16_t* bout, int shift, uint32_t mask,
                      const uint32_t* off, uint32_t* desc, uint32_t* tc, uint32_t* status, const uint32_t* flags) {
#define GTC_LP(T, K) \
  return launch_lp_shape<FIRST, T, K>(s, n, kin, vin, bin, kout, vout, bout, shift, mask, off, desc, tc, status, flags)
  switch (v) {
    case 1: GTC_LP(512, 12);
    case 2: GTC_LP(384, 16);
    case 3: GTC_LP(512, 8);
    default: GTC_LP(256, 16);
  }
#undef GTC_LP
}

std::atomic<int> g_lp_pinned{-1};  // gtc_learned_set_variant

gtc_status prepare_sample(gtc_ctx* ctx, gtc_learned_model* m, const uint64_t* sorted, uint32_t n, uint32_t stride,
                          cudaStream_t s) {
  const uint32_t ns = (n + stride - 1) / stride;
  if (ns < (uint32_t)m->B) return context_error(ctx, GTC_ERR_INVALID_ARG, "sample smaller than the bucket count", cudaSuccess);
  if (m->sample_cap < ns) {
    if (m->sample) cudaFree(m->sample);
    m->sample = nullptr;
    m->sample_cap = 0;
    LTRY(ctx, cudaMalloc(&m->sample, (size_t)ns * 8));
    m->sample_cap = ns;
  }
  m->ns = ns;
  sample_kernel<<<min(ceil_div(ns, 256), 4096u), 256, 0, s>>>(sorted, ns, stride, m->sample);
  LTRY(ctx, cudaGetLastError());
  return GTC_OK;
}
}  // namespace

extern "C" {

GTC_API gtc_status gtc_learned_model_create(gtc_ctx* ctx, int buckets, gtc_learned_model** out) {
  if (!ctx || !out) return GTC_ERR_INVALID_ARG;
  *out = nullptr;
  if (buckets < 2 || buckets > MAX_BUCKETS || (buckets & (buckets - 1)))
    return context_error(ctx, GTC_ERR_INVALID_ARG, "buckets must be a power of two in [2, 16384]", cudaSuccess);
  gtc_learned_model* m = new (std::nothrow) gtc_learned_model();
  if (!m) return GTC_ERR_OOM;
  m->B = buckets;
  const size_t nb = (size_t)buckets + 1;
  cudaError_t e = cudaMalloc(&m->knots, nb * 8);
  if (e == cudaSuccess) e = cudaMalloc(&m->heights, nb * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->m1, nb * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->m2, nb * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->grad, nb * 4);
  if (e == cudaSuccess) e = cudaMalloc(&m->loss, 256);
  if (e == cudaSuccess) e = cudaMalloc(&m->eytz, (size_t)buckets * 8);
  if (e != cudaSuccess) {
    gtc_learned_model_destroy(m);
    return cuda_fail(ctx, "allocating the learned model", e);
  }
  *out = m;
  return GTC_OK;
}

GTC_API gtc_status gtc_learned_model_destroy(gtc_learned_model* m) {
  if (!m) return GTC_OK;
  void* ptrs[] = {m->knots, m->heights, m->m1, m->m2, m->grad, m->loss, m->sample, m->eytz};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete m;
  return GTC_OK;
}

GTC_API gtc_status gtc_learned_model_params(gtc_learned_model* m, int* buckets, uint64_t** d_knots, float** d_heights) {
  if (!m) return GTC_ERR_INVALID_ARG;
  if (buckets) *buckets = m->B;
  if (d_knots) *d_knots = m->knots;
  if (d_heights) *d_heights = m->heights;
  return GTC_OK;
}

GTC_API gtc_status gtc_learned_model_export(gtc_learned_model* m, uint64_t* host_knots, float* host_heights) {
  if (!m) return GTC_ERR_INVALID_ARG;
  const size_t nb = (size_t)m->B + 1;
  if (cudaDeviceSynchronize() != cudaSuccess) return GTC_ERR_CUDA;
  if (host_knots && cudaMemcpy(host_knots, m->knots, nb * 8, cudaMemcpyDeviceToHost) != cudaSuccess) return GTC_ERR_CUDA;
  if (host_heights && cudaMemcpy(host_heights, m->heights, nb * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return GTC_ERR_CUDA;
  return GTC_OK;
}

GTC_API gtc_status gtc_learned_train_u64(gtc_ctx* ctx, gtc_learned_model* m, const uint64_t* sorted_keys, uint32_t n,
                                         uint32_t sample_stride, int iters, float lr, float* d_loss,
                                         gtc_stream_t stream) {
  if (!ctx || !m || !sorted_keys || sample_stride == 0 || iters < 0) return GTC_ERR_INVALID_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  gtc_status st = prepare_sample(ctx, m, sorted_keys, n, sample_stride, s);
  if (st != GTC_OK) return st;
  const int B = m->B;
  knots_init_kernel<<<ceil_div(B + 1, 256), 256, 0, s>>>(m->sample, m->ns, B, m->knots, m->heights, m->m1, m->m2);
  LTRY(ctx, cudaGetLastError());
  for (int it = 1; it <= iters; ++it) {
    // learning rate: lr at the first step, decaying exponentially to lr / 10^4 at the last
    const float lr_t = (iters > 1) ? lr * powf(1e-4f, (float)(it - 1) / (float)(iters - 1)) : lr;
    grad_kernel<<<ceil_div(B + 1, 128), 128, 0, s>>>(m->sample, m->ns, m->knots, m->heights, B, m->grad);
    adam_kernel<<<1, 1024, 0, s>>>(m->heights, m->grad, m->m1, m->m2, B, lr_t, it);
  }
  LTRY(ctx, cudaGetLastError());
  LTRY(ctx, cudaMemsetAsync(m->loss, 0, 4, s));
  loss_kernel<<<min(ceil_div(m->ns, 256), 1024u), 256, 0, s>>>(m->sample, m->ns, m->knots, m->heights, B, m->loss);
  LTRY(ctx, cudaGetLastError());
  if (d_loss) LTRY(ctx, cudaMemcpyAsync(d_loss, m->loss, 4, cudaMemcpyDeviceToDevice, s));
  return GTC_OK;
}

GTC_API gtc_status gtc_learned_gradient_u64(gtc_ctx* ctx, gtc_learned_model* m, const uint64_t* sorted_keys, uint32_t n,
                                            uint32_t sample_stride, int init, float* d_grad, float* d_loss,
                                            gtc_stream_t stream) {
  if (!ctx || !m || !sorted_keys || sample_stride == 0 || !d_grad) return GTC_ERR_INVALID_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  gtc_status st = prepare_sample(ctx, m, sorted_keys, n, sample_stride, s);
  if (st != GTC_OK) return st;
  const int B = m->B;
  if (init)
    knots_init_kernel<<<ceil_div(B + 1, 256), 256, 0, s>>>(m->sample, m->ns, B, m->knots, m->heights, m->m1, m->m2);
  grad_kernel<<<ceil_div(B + 1, 128), 128, 0, s>>>(m->sample, m->ns, m->knots, m->heights, B, d_grad);
  if (d_loss) {
    LTRY(ctx, cudaMemsetAsync(d_loss, 0, 4, s));
    loss_kernel<<<min(ceil_div(m->ns, 256), 1024u), 256, 0, s>>>(m->sample, m->ns, m->knots, m->heights, B, d_loss);
  }
  LTRY(ctx, cudaGetLastError());
  return GTC_OK;
}

GTC_API gtc_status gtc_learned_histogram_u64(gtc_ctx* ctx, const gtc_learned_model* m, const uint64_t* keys,
                                             uint32_t n, uint32_t* d_counts, gtc_stream_t stream) {
  if (!ctx || !m || !d_counts || (n && !keys)) return GTC_ERR_INVALID_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int B = m->B;
  LTRY(ctx, cudaMemsetAsync(d_counts, 0, (size_t)B * 4, s));
  if (n == 0) return GTC_OK;
  gtc_status st = prepare_model(ctx, m, nullptr, s);
  if (st != GTC_OK) return st;
  return launch_count(ctx, m, keys, n, d_counts, nullptr, nullptr, s);
}

}  // extern "C"

namespace gtc {
int learned_select_variant(uint32_t n) {
  const int pinned = g_lp_pinned.load(std::memory_order_relaxed);
  if (pinned >= 0) return pinned;
  const int t = tuned_learned_variant(n);
  return (t >= 0 && t < kLpNumVariants) ? t : 0;
}
int learned_num_variants() { return kLpNumVariants; }

// The learned sort with the grouping passes' tile shape given.
gtc_status learned_sort_variant(gtc_ctx* ctx, const gtc_learned_model* m, const uint64_t* keys, const uint32_t* vals,
                                uint64_t* keys_out, uint32_t* vals_out, uint32_t n, void* ws, size_t ws_bytes,
                                uint32_t* d_flags, gtc_stream_t stream, int variant) {
  if (!ctx || !m || !d_flags) return GTC_ERR_INVALID_ARG;
  if (variant < 0 || variant >= kLpNumVariants)
    return context_error(ctx, GTC_ERR_INVALID_ARG, "no such learned variant", cudaSuccess);
  if (n >= (1u << 30)) return context_error(ctx, GTC_ERR_INVALID_ARG, "n must be < 2^30", cudaSuccess);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  LTRY(ctx, cudaMemsetAsync(d_flags, 0, 4, s));
  if (n == 0) return GTC_OK;
  if (!keys || !keys_out || !vals_out)
    return context_error(ctx, GTC_ERR_INVALID_ARG, "keys, keys_out and vals_out are required", cudaSuccess);
  if (keys == keys_out || (vals && vals == vals_out))
    return context_error(ctx, GTC_ERR_INVALID_ARG, "the learned sort is out of place", cudaSuccess);
  const int B = m->B;
  const size_t need = learned_ws_layout(n, B, nullptr, nullptr);
  if (!ws || ws_bytes < need || (reinterpret_cast<uintptr_t>(ws) & 255))
    return context_error(ctx, GTC_ERR_INVALID_ARG, "learned sort workspace missing, too small or unaligned",
                         cudaSuccess);
  LearnedWorkspace W;
  learned_ws_layout(n, B, &W, reinterpret_cast<char*>(ws));
  const int lb = 31 - __builtin_clz((unsigned)B);  // bucket-id bits
  const int db1 = (lb + 1) / 2, db2 = lb - db1;      // digit widths of the two passes (<= 7 each)
  LTRY(ctx, kernel_setup(bucket_sort_kernel, BS_THREADS, sizeof(BucketSmem)));
  const Launch L0 = context_launch(ctx, stream);
  LTRY(ctx, cudaMemsetAsync(W.misc, 0, 256, s));
  LTRY(ctx, cudaMemsetAsync(W.totals, 0, (size_t)B * 4, s));
  LTRY(ctx, cudaMemsetAsync(W.desc, 0, 2 * W.desc_words * 4, s));
  gtc_status st = prepare_model(ctx, m, d_flags, s);
  if (st == GTC_OK) st = launch_count(ctx, m, keys, n, W.totals, W.bid, d_flags, s);
  if (st != GTC_OK) return st;
  learned_scan_kernel<<<1, 1024, 0, s>>>(W.totals, B, db1, m->heights, W.base, W.off1, W.off2, d_flags);
  LTRY(ctx, cudaGetLastError());
  LTRY(ctx, launch_lp<true>(variant, s, n, keys, vals, W.bid, db2 ? W.tkeys : W.ukeys, db2 ? W.tvals : W.uvals,
                            W.bid2, 0, (1u << db1) - 1, W.off1, W.desc, W.misc + 1, L0.status, d_flags));
  if (db2)
    LTRY(ctx, launch_lp<false>(variant, s, n, W.tkeys, W.tvals, W.bid2, W.ukeys, W.uvals, nullptr, db1,
                               (1u << db2) - 1, W.off2, W.desc + W.desc_words, W.misc + 2, L0.status, d_flags));
  bucket_sort_kernel<<<B, BS_THREADS, sizeof(BucketSmem), s>>>(W.ukeys, W.uvals, W.base, W.totals, keys_out, vals_out,
                                                               W.bmin, W.bmax, d_flags);
  learned_order_check_kernel<<<ceil_div(B, 256), 256, 0, s>>>(W.totals, W.bmin, W.bmax, B, d_flags);
  LTRY(ctx, cudaGetLastError());
  // Fallback: copy + plain onesweep, all gated on the flag word.
  cond_copy_kernel<<<L0.num_sms * 4, 256, 0, s>>>(keys, vals, keys_out, vals_out, n, d_flags);
  Launch L = L0;
  L.run_if = d_flags;
  const SortWorkspace SW = carve_sort_workspace(W.sort_ws, n, 8, 0);
  LTRY(ctx, cudaMemsetAsync(SW.header, 0, SW.header_words * 4, s));
  LTRY(ctx, launch_global_hist<uint64_t>(L, keys_out, n, 0, 64, SW, 8));
  bool in_alt = false;
  // Variant 4 is a persistent kernel (one resident wave of CTAs pulling
  // tiles): when the learned path succeeded, each gated pass costs one wave
  // of CTAs that read the flag word and exit, not one CTA per tile.
  LTRY(ctx, launch_onesweep_passes<uint64_t>(L, keys_out, vals_out, W.tkeys, W.tvals, n, 0, 64, SW, 8, &in_alt,
                                             nullptr, kFallbackVariant));
  return GTC_OK;
}
}  // namespace gtc

extern "C" {

GTC_API gtc_status gtc_learned_sort_u64(gtc_ctx* ctx, const gtc_learned_model* m, const uint64_t* keys,
                                        const uint32_t* vals, uint64_t* keys_out, uint32_t* vals_out, uint32_t n,
                                        void* ws, size_t ws_bytes, uint32_t* d_flags, gtc_stream_t stream) {
  return learned_sort_variant(ctx, m, keys, vals, keys_out, vals_out, n, ws, ws_bytes, d_flags, stream,
                              learned_select_variant(n));
}

GTC_API int gtc_learned_num_variants(void) { return kLpNumVariants; }

GTC_API gtc_status gtc_learned_variant_shape(int variant, int* threads, int* keys_per_thread) {
  if (variant < 0 || variant >= kLpNumVariants) return GTC_ERR_INVALID_ARG;
  if (threads) *threads = kLpVariants[variant].threads;
  if (keys_per_thread) *keys_per_thread = kLpVariants[variant].kpt;
  return GTC_OK;
}

GTC_API gtc_status gtc_learned_set_variant(int variant) {
  if (variant < -1 || variant >= kLpNumVariants) return GTC_ERR_INVALID_ARG;
  g_lp_pinned.store(variant, std::memory_order_relaxed);
  return GTC_OK;
}

GTC_API int gtc_learned_get_variant(uint32_t n) { return learned_select_variant(n); }

}  // extern "C"
