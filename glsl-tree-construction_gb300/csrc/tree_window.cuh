// tree_window.cuh - the Karras radix tree built per split from a shared-memory
// window of adjacent-key prefix lengths (single cloud and batched clouds).
//
// Same output as build_radix_tree.comp:71-144 with D1/D16 (and the edge count
// of edge_count.comp:30-41), computed another way.  With d[x] = δ(code_x,
// code_{x+1}) for the m = u - 1 adjacent pairs, the internal node whose split
// is x covers the keys [L + 1, R], where L < x and R > x are the nearest pair
// positions with d < d[x] (or the ends of the cloud); its prefix length is
// d[x]; its parent's split is whichever of L and R has the larger d (the two
// never tie for distinct keys), and it is stored at Karras index R when it is
// that parent's left child, L + 1 when it is the right child, 0 for the root.
// So the whole tree is an all-nearest-smaller-values problem over d.
//
// One block handles T consecutive splits.  It loads d over the splits plus a
// halo of H positions on each side into shared memory (positions outside the
// key array, and pairs that straddle two clouds, read as 0: smaller than any
// real prefix length), then answers the nearest-smaller queries in three
// tiers, none of which loops over a node's range:
//   1. every lane answers the queries inside its own chunk of 16 splits
//      with byte-parallel compares (the same work on every lane); about 80% of the answers are inside the
//      chunk;
//   2. the rest are found through two threshold tables: for every value v,
//      which of a warp-block's 32 chunks has a minimum below v, and which of
//      the window's 20 warp-blocks does - a few bit operations name the
//      first chunk holding a smaller value, and one 16-byte SIMD compare
//      finds the position inside it;
//   3. a split whose range reaches past the halo (0.04% of the splits of the
//      10M clustered cloud) is kept in a block-local queue and resolved at
//      the end of the block by a warp that searches the codes cooperatively,
//      both range ends together, 32 probes per end per round; splits beyond
//      the local queue's capacity go to radix_tree_slow_kernel, which does
//      the same.
#pragma once

#include "gtc_internal.cuh"

namespace gtc {

constexpr int TW_THREADS = 512;
constexpr int TW_C = 16;                   // splits per chunk (one lane's in-chunk pass)
constexpr int TW_T = TW_THREADS * TW_C;    // 8192 splits per block
constexpr int TW_H = 1024;                 // halo on each side
constexpr int TW_W = TW_T + 2 * TW_H;      // 10240 window positions
constexpr int TW_NCH = TW_W / TW_C;        // 640 chunks
constexpr int TW_NWB = TW_NCH / 32;        // 20 warp-blocks of 32 chunks
constexpr int TW_TV = 64;                  // prefix lengths are < 64
constexpr int TW_MAXB = 512;               // cloud starts cached per window (batched)
constexpr int TW_LQ = 128;                 // long-range splits a block resolves itself
static_assert(TW_H % (32 * TW_C) == 0, "the tile starts on a warp-block");
static_assert(TW_NWB <= 32, "one ballot covers the window's warp-blocks");

// First index in a[0..n) with a[i] > x.
__device__ __forceinline__ uint32_t upper_bound_u32(const uint32_t* a, uint32_t n, uint32_t x) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a[mid] <= x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// The cloud that owns position x of a run of offsets off[0..S] (off[S] > x):
// the last c with off[c] <= x, which skips empty clouds.
__device__ __forceinline__ uint32_t owner(const uint32_t* off, uint32_t S, uint32_t x) {
  return upper_bound_u32(off, S + 1, x) - 1;
}

struct TwSmem {
  alignas(16) uint8_t d[TW_W];   // prefix length of pair w0 + i (0 = boundary)
  alignas(16) uint8_t lr[TW_T];  // per split: (left answer in chunk << 4) | right answer in chunk
  uint8_t cmin[TW_NCH];          // chunk minima
  uint32_t t4[TW_NWB][TW_TV];    // t4[b][v] bit k: chunk 32b + k has a value < v
  uint32_t t9[TW_TV];            // t9[v] bit b: warp-block b has a value < v
  uint32_t cb[TW_MAXB];          // batched: cloud starts from c_first on
  uint32_t lq[TW_LQ];            // this block's splits whose range reaches past the window
  uint32_t c_first, nb, lq_n;
};

// Bytes of a word below t (prefix lengths < 128): bit 7 of each byte of
// (w | 0x80) - t is clear exactly where the byte is below t.
__device__ __forceinline__ uint32_t tw_below(uint32_t w, uint32_t tt) {
  return ~((w | 0x80808080u) - tt) & 0x80808080u;
}

// Nearest smaller values inside this lane's chunk of 16 prefix lengths,
// without a stack (a stack pass pops a data-dependent number of entries per
// step, which diverges across the warp).  The chunk is transposed so that
// word k holds positions k, k + 4, k + 8, k + 12; position p = 4b + k then
// sits at bit 8b + k of a 32-bit mask, and bit order follows position
// order.  Four tw_below give the mask of every position below d[j], and the
// nearest on each side is a bit scan.  Result per split, one byte: left
// answer in the chunk (15 = none) << 4 | right answer (0 = none).  Equal
// lengths never face each other across larger ones for distinct keys, so
// strictly smaller and smaller-or-equal give the same answers; boundaries
// (0) have no answers of their own and are never queried.
__device__ __forceinline__ void tw_chunk_stack(TwSmem& s, int chunk) {
  const uint4 dv = *reinterpret_cast<const uint4*>(s.d + TW_H + chunk * TW_C);
  const uint32_t a01 = __byte_perm(dv.x, dv.y, 0x5140), a23 = __byte_perm(dv.z, dv.w, 0x5140);
  const uint32_t c01 = __byte_perm(dv.x, dv.y, 0x7362), c23 = __byte_perm(dv.z, dv.w, 0x7362);
  const uint32_t wt[4] = {__byte_perm(a01, a23, 0x5410), __byte_perm(a01, a23, 0x7632), __byte_perm(c01, c23, 0x5410),
                          __byte_perm(c01, c23, 0x7632)};
  const uint32_t dw[4] = {dv.x, dv.y, dv.z, dv.w};
  uint32_t out[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    uint32_t o = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int bj = 8 * q + b;  // bit of position 4q + b
      const uint32_t tt = ((dw[q] >> (8 * b)) & 0xffu) * 0x01010101u;
      uint32_t m = 0;  // bit 8b' + k: d[4b' + k] < d[4q + b]
#pragma unroll
      for (int k = 0; k < 4; ++k) m |= tw_below(wt[k], tt) >> (7 - k);
      const uint32_t lm = m & ((1u << bj) - 1u);
      const uint32_t rm = m & ~((2u << bj) - 1u);
      const uint32_t lb = 31 - __clz(lm), rb = __ffs(rm) - 1;
      const uint32_t l = lm ? 4 * (lb >> 3) + (lb & 7) : 15u;
      const uint32_t r = rm ? 4 * (rb >> 3) + (rb & 7) : 0u;
      o |= ((l << 4) | r) << (8 * b);
    }
    out[q] = o;
  }
  *reinterpret_cast<uint4*>(s.lr + chunk * TW_C) = make_uint4(out[0], out[1], out[2], out[3]);
}

// Inclusive prefix OR over a 64-row table, rows lane and lane + 32 per lane.
__device__ __forceinline__ void tw_prefix_or_rows(uint32_t* rows, int lane) {
  uint32_t a = rows[lane], b = rows[lane + 32];
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t pa = __shfl_up_sync(0xffffffffu, a, o), pb = __shfl_up_sync(0xffffffffu, b, o);
    if (lane >= o) {
      a |= pa;
      b |= pb;
    }
  }
  b |= __shfl_sync(0xffffffffu, a, 31);
  rows[lane] = a;
  rows[lane + 32] = b;
}

// First / last byte of a 16-byte chunk below t (one exists).
__device__ __forceinline__ int tw_first_below(const uint8_t* p, uint32_t t) {
  const uint4 q = *reinterpret_cast<const uint4*>(p);
  const uint32_t tt = t * 0x01010101u;
  uint32_t c;
  int base;
  if ((c = tw_below(q.x, tt))) base = 0;
  else if ((c = tw_below(q.y, tt))) base = 4;
  else if ((c = tw_below(q.z, tt))) base = 8;
  else {
    c = tw_below(q.w, tt);
    base = 12;
  }
  return base + ((__ffs(c) - 1) >> 3);
}
__device__ __forceinline__ int tw_last_below(const uint8_t* p, uint32_t t) {
  const uint4 q = *reinterpret_cast<const uint4*>(p);
  const uint32_t tt = t * 0x01010101u;
  uint32_t c;
  int base;
  if ((c = tw_below(q.w, tt))) base = 12;
  else if ((c = tw_below(q.z, tt))) base = 8;
  else if ((c = tw_below(q.y, tt))) base = 4;
  else {
    c = tw_below(q.x, tt);
    base = 0;
  }
  return base + ((31 - __clz(c)) >> 3);
}

// First window position after chunk c with a value < t, or -1.
__device__ __forceinline__ int tw_next_tab(const TwSmem& s, int c, uint32_t t) {
  const int b = c >> 5, k = c & 31;
  const uint32_t m = s.t4[b][t] & ~((2u << k) - 1u);
  int cc;
  if (m) {
    cc = (b << 5) + __ffs(m) - 1;
  } else {
    const uint32_t m9 = s.t9[t] & ~((2u << b) - 1u);
    if (!m9) return -1;
    const int b2 = __ffs(m9) - 1;
    cc = (b2 << 5) + __ffs(s.t4[b2][t]) - 1;
  }
  return cc * TW_C + tw_first_below(s.d + cc * TW_C, t);
}

// Last window position before chunk c with a value < t, or -1.
__device__ __forceinline__ int tw_prev_tab(const TwSmem& s, int c, uint32_t t) {
  const int b = c >> 5, k = c & 31;
  const uint32_t m = s.t4[b][t] & ((1u << k) - 1u);
  int cc;
  if (m) {
    cc = (b << 5) + 31 - __clz(m);
  } else {
    const uint32_t m9 = s.t9[t] & ((1u << b) - 1u);
    if (!m9) return -1;
    const int b2 = 31 - __clz(m9);
    cc = (b2 << 5) + 31 - __clz(s.t4[b2][t]);
  }
  return cc * TW_C + tw_last_below(s.d + cc * TW_C, t);
}

// Global fallbacks.  Largest y in [x + 1, last] with δ(code_x, code_y) >= t,
// and smallest y in [first, x] with δ(code_{x+1}, code_y) >= t (δ of a key
// with keys further away never increases, so both are monotone searches).
// Single-thread forms (stage API, no queue) and a warp-cooperative form.

// Both range ends of split x (prefix length t) in the cloud [first, last]
// by the whole warp: the largest hi in [x + 1, last] with δ(code_x, code_hi)
// >= t and the smallest lo in [first, x] with δ(code_{x+1}, code_lo) >= t.
// Each side is a monotone predicate over an offset o >= 1 that holds at o = 1.
// Every lane probes one offset of each side per round (the two loads in
// flight together): exponentially spaced offsets first, then 32 equal steps
// of each remaining interval, so a range of 2^20 keys takes 5 dependent
// rounds for both ends.  Every lane of the warp calls it with the same x.
template <class K>
__device__ __forceinline__ uint2 tw_warp_range(const K* codes, uint32_t x, uint32_t first, uint32_t last, int t) {
  const int lane = threadIdx.x & 31;
  const K cx = codes[x], c1 = codes[x + 1];
  const uint32_t lim_r = last - x, lim_l = x + 1 - first;  // offsets available on each side
  auto good_r = [&](uint64_t o) -> bool { return o >= 1 && o <= lim_r && delta_key(cx, codes[x + o]) >= t; };
  auto good_l = [&](uint64_t o) -> bool {
    return o >= 1 && o <= lim_l && delta_key(c1, codes[(uint64_t)x + 1 - o]) >= t;
  };
  bool pr = false, pl = false;
  if (lane < 31) {
    pr = good_r(1ull << lane);
    pl = good_l(1ull << lane);
  }
  const uint32_t er = __ballot_sync(0xffffffffu, pr), el = __ballot_sync(0xffffffffu, pl);
  const int kr = 31 - __clz(er | 1u), kl = 31 - __clz(el | 1u);  // o = 1 always holds
  uint64_t lo_r = 1ull << kr, hi_r = min((uint64_t)(1ull << (kr + 1)), (uint64_t)lim_r + 1);
  uint64_t lo_l = 1ull << kl, hi_l = min((uint64_t)(1ull << (kl + 1)), (uint64_t)lim_l + 1);
  while (hi_r - lo_r > 1 || hi_l - lo_l > 1) {  // warp-uniform
    const uint64_t sr = (hi_r - lo_r + 31) / 32, sl = (hi_l - lo_l + 31) / 32;
    const uint64_t qr = lo_r + (uint64_t)(lane + 1) * sr, ql = lo_l + (uint64_t)(lane + 1) * sl;
    const bool gr = hi_r - lo_r > 1 && qr < hi_r && good_r(qr);
    const bool gl = hi_l - lo_l > 1 && ql < hi_l && good_l(ql);
    const uint32_t br = __ballot_sync(0xffffffffu, gr), bl = __ballot_sync(0xffffffffu, gl);
    if (hi_r - lo_r > 1) {
      const uint64_t n = br ? lo_r + (uint64_t)(32 - __clz(br)) * sr : lo_r;
      hi_r = min(n + sr, hi_r);
      lo_r = n;
    }
    if (hi_l - lo_l > 1) {
      const uint64_t n = bl ? lo_l + (uint64_t)(32 - __clz(bl)) * sl : lo_l;
      hi_l = min(n + sl, hi_l);
      lo_l = n;
    }
  }
  return make_uint2(x + 1 - (uint32_t)lo_l, x + (uint32_t)lo_r);
}

template <class K>
__device__ __forceinline__ uint32_t tw_range_hi(const K* codes, uint32_t x, uint32_t last, int t) {
  const K cx = codes[x];
  const uint32_t lim = last - x;
  uint32_t stp = 2;
  while (stp <= lim && delta_key(cx, codes[x + stp]) >= t) stp <<= 1;
  uint32_t l = stp >> 1;
  for (uint32_t b = stp >> 2; b >= 1; b >>= 1)
    if (l + b <= lim && delta_key(cx, codes[x + l + b]) >= t) l += b;
  return x + l;
}
template <class K>
__device__ __forceinline__ uint32_t tw_range_lo(const K* codes, uint32_t x, uint32_t first, int t) {
  const K c1 = codes[x + 1];
  const uint32_t lim = x + 1 - first;
  uint32_t stp = 2;
  while (stp <= lim && delta_key(c1, codes[x + 1 - stp]) >= t) stp <<= 1;
  uint32_t l = stp >> 1;
  for (uint32_t b = stp >> 2; b >= 1; b >>= 1)
    if (l + b <= lim && delta_key(c1, codes[x + 1 - (l + b)]) >= t) l += b;
  return x + 1 - l;
}

// The outputs of the node whose split is x (prefix length t) covering keys
// [lo, hi] of the cloud starting at U0, with dL / dR the prefix lengths at
// lo - 1 and hi (0 at a cloud end).
template <int A>
__device__ __forceinline__ void tw_emit(uint32_t x, uint32_t t, uint32_t lo, uint32_t hi, uint32_t dL, uint32_t dR,
                                        uint32_t U0, uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr, int32_t* left,
                                        int32_t* parent, uint32_t* edge) {
  uint32_t idx;
  uint32_t e = 0;
  if (dL == 0 && dR == 0) {
    idx = U0;  // the root of this cloud (D13: its parent reads 0)
    parent[idx] = 0;
  } else {
    idx = dR > dL ? hi : lo;  // left child of the split at hi, or right child of the split at lo - 1
    e = (t - A) / 3 - (max(dL, dR) - A) / 3;
  }
  if (edge) edge[idx] = e;
  prefix_n[idx] = (uint8_t)t;
  left[idx] = (int32_t)(x - U0);
  hll[idx] = lo == x;
  hlr[idx] = hi == x + 1;
  if (lo != x) parent[x] = (int32_t)(idx - U0);
  if (hi != x + 1) parent[x + 1] = (int32_t)(idx - U0);
}

// One split's node found by tw_warp_range (called by a whole warp; lane 0
// stores), cloud [U0, U1).
template <class K>
__device__ __forceinline__ void tw_warp_split(const K* codes, uint32_t x, uint32_t U0, uint32_t U1,
                                              uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr, int32_t* left,
                                              int32_t* parent, uint32_t* edge) {
  constexpr int A = KeyTraits<K>::A;
  const int t = delta_key(codes[x], codes[x + 1]);
  const uint2 r = tw_warp_range<K>(codes, x, U0, U1 - 1, t);
  if ((threadIdx.x & 31) == 0) {
    const uint32_t lo = r.x, hi = r.y;
    const uint32_t dR = (hi + 1 < U1) ? (uint32_t)delta_key(codes[hi], codes[hi + 1]) : 0u;
    const uint32_t dL = (lo > U0) ? (uint32_t)delta_key(codes[lo - 1], codes[lo]) : 0u;
    tw_emit<A>(x, (uint32_t)t, lo, hi, dL, dR, U0, prefix_n, hll, hlr, left, parent, edge);
  }
}

// One block: splits [blockIdx.x * T, + T).  SEG: clouds of codes start at
// uoff[0..S] (uoff[S] = U), indices written are cloud-local, and the last
// slot of every cloud gets edge 0.  Otherwise one cloud of U codes.  With a
// queue (capacity: one entry per split), splits whose range reaches past
// the halo are appended to it for radix_tree_slow_kernel; without one they
// are searched here by their own thread.
template <class K, bool SEG>
__global__ void __launch_bounds__(TW_THREADS, 4) radix_tree_window_kernel(
    const K* __restrict__ codes, const uint32_t* d_u, uint32_t u_host, const uint32_t* uoff, uint32_t S,
    uint8_t* __restrict__ prefix_n, uint8_t* __restrict__ hll, uint8_t* __restrict__ hlr,
    int32_t* __restrict__ left, int32_t* __restrict__ parent, uint32_t* __restrict__ edge, uint32_t* d_m,
    uint32_t* queue, uint32_t* q_count) {
  griddep_wait();
  constexpr int A = KeyTraits<K>::A;
  __shared__ TwSmem s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t U = SEG ? uoff[S] : (d_u ? *d_u : u_host);
  const uint32_t P = U > 0 ? U - 1 : 0;  // pair positions [0, P)
  if (!SEG && blockIdx.x == 0 && tid == 0 && d_m) *d_m = P;
  // Positions fit in int: U < 2^30, and the window starts at most H before 0.
  const int t0 = (int)blockIdx.x * TW_T;
  const int x_end = min(t0 + TW_T, (int)(SEG ? U : P));
  if (t0 >= x_end) return;
  const int w0 = t0 - TW_H;
  if (tid == 0) s.lq_n = 0;

  // 1. prefix lengths of the window's pairs.
  // Four adjacent pairs per thread and step: five codes (two 16-byte loads
  // and one more) give four lengths, stored as one word.
  const bool vec = (reinterpret_cast<uintptr_t>(codes) & 15) == 0;
#pragma unroll
  for (int g = tid; g < TW_W / 4; g += TW_THREADS) {
    const int x = w0 + 4 * g;
    uint32_t v = 0;
    if (vec && x >= 0 && x + 4 <= (int)P) {
      K c[5];
      if (sizeof(K) == 8) {
        const uint4 q0 = __ldg(reinterpret_cast<const uint4*>(codes + x));
        const uint4 q1 = __ldg(reinterpret_cast<const uint4*>(codes + x + 2));
        c[0] = (K)(q0.x | ((uint64_t)q0.y << 32));
        c[1] = (K)(q0.z | ((uint64_t)q0.w << 32));
        c[2] = (K)(q1.x | ((uint64_t)q1.y << 32));
        c[3] = (K)(q1.z | ((uint64_t)q1.w << 32));
      } else {
        const uint4 q0 = __ldg(reinterpret_cast<const uint4*>(codes + x));
        c[0] = (K)q0.x;
        c[1] = (K)q0.y;
        c[2] = (K)q0.z;
        c[3] = (K)q0.w;
      }
      c[4] = __ldg(codes + x + 4);
#pragma unroll
      for (int e = 0; e < 4; ++e) v |= (uint32_t)delta_key(c[e], c[e + 1]) << (8 * e);
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (x + e >= 0 && x + e < (int)P)
          v |= (uint32_t)delta_key(__ldg(codes + x + e), __ldg(codes + x + e + 1)) << (8 * e);
    }
    reinterpret_cast<uint32_t*>(s.d)[g] = v;
  }
  if (SEG) {
    if (tid == 0) {
      const uint32_t lo_pos = (uint32_t)max(w0, 0);
      const uint32_t hi_pos = (uint32_t)min(w0 + TW_W, (int)U);
      s.c_first = owner(uoff, S, lo_pos);
      s.nb = upper_bound_u32(uoff, S + 1, hi_pos) - s.c_first;  // clouds starting at or before hi_pos
    }
    __syncthreads();
    const uint32_t c_first = s.c_first, nb = s.nb;
    // A pair that straddles two clouds is no split: mark it as a boundary.
    for (uint32_t k = 1 + tid; k < nb; k += TW_THREADS) {
      const int p = (int)uoff[c_first + k] - 1 - w0;
      if (p >= 0 && p < TW_W) s.d[p] = 0;
    }
    for (uint32_t k = tid; k < min(nb, (uint32_t)TW_MAXB); k += TW_THREADS) s.cb[k] = uoff[c_first + k];
  }
  __syncthreads();

  // 2. chunk minima.
  for (int c = tid; c < TW_NCH; c += TW_THREADS) {
    const uint4 q = *reinterpret_cast<const uint4*>(s.d + c * TW_C);
    const uint32_t m = __vminu4(__vminu4(q.x, q.y), __vminu4(q.z, q.w));
    s.cmin[c] = (uint8_t)min(min(m & 0xffu, (m >> 8) & 0xffu), min((m >> 16) & 0xffu, m >> 24));
  }
  __syncthreads();

  // 3. the two threshold tables, and the per-lane in-chunk pass.  A table row
  // for threshold v is the OR of the bits of every entry whose minimum is
  // below v: each entry ORs its bit into row min + 1, then a prefix-OR over
  // the 64 rows (two per lane) completes them.
  for (int b = warp; b < TW_NWB; b += TW_THREADS / 32) {
    s.t4[b][lane] = 0;
    s.t4[b][lane + 32] = 0;
    __syncwarp();
    const uint32_t m = s.cmin[b * 32 + lane];
    if (m + 1 < TW_TV) atomicOr(&s.t4[b][m + 1], 1u << lane);
    __syncwarp();
    tw_prefix_or_rows(s.t4[b], lane);
  }
  if (warp == 0) {
    s.t9[lane] = 0;
    s.t9[lane + 32] = 0;
    __syncwarp();
    if (lane < TW_NWB) {
      const uint4 q0 = *reinterpret_cast<const uint4*>(s.cmin + lane * 32);
      const uint4 q1 = *reinterpret_cast<const uint4*>(s.cmin + lane * 32 + 16);
      const uint32_t m = __vminu4(__vminu4(__vminu4(q0.x, q0.y), __vminu4(q0.z, q0.w)),
                                  __vminu4(__vminu4(q1.x, q1.y), __vminu4(q1.z, q1.w)));
      const uint32_t m9 = min(min(m & 0xffu, (m >> 8) & 0xffu), min((m >> 16) & 0xffu, m >> 24));
      if (m9 + 1 < TW_TV) atomicOr(&s.t9[m9 + 1], 1u << lane);
    }
    __syncwarp();
    tw_prefix_or_rows(s.t9, lane);
  }
  tw_chunk_stack(s, tid);
  __syncthreads();

  // 4. each split: its two answers, then its node.
  for (int xx = t0 + tid; xx < x_end; xx += TW_THREADS) {
    const uint32_t x = (uint32_t)xx;
    const int xi = xx - w0;
    const int ti = xx - t0;
    const int chunk = xi / TW_C;  // window chunk
    const int cstart = chunk * TW_C;
    const uint32_t lr = s.lr[ti];
    uint32_t U0 = 0, U1 = U;
    if (SEG) {
      uint32_t c;
      if (s.nb <= (uint32_t)TW_MAXB) {
        uint32_t lo = 0, hi = s.nb;  // last cached start <= x
        while (lo < hi) {
          const uint32_t mid = (lo + hi) >> 1;
          if (s.cb[mid] <= x) lo = mid + 1;
          else hi = mid;
        }
        c = s.c_first + lo - 1;
      } else {
        c = owner(uoff, S, x);
      }
      U0 = uoff[c];
      U1 = uoff[c + 1];
    }
    const uint32_t t = s.d[xi];
    if (t == 0) {  // the last key of a cloud: no split here
      if (SEG && edge) edge[x] = 0;
      continue;
    }
    const int r = (lr & 15) ? cstart + (int)(lr & 15) : tw_next_tab(s, chunk, t);
    const int l = (lr >> 4) != 15 ? cstart + (int)(lr >> 4) : tw_prev_tab(s, chunk, t);
    if (r < 0 || l < 0) {  // the range reaches past the window: step 5, or the queue
      const uint32_t k = atomicAdd(&s.lq_n, 1u);
      if (k < (uint32_t)TW_LQ) {
        s.lq[k] = x;
        continue;
      }
      if (queue) {
        queue[atomicAdd(q_count, 1u)] = x;
        continue;
      }
    }
    uint32_t hi, dR;
    if (r >= 0) {
      hi = (uint32_t)(w0 + r);
      dR = s.d[r];
    } else {
      hi = tw_range_hi<K>(codes, x, U1 - 1, (int)t);
      dR = (hi + 1 < U1) ? (uint32_t)delta_key(codes[hi], codes[hi + 1]) : 0u;
    }
    uint32_t lo, dL;
    if (l >= 0) {
      lo = (uint32_t)(w0 + l + 1);
      dL = s.d[l];
    } else {
      lo = tw_range_lo<K>(codes, x, U0, (int)t);
      dL = (lo > U0) ? (uint32_t)delta_key(codes[lo - 1], codes[lo]) : 0u;
    }
    tw_emit<A>(x, t, lo, hi, dL, dR, U0, prefix_n, hll, hlr, left, parent, edge);
  }

  // 5. the block's long-range splits, one warp each (both ends searched
  // over the codes together).
  __syncthreads();
  const uint32_t nl = min(s.lq_n, (uint32_t)TW_LQ);
  for (uint32_t q = warp; q < nl; q += TW_THREADS / 32) {  // warp-uniform
    const uint32_t x = s.lq[q];
    uint32_t U0 = 0, U1 = U;
    if (SEG) {
      const uint32_t c = owner(uoff, S, x);
      U0 = uoff[c];
      U1 = uoff[c + 1];
    }
    tw_warp_split<K>(codes, x, U0, U1, prefix_n, hll, hlr, left, parent, edge);
  }
}

// The queued splits, one warp each: both range ends by warp-cooperative
// search over the codes (the answers the window would give, for ranges of
// any length).
template <class K, bool SEG>
__global__ void __launch_bounds__(256) radix_tree_slow_kernel(const K* __restrict__ codes, const uint32_t* d_u,
                                                              uint32_t u_host, const uint32_t* uoff, uint32_t S,
                                                              uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr,
                                                              int32_t* left, int32_t* parent, uint32_t* edge,
                                                              const uint32_t* queue, const uint32_t* q_count) {
  griddep_wait();
  const uint32_t U = SEG ? uoff[S] : (d_u ? *d_u : u_host);
  const uint32_t nq = *q_count;
  const uint32_t warps = gridDim.x * (blockDim.x / 32);
  for (uint32_t q = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); q < nq; q += warps) {
    const uint32_t x = queue[q];
    uint32_t U0 = 0, U1 = U;
    if (SEG) {
      const uint32_t c = owner(uoff, S, x);
      U0 = uoff[c];
      U1 = uoff[c + 1];
    }
    tw_warp_split<K>(codes, x, U0, U1, prefix_n, hll, hlr, left, parent, edge);
  }
}

}  // namespace gtc
