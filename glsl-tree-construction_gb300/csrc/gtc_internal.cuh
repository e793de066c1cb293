// gtc_internal.cuh - shared device helpers and launcher declarations.
#pragma once

#include <utility>

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "gtc.h"

namespace gtc {

// Bits of the device status word (ctx-owned, read by gtc_device_status).
constexpr uint32_t DEV_TIMEOUT = 1u;   // a bounded spin ran out
constexpr uint32_t DEV_CAPACITY = 2u;  // an output buffer was too small
constexpr uint32_t DEV_INTERNAL = 4u;  // an impossible state was detected
constexpr uint32_t DEV_BAD_INPUT = 8u;  // device-resident arguments failed their checks

// Descriptor flags for decoupled look-back: value << 2 | flag.
constexpr uint32_t FLAG_NOT_READY = 0u;
constexpr uint32_t FLAG_AGGREGATE = 1u;
constexpr uint32_t FLAG_INCLUSIVE = 2u;

// Default poll budget of a bounded spin (with __nanosleep backoff after the
// first few polls), well under a second, before it gives up with DEV_TIMEOUT.
// gtc_set_spin_limit replaces it per context.
constexpr uint32_t SPIN_LIMIT = 1u << 20;

constexpr int NUM_SMS_GB300 = 152;

template <class K>
struct KeyTraits;
template <>
struct KeyTraits<uint32_t> {
  static constexpr int W = 32;
  static constexpr int B = 10;   // bits per axis
  static constexpr int A = 2;    // unused high bits
};
template <>
struct KeyTraits<uint64_t> {
  static constexpr int W = 64;
  static constexpr int B = 21;
  static constexpr int A = 1;
};

__device__ __forceinline__ int clz_key(uint32_t x) { return __clz(x); }
__device__ __forceinline__ int clz_key(uint64_t x) { return __clzll(x); }

// delta(a, b) of build_radix_tree.comp:48-58: leading common bits, W if equal.
template <class K>
__device__ __forceinline__ int delta_key(K a, K b) {
  const K x = a ^ b;
  return x == 0 ? KeyTraits<K>::W : clz_key(x);
}

// ----------------------------------------------------------- relaxed I/O --
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// ------------------------------------------------- L2 eviction priority --
// Loads that tag their lines for L2 to keep (evict_last: data read again soon
// by the same kernel) or to drop first (evict_first: last use).
__device__ __forceinline__ uint64_t l2_keep_policy() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_drop_policy() {
  uint64_t p;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint32_t ld_hint(const uint32_t* p, uint64_t pol) {
  uint32_t v;
  asm volatile("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ uint64_t ld_hint(const uint64_t* p, uint64_t pol) {
  uint64_t v;
  asm volatile("ld.global.nc.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(v) : "l"(p), "l"(pol));
  return v;
}

__device__ __forceinline__ uint4 ld_hint(const uint4* p, uint64_t pol) {
  uint4 v;
  asm volatile("ld.global.nc.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p), "l"(pol));
  return v;
}

__device__ __forceinline__ void st_hint(uint32_t* p, uint32_t v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.u32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_hint(uint64_t* p, uint64_t v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.u64 [%0], %1, %2;" ::"l"(p), "l"(v), "l"(pol) : "memory");
}

// Hint: fetch the 128-byte line holding p into L2.
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Poll budget of the bounded waits: word 1 of the context's status buffer
// when nonzero (gtc_set_spin_limit), else SPIN_LIMIT.  Read only once a wait
// has actually started.
__device__ __forceinline__ uint32_t spin_budget(const uint32_t* status) {
  const uint32_t b = ld_relaxed(status + 1);
  return b ? b : SPIN_LIMIT;
}

// Waits until *p carries a flag, at most spin_budget() polls.  On expiry
// records DEV_TIMEOUT and returns an INCLUSIVE descriptor of value 0 so the
// caller's look-back ends.
__device__ __forceinline__ uint32_t spin_descriptor(const uint32_t* p, uint32_t* status) {
  uint32_t v = ld_relaxed(p);
  if ((v & 3u) != FLAG_NOT_READY) return v;
  const uint32_t limit = spin_budget(status);
  uint32_t it = 0;
  while ((v & 3u) == FLAG_NOT_READY) {
    if (++it > limit) {
      atomicOr(status, DEV_TIMEOUT);
      return FLAG_INCLUSIVE;
    }
    if (it > 16) __nanosleep(32);
    v = ld_relaxed(p);
  }
  return v;
}

// Exclusive prefix of one digit over tiles [0, tile) by decoupled look-back
// over descriptors laid out [tile][RADIX].  Loads a window of W predecessors
// at once (independent loads, one memory latency per window instead of one
// per tile) and consumes them nearest-first until an INCLUSIVE descriptor.
template <int W, int RADIX_>
__device__ __forceinline__ uint32_t lookback_window(const uint32_t* desc, uint32_t tile, uint32_t digit,
                                                    uint32_t* status) {
  uint32_t excl = 0;
  int k = (int)tile - 1;
  while (k >= 0) {
    uint32_t v[W];
#pragma unroll
    for (int w = 0; w < W; ++w)
      v[w] = (k - w >= 0) ? ld_relaxed(desc + (size_t)(k - w) * RADIX_ + digit) : FLAG_INCLUSIVE;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      uint32_t x = v[w];
      if ((x & 3u) == FLAG_NOT_READY) x = spin_descriptor(desc + (size_t)(k - w) * RADIX_ + digit, status);
      excl += x >> 2;
      if ((x & 3u) == FLAG_INCLUSIVE) return excl;
    }
    k -= W;
  }
  return excl;
}

// ------------------------------------------------ TMA bulk copy / mbarrier --
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// Orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (TMA) writes to the same shared memory.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
// 1-D bulk copy global -> shared (both 16-byte aligned, bytes % 16 == 0),
// completion signalled on `bar` as transaction bytes.
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase with the given parity to complete.  Returns
// false (and records DEV_TIMEOUT) if the copy never lands.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t* status) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint32_t limit = spin_budget(status);
  for (uint32_t it = 0; it < limit; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (it > 16) __nanosleep(32);
  }
  atomicOr(status, DEV_TIMEOUT);
  return false;
}

// ---------------------------------------------------------------- morton --
// D17 saturating conversion, identical to the oracle's.
__device__ __forceinline__ uint32_t f2u_sat(float a) {
  if (!(a > 0.0f)) return 0u;
  if (a >= 4294967296.0f) return 0xFFFFFFFFu;
  return __float2uint_rz(a);
}

// morton.comp:50-56: (v - min) / range, then * 2^B, each op rounded to nearest.
// inv_rg != 0 is 1 / range for a range that is a power of two
// (pow2_reciprocal): the quotient and the product by the exact reciprocal are
// the same real number rounded once, so they are the same float, and the
// product costs one instruction instead of a full division.  Q picks the
// form at compile time (1: product, 2: division) or per call (0).
template <int Q = 0>
__device__ __forceinline__ uint32_t quantize(float v, float mn, float rg, float inv_rg, float scale) {
  const float d = __fsub_rn(v, mn);
  float t;
  if (Q == 1)
    t = __fmul_rn(d, inv_rg);
  else if (Q == 2)
    t = __fdiv_rn(d, rg);
  else
    t = (inv_rg != 0.0f) ? __fmul_rn(d, inv_rg) : __fdiv_rn(d, rg);
  return f2u_sat(__fmul_rn(t, scale));
}

// 1 / rg when rg is a power of two whose reciprocal is a normal float, else 0.
inline float pow2_reciprocal(float rg) {
  if (!(rg > 0.0f) || !(rg < 3.0e38f)) return 0.0f;
  int e = 0;
  const float m = std::frexp(rg, &e);
  if (m != 0.5f) return 0.0f;
  const int k = 1 - e;  // rg = 2^(e - 1)
  if (k < -126 || k > 127) return 0.0f;
  return std::ldexp(1.0f, k);
}

// The low 11 bits of v spread to every third bit (bit i -> bit 3i).
__device__ __forceinline__ uint32_t spread11(uint32_t v) {
  uint32_t x = v & 0x7ffu;
  x = (x | x << 16) & 0xff0000ffu;
  x = (x | x << 8) & 0x0f00f00fu;
  x = (x | x << 4) & 0xc30c30c3u;
  x = (x | x << 2) & 0x49249249u;
  return x;
}

__device__ __forceinline__ uint32_t split3_32(uint32_t b) {  // morton.comp:36-44
  uint32_t x = b & 0x000003ffu;
  x = (x | x << 16) & 0x030000ffu;
  x = (x | x << 8) & 0x0300f00fu;
  x = (x | x << 4) & 0x030c30c3u;
  x = (x | x << 2) & 0x09249249u;
  return x;
}
__device__ __forceinline__ uint64_t split3_64(uint32_t b) {
  uint64_t x = b & 0x1fffffull;
  x = (x | x << 32) & 0x001f00000000ffffull;
  x = (x | x << 16) & 0x001f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}
__device__ __forceinline__ uint32_t third_bits(uint32_t m) {  // morton.rs:62-68
  uint32_t x = m & 0x09249249u;
  x = (x ^ (x >> 2)) & 0x030c30c3u;
  x = (x ^ (x >> 4)) & 0x0300f00fu;
  x = (x ^ (x >> 8)) & 0x030000ffu;
  x = (x ^ (x >> 16)) & 0x000003ffu;
  return x;
}
// The 11 bits at positions 0, 3, ..., 30 of a 32-bit word, packed.
__device__ __forceinline__ uint32_t compact11(uint32_t x) {
  x &= 0x49249249u;
  x = (x ^ (x >> 2)) & 0xc30c30c3u;
  x = (x ^ (x >> 4)) & 0x0f00f00fu;
  x = (x ^ (x >> 8)) & 0xff0000ffu;
  x = (x ^ (x >> 16)) & 0x000007ffu;
  return x;
}
// Bits 0, 3, ..., 60 of m (morton.rs:62-68 widened to 21 bits per axis), as
// two 32-bit halves: bits 0..30 from the low word, bits 33..60 from the high.
__device__ __forceinline__ uint32_t third_bits(uint64_t m) {
  const uint32_t lo = (uint32_t)m, hi = (uint32_t)(m >> 32);
  return compact11(lo) | (compact11((hi >> 1) & 0x09249249u) << 11);
}

template <class K, int Q = 0>
struct Encoder;
template <int Q>
struct Encoder<uint32_t, Q> {
  static __device__ __forceinline__ uint32_t run(float4 p, float mn, float rg, float inv_rg) {
    return split3_32(quantize<Q>(p.x, mn, rg, inv_rg, 1024.0f)) |
           (split3_32(quantize<Q>(p.y, mn, rg, inv_rg, 1024.0f)) << 1) |
           (split3_32(quantize<Q>(p.z, mn, rg, inv_rg, 1024.0f)) << 2);
  }
};
template <int Q>
struct Encoder<uint64_t, Q> {
  static __device__ __forceinline__ uint64_t run(float4 p, float mn, float rg, float inv_rg) {
  // split3_64(x) | split3_64(y) << 1 | split3_64(z) << 2, built as two 32-bit
  // halves: x, y bits 0..10 and z bits 0..9 fill the low word, the rest the
  // high word.
    const float s = 2097152.0f;
    const uint32_t x = quantize<Q>(p.x, mn, rg, inv_rg, s) & 0x1fffffu;
    const uint32_t y = quantize<Q>(p.y, mn, rg, inv_rg, s) & 0x1fffffu;
    const uint32_t z = quantize<Q>(p.z, mn, rg, inv_rg, s) & 0x1fffffu;
    const uint32_t lo = spread11(x) | (spread11(y) << 1) | (spread11(z & 0x3ffu) << 2);
    const uint32_t hi = (spread11(x >> 11) << 1) | (spread11(y >> 11) << 2) | spread11(z >> 10);
    return ((uint64_t)hi << 32) | lo;
  }
};
template <class K, int Q = 0>
__device__ __forceinline__ K encode_point(float4 p, float mn, float rg, float inv_rg) {
  return Encoder<K, Q>::run(p, mn, rg, inv_rg);
}

// morton32_to_xyz (morton.rs:43-60): (q / 2^B) * range + min, no contraction.
template <class K>
__device__ __forceinline__ float4 decode_corner(K code, float mn, float rg) {
  const float bs = (KeyTraits<K>::B == 10) ? 1024.0f : 2097152.0f;
  float4 r;
  r.x = __fadd_rn(__fmul_rn(__fdiv_rn((float)third_bits(code), bs), rg), mn);
  r.y = __fadd_rn(__fmul_rn(__fdiv_rn((float)third_bits((K)(code >> 1)), bs), rg), mn);
  r.z = __fadd_rn(__fmul_rn(__fdiv_rn((float)third_bits((K)(code >> 2)), bs), rg), mn);
  r.w = 1.0f;
  return r;
}

// 2^-k as a float, exact (0 <= k <= 126).
__device__ __forceinline__ float exp2_neg(int k) { return __int_as_float((127 - k) << 23); }

// Integer cell coordinates of a code: the decode of morton.rs:43-74 without
// the scaling.
template <class K>
__device__ __forceinline__ uint3 code_xyz(K code) {
  return make_uint3(third_bits(code), third_bits((K)(code >> 1)), third_bits((K)(code >> 2)));
}

// decode_corner of a code's prefix of `level` octants, from the code's cell
// coordinates q: the prefix clears the low B - level bits of every axis.
// Division by 2^B is the exact scaling by 2^-B in IEEE arithmetic (the same
// correctly rounded value), so a multiplication by 2^-B gives decode_corner's
// result bit for bit at a fraction of the cost.
template <class K>
__device__ __forceinline__ float4 corner_at(uint3 q, int level, float mn, float rg) {
  constexpr int B = KeyTraits<K>::B;
  const uint32_t m = ~((1u << (B - level)) - 1u);
  const float s = exp2_neg(B);
  float4 r;
  r.x = __fadd_rn(__fmul_rn(__fmul_rn((float)(q.x & m), s), rg), mn);
  r.y = __fadd_rn(__fmul_rn(__fmul_rn((float)(q.y & m), s), rg), mn);
  r.z = __fadd_rn(__fmul_rn(__fmul_rn((float)(q.z & m), s), rg), mn);
  r.w = 1.0f;
  return r;
}

// ----------------------------------------------------------- warp scans ---
// Lanes of the (full) warp whose value agrees with this lane's on bits
// [0, BITS) of d: one ballot per bit.  Each bit's ballot predicate comes
// straight from an and/setp, and the ballot is complemented under the same
// predicate where this lane's bit is clear, so a bit costs the vote plus
// about three simple instructions.  Called by all 32 lanes.
template <int BITS>
__device__ __forceinline__ uint32_t warp_peers(uint32_t d) {
  uint32_t peers = 0xffffffffu;
#pragma unroll
  for (int b = 0; b < BITS; ++b) {
    uint32_t m;
    asm volatile(
        "{\n\t.reg .pred p;\n\t.reg .b32 t;\n\t"
        "and.b32 t, %1, %2;\n\t"
        "setp.ne.u32 p, t, 0;\n\t"
        "vote.sync.ballot.b32 %0, p, 0xffffffff;\n\t"
        "@!p not.b32 %0, %0;\n\t}"
        : "=r"(m)
        : "r"(d), "r"(1u << b));
    peers &= m;
  }
  return peers;
}

__device__ __forceinline__ uint32_t warp_inclusive_sum(uint32_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Literal-mode switches (GTC_LITERAL_*), process-wide.
uint32_t literal_flags();
// child_leaf_mask bits kept by the octree kernels: none under GTC_LITERAL_D6.
inline uint32_t leaf_mask_keep() { return (literal_flags() & GTC_LITERAL_D6) ? 0u : 0xffu; }

// ------------------------------------------------------- launcher table ---
struct Launch {
  cudaStream_t stream;
  uint32_t* status;  // device status word
  int num_sms;
  // Sort kernels launched with run_if set do their work only when *run_if is
  // nonzero (a decision taken on the device, e.g. the learned sort's
  // fallback), so a stream or graph can hold them unconditionally.
  const uint32_t* run_if = nullptr;
  // Programmatic dependent launch: the kernel's blocks may be scheduled
  // while the previous kernel of the stream drains; each kernel calls
  // griddep_wait() before its first global memory access, so only the launch
  // and block start-up overlap.
  bool pdl = false;
  // The unique / scan / tree-queue workspaces of this launch were zeroed by
  // an earlier kernel of the stream: no memset node in front of them.
  bool ws_zeroed = false;
};

// Start of every kernel that may run under a programmatic dependent launch:
// wait until the previous grid has completed and its writes are visible
// (a no-op for a normal launch), then let the next grid's blocks be
// scheduled.
__device__ __forceinline__ void griddep_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Per-device kernel set-up.  The dynamic shared memory opt-in
// (cudaFuncSetAttribute) and the resident-blocks answer belong to the device
// that is current when they are made, so they are cached per device: one entry
// per (current device, kernel, block size, dynamic shared bytes), read and
// filled under a mutex because several host threads may launch at once.  The
// first launch of a kernel shape on a device does the set-up; later ones only
// read the cache.  smem above the 48 KB default gets the opt-in;
// blocks_per_sm (nullable) receives the occupancy answer (at least 1).
cudaError_t kernel_setup(const void* kern, int threads, size_t smem, int* blocks_per_sm);
template <class... P>
cudaError_t kernel_setup(void (*kern)(P...), int threads, size_t smem, int* blocks_per_sm = nullptr) {
  return kernel_setup(reinterpret_cast<const void*>(kern), threads, smem, blocks_per_sm);
}

// Kernel launch honouring Launch::pdl (cudaLaunchKernelEx with the
// programmatic stream serialization attribute).
template <class... P, class... A>
cudaError_t launch_kernel(const Launch& L, void (*kern)(P...), dim3 grid, dim3 block, size_t smem, A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = L.stream;
  cudaLaunchAttribute at[1];
  if (L.pdl) {
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelEx(&cfg, kern, std::forward<A>(args)...);
}

// Sort tuning knobs, chosen from the compiled variant table.
struct SortConfig {
  int threads;
  int kpt;
  int variant;  // index into the compiled table
};

// Workspace layout of a sort of n keys with `passes` 8-bit passes.
struct SortWorkspace {
  uint32_t* header;       // done counter, tile counters[passes]
  uint32_t* counts;       // [passes][256]
  uint32_t* bin_offsets;  // [passes][256]
  uint32_t* desc;         // [passes][tiles][256]
  size_t header_words;    // words zeroed per call (header + counts)
  size_t desc_words;
  uint32_t tiles;
};

size_t sort_workspace_bytes(uint32_t n, int passes, int tile_keys);
SortWorkspace carve_sort_workspace(void* ws, uint32_t n, int passes, int tile_keys);

// Kernels' host launchers (morton.cu / onesweep.cu / scan.cu / tree.cu / octree.cu).
cudaError_t launch_morton32(const Launch& L, const float4* pts, uint32_t* keys, uint32_t* idx, uint32_t n, float mn,
                            float rg);
cudaError_t launch_morton64(const Launch& L, const float4* pts, uint64_t* keys, uint32_t* idx, uint32_t n, float mn,
                            float rg);
// Low bits of a 64-bit Morton code that the pipeline's sort leaves to the
// run fixup: its onesweep passes cover bits [RUN_FIXUP_BITS, 63).
constexpr int RUN_FIXUP_BITS = 23;  // 5 full 8-bit passes over bits 23..62
// Fused Morton encode + global histogram for a following sort of bits
// [begin_bit, 3B) of the code (begin_bit 0 or RUN_FIXUP_BITS; passes must be
// ceil((3B - begin_bit) / 8)); zeroes W.desc[0, W.desc_words).
template <class K>
cudaError_t launch_morton_hist(const Launch& L, const float4* pts, K* keys, uint32_t n, float mn, float rg,
                               const SortWorkspace& W, int begin_bit, int passes);
// Completes a stable LSD sort over bits [low_bits, 64) into a sort of the
// whole key: every run of keys that agree above low_bits is sorted stably by
// its low bits (1 <= low_bits <= 32), in place; the scratch arrays hold n
// entries.
template <class K>
cudaError_t launch_run_fixup(const Launch& L, K* keys, uint32_t* vals, K* scratch_keys, uint32_t* scratch_vals,
                             uint32_t n, int low_bits);

template <class K>
cudaError_t launch_global_hist(const Launch& L, const K* keys, uint32_t n, int begin_bit, int end_bit,
                               const SortWorkspace& W, int passes, int db = 8);
// variant < 0: the pinned variant, else the autotuned one for (key width,
// bits, n), else the built-in default.  iota_vals: the values' input is the
// position (vals is still the buffer the payload lives in between passes),
// made by the first pass instead of read.  db: digit width in bits (1..8);
// pass p sorts bits [begin_bit + db p, begin_bit + db (p + 1)), and the
// histogram must have been built with the same width.
template <class K>
cudaError_t launch_onesweep_passes(const Launch& L, K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt,
                                   uint32_t n, int begin_bit, int end_bit, const SortWorkspace& W, int passes,
                                   bool* result_in_alt, cudaEvent_t* ev_pass /* nullable [2*passes] */,
                                   int variant = -1, bool iota_vals = false, int db = 8);
// The variant a sort of n keys of key_bits width over `bits` bits will use.
int sort_select_variant(int key_bits, int bits, uint32_t n);
// Autotuner cache (tune.cu): the tuned variant for (key width, bits, n), or -1.
int tuned_variant(int key_bits, int bits, uint32_t n);
// The tuned digit width (6..8) for (key width, bits, n), or -1 (tune.cu).
int tuned_digit_bits(int key_bits, int bits, uint32_t n);
// Digit width of a sort (sort.cu): pinned, else tuned, else 8; and whether a
// width fits the bit range in the workspace's passes.
int sort_select_digit_bits(int key_bits, int bits, uint32_t n);
bool sort_digit_bits_ok(int bits, int db);
bool sort_set_digit_bits(int key_bits, int db);
int sort_max_passes();
// The tuned batched onesweep shape for a batch of n points, or -1 (tune.cu).
int tuned_batched_variant(uint32_t n);
// The tuned learned-sort grouping pass shape for n keys, or -1 (tune.cu).
int tuned_learned_variant(uint32_t n);
// The learned sort with the grouping passes' shape given (learned.cu).
int learned_num_variants();
gtc_status learned_sort_variant(gtc_ctx* ctx, const gtc_learned_model* m, const uint64_t* keys, const uint32_t* vals,
                                uint64_t* keys_out, uint32_t* vals_out, uint32_t n, void* ws, size_t ws_bytes,
                                uint32_t* d_flags, gtc_stream_t stream, int variant);
// The batched build with the segmented onesweep shape given (batched.cu).
int batched_num_variants();
gtc_status build_octree_batched_variant(gtc_ctx* ctx, const float* pts, const uint32_t* d_offsets,
                                        uint32_t n_clouds, uint32_t n_total, float min_coord, float range,
                                        const gtc_batch_buffers* out, void* ws, size_t ws_bytes,
                                        gtc_stream_t stream, int variant);

// Decoupled look-back scans: unique compaction and node offsets.
size_t scan_workspace_bytes(uint32_t n);
size_t learned_workspace_bytes(uint32_t n);
template <class K>
cudaError_t launch_unique(const Launch& L, const K* keys_in, const uint32_t* vals_in, K* keys_out,
                          uint32_t* vals_out, uint32_t n, uint32_t* d_count, void* ws);
cudaError_t launch_inclusive_scan(const Launch& L, const uint32_t* in, uint32_t* out, uint32_t n, void* ws);
// Inclusive scan of *d_count (<= n_max) elements, the count read on the device.
cudaError_t launch_inclusive_scan_dev(const Launch& L, const uint32_t* in, uint32_t* out, const uint32_t* d_count,
                                      uint32_t n_max, void* ws);
// Node offsets over u = m + 1 entries, m = (d_u ? *d_u - 1 : m_host).
cudaError_t launch_node_offsets(const Launch& L, const uint32_t* edge, uint32_t* ps, const uint32_t* d_u,
                                uint32_t m_host, uint32_t n_max, uint32_t* d_o, void* ws);

template <class K>
cudaError_t launch_radix_tree(const Launch& L, const K* codes, const uint32_t* d_u, int32_t m_host, uint32_t n_max,
                              uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr, int32_t* left, int32_t* parent,
                              uint32_t* edge, uint32_t* d_m /* nullable: receives m */,
                              uint32_t* queue = nullptr /* n_max words: long-range splits go to a warp pass */,
                              uint32_t* q_count = nullptr /* one word, zeroed here */);
// Radix tree method: 1 split-indexed window kernel (default), 0 per-node Karras.
int tree_get_method();
bool tree_set_method(int m);
cudaError_t launch_gather_points(const Launch& L, const float4* pts, uint32_t n_pts, const uint32_t* idx,
                                 uint32_t count, float4* out);
cudaError_t launch_edge_count(const Launch& L, const uint8_t* prefix_n, const int32_t* parent, uint32_t* edge,
                              uint32_t m, int unused_bits);
template <class K>
cudaError_t launch_octree_make(const Launch& L, const K* codes, const uint32_t* d_u, uint32_t u_host,
                               uint32_t n_max, const uint8_t* prefix_n, const uint8_t* hll, const uint8_t* hlr,
                               const int32_t* left, const uint32_t* edge, const uint32_t* ps, float mn, float rg,
                               gtc_octnode* nodes, uint32_t capacity, bool with_leaves);
template <class K>
cudaError_t launch_octree_link(const Launch& L, const K* codes, uint32_t m, const uint8_t* prefix_n,
                               const uint8_t* hll, const uint8_t* hlr, const int32_t* left, const int32_t* parent,
                               const uint32_t* edge, const uint32_t* ps, gtc_octnode* nodes, uint32_t capacity);

inline uint32_t ceil_div(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }
inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace gtc
