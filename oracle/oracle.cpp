// oracle.cpp - CPU restatement of the reference's point-cloud -> octree path.
// TEST INFRASTRUCTURE ONLY (see oracle.h): the checker for the CUDA path and
// the timed CPU baseline, never linked into the product library.
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fopenmp -shared -fPIC
// (oracle/Makefile).  -ffp-contract=off keeps every float op separately
// rounded (D10), which is what the CUDA kernels do with __f*_rn intrinsics.

#include "oracle.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <class K>
struct KeyTraits;
template <>
struct KeyTraits<uint32_t> {
  static constexpr int W = 32;    // key bits
  static constexpr int B = 10;    // bits per axis
  static constexpr float SCALE = 1024.0f;
  static int clz(uint32_t x) { return __builtin_clz(x); }
};
template <>
struct KeyTraits<uint64_t> {
  static constexpr int W = 64;
  static constexpr int B = 21;
  static constexpr float SCALE = 2097152.0f;
  static int clz(uint64_t x) { return __builtin_clzll(x); }
};

// D17: saturating float -> uint32 conversion (truncation toward zero inside
// the range, NaN and non-positive -> 0, >= 2^32 -> 2^32 - 1).
inline uint32_t f2u_sat(float a) {
  if (!(a > 0.0f)) return 0u;
  if (a >= 4294967296.0f) return 0xFFFFFFFFu;
  return static_cast<uint32_t>(a);
}

// morton.comp:36-44 (morton3D_SplitBy3bits)
inline uint32_t split3_32(uint32_t b) {
  uint32_t x = b & 0x000003ffu;
  x = (x | x << 16) & 0x030000ffu;
  x = (x | x << 8) & 0x0300f00fu;
  x = (x | x << 4) & 0x030c30c3u;
  x = (x | x << 2) & 0x09249249u;
  return x;
}
// 21-bit extension of the same spread (not in the reference).
inline uint64_t split3_64(uint32_t b) {
  uint64_t x = b & 0x1fffffull;
  x = (x | x << 32) & 0x001f00000000ffffull;
  x = (x | x << 16) & 0x001f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}
// morton.rs:62-68 (morton3_d_get_third_bits)
inline uint32_t third_bits32(uint32_t m) {
  uint32_t x = m & 0x09249249u;
  x = (x ^ (x >> 2)) & 0x030c30c3u;
  x = (x ^ (x >> 4)) & 0x0300f00fu;
  x = (x ^ (x >> 8)) & 0x030000ffu;
  x = (x ^ (x >> 16)) & 0x000003ffu;
  return x;
}
inline uint32_t third_bits64(uint64_t m) {
  uint64_t x = m & 0x1249249249249249ull;
  x = (x ^ (x >> 2)) & 0x10c30c30c30c30c3ull;
  x = (x ^ (x >> 4)) & 0x100f00f00f00f00full;
  x = (x ^ (x >> 8)) & 0x001f0000ff0000ffull;
  x = (x ^ (x >> 16)) & 0x001f00000000ffffull;
  x = (x ^ (x >> 32)) & 0x00000000001fffffull;
  return static_cast<uint32_t>(x);
}

// morton.comp:50-56 (single_point_to_code_v2): divide first, then scale.
inline uint32_t quantize(float v, float min_coord, float range, float scale) {
  float t = (v - min_coord) / range;
  return f2u_sat(t * scale);
}

template <class K>
inline K encode(const float* p, float min_coord, float range);
template <>
inline uint32_t encode<uint32_t>(const float* p, float mn, float rg) {
  return split3_32(quantize(p[0], mn, rg, 1024.0f)) | (split3_32(quantize(p[1], mn, rg, 1024.0f)) << 1) |
         (split3_32(quantize(p[2], mn, rg, 1024.0f)) << 2);
}
template <>
inline uint64_t encode<uint64_t>(const float* p, float mn, float rg) {
  const float s = 2097152.0f;
  return split3_64(quantize(p[0], mn, rg, s)) | (split3_64(quantize(p[1], mn, rg, s)) << 1) |
         (split3_64(quantize(p[2], mn, rg, s)) << 2);
}

// morton.rs:43-60 / octree.comp:102-124: (q / scale) * range + min, each op
// rounded separately.
template <class K>
inline void decode(float* ret, K code, float min_coord, float range);
template <>
inline void decode<uint32_t>(float* ret, uint32_t code, float mn, float rg) {
  const float bs = 1024.0f;
  ret[0] = (static_cast<float>(third_bits32(code)) / bs) * rg + mn;
  ret[1] = (static_cast<float>(third_bits32(code >> 1)) / bs) * rg + mn;
  ret[2] = (static_cast<float>(third_bits32(code >> 2)) / bs) * rg + mn;
  ret[3] = 1.0f;
}
template <>
inline void decode<uint64_t>(float* ret, uint64_t code, float mn, float rg) {
  const float bs = 2097152.0f;
  ret[0] = (static_cast<float>(third_bits64(code)) / bs) * rg + mn;
  ret[1] = (static_cast<float>(third_bits64(code >> 1)) / bs) * rg + mn;
  ret[2] = (static_cast<float>(third_bits64(code >> 2)) / bs) * rg + mn;
  ret[3] = 1.0f;
}

// ---------------------------------------------------------------- sort ----
template <class K>
struct Pair {
  K key;
  uint32_t val;
};

template <class K>
void sort_pairs(K* keys, uint32_t* vals, uint32_t n, int threads) {
  std::vector<Pair<K>> a(n);
  for (uint32_t i = 0; i < n; ++i) a[i] = {keys[i], vals[i]};
  auto less = [](const Pair<K>& x, const Pair<K>& y) { return x.key < y.key; };
#ifdef _OPENMP
  if (threads > 1 && n >= (1u << 16)) {
    // Chunked stable sort, then rounds of stable pairwise merges (std::merge
    // takes equal keys from the first range first).
    int t = threads;
    std::vector<size_t> bounds(t + 1);
    for (int c = 0; c <= t; ++c) bounds[c] = (size_t)n * c / t;
#pragma omp parallel for num_threads(threads) schedule(static, 1)
    for (int c = 0; c < t; ++c) std::stable_sort(a.begin() + bounds[c], a.begin() + bounds[c + 1], less);
    std::vector<Pair<K>> b(n);
    std::vector<Pair<K>>* src = &a;
    std::vector<Pair<K>>* dst = &b;
    while (bounds.size() > 2) {
      size_t runs = bounds.size() - 1;
      size_t pairs = runs / 2;
      std::vector<size_t> nb;
      nb.push_back(0);
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
      for (long p = 0; p < (long)pairs; ++p) {
        size_t lo = bounds[2 * p], mid = bounds[2 * p + 1], hi = bounds[2 * p + 2];
        std::merge(src->begin() + lo, src->begin() + mid, src->begin() + mid, src->begin() + hi,
                   dst->begin() + lo, less);
      }
      if (runs % 2) std::copy(src->begin() + bounds[runs - 1], src->begin() + bounds[runs], dst->begin() + bounds[runs - 1]);
      for (size_t p = 0; p < pairs; ++p) nb.push_back(bounds[2 * p + 2]);
      if (runs % 2) nb.push_back(bounds[runs]);
      bounds.swap(nb);
      std::swap(src, dst);
    }
    if (src != &a) a.swap(b);
  } else
#endif
  {
    (void)threads;
    std::stable_sort(a.begin(), a.end(), less);
  }
  for (uint32_t i = 0; i < n; ++i) {
    keys[i] = a[i].key;
    vals[i] = a[i].val;
  }
}

// --------------------------------------------------------------- unique ---
// unique.comp:31-45, payload of the first occurrence carried along.
template <class K>
uint32_t unique(K* keys, uint32_t* vals, uint32_t n) {
  if (n == 0) return 0;
  uint32_t j = 0;
  for (uint32_t i = 1; i < n; ++i) {
    if (keys[i] != keys[j]) {
      ++j;
      keys[j] = keys[i];
      if (vals) vals[j] = vals[i];
    }
  }
  return j + 1;
}

// ----------------------------------------------------------- radix tree ---
template <class K>
inline int delta(K a, K b) {
  K x = a ^ b;
  return x == 0 ? KeyTraits<K>::W : KeyTraits<K>::clz(x);
}

inline int log2_ceil(int64_t x) {  // build_radix_tree.comp:60-68, x >= 1
  int msb = 63 - __builtin_clzll((unsigned long long)x);
  return msb + (((int64_t)1 << msb) < x ? 1 : 0);
}

// build_radix_tree.comp:71-144 for node i of m.
template <class K>
uint32_t radix_tree(const K* codes, int32_t m, uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr, int32_t* left,
                    int32_t* parent, uint32_t flags) {
  if (m <= 0) return 0;
  std::vector<uint8_t> writes(m, 0);
  parent[0] = 0;  // D13
  for (int64_t i = 0; i < m; ++i) {
    const K ci = codes[i];
    int d;
    if (i == 0) {
      d = 1;
    } else {
      int dr = delta(ci, codes[i + 1]);
      int dl = delta(ci, codes[i - 1]);
      if (flags & ORC_LITERAL_D1) {
        uint8_t dd = static_cast<uint8_t>(dr - dl);  // uint8_t wrap: never < 0
        d = (dd > 0) ? 1 : 0;
      } else {
        d = (dr > dl) - (dr < dl);
      }
    }
    int64_t l = 0;
    if (i == 0) {
      l = (flags & ORC_LITERAL_D16) ? (int64_t)m - 1 : (int64_t)m;  // D16
    } else {
      const int dmin = delta(ci, codes[i - d]);
      int64_t lmax = 2;
      while (i + lmax * d >= 0 && i + lmax * d <= m && delta(ci, codes[i + lmax * d]) > dmin) lmax *= 2;
      const int64_t lcut = (d == -1) ? i : (int64_t)m - i;
      for (int64_t t = lmax / 2, div = 2; t >= 1; div *= 2, t = lmax / div) {
        if (l + t <= lcut && delta(ci, codes[i + (l + t) * d]) > dmin) l += t;
      }
    }
    const int64_t j = i + l * d;
    const int dnode = delta(codes[i], codes[j]);
    prefix_n[i] = static_cast<uint8_t>(dnode);
    int64_t s = 0;
    const int64_t maxdiv = (l >= 1) ? ((int64_t)1 << log2_ceil(l)) : 1;  // D14 guard
    const int64_t scut = (d == -1) ? i - 1 : (int64_t)m - i - 1;
    int64_t div = 2;
    for (int64_t t = (l + 1) / 2; div <= maxdiv; div <<= 1, t = (l + div - 1) / div) {
      if (s + t <= scut && delta(ci, codes[i + (s + t) * d]) > dnode) s += t;
    }
    const int64_t gamma = i + s * d + std::min(d, 0);
    left[i] = static_cast<int32_t>(gamma);
    hll[i] = (std::min(i, j) == gamma) ? 1 : 0;
    hlr[i] = (std::max(i, j) == gamma + 1) ? 1 : 0;
    if (!hll[i] && gamma >= 0 && gamma < m) {
      parent[gamma] = static_cast<int32_t>(i);
      if (writes[gamma] < 255) ++writes[gamma];
    }
    if (!hlr[i] && gamma + 1 >= 0 && gamma + 1 < m) {
      parent[gamma + 1] = static_cast<int32_t>(i);
      if (writes[gamma + 1] < 255) ++writes[gamma + 1];
    }
  }
  uint32_t multi = 0;
  for (int32_t k = 0; k < m; ++k) multi += writes[k] > 1;
  return multi;
}

// -------------------------------------------------------------- octree ----
struct OctCtx {
  uint32_t flags;
  int A;
  const uint8_t* prefix_n;
  const uint32_t* edge;
  const uint32_t* ps;
  const int32_t* parent;
  int depth(uint32_t i) const {
    return (flags & ORC_LITERAL_D2) ? prefix_n[i] / 3 : (prefix_n[i] - A) / 3;
  }
  int64_t base(uint32_t i) const {  // first octree slot of radix node i
    if (flags & ORC_LITERAL_D3) return ps[i];
    if (i == 0) return 0;  // the root radix node owns slot 0
    return (int64_t)ps[i] - edge[i] + 1;
  }
  // D7: nearest ancestor (from rt up) that contributes octree nodes; the root
  // stops the walk.
  uint32_t walk(uint32_t rt, uint32_t* cap_hits) const {
    int steps = 0;
    while (edge[rt] == 0 && rt != 0) {
      rt = parent[rt];
      if (++steps > 64) {
        ++*cap_hits;
        break;
      }
    }
    return rt;
  }
};

template <class K>
uint32_t octree(const K* codes, uint32_t u, const uint8_t* prefix_n, const uint8_t* hll, const uint8_t* hlr,
                const int32_t* left, const int32_t* parent, const uint32_t* edge, const uint32_t* ps, float mn,
                float rg, orc_octnode* out, uint32_t flags, uint32_t* conflicts, uint32_t* cap_hits) {
  constexpr int B = KeyTraits<K>::B;
  constexpr int W = KeyTraits<K>::W;
  *conflicts = 0;
  *cap_hits = 0;
  if (u == 0) return 0;
  const uint32_t m = u - 1;
  // A racy literal tree (ORC_LITERAL_D1) can give negative depth differences,
  // which wrap to huge edge counts: report them and build nothing.
  uint32_t bad_edges = 0;
  for (uint32_t i = 0; i < m; ++i) bad_edges += edge[i] > (uint32_t)B;
  if (bad_edges) {
    *conflicts = bad_edges;
    return 0;
  }
  const uint32_t o = 1 + (m > 0 ? ps[u - 1] : 0);
  // Literal D3 ranges can run past o; build into a padded scratch array.
  std::vector<orc_octnode> nodes((size_t)o + 64);
  std::memset(nodes.data(), 0, nodes.size() * sizeof(orc_octnode));
  std::vector<uint8_t> used(nodes.size(), 0);
  auto set_slot = [&](int64_t node, int which, int32_t value, bool leaf) {
    if (node < 0 || node >= (int64_t)nodes.size()) {
      ++*conflicts;
      return;
    }
    orc_octnode& nd = nodes[node];
    if (used[node] & (1u << which)) ++*conflicts;
    used[node] |= (uint8_t)(1u << which);
    nd.children[which] = value;
    if (!leaf) {
      nd.child_node_mask |= 1 << which;  // SetChild, octree.comp:22-25
    } else if (flags & ORC_LITERAL_D6) {
      nd.child_leaf_mask &= ~(1 << which);  // SetLeaf as written, octree.comp:27-30
    } else {
      nd.child_leaf_mask |= 1 << which;  // D6
    }
  };
  auto shift_of = [&](int level) { return std::max(0, 3 * B - 3 * level); };

  OctCtx c{flags, W - 3 * B, prefix_n, edge, ps, parent};
  // Root node setup, main.rs:140-153 (D18 when m == 0).
  const int root_level = (m > 0) ? c.depth(0) : 0;
  {
    const int sh = shift_of(root_level);
    K root_prefix = (sh >= W) ? 0 : (codes[0] >> sh);
    decode<K>(nodes[0].corner, (sh >= W) ? 0 : (K)(root_prefix << sh), mn, rg);
    nodes[0].cell_size = rg;
  }
  // k_MakeOctNodes, octree.comp:126-186.
  for (uint32_t i = 0; i < m; ++i) {
    const uint32_t cnt = edge[i];
    if (cnt == 0) continue;
    int64_t idx = c.base(i);
    const int di = c.depth(i);
    for (uint32_t j = 0; j + 1 < cnt; ++j) {
      const int level = di - (int)j;
      const int sh = shift_of(level);
      const K prefix = codes[i] >> sh;
      const int which = (int)(prefix & 7);
      const int64_t par = idx + 1;
      set_slot(par, which, (int32_t)idx, false);
      if (idx >= 0 && idx < (int64_t)nodes.size()) {
        decode<K>(nodes[idx].corner, (K)(prefix << sh), mn, rg);
        nodes[idx].cell_size = rg / (float)(1 << (level - root_level));
      }
      idx = par;
    }
    const uint32_t rt = c.walk((uint32_t)parent[i], cap_hits);
    const int64_t oct_parent = c.base(rt);
    const int top_level = di - (int)cnt + 1;
    const int sh = shift_of(top_level);
    const K top_prefix = codes[i] >> sh;
    set_slot(oct_parent, (int)(top_prefix & 7), (int32_t)idx, false);
    if (idx >= 0 && idx < (int64_t)nodes.size()) {
      decode<K>(nodes[idx].corner, (K)(top_prefix << sh), mn, rg);
      nodes[idx].cell_size = rg / (float)(1 << (top_level - root_level));
    }
  }
  // k_LinkLeafNodes, octree.comp:188-222 (D8: after make).
  for (uint32_t i = 0; i < m; ++i) {
    for (int side = 0; side < 2; ++side) {
      if (!(side ? hlr[i] : hll[i])) continue;
      const int32_t leaf = left[i] + side;
      const int leaf_level = c.depth(i) + 1;
      const int which = (int)((codes[leaf] >> shift_of(leaf_level)) & 7);
      const uint32_t rt = c.walk(i, cap_hits);
      set_slot(c.base(rt), which, leaf, true);
    }
  }
  std::memcpy(out, nodes.data(), (size_t)o * sizeof(orc_octnode));
  return o;
}

template <class K>
void hist_exclusive(const K* keys, uint32_t n, int passes, uint32_t* hist, uint32_t flags) {
  std::vector<uint64_t> cnt((size_t)passes * 256, 0);
  // histogram.comp:117-143: non-last workgroups read 4 keys per step; the
  // second key's second digit is masked with 0xF (line 128, D11).
  const uint64_t nwg = ((uint64_t)n + 65535) / 65536;
  const uint64_t literal_end = nwg > 0 ? (nwg - 1) * 65536 : 0;
  for (uint32_t i = 0; i < n; ++i) {
    const K k = keys[i];
    for (int p = 0; p < passes; ++p) {
      uint32_t dgt = (uint32_t)((k >> (8 * p)) & 0xFF);
      if ((flags & ORC_LITERAL_D11) && p == 1 && i < literal_end && (i & 3) == 1) dgt = (uint32_t)((k >> 8) & 0xF);
      ++cnt[(size_t)p * 256 + dgt];
    }
  }
  for (int p = 0; p < passes; ++p) {
    uint64_t run = 0;
    for (int d = 0; d < 256; ++d) {
      hist[p * 256 + d] = (uint32_t)run;
      run += cnt[(size_t)p * 256 + d];
    }
  }
}

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

template <class K>
int build_octree(const float* pts, uint32_t n, float mn, float rg, K* keys, uint32_t* idx, uint8_t* prefix_n,
                 uint8_t* hll, uint8_t* hlr, int32_t* left, int32_t* parent, uint32_t* edge, uint32_t* ps,
                 orc_octnode* nodes, uint32_t* counts, uint32_t flags, int threads, double* stage_ms) {
  constexpr int W = KeyTraits<K>::W;
  constexpr int B = KeyTraits<K>::B;
  double tms[8] = {0};
  auto t0 = std::chrono::steady_clock::now();
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads > 0 ? threads : 1) schedule(static)
#endif
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    keys[i] = encode<K>(pts + 4 * i, mn, rg);
    idx[i] = (uint32_t)i;
  }
  tms[0] = ms_since(t0);
  t0 = std::chrono::steady_clock::now();
  sort_pairs<K>(keys, idx, n, threads);
  tms[1] = ms_since(t0);
  t0 = std::chrono::steady_clock::now();
  const uint32_t u = unique<K>(keys, idx, n);
  tms[2] = ms_since(t0);
  const uint32_t m = u > 0 ? u - 1 : 0;
  t0 = std::chrono::steady_clock::now();
  radix_tree<K>(keys, (int32_t)m, prefix_n, hll, hlr, left, parent, flags);
  tms[3] = ms_since(t0);
  t0 = std::chrono::steady_clock::now();
  for (uint32_t i = 0; i < m; ++i) {
    const int a = (flags & ORC_LITERAL_D2) ? prefix_n[i] / 3 : (prefix_n[i] - (W - 3 * B)) / 3;
    const int b = (flags & ORC_LITERAL_D2) ? prefix_n[parent[i]] / 3 : (prefix_n[parent[i]] - (W - 3 * B)) / 3;
    edge[i] = (uint32_t)(a - b);
  }
  tms[4] = ms_since(t0);
  t0 = std::chrono::steady_clock::now();
  if (u > 0) orc_prefix_sum(edge, u, ps);
  tms[5] = ms_since(t0);
  t0 = std::chrono::steady_clock::now();
  uint32_t conflicts = 0, caps = 0;
  const uint32_t o = octree<K>(keys, u, prefix_n, hll, hlr, left, parent, edge, ps, mn, rg, nodes, flags,
                               &conflicts, &caps);
  tms[6] = ms_since(t0);
  counts[0] = u;
  counts[1] = m;
  counts[2] = o;
  if (stage_ms)
    for (int s = 0; s < 8; ++s) stage_ms[s] = tms[s];
  return (int)(conflicts + caps);
}

}  // namespace

extern "C" {

void orc_morton32(const float* pts, uint32_t n, float mn, float rg, uint32_t* keys) {
  for (uint32_t i = 0; i < n; ++i) keys[i] = encode<uint32_t>(pts + 4 * (size_t)i, mn, rg);
}
void orc_morton64(const float* pts, uint32_t n, float mn, float rg, uint64_t* keys) {
  for (uint32_t i = 0; i < n; ++i) keys[i] = encode<uint64_t>(pts + 4 * (size_t)i, mn, rg);
}
void orc_morton32_to_xyz(float* ret, uint32_t code, float mn, float rg) { decode<uint32_t>(ret, code, mn, rg); }
void orc_morton64_to_xyz(float* ret, uint64_t code, float mn, float rg) { decode<uint64_t>(ret, code, mn, rg); }

void orc_global_hist_u32(const uint32_t* keys, uint32_t n, int passes, uint32_t* hist, uint32_t flags) {
  hist_exclusive<uint32_t>(keys, n, passes, hist, flags);
}
void orc_global_hist_u64(const uint64_t* keys, uint32_t n, int passes, uint32_t* hist) {
  hist_exclusive<uint64_t>(keys, n, passes, hist, 0);
}

void orc_sort_pairs_u32(uint32_t* keys, uint32_t* vals, uint32_t n, int threads) {
  sort_pairs<uint32_t>(keys, vals, n, threads);
}
void orc_sort_pairs_u64(uint64_t* keys, uint32_t* vals, uint32_t n, int threads) {
  sort_pairs<uint64_t>(keys, vals, n, threads);
}

uint32_t orc_unique_u32(uint32_t* keys, uint32_t* vals, uint32_t n) { return unique<uint32_t>(keys, vals, n); }
uint32_t orc_unique_u64(uint64_t* keys, uint32_t* vals, uint32_t n) { return unique<uint64_t>(keys, vals, n); }

uint32_t orc_radix_tree_u32(const uint32_t* codes, int32_t m, uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr,
                            int32_t* left, int32_t* parent, uint32_t flags) {
  return radix_tree<uint32_t>(codes, m, prefix_n, hll, hlr, left, parent, flags);
}
uint32_t orc_radix_tree_u64(const uint64_t* codes, int32_t m, uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr,
                            int32_t* left, int32_t* parent, uint32_t flags) {
  return radix_tree<uint64_t>(codes, m, prefix_n, hll, hlr, left, parent, flags);
}

void orc_edge_count(const uint8_t* prefix_n, const int32_t* parent, uint32_t m, int A, uint32_t* edge,
                    uint32_t flags) {
  for (uint32_t i = 0; i < m; ++i) {
    const int a = (flags & ORC_LITERAL_D2) ? prefix_n[i] / 3 : (prefix_n[i] - A) / 3;
    const int b = (flags & ORC_LITERAL_D2) ? prefix_n[parent[i]] / 3 : (prefix_n[parent[i]] - A) / 3;
    edge[i] = (uint32_t)(a - b);
  }
}

uint32_t orc_prefix_sum(const uint32_t* edge, uint32_t u, uint32_t* ps) {
  if (u == 0) return 0;
  const uint32_t m = u - 1;
  uint32_t run = 0;
  for (uint32_t k = 0; k < u; ++k) {
    run += (k < m) ? edge[k] : 0u;  // D4: edge[m] reads as 0
    ps[k] = run;
  }
  ps[0] = 0;  // main.rs:129
  return ps[u - 1];
}

uint32_t orc_octree_u32(const uint32_t* codes, uint32_t u, const uint8_t* prefix_n, const uint8_t* hll,
                        const uint8_t* hlr, const int32_t* left, const int32_t* parent, const uint32_t* edge,
                        const uint32_t* ps, float mn, float rg, orc_octnode* nodes, uint32_t flags,
                        uint32_t* conflicts, uint32_t* caps) {
  return octree<uint32_t>(codes, u, prefix_n, hll, hlr, left, parent, edge, ps, mn, rg, nodes, flags, conflicts,
                          caps);
}
uint32_t orc_octree_u64(const uint64_t* codes, uint32_t u, const uint8_t* prefix_n, const uint8_t* hll,
                        const uint8_t* hlr, const int32_t* left, const int32_t* parent, const uint32_t* edge,
                        const uint32_t* ps, float mn, float rg, orc_octnode* nodes, uint32_t flags,
                        uint32_t* conflicts, uint32_t* caps) {
  return octree<uint64_t>(codes, u, prefix_n, hll, hlr, left, parent, edge, ps, mn, rg, nodes, flags, conflicts,
                          caps);
}

int orc_validate_octree(const orc_octnode* nodes, uint32_t o, uint32_t u, float range) {
  if (o == 0) return u == 0 ? 0 : 1;
  if (nodes[0].cell_size != range) return 2;
  std::vector<uint32_t> parents(o, 0), leaves(u, 0);
  for (uint32_t s = 0; s < o; ++s) {
    const orc_octnode& nd = nodes[s];
    if (nd.child_node_mask & nd.child_leaf_mask) return 3;
    for (int b = 0; b < 8; ++b) {
      const int32_t ch = nd.children[b];
      if (nd.child_node_mask & (1 << b)) {
        if (ch <= 0 || (uint32_t)ch >= o) return 4;
        ++parents[ch];
        if (nodes[ch].cell_size * 2.0f != nd.cell_size) return 5;
      } else if (nd.child_leaf_mask & (1 << b)) {
        if (ch < 0 || (uint32_t)ch >= u) return 6;
        ++leaves[ch];
      } else if (ch != 0) {
        return 7;
      }
    }
  }
  for (uint32_t s = 1; s < o; ++s)
    if (parents[s] != 1) return 8;
  if (u >= 2)
    for (uint32_t k = 0; k < u; ++k)
      if (leaves[k] != 1) return 9;
  return 0;
}

int orc_build_octree(const float* pts, uint32_t n, float mn, float rg, int key_bits, void* keys, uint32_t* idx,
                     uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr, int32_t* left, int32_t* parent, uint32_t* edge,
                     uint32_t* ps, orc_octnode* nodes, uint32_t* counts, uint32_t flags, int threads,
                     double* stage_ms) {
  if (key_bits == 32)
    return build_octree<uint32_t>(pts, n, mn, rg, (uint32_t*)keys, idx, prefix_n, hll, hlr, left, parent, edge, ps,
                                  nodes, counts, flags, threads, stage_ms);
  if (key_bits == 64)
    return build_octree<uint64_t>(pts, n, mn, rg, (uint64_t*)keys, idx, prefix_n, hll, hlr, left, parent, edge, ps,
                                  nodes, counts, flags, threads, stage_ms);
  return -1;
}

static int pwl_segment(uint64_t key, const uint64_t* kn, int B) {
  int lo = 0, hi = B;
  while (hi - lo > 1) {
    const int mid = (lo + hi) / 2;
    if (kn[mid] <= key) lo = mid;
    else hi = mid;
  }
  return lo;
}

double orc_pwl_loss_grad(const uint64_t* s, uint32_t ns, const uint64_t* kn, const float* y, int B, double* grad) {
  for (int k = 0; k <= B; ++k) grad[k] = 0.0;
  double loss = 0.0;
  for (uint32_t j = 0; j < ns; ++j) {
    const int seg = pwl_segment(s[j], kn, B);
    const uint64_t k0 = kn[seg], k1 = kn[seg + 1];
    const double w = (k1 > k0) ? (double)(s[j] - k0) / (double)(k1 - k0) : 0.0;
    const double F = (double)y[seg] + ((double)y[seg + 1] - (double)y[seg]) * w;
    const double r = F - ((double)j + 0.5) / (double)ns;
    loss += r * r;
    grad[seg] += 2.0 * r * (1.0 - w) / ns;
    grad[seg + 1] += 2.0 * r * w / ns;
  }
  return loss / ns;
}

void orc_pwl_buckets(const uint64_t* keys, uint32_t n, const uint64_t* kn, const float* y, int B, uint32_t* out) {
  // The bucket line of the GPU model, operation for operation in FP32 with
  // round-to-nearest and no contraction: t = B*y0 + c * float(key - k0),
  // c = B*(y1 - y0) / float(k1 - k0), clamped to B*y1, truncated.
  const float fb = (float)B;
  for (uint32_t i = 0; i < n; ++i) {
    const int seg = pwl_segment(keys[i], kn, B);
    const uint64_t k0 = kn[seg], k1 = kn[seg + 1];
    const float y0 = y[seg], y1 = y[seg + 1];
    const float dy = fb * (y1 - y0);
    const float c = (k1 > k0 && dy > 0.0f) ? dy / (float)(k1 - k0) : 0.0f;
    const float a = fb * y0, amax = fb * y1;
    float t = a + c * (float)(keys[i] - k0);
    t = std::min(t, amax);
    const int b = (int)t;
    out[i] = (uint32_t)std::min(std::max(b, 0), B - 1);
  }
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
