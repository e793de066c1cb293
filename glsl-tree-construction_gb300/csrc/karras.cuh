// karras.cuh - one node of the Karras radix tree (build_radix_tree.comp:71-144)
// with the edge count of its internal children (edge_count.comp:30-41), as a
// device function shared by the single-cloud and the batched kernels.
#pragma once

#include "gtc_internal.cuh"

namespace gtc {

// Node i of m over codes[0..m].  Writes prefix_n[i], left[i], hll[i], hlr[i]
// and, for each internal child c, parent[c] = i and edge[c] (nullable).
//   * direction d = sign(delta(i, i+1) - delta(i, i-1)), computed signed;
//   * node 0 covers all m + 1 keys;
//   * exponential + binary search for the range end, binary search for the
//     split; all index arithmetic in 32 bits (u < 2^30);
//   * a child's depth comes from the delta of its range ends, so the edge
//     count needs no second pass over parent[].
template <class K>
__device__ __forceinline__ void karras_node(const K* __restrict__ codes, int m, int i, uint8_t* __restrict__ prefix_n,
                                            uint8_t* __restrict__ hll, uint8_t* __restrict__ hlr,
                                            int32_t* __restrict__ left, int32_t* __restrict__ parent,
                                            uint32_t* __restrict__ edge) {
  constexpr int A = KeyTraits<K>::A;
  const K ci = __ldg(codes + i);
  int d = 1;
  if (i > 0) {
    const int dr = delta_key(ci, __ldg(codes + i + 1));
    const int dl = delta_key(ci, __ldg(codes + i - 1));
    d = (dr > dl) - (dr < dl);
  }
  uint32_t l = 0;  // range length in keys, away from i in direction d
  if (i == 0) {
    l = (uint32_t)m;
  } else {
    const int dmin = delta_key(ci, __ldg(codes + i - d));
    const uint32_t lim = (d > 0) ? (uint32_t)(m - i) : (uint32_t)i;  // farthest reachable step
    uint32_t lmax = 2;
    while (lmax <= lim && delta_key(ci, __ldg(codes + i + (int)lmax * d)) > dmin) lmax <<= 1;
    for (uint32_t t = lmax >> 1; t >= 1; t >>= 1) {
      if (l + t <= lim && delta_key(ci, __ldg(codes + i + (int)(l + t) * d)) > dmin) l += t;
    }
  }
  const int j = i + (int)l * d;
  const int dnode = delta_key(ci, __ldg(codes + j));
  // Split search: t = ceil(l / 2^k) for 2^k up to 2^ceil(log2 l).  The shader
  // bounds s + t by the array (i - 1 or m - i - 1); a probe at s + t == l lands
  // on the range end, whose delta equals dnode and never advances s, so
  // bounding by l - 1 gives the same split.
  uint32_t s = 0;
  if (l > 1) {
    const uint32_t scut = l - 1;
    const int lg = 32 - __clz(l - 1);  // ceil(log2 l)
    for (int k = 1; k <= lg; ++k) {
      const uint32_t t = (l + (1u << k) - 1) >> k;
      if (s + t <= scut && delta_key(ci, __ldg(codes + i + (int)(s + t) * d)) > dnode) s += t;
    }
  }
  const int gamma = i + (int)s * d + (d < 0 ? -1 : 0);
  const int lo = d > 0 ? i : j;
  const int hi = d > 0 ? j : i;
  const bool leaf_l = (lo == gamma);
  const bool leaf_r = (hi == gamma + 1);
  prefix_n[i] = (uint8_t)dnode;
  left[i] = gamma;
  hll[i] = leaf_l;
  hlr[i] = leaf_r;
  const int depth_i = (dnode - A) / 3;
  if (!leaf_l) {
    parent[gamma] = i;
    if (edge) edge[gamma] = (uint32_t)((delta_key(__ldg(codes + lo), __ldg(codes + gamma)) - A) / 3 - depth_i);
  }
  if (!leaf_r) {
    parent[gamma + 1] = i;
    if (edge) edge[gamma + 1] = (uint32_t)((delta_key(__ldg(codes + gamma + 1), __ldg(codes + hi)) - A) / 3 - depth_i);
  }
}

}  // namespace gtc
