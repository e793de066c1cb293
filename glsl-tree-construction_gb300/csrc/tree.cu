// tree.cu - Karras radix tree with the edge count fused in, and the
// standalone edge-count operator.
//
// build_radix_tree.comp:71-144 restated for 32- and 64-bit codes:
//   * delta(a, b) = __clz / __clzll of a ^ b (W when equal);
//   * direction d = sign(delta(i, i+1) - delta(i, i-1)) computed signed (the
//     shader computes it in uint8_t, so d is never -1);
//   * node 0 covers all u = m + 1 keys (the shader's l = n - 1 with n = m
//     drops the last key);
//   * exponential + binary search for the range end j, binary search for the
//     split gamma, leaf flags, parent scatter.
// The kernel is bound by instruction issue (the searches are data-dependent
// loops), so all index arithmetic is 32-bit (u < 2^30) and the code loads go
// through the read-only L1 path, which serves the short searches that make
// up most nodes.
// The edge count of edge_count.comp:30-41 needs depth(parent): a node knows
// the exact key ranges of both children ([lo, gamma] and [gamma + 1, hi]),
// so it computes each internal child's prefix length from the range ends and
// writes the child's edge count next to its parent index.

#include "gtc_internal.cuh"

namespace gtc {

constexpr int TREE_THREADS = 256;

template <class K>
__global__ void __launch_bounds__(TREE_THREADS) radix_tree_kernel(const K* __restrict__ codes, const uint32_t* d_u,
                                                                  int32_t m_host, uint8_t* __restrict__ prefix_n,
                                                                  uint8_t* __restrict__ hll,
                                                                  uint8_t* __restrict__ hlr,
                                                                  int32_t* __restrict__ left,
                                                                  int32_t* __restrict__ parent,
                                                                  uint32_t* __restrict__ edge, uint32_t* d_m) {
  constexpr int A = KeyTraits<K>::A;
  const int m = d_u ? (int)max(*d_u, 1u) - 1 : m_host;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (d_m) *d_m = (uint32_t)m;
    if (m > 0) {
      parent[0] = 0;  // D13
      if (edge) edge[0] = 0;
    }
  }
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
    const K ci = __ldg(codes + i);
    int d = 1;
    if (i > 0) {
      const int dr = delta_key(ci, __ldg(codes + i + 1));
      const int dl = delta_key(ci, __ldg(codes + i - 1));
      d = (dr > dl) - (dr < dl);
    }
    // Range length l (in keys) away from i in direction d.
    uint32_t l = 0;
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
    // Split search: t = ceil(l / 2^k) for 2^k up to 2^ceil(log2 l).
    uint32_t s = 0;
    if (l > 1) {
      // The shader bounds s + t by the array (i - 1 or m - i - 1); a probe at
      // s + t == l lands on the range end, whose delta equals dnode and never
      // advances s, so bounding by l - 1 gives the same split.
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
}

template <class K>
cudaError_t launch_radix_tree(const Launch& L, const K* codes, const uint32_t* d_u, int32_t m_host, uint32_t n_max,
                              uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr, int32_t* left, int32_t* parent,
                              uint32_t* edge, uint32_t* d_m) {
  const uint32_t work = d_u ? n_max : (uint32_t)max(m_host, 0);
  if (work == 0 && !d_m) return cudaSuccess;
  const uint32_t grid = max(1u, min(ceil_div(work, TREE_THREADS), (uint32_t)L.num_sms * 8));
  radix_tree_kernel<K><<<grid, TREE_THREADS, 0, L.stream>>>(codes, d_u, m_host, prefix_n, hll, hlr, left, parent,
                                                             edge, d_m);
  return cudaGetLastError();
}
template cudaError_t launch_radix_tree<uint32_t>(const Launch&, const uint32_t*, const uint32_t*, int32_t, uint32_t,
                                                 uint8_t*, uint8_t*, uint8_t*, int32_t*, int32_t*, uint32_t*, uint32_t*);
template cudaError_t launch_radix_tree<uint64_t>(const Launch&, const uint64_t*, const uint32_t*, int32_t, uint32_t,
                                                 uint8_t*, uint8_t*, uint8_t*, int32_t*, int32_t*, uint32_t*, uint32_t*);

// edge_count.comp:30-41 over exactly m nodes, depth = (prefix_n - A) / 3.
__global__ void edge_count_kernel(const uint8_t* __restrict__ prefix_n, const int32_t* __restrict__ parent,
                                  uint32_t* __restrict__ edge, uint32_t m, int A) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
    const int mine = (prefix_n[i] - A) / 3;
    const int par = (prefix_n[parent[i]] - A) / 3;
    edge[i] = (uint32_t)(mine - par);
  }
}

cudaError_t launch_edge_count(const Launch& L, const uint8_t* prefix_n, const int32_t* parent, uint32_t* edge,
                              uint32_t m, int A) {
  if (m == 0) return cudaSuccess;
  const uint32_t grid = max(1u, min(ceil_div(m, 256), (uint32_t)L.num_sms * 8));
  edge_count_kernel<<<grid, 256, 0, L.stream>>>(prefix_n, parent, edge, m, A);
  return cudaGetLastError();
}

}  // namespace gtc
