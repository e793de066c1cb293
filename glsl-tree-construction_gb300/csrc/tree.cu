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
// The searches are dependent loads; most ranges are short, so each block
// stages the codes of its tile plus a halo on either side in shared memory
// and only the rare long searches go to global memory (L2).
// The edge count of edge_count.comp:30-41 needs depth(parent): a node knows
// the exact key ranges of both children ([lo, gamma] and [gamma + 1, hi]),
// so it computes each internal child's prefix length from the range ends and
// writes the child's edge count next to its parent index.

#include "gtc_internal.cuh"

namespace gtc {

constexpr int TREE_THREADS = 256;
constexpr int TREE_NPT = 8;                            // nodes per thread per tile
constexpr int TREE_TILE = TREE_THREADS * TREE_NPT;     // 2048 nodes
constexpr int TREE_HALO = 1024;                        // staged codes on each side

template <class K>
__global__ void __launch_bounds__(TREE_THREADS) radix_tree_kernel(const K* __restrict__ codes, const uint32_t* d_u,
                                                                  int32_t m_host, uint8_t* __restrict__ prefix_n,
                                                                  uint8_t* __restrict__ hll,
                                                                  uint8_t* __restrict__ hlr,
                                                                  int32_t* __restrict__ left,
                                                                  int32_t* __restrict__ parent,
                                                                  uint32_t* __restrict__ edge, uint32_t* d_m) {
  constexpr int A = KeyTraits<K>::A;
  __shared__ K s_codes[TREE_TILE + 2 * TREE_HALO + 1];
  const int64_t m = d_u ? (int64_t)max(*d_u, 1u) - 1 : (int64_t)m_host;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (d_m) *d_m = (uint32_t)m;
    if (m > 0) {
      parent[0] = 0;  // D13
      if (edge) edge[0] = 0;
    }
  }
  for (int64_t tb = (int64_t)blockIdx.x * TREE_TILE; tb < m; tb += (int64_t)gridDim.x * TREE_TILE) {
    // Window [wlo, whi] of codes (code indices run 0..m).
    const int64_t wlo = tb > TREE_HALO ? tb - TREE_HALO : 0;
    const int64_t whi = min(tb + TREE_TILE + TREE_HALO, m);
    __syncthreads();
    for (int64_t x = wlo + threadIdx.x; x <= whi; x += TREE_THREADS) s_codes[x - wlo] = codes[x];
    __syncthreads();
    auto C = [&](int64_t x) -> K { return (x >= wlo && x <= whi) ? s_codes[x - wlo] : __ldg(codes + x); };
#pragma unroll 1
    for (int r = 0; r < TREE_NPT; ++r) {
      const int64_t i = tb + (int64_t)r * TREE_THREADS + threadIdx.x;
      if (i >= m) break;
      const K ci = C(i);
      int d = 1;
      if (i > 0) {
        const int dr = delta_key(ci, C(i + 1));
        const int dl = delta_key(ci, C(i - 1));
        d = (dr > dl) - (dr < dl);
      }
      int64_t l = 0;
      if (i == 0) {
        l = m;
      } else {
        const int dmin = delta_key(ci, C(i - d));
        int64_t lmax = 2;
        while (true) {
          const int64_t p = i + lmax * d;
          if (p < 0 || p > m) break;
          if (delta_key(ci, C(p)) <= dmin) break;
          lmax *= 2;
        }
        const int64_t lcut = (d == -1) ? i : m - i;
        for (int64_t t = lmax >> 1; t >= 1; t >>= 1) {
          if (l + t <= lcut && delta_key(ci, C(i + (l + t) * d)) > dmin) l += t;
        }
      }
      const int64_t j = i + l * d;
      const int dnode = delta_key(ci, C(j));
      // Split search: t = ceil(l / 2^k) for 2^k up to 2^ceil(log2 l).
      int64_t s = 0;
      const int64_t scut = (d == -1) ? i - 1 : m - i - 1;
      if (l > 1) {
        const int lg = 64 - __clzll((unsigned long long)(l - 1));  // ceil(log2 l)
        for (int k = 1; k <= lg; ++k) {
          const int64_t t = (l + ((int64_t)1 << k) - 1) >> k;
          if (s + t <= scut && delta_key(ci, C(i + (s + t) * d)) > dnode) s += t;
        }
      }
      const int64_t gamma = i + s * d + (d < 0 ? -1 : 0);
      const int64_t lo = d > 0 ? i : j;
      const int64_t hi = d > 0 ? j : i;
      const bool leaf_l = (lo == gamma);
      const bool leaf_r = (hi == gamma + 1);
      prefix_n[i] = (uint8_t)dnode;
      left[i] = (int32_t)gamma;
      hll[i] = leaf_l;
      hlr[i] = leaf_r;
      const int depth_i = (dnode - A) / 3;
      if (!leaf_l) {
        parent[gamma] = (int32_t)i;
        if (edge) edge[gamma] = (uint32_t)((delta_key(C(lo), C(gamma)) - A) / 3 - depth_i);
      }
      if (!leaf_r) {
        parent[gamma + 1] = (int32_t)i;
        if (edge) edge[gamma + 1] = (uint32_t)((delta_key(C(gamma + 1), C(hi)) - A) / 3 - depth_i);
      }
    }
  }
}

template <class K>
cudaError_t launch_radix_tree(const Launch& L, const K* codes, const uint32_t* d_u, int32_t m_host, uint32_t n_max,
                              uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr, int32_t* left, int32_t* parent,
                              uint32_t* edge, uint32_t* d_m) {
  const uint32_t work = d_u ? n_max : (uint32_t)max(m_host, 0);
  if (work == 0 && !d_m) return cudaSuccess;
  const uint32_t grid = max(1u, min(ceil_div(work, TREE_TILE), (uint32_t)L.num_sms * 6));
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
