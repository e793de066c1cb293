// tree.cu - Karras radix tree with the edge count fused in, and the
// standalone edge-count operator.
//
// build_radix_tree.comp:71-144 restated for 32- and 64-bit codes (the per-node
// work is karras_node in karras.cuh): signed direction, a root covering all
// u = m + 1 keys, exponential + binary range search, binary split search,
// leaf flags, parent scatter.  The kernel is bound by instruction issue (the
// searches are data-dependent loops), so all index arithmetic is 32-bit and
// the code loads go through the read-only L1 path, which serves the short
// searches that make up most nodes.

#include <atomic>

#include "karras.cuh"
#include "tree_window.cuh"

namespace gtc {

constexpr int TREE_THREADS = 256;

// 1: split-indexed window kernel (tree_window.cuh); 0: per-node Karras search.
static std::atomic<int> g_tree_method{1};
int tree_get_method() { return g_tree_method.load(std::memory_order_relaxed); }
bool tree_set_method(int m) {
  if (m != 0 && m != 1) return false;
  g_tree_method.store(m, std::memory_order_relaxed);
  return true;
}

template <class K>
__global__ void __launch_bounds__(TREE_THREADS) radix_tree_kernel(const K* __restrict__ codes, const uint32_t* d_u,
                                                                  int32_t m_host, uint8_t* __restrict__ prefix_n,
                                                                  uint8_t* __restrict__ hll,
                                                                  uint8_t* __restrict__ hlr,
                                                                  int32_t* __restrict__ left,
                                                                  int32_t* __restrict__ parent,
                                                                  uint32_t* __restrict__ edge, uint32_t* d_m) {
  const int m = d_u ? (int)max(*d_u, 1u) - 1 : m_host;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (d_m) *d_m = (uint32_t)m;
    if (m > 0) {
      parent[0] = 0;  // D13
      if (edge) edge[0] = 0;
    }
  }
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride)
    karras_node<K>(codes, m, i, prefix_n, hll, hlr, left, parent, edge);
}

template <class K>
cudaError_t launch_radix_tree(const Launch& L, const K* codes, const uint32_t* d_u, int32_t m_host, uint32_t n_max,
                              uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr, int32_t* left, int32_t* parent,
                              uint32_t* edge, uint32_t* d_m, uint32_t* queue, uint32_t* q_count) {
  const uint32_t work = d_u ? n_max : (uint32_t)max(m_host, 0);
  if (work == 0 && !d_m) return cudaSuccess;
  if (g_tree_method.load(std::memory_order_relaxed) == 1) {
    const uint32_t u_host = d_u ? 0u : (uint32_t)max(m_host, 0) + 1;
    if (queue && !L.ws_zeroed) {
      cudaError_t e = cudaMemsetAsync(q_count, 0, 4, L.stream);
      if (e != cudaSuccess) return e;
    }
    cudaError_t e = launch_kernel(L, radix_tree_window_kernel<K, false>, max(1u, ceil_div(work, TW_T)), TW_THREADS, 0,
                                  codes, d_u, u_host, nullptr, 0u, prefix_n, hll, hlr, left, parent, edge, d_m, queue,
                                  q_count);
    if (e != cudaSuccess || !queue) return e;
    return launch_kernel(L, radix_tree_slow_kernel<K, false>, L.num_sms * 2, 256, 0, codes, d_u, u_host, nullptr, 0u,
                         prefix_n, hll, hlr, left, parent, edge, queue, q_count);
  }
  const uint32_t grid = max(1u, min(ceil_div(work, TREE_THREADS), (uint32_t)L.num_sms * 8));
  radix_tree_kernel<K><<<grid, TREE_THREADS, 0, L.stream>>>(codes, d_u, m_host, prefix_n, hll, hlr, left, parent,
                                                             edge, d_m);
  return cudaGetLastError();
}
template cudaError_t launch_radix_tree<uint32_t>(const Launch&, const uint32_t*, const uint32_t*, int32_t, uint32_t,
                                                 uint8_t*, uint8_t*, uint8_t*, int32_t*, int32_t*, uint32_t*, uint32_t*,
                                                 uint32_t*, uint32_t*);
template cudaError_t launch_radix_tree<uint64_t>(const Launch&, const uint64_t*, const uint32_t*, int32_t, uint32_t,
                                                 uint8_t*, uint8_t*, uint8_t*, int32_t*, int32_t*, uint32_t*, uint32_t*,
                                                 uint32_t*, uint32_t*);

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
