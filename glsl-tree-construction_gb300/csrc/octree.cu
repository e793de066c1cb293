// octree.cu - octree make (pull form, octree_dev.cuh) and the push-form link
// operator for callers that run make and link as separate stages.

#include "octree_dev.cuh"

namespace gtc {

constexpr int OCT_THREADS = 256;
// The kernel is bound by the latency of its dependent loads (node -> child ->
// grandchild) and, with one node per thread, by the divergence of the
// descents.  Only about a third of the radix nodes own octree nodes, so each
// warp first compacts the contributing nodes of consecutive 32-node slices
// into a queue in shared memory (ballot + popc) and runs a batch on every 32
// of them (octree_warp_batch: breadth-first descents, every lane busy).  No
// block barriers; 16-byte stores straight to HBM.
template <class K, bool WITH_LEAVES>
__global__ void __launch_bounds__(OCT_THREADS) octree_make_kernel(const K* __restrict__ codes, const uint32_t* d_u,
                                                                  uint32_t u_host, const uint8_t* __restrict__ prefix_n,
                                                                  const uint8_t* __restrict__ hll,
                                                                  const uint8_t* __restrict__ hlr,
                                                                  const int32_t* __restrict__ left,
                                                                  const uint32_t* __restrict__ edge,
                                                                  const uint32_t* __restrict__ ps, float mn, float rg,
                                                                  gtc_octnode* __restrict__ nodes, uint32_t capacity,
                                                                  uint32_t lmask_keep, uint32_t* status) {
  griddep_wait();
  constexpr int A = KeyTraits<K>::A;
  constexpr int WARPS = OCT_THREADS / 32;
  __shared__ OctWarp s_warp[WARPS];
  const uint32_t u = d_u ? *d_u : u_host;
  if (u == 0) return;
  const uint32_t m = u - 1;
  if (m == 0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) octree_root_only<K>(nodes, capacity, mn, rg, status);
    return;
  }
  const OctCloud cl{0u, m, 0u, (prefix_n[0] - A) / 3, nodes, capacity};
  const int lane = threadIdx.x & 31;
  OctWarp& S = s_warp[threadIdx.x >> 5];
  uint32_t qn = 0;  // warp-uniform
  const uint32_t warps = gridDim.x * WARPS;
  for (uint32_t base = (blockIdx.x * WARPS + (threadIdx.x >> 5)) * 32; base < m; base += warps * 32) {
    const uint32_t k = base + lane;
    const bool act = k < m && (k == 0 || edge[k] > 0);
    const uint32_t bal = __ballot_sync(0xffffffffu, act);
    if (act) S.q[qn + __popc(bal & ((1u << lane) - 1u))] = k;
    qn += __popc(bal);
    __syncwarp();
    if (qn >= 32) {
      const uint32_t kk = S.q[lane];
      const uint32_t rest = (lane + 32 < qn) ? S.q[lane + 32] : 0u;
      __syncwarp();
      if (lane + 32 < qn) S.q[lane] = rest;
      qn -= 32;
      octree_warp_batch<K, WITH_LEAVES>(S, true, kk, cl, codes, prefix_n, hll, hlr, left, edge, ps, mn, rg,
                                        lmask_keep, status);
    }
  }
  if (qn > 0) {
    const uint32_t kk = S.q[lane];
    octree_warp_batch<K, WITH_LEAVES>(S, lane < qn, kk, cl, codes, prefix_n, hll, hlr, left, edge, ps, mn, rg,
                                      lmask_keep, status);
  }
}

template <class K>
cudaError_t launch_octree_make(const Launch& L, const K* codes, const uint32_t* d_u, uint32_t u_host,
                               uint32_t n_max, const uint8_t* prefix_n, const uint8_t* hll, const uint8_t* hlr,
                               const int32_t* left, const uint32_t* edge, const uint32_t* ps, float mn, float rg,
                               gtc_octnode* nodes, uint32_t capacity, bool with_leaves) {
  const uint32_t work = d_u ? n_max : u_host;
  if (work == 0) return cudaSuccess;
  // One resident wave; each warp walks many 32-node slices, so the partial
  // batch at its end is small.
  int occ = 4;  // blocks per SM
  const void* kern = with_leaves ? (const void*)octree_make_kernel<K, true> : (const void*)octree_make_kernel<K, false>;
  if (kernel_setup(kern, OCT_THREADS, 0, &occ) != cudaSuccess) {
    cudaGetLastError();
    occ = 4;
  }
  const uint32_t grid = max(1u, min(ceil_div(work, OCT_THREADS), (uint32_t)(L.num_sms * occ)));
  if (with_leaves)
    return launch_kernel(L, octree_make_kernel<K, true>, grid, OCT_THREADS, 0, codes, d_u, u_host, prefix_n, hll, hlr,
                         left, edge, ps, mn, rg, nodes, capacity, leaf_mask_keep(), L.status);
  return launch_kernel(L, octree_make_kernel<K, false>, grid, OCT_THREADS, 0, codes, d_u, u_host, prefix_n, hll, hlr,
                       left, edge, ps, mn, rg, nodes, capacity, 0xffu, L.status);
}
template cudaError_t launch_octree_make<uint32_t>(const Launch&, const uint32_t*, const uint32_t*, uint32_t, uint32_t,
                                                  const uint8_t*, const uint8_t*, const uint8_t*, const int32_t*,
                                                  const uint32_t*, const uint32_t*, float, float, gtc_octnode*,
                                                  uint32_t, bool);
template cudaError_t launch_octree_make<uint64_t>(const Launch&, const uint64_t*, const uint32_t*, uint32_t, uint32_t,
                                                  const uint8_t*, const uint8_t*, const uint8_t*, const int32_t*,
                                                  const uint32_t*, const uint32_t*, float, float, gtc_octnode*,
                                                  uint32_t, bool);

// k_LinkLeafNodes (octree.comp:188-222) in push form: each leaf child is
// stored into the bottom node of the nearest contributing ancestor (the walk
// stops at the root, D7) and its bit OR-ed into child_leaf_mask (D6).
template <class K>
__global__ void __launch_bounds__(256) octree_link_kernel(const K* __restrict__ codes, uint32_t m,
                                                          const uint8_t* __restrict__ prefix_n,
                                                          const uint8_t* __restrict__ hll,
                                                          const uint8_t* __restrict__ hlr,
                                                          const int32_t* __restrict__ left,
                                                          const int32_t* __restrict__ parent,
                                                          const uint32_t* __restrict__ edge,
                                                          const uint32_t* __restrict__ ps, gtc_octnode* nodes,
                                                          uint32_t capacity, bool leaf_mask, uint32_t* status) {
  constexpr int A = KeyTraits<K>::A;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
    const bool l = hll[i], r = hlr[i];
    if (!l && !r) continue;
    uint32_t rt = i;
    int steps = 0;
    while (edge[rt] == 0 && rt != 0) {
      rt = (uint32_t)parent[rt];
      if (++steps > 64) {
        atomicOr(status, DEV_INTERNAL);
        break;
      }
    }
    const uint32_t slot = (rt == 0) ? 0u : ps[rt] - edge[rt] + 1;
    if (slot >= capacity) {
      atomicOr(status, DEV_CAPACITY);
      continue;
    }
    const int level = (prefix_n[i] - A) / 3 + 1;
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      if (!(side ? r : l)) continue;
      const int32_t leaf = left[i] + side;
      const int w = child_slot<K>(codes[leaf], level);
      nodes[slot].children[w] = leaf;
      if (leaf_mask) atomicOr(&nodes[slot].child_leaf_mask, 1 << w);
    }
  }
}

template <class K>
cudaError_t launch_octree_link(const Launch& L, const K* codes, uint32_t m, const uint8_t* prefix_n,
                               const uint8_t* hll, const uint8_t* hlr, const int32_t* left, const int32_t* parent,
                               const uint32_t* edge, const uint32_t* ps, gtc_octnode* nodes, uint32_t capacity) {
  if (m == 0) return cudaSuccess;
  const uint32_t grid = max(1u, min(ceil_div(m, 256), (uint32_t)L.num_sms * 8));
  octree_link_kernel<K><<<grid, 256, 0, L.stream>>>(codes, m, prefix_n, hll, hlr, left, parent, edge, ps, nodes,
                                                    capacity, leaf_mask_keep() != 0, L.status);
  return cudaGetLastError();
}
template cudaError_t launch_octree_link<uint32_t>(const Launch&, const uint32_t*, uint32_t, const uint8_t*,
                                                  const uint8_t*, const uint8_t*, const int32_t*, const int32_t*,
                                                  const uint32_t*, const uint32_t*, gtc_octnode*, uint32_t);
template cudaError_t launch_octree_link<uint64_t>(const Launch&, const uint64_t*, uint32_t, const uint8_t*,
                                                  const uint8_t*, const uint8_t*, const int32_t*, const int32_t*,
                                                  const uint32_t*, const uint32_t*, gtc_octnode*, uint32_t);

}  // namespace gtc
