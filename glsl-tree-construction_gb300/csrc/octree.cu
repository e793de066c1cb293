// octree.cu - octree make and link.
//
// Reference: k_MakeOctNodes / k_LinkLeafNodes (octree.comp:126-222) push every
// child pointer into its parent node: chain links inside a radix node's run of
// octree nodes, the run's top node into the bottom node of the nearest
// contributing ancestor (a walk up the radix tree), and leaves into the
// bottom node of their radix node's nearest contributing ancestor.  Those
// pushes need a cleared node array, read-modify-write masks and a grid-wide
// ordering between make and link (D8).
//
// Here each octree node is written exactly once, whole (64 B), by the thread
// of the radix node that owns it (pull form):
//   * radix node k with edge[k] = c > 0 owns slots [ps[k] - c + 1, ps[k]]
//     (bottom .. top, levels depth(k) .. depth(k) - c + 1); the root radix
//     node owns slot 0 (level = depth(0));
//   * chain node above the bottom: its one child is the slot below it;
//   * the bottom node's children are gathered by descending from k through
//     internal children with edge == 0 (same depth, at most two levels): an
//     internal child ch with edge[ch] > 0 contributes its top slot ps[ch];
//     a leaf child contributes its unique-key index.
// This is the same relation the reference's ancestor walk computes
// (checked slot for slot against the oracle), with no atomics and no clearing.

#include "gtc_internal.cuh"

namespace gtc {

template <class K>
__device__ __forceinline__ void store_node(gtc_octnode* nodes, uint32_t slot, const int32_t ch[8], float4 corner,
                                           float cell, int32_t nmask, int32_t lmask) {
  int4* p = reinterpret_cast<int4*>(nodes + slot);
  p[0] = make_int4(ch[0], ch[1], ch[2], ch[3]);
  p[1] = make_int4(ch[4], ch[5], ch[6], ch[7]);
  p[2] = make_int4(__float_as_int(corner.x), __float_as_int(corner.y), __float_as_int(corner.z),
                   __float_as_int(corner.w));
  p[3] = make_int4(__float_as_int(cell), nmask, lmask, 0);
}

template <class K>
__device__ __forceinline__ K level_prefix(K code, int level) {  // top 3*level bits, kept in place
  constexpr int B = KeyTraits<K>::B;
  const int sh = 3 * B - 3 * level;
  return (code >> sh) << sh;
}

template <class K>
__device__ __forceinline__ int child_slot(K code, int level) {  // octant at `level`
  constexpr int B = KeyTraits<K>::B;
  return (int)((code >> (3 * B - 3 * level)) & 7);
}

template <class K, bool WITH_LEAVES>
__global__ void __launch_bounds__(256) octree_make_kernel(const K* __restrict__ codes, const uint32_t* d_u,
                                                          uint32_t u_host, const uint8_t* __restrict__ prefix_n,
                                                          const uint8_t* __restrict__ hll,
                                                          const uint8_t* __restrict__ hlr,
                                                          const int32_t* __restrict__ left,
                                                          const uint32_t* __restrict__ edge,
                                                          const uint32_t* __restrict__ ps, float mn, float rg,
                                                          gtc_octnode* __restrict__ nodes, uint32_t capacity,
                                                          uint32_t* status) {
  constexpr int A = KeyTraits<K>::A;
  const uint32_t u = d_u ? *d_u : u_host;
  if (u == 0) return;
  const uint32_t m = u - 1;
  if (m == 0) {  // D18: one distinct key, a root without children
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      if (capacity < 1) {
        atomicOr(status, DEV_CAPACITY);
        return;
      }
      const int32_t none[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      store_node<K>(nodes, 0, none, decode_corner<K>((K)0, mn, rg), rg, 0, 0);
    }
    return;
  }
  const int root_level = (prefix_n[0] - A) / 3;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += stride) {
    const uint32_t c = edge[k];
    if (c == 0 && k != 0) continue;
    const K code_k = codes[k];
    const int dk = (prefix_n[k] - A) / 3;
    const uint32_t top = ps[k];
    const uint32_t bottom = (k == 0) ? 0u : top - c + 1;
    if (k != 0 && c > top) {  // slot 0 is the root's: inconsistent offsets
      atomicOr(status, DEV_INTERNAL);
      continue;
    }
    if ((k == 0 ? 1u : top + 1) > capacity) {
      atomicOr(status, DEV_CAPACITY);
      continue;
    }
    // Bottom node: gather children through same-depth descendants.
    int32_t ch[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int32_t nmask = 0, lmask = 0;
    uint32_t stack[4];
    int sp = 0;
    stack[sp++] = k;
    while (sp > 0) {
      const uint32_t q = stack[--sp];
      const int32_t lc = left[q];
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        const uint32_t x = (uint32_t)(lc + side);
        const bool leaf = side ? hlr[q] : hll[q];
        if (leaf) {
          if (WITH_LEAVES) {
            const int w = child_slot<K>(codes[x], dk + 1);
            ch[w] = (int32_t)x;
            lmask |= 1 << w;
          }
        } else if (edge[x] > 0) {
          const int w = child_slot<K>(codes[x], dk + 1);
          ch[w] = (int32_t)ps[x];
          nmask |= 1 << w;
        } else if (sp < 4) {
          stack[sp++] = x;
        } else {
          atomicOr(status, DEV_INTERNAL);
        }
      }
    }
    store_node<K>(nodes, bottom, ch, decode_corner<K>(level_prefix<K>(code_k, dk), mn, rg),
                  __fdiv_rn(rg, (float)(1u << (dk - root_level))), nmask, lmask);
    // Chain nodes above the bottom (levels dk - 1 .. dk - c + 1).
    for (uint32_t j = 1; j < c; ++j) {
      const int level = dk - (int)j;
      int32_t one[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      const int w = child_slot<K>(code_k, level + 1);
      one[w] = (int32_t)(bottom + j - 1);
      store_node<K>(nodes, bottom + j, one, decode_corner<K>(level_prefix<K>(code_k, level), mn, rg),
                    __fdiv_rn(rg, (float)(1u << (level - root_level))), 1 << w, 0);
    }
  }
}

template <class K>
cudaError_t launch_octree_make(const Launch& L, const K* codes, const uint32_t* d_u, uint32_t u_host,
                               uint32_t n_max, const uint8_t* prefix_n, const uint8_t* hll, const uint8_t* hlr,
                               const int32_t* left, const uint32_t* edge, const uint32_t* ps, float mn, float rg,
                               gtc_octnode* nodes, uint32_t capacity, bool with_leaves) {
  const uint32_t work = d_u ? n_max : u_host;
  if (work == 0) return cudaSuccess;
  const uint32_t grid = max(1u, min(ceil_div(work, 256), (uint32_t)L.num_sms * 8));
  if (with_leaves)
    octree_make_kernel<K, true><<<grid, 256, 0, L.stream>>>(codes, d_u, u_host, prefix_n, hll, hlr, left, edge, ps,
                                                             mn, rg, nodes, capacity, L.status);
  else
    octree_make_kernel<K, false><<<grid, 256, 0, L.stream>>>(codes, d_u, u_host, prefix_n, hll, hlr, left, edge, ps,
                                                              mn, rg, nodes, capacity, L.status);
  return cudaGetLastError();
}
template cudaError_t launch_octree_make<uint32_t>(const Launch&, const uint32_t*, const uint32_t*, uint32_t, uint32_t,
                                                  const uint8_t*, const uint8_t*, const uint8_t*, const int32_t*,
                                                  const uint32_t*, const uint32_t*, float, float, gtc_octnode*,
                                                  uint32_t, bool);
template cudaError_t launch_octree_make<uint64_t>(const Launch&, const uint64_t*, const uint32_t*, uint32_t, uint32_t,
                                                  const uint8_t*, const uint8_t*, const uint8_t*, const int32_t*,
                                                  const uint32_t*, const uint32_t*, float, float, gtc_octnode*,
                                                  uint32_t, bool);

// k_LinkLeafNodes (octree.comp:188-222) in push form, for callers that run
// make and link as separate operators: each leaf child is stored into the
// bottom node of the nearest contributing ancestor (the walk stops at the
// root, D7) and its bit OR-ed into child_leaf_mask (D6).
template <class K>
__global__ void __launch_bounds__(256) octree_link_kernel(const K* __restrict__ codes, uint32_t m,
                                                          const uint8_t* __restrict__ prefix_n,
                                                          const uint8_t* __restrict__ hll,
                                                          const uint8_t* __restrict__ hlr,
                                                          const int32_t* __restrict__ left,
                                                          const int32_t* __restrict__ parent,
                                                          const uint32_t* __restrict__ edge,
                                                          const uint32_t* __restrict__ ps, gtc_octnode* nodes,
                                                          uint32_t capacity, uint32_t* status) {
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
      atomicOr(&nodes[slot].child_leaf_mask, 1 << w);
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
                                                    capacity, L.status);
  return cudaGetLastError();
}
template cudaError_t launch_octree_link<uint32_t>(const Launch&, const uint32_t*, uint32_t, const uint8_t*,
                                                  const uint8_t*, const uint8_t*, const int32_t*, const int32_t*,
                                                  const uint32_t*, const uint32_t*, gtc_octnode*, uint32_t);
template cudaError_t launch_octree_link<uint64_t>(const Launch&, const uint64_t*, uint32_t, const uint8_t*,
                                                  const uint8_t*, const uint8_t*, const int32_t*, const int32_t*,
                                                  const uint32_t*, const uint32_t*, gtc_octnode*, uint32_t);

}  // namespace gtc
