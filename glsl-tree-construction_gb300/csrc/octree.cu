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

constexpr int OCT_THREADS = 256;

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

// children[w] = v with w known only at run time, kept in registers.
__device__ __forceinline__ void set_child(int4& lo, int4& hi, int w, int32_t v) {
  lo.x = (w == 0) ? v : lo.x;
  lo.y = (w == 1) ? v : lo.y;
  lo.z = (w == 2) ? v : lo.z;
  lo.w = (w == 3) ? v : lo.w;
  hi.x = (w == 4) ? v : hi.x;
  hi.y = (w == 5) ? v : hi.y;
  hi.z = (w == 6) ? v : hi.z;
  hi.w = (w == 7) ? v : hi.w;
}

// Writes one 64-byte node (four 16-byte stores), straight to HBM or into a
// staging area.
struct NodeSink {
  int4* stage;
  gtc_octnode* nodes;
  uint32_t first;
  bool staged;
  __device__ __forceinline__ void put(uint32_t slot, int4 a, int4 b, int4 c, int4 d) const {
    int4* p = staged ? stage + (size_t)(slot - first) * 4 : reinterpret_cast<int4*>(nodes + slot);
    p[0] = a;
    p[1] = b;
    p[2] = c;
    p[3] = d;
  }
};

// Children of the bottom octree node of radix node k: descend from q through
// internal children of the same depth (edge == 0); a depth band holds at
// most three prefix lengths, so LEVEL never exceeds 2 on valid input.
template <class K, bool WITH_LEAVES, int LEVEL>
__device__ __forceinline__ void gather(uint32_t q, int level, const K* __restrict__ codes,
                                       const uint8_t* __restrict__ hll, const uint8_t* __restrict__ hlr,
                                       const int32_t* __restrict__ left, const uint32_t* __restrict__ edge,
                                       const uint32_t* __restrict__ ps, int4& lo, int4& hi, int32_t& nmask,
                                       int32_t& lmask, uint32_t* status) {
  const int32_t lc = left[q];
  const bool leaf_side[2] = {hll[q] != 0, hlr[q] != 0};
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const uint32_t x = (uint32_t)(lc + side);
    if (leaf_side[side]) {
      if (WITH_LEAVES) {
        const int w = child_slot<K>(codes[x], level);
        set_child(lo, hi, w, (int32_t)x);
        lmask |= 1 << w;
      }
    } else {
      const uint32_t e = edge[x];
      if (e > 0) {
        const int w = child_slot<K>(codes[x], level);
        set_child(lo, hi, w, (int32_t)ps[x]);
        nmask |= 1 << w;
      } else if (LEVEL < 2) {
        gather<K, WITH_LEAVES, (LEVEL < 2 ? LEVEL + 1 : 2)>(x, level, codes, hll, hlr, left, edge, ps, lo, hi, nmask,
                                                            lmask, status);
      } else {
        atomicOr(status, DEV_INTERNAL);
      }
    }
  }
}

template <class K, bool WITH_LEAVES>
__global__ void __launch_bounds__(OCT_THREADS) octree_make_kernel(const K* __restrict__ codes, const uint32_t* d_u,
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
      const float4 c = decode_corner<K>((K)0, mn, rg);
      NodeSink sink{nullptr, nodes, 0, false};
      sink.put(0, make_int4(0, 0, 0, 0), make_int4(0, 0, 0, 0),
               make_int4(__float_as_int(c.x), __float_as_int(c.y), __float_as_int(c.z), __float_as_int(c.w)),
               make_int4(__float_as_int(rg), 0, 0, 0));
    }
    return;
  }
  const int root_level = (prefix_n[0] - A) / 3;
  // The kernel is bound by the latency of its dependent loads (node -> child
  // -> grandchild), not by bandwidth: one thread per radix node, no block
  // barriers, 16-byte stores straight to HBM.
  const NodeSink sink{nullptr, nodes, 0, false};
  const uint32_t stride = gridDim.x * OCT_THREADS;
  for (uint32_t k = blockIdx.x * OCT_THREADS + threadIdx.x; k < m; k += stride) {
    {
      const uint32_t c = edge[k];
      const uint32_t top = ps[k];
      if (k == 0 || c > 0) {
        if (k != 0 && c > top) {  // slot 0 is the root's: inconsistent offsets
          atomicOr(status, DEV_INTERNAL);
        } else if ((k == 0 ? 1u : top + 1) > capacity) {
          atomicOr(status, DEV_CAPACITY);
        } else {
          const uint32_t bottom = (k == 0) ? 0u : top - c + 1;
          const K code_k = codes[k];
          const int dk = (prefix_n[k] - A) / 3;
          int4 lo = make_int4(0, 0, 0, 0), hi = make_int4(0, 0, 0, 0);
          int32_t nmask = 0, lmask = 0;
          gather<K, WITH_LEAVES, 0>(k, dk + 1, codes, hll, hlr, left, edge, ps, lo, hi, nmask, lmask, status);
          float4 cr = decode_corner<K>(level_prefix<K>(code_k, dk), mn, rg);
          float cell = __fdiv_rn(rg, (float)(1u << (dk - root_level)));
          sink.put(bottom, lo, hi,
                   make_int4(__float_as_int(cr.x), __float_as_int(cr.y), __float_as_int(cr.z), __float_as_int(cr.w)),
                   make_int4(__float_as_int(cell), nmask, lmask, 0));
          // Chain nodes above the bottom (levels dk - 1 .. dk - c + 1).
          for (uint32_t j = 1; j < c; ++j) {
            const int level = dk - (int)j;
            int4 a = make_int4(0, 0, 0, 0), b = make_int4(0, 0, 0, 0);
            const int w = child_slot<K>(code_k, level + 1);
            set_child(a, b, w, (int32_t)(bottom + j - 1));
            cr = decode_corner<K>(level_prefix<K>(code_k, level), mn, rg);
            cell = __fdiv_rn(rg, (float)(1u << (level - root_level)));
            sink.put(bottom + j, a, b,
                     make_int4(__float_as_int(cr.x), __float_as_int(cr.y), __float_as_int(cr.z),
                               __float_as_int(cr.w)),
                     make_int4(__float_as_int(cell), 1 << w, 0, 0));
          }
        }
      }
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
  const uint32_t grid = max(1u, min(ceil_div(work, OCT_THREADS), (uint32_t)L.num_sms * 16));
  if (with_leaves)
    octree_make_kernel<K, true><<<grid, OCT_THREADS, 0, L.stream>>>(codes, d_u, u_host, prefix_n, hll, hlr, left, edge, ps,
                                                             mn, rg, nodes, capacity, L.status);
  else
    octree_make_kernel<K, false><<<grid, OCT_THREADS, 0, L.stream>>>(codes, d_u, u_host, prefix_n, hll, hlr, left, edge, ps,
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
