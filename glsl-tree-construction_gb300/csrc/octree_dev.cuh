// octree_dev.cuh - per-radix-node octree construction (pull form), shared by
// the single-cloud and the batched kernels.
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
// This is the same relation the reference's ancestor walk computes (checked
// slot for slot against the oracle), with no atomics and no clearing.
#pragma once

#include "gtc_internal.cuh"

namespace gtc {

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

// One 64-byte node as four 16-byte stores.
__device__ __forceinline__ void store_node(gtc_octnode* nodes, uint32_t slot, int4 a, int4 b, float4 corner,
                                           float cell, int32_t nmask, int32_t lmask) {
  int4* p = reinterpret_cast<int4*>(nodes + slot);
  p[0] = a;
  p[1] = b;
  p[2] = make_int4(__float_as_int(corner.x), __float_as_int(corner.y), __float_as_int(corner.z),
                   __float_as_int(corner.w));
  p[3] = make_int4(__float_as_int(cell), nmask, lmask, 0);
}

// Children of the bottom octree node of radix node k: descend from q through
// internal children of the same depth (edge == 0); a depth band holds at
// most three prefix lengths, so LEVEL never exceeds 2 on valid input.
template <class K, bool WITH_LEAVES, int LEVEL>
__device__ __forceinline__ void gather(uint32_t q, int level, const K* __restrict__ codes,
                                       const uint8_t* __restrict__ hll, const uint8_t* __restrict__ hlr,
                                       const int32_t* __restrict__ left, const uint32_t* __restrict__ edge,
                                       const uint32_t* __restrict__ ps, uint32_t ps_bias, int4& lo, int4& hi,
                                       int32_t& nmask, int32_t& lmask, uint32_t* status) {
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
        set_child(lo, hi, w, (int32_t)(ps[x] - ps_bias));
        nmask |= 1 << w;
      } else if (LEVEL < 2) {
        gather<K, WITH_LEAVES, (LEVEL < 2 ? LEVEL + 1 : 2)>(x, level, codes, hll, hlr, left, edge, ps, ps_bias, lo,
                                                            hi, nmask, lmask, status);
      } else {
        atomicOr(status, DEV_INTERNAL);
      }
    }
  }
}

// D18: a single distinct key gives one root node without children.
template <class K>
__device__ __forceinline__ void octree_root_only(gtc_octnode* nodes, uint32_t capacity, float mn, float rg,
                                                 uint32_t* status) {
  if (capacity < 1) {
    atomicOr(status, DEV_CAPACITY);
    return;
  }
  store_node(nodes, 0, make_int4(0, 0, 0, 0), make_int4(0, 0, 0, 0), decode_corner<K>((K)0, mn, rg), rg, 0, 0);
}

// All octree nodes owned by radix node k (see the top of this file).  Node
// offsets are ps[x] - ps_bias (a bias lets batched clouds share one scan).
template <class K, bool WITH_LEAVES>
__device__ __forceinline__ void octree_make_node(uint32_t k, const K* __restrict__ codes,
                                                 const uint8_t* __restrict__ prefix_n,
                                                 const uint8_t* __restrict__ hll, const uint8_t* __restrict__ hlr,
                                                 const int32_t* __restrict__ left,
                                                 const uint32_t* __restrict__ edge,
                                                 const uint32_t* __restrict__ ps, uint32_t ps_bias, int root_level,
                                                 float mn, float rg, gtc_octnode* __restrict__ nodes,
                                                 uint32_t capacity, uint32_t lmask_keep, uint32_t* status) {
  constexpr int A = KeyTraits<K>::A;
  const uint32_t c = edge[k];
  if (!(k == 0 || c > 0)) return;
  const uint32_t top = ps[k] - ps_bias;
  if (k != 0 && c > top) {  // slot 0 is the root's: inconsistent offsets
    atomicOr(status, DEV_INTERNAL);
    return;
  }
  if ((k == 0 ? 1u : top + 1) > capacity) {
    atomicOr(status, DEV_CAPACITY);
    return;
  }
  const uint32_t bottom = (k == 0) ? 0u : top - c + 1;
  const K code_k = codes[k];
  const int dk = (prefix_n[k] - A) / 3;
  int4 lo = make_int4(0, 0, 0, 0), hi = make_int4(0, 0, 0, 0);
  int32_t nmask = 0, lmask = 0;
  gather<K, WITH_LEAVES, 0>(k, dk + 1, codes, hll, hlr, left, edge, ps, ps_bias, lo, hi, nmask, lmask, status);
  // Corners from the cell coordinates decoded once; cell sizes rg / 2^k as
  // the exact scaling rg * 2^-k (octree.comp:111-116, 181-182).
  const uint3 q = code_xyz<K>(code_k);
  store_node(nodes, bottom, lo, hi, corner_at<K>(q, dk, mn, rg), __fmul_rn(rg, exp2_neg(dk - root_level)), nmask,
             lmask & (int32_t)lmask_keep);
  // Chain nodes above the bottom (levels dk - 1 .. dk - c + 1).
  for (uint32_t j = 1; j < c; ++j) {
    const int level = dk - (int)j;
    int4 a = make_int4(0, 0, 0, 0), b = make_int4(0, 0, 0, 0);
    const int w = child_slot<K>(code_k, level + 1);
    set_child(a, b, w, (int32_t)(bottom + j - 1));
    store_node(nodes, bottom + j, a, b, corner_at<K>(q, level, mn, rg), __fmul_rn(rg, exp2_neg(level - root_level)),
               1 << w, 0);
  }
}

}  // namespace gtc
