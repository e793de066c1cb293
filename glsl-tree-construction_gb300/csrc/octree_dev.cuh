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

// One 64-byte node as four 16-byte streaming stores: nothing in the build
// reads the nodes back, so they are marked to leave L2 first and the radix
// tree arrays the octree gathers from stay cached longer.
__device__ __forceinline__ void store_node(gtc_octnode* nodes, uint32_t slot, int4 a, int4 b, float4 corner,
                                           float cell, int32_t nmask, int32_t lmask) {
  int4* p = reinterpret_cast<int4*>(nodes + slot);
  __stcs(p + 0, a);
  __stcs(p + 1, b);
  __stcs(p + 2, make_int4(__float_as_int(corner.x), __float_as_int(corner.y), __float_as_int(corner.z),
                          __float_as_int(corner.w)));
  __stcs(p + 3, make_int4(__float_as_int(cell), nmask, lmask, 0));
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

// ------------------------------------------- warp batches (pull form) --
constexpr int OCT_RING = 256;

// A child slot in shared memory: the child's index with a flag for a present
// child and one for a leaf (indices are < 2^30), so no mask has to be kept
// beside the slots.
constexpr uint32_t OCT_PRESENT = 1u << 31, OCT_LEAF = 1u << 30, OCT_INDEX = OCT_LEAF - 1u;

// Per-warp scratch of the make kernel.
struct OctWarp {
  uint32_t q[64];           // contributing radix nodes waiting for a batch
  uint32_t ch[32][9];       // child slots of the batch's bottom nodes, by lane; rows of 9 words so that
                            // slot w of different lanes, and different slots of one lane, fall in
                            // different banks
  alignas(16) uint2 ring[OCT_RING];  // descent candidates {index, owner | leaf << 5 | deep << 6 | level << 8};
                                     // pushed in pairs at even positions, one 16-byte store per pair
};

// One batch of up to 32 contributing radix nodes, one per lane (k valid when
// `valid`), all 32 lanes taking part.  The bottom node's children are found
// breadth-first so that every step is a full-warp step:
//   level 1  every lane examines both radix children of its node; an internal
//            child with edge > 0 or a leaf is a child of the bottom node, an
//            internal child with edge == 0 (same octree depth) is a descent
//            whose two children go to the warp's ring;
//   rounds   32 ring entries at a time; a depth band holds at most three
//            prefix lengths, so entries pushed by a descent are never
//            descents themselves on valid input (checked).
// Loads of a candidate's own data (edge, code, offset) and of its children
// (left, leaf flags) are issued together, so each level costs one round trip.
// Children collect in shared memory as flagged slots, then every lane writes its
// node (4 x 16 B) and the chain nodes above it.
// Per-lane cloud of a batch node: codes and tree arrays are indexed
// globally, the cloud's keys are [u0, mend] (mend = u0 + its radix nodes),
// left children are cloud-local, and node offsets carry a bias.  A single
// cloud is u0 = 0, bias = 0.
struct OctCloud {
  uint32_t u0, mend, bias;
  int root_level;
  gtc_octnode* nodes;  // the cloud's first octree node
  uint32_t capacity;   // nodes available from there
};

template <class K, bool WITH_LEAVES>
__device__ __forceinline__ void octree_warp_batch(OctWarp& S, bool valid, uint32_t k, const OctCloud& cl,
                                                  const K* __restrict__ codes, const uint8_t* __restrict__ prefix_n,
                                                  const uint8_t* __restrict__ hll, const uint8_t* __restrict__ hlr,
                                                  const int32_t* __restrict__ left, const uint32_t* __restrict__ edge,
                                                  const uint32_t* __restrict__ ps, float mn, float rg,
                                                  uint32_t lmask_keep, uint32_t* status) {
  constexpr int A = KeyTraits<K>::A;
  const int lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  bool ok = valid;
  uint32_t c = 0, top = 0, lc = 0, fl = 0;
  K code_k = 0;
  int dk = 0;
  const uint32_t kl = k - cl.u0;  // cloud-local index of the node
  if (ok) {
    c = edge[k];
    top = ps[k] - cl.bias;
    code_k = codes[k];
    dk = (prefix_n[k] - A) / 3;
    lc = cl.u0 + (uint32_t)left[k];
    fl = (uint32_t)(hll[k] != 0) | ((uint32_t)(hlr[k] != 0) << 1);
    if (kl != 0 && c > top) {  // slot 0 is the root's: inconsistent offsets
      atomicOr(status, DEV_INTERNAL);
      ok = false;
    } else if ((kl == 0 ? 1u : top + 1) > cl.capacity) {
      atomicOr(status, DEV_CAPACITY);
      ok = false;
    } else if (lc < cl.u0 || lc + 1 > cl.mend || ((fl & 1) == 0 && lc >= cl.mend) ||
               ((fl & 2) == 0 && lc + 1 >= cl.mend)) {
      atomicOr(status, DEV_INTERNAL);
      ok = false;
    }
  }
  const int level = dk + 1;
#pragma unroll
  for (int w = 0; w < 8; ++w) S.ch[lane][w] = 0u;

  // Level 1: both radix children of k.
  bool dsc[2] = {false, false};
  uint32_t dl[2] = {0, 0}, df[2] = {0, 0};
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const uint32_t x = lc + side;
    const bool leaf = (fl >> side) & 1;
    if (ok && leaf) {
      if (WITH_LEAVES) {
        const int w = child_slot<K>(codes[x], level);
        S.ch[lane][w] = (x - cl.u0) | OCT_PRESENT | OCT_LEAF;
      }
    } else if (ok) {
      const uint32_t e = edge[x];
      const K cx = codes[x];
      const uint32_t p = ps[x];
      const uint32_t lx = (uint32_t)left[x];
      const uint32_t f = (uint32_t)(hll[x] != 0) | ((uint32_t)(hlr[x] != 0) << 1);
      if (e > 0) {
        const int w = child_slot<K>(cx, level);
        S.ch[lane][w] = (p - cl.bias) | OCT_PRESENT;
      } else {
        dsc[side] = true;
        dl[side] = cl.u0 + lx;
        df[side] = f;
      }
    }
  }
  const uint32_t b0 = __ballot_sync(0xffffffffu, dsc[0]);
  const uint32_t b1 = __ballot_sync(0xffffffffu, dsc[1]);
  uint32_t tail = 2u * (__popc(b0) + __popc(b1));  // <= 128: fits the ring
  {
    uint32_t pos = 2u * (__popc(b0 & lt) + __popc(b1 & lt));
    const uint32_t meta = (uint32_t)lane | (1u << 6) | ((uint32_t)level << 8);
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      if (dsc[side]) {
        *reinterpret_cast<uint4*>(&S.ring[pos]) =
            make_uint4(dl[side], meta | ((df[side] & 1u) << 5), dl[side] + 1, meta | ((df[side] >> 1) << 5));
        pos += 2;
      }
    }
  }
  __syncwarp();

  // Descent rounds over the ring (FIFO; live entries are [head, tail)).  An
  // entry's cloud is its owner lane's (shuffled in).
  uint32_t head = 0;
  while (head < tail) {  // warp-uniform
    const uint32_t idx = head + lane;
    const bool have = idx < tail;
    const uint2 en = have ? S.ring[idx % OCT_RING] : make_uint2(0, 0);
    const uint32_t y = en.x, owner = en.y & 31u;
    const bool leaf = (en.y >> 5) & 1u, deep = (en.y >> 6) & 1u;
    const int lev = (int)(en.y >> 8);
    const uint32_t o_u0 = __shfl_sync(0xffffffffu, cl.u0, owner);
    const uint32_t o_mend = __shfl_sync(0xffffffffu, cl.mend, owner);
    const uint32_t o_bias = __shfl_sync(0xffffffffu, cl.bias, owner);
    bool push = false;
    uint32_t ly = 0, fy = 0;
    if (have && (y < o_u0 || (leaf ? y > o_mend : y >= o_mend))) {
      atomicOr(status, DEV_INTERNAL);
    } else if (have && leaf) {
      if (WITH_LEAVES) {
        const int w = child_slot<K>(codes[y], lev);
        S.ch[owner][w] = (y - o_u0) | OCT_PRESENT | OCT_LEAF;
      }
    } else if (have) {
      const uint32_t e = edge[y];
      const K cy = codes[y];
      const uint32_t p = ps[y];
      if (deep) {
        ly = o_u0 + (uint32_t)left[y];
        fy = (uint32_t)(hll[y] != 0) | ((uint32_t)(hlr[y] != 0) << 1);
      }
      if (e > 0) {
        const int w = child_slot<K>(cy, lev);
        S.ch[owner][w] = (p - o_bias) | OCT_PRESENT;
      } else if (deep) {
        push = true;
      } else {
        atomicOr(status, DEV_INTERNAL);
      }
    }
    head += min(32u, tail - head);
    const uint32_t bp = __ballot_sync(0xffffffffu, push);
    uint32_t npush = 2u * __popc(bp);
    if (tail + npush - head > (uint32_t)OCT_RING) {  // cannot happen on valid input
      if (lane == 0) atomicOr(status, DEV_INTERNAL);
      npush = 0;
      push = false;
    }
    __syncwarp();  // every lane has read its entry before slots are reused
    if (push) {
      const uint32_t pos = tail + 2u * __popc(bp & lt);
      const uint32_t meta = owner | ((uint32_t)lev << 8);
      *reinterpret_cast<uint4*>(&S.ring[pos % OCT_RING]) =  // pos is even: the pair does not wrap
          make_uint4(ly, meta | ((fy & 1u) << 5), ly + 1, meta | ((fy >> 1) << 5));
    }
    tail += npush;
    __syncwarp();
  }

  if (ok) {
    uint32_t cv[8], nmask = 0, lmask = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
      const uint32_t v = S.ch[lane][w];
      if (v & OCT_PRESENT) {
        if (v & OCT_LEAF) lmask |= 1u << w;
        else nmask |= 1u << w;
      }
      cv[w] = v & OCT_INDEX;
    }
    lmask &= lmask_keep;
    const int4 a = make_int4((int)cv[0], (int)cv[1], (int)cv[2], (int)cv[3]);
    const int4 b = make_int4((int)cv[4], (int)cv[5], (int)cv[6], (int)cv[7]);
    const uint32_t bottom = (kl == 0) ? 0u : top - c + 1;
    // Corners from the cell coordinates decoded once; cell sizes rg / 2^k as
    // the exact scaling rg * 2^-k (octree.comp:111-116, 181-182).
    const uint3 qc = code_xyz<K>(code_k);
    store_node(cl.nodes, bottom, a, b, corner_at<K>(qc, dk, mn, rg), __fmul_rn(rg, exp2_neg(dk - cl.root_level)),
               (int32_t)nmask, (int32_t)lmask);
    // Chain nodes above the bottom (levels dk - 1 .. dk - c + 1).
    for (uint32_t j = 1; j < c; ++j) {
      const int lv = dk - (int)j;
      int4 ca = make_int4(0, 0, 0, 0), cb = make_int4(0, 0, 0, 0);
      const int w = child_slot<K>(code_k, lv + 1);
      set_child(ca, cb, w, (int32_t)(bottom + j - 1));
      store_node(cl.nodes, bottom + j, ca, cb, corner_at<K>(qc, lv, mn, rg),
                 __fmul_rn(rg, exp2_neg(lv - cl.root_level)), 1 << w, 0);
    }
  }
  __syncwarp();  // the batch's scratch is free again
}

}  // namespace gtc
