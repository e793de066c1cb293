// octree.cu - octree make (pull form, octree_dev.cuh) and the push-form link
// operator for callers that run make and link as separate stages.

#include "octree_dev.cuh"

namespace gtc {

constexpr int OCT_THREADS = 256;
constexpr int OCT_RING = 256;

// Per-warp scratch of the make kernel.
struct OctWarp {
  uint32_t q[64];           // contributing radix nodes waiting for a batch
  int32_t ch[32][8];        // children of the batch's bottom nodes, by lane
  uint32_t mk[32];          // child masks found by the descent rounds (node | leaf << 8)
  uint2 ring[OCT_RING];     // descent candidates {index, owner | leaf << 5 | deep << 6 | level << 8}
};

// A radix child x of an octree node at `level`: its octant, and what the
// node stores for it (leaf: the unique-key index; internal with edge > 0: the
// child's top octree slot).
template <class K>
__device__ __forceinline__ int octant_of(const K* __restrict__ codes, uint32_t x, int level) {
  return child_slot<K>(codes[x], level);
}

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
// Children and masks collect in shared memory, then every lane writes its
// node (4 x 16 B) and the chain nodes above it.
template <class K, bool WITH_LEAVES>
__device__ __forceinline__ void octree_warp_batch(OctWarp& S, bool valid, uint32_t k, uint32_t m,
                                                  const K* __restrict__ codes, const uint8_t* __restrict__ prefix_n,
                                                  const uint8_t* __restrict__ hll, const uint8_t* __restrict__ hlr,
                                                  const int32_t* __restrict__ left, const uint32_t* __restrict__ edge,
                                                  const uint32_t* __restrict__ ps, uint32_t ps_bias, int root_level,
                                                  float mn, float rg, gtc_octnode* __restrict__ nodes,
                                                  uint32_t capacity, uint32_t lmask_keep, uint32_t* status) {
  constexpr int A = KeyTraits<K>::A;
  const int lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  bool ok = valid;
  uint32_t c = 0, top = 0, lc = 0, fl = 0;
  K code_k = 0;
  int dk = 0;
  if (ok) {
    c = edge[k];
    top = ps[k] - ps_bias;
    code_k = codes[k];
    dk = (prefix_n[k] - A) / 3;
    lc = (uint32_t)left[k];
    fl = (uint32_t)(hll[k] != 0) | ((uint32_t)(hlr[k] != 0) << 1);
    if (k != 0 && c > top) {  // slot 0 is the root's: inconsistent offsets
      atomicOr(status, DEV_INTERNAL);
      ok = false;
    } else if ((k == 0 ? 1u : top + 1) > capacity) {
      atomicOr(status, DEV_CAPACITY);
      ok = false;
    } else if (lc + 1 > m || ((fl & 1) == 0 && lc >= m) || ((fl & 2) == 0 && lc + 1 >= m)) {
      atomicOr(status, DEV_INTERNAL);
      ok = false;
    }
  }
  const int level = dk + 1;
  int4* chl = reinterpret_cast<int4*>(S.ch[lane]);
  chl[0] = make_int4(0, 0, 0, 0);
  chl[1] = make_int4(0, 0, 0, 0);
  S.mk[lane] = 0;
  uint32_t nmask = 0, lmask = 0;

  // Level 1: both radix children of k.
  bool dsc[2] = {false, false};
  uint32_t dl[2] = {0, 0}, df[2] = {0, 0};
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const uint32_t x = lc + side;
    const bool leaf = (fl >> side) & 1;
    if (ok && leaf) {
      if (WITH_LEAVES) {
        const int w = octant_of<K>(codes, x, level);
        S.ch[lane][w] = (int32_t)x;
        lmask |= 1u << w;
      }
    } else if (ok) {
      const uint32_t e = edge[x];
      const K cx = codes[x];
      const uint32_t p = ps[x];
      const uint32_t lx = (uint32_t)left[x];
      const uint32_t f = (uint32_t)(hll[x] != 0) | ((uint32_t)(hlr[x] != 0) << 1);
      if (e > 0) {
        const int w = child_slot<K>(cx, level);
        S.ch[lane][w] = (int32_t)(p - ps_bias);
        nmask |= 1u << w;
      } else {
        dsc[side] = true;
        dl[side] = lx;
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
        S.ring[pos] = make_uint2(dl[side], meta | ((df[side] & 1u) << 5));
        S.ring[pos + 1] = make_uint2(dl[side] + 1, meta | ((df[side] >> 1) << 5));
        pos += 2;
      }
    }
  }
  __syncwarp();

  // Descent rounds over the ring (FIFO; live entries are [head, tail)).
  uint32_t head = 0;
  while (head < tail) {  // warp-uniform
    const uint32_t idx = head + lane;
    const bool have = idx < tail;
    const uint2 en = have ? S.ring[idx % OCT_RING] : make_uint2(0, 0);
    const uint32_t y = en.x, owner = en.y & 31u;
    const bool leaf = (en.y >> 5) & 1u, deep = (en.y >> 6) & 1u;
    const int lev = (int)(en.y >> 8);
    bool push = false;
    uint32_t ly = 0, fy = 0;
    if (have && (leaf ? y >= m + 1 : y >= m)) {
      atomicOr(status, DEV_INTERNAL);
    } else if (have && leaf) {
      if (WITH_LEAVES) {
        const int w = octant_of<K>(codes, y, lev);
        S.ch[owner][w] = (int32_t)y;
        atomicOr(&S.mk[owner], 1u << (8 + w));
      }
    } else if (have) {
      const uint32_t e = edge[y];
      const K cy = codes[y];
      const uint32_t p = ps[y];
      if (deep) {
        ly = (uint32_t)left[y];
        fy = (uint32_t)(hll[y] != 0) | ((uint32_t)(hlr[y] != 0) << 1);
      }
      if (e > 0) {
        const int w = child_slot<K>(cy, lev);
        S.ch[owner][w] = (int32_t)(p - ps_bias);
        atomicOr(&S.mk[owner], 1u << w);
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
      S.ring[pos % OCT_RING] = make_uint2(ly, meta | ((fy & 1u) << 5));
      S.ring[(pos + 1) % OCT_RING] = make_uint2(ly + 1, meta | ((fy >> 1) << 5));
    }
    tail += npush;
    __syncwarp();
  }

  if (ok) {
    const int4 a = chl[0], b = chl[1];
    const uint32_t mk = S.mk[lane];
    nmask |= mk & 0xffu;
    lmask = (lmask | (mk >> 8)) & lmask_keep;
    const uint32_t bottom = (k == 0) ? 0u : top - c + 1;
    // Corners from the cell coordinates decoded once; cell sizes rg / 2^k as
    // the exact scaling rg * 2^-k (octree.comp:111-116, 181-182).
    const uint3 qc = code_xyz<K>(code_k);
    store_node(nodes, bottom, a, b, corner_at<K>(qc, dk, mn, rg), __fmul_rn(rg, exp2_neg(dk - root_level)),
               (int32_t)nmask, (int32_t)lmask);
    // Chain nodes above the bottom (levels dk - 1 .. dk - c + 1).
    for (uint32_t j = 1; j < c; ++j) {
      const int lv = dk - (int)j;
      int4 ca = make_int4(0, 0, 0, 0), cb = make_int4(0, 0, 0, 0);
      const int w = child_slot<K>(code_k, lv + 1);
      set_child(ca, cb, w, (int32_t)(bottom + j - 1));
      store_node(nodes, bottom + j, ca, cb, corner_at<K>(qc, lv, mn, rg), __fmul_rn(rg, exp2_neg(lv - root_level)),
                 1 << w, 0);
    }
  }
  __syncwarp();  // the batch's scratch is free again
}

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
  const int root_level = (prefix_n[0] - A) / 3;
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
      octree_warp_batch<K, WITH_LEAVES>(S, true, kk, m, codes, prefix_n, hll, hlr, left, edge, ps, 0u, root_level,
                                        mn, rg, nodes, capacity, lmask_keep, status);
    }
  }
  if (qn > 0) {
    const uint32_t kk = S.q[lane];
    octree_warp_batch<K, WITH_LEAVES>(S, lane < qn, kk, m, codes, prefix_n, hll, hlr, left, edge, ps, 0u, root_level,
                                      mn, rg, nodes, capacity, lmask_keep, status);
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
  static int resident[2] = {0, 0};  // blocks per SM of each instantiation, queried once
  int& occ = resident[with_leaves ? 1 : 0];
  if (occ == 0) {
    const void* kern = with_leaves ? (const void*)octree_make_kernel<K, true> : (const void*)octree_make_kernel<K, false>;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, OCT_THREADS, 0) != cudaSuccess || occ < 1) {
      cudaGetLastError();
      occ = 4;
    }
  }
  const uint32_t grid = max(1u, min(ceil_div(work, OCT_THREADS), (uint32_t)(L.num_sms * occ)));
  if (with_leaves)
    octree_make_kernel<K, true><<<grid, OCT_THREADS, 0, L.stream>>>(codes, d_u, u_host, prefix_n, hll, hlr, left,
                                                                     edge, ps, mn, rg, nodes, capacity,
                                                                     leaf_mask_keep(), L.status);
  else
    octree_make_kernel<K, false><<<grid, OCT_THREADS, 0, L.stream>>>(codes, d_u, u_host, prefix_n, hll, hlr, left,
                                                                      edge, ps, mn, rg, nodes, capacity, 0xffu,
                                                                      L.status);
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
