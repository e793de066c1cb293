/*
 * oracle.h - CPU restatement of the point-cloud -> octree path of
 * ucsc-redwood/glsl-tree-construction (vulkan/radixsort-vulkan).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py (its CPU-baseline leg and
 * its `--impl reference` arm) may load it.  The product library never links,
 * loads or calls it, and nothing in the product falls back to it.
 *
 * Parity status: pinned to the reference's own code.  The reference (Rust
 * host + GLSL compute shaders) cannot run here (no Rust toolchain, no
 * graphics stack), but its shader function bodies are C-like:
 * oracle/ref_shaders.py compiles the function bodies of morton.comp,
 * unique.comp, build_radix_tree.comp, edge_count.comp, partial_sum.comp and
 * octree.comp as written, as C++ on the CPU (oracle/_ref/, with ref_glue.cpp supplying the
 * GLSL names and the host steps of main.rs:60-170), once per set of named
 * deviation patches.  tests/test_oracle_ref_pin.py checks every stage here
 * against that build byte for byte: the corrected forms against the fully
 * patched shaders, each ORC_LITERAL_* switch against the shaders with that one
 * deviation left in, and the 64-bit forms against the shaders with 64-bit
 * codes substituted.  tests/golden/ref_pipeline_{32,64}.npz hold that build's
 * outputs for machines without the reference checkout.  The global digit
 * histogram of `test_radix_sort` (output.txt:7684-8707) is reproduced by
 * orc_global_hist_u32(..., ORC_LITERAL_D11) up to a constant offset of 9n on
 * every bin d >= 1 (tests/test_oracle_pin.py).  The 64-bit Morton encode has
 * no reference counterpart and is checked against known answers.
 *
 * Reference-intent corrections (default) and the switches that restore the
 * literal form where the literal form is deterministic:
 *   D1  radix-tree direction computed signed (build_radix_tree.comp:79-82 uses
 *       uint8_t, so d is never -1).  ORC_LITERAL_D1 reproduces the literal
 *       form sequentially (last writer wins in index order).
 *   D2  depth = (prefix_n - A) / 3, A = key bits - 3*bits per axis
 *       (edge_count.comp:34, octree.comp:127 use prefix_n / 3).  ORC_LITERAL_D2.
 *   D3  octree slot base(i) = ps[i] - edge[i] + 1 (octree.comp:130 uses ps[i]).
 *       ORC_LITERAL_D3.
 *   D4  per-node stages run over exactly m = u - 1 nodes; the element past the
 *       end of edge[] reads as 0 (main.rs:120,128,164).
 *   D5  cell sizes relative to the depth of the tree root (octree.comp:127).
 *   D6  SetLeaf sets the leaf-mask bit (octree.comp:29 clears it from 0).
 *       ORC_LITERAL_D6.
 *   D7  walks to the nearest contributing ancestor stop at the root, which owns
 *       octree slot 0 (octree.comp:157-165,199-201 have no/ a 30-step cap).
 *   D8  link runs after make completes (octree.comp:229-236 is commented out).
 *   D9  OctNode is the 64-byte std430 layout (octree.comp:14-20).
 *   D10 IEEE round-to-nearest float ops, no contraction (compile with
 *       -ffp-contract=off).
 *   D11 correct digit histograms (histogram.comp:128 masks with 0xF).
 *       ORC_LITERAL_D11.
 *   D13 parent[0] = 0 written explicitly.
 *   D15 has_leaf_* stored as one byte 0/1.
 *   D16 the root covers all u keys: l = m for i = 0
 *       (build_radix_tree.comp:90-91 sets l = n - 1 with n = m, which drops the
 *       last key whenever the top split falls at it).  ORC_LITERAL_D16.
 *   D17 float -> unsigned conversion in Morton encode saturates (NaN -> 0,
 *       negative -> 0, >= 2^32 -> 2^32-1) before the axis mask; the GLSL
 *       conversion is undefined outside [0, 2^32).
 *   D18 u == 1 (one distinct key): m = 0, a single root node with corner =
 *       decode(0), cell = range and no children; u == 0: nothing.
 */
#ifndef GTC_ORACLE_H
#define GTC_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_LITERAL_D1 = 1u << 1,
  ORC_LITERAL_D2 = 1u << 2,
  ORC_LITERAL_D3 = 1u << 3,
  ORC_LITERAL_D6 = 1u << 6,
  ORC_LITERAL_D11 = 1u << 11,
  ORC_LITERAL_D16 = 1u << 16,
};

/* 64-byte octree node, std430 layout of octree.comp:14-20 (D9). */
typedef struct orc_octnode {
  int32_t children[8];
  float corner[4];
  float cell_size;
  int32_t child_node_mask;
  int32_t child_leaf_mask;
  int32_t _pad;
} orc_octnode;

/* Morton encode, morton.comp:36-67.  pts is float[n][4].  keys32: 10 bits per
 * axis; keys64: 21 bits per axis (same rounding, extended masks). */
void orc_morton32(const float* pts, uint32_t n, float min_coord, float range, uint32_t* keys);
void orc_morton64(const float* pts, uint32_t n, float min_coord, float range, uint64_t* keys);
/* Morton decode, morton.rs:43-74 / octree.comp:87-124. */
void orc_morton32_to_xyz(float* ret4, uint32_t code, float min_coord, float range);
void orc_morton64_to_xyz(float* ret4, uint64_t code, float min_coord, float range);

/* Global digit histograms as exclusive prefixes, histogram.comp:103-195
 * (layout b_globalHist[pass*256 + digit]).  passes = ceil(key_bits / 8). */
void orc_global_hist_u32(const uint32_t* keys, uint32_t n, int passes, uint32_t* hist, uint32_t flags);
void orc_global_hist_u64(const uint64_t* keys, uint32_t n, int passes, uint32_t* hist);

/* Stable sort of (key, value) pairs by key (main.rs:85; new_radix_sort.comp is
 * a stable LSD sort).  threads > 1 uses a chunked stable sort + stable merges. */
void orc_sort_pairs_u32(uint32_t* keys, uint32_t* vals, uint32_t n, int threads);
void orc_sort_pairs_u64(uint64_t* keys, uint32_t* vals, uint32_t n, int threads);

/* unique.comp:31-45: keep the first of each run, in place; vals may be NULL. */
uint32_t orc_unique_u32(uint32_t* keys, uint32_t* vals, uint32_t n);
uint32_t orc_unique_u64(uint64_t* keys, uint32_t* vals, uint32_t n);

/* Karras radix tree, build_radix_tree.comp:44-153, over m = n_brt_nodes
 * internal nodes (codes has m + 1 entries).  Returns the number of parent
 * slots written more than once (0 unless ORC_LITERAL_D1 / D16). */
uint32_t orc_radix_tree_u32(const uint32_t* codes, int32_t m, uint8_t* prefix_n, uint8_t* has_leaf_left,
                            uint8_t* has_leaf_right, int32_t* left_child, int32_t* parent, uint32_t flags);
uint32_t orc_radix_tree_u64(const uint64_t* codes, int32_t m, uint8_t* prefix_n, uint8_t* has_leaf_left,
                            uint8_t* has_leaf_right, int32_t* left_child, int32_t* parent, uint32_t flags);

/* edge_count.comp:30-41, over exactly m nodes (D4).  unused_bits = A. */
void orc_edge_count(const uint8_t* prefix_n, const int32_t* parent, uint32_t m, int unused_bits,
                    uint32_t* edge, uint32_t flags);

/* partial_sum.comp:23-39 + main.rs:127-129: inclusive scan of edge over
 * [0, u) (edge[m] reads as 0), then ps[0] = 0.  Returns ps[u-1]. */
uint32_t orc_prefix_sum(const uint32_t* edge, uint32_t u, uint32_t* ps);

/* Octree make (octree.comp:126-186) then link (octree.comp:188-222) after the
 * root setup of main.rs:140-153.  nodes must hold o = 1 + ps[u-1] entries and
 * is zero-initialised here.  Returns o; *conflicts counts child slots written
 * twice, *walk_cap_hits counts ancestor walks that hit the step cap. */
uint32_t orc_octree_u32(const uint32_t* codes, uint32_t u, const uint8_t* prefix_n, const uint8_t* has_leaf_left,
                        const uint8_t* has_leaf_right, const int32_t* left_child, const int32_t* parent,
                        const uint32_t* edge, const uint32_t* ps, float min_coord, float range,
                        orc_octnode* nodes, uint32_t flags, uint32_t* conflicts, uint32_t* walk_cap_hits);
uint32_t orc_octree_u64(const uint64_t* codes, uint32_t u, const uint8_t* prefix_n, const uint8_t* has_leaf_left,
                        const uint8_t* has_leaf_right, const int32_t* left_child, const int32_t* parent,
                        const uint32_t* edge, const uint32_t* ps, float min_coord, float range,
                        orc_octnode* nodes, uint32_t flags, uint32_t* conflicts, uint32_t* walk_cap_hits);

/* Structural validation of a built octree: every non-root node has exactly one
 * parent link, every unique key appears as exactly one leaf child, masks match
 * the children written, cell sizes halve per level.  Returns 0 when valid,
 * otherwise a nonzero code naming the first failed check. */
int orc_validate_octree(const orc_octnode* nodes, uint32_t o, uint32_t u, float range);

/* Whole path with caller-owned outputs sized for n (see gtc.h).  key_bits is
 * 32 (10 bits/axis) or 64 (21 bits/axis).  keys: uint32_t or uint64_t[n].
 * counts[0] = u, counts[1] = m, counts[2] = o.  threads: sort threads.
 * stage_ms (nullable, 8 entries) receives per-stage wall times. */
int orc_build_octree(const float* pts, uint32_t n, float min_coord, float range, int key_bits, void* keys,
                     uint32_t* idx, uint8_t* prefix_n, uint8_t* has_leaf_left, uint8_t* has_leaf_right,
                     int32_t* left_child, int32_t* parent, uint32_t* edge, uint32_t* ps, orc_octnode* nodes,
                     uint32_t* counts, uint32_t flags, int threads, double* stage_ms);

int orc_max_threads(void);

/* Learned-bucket model (no reference counterpart): loss and gradient of the
 * piecewise-linear CDF with knots kn[0..B] and heights y[0..B] on a sorted
 * sample s[0..ns): L = mean_j (F(s_j) - (j + 0.5)/ns)^2, F linear inside
 * segment [kn[k], kn[k+1]) (the segment of a key is the last knot <= key).
 * Double precision; the checker of the GPU backward kernel. */
double orc_pwl_loss_grad(const uint64_t* sample, uint32_t ns, const uint64_t* kn, const float* y, int B,
                         double* grad);
/* Bucket of each key under the model, the GPU's FP32 bucket line operation
 * for operation: in the key's segment s (last knot <= key),
 * t = B*y[s] + c * float(key - kn[s]) with c = B*(y[s+1] - y[s]) /
 * float(kn[s+1] - kn[s]), clamped to B*y[s+1], truncated. */
void orc_pwl_buckets(const uint64_t* keys, uint32_t n, const uint64_t* kn, const float* y, int B, uint32_t* out);

#ifdef __cplusplus
}
#endif
#endif
