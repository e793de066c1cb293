/*
 * gtc.h - C ABI of the GB300-native point-cloud -> octree construction path.
 *
 * Drop-in boundary for the stage-by-stage operator surface of
 * ucsc-redwood/glsl-tree-construction (vulkan/radixsort-vulkan/src/*.rs).
 * Every entry point below names the reference operator it replaces.
 *
 * Two families of entry points:
 *   1. Stream-ordered device entry points (gtc_*): device pointers, caller-owned
 *      buffers, an explicit cudaStream_t, no host synchronisation.  Sizes that
 *      depend on data (unique count, octree node count) stay on the device.
 *   2. Host-buffer shims with the reference's own parameter order (gtc_ref_*):
 *      synchronous, host arrays in and out, like the Rust functions they
 *      replace.  `group_size` (the reference's workgroup count) is accepted and
 *      ignored: launch shapes come from the tuned kernel table.
 *
 * Errors are returned as gtc_status; nothing aborts.  Device-side conditions
 * (a bounded wait that ran out, a capacity overflow) are recorded in a status
 * word that gtc_device_status() reads after synchronising.
 *
 * Key conventions: 32-bit Morton codes carry 10 bits per axis (30 bits used),
 * 64-bit codes carry 21 bits per axis (63 bits used).  Points are float[n][4]
 * (x, y, z, w), 16-byte stride, as in morton.comp:18-20.  All counts < 2^30.
 */
#ifndef GTC_H
#define GTC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GTC_API __attribute__((visibility("default")))
#else
#define GTC_API
#endif

/* A cudaStream_t (0 = legacy default stream). */
typedef void* gtc_stream_t;

typedef enum gtc_status {
  GTC_OK = 0,
  GTC_ERR_INVALID_ARG = 1,
  GTC_ERR_OOM = 2,
  GTC_ERR_CUDA = 3,
  GTC_ERR_TIMEOUT = 4,          /* a bounded device wait ran out */
  GTC_OVERFLOW_FALLBACK = 5,    /* learned path rejected the input; onesweep produced the result */
  GTC_ERR_UNSUPPORTED = 6,
  GTC_ERR_CAPACITY = 7          /* an output buffer was too small (octree nodes) */
} gtc_status;

/* Octree node: the 64-byte std430 layout of octree.comp:14-20
 * (children at 0, corner at 32, cell_size at 48, masks at 52/56). */
typedef struct gtc_octnode {
  int32_t children[8];
  float corner[4];
  float cell_size;
  int32_t child_node_mask;
  int32_t child_leaf_mask;
  int32_t _pad;
} gtc_octnode;

typedef struct gtc_ctx gtc_ctx;

/* ------------------------------------------------------------ context ---- */
GTC_API gtc_status gtc_create(gtc_ctx** out, int device);
GTC_API gtc_status gtc_destroy(gtc_ctx* ctx);
GTC_API const char* gtc_status_string(gtc_status s);
/* Text of the last error raised on this context (empty if none). */
GTC_API const char* gtc_last_error(gtc_ctx* ctx);
/* Synchronises `stream`, then returns and clears the device status word
 * (GTC_ERR_TIMEOUT / GTC_ERR_CAPACITY, or GTC_OK). */
GTC_API gtc_status gtc_device_status(gtc_ctx* ctx, gtc_stream_t stream);
/* Library version string and the number of kernel variants compiled in. */
GTC_API const char* gtc_version(void);

/* Bounded device waits.  Every spin of a kernel on another block's result (the
 * onesweep look-back, the resident segment scans, TMA copy completion) polls
 * at most a budget of times and then records GTC_ERR_TIMEOUT in the status
 * word and returns, so a lost predecessor never hangs the GPU; the reference's
 * look-back spin is unbounded (new_radix_sort.comp:209-223).  The budget is
 * 2^20 polls with backoff (well under a second); gtc_set_spin_limit sets it
 * for this context (polls = 0 restores the default).  gtc_debug_skip_first_tile
 * makes the next gtc_sort_pairs_u32/u64 on this context hand out its last
 * pass's tile tickets from 1, so that pass's tile 0 is never sorted and never
 * publishes its counts: the look-backs that reach it run out of polls (a test
 * of the timeout path; that sort's output is then undefined but every write
 * stays in bounds).  One-shot.  Neither has a counterpart in the reference. */
GTC_API gtc_status gtc_set_spin_limit(gtc_ctx* ctx, uint32_t polls);
GTC_API gtc_status gtc_debug_skip_first_tile(gtc_ctx* ctx);

/* Record per-stage CUDA events around every launch (0 = off, the default). */
GTC_API gtc_status gtc_set_profiling(gtc_ctx* ctx, int enable);
/* Sum of event-timed milliseconds per stage since the last reset, and the
 * number of launches timed; ms and launches hold GTC_STAGE_COUNT entries.
 * Stages: see GTC_STAGE_*.  Synchronises. */
enum {
  GTC_STAGE_MORTON = 0,
  GTC_STAGE_HISTOGRAM = 1,
  GTC_STAGE_ONESWEEP = 2,
  GTC_STAGE_UNIQUE = 3,
  GTC_STAGE_RADIX_TREE = 4,
  GTC_STAGE_PREFIX_SUM = 5,
  GTC_STAGE_OCTREE = 6,
  GTC_STAGE_LEARNED = 7,
  GTC_STAGE_RUN_FIXUP = 8, /* the fused pipeline's low-bit fixup after its 64-bit sort */
  GTC_STAGE_COUNT = 9
};
GTC_API gtc_status gtc_stage_times(gtc_ctx* ctx, float* ms, uint32_t* launches, int reset);

/* --------------------------------------------------------- workspace ----- */
typedef enum gtc_op {
  GTC_OP_SORT_PAIRS = 1,
  GTC_OP_UNIQUE = 2,
  GTC_OP_PARTIAL_SUM = 3,
  GTC_OP_BUILD_OCTREE = 4,
  GTC_OP_GLOBAL_HISTOGRAM = 5,
  GTC_OP_LEARNED_SORT = 6
} gtc_op;
/* Bytes of device workspace `op` needs for n elements of key_bits-wide keys.
 * Workspace pointers must be 256-byte aligned. */
GTC_API gtc_status gtc_workspace_size(gtc_ctx* ctx, gtc_op op, uint32_t n, int key_bits, size_t* bytes);

/* ----------------------------------------------------- stage operators --- */

/* Morton encode.  Replaces compute_morton (morton.rs:76-83, morton.comp:36-67):
 * q = trunc(((x - min) / range) * 2^B), masked to B bits, bits interleaved
 * x | y << 1 | z << 2.  idx (nullable) receives 0..n-1, the payload the sort
 * carries. */
GTC_API gtc_status gtc_morton32(gtc_ctx* ctx, const float* pts, uint32_t* keys, uint32_t* idx, uint32_t n,
                                float min_coord, float range, gtc_stream_t stream);
GTC_API gtc_status gtc_morton64(gtc_ctx* ctx, const float* pts, uint64_t* keys, uint32_t* idx, uint32_t n,
                                float min_coord, float range, gtc_stream_t stream);

/* Global digit histograms, written as exclusive prefixes per pass:
 * hist[pass * 256 + digit], passes = ceil((end_bit - begin_bit) / 8).
 * Replaces histogram (histogram.rs:38, histogram.comp:103-195), with correct
 * counts (the shader masks one digit with 0xF at histogram.comp:128). */
GTC_API gtc_status gtc_global_histogram_u32(gtc_ctx* ctx, const uint32_t* keys, uint32_t n, int begin_bit,
                                            int end_bit, uint32_t* hist, void* ws, size_t ws_bytes,
                                            gtc_stream_t stream);
GTC_API gtc_status gtc_global_histogram_u64(gtc_ctx* ctx, const uint64_t* keys, uint32_t n, int begin_bit,
                                            int end_bit, uint32_t* hist, void* ws, size_t ws_bytes,
                                            gtc_stream_t stream);

/* Stable LSD onesweep sort of (key, value) pairs on bits [begin_bit, end_bit).
 * The result is in keys/vals; keys_alt/vals_alt are scratch of the same size.
 * Replaces the onesweep driver test_radix_sort (main.rs:175-800,
 * new_radix_sort.comp:116-314) and radix_sort (radixsort.rs:36).  vals may be
 * NULL (keys only; vals_alt then ignored). */
GTC_API gtc_status gtc_sort_pairs_u32(gtc_ctx* ctx, uint32_t* keys, uint32_t* vals, uint32_t* keys_alt,
                                      uint32_t* vals_alt, uint32_t n, int begin_bit, int end_bit, void* ws,
                                      size_t ws_bytes, gtc_stream_t stream);
GTC_API gtc_status gtc_sort_pairs_u64(gtc_ctx* ctx, uint64_t* keys, uint32_t* vals, uint64_t* keys_alt,
                                      uint32_t* vals_alt, uint32_t n, int begin_bit, int end_bit, void* ws,
                                      size_t ws_bytes, gtc_stream_t stream);

/* In-place unique of sorted keys: keeps the first of each run and its value;
 * the count goes to *d_n_unique (device).  Replaces unique (unique.rs:37,
 * unique.comp:31-49).  vals may be NULL. */
GTC_API gtc_status gtc_unique_u32(gtc_ctx* ctx, uint32_t* keys, uint32_t* vals, uint32_t n, uint32_t* d_n_unique,
                                  void* ws, size_t ws_bytes, gtc_stream_t stream);
GTC_API gtc_status gtc_unique_u64(gtc_ctx* ctx, uint64_t* keys, uint32_t* vals, uint32_t n, uint32_t* d_n_unique,
                                  void* ws, size_t ws_bytes, gtc_stream_t stream);

/* Karras radix tree over n_brt_nodes = u - 1 internal nodes (codes holds u
 * sorted unique codes).  Replaces build_radix_tree (build_radix_tree.rs:34-43,
 * build_radix_tree.comp:44-153) with a signed direction and a root range that
 * covers all u keys.  edge_count (nullable) additionally receives the edge
 * counts of edge_count.comp (fused). */
GTC_API gtc_status gtc_build_radix_tree_u32(gtc_ctx* ctx, const uint32_t* codes, int32_t n_brt_nodes,
                                            uint8_t* prefix_n, uint8_t* has_leaf_left, uint8_t* has_leaf_right,
                                            int32_t* left_child, int32_t* parent, uint32_t* edge_count,
                                            gtc_stream_t stream);
GTC_API gtc_status gtc_build_radix_tree_u64(gtc_ctx* ctx, const uint64_t* codes, int32_t n_brt_nodes,
                                            uint8_t* prefix_n, uint8_t* has_leaf_left, uint8_t* has_leaf_right,
                                            int32_t* left_child, int32_t* parent, uint32_t* edge_count,
                                            gtc_stream_t stream);

/* edge[i] = depth(i) - depth(parent[i]), depth = (prefix_n - A) / 3 with
 * A = key_bits - 3 * bits_per_axis.  Replaces edge_count (edge_count.rs:41-47,
 * edge_count.comp:30-41) over exactly n_brt_nodes nodes. */
GTC_API gtc_status gtc_edge_count(gtc_ctx* ctx, const uint8_t* prefix_n, const int32_t* parent,
                                  uint32_t* edge_count, uint32_t n_brt_nodes, int key_bits, gtc_stream_t stream);

/* Inclusive scan of data[first, last) into d_first[0, last - first).
 * Replaces partial_sum (partial_sum.rs:43, partial_sum.comp:23-39). */
GTC_API gtc_status gtc_partial_sum_u32(gtc_ctx* ctx, const uint32_t* data, uint32_t first, uint32_t last,
                                       uint32_t* d_first, void* ws, size_t ws_bytes, gtc_stream_t stream);

/* Octree node offsets as the pipeline uses them (main.rs:127-129): inclusive
 * scan of edge_count over u = n_brt_nodes + 1 entries, edge[m] read as 0,
 * node_offsets[0] = 0.  d_n_oct_nodes (nullable, device) receives
 * o = 1 + node_offsets[u - 1]. */
GTC_API gtc_status gtc_node_offsets(gtc_ctx* ctx, const uint32_t* edge_count, uint32_t n_brt_nodes,
                                    uint32_t* node_offsets, uint32_t* d_n_oct_nodes, void* ws, size_t ws_bytes,
                                    gtc_stream_t stream);

/* Octree make: writes every octree node (root included, main.rs:140-153)
 * with its internal children, corners and cell sizes.  Replaces build_octree /
 * k_MakeOctNodes (octree.rs:73-87, octree.comp:126-186); same argument order.
 * Radix node i owns slots [node_offsets[i] - rt_node_counts[i] + 1,
 * node_offsets[i]]; the root owns slot 0.  oct_nodes must hold
 * 1 + node_offsets[n_brt_nodes] nodes (nodes_capacity). */
GTC_API gtc_status gtc_make_octree_u32(gtc_ctx* ctx, gtc_octnode* oct_nodes, uint32_t nodes_capacity,
                                       const uint32_t* node_offsets, const uint32_t* rt_node_counts,
                                       const uint32_t* codes, const uint8_t* rt_prefix_n, const int32_t* rt_parents,
                                       float min_coord, float range, int32_t n_brt_nodes,
                                       const uint8_t* rt_has_leaf_left, const uint8_t* rt_has_leaf_right,
                                       const int32_t* rt_left_child, gtc_stream_t stream);
GTC_API gtc_status gtc_make_octree_u64(gtc_ctx* ctx, gtc_octnode* oct_nodes, uint32_t nodes_capacity,
                                       const uint32_t* node_offsets, const uint32_t* rt_node_counts,
                                       const uint64_t* codes, const uint8_t* rt_prefix_n, const int32_t* rt_parents,
                                       float min_coord, float range, int32_t n_brt_nodes,
                                       const uint8_t* rt_has_leaf_left, const uint8_t* rt_has_leaf_right,
                                       const int32_t* rt_left_child, gtc_stream_t stream);
/* Octree link: adds the leaf children (k_LinkLeafNodes, octree.comp:188-222,
 * commented out in the reference) after gtc_make_octree_*. */
GTC_API gtc_status gtc_link_octree_u32(gtc_ctx* ctx, gtc_octnode* oct_nodes, uint32_t nodes_capacity,
                                       const uint32_t* node_offsets, const uint32_t* rt_node_counts,
                                       const uint32_t* codes, const uint8_t* rt_prefix_n, const int32_t* rt_parents,
                                       int32_t n_brt_nodes, const uint8_t* rt_has_leaf_left,
                                       const uint8_t* rt_has_leaf_right, const int32_t* rt_left_child,
                                       gtc_stream_t stream);
GTC_API gtc_status gtc_link_octree_u64(gtc_ctx* ctx, gtc_octnode* oct_nodes, uint32_t nodes_capacity,
                                       const uint32_t* node_offsets, const uint32_t* rt_node_counts,
                                       const uint64_t* codes, const uint8_t* rt_prefix_n, const int32_t* rt_parents,
                                       int32_t n_brt_nodes, const uint8_t* rt_has_leaf_left,
                                       const uint8_t* rt_has_leaf_right, const int32_t* rt_left_child,
                                       gtc_stream_t stream);

/* --------------------------------------------------- fused pipeline ------ */

/* Caller-owned device outputs of the whole path, each sized for n points
 * (n >= 1).  counts[0..3] (device) receives u, m = u - 1, o and a status. */
typedef struct gtc_octree_buffers {
  void* keys;              /* uint32_t or uint64_t [n]: sorted unique codes (first u) */
  uint32_t* idx;           /* [n]: original point index of each unique code (first u) */
  uint8_t* prefix_n;       /* [n]: first m */
  uint8_t* has_leaf_left;  /* [n]: first m */
  uint8_t* has_leaf_right; /* [n]: first m */
  int32_t* left_child;     /* [n]: first m */
  int32_t* parent;         /* [n]: first m */
  uint32_t* edge_count;    /* [n]: first m */
  uint32_t* node_offsets;  /* [n]: first u */
  gtc_octnode* nodes;      /* [nodes_capacity]: first o */
  uint32_t nodes_capacity;
  uint32_t* counts;        /* [4] device */
} gtc_octree_buffers;

/* Points -> Morton -> onesweep sort -> unique -> radix tree (+ edge count)
 * -> node offsets -> octree make+link, all stream-ordered with no host sync
 * (the commented pipeline of main.rs:60-170, with the GPU sort in place of the
 * CPU sort at main.rs:85).  key_bits = 32 or 64.  For 64-bit codes the sort
 * runs its passes over bits 23..62 and then sorts each run of codes equal in
 * those bits by bits 0..22: the same order as sorting all 63 bits. */
GTC_API gtc_status gtc_build_octree(gtc_ctx* ctx, const float* pts, uint32_t n, float min_coord, float range,
                                    int key_bits, const gtc_octree_buffers* out, void* ws, size_t ws_bytes,
                                    gtc_stream_t stream);

/* The same from HOST buffers: copies pts in, builds on the context's own
 * resident buffers, copies the o octree nodes out (host_nodes holds
 * host_nodes_capacity nodes) and host_counts[0..2] = u, m, o.  Synchronous.
 * Page-locked points (cudaHostAlloc / gtc_host_alloc) are read by the Morton
 * pass straight from host memory; other host memory is copied first.  The
 * nodes are copied back.  If o > host_nodes_capacity the call returns
 * GTC_ERR_CAPACITY with host_counts set and no nodes copied. */
GTC_API gtc_status gtc_build_octree_host(gtc_ctx* ctx, const float* host_pts, uint32_t n, float min_coord,
                                         float range, int key_bits, gtc_octnode* host_nodes,
                                         uint32_t host_nodes_capacity, uint32_t* host_counts);

/* Queued form of gtc_build_octree_host for back-to-back builds (a stream of
 * point clouds): the same outputs, with builds overlapped.  Builds take three
 * sets of device buffers in turn, each with its own streams.  A call queues
 * its points' upload (a copy engine) and its build, then waits on the host
 * for the previous build and queues that build's node read-back: a
 * copy-engine transfer of exactly o nodes.  Uploads, read-backs and kernels
 * of different builds run at the same time (the host link carries both
 * directions at once).  host_pts, host_nodes and host_counts must be
 * page-locked (gtc_host_alloc / cudaHostRegister) and stay untouched until
 * gtc_build_octree_host_wait returns.  Builds in flight need distinct output
 * buffers, except that every third call may reuse them: calls take the three
 * buffer sets in turn and a set's writes are ordered on its stream.  host_counts[0..2] = u, m, o;
 * host_nodes gets the o nodes (it may be NULL with capacity 0: counts only).
 * The device node buffer holds 1.5 n + 1024 nodes.  With o above either
 * capacity the wait returns GTC_ERR_CAPACITY (counts still set, no nodes);
 * gtc_build_octree_host sizes itself to any o.  n = 0 sets the counts to 0
 * at once. */
GTC_API gtc_status gtc_build_octree_host_async(gtc_ctx* ctx, const float* host_pts, uint32_t n, float min_coord,
                                               float range, int key_bits, gtc_octnode* host_nodes,
                                               uint32_t host_nodes_capacity, uint32_t* host_counts);
/* Waits for every queued build of the context; reports the first device
 * error of any of them (GTC_ERR_CAPACITY, GTC_ERR_TIMEOUT, ...). */
GTC_API gtc_status gtc_build_octree_host_wait(gtc_ctx* ctx);

/* ---------------------------------------------------- batched clouds ---- */
/* No counterpart in the reference: many independent point clouds of uneven
 * size built in one stream-ordered sequence of launches (graph-capturable, no
 * host sync), 32-bit codes only.  Cloud c is points [off[c], off[c+1]) of
 * pts; every cloud's outputs equal gtc_build_octree(key_bits = 32) on that
 * cloud alone, with cloud-local indices:
 *   keys, idx:                 [key_offset[c], key_offset[c] + u_c)
 *   prefix_n .. edge_count:    [key_offset[c], key_offset[c] + m_c)
 *   node_offsets:              [key_offset[c], key_offset[c] + u_c)
 *   nodes:                     [node_offset[c], node_offset[c] + o_c)
 * cloud_counts[3c .. 3c+2] = u_c, m_c, o_c; key_offset[n_clouds] = total
 * unique codes; node_offset[n_clouds] = total nodes.  Every array is device
 * memory; the per-code arrays hold n_total entries. */
typedef struct gtc_batch_buffers {
  uint32_t* keys;
  uint32_t* idx;
  uint8_t* prefix_n;
  uint8_t* has_leaf_left;
  uint8_t* has_leaf_right;
  int32_t* left_child;
  int32_t* parent;
  uint32_t* edge_count;
  uint32_t* node_offsets;
  gtc_octnode* nodes;
  uint32_t nodes_capacity;
  uint32_t* key_offset;   /* [n_clouds + 1] */
  uint32_t* node_offset;  /* [n_clouds + 1] */
  uint32_t* cloud_counts; /* [3 * n_clouds] */
} gtc_batch_buffers;

/* Workspace of a batch (n_total < 2^30 points, 1 <= n_clouds <= 2^20). */
GTC_API gtc_status gtc_batched_workspace_size(uint32_t n_total, uint32_t n_clouds, size_t* bytes);
/* d_offsets: device uint32[n_clouds + 1], non-decreasing, d_offsets[0] = 0,
 * d_offsets[n_clouds] = n_total; pts: device float[n_total][4]; ws: 256-byte
 * aligned, gtc_batched_workspace_size bytes.  A node array that is too small
 * sets GTC_ERR_CAPACITY in the device status word. */
GTC_API gtc_status gtc_build_octree_batched(gtc_ctx* ctx, const float* pts, const uint32_t* d_offsets,
                                            uint32_t n_clouds, uint32_t n_total, float min_coord, float range,
                                            const gtc_batch_buffers* out, void* ws, size_t ws_bytes,
                                            gtc_stream_t stream);
/* Tile shapes of the batch's segmented onesweep compiled into the library
 * (threads per block x keys per thread; the tile also divides the clouds for
 * the Morton pass).  A build uses the pinned variant, else the autotuner's
 * pick for its n_total (gtc_autotune_batched), else variant 0.  Every
 * variant gives identical output.  No reference counterpart. */
GTC_API int gtc_batched_num_variants(void);
GTC_API gtc_status gtc_batched_variant_shape(int variant, int* threads, int* keys_per_thread);
/* Pins one variant for every batched build; variant = -1 unpins. */
GTC_API gtc_status gtc_batched_set_variant(int variant);
/* The variant a batched build of n_total points uses now. */
GTC_API int gtc_batched_get_variant(uint32_t n_total);

/* The same sort of 32-bit keys (optionally with u32 values) for callers that
 * must not allocate device memory at the point where they sort: cudaMalloc /
 * cudaFree synchronise the device and can stall other streams for
 * milliseconds, and callers whose own allocator owns the device memory cannot
 * hand over a workspace on demand.  No counterpart in the reference.
 * Its scratch is a fixed 4,210,944-byte array inside the library, held by
 * every GPU that loads the library until the process exits, so n is limited
 * to GTC_NOALLOC_MAX_KEYS (larger n returns GTC_ERR_INVALID_ARG).  The call
 * allocates nothing.  The context's device must be the current device
 * (otherwise GTC_ERR_INVALID_ARG).  Its first call on a device looks up that
 * device's address of the array (once per device, with the device current);
 * make that first call before any stream capture.  All calls share the
 * array: calls that overlap on the GPU race, so issue them on one stream. */
#define GTC_NOALLOC_MAX_KEYS 4194304u
GTC_API gtc_status gtc_sort_pairs_u32_noalloc(gtc_ctx* ctx, uint32_t* keys, uint32_t* vals, uint32_t* keys_alt,
                                              uint32_t* vals_alt, uint32_t n, int begin_bit, int end_bit,
                                              gtc_stream_t stream);

/* ------------------------------------------------ learned-bucket sort --- */
/* No counterpart in the reference: a learned stand-in for the top radix
 * passes of the 64-bit sort, whose output is defined to be exactly the stable
 * onesweep result (gtc_sort_pairs_u64 on bits [0, 64)).
 *
 * The model is a piecewise-linear CDF with `buckets` segments (a power of two
 * <= 8192): knots at quantiles of a sample of previously sorted keys, FP32
 * heights trained on the GPU (forward / backward / Adam kernels, mean squared
 * error against the sample's empirical CDF).  gtc_learned_sort_u64 groups
 * the keys by model bucket (two stable passes over the bucket-id digits, equal
 * keys kept in input order), sorts each bucket on chip, and
 * checks on the device that no bucket overflowed its on-chip capacity (16384
 * keys) and that bucket key ranges are ordered.  If a check fails the flag
 * word *d_flags is nonzero and the plain onesweep, launched in the same stream
 * and gated on that word, produces the result instead (bits: 1 overflow,
 * 2 order, 4 non-monotone model; 8 is reserved). */
typedef struct gtc_learned_model gtc_learned_model;
GTC_API gtc_status gtc_learned_model_create(gtc_ctx* ctx, int buckets, gtc_learned_model** out);
GTC_API gtc_status gtc_learned_model_destroy(gtc_learned_model* model);
/* Device pointers of the model's knots (u64[buckets + 1]) and heights
 * (f32[buckets + 1]). */
GTC_API gtc_status gtc_learned_model_params(gtc_learned_model* model, int* buckets, uint64_t** d_knots,
                                            float** d_heights);
/* Synchronous copy of the knots and heights to host arrays of buckets + 1. */
GTC_API gtc_status gtc_learned_model_export(gtc_learned_model* model, uint64_t* host_knots, float* host_heights);
/* Samples every sample_stride-th key of `sorted_keys` (a previous sort's
 * output), places the knots at the sample's quantiles and runs `iters` Adam
 * steps of learning rate lr on the heights.  *d_loss (device, nullable)
 * receives the final mean squared error. */
GTC_API gtc_status gtc_learned_train_u64(gtc_ctx* ctx, gtc_learned_model* model, const uint64_t* sorted_keys,
                                         uint32_t n, uint32_t sample_stride, int iters, float lr, float* d_loss,
                                         gtc_stream_t stream);
/* Gradient (d_grad: f32[buckets + 1]) and loss of the current heights on the
 * sample of sorted_keys (init != 0 first resets knots and heights): the
 * backward kernel the training uses, exposed for gradient checks. */
GTC_API gtc_status gtc_learned_gradient_u64(gtc_ctx* ctx, gtc_learned_model* model, const uint64_t* sorted_keys,
                                            uint32_t n, uint32_t sample_stride, int init, float* d_grad,
                                            float* d_loss, gtc_stream_t stream);
/* Bucket occupancy of `keys` under the model (d_counts: u32[buckets]). */
GTC_API gtc_status gtc_learned_histogram_u64(gtc_ctx* ctx, const gtc_learned_model* model, const uint64_t* keys,
                                             uint32_t n, uint32_t* d_counts, gtc_stream_t stream);
/* Out-of-place sort of (keys, vals) into (keys_out, vals_out); vals may be
 * NULL (the payload is then the input index).  Workspace:
 * gtc_workspace_size(GTC_OP_LEARNED_SORT, n, 64). */
GTC_API gtc_status gtc_learned_sort_u64(gtc_ctx* ctx, const gtc_learned_model* model, const uint64_t* keys,
                                        const uint32_t* vals, uint64_t* keys_out, uint32_t* vals_out, uint32_t n,
                                        void* ws, size_t ws_bytes, uint32_t* d_flags, gtc_stream_t stream);
/* Tile shapes of the learned sort's two bucket-id grouping passes compiled
 * into the library (threads per block x keys per thread).  A sort uses the
 * pinned variant, else the autotuner's pick for its n
 * (gtc_autotune_learned), else variant 0.  Every variant gives identical
 * output.  No reference counterpart. */
GTC_API int gtc_learned_num_variants(void);
GTC_API gtc_status gtc_learned_variant_shape(int variant, int* threads, int* keys_per_thread);
/* Pins one variant for every learned sort; variant = -1 unpins. */
GTC_API gtc_status gtc_learned_set_variant(int variant);
/* The variant a learned sort of n keys uses now. */
GTC_API int gtc_learned_get_variant(uint32_t n);

/* ------------------------------------------------------ sort variants --- */
/* Onesweep tile shapes compiled into the library (threads per block and keys
 * per thread); the autotuner times them and selects one per key width.  No
 * reference counterpart: the reference hard-codes 512 x 15 (main.rs:182). */
GTC_API int gtc_sort_num_variants(void);
GTC_API gtc_status gtc_sort_variant_shape(int variant, int* threads, int* keys_per_thread);
/* Pins one variant for every sort of that key width (overriding the tuned
 * choice); variant = -1 unpins. */
GTC_API gtc_status gtc_sort_set_variant(int key_bits, int variant);
GTC_API int gtc_sort_get_variant(int key_bits);
/* Digit width of gtc_sort_pairs_u32/u64: 8 bits (4 / 8 passes over full
 * keys), or 7 or 6 where the bit range fits in 8 passes.  Pins one width
 * for every sort of that key width (6..8; -1 unpins: the autotuner's pick,
 * else 8); a pinned width that does not fit a sort's range is ignored for it.
 * gtc_sort_get_digit_bits returns the width a sort of `bits` bits over n keys
 * uses.  The reference's radix is fixed at 8 bits (new_radix_sort.comp:28-33);
 * the sort's output does not depend on the width.  gtc_workspace_size
 * (GTC_OP_SORT_PAIRS) leaves room for the passes of the narrowest width. */
GTC_API gtc_status gtc_sort_set_digit_bits(int key_bits, int digit_bits);
GTC_API int gtc_sort_get_digit_bits(int key_bits, int bits, uint32_t n);

/* Radix tree method, process-wide: 1 (default) builds each node from its
 * split with nearest-smaller queries over a shared-memory window of
 * adjacent-key prefix lengths; 0 runs the per-node Karras searches of
 * build_radix_tree.comp:71-144.  Both give identical output. */
GTC_API gtc_status gtc_tree_set_method(int method);
GTC_API int gtc_tree_get_method(void);

/* Autotuner.  Times every variant on n keys of key_bits width sorted over
 * [begin_bit, end_bit) - the caller's device keys d_sample_keys (n of them,
 * nullable) or seeded uniform keys - taking the best of `reps` timed runs
 * after one warm-up, and caches the fastest for (key_bits, end_bit -
 * begin_bit, ceil(log2 n)).  best_variant and times_ms[gtc_sort_num_variants()]
 * are nullable.  Synchronous; allocates its own buffers.  The cache is
 * process-wide; the file named by the environment variable GTC_TUNE_CACHE is
 * loaded on first use and rewritten after each tuning. */
GTC_API gtc_status gtc_autotune_sort(gtc_ctx* ctx, int key_bits, int begin_bit, int end_bit, uint32_t n,
                                     const void* d_sample_keys, int reps, int* best_variant, float* times_ms);
/* gtc_autotune_sort with the second axis reported: after the variants (at
 * 8-bit digits), the fastest variant is timed at 7- and 6-bit digits where
 * the bit range fits in 8 passes (32-bit keys, and 64-bit sorts of at most
 * 48 bits), and the fastest digit width is cached with the variant.
 * best_digit_bits and digit_times_ms[3] (6, 7, 8 bits; FLT_MAX where a width
 * does not fit) are nullable. */
GTC_API gtc_status gtc_autotune_sort_ex(gtc_ctx* ctx, int key_bits, int begin_bit, int end_bit, uint32_t n,
                                        const void* d_sample_keys, int reps, int* best_variant, float* times_ms,
                                        int* best_digit_bits, float* digit_times_ms);
/* The cached variant for a sort of that shape, or -1. */
GTC_API int gtc_autotune_lookup(int key_bits, int bits, uint32_t n);
/* The cached digit width for a sort of that shape, or -1. */
GTC_API int gtc_autotune_lookup_digit_bits(int key_bits, int bits, uint32_t n);
GTC_API gtc_status gtc_autotune_record(int key_bits, int bits, uint32_t n, int variant, float ms);
GTC_API gtc_status gtc_autotune_clear(void);
GTC_API int gtc_autotune_entries(void);
/* Times every batched variant on the caller's own batch: `reps` timed builds
 * after one warm-up each, through the caller's outputs and workspace
 * (arguments as gtc_build_octree_batched), and caches the fastest for
 * ceil(log2 n_total).  best_variant and times_ms[gtc_batched_num_variants()]
 * are nullable.  Synchronous. */
GTC_API gtc_status gtc_autotune_batched(gtc_ctx* ctx, const float* pts, const uint32_t* d_offsets, uint32_t n_clouds,
                                        uint32_t n_total, float min_coord, float range, const gtc_batch_buffers* out,
                                        void* ws, size_t ws_bytes, int reps, int* best_variant, float* times_ms);
/* The cached batched variant for n_total points, or -1. */
GTC_API int gtc_autotune_lookup_batched(uint32_t n_total);
/* Times every grouping-pass shape of the learned sort on the caller's keys
 * (arguments as gtc_learned_sort_u64) and caches the fastest for
 * ceil(log2 n).  best_variant and times_ms[gtc_learned_num_variants()] are
 * nullable.  Synchronous. */
GTC_API gtc_status gtc_autotune_learned(gtc_ctx* ctx, const gtc_learned_model* model, const uint64_t* keys,
                                        const uint32_t* vals, uint64_t* keys_out, uint32_t* vals_out, uint32_t n,
                                        void* ws, size_t ws_bytes, uint32_t* d_flags, int reps, int* best_variant,
                                        float* times_ms);
/* The cached learned-sort variant for n keys, or -1. */
GTC_API int gtc_autotune_lookup_learned(uint32_t n);
GTC_API gtc_status gtc_autotune_save(const char* path);
GTC_API gtc_status gtc_autotune_load(const char* path);

/* Pinned host memory helpers for callers without a CUDA runtime binding. */
GTC_API gtc_status gtc_host_alloc(void** ptr, size_t bytes);
GTC_API gtc_status gtc_host_free(void* ptr);

/* Literal-mode switches, process-wide (default 0: the corrected forms).  They
 * reproduce the reference's deterministic deviations for callers comparing
 * against buffers the reference wrote:
 *   GTC_LITERAL_D2  gtc_edge_count takes depth = prefix_n / 3, counting the
 *                   unused high bits (edge_count.comp:34), instead of
 *                   (prefix_n - A) / 3;
 *   GTC_LITERAL_D6  leaf links leave child_leaf_mask at 0, as SetLeaf's
 *                   `mask &= ~bit` does (octree.comp:27-30); leaf child slots
 *                   are still written.  Applies to make, link, and the fused
 *                   and batched builds.
 * The literal depth is not offered for the octree itself: there it maps
 * several children to one slot (child-slot conflicts), and the survivor
 * depends on write order. */
#define GTC_LITERAL_D2 (1u << 2)
#define GTC_LITERAL_D6 (1u << 6)
GTC_API gtc_status gtc_set_literal(uint32_t flags);
GTC_API uint32_t gtc_get_literal(void);

/* Points in sorted order: out[i] = pts[idx[i]] for i < count (float4 each),
 * e.g. with the payload of a sort or of unique (one point per distinct
 * code).  Indices >= n_pts give a zero point and flag GTC_ERR_INVALID_ARG on
 * the device status word. */
GTC_API gtc_status gtc_gather_points(gtc_ctx* ctx, const float* pts, uint32_t n_pts, const uint32_t* idx,
                                     uint32_t count, float* out, gtc_stream_t stream);

/* Little-endian binary export of a host buffer: count elements of elem_bytes
 * (1, 2, 4 or 8) each, written in order as the reference's dump writes its
 * buffers (write_u32::<LittleEndian> per element, radixsort-vulkan
 * main.rs:760-769).  append != 0 appends to an existing file. */
GTC_API gtc_status gtc_export_le(const char* path, const void* host_data, size_t count, int elem_bytes, int append);

/* ------------------------------------------- reference-signature shims --- */
/* Synchronous host-array versions with the Rust functions' parameter order.
 * They use a process-wide context on device 0. */

/* morton.rs:76-83  compute_morton(input, morton_keys, n, min_coord, range, group_size) */
GTC_API gtc_status gtc_ref_compute_morton(const float* input, uint32_t* morton_keys, uint32_t n, float min_coord,
                                          float range, uint32_t group_size);
/* morton.rs:43-60  morton32_to_xyz(ret, code, min_coord, range) */
GTC_API void gtc_ref_morton32_to_xyz(float* ret, uint32_t code, float min_coord, float range);
/* histogram.rs:38  histogram(input_size, input_data, global_hist[1024]) */
GTC_API gtc_status gtc_ref_histogram(uint32_t input_size, const uint32_t* input_data, uint32_t* global_hist);
/* radixsort.rs:36  radix_sort(in_data, n, out_data, group_size) (onesweep) */
GTC_API gtc_status gtc_ref_radix_sort(const uint32_t* in_data, uint32_t n, uint32_t* out_data, uint32_t group_size);
/* unique.rs:37  unique(u_sort, n) -> n_unique (in place) */
GTC_API uint32_t gtc_ref_unique(uint32_t* u_sort, uint32_t n);
/* build_radix_tree.rs:34-43 */
GTC_API gtc_status gtc_ref_build_radix_tree(int32_t n, const uint32_t* codes, uint8_t* prefix_n,
                                            uint8_t* has_leaf_left, uint8_t* has_leaf_right, int32_t* left_child,
                                            int32_t* parent, uint32_t group_size);
/* edge_count.rs:41-47 (n_brt_nodes is the number of radix-tree nodes, m) */
GTC_API gtc_status gtc_ref_edge_count(const uint8_t* prefix_n, const int32_t* parent, uint32_t* u_edge_count,
                                      uint32_t n_brt_nodes, uint32_t group_size);
/* partial_sum.rs:43 */
GTC_API gtc_status gtc_ref_partial_sum(const uint32_t* u_edge_count, uint32_t first, uint32_t last,
                                       uint32_t* d_first);
/* octree.rs:73-87 build_octree(...) followed by the link step; n = radix-tree
 * node count m; oct_nodes holds 1 + node_offsets[m] nodes. */
GTC_API gtc_status gtc_ref_build_octree(gtc_octnode* oct_nodes, const uint32_t* node_offsets,
                                        const uint32_t* rt_node_counts, const uint32_t* codes,
                                        const uint8_t* rt_prefix_n, const int32_t* rt_parents, float min_coord,
                                        float range, int32_t n, const uint8_t* rt_has_leaf_left,
                                        const uint8_t* rt_has_leaf_right, const int32_t* rt_left_child,
                                        uint32_t group_size);

#ifdef __cplusplus
}
#endif
#endif /* GTC_H */
