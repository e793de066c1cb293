// api.cu - the C ABI (include/gtc.h): context, workspace, stage operators,
// the fused stream-ordered pipeline and its host-buffer form.

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "gtc_internal.cuh"

namespace gtc {
int sort_num_variants();
int sort_get_variant(int key_bits);
bool sort_set_variant(int key_bits, int v);
void sort_variant_shape(int v, int* threads, int* kpt);

static std::atomic<uint32_t> g_literal{0};
uint32_t literal_flags() { return g_literal.load(std::memory_order_relaxed); }

namespace setup_cache {
struct SetupKey {
  int device;
  const void* kern;
  int threads;
  size_t smem;
  bool operator<(const SetupKey& o) const {
    if (device != o.device) return device < o.device;
    if (kern != o.kern) return kern < o.kern;
    if (threads != o.threads) return threads < o.threads;
    return smem < o.smem;
  }
};
std::mutex g_setup_mu;
std::map<SetupKey, int> g_setup;  // resident blocks per SM, per device and kernel shape
}  // namespace setup_cache
using namespace setup_cache;

cudaError_t kernel_setup(const void* kern, int threads, size_t smem, int* blocks_per_sm) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const SetupKey key{dev, kern, threads, smem};
  std::lock_guard<std::mutex> lock(g_setup_mu);
  auto it = g_setup.find(key);
  if (it == g_setup.end()) {
    if (smem > 48 * 1024) {
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, smem);
    if (e != cudaSuccess) return e;
    it = g_setup.emplace(key, occ > 0 ? occ : 1).first;
  }
  if (blocks_per_sm) *blocks_per_sm = it->second;
  return cudaSuccess;
}
}  // namespace gtc

using namespace gtc;

struct EventPair {
  cudaEvent_t a, b;
  int stage;
};

struct Resident {
  uint32_t n_cap = 0;
  int key_bits = 0;
  uint32_t nodes_cap = 0;
  float4* pts = nullptr;
  void* ws = nullptr;
  size_t ws_bytes = 0;
  void* keys = nullptr;
  uint32_t* idx = nullptr;
  uint8_t* prefix_n = nullptr;
  uint8_t* hll = nullptr;
  uint8_t* hlr = nullptr;
  int32_t* left = nullptr;
  int32_t* parent = nullptr;
  uint32_t* edge = nullptr;
  uint32_t* ps = nullptr;
  gtc_octnode* nodes = nullptr;
  uint32_t* counts = nullptr;
};

struct gtc_ctx {
  int device = 0;
  int num_sms = NUM_SMS_GB300;
  uint32_t* d_status = nullptr;
  std::string last_error;
  bool profiling = false;
  std::vector<EventPair> pending;
  std::vector<cudaEvent_t> free_events;
  float stage_ms[GTC_STAGE_COUNT] = {0};
  uint32_t stage_launches[GTC_STAGE_COUNT] = {0};
  void* own_ws = nullptr;
  size_t own_ws_bytes = 0;
  cudaStream_t own_stream = nullptr;
  Resident res;
  // Queued host builds (gtc_build_octree_host_async): two buffer sets and
  // streams, used alternately.
  struct QueuedOut {
    gtc_octnode* nodes = nullptr;
    uint32_t cap = 0;
    uint32_t* counts = nullptr;
    bool pending = false;  // built, node read-back not yet queued
  };
  static constexpr int NQ = 3;  // buffer sets used in turn
  Resident qres[NQ];
  cudaStream_t qstream[NQ] = {};  // builds and node read-backs
  cudaEvent_t qbuilt[NQ] = {};    // the slot's build and its counts are done
  QueuedOut qout[NQ];
  gtc_status qerr = GTC_OK;  // first host-side error of a queued build, reported by the wait
  int qnext = 0;
  bool skip_first_tile = false;  // gtc_debug_skip_first_tile: one-shot, consumed by the next sort
};

namespace {

gtc_status fail(gtc_ctx* ctx, gtc_status s, const char* what, cudaError_t e = cudaSuccess) {
  if (ctx) {
    char buf[512];
    if (e != cudaSuccess)
      snprintf(buf, sizeof buf, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    else
      snprintf(buf, sizeof buf, "%s", what);
    ctx->last_error = buf;
  }
  if (e != cudaSuccess) cudaGetLastError();  // clear a sticky launch error
  return s;
}

#define GTC_TRY(ctx, expr)                                                                           \
  do {                                                                                               \
    cudaError_t _e = (expr);                                                                         \
    if (_e != cudaSuccess) return fail((ctx), _e == cudaErrorMemoryAllocation ? GTC_ERR_OOM : GTC_ERR_CUDA, #expr, _e); \
  } while (0)

#define GTC_ARG(ctx, cond, msg)                      \
  do {                                               \
    if (!(cond)) return fail((ctx), GTC_ERR_INVALID_ARG, msg); \
  } while (0)

inline cudaStream_t S(gtc_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

inline Launch launch_of(gtc_ctx* ctx, gtc_stream_t s) { return Launch{S(s), ctx->d_status, ctx->num_sms}; }

// Clears status bits atomically, keeping every flag other builds raised.
__global__ void clear_status_bits_kernel(uint32_t* status, uint32_t bits) { atomicAnd(status, ~bits); }

cudaEvent_t get_event(gtc_ctx* ctx) {
  if (!ctx->free_events.empty()) {
    cudaEvent_t e = ctx->free_events.back();
    ctx->free_events.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Brackets launches of one stage with CUDA events when profiling is on.
struct StageTimer {
  gtc_ctx* ctx;
  cudaStream_t s;
  int stage;
  cudaEvent_t a = nullptr;
  StageTimer(gtc_ctx* c, gtc_stream_t st, int sg) : ctx(c), s(S(st)), stage(sg) {
    if (ctx->profiling) {
      a = get_event(ctx);
      cudaEventRecord(a, s);
    }
  }
  ~StageTimer() {
    if (a) {
      cudaEvent_t b = get_event(ctx);
      cudaEventRecord(b, s);
      ctx->pending.push_back({a, b, stage});
    }
  }
};

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }
bool aligned256(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 255) == 0; }

int passes_for(int begin_bit, int end_bit) { return (end_bit - begin_bit + 7) / 8; }

// Returns a workspace of `need` bytes: the caller's, or the context's own.
gtc_status resolve_ws(gtc_ctx* ctx, void*& ws, size_t ws_bytes, size_t need) {
  if (ws) {
    if (ws_bytes < need) return fail(ctx, GTC_ERR_INVALID_ARG, "workspace too small (see gtc_workspace_size)");
    if (!aligned256(ws)) return fail(ctx, GTC_ERR_INVALID_ARG, "workspace must be 256-byte aligned");
    return GTC_OK;
  }
  if (ctx->own_ws_bytes < need) {
    if (ctx->own_ws) {
      cudaDeviceSynchronize();
      cudaFree(ctx->own_ws);
      ctx->own_ws = nullptr;
      ctx->own_ws_bytes = 0;
    }
    GTC_TRY(ctx, cudaMalloc(&ctx->own_ws, need));
    ctx->own_ws_bytes = need;
  }
  ws = ctx->own_ws;
  return GTC_OK;
}

// The fused pipeline sorts 64-bit codes by onesweep passes over bits
// [RUN_FIXUP_BITS, 63) and completes the order with the run fixup; 32-bit
// codes take every pass.
template <class K>
constexpr int pipeline_begin_bit() {
  return sizeof(K) == 8 ? RUN_FIXUP_BITS : 0;
}

template <class K>
size_t pipeline_ws_bytes(uint32_t n) {
  const int passes = passes_for(pipeline_begin_bit<K>(), 3 * KeyTraits<K>::B);
  size_t b = align_up((size_t)n * sizeof(K), 256);   // keys_alt
  b += align_up((size_t)n * 4, 256);                  // vals_alt
  b += sort_workspace_bytes(n, passes, 0);
  b += 2 * scan_workspace_bytes(n);                   // unique, node offsets
  b += 256;                                           // long-range split and run counts
  return b;
}

template <class K>
gtc_status sort_pairs_impl(gtc_ctx* ctx, K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, uint32_t n,
                           int begin_bit, int end_bit, void* ws, size_t ws_bytes, gtc_stream_t stream) {
  constexpr int W = sizeof(K) * 8;
  GTC_ARG(ctx, ctx, "null context");
  GTC_ARG(ctx, 0 <= begin_bit && begin_bit < end_bit && end_bit <= W, "bit range must satisfy 0 <= begin < end <= key bits");
  GTC_ARG(ctx, n < (1u << 30), "n must be < 2^30");
  if (n == 0) return GTC_OK;
  GTC_ARG(ctx, keys && keys_alt, "keys and keys_alt are required");
  GTC_ARG(ctx, !vals || vals_alt, "vals_alt is required with vals");
  // digit width: pinned, else the autotuner's pick, else 8 bits
  const int db = sort_select_digit_bits(W, end_bit - begin_bit, n);
  const int passes = (end_bit - begin_bit + db - 1) / db;
  gtc_status st = resolve_ws(ctx, ws, ws_bytes, sort_workspace_bytes(n, passes, 0));
  if (st != GTC_OK) return st;
  const Launch L = launch_of(ctx, stream);
  const SortWorkspace Wk = carve_sort_workspace(ws, n, passes, 0);
  GTC_TRY(ctx, cudaMemsetAsync(Wk.header, 0, Wk.header_words * 4, S(stream)));
  if (ctx->skip_first_tile) {
    // The LAST pass's tile tickets start at 1 (header word 1 + p is pass p's
    // counter; byte 0 of the little-endian word): its tile 0 is never sorted
    // or published.  The last pass reads input whose digit counts match the
    // global histogram, so a tile's writes for digit d land in
    // [bin_off[d] + excl, bin_off[d] + excl + count) and a timed-out look-back
    // only makes excl smaller (the passes also check every write index).
    ctx->skip_first_tile = false;
    GTC_TRY(ctx, cudaMemsetAsync(Wk.header + passes, 1, 1, S(stream)));
  }
  {
    StageTimer t(ctx, stream, GTC_STAGE_HISTOGRAM);
    GTC_TRY(ctx, launch_global_hist<K>(L, keys, n, begin_bit, end_bit, Wk, passes, db));
  }
  bool in_alt = false;
  {
    std::vector<cudaEvent_t> ev;
    if (ctx->profiling)
      for (int i = 0; i < 2 * passes; ++i) ev.push_back(get_event(ctx));
    GTC_TRY(ctx, launch_onesweep_passes<K>(L, keys, vals, keys_alt, vals_alt, n, begin_bit, end_bit, Wk, passes,
                                           &in_alt, ev.empty() ? nullptr : ev.data(), -1, false, db));
    for (int p = 0; p < (int)ev.size() / 2; ++p) ctx->pending.push_back({ev[2 * p], ev[2 * p + 1], GTC_STAGE_ONESWEEP});
  }
  if (in_alt) {
    GTC_TRY(ctx, cudaMemcpyAsync(keys, keys_alt, (size_t)n * sizeof(K), cudaMemcpyDeviceToDevice, S(stream)));
    if (vals)
      GTC_TRY(ctx, cudaMemcpyAsync(vals, vals_alt, (size_t)n * 4, cudaMemcpyDeviceToDevice, S(stream)));
  }
  return GTC_OK;
}

template <class K>
gtc_status hist_impl(gtc_ctx* ctx, const K* keys, uint32_t n, int begin_bit, int end_bit, uint32_t* hist, void* ws,
                     size_t ws_bytes, gtc_stream_t stream) {
  constexpr int W = sizeof(K) * 8;
  GTC_ARG(ctx, ctx, "null context");
  GTC_ARG(ctx, 0 <= begin_bit && begin_bit < end_bit && end_bit <= W, "bad bit range");
  GTC_ARG(ctx, hist && (keys || n == 0), "null buffer");
  GTC_ARG(ctx, n < (1u << 30), "n must be < 2^30");
  const int passes = passes_for(begin_bit, end_bit);
  gtc_status st = resolve_ws(ctx, ws, ws_bytes, sort_workspace_bytes(n, passes, 0));
  if (st != GTC_OK) return st;
  const SortWorkspace Wk = carve_sort_workspace(ws, n, passes, 0);
  GTC_TRY(ctx, cudaMemsetAsync(Wk.header, 0, Wk.header_words * 4, S(stream)));
  if (n == 0) {
    GTC_TRY(ctx, cudaMemsetAsync(hist, 0, (size_t)passes * 256 * 4, S(stream)));
    return GTC_OK;
  }
  {
    StageTimer t(ctx, stream, GTC_STAGE_HISTOGRAM);
    GTC_TRY(ctx, launch_global_hist<K>(launch_of(ctx, stream), keys, n, begin_bit, end_bit, Wk, passes));
  }
  GTC_TRY(ctx, cudaMemcpyAsync(hist, Wk.bin_offsets, (size_t)passes * 256 * 4, cudaMemcpyDeviceToDevice, S(stream)));
  return GTC_OK;
}

template <class K>
gtc_status unique_impl(gtc_ctx* ctx, K* keys, uint32_t* vals, uint32_t n, uint32_t* d_n_unique, void* ws,
                       size_t ws_bytes, gtc_stream_t stream) {
  GTC_ARG(ctx, ctx, "null context");
  GTC_ARG(ctx, d_n_unique && (keys || n == 0), "null buffer");
  GTC_ARG(ctx, n < (1u << 30), "n must be < 2^30");
  gtc_status st = resolve_ws(ctx, ws, ws_bytes, scan_workspace_bytes(n));
  if (st != GTC_OK) return st;
  StageTimer t(ctx, stream, GTC_STAGE_UNIQUE);
  GTC_TRY(ctx, launch_unique<K>(launch_of(ctx, stream), keys, vals, keys, vals, n, d_n_unique, ws));
  return GTC_OK;
}

template <class K>
gtc_status tree_impl(gtc_ctx* ctx, const K* codes, int32_t m, uint8_t* prefix_n, uint8_t* hll, uint8_t* hlr,
                     int32_t* left, int32_t* parent, uint32_t* edge, gtc_stream_t stream) {
  GTC_ARG(ctx, ctx, "null context");
  GTC_ARG(ctx, m >= 0 && m < (1 << 30), "n_brt_nodes out of range");
  if (m == 0) return GTC_OK;
  GTC_ARG(ctx, codes && prefix_n && hll && hlr && left && parent, "null buffer");
  StageTimer t(ctx, stream, GTC_STAGE_RADIX_TREE);
  GTC_TRY(ctx, launch_radix_tree<K>(launch_of(ctx, stream), codes, nullptr, m, (uint32_t)m, prefix_n, hll, hlr, left,
                                    parent, edge, nullptr));
  return GTC_OK;
}

template <class K>
gtc_status make_impl(gtc_ctx* ctx, gtc_octnode* nodes, uint32_t cap, const uint32_t* ps, const uint32_t* edge,
                     const K* codes, const uint8_t* prefix_n, float mn, float rg, int32_t m, const uint8_t* hll,
                     const uint8_t* hlr, const int32_t* left, gtc_stream_t stream) {
  GTC_ARG(ctx, ctx, "null context");
  GTC_ARG(ctx, m >= 0 && m < (1 << 30), "n_brt_nodes out of range");
  GTC_ARG(ctx, nodes && codes && (m == 0 || (ps && edge && prefix_n && hll && hlr && left)), "null buffer");
  GTC_ARG(ctx, aligned16(nodes), "oct_nodes must be 16-byte aligned");
  StageTimer t(ctx, stream, GTC_STAGE_OCTREE);
  GTC_TRY(ctx, launch_octree_make<K>(launch_of(ctx, stream), codes, nullptr, (uint32_t)m + 1, (uint32_t)m + 1,
                                     prefix_n, hll, hlr, left, edge, ps, mn, rg, nodes, cap, false));
  return GTC_OK;
}

template <class K>
gtc_status link_impl(gtc_ctx* ctx, gtc_octnode* nodes, uint32_t cap, const uint32_t* ps, const uint32_t* edge,
                     const K* codes, const uint8_t* prefix_n, const int32_t* parent, int32_t m, const uint8_t* hll,
                     const uint8_t* hlr, const int32_t* left, gtc_stream_t stream) {
  GTC_ARG(ctx, ctx, "null context");
  GTC_ARG(ctx, m >= 0 && m < (1 << 30), "n_brt_nodes out of range");
  if (m == 0) return GTC_OK;
  GTC_ARG(ctx, nodes && codes && ps && edge && prefix_n && parent && hll && hlr && left, "null buffer");
  StageTimer t(ctx, stream, GTC_STAGE_OCTREE);
  GTC_TRY(ctx, launch_octree_link<K>(launch_of(ctx, stream), codes, (uint32_t)m, prefix_n, hll, hlr, left, parent,
                                     edge, ps, nodes, cap));
  return GTC_OK;
}

// The whole path, stream-ordered, no host synchronisation.
template <class K>
gtc_status pipeline(gtc_ctx* ctx, const float* pts, uint32_t n, float mn, float rg, const gtc_octree_buffers* o,
                    void* ws, size_t ws_bytes, gtc_stream_t stream) {
  constexpr int B = KeyTraits<K>::B;
  constexpr int BEGIN = pipeline_begin_bit<K>();
  const int passes = passes_for(BEGIN, 3 * B);
  gtc_status st = resolve_ws(ctx, ws, ws_bytes, pipeline_ws_bytes<K>(n));
  if (st != GTC_OK) return st;
  const Launch L = launch_of(ctx, stream);
  char* w = reinterpret_cast<char*>(ws);
  K* keys_alt = reinterpret_cast<K*>(w);
  w += align_up((size_t)n * sizeof(K), 256);
  uint32_t* vals_alt = reinterpret_cast<uint32_t*>(w);
  w += align_up((size_t)n * 4, 256);
  void* sort_ws = w;
  w += sort_workspace_bytes(n, passes, 0);
  void* unique_ws = w;
  w += scan_workspace_bytes(n);
  void* offsets_ws = w;
  w += scan_workspace_bytes(n);
  uint32_t* q_count = reinterpret_cast<uint32_t*>(w);  // [0] long-range splits
  w += 256;
  K* keys = reinterpret_cast<K*>(o->keys);
  const SortWorkspace Wk = carve_sort_workspace(sort_ws, n, passes, 0);
  // The Morton pass zeroes the sort's look-back descriptors and, in the same
  // sweep, the unique / node-offset / queue workspaces behind them, so no
  // memset node sits between the kernels of the build.
  SortWorkspace Wz = Wk;
  Wz.desc_words = (size_t)(reinterpret_cast<uint32_t*>(w) - Wk.desc);
  // Every kernel after the first starts under a programmatic dependent
  // launch (not while stage events are being recorded between them).
  Launch Lp = L;
  Lp.pdl = !ctx->profiling;
  Lp.ws_zeroed = true;



  GTC_TRY(ctx, cudaMemsetAsync(o->counts, 0, 16, S(stream)));
  GTC_TRY(ctx, cudaMemsetAsync(Wk.header, 0, Wk.header_words * 4, S(stream)));
  // The codes start in whichever pair of buffers makes the last sort pass
  // write the workspace pair (keys_alt, vals_alt): unique then compacts out
  // of place into the caller's buffers, which lets it use its resident
  // segment form.
  const bool odd_passes = (passes & 1) != 0;
  K* k0 = odd_passes ? keys : keys_alt;
  uint32_t* v0 = odd_passes ? o->idx : vals_alt;
  K* k1 = odd_passes ? keys_alt : keys;
  uint32_t* v1 = odd_passes ? vals_alt : o->idx;
  {
    StageTimer t(ctx, stream, GTC_STAGE_MORTON);
    // No payload written here: the first sort pass makes the iota itself.
    GTC_TRY(ctx, launch_morton_hist<K>(L, reinterpret_cast<const float4*>(pts), k0, n, mn, rg, Wz, BEGIN, passes));
  }
  {
    bool in_second = false;  // true for odd pass counts: then k1 holds the result, else k0
    std::vector<cudaEvent_t> ev;
    if (ctx->profiling)
      for (int i = 0; i < 2 * passes; ++i) ev.push_back(get_event(ctx));
    GTC_TRY(ctx, launch_onesweep_passes<K>(Lp, k0, v0, k1, v1, n, BEGIN, 3 * B, Wk, passes, &in_second,
                                           ev.empty() ? nullptr : ev.data(), -1, true));
    for (int p = 0; p < (int)ev.size() / 2; ++p) ctx->pending.push_back({ev[2 * p], ev[2 * p + 1], GTC_STAGE_ONESWEEP});
  }
  if (BEGIN) {
    // The low bits decide only within runs of equal high bits: sort those
    // runs in place; the caller's pair of buffers is free as scratch.
    StageTimer t(ctx, stream, GTC_STAGE_RUN_FIXUP);
    GTC_TRY(ctx, launch_run_fixup<K>(Lp, keys_alt, vals_alt, keys, o->idx, n, BEGIN));
  }
  {
    StageTimer t(ctx, stream, GTC_STAGE_UNIQUE);
    GTC_TRY(ctx, launch_unique<K>(Lp, keys_alt, vals_alt, keys, o->idx, n, o->counts + 0, unique_ws));
  }
  {
    // vals_alt is free once unique has compacted: it holds the queue of
    // long-range splits.
    StageTimer t(ctx, stream, GTC_STAGE_RADIX_TREE);
    GTC_TRY(ctx, launch_radix_tree<K>(Lp, keys, o->counts + 0, 0, n, o->prefix_n, o->has_leaf_left,
                                      o->has_leaf_right, o->left_child, o->parent, o->edge_count, o->counts + 1,
                                      vals_alt, q_count));
  }
  {
    StageTimer t(ctx, stream, GTC_STAGE_PREFIX_SUM);
    GTC_TRY(ctx, launch_node_offsets(Lp, o->edge_count, o->node_offsets, o->counts + 0, 0, n, o->counts + 2,
                                     offsets_ws));
  }
  {
    StageTimer t(ctx, stream, GTC_STAGE_OCTREE);
    GTC_TRY(ctx, launch_octree_make<K>(Lp, keys, o->counts + 0, 0, n, o->prefix_n, o->has_leaf_left,
                                       o->has_leaf_right, o->left_child, o->edge_count, o->node_offsets, mn, rg,
                                       o->nodes, o->nodes_capacity, true));
  }
  return GTC_OK;
}

void free_resident(Resident& r) {
  void* ptrs[] = {r.pts, r.ws, r.keys, r.idx, r.prefix_n, r.hll, r.hlr, r.left, r.parent, r.edge, r.ps, r.nodes, r.counts};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  r = Resident();
}

gtc_status ensure_resident(gtc_ctx* ctx, Resident& r, uint32_t n, int key_bits, uint32_t nodes_cap) {
  if (r.n_cap >= n && r.key_bits == key_bits && r.nodes_cap >= nodes_cap && r.pts) return GTC_OK;
  cudaDeviceSynchronize();
  const uint32_t cap = std::max<uint32_t>(std::max(n, r.key_bits == key_bits ? r.n_cap : 0u), 1);
  const uint32_t ncap = std::max<uint32_t>(nodes_cap, std::max<uint32_t>(r.nodes_cap, cap + 1024));
  free_resident(r);
  const size_t K = key_bits == 64 ? 8 : 4;
  r.ws_bytes = key_bits == 64 ? pipeline_ws_bytes<uint64_t>(cap) : pipeline_ws_bytes<uint32_t>(cap);
  GTC_TRY(ctx, cudaMalloc(&r.pts, (size_t)cap * 16));
  GTC_TRY(ctx, cudaMalloc(&r.ws, r.ws_bytes));
  GTC_TRY(ctx, cudaMalloc(&r.keys, (size_t)cap * K));
  GTC_TRY(ctx, cudaMalloc(&r.idx, (size_t)cap * 4));
  GTC_TRY(ctx, cudaMalloc(&r.prefix_n, cap));
  GTC_TRY(ctx, cudaMalloc(&r.hll, cap));
  GTC_TRY(ctx, cudaMalloc(&r.hlr, cap));
  GTC_TRY(ctx, cudaMalloc(&r.left, (size_t)cap * 4));
  GTC_TRY(ctx, cudaMalloc(&r.parent, (size_t)cap * 4));
  GTC_TRY(ctx, cudaMalloc(&r.edge, (size_t)cap * 4));
  GTC_TRY(ctx, cudaMalloc(&r.ps, (size_t)cap * 4));
  GTC_TRY(ctx, cudaMalloc(&r.nodes, (size_t)ncap * sizeof(gtc_octnode)));
  GTC_TRY(ctx, cudaMalloc(&r.counts, 16));
  r.n_cap = cap;
  r.key_bits = key_bits;
  r.nodes_cap = ncap;
  return GTC_OK;
}

}  // namespace

namespace gtc {
// Accessors for entry points defined in other translation units.
Launch context_launch(gtc_ctx* ctx, gtc_stream_t stream) { return launch_of(ctx, stream); }
int context_device(const gtc_ctx* ctx) { return ctx->device; }
gtc_status context_error(gtc_ctx* ctx, gtc_status s, const char* msg, cudaError_t e) { return fail(ctx, s, msg, e); }
cudaEvent_t context_stage_begin(gtc_ctx* ctx, gtc_stream_t stream) {
  if (!ctx->profiling) return nullptr;
  cudaEvent_t a = get_event(ctx);
  cudaEventRecord(a, S(stream));
  return a;
}
void context_stage_end(gtc_ctx* ctx, gtc_stream_t stream, cudaEvent_t a, int stage) {
  if (!a) return;
  cudaEvent_t b = get_event(ctx);
  cudaEventRecord(b, S(stream));
  ctx->pending.push_back({a, b, stage});
}
}  // namespace gtc

// =================================================================== C ABI ==
extern "C" {

GTC_API const char* gtc_version(void) { return "gtc 0.1 (sm_103a)"; }

GTC_API const char* gtc_status_string(gtc_status s) {
  switch (s) {
    case GTC_OK: return "ok";
    case GTC_ERR_INVALID_ARG: return "invalid argument";
    case GTC_ERR_OOM: return "out of device memory";
    case GTC_ERR_CUDA: return "CUDA error";
    case GTC_ERR_TIMEOUT: return "a bounded device wait ran out";
    case GTC_OVERFLOW_FALLBACK: return "learned model rejected the input; onesweep result returned";
    case GTC_ERR_UNSUPPORTED: return "unsupported";
    case GTC_ERR_CAPACITY: return "output capacity exceeded";
  }
  return "unknown status";
}

GTC_API gtc_status gtc_create(gtc_ctx** out, int device) {
  if (!out) return GTC_ERR_INVALID_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return GTC_ERR_CUDA;
  }
  if (device < 0 || device >= count) return GTC_ERR_INVALID_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return GTC_ERR_CUDA;
  gtc_ctx* ctx = new gtc_ctx();
  ctx->device = device;
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaMalloc(&ctx->d_status, 256) != cudaSuccess || cudaMemset(ctx->d_status, 0, 256) != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return GTC_ERR_OOM;
  }
  *out = ctx;
  return GTC_OK;
}

GTC_API gtc_status gtc_destroy(gtc_ctx* ctx) {
  if (!ctx) return GTC_OK;
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  for (auto& p : ctx->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto e : ctx->free_events) cudaEventDestroy(e);
  free_resident(ctx->res);
  for (int q = 0; q < gtc_ctx::NQ; ++q) {
    free_resident(ctx->qres[q]);
    if (ctx->qstream[q]) cudaStreamDestroy(ctx->qstream[q]);
    if (ctx->qbuilt[q]) cudaEventDestroy(ctx->qbuilt[q]);
  }
  if (ctx->own_ws) cudaFree(ctx->own_ws);
  if (ctx->d_status) cudaFree(ctx->d_status);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return GTC_OK;
}

GTC_API const char* gtc_last_error(gtc_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

GTC_API gtc_status gtc_device_status(gtc_ctx* ctx, gtc_stream_t stream) {
  if (!ctx) return GTC_ERR_INVALID_ARG;
  GTC_TRY(ctx, cudaStreamSynchronize(S(stream)));
  uint32_t word = 0;
  GTC_TRY(ctx, cudaMemcpy(&word, ctx->d_status, 4, cudaMemcpyDeviceToHost));
  GTC_TRY(ctx, cudaMemset(ctx->d_status, 0, 4));
  if (word & DEV_TIMEOUT) return fail(ctx, GTC_ERR_TIMEOUT, "a look-back wait ran out of its poll budget");
  if (word & DEV_CAPACITY) return fail(ctx, GTC_ERR_CAPACITY, "octree node buffer too small");
  if (word & DEV_BAD_INPUT) return fail(ctx, GTC_ERR_INVALID_ARG, "device-resident offsets are not a valid partition");
  if (word & DEV_INTERNAL) return fail(ctx, GTC_ERR_CUDA, "device consistency check failed");
  return GTC_OK;
}

GTC_API gtc_status gtc_set_spin_limit(gtc_ctx* ctx, uint32_t polls) {
  GTC_ARG(ctx, ctx, "null context");
  GTC_TRY(ctx, cudaMemcpy(ctx->d_status + 1, &polls, 4, cudaMemcpyHostToDevice));
  return GTC_OK;
}

GTC_API gtc_status gtc_debug_skip_first_tile(gtc_ctx* ctx) {
  GTC_ARG(ctx, ctx, "null context");
  ctx->skip_first_tile = true;
  return GTC_OK;
}

GTC_API gtc_status gtc_set_profiling(gtc_ctx* ctx, int enable) {
  if (!ctx) return GTC_ERR_INVALID_ARG;
  ctx->profiling = enable != 0;
  return GTC_OK;
}

GTC_API gtc_status gtc_stage_times(gtc_ctx* ctx, float* ms, uint32_t* launches, int reset) {
  if (!ctx) return GTC_ERR_INVALID_ARG;
  for (auto& p : ctx->pending) {
    GTC_TRY(ctx, cudaEventSynchronize(p.b));
    float t = 0;
    GTC_TRY(ctx, cudaEventElapsedTime(&t, p.a, p.b));
    ctx->stage_ms[p.stage] += t;
    ctx->stage_launches[p.stage] += 1;
    ctx->free_events.push_back(p.a);
    ctx->free_events.push_back(p.b);
  }
  ctx->pending.clear();
  for (int s = 0; s < GTC_STAGE_COUNT; ++s) {
    if (ms) ms[s] = ctx->stage_ms[s];
    if (launches) launches[s] = ctx->stage_launches[s];
    if (reset) {
      ctx->stage_ms[s] = 0;
      ctx->stage_launches[s] = 0;
    }
  }
  return GTC_OK;
}

GTC_API gtc_status gtc_workspace_size(gtc_ctx* ctx, gtc_op op, uint32_t n, int key_bits, size_t* bytes) {
  if (!bytes) return GTC_ERR_INVALID_ARG;
  if (key_bits != 32 && key_bits != 64) return fail(ctx, GTC_ERR_INVALID_ARG, "key_bits must be 32 or 64");
  const int passes = key_bits / 8;
  switch (op) {
    case GTC_OP_SORT_PAIRS:  // room for the passes of the narrowest digit width the sort may use
      *bytes = sort_workspace_bytes(n, std::min(sort_max_passes(), (key_bits + 5) / 6), 0);
      return GTC_OK;
    case GTC_OP_GLOBAL_HISTOGRAM: *bytes = sort_workspace_bytes(n, passes, 0); return GTC_OK;
    case GTC_OP_UNIQUE:
    case GTC_OP_PARTIAL_SUM: *bytes = scan_workspace_bytes(n); return GTC_OK;
    case GTC_OP_BUILD_OCTREE:
      *bytes = key_bits == 64 ? pipeline_ws_bytes<uint64_t>(n) : pipeline_ws_bytes<uint32_t>(n);
      return GTC_OK;
    case GTC_OP_LEARNED_SORT:
      if (key_bits != 64) return fail(ctx, GTC_ERR_INVALID_ARG, "the learned sort takes 64-bit keys");
      *bytes = learned_workspace_bytes(n);
      return GTC_OK;
  }
  return fail(ctx, GTC_ERR_INVALID_ARG, "unknown op");
}

GTC_API gtc_status gtc_morton32(gtc_ctx* ctx, const float* pts, uint32_t* keys, uint32_t* idx, uint32_t n,
                                float mn, float rg, gtc_stream_t stream) {
  GTC_ARG(ctx, ctx, "null context");
  GTC_ARG(ctx, n == 0 || (pts && keys), "null buffer");
  GTC_ARG(ctx, aligned16(pts), "pts must be 16-byte aligned float[n][4]");
  StageTimer t(ctx, stream, GTC_STAGE_MORTON);
  GTC_TRY(ctx, launch_morton32(launch_of(ctx, stream), reinterpret_cast<const float4*>(pts), keys, idx, n, mn, rg));
  return GTC_OK;
}

GTC_API gtc_status gtc_morton64(gtc_ctx* ctx, const float* pts, uint64_t* keys, uint32_t* idx, uint32_t n,
                                float mn, float rg, gtc_stream_t stream) {
  GTC_ARG(ctx, ctx, "null context");
  GTC_ARG(ctx, n == 0 || (pts && keys), "null buffer");
  GTC_ARG(ctx, aligned16(pts), "pts must be 16-byte aligned float[n][4]");
  StageTimer t(ctx, stream, GTC_STAGE_MORTON);
  GTC_TRY(ctx, launch_morton64(launch_of(ctx, stream), reinterpret_cast<const float4*>(pts), keys, idx, n, mn, rg));
  return GTC_OK;
}

GTC_API gtc_status gtc_global_histogram_u32(gtc_ctx* ctx, const uint32_t* keys, uint32_t n, int b, int e,
                                            uint32_t* hist, void* ws, size_t wsb, gtc_stream_t s) {
  return hist_impl<uint32_t>(ctx, keys, n, b, e, hist, ws, wsb, s);
}
GTC_API gtc_status gtc_global_histogram_u64(gtc_ctx* ctx, const uint64_t* keys, uint32_t n, int b, int e,
                                            uint32_t* hist, void* ws, size_t wsb, gtc_stream_t s) {
  return hist_impl<uint64_t>(ctx, keys, n, b, e, hist, ws, wsb, s);
}

GTC_API gtc_status gtc_sort_pairs_u32(gtc_ctx* ctx, uint32_t* keys, uint32_t* vals, uint32_t* ka, uint32_t* va,
                                      uint32_t n, int b, int e, void* ws, size_t wsb, gtc_stream_t s) {
  return sort_pairs_impl<uint32_t>(ctx, keys, vals, ka, va, n, b, e, ws, wsb, s);
}
GTC_API gtc_status gtc_sort_pairs_u64(gtc_ctx* ctx, uint64_t* keys, uint32_t* vals, uint64_t* ka, uint32_t* va,
                                      uint32_t n, int b, int e, void* ws, size_t wsb, gtc_stream_t s) {
  return sort_pairs_impl<uint64_t>(ctx, keys, vals, ka, va, n, b, e, ws, wsb, s);
}

GTC_API gtc_status gtc_unique_u32(gtc_ctx* ctx, uint32_t* keys, uint32_t* vals, uint32_t n, uint32_t* d_nu, void* ws,
                                  size_t wsb, gtc_stream_t s) {
  return unique_impl<uint32_t>(ctx, keys, vals, n, d_nu, ws, wsb, s);
}
GTC_API gtc_status gtc_unique_u64(gtc_ctx* ctx, uint64_t* keys, uint32_t* vals, uint32_t n, uint32_t* d_nu, void* ws,
                                  size_t wsb, gtc_stream_t s) {
  return unique_impl<uint64_t>(ctx, keys, vals, n, d_nu, ws, wsb, s);
}

GTC_API gtc_status gtc_build_radix_tree_u32(gtc_ctx* ctx, const uint32_t* codes, int32_t m, uint8_t* prefix_n,
                                            uint8_t* hll, uint8_t* hlr, int32_t* left, int32_t* parent,
                                            uint32_t* edge, gtc_stream_t s) {
  return tree_impl<uint32_t>(ctx, codes, m, prefix_n, hll, hlr, left, parent, edge, s);
}
GTC_API gtc_status gtc_build_radix_tree_u64(gtc_ctx* ctx, const uint64_t* codes, int32_t m, uint8_t* prefix_n,
                                            uint8_t* hll, uint8_t* hlr, int32_t* left, int32_t* parent,
                                            uint32_t* edge, gtc_stream_t s) {
  return tree_impl<uint64_t>(ctx, codes, m, prefix_n, hll, hlr, left, parent, edge, s);
}

GTC_API gtc_status gtc_edge_count(gtc_ctx* ctx, const uint8_t* prefix_n, const int32_t* parent, uint32_t* edge,
                                  uint32_t m, int key_bits, gtc_stream_t s) {
  GTC_ARG(ctx, ctx, "null context");
  GTC_ARG(ctx, key_bits == 32 || key_bits == 64, "key_bits must be 32 or 64");
  GTC_ARG(ctx, m == 0 || (prefix_n && parent && edge), "null buffer");
  StageTimer t(ctx, s, GTC_STAGE_RADIX_TREE);
  // GTC_LITERAL_D2: the reference's depth prefix_n / 3, unused bits included.
  const int A = (literal_flags() & GTC_LITERAL_D2) ? 0 : (key_bits == 32 ? 2 : 1);
  GTC_TRY(ctx, launch_edge_count(launch_of(ctx, s), prefix_n, parent, edge, m, A));
  return GTC_OK;
}

GTC_API gtc_status gtc_partial_sum_u32(gtc_ctx* ctx, const uint32_t* data, uint32_t first, uint32_t last,
                                       uint32_t* d_first, void* ws, size_t wsb, gtc_stream_t s) {
  GTC_ARG(ctx, ctx, "null context");
  GTC_ARG(ctx, first <= last, "first > last");
  const uint32_t n = last - first;
  if (n == 0) return GTC_OK;
  GTC_ARG(ctx, data && d_first, "null buffer");
  gtc_status st = resolve_ws(ctx, ws, wsb, scan_workspace_bytes(n));
  if (st != GTC_OK) return st;
  StageTimer t(ctx, s, GTC_STAGE_PREFIX_SUM);
  GTC_TRY(ctx, launch_inclusive_scan(launch_of(ctx, s), data + first, d_first, n, ws));
  return GTC_OK;
}

GTC_API gtc_status gtc_node_offsets(gtc_ctx* ctx, const uint32_t* edge, uint32_t m, uint32_t* ps, uint32_t* d_o,
                                    void* ws, size_t wsb, gtc_stream_t s) {
  GTC_ARG(ctx, ctx, "null context");
  GTC_ARG(ctx, ps && (edge || m == 0), "null buffer");
  GTC_ARG(ctx, m < (1u << 30), "n_brt_nodes out of range");
  gtc_status st = resolve_ws(ctx, ws, wsb, scan_workspace_bytes(m + 1));
  if (st != GTC_OK) return st;
  StageTimer t(ctx, s, GTC_STAGE_PREFIX_SUM);
  GTC_TRY(ctx, launch_node_offsets(launch_of(ctx, s), edge, ps, nullptr, m, m + 1, d_o, ws));
  return GTC_OK;
}

GTC_API gtc_status gtc_make_octree_u32(gtc_ctx* ctx, gtc_octnode* nodes, uint32_t cap, const uint32_t* ps,
                                       const uint32_t* edge, const uint32_t* codes, const uint8_t* prefix_n,
                                       const int32_t* /*rt_parents*/, float mn, float rg, int32_t m,
                                       const uint8_t* hll, const uint8_t* hlr, const int32_t* left, gtc_stream_t s) {
  return make_impl<uint32_t>(ctx, nodes, cap, ps, edge, codes, prefix_n, mn, rg, m, hll, hlr, left, s);
}
GTC_API gtc_status gtc_make_octree_u64(gtc_ctx* ctx, gtc_octnode* nodes, uint32_t cap, const uint32_t* ps,
                                       const uint32_t* edge, const uint64_t* codes, const uint8_t* prefix_n,
                                       const int32_t* /*rt_parents*/, float mn, float rg, int32_t m,
                                       const uint8_t* hll, const uint8_t* hlr, const int32_t* left, gtc_stream_t s) {
  return make_impl<uint64_t>(ctx, nodes, cap, ps, edge, codes, prefix_n, mn, rg, m, hll, hlr, left, s);
}
GTC_API gtc_status gtc_link_octree_u32(gtc_ctx* ctx, gtc_octnode* nodes, uint32_t cap, const uint32_t* ps,
                                       const uint32_t* edge, const uint32_t* codes, const uint8_t* prefix_n,
                                       const int32_t* parent, int32_t m, const uint8_t* hll, const uint8_t* hlr,
                                       const int32_t* left, gtc_stream_t s) {
  return link_impl<uint32_t>(ctx, nodes, cap, ps, edge, codes, prefix_n, parent, m, hll, hlr, left, s);
}
GTC_API gtc_status gtc_link_octree_u64(gtc_ctx* ctx, gtc_octnode* nodes, uint32_t cap, const uint32_t* ps,
                                       const uint32_t* edge, const uint64_t* codes, const uint8_t* prefix_n,
                                       const int32_t* parent, int32_t m, const uint8_t* hll, const uint8_t* hlr,
                                       const int32_t* left, gtc_stream_t s) {
  return link_impl<uint64_t>(ctx, nodes, cap, ps, edge, codes, prefix_n, parent, m, hll, hlr, left, s);
}

GTC_API gtc_status gtc_build_octree(gtc_ctx* ctx, const float* pts, uint32_t n, float mn, float rg, int key_bits,
                                    const gtc_octree_buffers* out, void* ws, size_t wsb, gtc_stream_t s) {
  GTC_ARG(ctx, ctx, "null context");
  GTC_ARG(ctx, key_bits == 32 || key_bits == 64, "key_bits must be 32 or 64");
  GTC_ARG(ctx, out, "null output descriptor");
  GTC_ARG(ctx, n < (1u << 30), "n must be < 2^30");
  GTC_ARG(ctx, out->counts, "counts buffer is required");
  if (n == 0) {
    GTC_TRY(ctx, cudaMemsetAsync(out->counts, 0, 16, S(s)));
    return GTC_OK;
  }
  GTC_ARG(ctx, pts && aligned16(pts), "pts must be a 16-byte aligned float[n][4]");
  GTC_ARG(ctx, out->keys && out->idx && out->prefix_n && out->has_leaf_left && out->has_leaf_right &&
                   out->left_child && out->parent && out->edge_count && out->node_offsets && out->nodes,
          "null output buffer");
  GTC_ARG(ctx, aligned16(out->nodes), "nodes must be 16-byte aligned");
  if (key_bits == 32) return pipeline<uint32_t>(ctx, pts, n, mn, rg, out, ws, wsb, s);
  return pipeline<uint64_t>(ctx, pts, n, mn, rg, out, ws, wsb, s);
}

// The device address of page-locked host memory (cudaHostAlloc /
// cudaHostRegister), or null for any other pointer.
static const void* device_view(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

GTC_API gtc_status gtc_build_octree_host(gtc_ctx* ctx, const float* host_pts, uint32_t n, float mn, float rg,
                                         int key_bits, gtc_octnode* host_nodes, uint32_t host_cap,
                                         uint32_t* host_counts) {
  GTC_ARG(ctx, ctx, "null context");
  GTC_ARG(ctx, key_bits == 32 || key_bits == 64, "key_bits must be 32 or 64");
  GTC_ARG(ctx, host_counts && (n == 0 || host_pts), "null buffer");
  GTC_ARG(ctx, n < (1u << 30), "n must be < 2^30");
  if (n == 0) {
    host_counts[0] = host_counts[1] = host_counts[2] = 0;
    return GTC_OK;
  }
  if (!ctx->own_stream) GTC_TRY(ctx, cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
  cudaStream_t st = ctx->own_stream;
  gtc_status s = ensure_resident(ctx, ctx->res, n, key_bits, 0);
  if (s != GTC_OK) return s;
  // Page-locked input is streamed from host memory by the Morton pass itself,
  // so the transfer overlaps the encoding; other host memory is copied first.
  const float* d_in = reinterpret_cast<const float*>(device_view(host_pts));
  if (d_in && (reinterpret_cast<uintptr_t>(d_in) & 15) != 0) d_in = nullptr;
  for (int attempt = 0; attempt < 2; ++attempt) {
    Resident& r = ctx->res;
    if (!d_in) GTC_TRY(ctx, cudaMemcpyAsync(r.pts, host_pts, (size_t)n * 16, cudaMemcpyHostToDevice, st));
    gtc_octree_buffers b{r.keys, r.idx, r.prefix_n, r.hll, r.hlr, r.left, r.parent, r.edge, r.ps, r.nodes,
                         r.nodes_cap, r.counts};
    s = gtc_build_octree(ctx, d_in ? d_in : reinterpret_cast<const float*>(r.pts), n, mn, rg, key_bits, &b, r.ws,
                         r.ws_bytes, st);
    if (s != GTC_OK) return s;
    uint32_t c[4];
    GTC_TRY(ctx, cudaMemcpyAsync(c, r.counts, 16, cudaMemcpyDeviceToHost, st));
    GTC_TRY(ctx, cudaStreamSynchronize(st));
    const uint32_t o = c[2];
    if (o > r.nodes_cap) {  // rare: long single-child chains; grow and rebuild
      // Clear only the capacity flag this build raised: the status word is
      // shared with queued builds, whose other flags (a timeout) must stay.
      clear_status_bits_kernel<<<1, 1, 0, st>>>(ctx->d_status, DEV_CAPACITY);
      GTC_TRY(ctx, cudaGetLastError());
      s = ensure_resident(ctx, ctx->res, n, key_bits, o);
      if (s != GTC_OK) return s;
      continue;
    }
    host_counts[0] = c[0];
    host_counts[1] = c[1];
    host_counts[2] = o;
    if (o > host_cap) return fail(ctx, GTC_ERR_CAPACITY, "host node buffer too small");
    if (host_nodes && o)
      GTC_TRY(ctx, cudaMemcpyAsync(host_nodes, r.nodes, (size_t)o * sizeof(gtc_octnode), cudaMemcpyDeviceToHost, st));
    return gtc_device_status(ctx, st);
  }
  return fail(ctx, GTC_ERR_CAPACITY, "octree node capacity");
}

// Queues the node read-back of slot q's finished build on the slot's stream
// (a copy-engine transfer of exactly o nodes, so it takes no SM time from
// the build that runs meanwhile).  Waits on the host for that build first.
static gtc_status queue_readback(gtc_ctx* ctx, int q) {
  gtc_ctx::QueuedOut& out = ctx->qout[q];
  if (!out.pending) return GTC_OK;
  out.pending = false;
  GTC_TRY(ctx, cudaEventSynchronize(ctx->qbuilt[q]));
  const uint32_t o = out.counts[2];
  if (o > ctx->qres[q].nodes_cap) {  // the device node buffer was too small: reported by the wait
    if (ctx->qerr == GTC_OK) ctx->qerr = fail(ctx, GTC_ERR_CAPACITY, "octree node capacity of a queued build");
    return GTC_OK;
  }
  if (!out.nodes) return GTC_OK;                   // counts only
  if (o > out.cap) {
    if (ctx->qerr == GTC_OK) ctx->qerr = fail(ctx, GTC_ERR_CAPACITY, "host node buffer too small");
    return GTC_OK;
  }
  if (o)
    GTC_TRY(ctx, cudaMemcpyAsync(out.nodes, ctx->qres[q].nodes, (size_t)o * sizeof(gtc_octnode),
                                 cudaMemcpyDeviceToHost, ctx->qstream[q]));
  return GTC_OK;
}

GTC_API gtc_status gtc_build_octree_host_async(gtc_ctx* ctx, const float* host_pts, uint32_t n, float mn, float rg,
                                               int key_bits, gtc_octnode* host_nodes, uint32_t host_cap,
                                               uint32_t* host_counts) {
  GTC_ARG(ctx, ctx, "null context");
  GTC_ARG(ctx, key_bits == 32 || key_bits == 64, "key_bits must be 32 or 64");
  GTC_ARG(ctx, n < (1u << 30), "n must be < 2^30");
  GTC_ARG(ctx, host_counts, "null counts buffer");
  if (n == 0) {
    host_counts[0] = host_counts[1] = host_counts[2] = 0;
    return GTC_OK;
  }
  const float* d_in = reinterpret_cast<const float*>(device_view(host_pts));
  GTC_ARG(ctx, device_view(host_counts), "host_counts must be page-locked");
  GTC_ARG(ctx, host_pts && d_in && aligned16(d_in), "host_pts must be page-locked and 16-byte aligned");
  GTC_ARG(ctx, !host_nodes || device_view(host_nodes), "host_nodes must be page-locked");
  const int q = ctx->qnext;
  if (!ctx->qstream[q]) {
    GTC_TRY(ctx, cudaStreamCreateWithFlags(&ctx->qstream[q], cudaStreamNonBlocking));
    GTC_TRY(ctx, cudaEventCreateWithFlags(&ctx->qbuilt[q], cudaEventDisableTiming));
  }
  cudaStream_t st = ctx->qstream[q];
  // A slot that has to grow synchronises the device first (ensure_resident).
  gtc_status s = ensure_resident(ctx, ctx->qres[q], n, key_bits, n + (n >> 1) + 1024);
  if (s != GTC_OK) return s;
  Resident& r = ctx->qres[q];
  // The Morton pass reads the page-locked points over the host link itself
  // (no copy-engine upload, which would queue behind the node read-backs).
  // The slot's previous node read-back was queued on this stream by a later
  // call, so stream order keeps the slot's buffers safe.
  gtc_octree_buffers b{r.keys, r.idx, r.prefix_n, r.hll, r.hlr, r.left, r.parent, r.edge, r.ps, r.nodes,
                       r.nodes_cap, r.counts};
  s = gtc_build_octree(ctx, d_in, n, mn, rg, key_bits, &b, r.ws, r.ws_bytes, st);
  if (s != GTC_OK) return s;
  GTC_TRY(ctx, cudaMemcpyAsync(host_counts, r.counts, 12, cudaMemcpyDeviceToHost, st));
  GTC_TRY(ctx, cudaEventRecord(ctx->qbuilt[q], st));
  ctx->qout[q] = {host_nodes, host_nodes ? host_cap : 0u, host_counts, true};
  ctx->qnext = (q + 1) % gtc_ctx::NQ;
  // The previous build is read back while this one runs.
  return queue_readback(ctx, (q + gtc_ctx::NQ - 1) % gtc_ctx::NQ);
}

GTC_API gtc_status gtc_build_octree_host_wait(gtc_ctx* ctx) {
  GTC_ARG(ctx, ctx, "null context");
  for (int i = 0; i < gtc_ctx::NQ; ++i) {  // oldest slot first
    const int q = (ctx->qnext + i) % gtc_ctx::NQ;
    gtc_status s = queue_readback(ctx, q);
    if (s != GTC_OK) return s;
  }
  for (int q = 0; q < gtc_ctx::NQ; ++q)
    if (ctx->qstream[q]) GTC_TRY(ctx, cudaStreamSynchronize(ctx->qstream[q]));
  gtc_status s = gtc_device_status(ctx, ctx->qstream[0]);
  if (s == GTC_OK && ctx->qerr != GTC_OK) s = ctx->qerr;
  ctx->qerr = GTC_OK;
  return s;
}

GTC_API gtc_status gtc_host_alloc(void** ptr, size_t bytes) {
  if (!ptr) return GTC_ERR_INVALID_ARG;
  cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return GTC_ERR_OOM;
  }
  return GTC_OK;
}
GTC_API gtc_status gtc_host_free(void* ptr) {
  if (ptr) cudaFreeHost(ptr);
  return GTC_OK;
}

// Sort variant table (used by the autotuner).
GTC_API int gtc_sort_num_variants(void) { return sort_num_variants(); }
GTC_API gtc_status gtc_sort_variant_shape(int v, int* threads, int* keys_per_thread) {
  if (v < 0 || v >= sort_num_variants() || !threads || !keys_per_thread) return GTC_ERR_INVALID_ARG;
  sort_variant_shape(v, threads, keys_per_thread);
  return GTC_OK;
}
GTC_API gtc_status gtc_sort_set_variant(int key_bits, int v) {
  if (key_bits != 32 && key_bits != 64) return GTC_ERR_INVALID_ARG;
  return sort_set_variant(key_bits, v) ? GTC_OK : GTC_ERR_INVALID_ARG;
}
GTC_API int gtc_sort_get_variant(int key_bits) { return sort_get_variant(key_bits); }
GTC_API gtc_status gtc_tree_set_method(int method) { return tree_set_method(method) ? GTC_OK : GTC_ERR_INVALID_ARG; }
GTC_API int gtc_tree_get_method(void) { return tree_get_method(); }

GTC_API gtc_status gtc_set_literal(uint32_t flags) {
  if (flags & ~(GTC_LITERAL_D2 | GTC_LITERAL_D6)) return GTC_ERR_INVALID_ARG;
  g_literal.store(flags);
  return GTC_OK;
}
GTC_API uint32_t gtc_get_literal(void) { return g_literal.load(); }

GTC_API gtc_status gtc_gather_points(gtc_ctx* ctx, const float* pts, uint32_t n_pts, const uint32_t* idx,
                                     uint32_t count, float* out, gtc_stream_t s) {
  GTC_ARG(ctx, ctx, "null context");
  if (count == 0) return GTC_OK;
  GTC_ARG(ctx, pts && idx && out, "null buffer");
  GTC_ARG(ctx, ((reinterpret_cast<uintptr_t>(pts) | reinterpret_cast<uintptr_t>(out)) & 15) == 0,
          "points must be 16-byte aligned float4");
  GTC_TRY(ctx, launch_gather_points(launch_of(ctx, s), reinterpret_cast<const float4*>(pts), n_pts, idx, count,
                                    reinterpret_cast<float4*>(out)));
  return GTC_OK;
}

GTC_API gtc_status gtc_export_le(const char* path, const void* host_data, size_t count, int elem_bytes, int append) {
  if (!path || (count > 0 && !host_data) || !(elem_bytes == 1 || elem_bytes == 2 || elem_bytes == 4 || elem_bytes == 8))
    return GTC_ERR_INVALID_ARG;
  FILE* f = std::fopen(path, append ? "ab" : "wb");
  if (!f) return GTC_ERR_INVALID_ARG;
  // Bytes of each element least significant first, whatever the host order.
  const unsigned char* src = static_cast<const unsigned char*>(host_data);
  const uint16_t probe = 1;
  const bool little = *reinterpret_cast<const unsigned char*>(&probe) == 1;
  bool ok = true;
  if (little) {
    ok = std::fwrite(src, (size_t)elem_bytes, count, f) == count;
  } else {
    unsigned char buf[8];
    for (size_t i = 0; i < count && ok; ++i) {
      for (int b = 0; b < elem_bytes; ++b) buf[b] = src[i * elem_bytes + (elem_bytes - 1 - b)];
      ok = std::fwrite(buf, (size_t)elem_bytes, 1, f) == 1;
    }
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? GTC_OK : GTC_ERR_INVALID_ARG;
}

}  // extern "C"
