// tune.cu - the onesweep autotuner.
//
// No counterpart in the reference (main.rs:182 hard-codes one tile shape).
// gtc_autotune_sort times every compiled onesweep variant (threads per block,
// keys per thread, ranking scheme) on n keys of a given width and bit range -
// the caller's own keys, or seeded uniform keys - and caches the fastest per
// (key width, bits sorted, ceil(log2 n)).  Every later sort of that shape
// uses the cached variant unless one is pinned (gtc_sort_set_variant).
// The cache is kept as text ("sort <key_bits> <bits> <log2n> <variant>
// <ms>" per line): gtc_autotune_save / gtc_autotune_load, and the file named
// by GTC_TUNE_CACHE is loaded on first use and rewritten after each tuning.

#include <cfloat>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "gtc_internal.cuh"

namespace gtc {

Launch context_launch(gtc_ctx* ctx, gtc_stream_t stream);
gtc_status context_error(gtc_ctx* ctx, gtc_status s, const char* msg, cudaError_t e);
int sort_num_variants();

namespace {

struct TuneKey {
  int key_bits, bits, log2n;
  bool operator<(const TuneKey& o) const {
    return std::tie(key_bits, bits, log2n) < std::tie(o.key_bits, o.bits, o.log2n);
  }
};
struct TuneEntry {
  int variant;
  float ms;
  int db = 8;  // sort entries: digit width in bits
};

std::mutex g_mu;
std::map<TuneKey, TuneEntry> g_cache;
// Other tuned shapes by (kind, ceil(log2 n)): the batched build's segmented
// onesweep ("batched") and the learned sort's grouping passes ("learned").
enum TuneKind { TK_BATCHED = 0, TK_LEARNED = 1 };
const char* const kKindName[] = {"batched", "learned"};
std::map<std::pair<int, int>, TuneEntry> g_xcache;
bool g_env_loaded = false;

int log2_bucket(uint32_t n) {
  int b = 0;
  while (b < 32 && (1ull << b) < n) ++b;
  return b;
}

bool load_locked(const char* path) {
  FILE* f = fopen(path, "r");
  if (!f) return false;
  char line[256];
  while (fgets(line, sizeof line, f)) {
    int kb, bits, lg, v, db = 8;
    float ms;
    const int got = sscanf(line, "sort %d %d %d %d %f %d", &kb, &bits, &lg, &v, &ms, &db);
    if (got >= 5 && (kb == 32 || kb == 64) && bits >= 1 && bits <= kb && lg >= 0 && lg <= 32 && v >= 0 &&
        v < sort_num_variants() && sort_digit_bits_ok(bits, db))
      g_cache[TuneKey{kb, bits, lg}] = TuneEntry{v, ms, db};
    else if (sscanf(line, "batched %d %d %f", &lg, &v, &ms) == 3 && lg >= 0 && lg <= 32 && v >= 0 &&
             v < batched_num_variants())
      g_xcache[{TK_BATCHED, lg}] = TuneEntry{v, ms};
    else if (sscanf(line, "learned %d %d %f", &lg, &v, &ms) == 3 && lg >= 0 && lg <= 32 && v >= 0 &&
             v < learned_num_variants())
      g_xcache[{TK_LEARNED, lg}] = TuneEntry{v, ms};
  }
  fclose(f);
  return true;
}

bool save_locked(const char* path) {
  FILE* f = fopen(path, "w");
  if (!f) return false;
  fprintf(f, "# gtc autotune cache: sort <key_bits> <bits> <log2n> <variant> <ms> <digit bits>, "
             "batched|learned <log2n> <variant> <ms>\n");
  for (const auto& kv : g_cache)
    fprintf(f, "sort %d %d %d %d %.6f %d\n", kv.first.key_bits, kv.first.bits, kv.first.log2n, kv.second.variant,
            kv.second.ms, kv.second.db);
  for (const auto& kv : g_xcache)
    fprintf(f, "%s %d %d %.6f\n", kKindName[kv.first.first], kv.first.second, kv.second.variant, kv.second.ms);
  fclose(f);
  return true;
}

void load_env_once_locked() {
  if (g_env_loaded) return;
  g_env_loaded = true;
  const char* p = getenv("GTC_TUNE_CACHE");
  if (p && *p) load_locked(p);
}

// Seeded uniform keys over [begin, end) (SplitMix64 of the index) and an
// iota payload.
template <class K>
__global__ void tune_fill_kernel(K* keys, uint32_t* vals, uint32_t n, uint64_t seed, int begin_bit, int end_bit) {
  const uint32_t stride = gridDim.x * blockDim.x;
  const int bits = end_bit - begin_bit;
  const K mask = bits >= (int)(8 * sizeof(K)) ? ~K(0) : ((K(1) << bits) - 1);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    uint64_t z = seed + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    keys[i] = (K)(((K)z & mask) << begin_bit);
    vals[i] = i;
  }
}

// Times every variant at 8-bit digits, then the fastest variant at 7- and
// 6-bit digits (where the bit range fits the workspace's passes), and caches
// the fastest (variant, digit width).  digit_ms[0..2]: 6, 7, 8 bits (FLT_MAX
// where a width does not fit).
template <class K>
gtc_status tune_impl(gtc_ctx* ctx, int begin_bit, int end_bit, uint32_t n, const void* sample, int reps, int* best,
                     float* times_ms, int* best_db, float* digit_ms) {
  const int passes = sort_max_passes();  // workspace room for any digit width
  const int nv = sort_num_variants();
  std::vector<void*> bufs;
  cudaStream_t s = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  gtc_status st = GTC_OK;
  auto alloc = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    bufs.push_back(p);
    return p;
  };
  std::vector<float> t(nv, FLT_MAX);
  float dt[3] = {FLT_MAX, FLT_MAX, FLT_MAX};  // 6, 7, 8-bit digits at the best variant
  int bv = 0;
  cudaError_t e = cudaSuccess;
  do {
    // The sample is copied on a private stream: first let every queued write
    // of the caller's keys finish.
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) {
      st = context_error(ctx, GTC_ERR_CUDA, "autotune: sync", e);
      break;
    }
    if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&a)) != cudaSuccess || (e = cudaEventCreate(&b)) != cudaSuccess) {
      st = context_error(ctx, GTC_ERR_CUDA, "autotune: stream/event creation", e);
      break;
    }
    K* src_k = static_cast<K*>(alloc((size_t)n * sizeof(K)));
    uint32_t* src_v = static_cast<uint32_t*>(alloc((size_t)n * 4));
    K* k = static_cast<K*>(alloc((size_t)n * sizeof(K)));
    uint32_t* v = static_cast<uint32_t*>(alloc((size_t)n * 4));
    K* ka = static_cast<K*>(alloc((size_t)n * sizeof(K)));
    uint32_t* va = static_cast<uint32_t*>(alloc((size_t)n * 4));
    void* ws = alloc(sort_workspace_bytes(n, passes, 0));
    if (!src_k || !src_v || !k || !v || !ka || !va || !ws) {
      st = context_error(ctx, GTC_ERR_OOM, "autotune: device allocation", cudaErrorMemoryAllocation);
      break;
    }
    tune_fill_kernel<K><<<1024, 256, 0, s>>>(src_k, src_v, n, 0x6a09e667f3bcc908ull, begin_bit, end_bit);
    if (sample && (e = cudaMemcpyAsync(src_k, sample, (size_t)n * sizeof(K), cudaMemcpyDeviceToDevice, s)) !=
                      cudaSuccess) {
      st = context_error(ctx, GTC_ERR_CUDA, "autotune: sample copy", e);
      break;
    }
    const Launch L = context_launch(ctx, s);
    const SortWorkspace W = carve_sort_workspace(ws, n, passes, 0);
    // best time of `reps` sorts (after one warm-up) of variant vi at db-bit digits
    auto time_sort = [&](int vi, int db, float* out) {
      const int np = (end_bit - begin_bit + db - 1) / db;
      for (int r = 0; r <= reps; ++r) {  // r = 0 warms up (and sets kernel attributes)
        bool in_alt = false;
        cudaMemcpyAsync(k, src_k, (size_t)n * sizeof(K), cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(v, src_v, (size_t)n * 4, cudaMemcpyDeviceToDevice, s);
        cudaEventRecord(a, s);
        cudaMemsetAsync(W.header, 0, W.header_words * 4, s);
        e = launch_global_hist<K>(L, k, n, begin_bit, end_bit, W, np, db);
        if (e == cudaSuccess)
          e = launch_onesweep_passes<K>(L, k, v, ka, va, n, begin_bit, end_bit, W, np, &in_alt, nullptr, vi, false,
                                        db);
        cudaEventRecord(b, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        if (e != cudaSuccess) {
          st = context_error(ctx, GTC_ERR_CUDA, "autotune: timed sort", e);
          return;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (r > 0 && ms < *out) *out = ms;
      }
    };
    for (int vi = 0; vi < nv && st == GTC_OK; ++vi) time_sort(vi, 8, &t[vi]);
    if (st != GTC_OK) break;
    for (int vi = 1; vi < nv; ++vi)
      if (t[vi] < t[bv]) bv = vi;
    dt[2] = t[bv];
    for (int db = 7; db >= 6 && st == GTC_OK; --db)
      if (sort_digit_bits_ok(end_bit - begin_bit, db)) time_sort(bv, db, &dt[db - 6]);
  } while (false);
  if (s) cudaStreamSynchronize(s);
  for (void* p : bufs) cudaFree(p);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (s) cudaStreamDestroy(s);
  if (st != GTC_OK) return st;
  int bdb = 8;
  for (int db = 6; db <= 7; ++db)
    if (dt[db - 6] < dt[bdb - 6]) bdb = db;
  if (best) *best = bv;
  if (times_ms)
    for (int vi = 0; vi < nv; ++vi) times_ms[vi] = t[vi];
  if (best_db) *best_db = bdb;
  if (digit_ms)
    for (int i = 0; i < 3; ++i) digit_ms[i] = dt[i];
  std::lock_guard<std::mutex> g(g_mu);
  load_env_once_locked();
  g_cache[TuneKey{(int)(8 * sizeof(K)), end_bit - begin_bit, log2_bucket(n)}] = TuneEntry{bv, dt[bdb - 6], bdb};
  const char* p = getenv("GTC_TUNE_CACHE");
  if (p && *p) save_locked(p);
  return GTC_OK;
}

}  // namespace

int tuned_variant(int key_bits, int bits, uint32_t n) {
  std::lock_guard<std::mutex> g(g_mu);
  load_env_once_locked();
  const auto it = g_cache.find(TuneKey{key_bits, bits, log2_bucket(n)});
  return it == g_cache.end() ? -1 : it->second.variant;
}

int tuned_digit_bits(int key_bits, int bits, uint32_t n) {
  std::lock_guard<std::mutex> g(g_mu);
  load_env_once_locked();
  const auto it = g_cache.find(TuneKey{key_bits, bits, log2_bucket(n)});
  return it == g_cache.end() ? -1 : it->second.db;
}

static int tuned_kind_variant(int kind, uint32_t n) {
  std::lock_guard<std::mutex> g(g_mu);
  load_env_once_locked();
  const auto it = g_xcache.find({kind, log2_bucket(n)});
  return it == g_xcache.end() ? -1 : it->second.variant;
}
int tuned_batched_variant(uint32_t n) { return tuned_kind_variant(TK_BATCHED, n); }
int tuned_learned_variant(uint32_t n) { return tuned_kind_variant(TK_LEARNED, n); }

// Times run(variant) for every variant: `reps` timed calls after one warm-up
// each, on a private stream, best time kept; caches the fastest for (kind,
// ceil(log2 n)).
template <class Run>
static gtc_status tune_kind(gtc_ctx* ctx, int kind, int nv, uint32_t n, int reps, Run run, int* best, float* times) {
  std::vector<float> t(nv, FLT_MAX);
  cudaStream_t s = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  gtc_status st = GTC_OK;
  cudaError_t e;
  // The runs go to a private stream: first let every queued write of the
  // caller's inputs finish.
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return context_error(ctx, GTC_ERR_CUDA, "autotune: sync", e);
  if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreate(&a)) != cudaSuccess || (e = cudaEventCreate(&b)) != cudaSuccess)
    st = context_error(ctx, GTC_ERR_CUDA, "autotune: stream/event creation", e);
  for (int vi = 0; vi < nv && st == GTC_OK; ++vi) {
    for (int r = 0; r <= reps && st == GTC_OK; ++r) {  // r = 0 warms up (and sets kernel attributes)
      cudaEventRecord(a, s);
      st = run(vi, reinterpret_cast<gtc_stream_t>(s));
      cudaEventRecord(b, s);
      if (st == GTC_OK && (e = cudaEventSynchronize(b)) != cudaSuccess)
        st = context_error(ctx, GTC_ERR_CUDA, "autotune: timed run", e);
      float ms = 0.f;
      if (st == GTC_OK && r > 0 && cudaEventElapsedTime(&ms, a, b) == cudaSuccess && ms < t[vi]) t[vi] = ms;
    }
  }
  if (s) cudaStreamSynchronize(s);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (s) cudaStreamDestroy(s);
  if (st != GTC_OK) return st;
  int bv = 0;
  for (int vi = 1; vi < nv; ++vi)
    if (t[vi] < t[bv]) bv = vi;
  if (best) *best = bv;
  if (times)
    for (int vi = 0; vi < nv; ++vi) times[vi] = t[vi];
  std::lock_guard<std::mutex> g(g_mu);
  load_env_once_locked();
  g_xcache[{kind, log2_bucket(n)}] = TuneEntry{bv, t[bv]};
  const char* p = getenv("GTC_TUNE_CACHE");
  if (p && *p) save_locked(p);
  return GTC_OK;
}

}  // namespace gtc

using namespace gtc;

extern "C" {

GTC_API gtc_status gtc_autotune_sort(gtc_ctx* ctx, int key_bits, int begin_bit, int end_bit, uint32_t n,
                                     const void* d_sample_keys, int reps, int* best_variant, float* times_ms) {
  if (!ctx) return GTC_ERR_INVALID_ARG;
  if ((key_bits != 32 && key_bits != 64) || begin_bit < 0 || begin_bit >= end_bit || end_bit > key_bits)
    return context_error(ctx, GTC_ERR_INVALID_ARG, "autotune: bad key width or bit range", cudaSuccess);
  if (n == 0 || n >= (1u << 30) || reps < 1 || reps > 100)
    return context_error(ctx, GTC_ERR_INVALID_ARG, "autotune: need 0 < n < 2^30 and 1 <= reps <= 100", cudaSuccess);
  return key_bits == 32 ? tune_impl<uint32_t>(ctx, begin_bit, end_bit, n, d_sample_keys, reps, best_variant, times_ms,
                                              nullptr, nullptr)
                        : tune_impl<uint64_t>(ctx, begin_bit, end_bit, n, d_sample_keys, reps, best_variant, times_ms,
                                              nullptr, nullptr);
}

GTC_API gtc_status gtc_autotune_sort_ex(gtc_ctx* ctx, int key_bits, int begin_bit, int end_bit, uint32_t n,
                                        const void* d_sample_keys, int reps, int* best_variant, float* times_ms,
                                        int* best_digit_bits, float* digit_times_ms) {
  if (!ctx) return GTC_ERR_INVALID_ARG;
  if ((key_bits != 32 && key_bits != 64) || begin_bit < 0 || begin_bit >= end_bit || end_bit > key_bits)
    return context_error(ctx, GTC_ERR_INVALID_ARG, "autotune: bad key width or bit range", cudaSuccess);
  if (n == 0 || n >= (1u << 30) || reps < 1 || reps > 100)
    return context_error(ctx, GTC_ERR_INVALID_ARG, "autotune: need 0 < n < 2^30 and 1 <= reps <= 100", cudaSuccess);
  return key_bits == 32 ? tune_impl<uint32_t>(ctx, begin_bit, end_bit, n, d_sample_keys, reps, best_variant, times_ms,
                                              best_digit_bits, digit_times_ms)
                        : tune_impl<uint64_t>(ctx, begin_bit, end_bit, n, d_sample_keys, reps, best_variant, times_ms,
                                              best_digit_bits, digit_times_ms);
}

GTC_API int gtc_autotune_lookup_digit_bits(int key_bits, int bits, uint32_t n) {
  return tuned_digit_bits(key_bits, bits, n);
}

GTC_API gtc_status gtc_sort_set_digit_bits(int key_bits, int digit_bits) {
  if (key_bits != 32 && key_bits != 64) return GTC_ERR_INVALID_ARG;
  return sort_set_digit_bits(key_bits, digit_bits) ? GTC_OK : GTC_ERR_INVALID_ARG;
}

GTC_API int gtc_sort_get_digit_bits(int key_bits, int bits, uint32_t n) {
  if ((key_bits != 32 && key_bits != 64) || bits < 1 || bits > key_bits) return -1;
  return sort_select_digit_bits(key_bits, bits, n);
}

GTC_API int gtc_autotune_lookup(int key_bits, int bits, uint32_t n) { return tuned_variant(key_bits, bits, n); }

GTC_API gtc_status gtc_autotune_record(int key_bits, int bits, uint32_t n, int variant, float ms) {
  if ((key_bits != 32 && key_bits != 64) || bits < 1 || bits > key_bits || variant < 0 ||
      variant >= sort_num_variants())
    return GTC_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(g_mu);
  load_env_once_locked();
  g_cache[TuneKey{key_bits, bits, log2_bucket(n)}] = TuneEntry{variant, ms};
  return GTC_OK;
}

GTC_API gtc_status gtc_autotune_clear(void) {
  std::lock_guard<std::mutex> g(g_mu);
  g_env_loaded = true;  // an explicit clear also drops the environment's file
  g_cache.clear();
  g_xcache.clear();
  return GTC_OK;
}

GTC_API int gtc_autotune_entries(void) {
  std::lock_guard<std::mutex> g(g_mu);
  load_env_once_locked();
  return (int)(g_cache.size() + g_xcache.size());
}

GTC_API gtc_status gtc_autotune_batched(gtc_ctx* ctx, const float* pts, const uint32_t* d_offsets, uint32_t n_clouds,
                                        uint32_t n_total, float min_coord, float range, const gtc_batch_buffers* out,
                                        void* ws, size_t ws_bytes, int reps, int* best_variant, float* times_ms) {
  if (!ctx) return GTC_ERR_INVALID_ARG;
  if (n_total == 0 || reps < 1 || reps > 100)
    return context_error(ctx, GTC_ERR_INVALID_ARG, "autotune: need n_total > 0 and 1 <= reps <= 100", cudaSuccess);
  auto run = [&](int v, gtc_stream_t s) {
    return build_octree_batched_variant(ctx, pts, d_offsets, n_clouds, n_total, min_coord, range, out, ws, ws_bytes,
                                        s, v);
  };
  return tune_kind(ctx, TK_BATCHED, batched_num_variants(), n_total, reps, run, best_variant, times_ms);
}

GTC_API gtc_status gtc_autotune_learned(gtc_ctx* ctx, const gtc_learned_model* model, const uint64_t* keys,
                                        const uint32_t* vals, uint64_t* keys_out, uint32_t* vals_out, uint32_t n,
                                        void* ws, size_t ws_bytes, uint32_t* d_flags, int reps, int* best_variant,
                                        float* times_ms) {
  if (!ctx) return GTC_ERR_INVALID_ARG;
  if (n == 0 || reps < 1 || reps > 100)
    return context_error(ctx, GTC_ERR_INVALID_ARG, "autotune: need n > 0 and 1 <= reps <= 100", cudaSuccess);
  auto run = [&](int v, gtc_stream_t s) {
    return learned_sort_variant(ctx, model, keys, vals, keys_out, vals_out, n, ws, ws_bytes, d_flags, s, v);
  };
  return tune_kind(ctx, TK_LEARNED, learned_num_variants(), n, reps, run, best_variant, times_ms);
}

GTC_API int gtc_autotune_lookup_learned(uint32_t n) { return tuned_learned_variant(n); }

GTC_API int gtc_autotune_lookup_batched(uint32_t n_total) { return tuned_batched_variant(n_total); }

GTC_API gtc_status gtc_autotune_save(const char* path) {
  if (!path) return GTC_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(g_mu);
  load_env_once_locked();
  return save_locked(path) ? GTC_OK : GTC_ERR_INVALID_ARG;
}

GTC_API gtc_status gtc_autotune_load(const char* path) {
  if (!path) return GTC_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> g(g_mu);
  load_env_once_locked();
  return load_locked(path) ? GTC_OK : GTC_ERR_INVALID_ARG;
}

}  // extern "C"
