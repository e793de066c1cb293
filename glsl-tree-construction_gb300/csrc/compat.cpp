// compat.cpp - synchronous host-array shims with the reference's Rust
// signatures (radixsort-vulkan/src/*.rs).  Each call uploads its inputs,
// runs the stage on the GPU and downloads the outputs, like the reference's
// per-call "upload, dispatch, fence, read back" shape - but on one resident
// CUDA context instead of a fresh Vulkan instance per call.

#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <vector>

#include "gtc.h"

namespace {

std::mutex g_mu;
gtc_ctx* g_ctx = nullptr;

gtc_ctx* ctx() {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_ctx) gtc_create(&g_ctx, 0);
  return g_ctx;
}

// RAII device buffer.
struct Dev {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t err = cudaSuccess;
  explicit Dev(size_t b) : bytes(b) {
    if (b) err = cudaMalloc(&p, b);
  }
  ~Dev() {
    if (p) cudaFree(p);
  }
  template <class T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
  bool ok() const { return err == cudaSuccess; }
};

gtc_status up(Dev& d, const void* h, size_t b) {
  if (!d.ok()) return GTC_ERR_OOM;
  if (b && cudaMemcpy(d.p, h, b, cudaMemcpyHostToDevice) != cudaSuccess) return GTC_ERR_CUDA;
  return GTC_OK;
}
gtc_status down(void* h, const Dev& d, size_t b) {
  if (b && cudaMemcpy(h, d.p, b, cudaMemcpyDeviceToHost) != cudaSuccess) return GTC_ERR_CUDA;
  return GTC_OK;
}

#define CHK(x)                     \
  do {                             \
    gtc_status _s = (x);           \
    if (_s != GTC_OK) return _s;   \
  } while (0)

gtc_status finish(gtc_ctx* c) { return gtc_device_status(c, nullptr); }

}  // namespace

extern "C" {

GTC_API gtc_status gtc_ref_compute_morton(const float* input, uint32_t* morton_keys, uint32_t n, float min_coord,
                                          float range, uint32_t /*group_size*/) {
  gtc_ctx* c = ctx();
  if (!c) return GTC_ERR_CUDA;
  if (n == 0) return GTC_OK;
  if (!input || !morton_keys) return GTC_ERR_INVALID_ARG;
  Dev pts((size_t)n * 16), keys((size_t)n * 4);
  CHK(up(pts, input, (size_t)n * 16));
  if (!keys.ok()) return GTC_ERR_OOM;
  CHK(gtc_morton32(c, pts.as<float>(), keys.as<uint32_t>(), nullptr, n, min_coord, range, nullptr));
  CHK(finish(c));
  return down(morton_keys, keys, (size_t)n * 4);
}

GTC_API void gtc_ref_morton32_to_xyz(float* ret, uint32_t code, float min_coord, float range) {
  // Host-side decode (morton.rs:43-74): every third bit, then
  // (q / 1024) * range + min with each operation rounded separately.
  auto third = [](uint32_t m) {
    uint32_t x = m & 0x09249249u;
    x = (x ^ (x >> 2)) & 0x030c30c3u;
    x = (x ^ (x >> 4)) & 0x0300f00fu;
    x = (x ^ (x >> 8)) & 0x030000ffu;
    x = (x ^ (x >> 16)) & 0x000003ffu;
    return (float)x;
  };
  volatile float q;  // keep each operation separately rounded
  q = third(code) / 1024.0f;
  q = q * range;
  ret[0] = q + min_coord;
  q = third(code >> 1) / 1024.0f;
  q = q * range;
  ret[1] = q + min_coord;
  q = third(code >> 2) / 1024.0f;
  q = q * range;
  ret[2] = q + min_coord;
  ret[3] = 1.0f;
}

GTC_API gtc_status gtc_ref_histogram(uint32_t input_size, const uint32_t* input_data, uint32_t* global_hist) {
  gtc_ctx* c = ctx();
  if (!c) return GTC_ERR_CUDA;
  if (!global_hist || (input_size && !input_data)) return GTC_ERR_INVALID_ARG;
  Dev keys((size_t)input_size * 4), hist(1024 * 4);
  CHK(up(keys, input_data, (size_t)input_size * 4));
  if (!hist.ok()) return GTC_ERR_OOM;
  CHK(gtc_global_histogram_u32(c, keys.as<uint32_t>(), input_size, 0, 32, hist.as<uint32_t>(), nullptr, 0, nullptr));
  CHK(finish(c));
  return down(global_hist, hist, 1024 * 4);
}

GTC_API gtc_status gtc_ref_radix_sort(const uint32_t* in_data, uint32_t n, uint32_t* out_data, uint32_t) {
  gtc_ctx* c = ctx();
  if (!c) return GTC_ERR_CUDA;
  if (n == 0) return GTC_OK;
  if (!in_data || !out_data) return GTC_ERR_INVALID_ARG;
  Dev keys((size_t)n * 4), alt((size_t)n * 4);
  CHK(up(keys, in_data, (size_t)n * 4));
  if (!alt.ok()) return GTC_ERR_OOM;
  CHK(gtc_sort_pairs_u32(c, keys.as<uint32_t>(), nullptr, alt.as<uint32_t>(), nullptr, n, 0, 32, nullptr, 0, nullptr));
  CHK(finish(c));
  return down(out_data, keys, (size_t)n * 4);
}

GTC_API uint32_t gtc_ref_unique(uint32_t* u_sort, uint32_t n) {
  // unique.rs:37 returns the count; errors surface as 0 (the Rust version
  // panics).
  gtc_ctx* c = ctx();
  if (!c || n == 0 || !u_sort) return 0;
  Dev keys((size_t)n * 4), cnt(4);
  if (up(keys, u_sort, (size_t)n * 4) != GTC_OK || !cnt.ok()) return 0;
  if (gtc_unique_u32(c, keys.as<uint32_t>(), nullptr, n, cnt.as<uint32_t>(), nullptr, 0, nullptr) != GTC_OK) return 0;
  if (finish(c) != GTC_OK) return 0;
  uint32_t u = 0;
  if (down(&u, cnt, 4) != GTC_OK) return 0;
  if (down(u_sort, keys, (size_t)u * 4) != GTC_OK) return 0;
  return u;
}

GTC_API gtc_status gtc_ref_build_radix_tree(int32_t n, const uint32_t* codes, uint8_t* prefix_n,
                                            uint8_t* has_leaf_left, uint8_t* has_leaf_right, int32_t* left_child,
                                            int32_t* parent, uint32_t) {
  gtc_ctx* c = ctx();
  if (!c) return GTC_ERR_CUDA;
  if (n < 0) return GTC_ERR_INVALID_ARG;
  if (n == 0) return GTC_OK;
  if (!codes || !prefix_n || !has_leaf_left || !has_leaf_right || !left_child || !parent) return GTC_ERR_INVALID_ARG;
  const size_t m = (size_t)n;
  Dev dc((m + 1) * 4), dp(m), dl(m), dr(m), dlc(m * 4), dpa(m * 4);
  CHK(up(dc, codes, (m + 1) * 4));
  if (!dp.ok() || !dl.ok() || !dr.ok() || !dlc.ok() || !dpa.ok()) return GTC_ERR_OOM;
  CHK(gtc_build_radix_tree_u32(c, dc.as<uint32_t>(), n, dp.as<uint8_t>(), dl.as<uint8_t>(), dr.as<uint8_t>(),
                               dlc.as<int32_t>(), dpa.as<int32_t>(), nullptr, nullptr));
  CHK(finish(c));
  CHK(down(prefix_n, dp, m));
  CHK(down(has_leaf_left, dl, m));
  CHK(down(has_leaf_right, dr, m));
  CHK(down(left_child, dlc, m * 4));
  return down(parent, dpa, m * 4);
}

GTC_API gtc_status gtc_ref_edge_count(const uint8_t* prefix_n, const int32_t* parent, uint32_t* u_edge_count,
                                      uint32_t n_brt_nodes, uint32_t) {
  gtc_ctx* c = ctx();
  if (!c) return GTC_ERR_CUDA;
  const size_t m = n_brt_nodes;
  if (m == 0) return GTC_OK;
  if (!prefix_n || !parent || !u_edge_count) return GTC_ERR_INVALID_ARG;
  Dev dp(m), dpa(m * 4), de(m * 4);
  CHK(up(dp, prefix_n, m));
  CHK(up(dpa, parent, m * 4));
  if (!de.ok()) return GTC_ERR_OOM;
  CHK(gtc_edge_count(c, dp.as<uint8_t>(), dpa.as<int32_t>(), de.as<uint32_t>(), n_brt_nodes, 32, nullptr));
  CHK(finish(c));
  return down(u_edge_count, de, m * 4);
}

GTC_API gtc_status gtc_ref_partial_sum(const uint32_t* data, uint32_t first, uint32_t last, uint32_t* d_first) {
  gtc_ctx* c = ctx();
  if (!c) return GTC_ERR_CUDA;
  if (first > last) return GTC_ERR_INVALID_ARG;
  const size_t k = last - first;
  if (k == 0) return GTC_OK;
  if (!data || !d_first) return GTC_ERR_INVALID_ARG;
  Dev din(k * 4), dout(k * 4);
  CHK(up(din, data + first, k * 4));
  if (!dout.ok()) return GTC_ERR_OOM;
  CHK(gtc_partial_sum_u32(c, din.as<uint32_t>(), 0, (uint32_t)k, dout.as<uint32_t>(), nullptr, 0, nullptr));
  CHK(finish(c));
  return down(d_first, dout, k * 4);
}

GTC_API gtc_status gtc_ref_build_octree(gtc_octnode* oct_nodes, const uint32_t* node_offsets,
                                        const uint32_t* rt_node_counts, const uint32_t* codes,
                                        const uint8_t* rt_prefix_n, const int32_t* rt_parents, float min_coord,
                                        float range, int32_t n, const uint8_t* rt_has_leaf_left,
                                        const uint8_t* rt_has_leaf_right, const int32_t* rt_left_child, uint32_t) {
  gtc_ctx* c = ctx();
  if (!c) return GTC_ERR_CUDA;
  if (n < 0 || !oct_nodes || !codes) return GTC_ERR_INVALID_ARG;
  const size_t m = (size_t)n;
  if (m > 0 && (!node_offsets || !rt_node_counts || !rt_prefix_n || !rt_parents || !rt_has_leaf_left ||
                !rt_has_leaf_right || !rt_left_child))
    return GTC_ERR_INVALID_ARG;
  const uint32_t o = 1 + (m > 0 ? node_offsets[m] : 0);  // node_offsets holds u = m + 1 entries
  const size_t mm = m > 0 ? m : 1;
  Dev dn((size_t)o * sizeof(gtc_octnode)), dps((mm + 1) * 4), de(mm * 4), dc((m + 1) * 4), dp(mm), dpa(mm * 4),
      dl(mm), dr(mm), dlc(mm * 4);
  CHK(up(dc, codes, (m + 1) * 4));
  if (m > 0) {
    CHK(up(dps, node_offsets, (m + 1) * 4));
    CHK(up(de, rt_node_counts, m * 4));
    CHK(up(dp, rt_prefix_n, m));
    CHK(up(dpa, rt_parents, m * 4));
    CHK(up(dl, rt_has_leaf_left, m));
    CHK(up(dr, rt_has_leaf_right, m));
    CHK(up(dlc, rt_left_child, m * 4));
  }
  if (!dn.ok()) return GTC_ERR_OOM;
  CHK(gtc_make_octree_u32(c, dn.as<gtc_octnode>(), o, dps.as<uint32_t>(), de.as<uint32_t>(), dc.as<uint32_t>(),
                          dp.as<uint8_t>(), dpa.as<int32_t>(), min_coord, range, n, dl.as<uint8_t>(), dr.as<uint8_t>(),
                          dlc.as<int32_t>(), nullptr));
  CHK(gtc_link_octree_u32(c, dn.as<gtc_octnode>(), o, dps.as<uint32_t>(), de.as<uint32_t>(), dc.as<uint32_t>(),
                          dp.as<uint8_t>(), dpa.as<int32_t>(), n, dl.as<uint8_t>(), dr.as<uint8_t>(),
                          dlc.as<int32_t>(), nullptr));
  CHK(finish(c));
  return down(oct_nodes, dn, (size_t)o * sizeof(gtc_octnode));
}

}  // extern "C"
