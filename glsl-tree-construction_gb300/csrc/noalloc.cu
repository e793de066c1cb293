// noalloc.cu - the onesweep sort of 32-bit keys without any device allocation.
//
// Who needs this: callers that sort inside a loop where the device allocator
// must not be touched.  cudaMalloc / cudaFree synchronise the whole device and
// can block for milliseconds, which stalls every other stream of a serving or
// real-time pipeline; some callers also hand all of HBM to their own
// allocator up front and have no way to give this library a workspace of the
// right size on demand.  gtc_sort_pairs_u32 needs a workspace from the caller
// (or allocates one in the context); gtc_sort_pairs_u32_noalloc instead keeps
// its scratch in a fixed array compiled into this library.
//
// The scratch: g_sort_scratch below, 4,210,944 bytes, enough for the
// histograms and look-back descriptors of up to GTC_NOALLOC_MAX_KEYS
// (4,194,304) keys.  Every GPU that loads the library holds it until the
// process exits.  All calls share it, so calls that overlap on the GPU (two
// streams, or two threads) race and corrupt each other's results; serialise
// them on one stream.  Each call clears the parts that must start at zero
// (counters and histograms with a memset, look-back descriptors inside the
// histogram kernel) before using them; nothing else of the previous call's
// contents is read.

#include <mutex>

#include "gtc_internal.cuh"

namespace gtc {

constexpr uint32_t NOALLOC_MAX_KEYS = 1u << 22;
// Same layout as sort_workspace_bytes(NOALLOC_MAX_KEYS, 4, ...): a 4160-word
// header (counters, counts, bin offsets) + 4 passes x 1024 tiles x 256 digits.
constexpr size_t NOALLOC_SCRATCH_BYTES = (4160 + 4ull * 1024 * 256) * 4;

static __device__ __align__(256) unsigned char g_sort_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of g_sort_scratch per device ordinal.  In host code the
// symbol g_sort_scratch is only a host-side stand-in, so its address is looked
// up once per device (with that device current) and cached.
static std::mutex g_scratch_mu;
static void* g_scratch_addr[64] = {};

static cudaError_t scratch_address(int dev, void** out) {
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

Launch context_launch(gtc_ctx* ctx, gtc_stream_t stream);
int context_device(const gtc_ctx* ctx);
gtc_status context_error(gtc_ctx* ctx, gtc_status s, const char* msg, cudaError_t e);

}  // namespace gtc

using namespace gtc;

extern "C" GTC_API gtc_status gtc_sort_pairs_u32_noalloc(gtc_ctx* ctx, uint32_t* keys, uint32_t* vals,
                                                         uint32_t* keys_alt, uint32_t* vals_alt, uint32_t n,
                                                         int begin_bit, int end_bit, gtc_stream_t stream) {
  if (!ctx) return GTC_ERR_INVALID_ARG;
  if (!(0 <= begin_bit && begin_bit < end_bit && end_bit <= 32))
    return context_error(ctx, GTC_ERR_INVALID_ARG, "bit range must satisfy 0 <= begin < end <= 32", cudaSuccess);
  if (n > NOALLOC_MAX_KEYS)
    return context_error(ctx, GTC_ERR_INVALID_ARG,
                         "gtc_sort_pairs_u32_noalloc: n exceeds the 4194304-key limit of its static scratch",
                         cudaSuccess);
  if (n == 0) return GTC_OK;
  if (!keys || !keys_alt || (vals && !vals_alt))
    return context_error(ctx, GTC_ERR_INVALID_ARG, "keys, keys_alt (and vals_alt with vals) are required",
                         cudaSuccess);
  const int passes = (end_bit - begin_bit + 7) / 8;
  if (sort_workspace_bytes(n, passes, 0) > NOALLOC_SCRATCH_BYTES)
    return context_error(ctx, GTC_ERR_INVALID_ARG, "static scratch smaller than the sort layout", cudaSuccess);
  // The scratch address belongs to the current device, the stream and the
  // status word to the context's: the two must agree.
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return context_error(ctx, GTC_ERR_CUDA, "cudaGetDevice", e);
  if (dev != context_device(ctx))
    return context_error(ctx, GTC_ERR_INVALID_ARG,
                         "gtc_sort_pairs_u32_noalloc: the context's device must be the current device", cudaSuccess);
  void* scratch = nullptr;
  e = scratch_address(dev, &scratch);
  if (e != cudaSuccess) return context_error(ctx, GTC_ERR_CUDA, "cudaGetSymbolAddress(g_sort_scratch)", e);

  const Launch L = context_launch(ctx, stream);
  const SortWorkspace W = carve_sort_workspace(scratch, n, passes, 0);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if ((e = cudaMemsetAsync(W.header, 0, W.header_words * 4, s)) != cudaSuccess)
    return context_error(ctx, GTC_ERR_CUDA, "clearing the static scratch", e);
  if ((e = launch_global_hist<uint32_t>(L, keys, n, begin_bit, end_bit, W, passes)) != cudaSuccess)
    return context_error(ctx, GTC_ERR_CUDA, "global histogram", e);
  bool in_alt = false;
  if ((e = launch_onesweep_passes<uint32_t>(L, keys, vals, keys_alt, vals_alt, n, begin_bit, end_bit, W, passes,
                                            &in_alt, nullptr)) != cudaSuccess)
    return context_error(ctx, GTC_ERR_CUDA, "onesweep passes", e);
  if (in_alt) {
    if ((e = cudaMemcpyAsync(keys, keys_alt, (size_t)n * 4, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
      return context_error(ctx, GTC_ERR_CUDA, "copy back", e);
    if (vals && (e = cudaMemcpyAsync(vals, vals_alt, (size_t)n * 4, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
      return context_error(ctx, GTC_ERR_CUDA, "copy back", e);
  }
  return GTC_OK;
}
