// morton.cu - standalone Morton encode (k_ComputeMortonCode,
// morton.comp:60-67): one 16-byte point load per key, streaming loads, the
// key and (optionally) the iota payload written coalesced.

#include "gtc_internal.cuh"

namespace gtc {

template <class K>
__global__ void __launch_bounds__(256) morton_kernel(const float4* __restrict__ pts, K* __restrict__ keys,
                                                     uint32_t* __restrict__ idx, uint32_t n, float mn, float rg,
                                                     float inv_rg) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    keys[i] = encode_point<K>(__ldcs(pts + i), mn, rg, inv_rg);
    if (idx) idx[i] = (uint32_t)i;
  }
}

template <class K>
static cudaError_t launch_morton(const Launch& L, const float4* pts, K* keys, uint32_t* idx, uint32_t n, float mn,
                                 float rg) {
  if (n == 0) return cudaSuccess;
  const uint32_t grid = max(1u, min(ceil_div(n, 256 * 4), (uint32_t)L.num_sms * 16));
  morton_kernel<K><<<grid, 256, 0, L.stream>>>(pts, keys, idx, n, mn, rg, pow2_reciprocal(rg));
  return cudaGetLastError();
}

// Points in the order of a payload: out[i] = pts[idx[i]].  One 16-byte load
// and store per point; out-of-range indices give zeros and flag the status.
__global__ void __launch_bounds__(256) gather_points_kernel(const float4* __restrict__ pts, uint32_t n_pts,
                                                            const uint32_t* __restrict__ idx, uint32_t count,
                                                            float4* __restrict__ out, uint32_t* status) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const uint32_t j = idx[i];
    if (j < n_pts) {
      out[i] = pts[j];
    } else {
      out[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      atomicOr(status, DEV_BAD_INPUT);
    }
  }
}

cudaError_t launch_gather_points(const Launch& L, const float4* pts, uint32_t n_pts, const uint32_t* idx,
                                 uint32_t count, float4* out) {
  if (count == 0) return cudaSuccess;
  const uint32_t grid = max(1u, min(ceil_div(count, 256 * 4), (uint32_t)L.num_sms * 16));
  gather_points_kernel<<<grid, 256, 0, L.stream>>>(pts, n_pts, idx, count, out, L.status);
  return cudaGetLastError();
}

cudaError_t launch_morton32(const Launch& L, const float4* pts, uint32_t* keys, uint32_t* idx, uint32_t n, float mn,
                            float rg) {
  return launch_morton<uint32_t>(L, pts, keys, idx, n, mn, rg);
}
cudaError_t launch_morton64(const Launch& L, const float4* pts, uint64_t* keys, uint32_t* idx, uint32_t n, float mn,
                            float rg) {
  return launch_morton<uint64_t>(L, pts, keys, idx, n, mn, rg);
}

}  // namespace gtc
