// cub_sort.cu - CUB's DeviceRadixSort::SortPairs behind a small C ABI, as a
// comparison point for bench.py's sort workload only (--workload cub_sort).
//
// Never linked into libgtc.so and never on the product path: it is built on
// demand by bench.py into its own library, so that the onesweep passes of
// this project can be timed beside the toolkit's onesweep implementation on
// the same keys, bit range and GPU.

#include <cstddef>
#include <cstdint>

#include <cub/device/device_radix_sort.cuh>
#include <cuda_runtime.h>

extern "C" {

// Temporary storage CUB needs for n pairs of key_bits-wide keys.
int cubref_ws_bytes(uint32_t n, int key_bits, size_t* bytes) {
  cudaError_t e;
  if (key_bits == 64) {
    cub::DoubleBuffer<uint64_t> k(nullptr, nullptr);
    cub::DoubleBuffer<uint32_t> v(nullptr, nullptr);
    e = cub::DeviceRadixSort::SortPairs(nullptr, *bytes, k, v, (int)n);
  } else {
    cub::DoubleBuffer<uint32_t> k(nullptr, nullptr);
    cub::DoubleBuffer<uint32_t> v(nullptr, nullptr);
    e = cub::DeviceRadixSort::SortPairs(nullptr, *bytes, k, v, (int)n);
  }
  return (int)e;
}

// Stable sort of (keys, vals) on bits [begin_bit, end_bit) with ping-pong
// buffers; *in_alt receives 1 when the result is in keys_alt / vals_alt.
int cubref_sort_pairs(void* keys, uint32_t* vals, void* keys_alt, uint32_t* vals_alt, uint32_t n, int key_bits,
                      int begin_bit, int end_bit, void* ws, size_t ws_bytes, void* stream, int* in_alt) {
  cudaError_t e;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cub::DoubleBuffer<uint32_t> v(vals, vals_alt);
  if (key_bits == 64) {
    cub::DoubleBuffer<uint64_t> k(static_cast<uint64_t*>(keys), static_cast<uint64_t*>(keys_alt));
    e = cub::DeviceRadixSort::SortPairs(ws, ws_bytes, k, v, (int)n, begin_bit, end_bit, s);
    *in_alt = k.selector;
  } else {
    cub::DoubleBuffer<uint32_t> k(static_cast<uint32_t*>(keys), static_cast<uint32_t*>(keys_alt));
    e = cub::DeviceRadixSort::SortPairs(ws, ws_bytes, k, v, (int)n, begin_bit, end_bit, s);
    *in_alt = k.selector;
  }
  return (int)e;
}

}  // extern "C"
