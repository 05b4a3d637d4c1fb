// The library bar for the sort leg of bench.py: CUB's DeviceRadixSort::SortPairs (the onesweep radix sort the CUDA
// toolkit ships) on 16-bit keys with 32-bit values over bits [0, end_bit).  A comparison baseline only: the pipeline
// never calls it.  Built as its own small library (libcub_sort.so) by splatlight_gb300/build.py.
#include <cstdint>

#include <cub/device/device_radix_sort.cuh>

extern "C" {

// Sorts n (key, value) pairs by the low end_bit bits of the keys, stably.  temp / temp_bytes: CUB's scratch; with
// temp NULL only *temp_bytes is set.  Returns the cudaError_t.
__attribute__((visibility("default"))) int cub_sort_pairs16(const uint16_t* keys_in, uint16_t* keys_out,
                                                            const uint32_t* vals_in, uint32_t* vals_out, uint32_t n,
                                                            int end_bit, void* temp, size_t* temp_bytes,
                                                            void* stream) {
  return (int)cub::DeviceRadixSort::SortPairs(temp, *temp_bytes, keys_in, keys_out, vals_in, vals_out, (int64_t)n, 0,
                                               end_bit, reinterpret_cast<cudaStream_t>(stream));
}

__attribute__((visibility("default"))) int cub_sort_pairs32(const uint32_t* keys_in, uint32_t* keys_out,
                                                            const uint32_t* vals_in, uint32_t* vals_out, uint32_t n,
                                                            int end_bit, void* temp, size_t* temp_bytes,
                                                            void* stream) {
  return (int)cub::DeviceRadixSort::SortPairs(temp, *temp_bytes, keys_in, keys_out, vals_in, vals_out, (int64_t)n, 0,
                                               end_bit, reinterpret_cast<cudaStream_t>(stream));
}

}  // extern "C"
