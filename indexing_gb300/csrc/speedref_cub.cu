// speedref_cub.cu -- an external speed reference for the sort phase, used by
// the benchmark only (never by the library): CUB's device-wide radix sort of
// (key, row id) pairs over the same column, so the hand-written digit passes
// of wah_sort.cu can be read against a widely used GPU radix sort on the same
// GB300.  Built into its own library, libwah_speedref.so.
#include <cub/device/device_radix_sort.cuh>
#include <cuda_runtime.h>
#include <stdint.h>

extern "C" {

// Temporary storage CUB needs for n pairs of (32-bit key, 32-bit value).
size_t speedref_sort_pairs_u32_bytes(uint64_t n) {
  size_t bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, bytes, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                  (const uint32_t*)nullptr, (uint32_t*)nullptr, (int64_t)n);
  return bytes;
}

// Temporary storage CUB needs for n pairs of (16-bit key, 32-bit value).
size_t speedref_sort_pairs_u16_bytes(uint64_t n) {
  size_t bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, bytes, (const uint16_t*)nullptr, (uint16_t*)nullptr,
                                  (const uint32_t*)nullptr, (uint32_t*)nullptr, (int64_t)n);
  return bytes;
}

// Stable sort of (keys_in, vals_in) by bits [begin_bit, end_bit) of the
// 32-bit keys; returns a cudaError_t.
int speedref_sort_pairs_u32(const uint32_t* keys_in, uint32_t* keys_out, const uint32_t* vals_in,
                            uint32_t* vals_out, uint64_t n, int begin_bit, int end_bit,
                            void* temp, size_t temp_bytes, void* stream) {
  return (int)cub::DeviceRadixSort::SortPairs(temp, temp_bytes, keys_in, keys_out, vals_in,
                                              vals_out, (int64_t)n, begin_bit, end_bit,
                                              static_cast<cudaStream_t>(stream));
}

// Stable sort of (keys_in, vals_in) by all 16 bits of the keys.
int speedref_sort_pairs_u16(const uint16_t* keys_in, uint16_t* keys_out, const uint32_t* vals_in,
                            uint32_t* vals_out, uint64_t n, void* temp, size_t temp_bytes,
                            void* stream) {
  return (int)cub::DeviceRadixSort::SortPairs(temp, temp_bytes, keys_in, keys_out, vals_in,
                                              vals_out, (int64_t)n, 0, 16,
                                              static_cast<cudaStream_t>(stream));
}

}  // extern "C"
