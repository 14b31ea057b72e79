/* CPU oracle of the sort path (test infrastructure only; see oracle.cpp). */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Bit-ordered comparison key of one raw key (cub/test/catch2_radix_sort_helper.cuh:174-214). */
uint64_t oracle_striped_key(uint64_t raw, int bytes, int kind, int begin_bit, int end_bit);
uint64_t oracle_striped_key_ex(uint64_t raw, int bytes, int kind, int begin_bit, int end_bit, int zero_to_minus);

/* Stable permutation that sorts `keys` (cccl_type_enum key_type) by their striped bits. */
int oracle_radix_permutation(
  int key_type, const void* keys, uint64_t n, int begin_bit, int end_bit, int descending, int threads, uint64_t* perm);

/* DeviceRadixSort result: keys (and values when value_bytes > 0) gathered by the permutation. */
int oracle_radix_sort(int key_type,
                      const void* keys_in,
                      void* keys_out,
                      uint64_t value_bytes,
                      const void* values_in,
                      void* values_out,
                      uint64_t n,
                      int begin_bit,
                      int end_bit,
                      int descending,
                      int threads);

/* DeviceSegmentedSort result (cub::DeviceSegmentedSort size classes and merge network). */
int oracle_segmented_sort(int key_type,
                          const void* keys_in,
                          void* keys_out,
                          uint64_t value_bytes,
                          const void* values_in,
                          void* values_out,
                          uint64_t num_items,
                          uint64_t num_segments,
                          const int64_t* begin_offsets,
                          const int64_t* end_offsets,
                          int descending,
                          int threads);

#ifdef __cplusplus
}
#endif
