/* Segmented radix sort: the semantics of cub::DeviceSegmentedRadixSort
 * (cub/cub/device/device_segmented_radix_sort.cuh:234-270) through the segmented sort's build.
 *
 * No counterpart in the reference's C ABI, which exposes only DeviceSegmentedSort
 * (c/parallel/include/cccl/c/segmented_sort.h). Differences from cccl_device_segmented_sort:
 * every segment is sorted by radix digits over key bits [begin_bit, end_bit) (no merge
 * networks, so NaNs and -0.0/+0.0 order by their bit patterns, -0.0 equal to +0.0, ties
 * stable), and the returned selector follows DeviceSegmentedRadixSort's dispatch:
 * (max(ceil((end_bit - begin_bit) / 6), 1) & 1) when overwriting is allowed (5-bit digits
 * for 1-byte keys), else the result is in d_keys_out.
 *
 * The build is a cccl_device_segmented_sort_build_result_t of the same key/value types and
 * order; offsets are pointers to 32- or 64-bit integers; values are absent, 4 or 8 bytes.
 */
#pragma once

#ifndef CCCL_C_EXPERIMENTAL
#  error "C exposure is experimental and subject to change. Define CCCL_C_EXPERIMENTAL to acknowledge this notice."
#endif

#include <cuda.h>

#include <stdbool.h>
#include <stdint.h>

#include <cccl/c/extern_c.h>
#include <cccl/c/segmented_sort.h>
#include <cccl_gb300/sort_trace.h>

CCCL_C_EXTERN_C_BEGIN

CCCL_GB300_API CUresult cccl_gb300_segmented_radix_sort(
  cccl_device_segmented_sort_build_result_t build,
  void* d_temp_storage,
  size_t* temp_storage_bytes,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_keys_out,
  cccl_iterator_t d_values_in,
  cccl_iterator_t d_values_out,
  uint64_t num_items,
  uint64_t num_segments,
  cccl_iterator_t start_offset_in,
  cccl_iterator_t end_offset_in,
  int begin_bit,
  int end_bit,
  bool is_overwrite_okay,
  int* selector,
  CUstream stream);

CCCL_C_EXTERN_C_END
