/* Build-result serialization helpers.
 * Replaces c/parallel/include/cccl/c/serialization.h (algorithm tags :27-41 and
 * cccl_serialization_buffer_free :45-46 keep the reference's values and signature). */
#pragma once

#ifndef CCCL_C_EXPERIMENTAL
#  error "C exposure is experimental and subject to change. Define CCCL_C_EXPERIMENTAL to acknowledge this notice."
#endif

#include <stddef.h>
#include <stdint.h>

#include <cccl/c/extern_c.h>
#include <cccl/c/types.h>

CCCL_C_EXTERN_C_BEGIN

typedef enum cccl_serialization_algo_t
{
  CCCL_SERIALIZATION_ALGO_REDUCE = 1,
  CCCL_SERIALIZATION_ALGO_SCAN = 2,
  CCCL_SERIALIZATION_ALGO_SEGMENTED_REDUCE = 3,
  CCCL_SERIALIZATION_ALGO_TRANSFORM = 4,
  CCCL_SERIALIZATION_ALGO_BINARY_SEARCH = 5,
  CCCL_SERIALIZATION_ALGO_MERGE_SORT = 6,
  CCCL_SERIALIZATION_ALGO_RADIX_SORT = 7,
  CCCL_SERIALIZATION_ALGO_SEGMENTED_SORT = 8,
  CCCL_SERIALIZATION_ALGO_THREE_WAY_PARTITION = 9,
  CCCL_SERIALIZATION_ALGO_UNIQUE_BY_KEY = 10,
  CCCL_SERIALIZATION_ALGO_HISTOGRAM = 11,
  CCCL_SERIALIZATION_ALGO_FOR = 12,
} cccl_serialization_algo_t;

/* Frees a buffer returned by cccl_device_radix_sort_serialize or
 * cccl_device_segmented_sort_serialize (the allocation belongs to this library). */
CCCL_C_API void cccl_serialization_buffer_free(void* buf);

CCCL_C_EXTERN_C_END
