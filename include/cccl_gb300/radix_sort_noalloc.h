/* Radix sort of 32-bit unsigned keys (optionally carrying 32-bit values) that allocates no
 * memory.
 *
 * No counterpart in the reference: CCCL's sort asks the caller for temporary storage, which
 * the caller normally gets from cudaMalloc. Some callers cannot allocate on their sort path:
 * cudaMalloc/cudaFree synchronize the device and would stall every other stream, and code
 * that runs inside a host framework or service with a fixed device-memory budget may not be
 * allowed to allocate outside that budget at all. This entry point needs no temporary
 * storage argument: its scratch space is a fixed array of device memory inside the library
 * (about 8.4 MB per GPU, held by every GPU that loads the library until the process exits).
 *
 * Limits and behaviour:
 *  - num_items <= CCCL_GB300_NOALLOC_MAX_ITEMS; larger inputs are rejected with
 *    CUDA_ERROR_INVALID_VALUE and an explanatory message, nothing is launched;
 *  - keys and values are read from *_in and the sorted result is written to *_out
 *    (the inputs are not modified); pass NULL values for a keys-only sort;
 *  - order and [begin_bit, end_bit) follow cccl_device_radix_sort; the output is
 *    identical to cccl_device_radix_sort's for the same arguments;
 *  - the first call on a device looks up the scratch array's device address (and sets
 *    kernel attributes) for that device; make that first call before any stream capture;
 *  - every call uses the same scratch array, so calls whose work overlaps on the GPU
 *    (different streams, or different host threads on one device) race and corrupt each
 *    other's results: order them on one stream or synchronize between them;
 *  - work is enqueued on `stream` and the call returns without waiting for it.
 */
#pragma once

#include <cuda.h>
#include <stdbool.h>
#include <stdint.h>

#include <cccl/c/extern_c.h>

#if defined(_WIN32)
#  define CCCL_GB300_API __declspec(dllexport)
#else
#  define CCCL_GB300_API __attribute__((__visibility__("default")))
#endif

#define CCCL_GB300_NOALLOC_MAX_ITEMS (1u << 20)

CCCL_C_EXTERN_C_BEGIN

CCCL_GB300_API CUresult cccl_gb300_radix_sort_u32_noalloc(
  const uint32_t* d_keys_in,
  uint32_t* d_keys_out,
  const uint32_t* d_values_in,
  uint32_t* d_values_out,
  uint64_t num_items,
  int begin_bit,
  int end_bit,
  bool descending,
  CUstream stream);

CCCL_C_EXTERN_C_END
