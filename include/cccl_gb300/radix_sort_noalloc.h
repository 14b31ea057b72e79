/* Radix sort of 32-bit unsigned keys (optionally carrying 32-bit values) that allocates no
 * memory.
 *
 * No counterpart in the reference: CCCL's sort asks the caller for temporary storage, which
 * the caller normally gets from cudaMalloc. Some callers cannot allocate on their sort path:
 * cudaMalloc/cudaFree synchronize the device and would stall every other stream, and code
 * that runs inside a host framework or service with a fixed device-memory budget may not be
 * allowed to allocate outside that budget at all. This entry point needs no temporary
 * storage argument: its scratch space is a fixed array of device memory inside the library
 * (CCCL_GB300_NOALLOC_SCRATCH_BYTES = 8,763,648 bytes, 8.36 MiB, held in every CUDA context
 * that loads the library until the context is destroyed or the process exits).
 *
 * Limits and behaviour:
 *  - num_items <= CCCL_GB300_NOALLOC_MAX_ITEMS; larger inputs are rejected with
 *    CUDA_ERROR_INVALID_VALUE and an explanatory message, nothing is launched;
 *  - keys and values are read from *_in and the sorted result is written to *_out
 *    (the inputs are not modified); pass NULL values for a keys-only sort;
 *  - order and [begin_bit, end_bit) follow cccl_device_radix_sort; the output is
 *    identical to cccl_device_radix_sort's for the same arguments;
 *  - it runs in the CUDA context current on the calling thread (the runtime's primary
 *    context of the current device when none is); the first call in each context looks up
 *    that context's copy of the scratch array (and sets kernel attributes); make that first
 *    call before any stream capture;
 *  - every call in a context uses the same scratch array, so calls whose work overlaps on
 *    the GPU (different streams, or different host threads on one device) race and corrupt
 *    each other's results: order them on one stream or synchronize between them;
 *  - work is enqueued on `stream` and the call returns without waiting for it;
 *    cccl_gb300_sort_status(NULL, 0, stream, &bits) (sort_status.h) waits for it and
 *    reports whether a bounded wait inside the sort ran out.
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
#define CCCL_GB300_NOALLOC_SCRATCH_BYTES 8763648u

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
