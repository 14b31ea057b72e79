/* Error status of a finished sort.
 *
 * The reference's entry points return a CUresult for what they can check on the host
 * (c/parallel/src/radix_sort.cu:646-652) and leave everything that happens on the GPU to
 * CUDA's sticky errors; its look-back spins without a limit
 * (cub/cub/agent/agent_radix_sort_onesweep.cuh:315-325). Here every wait on the GPU is
 * bounded: a kernel that gives up records why in a status word, disables its stores and
 * returns, so the process and the context stay usable. The status word is word 0 of the
 * temporary storage of every cccl_device_radix_sort, cccl_device_segmented_sort,
 * cccl_gb300_segmented_radix_sort and cccl_gb300_learned_sort call (the allocation-free
 * entry point keeps it in its built-in array). This query reads it after the call's work
 * is done.
 */
#pragma once

#include <cuda.h>
#include <stddef.h>
#include <stdint.h>

#include <cccl/c/extern_c.h>

#if !defined(CCCL_GB300_API)
#  if defined(_WIN32)
#    define CCCL_GB300_API __declspec(dllexport)
#  else
#    define CCCL_GB300_API __attribute__((__visibility__("default")))
#  endif
#endif

/* Bits of the status word. */
#define CCCL_GB300_STATUS_WAIT_TIMEOUT 1u   /* a wait on another tile or a bulk copy ran out: result incomplete */
#define CCCL_GB300_STATUS_BAD_SEGMENT 2u    /* a segment reached past num_items, or held 2^30 keys or more: left unsorted */
#define CCCL_GB300_STATUS_SEG_CAPACITY 4u   /* overlapping segments held more large segments than planned: those skipped */

CCCL_C_EXTERN_C_BEGIN

/* Waits for `stream`, then reads and clears the status word of the sort that last ran with
 * `d_temp_storage` (of `temp_storage_bytes` bytes, the size the call was given). With
 * d_temp_storage == NULL it reads the allocation-free entry point's status for the current
 * context. *status_bits (may be NULL) receives the CCCL_GB300_STATUS_* bits. Returns
 *   CUDA_SUCCESS                 no bit set (also for temp storage under 4 bytes: such calls wait on nothing);
 *   CUDA_ERROR_LAUNCH_TIMEOUT    CCCL_GB300_STATUS_WAIT_TIMEOUT;
 *   CUDA_ERROR_INVALID_VALUE     CCCL_GB300_STATUS_BAD_SEGMENT or CCCL_GB300_STATUS_SEG_CAPACITY;
 *   the error of the stream synchronisation or of the read, if one fails. */
CCCL_GB300_API CUresult cccl_gb300_sort_status(
  const void* d_temp_storage, size_t temp_storage_bytes, CUstream stream, uint32_t* status_bits);

/* For tests of the failure path only. Changes the bounded waits of the kernels of one
 * loaded radix-sort build (its CUlibrary, in the current context): in every digit pass the
 * tile with index `skip_tile` keeps its look-back counts to itself, and every wait gives up
 * after `wait_limit_ns`. Successors of that tile then stop waiting, the pass reports
 * CCCL_GB300_STATUS_WAIT_TIMEOUT and all kernels return. skip_tile = 0xffffffff and
 * wait_limit_ns = 1000000000 restore the defaults. Not thread-safe against sorts in flight
 * on the same build. */
CCCL_GB300_API CUresult cccl_gb300_testing_set_wait_fault(CUlibrary radix_library, uint32_t skip_tile, uint64_t wait_limit_ns);

CCCL_C_EXTERN_C_END
