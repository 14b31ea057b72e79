/* Launch tracing of the sort library.
 *
 * No counterpart in the reference's C ABI. It plays the role of CUB's debug launch log
 * (CUB_DEBUG_LOG in cub/cub/device/dispatch/dispatch_radix_sort.cuh:633-668,742-753):
 * when an observer is installed, the dispatcher calls it immediately before and after
 * enqueuing every kernel, on the host thread that issued the sort, with the kernel's
 * role ("init", "histogram", "onesweep", "single_tile", ...) and its stream. A profiler
 * or benchmark can record CUDA events on that stream to time each kernel. The observer
 * must not launch work that depends on the sort. Pass NULL to remove it.
 */
#pragma once

#include <cuda.h>

#include <cccl/c/extern_c.h>

#if defined(_WIN32)
#  define CCCL_GB300_API __declspec(dllexport)
#else
#  define CCCL_GB300_API __attribute__((__visibility__("default")))
#endif

CCCL_C_EXTERN_C_BEGIN

/* phase: 0 = before the launch is enqueued, 1 = after. */
typedef void (*cccl_gb300_launch_observer_t)(void* user, const char* role, int phase, CUstream stream);

CCCL_GB300_API void cccl_gb300_set_launch_observer(cccl_gb300_launch_observer_t observer, void* user);

CCCL_C_EXTERN_C_END
