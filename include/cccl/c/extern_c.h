/* C linkage helpers for the sort C ABI.
 * Replaces c/parallel/include/cccl/c/extern_c.h (same macro names, so code written
 * against the reference headers compiles unchanged). */
#pragma once

#ifdef __cplusplus
#  define CCCL_C_EXTERN_C_BEGIN extern "C" {
#  define CCCL_C_EXTERN_C_END }
#else
#  define CCCL_C_EXTERN_C_BEGIN
#  define CCCL_C_EXTERN_C_END
#endif
