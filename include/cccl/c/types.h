/* Shared C-ABI types of the sort path.
 *
 * Replaces c/parallel/include/cccl/c/types.h. Every enum value, struct member and
 * member order below is kept identical to the reference so that a caller built against
 * the reference header (ctypes/cython/C) can bind this library unchanged:
 *   cccl_type_enum        types.h:31-47     cccl_type_info     types.h:49-54
 *   cccl_op_kind_t        types.h:56-89     cccl_op_t          types.h:97-111
 *   cccl_build_config     types.h:113-119   cccl_iterator_t    types.h:141-151
 *   cccl_sort_order_t     types.h:153-157   cccl_payload_kind_t types.h:179-183
 */
#pragma once

#ifndef CCCL_C_EXPERIMENTAL
#  error "C exposure is experimental and subject to change. Define CCCL_C_EXPERIMENTAL to acknowledge this notice."
#endif

#if defined(_WIN32)
#  define CCCL_C_API __declspec(dllexport)
#else
#  define CCCL_C_API __attribute__((__visibility__("default")))
#endif

#include <stddef.h>
#include <stdint.h>

#include <cccl/c/extern_c.h>

CCCL_C_EXTERN_C_BEGIN

typedef enum cccl_type_enum
{
  CCCL_INT8 = 0,
  CCCL_INT16 = 1,
  CCCL_INT32 = 2,
  CCCL_INT64 = 3,
  CCCL_UINT8 = 4,
  CCCL_UINT16 = 5,
  CCCL_UINT32 = 6,
  CCCL_UINT64 = 7,
  CCCL_FLOAT16 = 8,
  CCCL_FLOAT32 = 9,
  CCCL_FLOAT64 = 10,
  CCCL_STORAGE = 11, /* opaque bytes: allowed as a sort value, not as a key */
  CCCL_BOOLEAN = 12,
} cccl_type_enum;

typedef struct cccl_type_info
{
  size_t size;
  size_t alignment;
  cccl_type_enum type;
} cccl_type_info;

typedef enum cccl_op_kind_t
{
  CCCL_STATELESS = 0,
  CCCL_STATEFUL = 1,
  CCCL_PLUS = 2,
  CCCL_MINUS = 3,
  CCCL_MULTIPLIES = 4,
  CCCL_DIVIDES = 5,
  CCCL_MODULUS = 6,
  CCCL_EQUAL_TO = 7,
  CCCL_NOT_EQUAL_TO = 8,
  CCCL_GREATER = 9,
  CCCL_LESS = 10,
  CCCL_GREATER_EQUAL = 11,
  CCCL_LESS_EQUAL = 12,
  CCCL_LOGICAL_AND = 13,
  CCCL_LOGICAL_OR = 14,
  CCCL_LOGICAL_NOT = 15,
  CCCL_BIT_AND = 16,
  CCCL_BIT_OR = 17,
  CCCL_BIT_XOR = 18,
  CCCL_BIT_NOT = 19,
  CCCL_IDENTITY = 20,
  CCCL_NEGATE = 21,
  CCCL_MINIMUM = 22,
  CCCL_MAXIMUM = 23,
} cccl_op_kind_t;

typedef enum cccl_op_code_type
{
  CCCL_OP_LTOIR = 0,
  CCCL_OP_CPP_SOURCE = 1
} cccl_op_code_type;

/* A user operator. The sort path only inspects `name`: an empty or null name means
 * "no decomposer" (the identity decomposer); anything else is rejected with
 * CUDA_ERROR_NOT_SUPPORTED because custom key decomposition is not offered. */
typedef struct cccl_op_t
{
  cccl_op_kind_t type;
  const char* name;
  const char* code;
  size_t code_size;
  cccl_op_code_type code_type;
  size_t size;
  size_t alignment;
  void* state;
  const char** extra_ltoirs;
  size_t* extra_ltoir_sizes;
  size_t num_extra_ltoirs;
  cccl_op_code_type* extra_code_types;
} cccl_op_t;

/* Accepted for signature compatibility; kernels are precompiled, so the flags and
 * include directories have no effect. */
typedef struct cccl_build_config
{
  const char** extra_compile_flags;
  size_t num_extra_compile_flags;
  const char** extra_include_dirs;
  size_t num_extra_include_dirs;
} cccl_build_config;

typedef enum cccl_iterator_kind_t
{
  CCCL_POINTER = 0,
  CCCL_ITERATOR = 1,
} cccl_iterator_kind_t;

typedef struct cccl_value_t
{
  cccl_type_info type;
  void* state;
} cccl_value_t;

typedef union
{
  int64_t signed_offset;
  uint64_t unsigned_offset;
} cccl_increment_t;

typedef void (*cccl_host_op_fn_ptr_t)(void*, cccl_increment_t);

/* For CCCL_POINTER iterators `state` is the device pointer itself. */
typedef struct cccl_iterator_t
{
  size_t size;
  size_t alignment;
  cccl_iterator_kind_t type;
  cccl_op_t advance;
  cccl_op_t dereference;
  cccl_type_info value_type;
  void* state;
  cccl_host_op_fn_ptr_t host_advance;
} cccl_iterator_t;

typedef enum cccl_sort_order_t
{
  CCCL_ASCENDING = 0,
  CCCL_DESCENDING = 1,
} cccl_sort_order_t;

typedef enum cccl_init_kind_t
{
  CCCL_VALUE_INIT = 0,
  CCCL_FUTURE_VALUE_INIT = 1,
  CCCL_NO_INIT = 2,
} cccl_init_kind_t;

typedef enum cccl_determinism_t
{
  CCCL_NOT_GUARANTEED = 0,
  CCCL_RUN_TO_RUN = 1,
  CCCL_GPU_TO_GPU = 2,
} cccl_determinism_t;

typedef enum cccl_binary_search_mode_t
{
  CCCL_BINARY_SEARCH_LOWER_BOUND = 0,
  CCCL_BINARY_SEARCH_UPPER_BOUND = 1,
} cccl_binary_search_mode_t;

typedef enum cccl_payload_kind_t
{
  CCCL_PAYLOAD_LTOIR = 0,
  CCCL_PAYLOAD_CUBIN = 1,
} cccl_payload_kind_t;

CCCL_C_EXTERN_C_END
