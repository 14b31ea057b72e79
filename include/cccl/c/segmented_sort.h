/* C ABI of the batched segmented sort.
 *
 * Replaces c/parallel/include/cccl/c/segmented_sort.h. The build-result struct keeps
 * the reference's member list and order (segmented_sort.h:27-53).
 *
 * What the members hold here:
 *  - payload: the library's precompiled sm_103a cubin (CCCL_PAYLOAD_CUBIN).
 *  - segmented_sort_kernel_small   warp-class kernel (segments <= the medium tile), which
 *                                  reproduces CUB's sub-warp merge sort exactly
 *  - segmented_sort_kernel_large   block-class kernel (one CTA sorts one segment in
 *                                  shared memory with stable 8-bit radix passes)
 *  - segmented_sort_fallback_kernel  device-class driver: segments too large for one
 *                                  CTA go through the plain onesweep pass kernel
 *  - three_way_partition_*_kernel  on-device size-class binning (no host round trip)
 *  - large/small_segments_selector_op: zero-filled (the size classes are built in).
 */
#pragma once

#ifndef CCCL_C_EXPERIMENTAL
#  error "C exposure is experimental and subject to change. Define CCCL_C_EXPERIMENTAL to acknowledge this notice."
#endif

#include <cuda.h>
#include <stdbool.h>
#include <stdint.h>

#include <cccl/c/extern_c.h>
#include <cccl/c/types.h>

CCCL_C_EXTERN_C_BEGIN

typedef struct cccl_device_segmented_sort_build_result_t
{
  int cc;
  void* payload;
  size_t payload_size;
  cccl_payload_kind_t payload_kind;
  CUlibrary library;
  cccl_type_info key_type;
  cccl_type_info offset_type;
  cccl_op_t large_segments_selector_op;
  cccl_op_t small_segments_selector_op;
  CUkernel segmented_sort_fallback_kernel;
  CUkernel segmented_sort_kernel_small;
  CUkernel segmented_sort_kernel_large;
  CUkernel three_way_partition_init_kernel;
  CUkernel three_way_partition_kernel;
  void* runtime_policy;
  size_t runtime_policy_size;
  void* partition_runtime_policy;
  size_t partition_runtime_policy_size;
  cccl_sort_order_t order;
  char* segmented_sort_fallback_kernel_lowered_name;
  char* segmented_sort_kernel_small_lowered_name;
  char* segmented_sort_kernel_large_lowered_name;
  char* three_way_partition_init_kernel_lowered_name;
  char* three_way_partition_kernel_lowered_name;
} cccl_device_segmented_sort_build_result_t;

/* Replaces segmented_sort.h:56-69 (segmented_sort.cu build). */
CCCL_C_API CUresult cccl_device_segmented_sort_build(
  cccl_device_segmented_sort_build_result_t* build,
  cccl_sort_order_t sort_order,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_values_in,
  cccl_iterator_t begin_offset_in,
  cccl_iterator_t end_offset_in,
  int cc_major,
  int cc_minor,
  const char* cub_path,
  const char* thrust_path,
  const char* libcudacxx_path,
  const char* ctk_path);

/* Replaces segmented_sort.h:72-85. `config` is accepted and ignored. */
CCCL_C_API CUresult cccl_device_segmented_sort_build_ex(
  cccl_device_segmented_sort_build_result_t* build,
  cccl_sort_order_t sort_order,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_values_in,
  cccl_iterator_t begin_offset_in,
  cccl_iterator_t end_offset_in,
  int cc_major,
  int cc_minor,
  const char* cub_path,
  const char* thrust_path,
  const char* libcudacxx_path,
  const char* ctk_path,
  cccl_build_config* config);

/* Replaces segmented_sort.h:87-99. */
CCCL_C_API CUresult cccl_device_segmented_sort_compile(
  cccl_device_segmented_sort_build_result_t* build,
  cccl_sort_order_t sort_order,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_values_in,
  cccl_iterator_t begin_offset_in,
  cccl_iterator_t end_offset_in,
  int cc_major,
  int cc_minor,
  const char* cub_path,
  const char* thrust_path,
  const char* libcudacxx_path,
  const char* ctk_path,
  cccl_build_config* config);

/* Replaces segmented_sort.h:101. */
CCCL_C_API CUresult cccl_device_segmented_sort_load(cccl_device_segmented_sort_build_result_t* build);

/* Runs the sort. Replaces segmented_sort.h:103-117 (segmented_sort.cu:859-985).
 * Segment i is [start_offset_in[i], end_offset_in[i]); offsets are pointers to int32 or
 * int64. `selector` must not be NULL. Keys inside each segment follow
 * cub::DeviceSegmentedSort order, including its placement of NaN keys. */
CCCL_C_API CUresult cccl_device_segmented_sort(
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
  bool is_overwrite_okay,
  int* selector,
  CUstream stream);

/* Replaces segmented_sort.h:119-123. */
CCCL_C_API CUresult cccl_device_segmented_sort_link_ltoir(
  cccl_device_segmented_sort_build_result_t* build,
  const void** input_blobs,
  const size_t* input_sizes,
  size_t num_inputs);

/* Replaces segmented_sort.h:125-131. */
CCCL_C_API CUresult cccl_device_segmented_sort_serialize(
  const cccl_device_segmented_sort_build_result_t* build, void** out_buf, size_t* out_size);

/* Replaces segmented_sort.h:133-137. */
CCCL_C_API CUresult
cccl_device_segmented_sort_deserialize(cccl_device_segmented_sort_build_result_t* build, const void* buf, size_t size);

/* Replaces segmented_sort.h:139. */
CCCL_C_API CUresult cccl_device_segmented_sort_cleanup(cccl_device_segmented_sort_build_result_t* bld_ptr);

CCCL_C_EXTERN_C_END
