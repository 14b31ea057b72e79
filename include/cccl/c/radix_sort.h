/* C ABI of the device radix sort (plain path).
 *
 * Replaces c/parallel/include/cccl/c/radix_sort.h. The build-result struct keeps the
 * reference's member list and order (radix_sort.h:27-61) so that existing bindings
 * (python/cuda_cccl's cython wrapper, c/parallel/test) can use it unchanged.
 *
 * What the members hold here:
 *  - payload / payload_kind: the library's precompiled sm_103a cubin (CCCL_PAYLOAD_CUBIN);
 *    nothing is JIT-compiled, so the *_path arguments of build/compile are ignored.
 *  - library: the CUlibrary loaded from that cubin by cccl_device_radix_sort_load.
 *  - kernel handles, named for the role CUB's kernels play:
 *      histogram_kernel              all-pass digit histogram + fused exclusive scan
 *      exclusive_sum_kernel          same kernel as histogram_kernel (the scan is fused)
 *      init_bins_and_counters_kernel control-block initialisation
 *      init_lookback_kernel          same kernel as init_bins_and_counters_kernel
 *      onesweep_kernel               one 8-bit digit pass (rank, look-back, scatter); persistent,
 *                                    bulk-copy prefetch, cooperative launch
 *      downsweep_kernel              the same pass, one CTA per tile, for buffers that are not
 *                                    16-byte aligned
 *      single_tile_kernel            whole sort in one CTA for small inputs
 *      alt_downsweep_kernel          first-pass variant for full-width integer keys-only
 *                                    sorts (order inside a digit bucket is free there)
 *      upsweep/scan_bins/alt_upsweep: CUB's multi-pass kernels are never used on
 *      sm_90+; these members alias the histogram kernel so they are non-null.
 *  - runtime_policy: the tile configuration chosen for the key/value types.
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

typedef struct cccl_device_radix_sort_build_result_t
{
  int cc;
  void* payload;
  size_t payload_size;
  cccl_payload_kind_t payload_kind;
  CUlibrary library;
  cccl_type_info key_type;
  cccl_type_info value_type;
  CUkernel single_tile_kernel;
  CUkernel upsweep_kernel;
  CUkernel alt_upsweep_kernel;
  CUkernel scan_bins_kernel;
  CUkernel downsweep_kernel;
  CUkernel alt_downsweep_kernel;
  CUkernel histogram_kernel;
  CUkernel exclusive_sum_kernel;
  CUkernel init_bins_and_counters_kernel;
  CUkernel init_lookback_kernel;
  CUkernel onesweep_kernel;
  cccl_sort_order_t order;
  void* runtime_policy;
  size_t runtime_policy_size;
  char* single_tile_kernel_lowered_name;
  char* upsweep_kernel_lowered_name;
  char* alt_upsweep_kernel_lowered_name;
  char* scan_bins_kernel_lowered_name;
  char* downsweep_kernel_lowered_name;
  char* alt_downsweep_kernel_lowered_name;
  char* histogram_kernel_lowered_name;
  char* exclusive_sum_kernel_lowered_name;
  char* init_bins_and_counters_kernel_lowered_name;
  char* init_lookback_kernel_lowered_name;
  char* onesweep_kernel_lowered_name;
} cccl_device_radix_sort_build_result_t;

/* compile + load. Replaces radix_sort.h:63-75 (radix_sort.cu:700-728). */
CCCL_C_API CUresult cccl_device_radix_sort_build(
  cccl_device_radix_sort_build_result_t* build,
  cccl_sort_order_t sort_order,
  cccl_iterator_t input_keys_it,
  cccl_iterator_t input_values_it,
  cccl_op_t decomposer,
  const char* decomposer_return_type,
  int cc_major,
  int cc_minor,
  const char* cub_path,
  const char* thrust_path,
  const char* libcudacxx_path,
  const char* ctk_path);

/* Replaces radix_sort.h:78-91 (radix_sort.cu:541-580). `config` is accepted and ignored. */
CCCL_C_API CUresult cccl_device_radix_sort_build_ex(
  cccl_device_radix_sort_build_result_t* build,
  cccl_sort_order_t sort_order,
  cccl_iterator_t input_keys_it,
  cccl_iterator_t input_values_it,
  cccl_op_t decomposer,
  const char* decomposer_return_type,
  int cc_major,
  int cc_minor,
  const char* cub_path,
  const char* thrust_path,
  const char* libcudacxx_path,
  const char* ctk_path,
  cccl_build_config* config);

/* Fills the build result (payload, names, policy) without touching the GPU.
 * Replaces radix_sort.h:93-106 (radix_sort.cu:221-472). Only cc 10.3 (GB300) is
 * accepted; other targets return CUDA_ERROR_NOT_SUPPORTED. */
CCCL_C_API CUresult cccl_device_radix_sort_compile(
  cccl_device_radix_sort_build_result_t* build,
  cccl_sort_order_t sort_order,
  cccl_iterator_t input_keys_it,
  cccl_iterator_t input_values_it,
  cccl_op_t decomposer,
  const char* decomposer_return_type,
  int cc_major,
  int cc_minor,
  const char* cub_path,
  const char* thrust_path,
  const char* libcudacxx_path,
  const char* ctk_path,
  cccl_build_config* config);

/* Loads the payload into a CUlibrary and resolves the kernels.
 * Replaces radix_sort.h:108 (radix_sort.cu:474-539). */
CCCL_C_API CUresult cccl_device_radix_sort_load(cccl_device_radix_sort_build_result_t* build);

/* Runs the sort. Replaces radix_sort.h:110-124 (radix_sort.cu:582-698).
 * d_temp_storage == NULL: writes the required size to *temp_storage_bytes and returns.
 * All four iterators must be CCCL_POINTER; values are absent when d_values_in.state is
 * NULL. With is_overwrite_okay the result is in the buffer *selector names
 * (0 = the *_in buffers, 1 = the *_out buffers); otherwise it is always in *_out. */
CCCL_C_API CUresult cccl_device_radix_sort(
  cccl_device_radix_sort_build_result_t build,
  void* d_temp_storage,
  size_t* temp_storage_bytes,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_keys_out,
  cccl_iterator_t d_values_in,
  cccl_iterator_t d_values_out,
  cccl_op_t decomposer,
  uint64_t num_items,
  int begin_bit,
  int end_bit,
  bool is_overwrite_okay,
  int* selector,
  CUstream stream);

/* Replaces radix_sort.h:126-127. The payload is already a linked cubin, so this only
 * validates its arguments and returns CUDA_ERROR_INVALID_VALUE for an LTO-IR request. */
CCCL_C_API CUresult cccl_device_radix_sort_link_ltoir(
  cccl_device_radix_sort_build_result_t* build, const void** input_blobs, const size_t* input_sizes, size_t num_inputs);

/* Replaces radix_sort.h:129-132. The buffer is freed with cccl_serialization_buffer_free;
 * CUlibrary/CUkernel handles are not serialized. */
CCCL_C_API CUresult
cccl_device_radix_sort_serialize(const cccl_device_radix_sort_build_result_t* build, void** out_buf, size_t* out_size);

/* Replaces radix_sort.h:134-141. Handles stay null until cccl_device_radix_sort_load. */
CCCL_C_API CUresult
cccl_device_radix_sort_deserialize(cccl_device_radix_sort_build_result_t* build, const void* buf, size_t size);

/* Replaces radix_sort.h:143 (radix_sort.cu:730-770). */
CCCL_C_API CUresult cccl_device_radix_sort_cleanup(cccl_device_radix_sort_build_result_t* bld_ptr);

CCCL_C_EXTERN_C_END
