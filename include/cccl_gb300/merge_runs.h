/* Stable merge of sorted runs, the last step of a sort across GPUs.
 *
 * After the exchange of a sort over several GPUs (cccl_gb300.distributed_sort), every rank
 * holds one run from every rank, each sorted, laid out back to back in rank order. The
 * reference merges such runs k ways (cudax/include/cuda/experimental/__multi_gpu/algorithm/
 * sort/hss/merge_k_way.h, a C++ template with no C entry point); this entry point merges them
 * pairwise on the GPU, ceil(log2(num_runs)) rounds of stable two-way merges, each round one
 * read and one write of the items.
 *
 * `build` is a radix-sort build (cccl_device_radix_sort_build) for the keys' and values'
 * types and the order the runs are sorted in; the merge uses its kernels and its order
 * (radix order: -0.0 equal to +0.0, NaNs by their bits). Run r occupies items
 * [run_offsets[r], run_offsets[r + 1]) of d_keys_in (and d_values_in), run_offsets being a
 * host array of num_runs + 1 non-decreasing offsets starting at 0. The result, all items in
 * sorted order with equal keys in run order (and within a run in input order), goes to
 * d_keys_out / d_values_out, which must not overlap the inputs. Temporary storage: one size
 * query with d_temp_storage == NULL, as for the sort. Values of the widths the radix sort
 * carries directly (1, 2, 4, 8, 16 bytes) are taken; other widths return
 * CUDA_ERROR_NOT_SUPPORTED.
 */
#pragma once

#include <cuda.h>
#include <stddef.h>
#include <stdint.h>

#include <cccl/c/radix_sort.h>

#if !defined(CCCL_GB300_API)
#  if defined(_WIN32)
#    define CCCL_GB300_API __declspec(dllexport)
#  else
#    define CCCL_GB300_API __attribute__((__visibility__("default")))
#  endif
#endif

CCCL_C_EXTERN_C_BEGIN

CCCL_GB300_API CUresult cccl_gb300_merge_sorted_runs(
  cccl_device_radix_sort_build_result_t build,
  void* d_temp_storage,
  size_t* temp_storage_bytes,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_keys_out,
  cccl_iterator_t d_values_in,
  cccl_iterator_t d_values_out,
  const uint64_t* run_offsets,
  int num_runs,
  CUstream stream);

CCCL_C_EXTERN_C_END
