// C ABI of the batched segmented sort (reference: c/parallel/include/cccl/c/segmented_sort.h).
// Entry points are exported now; the run path is filled in with the segmented kernels.
#include <cccl/c/segmented_sort.h>

#include "abi_common.h"

using namespace gb300;

extern "C" {

CCCL_C_API CUresult cccl_device_segmented_sort_compile(
  cccl_device_segmented_sort_build_result_t*,
  cccl_sort_order_t,
  cccl_iterator_t,
  cccl_iterator_t,
  cccl_iterator_t,
  cccl_iterator_t,
  int,
  int,
  const char*,
  const char*,
  const char*,
  const char*,
  cccl_build_config*)
{
  return CUDA_ERROR_NOT_SUPPORTED;
}

CCCL_C_API CUresult cccl_device_segmented_sort_load(cccl_device_segmented_sort_build_result_t*)
{
  return CUDA_ERROR_NOT_SUPPORTED;
}

CCCL_C_API CUresult cccl_device_segmented_sort_build_ex(
  cccl_device_segmented_sort_build_result_t*,
  cccl_sort_order_t,
  cccl_iterator_t,
  cccl_iterator_t,
  cccl_iterator_t,
  cccl_iterator_t,
  int,
  int,
  const char*,
  const char*,
  const char*,
  const char*,
  cccl_build_config*)
{
  return CUDA_ERROR_NOT_SUPPORTED;
}

CCCL_C_API CUresult cccl_device_segmented_sort_build(
  cccl_device_segmented_sort_build_result_t*,
  cccl_sort_order_t,
  cccl_iterator_t,
  cccl_iterator_t,
  cccl_iterator_t,
  cccl_iterator_t,
  int,
  int,
  const char*,
  const char*,
  const char*,
  const char*)
{
  return CUDA_ERROR_NOT_SUPPORTED;
}

CCCL_C_API CUresult cccl_device_segmented_sort(
  cccl_device_segmented_sort_build_result_t,
  void*,
  size_t*,
  cccl_iterator_t,
  cccl_iterator_t,
  cccl_iterator_t,
  cccl_iterator_t,
  uint64_t,
  uint64_t,
  cccl_iterator_t,
  cccl_iterator_t,
  bool,
  int*,
  CUstream)
{
  return CUDA_ERROR_NOT_SUPPORTED;
}

CCCL_C_API CUresult
cccl_device_segmented_sort_link_ltoir(cccl_device_segmented_sort_build_result_t*, const void**, const size_t*, size_t)
{
  return CUDA_ERROR_NOT_SUPPORTED;
}

CCCL_C_API CUresult
cccl_device_segmented_sort_serialize(const cccl_device_segmented_sort_build_result_t*, void**, size_t*)
{
  return CUDA_ERROR_NOT_SUPPORTED;
}

CCCL_C_API CUresult
cccl_device_segmented_sort_deserialize(cccl_device_segmented_sort_build_result_t*, const void*, size_t)
{
  return CUDA_ERROR_NOT_SUPPORTED;
}

CCCL_C_API CUresult cccl_device_segmented_sort_cleanup(cccl_device_segmented_sort_build_result_t*)
{
  return CUDA_SUCCESS;
}

} // extern "C"
