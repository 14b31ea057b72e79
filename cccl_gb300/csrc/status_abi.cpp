// Status query of a finished sort and the test hook of the bounded waits
// (include/cccl_gb300/sort_status.h).
#include <cccl_gb300/sort_status.h>

#include "abi_common.h"

// Device address of the allocation-free entry point's status word in the current context
// (noalloc_sort.cu); 0 on success, else a cudaError_t.
int gb300_noalloc_status_word(uint32_t** dptr);

namespace
{

CUresult status_result(uint32_t bits)
{
  if (bits & gb300::STATUS_LOOKBACK_TIMEOUT)
  {
    return CUDA_ERROR_LAUNCH_TIMEOUT;
  }
  if (bits & (gb300::STATUS_BAD_SEGMENT | gb300::STATUS_SEG_CAPACITY))
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  return CUDA_SUCCESS;
}

} // namespace

static_assert(CCCL_GB300_STATUS_WAIT_TIMEOUT == gb300::STATUS_LOOKBACK_TIMEOUT, "status bits");
static_assert(CCCL_GB300_STATUS_BAD_SEGMENT == gb300::STATUS_BAD_SEGMENT, "status bits");
static_assert(CCCL_GB300_STATUS_SEG_CAPACITY == gb300::STATUS_SEG_CAPACITY, "status bits");

extern "C" CCCL_GB300_API CUresult
cccl_gb300_sort_status(const void* d_temp_storage, size_t temp_storage_bytes, CUstream stream, uint32_t* status_bits)
{
  using namespace gb300;
  try
  {
    context_guard ctx;
    if (status_bits != nullptr)
    {
      *status_bits = 0;
    }
    check(cuStreamSynchronize(stream), "cuStreamSynchronize");
    CUdeviceptr word = 0;
    if (d_temp_storage == nullptr)
    {
      uint32_t* p = nullptr;
      if (const int e = gb300_noalloc_status_word(&p); e != 0)
      {
        std::printf("\nERROR in cccl_gb300_sort_status(): the allocation-free entry point's scratch array is "
                    "not available (cudaError %d)\n",
                    e);
        return CUDA_ERROR_UNKNOWN;
      }
      word = CUdeviceptr(p);
    }
    else if (temp_storage_bytes >= 4)
    {
      word = CUdeviceptr(d_temp_storage);
    }
    else
    {
      return CUDA_SUCCESS; // calls that need no temporary storage wait on nothing
    }
    uint32_t bits = 0;
    check(cuMemcpyDtoH(&bits, word, sizeof(bits)), "cuMemcpyDtoH(status)");
    if (bits != 0u)
    {
      check(cuMemsetD32(word, 0u, 1), "cuMemsetD32(status)");
    }
    if (status_bits != nullptr)
    {
      *status_bits = bits;
    }
    return status_result(bits);
  }
  catch (const cuda_error& e)
  {
    std::printf("\nERROR in cccl_gb300_sort_status(): %s\n", e.what());
    return e.code;
  }
}

extern "C" CCCL_GB300_API CUresult
cccl_gb300_testing_set_wait_fault(CUlibrary radix_library, uint32_t skip_tile, uint64_t wait_limit_ns)
{
  using namespace gb300;
  if (radix_library == nullptr || wait_limit_ns == 0)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  try
  {
    context_guard ctx;
    CUdeviceptr p = 0;
    size_t bytes  = 0;
    check(cuLibraryGetGlobal(&p, &bytes, radix_library, "gb300_fault_skip_tile"), "cuLibraryGetGlobal(skip tile)");
    if (bytes != sizeof(skip_tile))
    {
      return CUDA_ERROR_INVALID_VALUE;
    }
    check(cuMemcpyHtoD(p, &skip_tile, sizeof(skip_tile)), "cuMemcpyHtoD(skip tile)");
    check(cuLibraryGetGlobal(&p, &bytes, radix_library, "gb300_wait_limit_ns"), "cuLibraryGetGlobal(wait limit)");
    if (bytes != sizeof(wait_limit_ns))
    {
      return CUDA_ERROR_INVALID_VALUE;
    }
    check(cuMemcpyHtoD(p, &wait_limit_ns, sizeof(wait_limit_ns)), "cuMemcpyHtoD(wait limit)");
    return CUDA_SUCCESS;
  }
  catch (const cuda_error& e)
  {
    std::printf("\nERROR in cccl_gb300_testing_set_wait_fault(): %s\n", e.what());
    return e.code;
  }
}
