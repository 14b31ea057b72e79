// Sorts whose values are carried as 32-bit indices and gathered afterwards (value_gather.h).
#include "value_gather.h"

#include <algorithm>

#include "abi_common.h"

namespace gb300
{

namespace
{
uint64_t ceil_div(uint64_t a, uint64_t b)
{
  return (a + b - 1) / b;
}

// Largest copy word (16, 8, 4, 2, 1 bytes) dividing the value width and both buffers' addresses.
uint32_t gather_word(uint32_t width, const void* a, const void* b)
{
  const uintptr_t bits = uintptr_t(width) | reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b);
  for (uint32_t w = 16; w > 1; w >>= 1)
  {
    if ((bits & (w - 1)) == 0)
    {
      return w;
    }
  }
  return 1;
}
} // namespace

void sort_with_gathered_values(CUlibrary library,
                               uint32_t value_bytes,
                               void* const values[2],
                               uint64_t n,
                               bool overwrite,
                               bool segmented,
                               void* d_temp_storage,
                               size_t* temp_storage_bytes,
                               CUstream stream,
                               const std::function<void(void* const idx[2], void* temp, size_t* temp_bytes, int* sel)>& inner,
                               int* selector)
{
  if (n > uint64_t(VALUES_SKIP))
  {
    throw cuda_error(CUDA_ERROR_NOT_SUPPORTED, "values of this width are sorted as 32-bit indices: at most 2^32 - 1 items");
  }
  const size_t idx_bytes = align_up(size_t(n) * 4, 256);
  if (d_temp_storage == nullptr)
  {
    // stand-in index buffers for the size query: 256-byte aligned, never dereferenced
    void* const fake[2] = {reinterpret_cast<void*>(uintptr_t(256)), reinterpret_cast<void*>(uintptr_t(512))};
    size_t inner_bytes  = 0;
    int sel             = 0;
    inner(fake, nullptr, &inner_bytes, &sel);
    *temp_storage_bytes = align_up(inner_bytes, 256) + 2 * idx_bytes;
    return;
  }
  if (values[0] == nullptr || values[1] == nullptr)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "value buffers are null");
  }
  // the inner sort's own size, for the same buffers
  void* const fake[2] = {reinterpret_cast<void*>(uintptr_t(256)), reinterpret_cast<void*>(uintptr_t(512))};
  size_t inner_bytes  = 0;
  {
    int sel = 0;
    inner(fake, nullptr, &inner_bytes, &sel);
  }
  const size_t inner_region = align_up(inner_bytes, 256);
  if (*temp_storage_bytes < inner_region + 2 * idx_bytes)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "temp storage is smaller than the size query returned");
  }
  auto* base      = static_cast<unsigned char*>(d_temp_storage);
  void* idx[2]    = {base + inner_region, base + inner_region + idx_bytes};
  CUkernel iota   = nullptr;
  CUkernel gather = nullptr;
  check(cuLibraryGetKernel(&iota, library, "gb300_values_iota"), "cuLibraryGetKernel(gb300_values_iota)");
  check(cuLibraryGetKernel(&gather, library, "gb300_values_gather"), "cuLibraryGetKernel(gb300_values_gather)");
  const unsigned grid = unsigned(std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(n, 256), uint64_t(sm_count()) * 16)));
  if (n > 0)
  {
    ValuesIotaParams ip{static_cast<uint32_t*>(idx[0]), n};
    launch("values_iota", iota, grid, 256, 0, stream, ip);
    // positions the sort does not write (outside every segment) are skipped by the gather;
    // the inner sort writes every other position of the buffer it leaves its result in
    check(cuMemsetD32Async(CUdeviceptr(idx[1]), VALUES_SKIP, size_t(n), stream), "cuMemsetD32Async(indices)");
  }
  size_t rest = inner_bytes;
  int sel     = 0;
  inner(idx, d_temp_storage, &rest, &sel);
  *selector = sel;
  if (n == 0)
  {
    return;
  }
  // the result's indices: in indices[sel] with a DoubleBuffer, else in indices[1]
  const void* res = overwrite ? idx[sel] : idx[1];
  ValuesGatherParams gp{};
  gp.src   = values[0];
  gp.dst   = values[1];
  gp.idx   = static_cast<const uint32_t*>(res);
  gp.n     = n;
  gp.width = value_bytes;
  gp.word  = gather_word(value_bytes, values[0], values[1]);
  launch("values_gather", gather, grid, 256, 0, stream, gp);
  if (overwrite && sel == 0)
  {
    // the result belongs in the current buffer: gathered into the alternate one, copied back
    check(cuMemcpyAsync(CUdeviceptr(values[0]), CUdeviceptr(values[1]), size_t(n) * value_bytes, stream),
          "cuMemcpyAsync(values)");
  }
  (void) segmented;
}

} // namespace gb300
