// Values of any width (the reference's custom value types): a sort whose kernels do not
// carry the caller's value width sorts 32-bit indices instead and gathers the values by them.
#pragma once

#include <cuda.h>

#include <cstddef>
#include <cstdint>
#include <functional>

namespace gb300
{

// Runs (or sizes) a sort with index values in place of the caller's values.
//   inner(values[2], temp, temp_bytes, selector) runs or sizes the sort with the given value
//   buffers (index arrays) and the temp storage that remains;
//   segmented: the sort leaves positions outside every segment untouched, so they stay
//   untouched in the caller's values too.
// Temp layout: [inner temp][indices 0][indices 1], each 256-byte aligned.
void sort_with_gathered_values(CUlibrary library,
                               uint32_t value_bytes,
                               void* const values[2],
                               uint64_t num_items,
                               bool overwrite,
                               bool segmented,
                               void* d_temp_storage,
                               size_t* temp_storage_bytes,
                               CUstream stream,
                               const std::function<void(void* const idx[2], void* temp, size_t* temp_bytes, int* sel)>& inner,
                               int* selector);

} // namespace gb300
