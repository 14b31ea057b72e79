// Segment offsets given as iterators instead of pointers.
//
// The reference compiles an iterator's advance and dereference operations into its kernels
// with NVRTC (c/parallel/src/segmented_sort.cu:910-917 wraps the offsets in iterators;
// c/parallel/src/jit_templates/templates/input_iterator.h gives the calling convention:
// `extern "C" __device__ void advance(void* state, const void* diff)` with a size_t
// difference, `extern "C" __device__ void dereference(const void* state, void* result)`).
// The sort kernels here are precompiled, so at build time one small kernel per iterator is
// compiled instead (NVRTC to LTO-IR, linked with the operations by nvJitLink): it evaluates
// the iterator at 0 .. n-1 into an offset array in the temporary storage, which the sort then
// reads like a pointer. NVRTC and nvJitLink are opened with dlopen the first time an
// iterator is compiled.
#pragma once

#include <cuda.h>

#include <cstddef>
#include <cstdint>

#include <cccl/c/types.h>

namespace gb300
{

struct OffsetIteratorKernel
{
  void* cubin;       // compiled at build time (malloc'd)
  size_t cubin_size;
  CUlibrary library; // loaded by load_offset_iterator
  CUkernel kernel;
  uint64_t state_size;
  uint64_t state_alignment;
  uint64_t value_size; // 4 or 8: the offset array's element size
};

// Largest iterator state passed by value to the evaluation kernel.
constexpr size_t MAX_OFFSET_STATE_BYTES = 1024;

// Compiles the evaluation kernel of `it` (a CCCL_ITERATOR over a 4- or 8-byte integer type)
// for sm_<cc_major><cc_minor>a. An operation of `it` given by name without code takes the code
// of `sibling`'s operation of that name (may be null). Throws cuda_error.
void compile_offset_iterator(
  const cccl_iterator_t& it, const cccl_iterator_t* sibling, int cc_major, int cc_minor, OffsetIteratorKernel& out);
void load_offset_iterator(OffsetIteratorKernel& k);
void free_offset_iterator(OffsetIteratorKernel& k);

// out[i] = *(it + i) (value_size bytes each), i < n, on `stream`. `it.state` holds the
// iterator's state bytes on the host (copied into the launch's parameters).
void evaluate_offset_iterator(
  const OffsetIteratorKernel& k, const cccl_iterator_t& it, uint64_t n, void* out, CUstream stream);

} // namespace gb300
