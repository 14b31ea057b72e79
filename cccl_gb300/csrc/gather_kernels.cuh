// Values of any width: a sort whose kernels do not carry the caller's value width moves
// 32-bit indices instead, and these kernels lay the indices down and then gather the values
// by them (value_gather.cpp). Included by the radix and segmented images.
#pragma once

#include <cstdint>

#include "sort_params.h"

namespace gb300
{

__device__ __forceinline__ void values_iota_body(const ValuesIotaParams& p)
{
  const unsigned long long stride = (unsigned long long) gridDim.x * blockDim.x;
  for (unsigned long long i = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; i < p.n; i += stride)
  {
    p.out[i] = uint32_t(i);
  }
}

// dst[i] = src[idx[i]] for every i with idx[i] != VALUES_SKIP, in words of `word` bytes
// (width is a multiple of word; both buffers are word-aligned).
template <class W>
__device__ __forceinline__ void values_gather_words(const ValuesGatherParams& p)
{
  const uint32_t words            = p.width / uint32_t(sizeof(W));
  const W* src                    = static_cast<const W*>(p.src);
  W* dst                          = static_cast<W*>(p.dst);
  const unsigned long long stride = (unsigned long long) gridDim.x * blockDim.x;
  for (unsigned long long i = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; i < p.n; i += stride)
  {
    const uint32_t j = p.idx[i];
    if (j != VALUES_SKIP)
    {
      const W* s = src + (unsigned long long) j * words;
      W* d       = dst + i * words;
      for (uint32_t w = 0; w < words; ++w)
      {
        d[w] = s[w];
      }
    }
  }
}

__device__ __forceinline__ void values_gather_body(const ValuesGatherParams& p)
{
  switch (p.word)
  {
    case 16: values_gather_words<uint4>(p); break;
    case 8: values_gather_words<unsigned long long>(p); break;
    case 4: values_gather_words<uint32_t>(p); break;
    case 2: values_gather_words<uint16_t>(p); break;
    default: values_gather_words<uint8_t>(p); break;
  }
}

} // namespace gb300

extern "C" __global__ void __launch_bounds__(256) gb300_values_iota(const gb300::ValuesIotaParams p)
{
  gb300::values_iota_body(p);
}

extern "C" __global__ void __launch_bounds__(256) gb300_values_gather(const gb300::ValuesGatherParams p)
{
  gb300::values_gather_body(p);
}
