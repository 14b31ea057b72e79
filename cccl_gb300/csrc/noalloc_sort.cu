// Allocation-free radix sort of u32 keys (+ optional u32 values): the temporary storage
// of the plain sort (control block, digit bases, look-back rows, ping-pong buffers) lives
// in one file-scope device array. See include/cccl_gb300/radix_sort_noalloc.h.
//
// The kernels are the plain path's (init, all-pass histogram, CTA-per-tile onesweep pass,
// single tile), instantiated here so the runtime API can launch them next to the array.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <mutex>

#include <cccl_gb300/radix_sort_noalloc.h>

#include "radix_kernels.cuh"
#include "sort_policy.h"

namespace
{
using namespace gb300;

constexpr int KB                = 4;
constexpr uint32_t MAX_ITEMS    = CCCL_GB300_NOALLOC_MAX_ITEMS;
constexpr int MAX_SORT_PASSES   = 4; // 32-bit keys
// smallest tile of the two pass kernels below (keys only, pairs): it sizes the look-back rows
constexpr int TILE_MIN          = ONESWEEP_TPB * std::min(onesweep_items(KB, 0), onesweep_items(KB, 4));
static_assert(TILE_MIN >= ONESWEEP_TPB, "a pass tile holds at least one key per thread");
constexpr uint32_t MAX_TILES    = (MAX_ITEMS + TILE_MIN - 1) / TILE_MIN;
constexpr size_t CTRL_BYTES     = (sizeof(SortControl) + 4 * MAX_SORT_PASSES + 255) / 256 * 256;
constexpr size_t BINS_BYTES     = 8 * 256 * MAX_SORT_PASSES;
constexpr size_t LOOKBACK_WORDS = size_t(MAX_TILES) * 256;
constexpr size_t LOOKBACK_BYTES = 2 * 4 * LOOKBACK_WORDS;
constexpr size_t TMP_BYTES      = size_t(MAX_ITEMS) * 4;
constexpr size_t SCRATCH_BYTES  = CTRL_BYTES + BINS_BYTES + LOOKBACK_BYTES + 2 * TMP_BYTES;
// The size the header documents (8,763,648 bytes = 8.36 MiB); a change of the tile table
// that moves it must move the documentation with it.
static_assert(SCRATCH_BYTES == CCCL_GB300_NOALLOC_SCRATCH_BYTES, "documented scratch size");
static_assert(offsetof(SortControl, status) == 0, "the status word is word 0 of the scratch array");

// The scratch space. In host code this name is only a stand-in for the symbol: the device
// address comes from cudaGetSymbolAddress (scratch_on_current_device below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

__global__ void __launch_bounds__(256) na_init(const InitParams p)
{
  init_body(p);
}
__global__ void __launch_bounds__(HISTOGRAM_TPB) na_histogram(const HistogramParams p)
{
  histogram_body<KB, false, HISTOGRAM_TPB>(p);
}
__global__ void __launch_bounds__(ONESWEEP_TPB) na_onesweep_keys(const OnesweepParams p)
{
  onesweep_body<KB, 0, false, ONESWEEP_TPB, onesweep_items(KB, 0), true>(p);
}
__global__ void __launch_bounds__(ONESWEEP_TPB) na_onesweep_pairs(const OnesweepParams p)
{
  onesweep_body<KB, 4, false, ONESWEEP_TPB, onesweep_items(KB, 4), true>(p);
}
__global__ void __launch_bounds__(SINGLE_TILE_TPB) na_single_tile_keys(const SingleTileParams p)
{
  single_tile_body<KB, 0, false, SINGLE_TILE_TPB, SINGLE_TILE_ITEMS>(p);
}
__global__ void __launch_bounds__(SINGLE_TILE_TPB) na_single_tile_pairs(const SingleTileParams p)
{
  single_tile_body<KB, 4, false, SINGLE_TILE_TPB, SINGLE_TILE_ITEMS>(p);
}

// Set-up, once per CUDA context (in the usual case, the runtime's primary context of each
// device, so once per device): with that context current, the array's device address from
// cudaGetSymbolAddress, and the shared-memory attributes of the kernels that need more than
// 48 KB. It is keyed on the context's unique id, not on the device number, so a caller that
// makes another context current, or a context created after cudaDeviceReset, gets that
// context's own copy of the array and never a stale address.
constexpr int MAX_CONTEXTS = 64;
struct ContextScratch
{
  unsigned long long ctx_id;
  unsigned char* ptr;
};
std::mutex g_setup_mutex;
ContextScratch g_scratch[MAX_CONTEXTS] = {};
int g_scratch_used                     = 0;

cudaError_t setup_current_context(unsigned char** out)
{
  void* ptr = nullptr;
  if (cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch); e != cudaSuccess)
  {
    return e;
  }
  const struct
  {
    const void* fn;
    size_t smem;
  } attrs[] = {{(const void*) na_onesweep_keys, onesweep_smem_bytes(KB, 0)},
               {(const void*) na_onesweep_pairs, onesweep_smem_bytes(KB, 4)},
               {(const void*) na_single_tile_keys, single_tile_smem_bytes(KB)},
               {(const void*) na_single_tile_pairs, single_tile_smem_bytes(KB)}};
  for (const auto& a : attrs)
  {
    if (cudaError_t e = cudaFuncSetAttribute(a.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(a.smem));
        e != cudaSuccess)
    {
      return e;
    }
  }
  *out = static_cast<unsigned char*>(ptr);
  return cudaSuccess;
}

cudaError_t scratch_on_current_context(unsigned char** out)
{
  CUcontext ctx = nullptr;
  if (cuCtxGetCurrent(&ctx) != CUDA_SUCCESS)
  {
    return cudaErrorInitializationError;
  }
  if (ctx == nullptr)
  {
    // no context yet: the runtime binds the current device's primary context on this call
    if (cudaError_t e = setup_current_context(out); e != cudaSuccess)
    {
      return e;
    }
    if (cuCtxGetCurrent(&ctx) != CUDA_SUCCESS || ctx == nullptr)
    {
      return cudaErrorInitializationError;
    }
  }
  unsigned long long id = 0;
  if (cuCtxGetId(ctx, &id) != CUDA_SUCCESS)
  {
    return cudaErrorInitializationError;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  for (int i = 0; i < g_scratch_used; ++i)
  {
    if (g_scratch[i].ctx_id == id)
    {
      *out = g_scratch[i].ptr;
      return cudaSuccess;
    }
  }
  if (cudaError_t e = setup_current_context(out); e != cudaSuccess)
  {
    return e;
  }
  if (g_scratch_used < MAX_CONTEXTS) // beyond that, every call repeats the set-up (still correct)
  {
    g_scratch[g_scratch_used++] = ContextScratch{id, *out};
  }
  return cudaSuccess;
}

CUresult fail(const char* what, cudaError_t e)
{
  std::printf("\nERROR in cccl_gb300_radix_sort_u32_noalloc(): %s: %s\n", what, cudaGetErrorString(e));
  return e == cudaErrorInvalidValue ? CUDA_ERROR_INVALID_VALUE : CUDA_ERROR_UNKNOWN;
}

KeyCodec unsigned_codec(bool descending)
{
  const unsigned long long all = 0xffffffffull;
  KeyCodec c{};
  c.fwd_pos = c.fwd_neg = c.inv_set = c.inv_clr = descending ? all : 0ull;
  return c;
}

} // namespace

extern "C" CCCL_GB300_API CUresult cccl_gb300_radix_sort_u32_noalloc(
  const uint32_t* d_keys_in,
  uint32_t* d_keys_out,
  const uint32_t* d_values_in,
  uint32_t* d_values_out,
  uint64_t num_items,
  int begin_bit,
  int end_bit,
  bool descending,
  CUstream stream_handle)
{
  if (num_items > MAX_ITEMS)
  {
    std::printf("\nERROR in cccl_gb300_radix_sort_u32_noalloc(): num_items = %llu exceeds the maximum of %u "
                "(the size of the built-in scratch space)\n",
                (unsigned long long) num_items,
                MAX_ITEMS);
    return CUDA_ERROR_INVALID_VALUE;
  }
  if (begin_bit < 0 || end_bit > 32 || begin_bit > end_bit
      || (num_items > 0
          && (d_keys_in == nullptr || d_keys_out == nullptr || ((d_values_in == nullptr) != (d_values_out == nullptr)))))
  {
    std::printf("\nERROR in cccl_gb300_radix_sort_u32_noalloc(): invalid arguments\n");
    return CUDA_ERROR_INVALID_VALUE;
  }
  unsigned char* scratch = nullptr;
  if (cudaError_t e = scratch_on_current_context(&scratch); e != cudaSuccess)
  {
    return fail("setup", e);
  }
  cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_handle);
  auto* ctrl          = reinterpret_cast<SortControl*>(scratch);
  // launches are checked one at a time, so an error names the kernel that failed
  auto launched = [](const char* kernel) {
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CUDA_SUCCESS : fail(kernel, e);
  };
  if (num_items == 0 || begin_bit == end_bit || num_items <= cub_single_tile_limit(KB, d_values_in ? 4 : 0))
  {
    // these paths wait on nothing: the status word must still read "no error" afterwards
    if (cudaError_t e = cudaMemsetAsync(&ctrl->status, 0, sizeof(uint32_t), stream); e != cudaSuccess)
    {
      return fail("status reset", e);
    }
  }
  if (num_items == 0)
  {
    return CUDA_SUCCESS;
  }
  const bool pairs      = d_values_in != nullptr;
  const uint64_t n      = num_items;
  const KeyCodec codec  = unsigned_codec(descending);
  if (begin_bit == end_bit)
  {
    cudaError_t e = cudaMemcpyAsync(d_keys_out, d_keys_in, n * 4, cudaMemcpyDeviceToDevice, stream);
    if (e == cudaSuccess && pairs)
    {
      e = cudaMemcpyAsync(d_values_out, d_values_in, n * 4, cudaMemcpyDeviceToDevice, stream);
    }
    return e == cudaSuccess ? CUDA_SUCCESS : fail("copy", e);
  }
  if (n <= cub_single_tile_limit(KB, pairs ? 4 : 0))
  {
    SingleTileParams p{};
    p.keys_in    = d_keys_in;
    p.keys_out   = d_keys_out;
    p.values_in  = d_values_in;
    p.values_out = d_values_out;
    p.num_items  = uint32_t(n);
    p.begin_bit  = begin_bit;
    p.end_bit    = end_bit;
    p.codec      = codec;
    if (pairs)
    {
      na_single_tile_pairs<<<1, SINGLE_TILE_TPB, single_tile_smem_bytes(KB), stream>>>(p);
      return launched("launch of the single-tile pairs kernel");
    }
    na_single_tile_keys<<<1, SINGLE_TILE_TPB, single_tile_smem_bytes(KB), stream>>>(p);
    return launched("launch of the single-tile keys kernel");
  }

  const int passes    = (end_bit - begin_bit + RADIX_BITS - 1) / RADIX_BITS;
  const uint64_t tile = uint64_t(ONESWEEP_TPB) * onesweep_items(KB, pairs ? 4 : 0);
  const uint32_t tiles = uint32_t((n + tile - 1) / tile);

  auto* tile_ctrs = reinterpret_cast<uint32_t*>(scratch + sizeof(SortControl));
  auto* bins      = reinterpret_cast<unsigned long long*>(scratch + CTRL_BYTES);
  uint32_t* lb[2] = {reinterpret_cast<uint32_t*>(scratch + CTRL_BYTES + BINS_BYTES),
                     reinterpret_cast<uint32_t*>(scratch + CTRL_BYTES + BINS_BYTES) + LOOKBACK_WORDS};
  auto* keys_tmp  = reinterpret_cast<uint32_t*>(scratch + CTRL_BYTES + BINS_BYTES + LOOKBACK_BYTES);
  auto* vals_tmp  = reinterpret_cast<uint32_t*>(scratch + CTRL_BYTES + BINS_BYTES + LOOKBACK_BYTES + TMP_BYTES);

  {
    InitParams p{};
    p.words     = reinterpret_cast<uint32_t*>(ctrl);
    p.num_words = CTRL_BYTES / 4; // counters and the status word restart from zero on every call
    na_init<<<unsigned((p.num_words + 255) / 256), 256, 0, stream>>>(p);
    if (const CUresult r = launched("launch of the init kernel"); r != CUDA_SUCCESS)
    {
      return r;
    }
  }
  {
    HistogramParams p{};
    p.keys           = d_keys_in;
    p.num_items      = n;
    p.codec          = codec;
    p.begin_bit      = begin_bit;
    p.end_bit        = end_bit;
    p.num_passes     = passes;
    p.num_portions   = 1;
    p.ctrl           = ctrl;
    p.bins           = bins;
    p.lookback_clear = lb[0];
    p.lookback_words = size_t(tiles) * 256;
    const unsigned grid = unsigned(std::min<uint64_t>(512, (n + HISTOGRAM_TPB * 4 - 1) / (HISTOGRAM_TPB * 4)));
    na_histogram<<<grid, HISTOGRAM_TPB, 0, stream>>>(p);
    if (const CUresult r = launched("launch of the histogram kernel"); r != CUDA_SUCCESS)
    {
      return r;
    }
  }
  const void* ksrc = d_keys_in;
  const void* vsrc = d_values_in;
  for (int pass = 0; pass < passes; ++pass)
  {
    const bool to_out = ((passes - 1 - pass) % 2) == 0;
    void* kdst        = to_out ? static_cast<void*>(d_keys_out) : static_cast<void*>(keys_tmp);
    void* vdst        = to_out ? static_cast<void*>(d_values_out) : static_cast<void*>(vals_tmp);
    const int bit     = begin_bit + pass * RADIX_BITS;
    OnesweepParams op{};
    op.keys_in         = ksrc;
    op.keys_out        = kdst;
    op.values_in       = pairs ? vsrc : nullptr;
    op.values_out      = pairs ? vdst : nullptr;
    op.portion_begin   = 0;
    op.num_items_total = n;
    op.portion_items   = uint32_t(n);
    op.portion_tiles   = tiles;
    op.tile_row_base   = 0;
    op.lookback        = lb[pass & 1];
    op.lookback_next   = (pass + 1 < passes) ? lb[(pass + 1) & 1] : nullptr;
    op.tile_counter    = tile_ctrs + pass;
    op.bins            = bins + size_t(pass) * 256;
    op.bins_next       = nullptr;
    op.status          = &ctrl->status;
    op.codec           = codec;
    op.current_bit     = bit;
    op.num_bits        = std::min(RADIX_BITS, end_bit - bit);
    op.encode_in       = pass == 0;
    op.decode_out      = pass == passes - 1;
    if (pairs)
    {
      na_onesweep_pairs<<<tiles, ONESWEEP_TPB, onesweep_smem_bytes(KB, 4), stream>>>(op);
    }
    else
    {
      na_onesweep_keys<<<tiles, ONESWEEP_TPB, onesweep_smem_bytes(KB, 0), stream>>>(op);
    }
    if (const CUresult r = launched(pairs ? "launch of the pairs digit pass" : "launch of the keys digit pass");
        r != CUDA_SUCCESS)
    {
      return r;
    }
    ksrc = kdst;
    vsrc = vdst;
  }
  return CUDA_SUCCESS;
}

// The status word of the allocation-free entry point in the current context, for
// cccl_gb300_sort_status (status_abi.cpp). Returns 0 or a cudaError_t.
int gb300_noalloc_status_word(uint32_t** dptr)
{
  unsigned char* scratch = nullptr;
  if (cudaError_t e = scratch_on_current_context(&scratch); e != cudaSuccess)
  {
    return int(e);
  }
  *dptr = &reinterpret_cast<SortControl*>(scratch)->status;
  return 0;
}
