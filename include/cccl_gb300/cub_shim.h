// C++ entry points with the signatures of cub::DeviceRadixSort, cub::DeviceSegmentedSort and
// cub::DeviceSegmentedRadixSort, running on this library's sm_103a kernels through its C ABI
// (cccl_device_radix_sort*, cccl_device_segmented_sort*, cccl_gb300_segmented_radix_sort).
// Header-only; link the program with libccclsort.so.
//
// Mirrored signatures (reference files, cub/cub/device/):
//   DeviceRadixSort (device_radix_sort.cuh): SortPairs :412 / DoubleBuffer :1127,
//     SortPairsDescending :1776 / :2295, SortKeys :3034 / :3644, SortKeysDescending :4211 / :4669.
//     Pointer overloads sort out of place (is_overwrite_okay = false); DoubleBuffer overloads
//     may use both buffers and leave the result in d_keys.Current(), as CUB does.
//   DeviceSegmentedSort (device_segmented_sort.cuh): SortKeys :361, SortPairs :2468-2494 and
//     the Descending, Stable and DoubleBuffer forms, with begin/end offsets given as
//     pointers to 32- or 64-bit integers (iterators other than pointers are not taken).
//   DeviceSegmentedRadixSort (device_segmented_radix_sort.cuh): SortPairs :234 / :417,
//     SortPairsDescending :887 / :1073, SortKeys :1531 / :1702 and SortKeysDescending, with
//     begin_bit / end_bit; values of 4 or 8 bytes.
// Differences: the functions live in namespace cccl_gb300::cub (alias it to cub to switch
// a program over); errors come back as cudaError_t (cudaErrorInvalidValue,
// cudaErrorNotSupported, cudaErrorUnknown); decomposers and custom key types are not taken.
// Builds (one per key type, value width and order) are made on first use and kept for the
// life of the process.
#pragma once

#ifndef CCCL_C_EXPERIMENTAL
#  define CCCL_C_EXPERIMENTAL 1
#endif

#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime_api.h>

#include <cccl/c/radix_sort.h>
#include <cccl/c/segmented_sort.h>
#include <cccl_gb300/segmented_radix_sort.h>

#include <cstddef>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <type_traits>

namespace cccl_gb300
{
namespace cub
{

// Same members and meaning as cub::DoubleBuffer (cub/cub/util_type.cuh).
template <typename T>
struct DoubleBuffer
{
  T* d_buffers[2];
  int selector;

  DoubleBuffer()
      : d_buffers{nullptr, nullptr}
      , selector(0)
  {}
  DoubleBuffer(T* d_current, T* d_alternate)
      : d_buffers{d_current, d_alternate}
      , selector(0)
  {}
  T* Current()
  {
    return d_buffers[selector];
  }
  T* Alternate()
  {
    return d_buffers[selector ^ 1];
  }
};

namespace detail
{

template <typename T, typename = void>
struct type_of
{
  static constexpr bool supported = false;
};
#define CCCL_GB300_TYPE(T, E)                       \
  template <>                                       \
  struct type_of<T>                                 \
  {                                                 \
    static constexpr bool supported   = true;       \
    static constexpr cccl_type_enum value = E;      \
  };
CCCL_GB300_TYPE(std::int8_t, CCCL_INT8)
CCCL_GB300_TYPE(std::int16_t, CCCL_INT16)
CCCL_GB300_TYPE(std::int32_t, CCCL_INT32)
CCCL_GB300_TYPE(std::int64_t, CCCL_INT64)
CCCL_GB300_TYPE(std::uint8_t, CCCL_UINT8)
CCCL_GB300_TYPE(std::uint16_t, CCCL_UINT16)
CCCL_GB300_TYPE(std::uint32_t, CCCL_UINT32)
CCCL_GB300_TYPE(std::uint64_t, CCCL_UINT64)
CCCL_GB300_TYPE(float, CCCL_FLOAT32)
CCCL_GB300_TYPE(double, CCCL_FLOAT64)
CCCL_GB300_TYPE(__half, CCCL_FLOAT16)
CCCL_GB300_TYPE(bool, CCCL_BOOLEAN)
#undef CCCL_GB300_TYPE
// long long / unsigned long long where they differ from the fixed-width types
template <typename T>
struct type_of<T,
               std::enable_if_t<std::is_integral_v<T> && !std::is_same_v<T, bool>
                                && !std::is_same_v<T, std::int8_t> && !std::is_same_v<T, std::int16_t>
                                && !std::is_same_v<T, std::int32_t> && !std::is_same_v<T, std::int64_t>
                                && !std::is_same_v<T, std::uint8_t> && !std::is_same_v<T, std::uint16_t>
                                && !std::is_same_v<T, std::uint32_t> && !std::is_same_v<T, std::uint64_t>>>
{
  static constexpr bool supported = sizeof(T) == 4 || sizeof(T) == 8;
  static constexpr cccl_type_enum value =
    std::is_signed_v<T> ? (sizeof(T) == 8 ? CCCL_INT64 : CCCL_INT32) : (sizeof(T) == 8 ? CCCL_UINT64 : CCCL_UINT32);
};

inline cudaError_t to_cuda_error(CUresult r)
{
  switch (r)
  {
    case CUDA_SUCCESS:
      return cudaSuccess;
    case CUDA_ERROR_INVALID_VALUE:
      return cudaErrorInvalidValue;
    case CUDA_ERROR_NOT_SUPPORTED:
      return cudaErrorNotSupported;
    case CUDA_ERROR_OUT_OF_MEMORY:
      return cudaErrorMemoryAllocation;
    default:
      return cudaErrorUnknown;
  }
}

inline cccl_iterator_t pointer_it(const void* p, cccl_type_enum t, size_t size)
{
  cccl_iterator_t it{};
  it.size       = size;
  it.alignment  = size;
  it.type       = CCCL_POINTER;
  it.state      = const_cast<void*>(p);
  it.value_type = cccl_type_info{size, size, t};
  return it;
}

// keys-only: a pointer iterator with no state (c/parallel/src/radix_sort.cu:240)
inline cccl_iterator_t no_values()
{
  return pointer_it(nullptr, CCCL_STORAGE, 4);
}

inline int current_cc(int& major, int& minor)
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess
      || cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess)
  {
    return -1;
  }
  return 0;
}

// One build per (key type, value width, order), made on first use.
struct radix_builds
{
  std::mutex m;
  std::map<std::tuple<int, size_t, int>, std::unique_ptr<cccl_device_radix_sort_build_result_t>> map;
  ~radix_builds()
  {
    // the driver may already be shut down at process exit: the builds are left to it
    for (auto& kv : map)
    {
      kv.second.release();
    }
  }
};

inline CUresult radix_build(cccl_type_enum kt, size_t ks, size_t vs, bool desc, cccl_device_radix_sort_build_result_t** out)
{
  static radix_builds b;
  std::lock_guard<std::mutex> lock(b.m);
  const auto key = std::make_tuple(int(kt), vs, int(desc));
  auto it        = b.map.find(key);
  if (it == b.map.end())
  {
    int major = 0, minor = 0;
    if (current_cc(major, minor) != 0)
    {
      return CUDA_ERROR_INVALID_CONTEXT;
    }
    auto r               = std::make_unique<cccl_device_radix_sort_build_result_t>();
    cccl_iterator_t keys = pointer_it(nullptr, kt, ks);
    cccl_iterator_t vals = vs ? pointer_it(reinterpret_cast<void*>(16), CCCL_STORAGE, vs) : no_values();
    vals.value_type.type = vs == 4 ? CCCL_UINT32 : vs == 8 ? CCCL_UINT64 : vals.value_type.type;
    cccl_op_t op{};
    const CUresult st = cccl_device_radix_sort_build(
      r.get(), desc ? CCCL_DESCENDING : CCCL_ASCENDING, keys, vals, op, "", major, minor, nullptr, nullptr, nullptr, nullptr);
    if (st != CUDA_SUCCESS)
    {
      return st;
    }
    it = b.map.emplace(key, std::move(r)).first;
  }
  *out = it->second.get();
  return CUDA_SUCCESS;
}

template <typename KeyT, typename ValueT>
cudaError_t radix_sort(bool desc,
                       void* d_temp_storage,
                       size_t& temp_storage_bytes,
                       const KeyT* keys_in,
                       KeyT* keys_out,
                       const ValueT* values_in,
                       ValueT* values_out,
                       std::uint64_t num_items,
                       int begin_bit,
                       int end_bit,
                       bool overwrite,
                       int* selector,
                       cudaStream_t stream)
{
  static_assert(type_of<KeyT>::supported, "key type not supported (custom key types need a decomposer)");
  constexpr size_t vs = std::is_void_v<ValueT> ? 0 : sizeof(std::conditional_t<std::is_void_v<ValueT>, char, ValueT>);
  cccl_device_radix_sort_build_result_t* build = nullptr;
  CUresult st = radix_build(type_of<KeyT>::value, sizeof(KeyT), vs, desc, &build);
  if (st != CUDA_SUCCESS)
  {
    return to_cuda_error(st);
  }
  const cccl_type_enum vt = vs == 4 ? CCCL_UINT32 : vs == 8 ? CCCL_UINT64 : CCCL_STORAGE;
  cccl_op_t op{};
  int sel = 0;
  st      = cccl_device_radix_sort(
    *build,
    d_temp_storage,
    &temp_storage_bytes,
    pointer_it(keys_in, type_of<KeyT>::value, sizeof(KeyT)),
    pointer_it(keys_out, type_of<KeyT>::value, sizeof(KeyT)),
    vs ? pointer_it(values_in, vt, vs) : no_values(),
    vs ? pointer_it(values_out, vt, vs) : no_values(),
    op,
    num_items,
    begin_bit,
    end_bit,
    overwrite,
    &sel,
    reinterpret_cast<CUstream>(stream));
  if (selector != nullptr)
  {
    *selector = sel;
  }
  return to_cuda_error(st);
}

} // namespace detail

struct DeviceRadixSort
{
  // ---- pairs ----
  template <typename KeyT, typename ValueT, typename NumItemsT>
  static cudaError_t SortPairs(void* d_temp_storage, size_t& temp_storage_bytes, const KeyT* d_keys_in, KeyT* d_keys_out,
                               const ValueT* d_values_in, ValueT* d_values_out, NumItemsT num_items, int begin_bit = 0,
                               int end_bit = sizeof(KeyT) * 8, cudaStream_t stream = 0)
  {
    return detail::radix_sort<KeyT, ValueT>(false, d_temp_storage, temp_storage_bytes, d_keys_in, d_keys_out, d_values_in,
                                            d_values_out, std::uint64_t(num_items), begin_bit, end_bit, false, nullptr, stream);
  }

  template <typename KeyT, typename ValueT, typename NumItemsT>
  static cudaError_t SortPairs(void* d_temp_storage, size_t& temp_storage_bytes, DoubleBuffer<KeyT>& d_keys,
                               DoubleBuffer<ValueT>& d_values, NumItemsT num_items, int begin_bit = 0,
                               int end_bit = sizeof(KeyT) * 8, cudaStream_t stream = 0)
  {
    return db_pairs(false, d_temp_storage, temp_storage_bytes, d_keys, d_values, num_items, begin_bit, end_bit, stream);
  }

  template <typename KeyT, typename ValueT, typename NumItemsT>
  static cudaError_t SortPairsDescending(void* d_temp_storage, size_t& temp_storage_bytes, const KeyT* d_keys_in,
                                         KeyT* d_keys_out, const ValueT* d_values_in, ValueT* d_values_out,
                                         NumItemsT num_items, int begin_bit = 0, int end_bit = sizeof(KeyT) * 8,
                                         cudaStream_t stream = 0)
  {
    return detail::radix_sort<KeyT, ValueT>(true, d_temp_storage, temp_storage_bytes, d_keys_in, d_keys_out, d_values_in,
                                            d_values_out, std::uint64_t(num_items), begin_bit, end_bit, false, nullptr, stream);
  }

  template <typename KeyT, typename ValueT, typename NumItemsT>
  static cudaError_t SortPairsDescending(void* d_temp_storage, size_t& temp_storage_bytes, DoubleBuffer<KeyT>& d_keys,
                                         DoubleBuffer<ValueT>& d_values, NumItemsT num_items, int begin_bit = 0,
                                         int end_bit = sizeof(KeyT) * 8, cudaStream_t stream = 0)
  {
    return db_pairs(true, d_temp_storage, temp_storage_bytes, d_keys, d_values, num_items, begin_bit, end_bit, stream);
  }

  // ---- keys ----
  template <typename KeyT, typename NumItemsT>
  static cudaError_t SortKeys(void* d_temp_storage, size_t& temp_storage_bytes, const KeyT* d_keys_in, KeyT* d_keys_out,
                              NumItemsT num_items, int begin_bit = 0, int end_bit = sizeof(KeyT) * 8,
                              cudaStream_t stream = 0)
  {
    return detail::radix_sort<KeyT, void>(false, d_temp_storage, temp_storage_bytes, d_keys_in, d_keys_out, nullptr,
                                          nullptr, std::uint64_t(num_items), begin_bit, end_bit, false, nullptr, stream);
  }

  template <typename KeyT, typename NumItemsT>
  static cudaError_t SortKeys(void* d_temp_storage, size_t& temp_storage_bytes, DoubleBuffer<KeyT>& d_keys,
                              NumItemsT num_items, int begin_bit = 0, int end_bit = sizeof(KeyT) * 8,
                              cudaStream_t stream = 0)
  {
    return db_keys(false, d_temp_storage, temp_storage_bytes, d_keys, num_items, begin_bit, end_bit, stream);
  }

  template <typename KeyT, typename NumItemsT>
  static cudaError_t SortKeysDescending(void* d_temp_storage, size_t& temp_storage_bytes, const KeyT* d_keys_in,
                                        KeyT* d_keys_out, NumItemsT num_items, int begin_bit = 0,
                                        int end_bit = sizeof(KeyT) * 8, cudaStream_t stream = 0)
  {
    return detail::radix_sort<KeyT, void>(true, d_temp_storage, temp_storage_bytes, d_keys_in, d_keys_out, nullptr,
                                          nullptr, std::uint64_t(num_items), begin_bit, end_bit, false, nullptr, stream);
  }

  template <typename KeyT, typename NumItemsT>
  static cudaError_t SortKeysDescending(void* d_temp_storage, size_t& temp_storage_bytes, DoubleBuffer<KeyT>& d_keys,
                                        NumItemsT num_items, int begin_bit = 0, int end_bit = sizeof(KeyT) * 8,
                                        cudaStream_t stream = 0)
  {
    return db_keys(true, d_temp_storage, temp_storage_bytes, d_keys, num_items, begin_bit, end_bit, stream);
  }

private:
  template <typename KeyT, typename ValueT, typename NumItemsT>
  static cudaError_t db_pairs(bool desc, void* d_temp_storage, size_t& temp_storage_bytes, DoubleBuffer<KeyT>& d_keys,
                              DoubleBuffer<ValueT>& d_values, NumItemsT num_items, int begin_bit, int end_bit,
                              cudaStream_t stream)
  {
    int sel = 0;
    const cudaError_t e = detail::radix_sort<KeyT, ValueT>(
      desc, d_temp_storage, temp_storage_bytes, d_keys.Current(), d_keys.Alternate(), d_values.Current(),
      d_values.Alternate(), std::uint64_t(num_items), begin_bit, end_bit, true, &sel, stream);
    if (e == cudaSuccess && d_temp_storage != nullptr)
    {
      d_keys.selector ^= sel; // the returned selector is relative to (current, alternate)
      d_values.selector = d_keys.selector;
    }
    return e;
  }

  template <typename KeyT, typename NumItemsT>
  static cudaError_t db_keys(bool desc, void* d_temp_storage, size_t& temp_storage_bytes, DoubleBuffer<KeyT>& d_keys,
                             NumItemsT num_items, int begin_bit, int end_bit, cudaStream_t stream)
  {
    int sel = 0;
    const cudaError_t e = detail::radix_sort<KeyT, void>(
      desc, d_temp_storage, temp_storage_bytes, d_keys.Current(), d_keys.Alternate(), nullptr, nullptr,
      std::uint64_t(num_items), begin_bit, end_bit, true, &sel, stream);
    if (e == cudaSuccess && d_temp_storage != nullptr)
    {
      d_keys.selector ^= sel;
    }
    return e;
  }
};

namespace detail
{
struct segmented_builds
{
  std::mutex m;
  std::map<std::tuple<int, size_t, int, int>, std::unique_ptr<cccl_device_segmented_sort_build_result_t>> map;
  ~segmented_builds()
  {
    for (auto& kv : map)
    {
      kv.second.release();
    }
  }
};

template <typename OffsetT>
constexpr cccl_type_enum offset_type()
{
  static_assert(std::is_integral_v<OffsetT> && (sizeof(OffsetT) == 4 || sizeof(OffsetT) == 8),
                "segment offsets must be pointers to 32- or 64-bit integers");
  return std::is_signed_v<OffsetT> ? (sizeof(OffsetT) == 8 ? CCCL_INT64 : CCCL_INT32)
                                   : (sizeof(OffsetT) == 8 ? CCCL_UINT64 : CCCL_UINT32);
}

template <typename KeyT, typename ValueT, typename BeginT, typename EndT>
cudaError_t segmented_sort(bool desc, void* d_temp_storage, size_t& temp_storage_bytes, const KeyT* keys_in,
                           KeyT* keys_out, const ValueT* values_in, ValueT* values_out, std::int64_t num_items,
                           std::int64_t num_segments, BeginT d_begin_offsets, EndT d_end_offsets, bool overwrite,
                           int* selector, cudaStream_t stream, bool radix_only = false, int begin_bit = 0,
                           int end_bit = 0)
{
  static_assert(std::is_pointer_v<BeginT> && std::is_pointer_v<EndT>, "segment offsets must be pointers");
  using BO = std::remove_cv_t<std::remove_pointer_t<BeginT>>;
  using EO = std::remove_cv_t<std::remove_pointer_t<EndT>>;
  static_assert(sizeof(BO) == sizeof(EO), "begin and end offsets of one width");
  static_assert(type_of<KeyT>::supported, "key type not supported");
  constexpr size_t vs = std::is_void_v<ValueT> ? 0 : sizeof(std::conditional_t<std::is_void_v<ValueT>, char, ValueT>);
  const cccl_type_enum vt = vs == 4 ? CCCL_UINT32 : vs == 8 ? CCCL_UINT64 : CCCL_STORAGE;

  static segmented_builds b;
  cccl_device_segmented_sort_build_result_t* build = nullptr;
  {
    std::lock_guard<std::mutex> lock(b.m);
    const auto key = std::make_tuple(int(type_of<KeyT>::value), vs, int(desc), int(sizeof(BO)));
    auto it        = b.map.find(key);
    if (it == b.map.end())
    {
      int major = 0, minor = 0;
      if (current_cc(major, minor) != 0)
      {
        return cudaErrorInvalidDevice;
      }
      auto r = std::make_unique<cccl_device_segmented_sort_build_result_t>();
      const CUresult st = cccl_device_segmented_sort_build(
        r.get(), desc ? CCCL_DESCENDING : CCCL_ASCENDING, pointer_it(nullptr, type_of<KeyT>::value, sizeof(KeyT)),
        vs ? pointer_it(reinterpret_cast<void*>(16), vt, vs) : no_values(),
        pointer_it(nullptr, offset_type<BO>(), sizeof(BO)), pointer_it(nullptr, offset_type<EO>(), sizeof(EO)), major,
        minor, "", nullptr, nullptr, nullptr);
      if (st != CUDA_SUCCESS)
      {
        return to_cuda_error(st);
      }
      it = b.map.emplace(key, std::move(r)).first;
    }
    build = it->second.get();
  }
  int sel = 0;
  const cccl_iterator_t ki = pointer_it(keys_in, type_of<KeyT>::value, sizeof(KeyT));
  const cccl_iterator_t ko = pointer_it(keys_out, type_of<KeyT>::value, sizeof(KeyT));
  const cccl_iterator_t vi = vs ? pointer_it(values_in, vt, vs) : no_values();
  const cccl_iterator_t vo = vs ? pointer_it(values_out, vt, vs) : no_values();
  const cccl_iterator_t bo = pointer_it(d_begin_offsets, offset_type<BO>(), sizeof(BO));
  const cccl_iterator_t eo = pointer_it(d_end_offsets, offset_type<EO>(), sizeof(EO));
  const CUresult st =
    radix_only
      ? cccl_gb300_segmented_radix_sort(*build, d_temp_storage, &temp_storage_bytes, ki, ko, vi, vo,
                                        std::uint64_t(num_items), std::uint64_t(num_segments), bo, eo, begin_bit,
                                        end_bit, overwrite, &sel, reinterpret_cast<CUstream>(stream))
      : cccl_device_segmented_sort(*build, d_temp_storage, &temp_storage_bytes, ki, ko, vi, vo,
                                   std::uint64_t(num_items), std::uint64_t(num_segments), bo, eo, overwrite, &sel,
                                   reinterpret_cast<CUstream>(stream));
  if (selector != nullptr)
  {
    *selector = sel;
  }
  return to_cuda_error(st);
}
} // namespace detail

// DeviceSegmentedSort: every form is stable (the reference documents SortKeys and
// StableSortKeys as the same algorithm, device_segmented_sort.cuh:3638-3652).
struct DeviceSegmentedSort
{
#define CCCL_GB300_SEG_KEYS(NAME, DESC)                                                                                 \
  template <typename KeyT, typename BeginOffsetIteratorT, typename EndOffsetIteratorT>                                \
  static cudaError_t NAME(void* d_temp_storage, size_t& temp_storage_bytes, const KeyT* d_keys_in, KeyT* d_keys_out,  \
                          std::int64_t num_items, std::int64_t num_segments, BeginOffsetIteratorT d_begin_offsets,    \
                          EndOffsetIteratorT d_end_offsets, cudaStream_t stream = 0)                                  \
  {                                                                                                                   \
    return detail::segmented_sort<KeyT, void>(DESC, d_temp_storage, temp_storage_bytes, d_keys_in, d_keys_out,        \
                                              nullptr, nullptr, num_items, num_segments, d_begin_offsets,             \
                                              d_end_offsets, false, nullptr, stream);                                 \
  }                                                                                                                   \
  template <typename KeyT, typename BeginOffsetIteratorT, typename EndOffsetIteratorT>                                \
  static cudaError_t NAME(void* d_temp_storage, size_t& temp_storage_bytes, DoubleBuffer<KeyT>& d_keys,               \
                          std::int64_t num_items, std::int64_t num_segments, BeginOffsetIteratorT d_begin_offsets,    \
                          EndOffsetIteratorT d_end_offsets, cudaStream_t stream = 0)                                  \
  {                                                                                                                   \
    int sel             = 0;                                                                                          \
    const cudaError_t e = detail::segmented_sort<KeyT, void>(                                                         \
      DESC, d_temp_storage, temp_storage_bytes, d_keys.Current(), d_keys.Alternate(), nullptr, nullptr, num_items,    \
      num_segments, d_begin_offsets, d_end_offsets, true, &sel, stream);                                              \
    if (e == cudaSuccess && d_temp_storage != nullptr)                                                                \
    {                                                                                                                 \
      d_keys.selector ^= sel;                                                                                         \
    }                                                                                                                 \
    return e;                                                                                                         \
  }

#define CCCL_GB300_SEG_PAIRS(NAME, DESC)                                                                                \
  template <typename KeyT, typename ValueT, typename BeginOffsetIteratorT, typename EndOffsetIteratorT>               \
  static cudaError_t NAME(void* d_temp_storage, size_t& temp_storage_bytes, const KeyT* d_keys_in, KeyT* d_keys_out,  \
                          const ValueT* d_values_in, ValueT* d_values_out, std::int64_t num_items,                    \
                          std::int64_t num_segments, BeginOffsetIteratorT d_begin_offsets,                            \
                          EndOffsetIteratorT d_end_offsets, cudaStream_t stream = 0)                                  \
  {                                                                                                                   \
    return detail::segmented_sort<KeyT, ValueT>(DESC, d_temp_storage, temp_storage_bytes, d_keys_in, d_keys_out,      \
                                                d_values_in, d_values_out, num_items, num_segments, d_begin_offsets,  \
                                                d_end_offsets, false, nullptr, stream);                               \
  }                                                                                                                   \
  template <typename KeyT, typename ValueT, typename BeginOffsetIteratorT, typename EndOffsetIteratorT>               \
  static cudaError_t NAME(void* d_temp_storage, size_t& temp_storage_bytes, DoubleBuffer<KeyT>& d_keys,               \
                          DoubleBuffer<ValueT>& d_values, std::int64_t num_items, std::int64_t num_segments,          \
                          BeginOffsetIteratorT d_begin_offsets, EndOffsetIteratorT d_end_offsets,                     \
                          cudaStream_t stream = 0)                                                                    \
  {                                                                                                                   \
    int sel             = 0;                                                                                          \
    const cudaError_t e = detail::segmented_sort<KeyT, ValueT>(                                                       \
      DESC, d_temp_storage, temp_storage_bytes, d_keys.Current(), d_keys.Alternate(), d_values.Current(),             \
      d_values.Alternate(), num_items, num_segments, d_begin_offsets, d_end_offsets, true, &sel, stream);             \
    if (e == cudaSuccess && d_temp_storage != nullptr)                                                                \
    {                                                                                                                 \
      d_keys.selector ^= sel;                                                                                         \
      d_values.selector = d_keys.selector;                                                                            \
    }                                                                                                                 \
    return e;                                                                                                         \
  }

  CCCL_GB300_SEG_KEYS(SortKeys, false)
  CCCL_GB300_SEG_KEYS(SortKeysDescending, true)
  CCCL_GB300_SEG_KEYS(StableSortKeys, false)
  CCCL_GB300_SEG_KEYS(StableSortKeysDescending, true)
  CCCL_GB300_SEG_PAIRS(SortPairs, false)
  CCCL_GB300_SEG_PAIRS(SortPairsDescending, true)
  CCCL_GB300_SEG_PAIRS(StableSortPairs, false)
  CCCL_GB300_SEG_PAIRS(StableSortPairsDescending, true)
#undef CCCL_GB300_SEG_KEYS
#undef CCCL_GB300_SEG_PAIRS
};

// DeviceSegmentedRadixSort: radix order in every segment over bits [begin_bit, end_bit), the
// returned DoubleBuffer selector follows that dispatch (dispatch_segmented_radix_sort.cuh:519-526).
struct DeviceSegmentedRadixSort
{
  template <typename KeyT, typename ValueT, typename BeginOffsetIteratorT, typename EndOffsetIteratorT>
  static cudaError_t SortPairs(void* d_temp_storage, size_t& temp_storage_bytes, const KeyT* d_keys_in, KeyT* d_keys_out,
                               const ValueT* d_values_in, ValueT* d_values_out, std::int64_t num_items,
                               std::int64_t num_segments, BeginOffsetIteratorT d_begin_offsets,
                               EndOffsetIteratorT d_end_offsets, int begin_bit = 0, int end_bit = sizeof(KeyT) * 8,
                               cudaStream_t stream = 0)
  {
    return detail::segmented_sort<KeyT, ValueT>(false, d_temp_storage, temp_storage_bytes, d_keys_in, d_keys_out,
                                                d_values_in, d_values_out, num_items, num_segments, d_begin_offsets,
                                                d_end_offsets, false, nullptr, stream, true, begin_bit, end_bit);
  }
  template <typename KeyT, typename ValueT, typename BeginOffsetIteratorT, typename EndOffsetIteratorT>
  static cudaError_t SortPairsDescending(void* d_temp_storage, size_t& temp_storage_bytes, const KeyT* d_keys_in,
                                         KeyT* d_keys_out, const ValueT* d_values_in, ValueT* d_values_out,
                                         std::int64_t num_items, std::int64_t num_segments,
                                         BeginOffsetIteratorT d_begin_offsets, EndOffsetIteratorT d_end_offsets,
                                         int begin_bit = 0, int end_bit = sizeof(KeyT) * 8, cudaStream_t stream = 0)
  {
    return detail::segmented_sort<KeyT, ValueT>(true, d_temp_storage, temp_storage_bytes, d_keys_in, d_keys_out,
                                                d_values_in, d_values_out, num_items, num_segments, d_begin_offsets,
                                                d_end_offsets, false, nullptr, stream, true, begin_bit, end_bit);
  }
  template <typename KeyT, typename ValueT, typename BeginOffsetIteratorT, typename EndOffsetIteratorT>
  static cudaError_t SortPairs(void* d_temp_storage, size_t& temp_storage_bytes, DoubleBuffer<KeyT>& d_keys,
                               DoubleBuffer<ValueT>& d_values, std::int64_t num_items, std::int64_t num_segments,
                               BeginOffsetIteratorT d_begin_offsets, EndOffsetIteratorT d_end_offsets,
                               int begin_bit = 0, int end_bit = sizeof(KeyT) * 8, cudaStream_t stream = 0)
  {
    return db_pairs(false, d_temp_storage, temp_storage_bytes, d_keys, d_values, num_items, num_segments,
                    d_begin_offsets, d_end_offsets, begin_bit, end_bit, stream);
  }
  template <typename KeyT, typename ValueT, typename BeginOffsetIteratorT, typename EndOffsetIteratorT>
  static cudaError_t SortPairsDescending(void* d_temp_storage, size_t& temp_storage_bytes, DoubleBuffer<KeyT>& d_keys,
                                         DoubleBuffer<ValueT>& d_values, std::int64_t num_items,
                                         std::int64_t num_segments, BeginOffsetIteratorT d_begin_offsets,
                                         EndOffsetIteratorT d_end_offsets, int begin_bit = 0,
                                         int end_bit = sizeof(KeyT) * 8, cudaStream_t stream = 0)
  {
    return db_pairs(true, d_temp_storage, temp_storage_bytes, d_keys, d_values, num_items, num_segments,
                    d_begin_offsets, d_end_offsets, begin_bit, end_bit, stream);
  }
  template <typename KeyT, typename BeginOffsetIteratorT, typename EndOffsetIteratorT>
  static cudaError_t SortKeys(void* d_temp_storage, size_t& temp_storage_bytes, const KeyT* d_keys_in, KeyT* d_keys_out,
                              std::int64_t num_items, std::int64_t num_segments, BeginOffsetIteratorT d_begin_offsets,
                              EndOffsetIteratorT d_end_offsets, int begin_bit = 0, int end_bit = sizeof(KeyT) * 8,
                              cudaStream_t stream = 0)
  {
    return detail::segmented_sort<KeyT, void>(false, d_temp_storage, temp_storage_bytes, d_keys_in, d_keys_out, nullptr,
                                              nullptr, num_items, num_segments, d_begin_offsets, d_end_offsets, false,
                                              nullptr, stream, true, begin_bit, end_bit);
  }
  template <typename KeyT, typename BeginOffsetIteratorT, typename EndOffsetIteratorT>
  static cudaError_t SortKeysDescending(void* d_temp_storage, size_t& temp_storage_bytes, const KeyT* d_keys_in,
                                        KeyT* d_keys_out, std::int64_t num_items, std::int64_t num_segments,
                                        BeginOffsetIteratorT d_begin_offsets, EndOffsetIteratorT d_end_offsets,
                                        int begin_bit = 0, int end_bit = sizeof(KeyT) * 8, cudaStream_t stream = 0)
  {
    return detail::segmented_sort<KeyT, void>(true, d_temp_storage, temp_storage_bytes, d_keys_in, d_keys_out, nullptr,
                                              nullptr, num_items, num_segments, d_begin_offsets, d_end_offsets, false,
                                              nullptr, stream, true, begin_bit, end_bit);
  }
  template <typename KeyT, typename BeginOffsetIteratorT, typename EndOffsetIteratorT>
  static cudaError_t SortKeys(void* d_temp_storage, size_t& temp_storage_bytes, DoubleBuffer<KeyT>& d_keys,
                              std::int64_t num_items, std::int64_t num_segments, BeginOffsetIteratorT d_begin_offsets,
                              EndOffsetIteratorT d_end_offsets, int begin_bit = 0, int end_bit = sizeof(KeyT) * 8,
                              cudaStream_t stream = 0)
  {
    return db_keys(false, d_temp_storage, temp_storage_bytes, d_keys, num_items, num_segments, d_begin_offsets,
                   d_end_offsets, begin_bit, end_bit, stream);
  }
  template <typename KeyT, typename BeginOffsetIteratorT, typename EndOffsetIteratorT>
  static cudaError_t SortKeysDescending(void* d_temp_storage, size_t& temp_storage_bytes, DoubleBuffer<KeyT>& d_keys,
                                        std::int64_t num_items, std::int64_t num_segments,
                                        BeginOffsetIteratorT d_begin_offsets, EndOffsetIteratorT d_end_offsets,
                                        int begin_bit = 0, int end_bit = sizeof(KeyT) * 8, cudaStream_t stream = 0)
  {
    return db_keys(true, d_temp_storage, temp_storage_bytes, d_keys, num_items, num_segments, d_begin_offsets,
                   d_end_offsets, begin_bit, end_bit, stream);
  }

private:
  template <typename KeyT, typename ValueT, typename B, typename E>
  static cudaError_t db_pairs(bool desc, void* d_temp_storage, size_t& temp_storage_bytes, DoubleBuffer<KeyT>& d_keys,
                              DoubleBuffer<ValueT>& d_values, std::int64_t num_items, std::int64_t num_segments, B b,
                              E e, int begin_bit, int end_bit, cudaStream_t stream)
  {
    int sel             = 0;
    const cudaError_t r = detail::segmented_sort<KeyT, ValueT>(
      desc, d_temp_storage, temp_storage_bytes, d_keys.Current(), d_keys.Alternate(), d_values.Current(),
      d_values.Alternate(), num_items, num_segments, b, e, true, &sel, stream, true, begin_bit, end_bit);
    if (r == cudaSuccess && d_temp_storage != nullptr)
    {
      d_keys.selector ^= sel;
      d_values.selector = d_keys.selector;
    }
    return r;
  }
  template <typename KeyT, typename B, typename E>
  static cudaError_t db_keys(bool desc, void* d_temp_storage, size_t& temp_storage_bytes, DoubleBuffer<KeyT>& d_keys,
                             std::int64_t num_items, std::int64_t num_segments, B b, E e, int begin_bit, int end_bit,
                             cudaStream_t stream)
  {
    int sel             = 0;
    const cudaError_t r = detail::segmented_sort<KeyT, void>(
      desc, d_temp_storage, temp_storage_bytes, d_keys.Current(), d_keys.Alternate(), nullptr, nullptr, num_items,
      num_segments, b, e, true, &sel, stream, true, begin_bit, end_bit);
    if (r == cudaSuccess && d_temp_storage != nullptr)
    {
      d_keys.selector ^= sel;
    }
    return r;
  }
};

} // namespace cub
} // namespace cccl_gb300
