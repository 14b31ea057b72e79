// CPU oracle of the sort path. TEST INFRASTRUCTURE ONLY: the parity tests, the smoke
// check and the CPU-baseline leg of the benchmark call it; the library never does.
//
// Plain radix sort (DeviceRadixSort) semantics, restating the reference's own CPU
// reference cub/test/catch2_radix_sort_helper.cuh:
//   get_striped_keys  :174-214  -0.0 -> +0.0 (floats), TwiddleIn, mask [begin_bit, end_bit)
//   get_permutation   :235-268  std::stable_sort of indices with < (asc) or > (desc)
//   radix_sort_reference :270-310  gather keys (and values) by that permutation
// TwiddleIn itself follows cub/cub/util_type.cuh:893-963 (signed: flip the high bit;
// float: flip all bits of negatives, the high bit of positives).
//
// Segmented sort (DeviceSegmentedSort) semantics are in oracle_segmented.cpp.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#if defined(_OPENMP)
#  include <parallel/algorithm>
#endif

#include "oracle.h"

namespace
{

// cccl_type_enum codes (c/parallel/include/cccl/c/types.h:31-47)
enum : int
{
  T_INT8 = 0,
  T_INT16,
  T_INT32,
  T_INT64,
  T_UINT8,
  T_UINT16,
  T_UINT32,
  T_UINT64,
  T_FLOAT16,
  T_FLOAT32,
  T_FLOAT64,
  T_STORAGE,
  T_BOOLEAN
};

struct key_desc
{
  int bytes;
  int kind; // 0 unsigned, 1 signed, 2 float
};

bool describe(int key_type, key_desc& d)
{
  switch (key_type)
  {
    case T_UINT8:
    case T_BOOLEAN:
      d = {1, 0};
      return true;
    case T_UINT16:
      d = {2, 0};
      return true;
    case T_UINT32:
      d = {4, 0};
      return true;
    case T_UINT64:
      d = {8, 0};
      return true;
    case T_INT8:
      d = {1, 1};
      return true;
    case T_INT16:
      d = {2, 1};
      return true;
    case T_INT32:
      d = {4, 1};
      return true;
    case T_INT64:
      d = {8, 1};
      return true;
    case T_FLOAT16:
      d = {2, 2};
      return true;
    case T_FLOAT32:
      d = {4, 2};
      return true;
    case T_FLOAT64:
      d = {8, 2};
      return true;
    default:
      return false;
  }
}

uint64_t load_bits(const unsigned char* p, int bytes)
{
  uint64_t v = 0;
  std::memcpy(&v, p, size_t(bytes)); // little endian on both x86_64 and aarch64
  return v;
}

} // namespace

// zero_to_minus: fold +0.0 into -0.0 instead of -0.0 into +0.0. That is the order CUB's
// onesweep passes give a descending sort: they complement the twiddled keys and then fold the
// twiddled -0.0 pattern (cub/cub/block/radix_rank_sort_operations.cuh:43-80), which in
// uncomplemented terms leaves both zeros at -0.0's pattern. Only a bit window narrower than
// the key can tell the two apart.
extern "C" uint64_t oracle_striped_key_ex(uint64_t raw, int bytes, int kind, int begin_bit, int end_bit, int zero_to_minus)
{
  const uint64_t all  = bytes == 8 ? ~0ull : ((1ull << (8 * bytes)) - 1ull);
  const uint64_t high = 1ull << (8 * bytes - 1);
  uint64_t key        = raw & all;
  if (kind == 2 && !zero_to_minus && key == high) // -0.0 becomes +0.0 before twiddling
  {
    key = 0;
  }
  if (kind == 2 && zero_to_minus && key == 0)
  {
    key = high;
  }
  if (kind == 1)
  {
    key ^= high;
  }
  else if (kind == 2)
  {
    key ^= (key & high) ? all : high;
  }
  const int num_bits = end_bit - begin_bit;
  if (begin_bit > 0 || end_bit < 8 * bytes)
  {
    const uint64_t m = (num_bits >= 64 ? ~0ull : ((1ull << num_bits) - 1ull)) << begin_bit;
    key &= m;
  }
  return key;
}

extern "C" uint64_t oracle_striped_key(uint64_t raw, int bytes, int kind, int begin_bit, int end_bit)
{
  return oracle_striped_key_ex(raw, bytes, kind, begin_bit, end_bit, 0);
}

extern "C" {

int oracle_radix_permutation(
  int key_type, const void* keys, uint64_t n, int begin_bit, int end_bit, int descending, int threads, uint64_t* perm)
{
  key_desc d{};
  if (!describe(key_type, d) || begin_bit < 0 || end_bit > 8 * d.bytes || begin_bit > end_bit)
  {
    return 1;
  }
  const auto* kp = static_cast<const unsigned char*>(keys);
  std::vector<uint64_t> striped(n);
  for (uint64_t i = 0; i < n; ++i)
  {
    // descending == 2: a descending sort with CUB onesweep's zero folding
    striped[i] =
      oracle_striped_key_ex(load_bits(kp + i * d.bytes, d.bytes), d.bytes, d.kind, begin_bit, end_bit, descending == 2);
  }
  std::iota(perm, perm + n, uint64_t(0));
  const uint64_t* s = striped.data();
  auto asc          = [s](uint64_t a, uint64_t b) {
    return s[a] < s[b];
  };
  auto desc = [s](uint64_t a, uint64_t b) {
    return s[a] > s[b];
  };
#if defined(_OPENMP)
  if (threads > 1)
  {
    if (descending)
    {
      __gnu_parallel::stable_sort(perm, perm + n, desc);
    }
    else
    {
      __gnu_parallel::stable_sort(perm, perm + n, asc);
    }
    return 0;
  }
#else
  (void) threads;
#endif
  if (descending)
  {
    std::stable_sort(perm, perm + n, desc);
  }
  else
  {
    std::stable_sort(perm, perm + n, asc);
  }
  return 0;
}

int oracle_radix_sort(
  int key_type,
  const void* keys_in,
  void* keys_out,
  uint64_t value_bytes,
  const void* values_in,
  void* values_out,
  uint64_t n,
  int begin_bit,
  int end_bit,
  int descending,
  int threads)
{
  key_desc d{};
  if (!describe(key_type, d))
  {
    return 1;
  }
  std::vector<uint64_t> perm(n);
  if (int rc = oracle_radix_permutation(key_type, keys_in, n, begin_bit, end_bit, descending, threads, perm.data()))
  {
    return rc;
  }
  const auto* ki = static_cast<const unsigned char*>(keys_in);
  auto* ko       = static_cast<unsigned char*>(keys_out);
  for (uint64_t i = 0; i < n; ++i)
  {
    std::memcpy(ko + i * d.bytes, ki + perm[i] * d.bytes, size_t(d.bytes));
  }
  if (value_bytes > 0 && values_in != nullptr && values_out != nullptr)
  {
    const auto* vi = static_cast<const unsigned char*>(values_in);
    auto* vo       = static_cast<unsigned char*>(values_out);
    for (uint64_t i = 0; i < n; ++i)
    {
      std::memcpy(vo + i * value_bytes, vi + perm[i] * value_bytes, size_t(value_bytes));
    }
  }
  return 0;
}

} // extern "C"
