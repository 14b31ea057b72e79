// CPU oracle of cub::DeviceSegmentedSort (test infrastructure only).
//
// Which algorithm sorts a segment decides where NaN keys land, so the oracle restates the
// reference's size classes and its sub-warp merge network step by step:
//   * policy for cc >= 8.6: cub/cub/device/dispatch/tuning/tuning_segmented_sort.cuh:182-195
//     (small: 2 threads x 9 items, or 8 x 7-scaled for > 4-byte types; medium: 16 threads x
//     7 items, or 9-scaled; items scaled by cub/cub/util_math.cuh:54-57);
//   * partitioning only when num_segments > 500 (dispatch_segmented_sort.cuh:465) with
//     large = size > medium tile, small = size < small tile + 1 (:494-497,
//     kernel_segmented_sort.cuh:33-84); otherwise the fallback kernel sorts sizes <= medium
//     tile with the medium network and the rest by radix (kernel_segmented_sort.cuh:209-270);
//   * sizes 1 and 2 short-circuit (agent_sub_warp_merge_sort.cuh:276-340), larger ones load
//     blocked with an out-of-bounds default key (:225-262), then WarpMergeSort runs
//     BlockMergeSortStrategy::Sort (block_merge_sort.cuh:425-520): fill past the valid items
//     with the thread's running maximum, per-thread stable odd-even sort (thread_sort.cuh:27-50),
//     then log2(threads) Merge Path + serial merge rounds (block_merge_sort.cuh:39-160);
//   * radix-sorted segments follow DeviceRadixSort order (oracle.cpp).
// The comparison is the key type's own operator< (or > for descending), so NaN compares
// false with everything, exactly as on the GPU.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#if defined(_OPENMP)
#  include <omp.h>
#endif

#include "oracle.h"

namespace
{

float half_to_float(uint16_t h)
{
  const uint32_t sign = uint32_t(h >> 15) << 31;
  const uint32_t exp  = (h >> 10) & 0x1f;
  const uint32_t mant = h & 0x3ff;
  uint32_t bits;
  if (exp == 0x1f)
  {
    bits = sign | 0x7f800000u | (mant << 13);
  }
  else if (exp == 0)
  {
    if (mant == 0)
    {
      bits = sign;
    }
    else
    {
      // subnormal half -> normal float
      int e      = -1;
      uint32_t m = mant;
      do
      {
        m <<= 1;
        ++e;
      } while ((m & 0x400) == 0);
      bits = sign | uint32_t(127 - 15 - e) << 23 | ((m & 0x3ff) << 13);
    }
  }
  else
  {
    bits = sign | ((exp + 112) << 23) | (mant << 13);
  }
  float f;
  std::memcpy(&f, &bits, 4);
  return f;
}

// A key as the merge network sees it: raw bits (what is moved) and a value to compare.
struct Key
{
  uint64_t bits;
  double cmp; // exact for every integer <= 2^53 is not needed: integers compare by `i`
  int64_t i;
  bool is_int;
};

struct KeyModel
{
  int bytes;
  int kind; // 0 unsigned, 1 signed, 2 float
  bool desc;

  Key make(const unsigned char* p) const
  {
    uint64_t b = 0;
    std::memcpy(&b, p, size_t(bytes));
    Key k{b, 0.0, 0, kind != 2};
    if (kind == 0)
    {
      k.i = int64_t(b); // unsigned 64-bit keys compare through the unsigned path below
    }
    else if (kind == 1)
    {
      const int sh = 64 - 8 * bytes;
      k.i          = int64_t(b << sh) >> sh;
    }
    else if (bytes == 2)
    {
      k.cmp = half_to_float(uint16_t(b));
    }
    else if (bytes == 4)
    {
      float f;
      uint32_t u = uint32_t(b);
      std::memcpy(&f, &u, 4);
      k.cmp = f;
    }
    else
    {
      std::memcpy(&k.cmp, &b, 8);
    }
    return k;
  }

  bool less(const Key& a, const Key& b) const
  {
    if (kind == 0)
    {
      return a.bits < b.bits;
    }
    if (kind == 1)
    {
      return a.i < b.i;
    }
    return a.cmp < b.cmp;
  }

  // BinaryOpT of agent_sub_warp_merge_sort.cuh:98-111
  bool op(const Key& a, const Key& b) const
  {
    return desc ? less(b, a) : less(a, b);
  }

  bool equal(const Key& a, const Key& b) const
  {
    if (kind == 2)
    {
      return a.cmp == b.cmp;
    }
    return a.bits == b.bits;
  }

  // max_raw_binary_key (ascending) / min_raw_binary_key (descending): the bit patterns that
  // TwiddleIn maps to all ones / all zeros.
  Key oob_default() const
  {
    const uint64_t all  = bytes == 8 ? ~0ull : ((1ull << (8 * bytes)) - 1ull);
    const uint64_t high = 1ull << (8 * bytes - 1);
    uint64_t b;
    if (kind == 0)
    {
      b = desc ? 0 : all;
    }
    else if (kind == 1)
    {
      b = desc ? high : (all ^ high);
    }
    else
    {
      b = desc ? all : (all ^ high);
    }
    unsigned char raw[8];
    std::memcpy(raw, &b, 8);
    return make(raw);
  }
};

struct NetworkShape
{
  int threads;
  int items;
};

int scale_items(int nominal, int dominant_size)
{
  return std::clamp(nominal * 4 / dominant_size, 1, nominal);
}

// Sub-warp merge sort of one segment (size >= 3), in place on keys (and values).
void warp_merge_sort(const KeyModel& m,
                     NetworkShape s,
                     std::vector<Key>& seg_keys,
                     std::vector<uint64_t>* seg_vals /* value slot indices */)
{
  const int T     = s.threads;
  const int I     = s.items;
  const int tile  = T * I;
  const int valid = int(seg_keys.size());
  const Key oob   = m.oob_default();

  std::vector<Key> k(size_t(tile) + 1, oob);
  std::vector<uint64_t> v(size_t(tile) + 1, 0);
  for (int x = 0; x < valid; ++x)
  {
    k[x] = seg_keys[x];
    v[x] = seg_vals ? (*seg_vals)[x] : 0;
  }

  // fill past the valid items with the thread's running maximum (first item excluded)
  for (int t = 0; t < T; ++t)
  {
    Key max_key = oob;
    for (int i = 1; i < I; ++i)
    {
      const int x = t * I + i;
      if (x < valid)
      {
        max_key = m.op(max_key, k[x]) ? k[x] : max_key;
      }
      else
      {
        k[x] = max_key;
      }
    }
  }
  // stable odd-even transposition sort inside each thread whose first item is valid
  for (int t = 0; t < T; ++t)
  {
    if (t * I >= valid)
    {
      continue;
    }
    Key* kk     = &k[size_t(t) * I];
    uint64_t* vv = &v[size_t(t) * I];
    for (int i = 0; i < I; ++i)
    {
      for (int j = 1 & i; j < I - 1; j += 2)
      {
        if (m.op(kk[j + 1], kk[j]))
        {
          std::swap(kk[j], kk[j + 1]);
          std::swap(vv[j], vv[j + 1]);
        }
      }
    }
  }
  // merge rounds: groups of 2, 4, ... threads, each thread producing I outputs
  std::vector<Key> shared(size_t(tile) + 1);
  std::vector<uint64_t> vshared(size_t(tile) + 1);
  std::vector<Key> nk(size_t(tile) + 1);
  std::vector<uint64_t> nv(size_t(tile) + 1);
  for (int target = 2; target <= T; target *= 2)
  {
    const int merged = target / 2;
    const int mask   = target - 1;
    for (int x = 0; x < tile; ++x)
    {
      shared[x]  = k[x];
      vshared[x] = v[x];
    }
    shared[tile]  = oob; // one past the end may be read, never used
    vshared[tile] = 0;
    for (int t = 0; t < T; ++t)
    {
      const int first  = ~mask & t;
      const int start  = I * first;
      const int size   = I * merged;
      const int local  = mask & t;
      const int diag   = std::min(valid, I * local);
      const int k1_beg = std::min(valid, start);
      const int k1_end = std::min(valid, k1_beg + size);
      const int k2_beg = k1_end;
      const int k2_end = std::min(valid, k2_beg + size);
      const int n1     = k1_end - k1_beg;
      const int n2     = k2_end - k2_beg;
      // Merge Path: how many of the diag first outputs come from sequence 1
      int lo = diag < n2 ? 0 : diag - n2;
      int hi = std::min(diag, n1);
      while (lo < hi)
      {
        const int mid = lo + (hi - lo) / 2;
        if (m.op(shared[k2_beg + diag - 1 - mid], shared[k1_beg + mid]))
        {
          hi = mid;
        }
        else
        {
          lo = mid + 1;
        }
      }
      int b1        = k1_beg + lo;
      int b2        = k2_beg + diag - lo;
      const int e1  = k1_end;
      const int e2  = k2_end;
      Key key1      = (e1 - b1) != 0 ? shared[b1] : oob;
      Key key2      = (e2 - b2) != 0 ? shared[b2] : oob;
      for (int i = 0; i < I; ++i)
      {
        const bool p       = (b2 < e2) && ((b1 >= e1) || m.op(key2, key1));
        nk[size_t(t) * I + i] = p ? key2 : key1;
        const int src      = p ? b2++ : b1++;
        nv[size_t(t) * I + i] = vshared[src];
        if (p)
        {
          key2 = shared[b2];
        }
        else
        {
          key1 = shared[b1];
        }
      }
    }
    for (int x = 0; x < tile; ++x)
    {
      k[x] = nk[x];
      v[x] = nv[x];
    }
  }
  for (int x = 0; x < valid; ++x)
  {
    seg_keys[x] = k[x];
    if (seg_vals)
    {
      (*seg_vals)[x] = v[x];
    }
  }
}

} // namespace

extern "C" int oracle_segmented_sort(int key_type,
                                     const void* keys_in,
                                     void* keys_out,
                                     uint64_t value_bytes,
                                     const void* values_in,
                                     void* values_out,
                                     uint64_t num_items,
                                     uint64_t num_segments,
                                     const int64_t* begin_offsets,
                                     const int64_t* end_offsets,
                                     int descending,
                                     int threads)
{
  int bytes = 0, kind = 0;
  switch (key_type)
  {
    case 0: bytes = 1, kind = 1; break;
    case 1: bytes = 2, kind = 1; break;
    case 2: bytes = 4, kind = 1; break;
    case 3: bytes = 8, kind = 1; break;
    case 4: case 12: bytes = 1, kind = 0; break;
    case 5: bytes = 2, kind = 0; break;
    case 6: bytes = 4, kind = 0; break;
    case 7: bytes = 8, kind = 0; break;
    case 8: bytes = 2, kind = 2; break;
    case 9: bytes = 4, kind = 2; break;
    case 10: bytes = 8, kind = 2; break;
    default: return 1;
  }
  const KeyModel m{bytes, kind, descending != 0};
  const bool has_vals    = value_bytes > 0 && values_in && values_out;
  const int dominant     = std::max<int>(bytes, has_vals ? int(value_bytes) : 0);
  const bool large_items = dominant > 4;
  const NetworkShape small{large_items ? 8 : 2, scale_items(large_items ? 7 : 9, dominant)};
  const NetworkShape medium{16, scale_items(large_items ? 9 : 7, dominant)};
  const int64_t small_tile  = small.threads * small.items;
  const int64_t medium_tile = medium.threads * medium.items;
  const bool partition      = num_segments > 500;

  const auto* ki = static_cast<const unsigned char*>(keys_in);
  auto* ko       = static_cast<unsigned char*>(keys_out);
  const auto* vi = static_cast<const unsigned char*>(values_in);
  auto* vo       = static_cast<unsigned char*>(values_out);
  (void) num_items;
  (void) threads;

#if defined(_OPENMP)
#  pragma omp parallel for schedule(dynamic, 16) if (threads > 1) num_threads(threads > 1 ? threads : 1)
#endif
  for (int64_t s = 0; s < int64_t(num_segments); ++s)
  {
    const int64_t b    = begin_offsets[s];
    const int64_t size = end_offsets[s] - b;
    if (size <= 0)
    {
      continue;
    }
    std::vector<uint64_t> order(static_cast<size_t>(size)); // source index (within the segment) of each output
    bool network   = false;
    NetworkShape shape{};
    if (partition)
    {
      if (size <= small_tile)
      {
        network = true, shape = small;
      }
      else if (size <= medium_tile)
      {
        network = true, shape = medium;
      }
    }
    else if (size <= medium_tile)
    {
      network = true, shape = medium;
    }
    if (network && size < 3)
    {
      order[0] = 0;
      if (size == 2)
      {
        const Key lhs = m.make(ki + size_t(b) * bytes);
        const Key rhs = m.make(ki + size_t(b + 1) * bytes);
        const bool keep = m.equal(lhs, rhs) || m.op(lhs, rhs);
        order[0]        = keep ? 0 : 1;
        order[1]        = keep ? 1 : 0;
      }
    }
    else if (network)
    {
      std::vector<Key> kk(static_cast<size_t>(size));
      for (int64_t x = 0; x < size; ++x)
      {
        kk[size_t(x)]    = m.make(ki + size_t(b + x) * bytes);
        order[size_t(x)] = uint64_t(x);
      }
      warp_merge_sort(m, shape, kk, &order);
    }
    else
    {
      oracle_radix_permutation(key_type, ki + size_t(b) * bytes, uint64_t(size), 0, 8 * bytes, descending, 1, order.data());
    }
    for (int64_t x = 0; x < size; ++x)
    {
      std::memcpy(ko + size_t(b + x) * bytes, ki + size_t(b + int64_t(order[size_t(x)])) * bytes, size_t(bytes));
      if (has_vals)
      {
        std::memcpy(vo + size_t(b + x) * value_bytes, vi + size_t(b + int64_t(order[size_t(x)])) * value_bytes,
                    size_t(value_bytes));
      }
    }
  }
  return 0;
}
