// Batched segmented sort kernels (cub::DeviceSegmentedSort semantics) for sm_103a.
//
// One call sorts every segment [begin[i], end[i]) of the keys (and values) in place of
// cub::DeviceSegmentedSort (cub/cub/device/dispatch/dispatch_segmented_sort.cuh). The work
// is split on the device, with no host round trip (the reference copies partition sizes to
// the host and synchronizes, dispatch_segmented_sort.cuh:883-895):
//   * seg_classify bins every segment into a size class and appends it to that class's
//     list (warp-aggregated atomics); large segments also get a contiguous range of tiles;
//   * warp class, size <= medium tile: a sub-warp of T lanes runs CUB's merge network for
//     that size (cub/cub/agent/agent_sub_warp_merge_sort.cuh:225-340,
//     cub/cub/block/block_merge_sort.cuh:39-160,425-520, cub/cub/thread/thread_sort.cuh:27-50)
//     with the key type's own operator<; this is what decides where NaN keys land, so it
//     is reproduced step for step;
//   * block class: one CTA sorts the segment in shared memory with stable 8-bit passes;
//   * device class: all large segments together run the onesweep machinery, one launch per
//     digit pass over every large segment's tiles, each segment with its own look-back
//     chain and digit bases (CUB sorts each large segment with a single CTA,
//     kernel_segmented_sort.cuh:430-573).
// Every class kernel is persistent (grid sized to the GPU, work taken from the lists), so
// the host never needs the class sizes.
#pragma once

#include <cuda_fp16.h>

#include "block_merge.cuh"
#include "onesweep.cuh"
#include "radix_kernels.cuh"

namespace gb300
{

__device__ __forceinline__ long long load_offset(const void* p, unsigned long long i, int wide)
{
  return wide ? static_cast<const long long*>(p)[i] : (long long) static_cast<const int*>(p)[i];
}

// Appends `item` to list[counter] with one atomic per warp and list.
__device__ __forceinline__ void warp_append(bool take, uint32_t* counter, uint32_t* list, uint32_t item)
{
  const uint32_t m = __ballot_sync(0xffffffffu, take);
  if (!take)
  {
    return;
  }
  const int lane    = threadIdx.x & 31;
  const int leader  = __ffs(m) - 1;
  uint32_t base     = 0;
  if (lane == leader)
  {
    base = atomicAdd(counter, uint32_t(__popc(m)));
  }
  base = __shfl_sync(m, base, leader);
  list[base + __popc(m & ((1u << lane) - 1u))] = item;
}

__device__ __forceinline__ void seg_classify_body(const SegClassifyParams& p)
{
  const unsigned long long stride = (unsigned long long) gridDim.x * blockDim.x;
  const unsigned long long n_round = (p.num_segments + 31) / 32 * 32; // whole warps take part in the ballots
  for (unsigned long long s = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; s < n_round; s += stride)
  {
    long long b = 0, size = 0;
    if (s < p.num_segments)
    {
      b    = load_offset(p.begin_offsets, s, p.offsets_64);
      size = load_offset(p.end_offsets, s, p.offsets_64) - b;
    }
    int cls = -1; // 0 small, 1 medium, 2 block small, 3 block large, 4 device, 5 block extra small
    if (size > 0 && (b < 0 || (unsigned long long) (b + size) > p.num_items))
    {
      atomicOr(p.status, STATUS_BAD_SEGMENT); // outside the keys: not sorted, never touched
      size = 0;
    }
    if (size > 0)
    {
      if (size <= p.medium_tile)
      {
        cls = (p.partition && size <= p.small_tile) ? 0 : 1;
      }
      else if (size <= p.block_xs_cap)
      {
        cls = 5;
      }
      else if (size <= p.block_small_cap)
      {
        cls = 2;
      }
      else if (size <= p.block_large_cap)
      {
        cls = 3;
      }
      else
      {
        cls = 4;
      }
      if (cls == 4 && size >= (1ll << 30))
      {
        atomicOr(p.status, STATUS_BAD_SEGMENT); // look-back counts hold 30 bits
        cls = -1;
      }
    }
    warp_append(cls == 0, p.counters + SEG_CTR_SMALL, p.small_list, uint32_t(s));
    warp_append(cls == 1, p.counters + SEG_CTR_MEDIUM, p.medium_list, uint32_t(s));
    warp_append(cls == 5, p.counters + SEG_CTR_BLOCK_XS, p.block_xs_list, uint32_t(s));
    warp_append(cls == 2, p.counters + SEG_CTR_BLOCK_S, p.block_s_list, uint32_t(s));
    warp_append(cls == 3, p.counters + SEG_CTR_BLOCK_L, p.block_l_list, uint32_t(s));
    uint32_t row = ~0u; // device-list index of this lane's segment, when it got one
    if (cls == 4)
    {
      const uint32_t tiles = uint32_t((size + p.device_tile - 1) / p.device_tile);
      const uint32_t idx   = atomicAdd(p.counters + SEG_CTR_DEVICE, 1u);
      const uint32_t base  = atomicAdd(p.counters + SEG_CTR_DEVICE_TILES, tiles);
      atomicAdd(reinterpret_cast<unsigned long long*>(p.counters + SEG_CTR_DEVICE_ITEMS), (unsigned long long) size);
      if (idx < p.max_device_segments && (unsigned long long) base + tiles <= p.max_tiles)
      {
        p.device_list[idx] = DeviceSegment{(unsigned long long) b, uint32_t(size), base};
        for (uint32_t t = 0; t < tiles; ++t)
        {
          p.tile_segment[base + t] = idx;
        }
        row = idx;
      }
      else
      {
        atomicOr(p.status, STATUS_SEG_CAPACITY); // overlapping segments exceed the plan
      }
    }
    // the warp clears the digit-count rows of its device segments (num_passes x 256 words
    // each, 16-byte aligned), so the per-call clearing covers only segments that exist
    uint32_t rows = __ballot_sync(0xffffffffu, row != ~0u);
    const int words = p.num_passes * RADIX_DIGITS;
    while (rows != 0u)
    {
      const int src   = __ffs(rows) - 1;
      rows &= rows - 1u;
      const uint32_t r = __shfl_sync(0xffffffffu, row, src);
      uint4* w         = reinterpret_cast<uint4*>(p.seg_counts + (size_t) r * words);
      for (int i = int(threadIdx.x & 31); i < words / 4; i += 32)
      {
        w[i] = make_uint4(0u, 0u, 0u, 0u);
      }
    }
  }
}

// ---------------------------------------------------------------------------------------
// warp class: CUB's sub-warp merge sort, T lanes x I items per segment
// ---------------------------------------------------------------------------------------
template <int BYTES>
struct signed_of;
template <>
struct signed_of<1>
{
  using type = signed char;
};
template <>
struct signed_of<2>
{
  using type = short;
};
template <>
struct signed_of<4>
{
  using type = int;
};
template <>
struct signed_of<8>
{
  using type = long long;
};

// Network kinds: 0 unsigned, 1 signed, 2 floating point (native comparisons, CUB's merge
// networks); NET_RADIX + FP mode: radix order of the digit source (see RadixNetworkCompare).
constexpr int NET_RADIX = 3;

template <int KB, int KIND>
struct NativeKey
{
  using U = typename uint_of<KB>::type;
  __device__ static bool less(U a, U b)
  {
    if constexpr (KIND == 0)
    {
      return a < b;
    }
    else if constexpr (KIND == 1)
    {
      using S = typename signed_of<KB>::type;
      return S(a) < S(b);
    }
    else if constexpr (KB == 2)
    {
      return __hlt(__ushort_as_half(a), __ushort_as_half(b));
    }
    else if constexpr (KB == 4)
    {
      return __uint_as_float(a) < __uint_as_float(b);
    }
    else
    {
      return __longlong_as_double((long long) a) < __longlong_as_double((long long) b);
    }
  }
  __device__ static bool equal(U a, U b)
  {
    if constexpr (KIND != 2)
    {
      return a == b;
    }
    else if constexpr (KB == 2)
    {
      return __heq(__ushort_as_half(a), __ushort_as_half(b));
    }
    else if constexpr (KB == 4)
    {
      return __uint_as_float(a) == __uint_as_float(b);
    }
    else
    {
      return __longlong_as_double((long long) a) == __longlong_as_double((long long) b);
    }
  }
};

template <int KB, int KIND>
struct NetworkCompare
{
  using U = typename uint_of<KB>::type;
  bool descending;
  __device__ bool operator()(U a, U b) const
  {
    return descending ? NativeKey<KB, KIND>::less(b, a) : NativeKey<KB, KIND>::less(a, b);
  }
  __device__ bool equal(U a, U b) const
  {
    return NativeKey<KB, KIND>::equal(a, b);
  }
};

// Radix order for the networks (segmented radix sort, learned buckets): keys compare by the
// bits [bit, bit + width) of their digit source, so a network sorts exactly as the radix
// passes would. FP is the key mode of digit_source.
template <int KB, int FP>
struct RadixNetworkCompare
{
  using U = typename uint_of<KB>::type;
  KeyCodec codec;
  int bit;
  U mask;
  __device__ U key(U a) const
  {
    return U(digit_source<U, FP>(encode_key<U>(a, codec)) >> bit) & mask;
  }
  __device__ bool operator()(U a, U b) const
  {
    return key(a) < key(b);
  }
  __device__ bool equal(U a, U b) const
  {
    return key(a) == key(b);
  }
};

// Bit pattern CUB loads past the end of a segment: the raw key that encodes to all ones
// (ascending) or all zeros (descending).
template <int KB, int KIND>
__device__ __forceinline__ typename uint_of<KB>::type network_oob(bool descending)
{
  using U      = typename uint_of<KB>::type;
  const U all  = U(~U(0));
  const U high = high_bit<U>();
  if constexpr (KIND == 0)
  {
    return descending ? U(0) : all;
  }
  else if constexpr (KIND == 1)
  {
    return descending ? high : U(all ^ high);
  }
  else
  {
    return descending ? all : U(all ^ high);
  }
}

template <int KB, int KIND, int VB, int T, int I>
struct NetworkSmem
{
  using U                      = typename uint_of<KB>::type;
  using V                      = typename value_word<VB>::type;
  static constexpr int TILE    = T * I;
  static constexpr int GROUPS  = 32 / T; // sub-warps per warp
  static constexpr size_t kgrp = ((sizeof(U) * (TILE + 1) + 15) / 16) * 16;
  static constexpr size_t vgrp = VB > 0 ? ((sizeof(V) * (TILE + 1) + 15) / 16) * 16 : 0;
  static constexpr size_t per_warp = GROUPS * (kgrp + vgrp);
};

// One sub-warp sorts one segment of `size` keys at `kin` into `kout` (may alias).
template <int KB, int VB, int T, int I, class Cmp>
__device__ __forceinline__ void network_sort_segment(
  const typename uint_of<KB>::type* kin,
  typename uint_of<KB>::type* kout,
  const typename value_word<VB>::type* vin,
  typename value_word<VB>::type* vout,
  int size,
  const Cmp& op,
  typename uint_of<KB>::type oob, // raw key past the end: compares after every key
  typename uint_of<KB>::type* kshared,
  typename value_word<VB>::type* vshared,
  uint32_t member_mask,
  int l) // lane within the sub-warp
{
  using U         = typename uint_of<KB>::type;
  using V         = typename value_word<VB>::type;
  constexpr int TILE = T * I;

  if (size < 3)
  {
    // short circuit: only the sub-warp's first lane works
    if (l == 0)
    {
      if (size == 1)
      {
        const U k0 = kin[0];
        V v0{};
        if constexpr (VB > 0)
        {
          v0 = vin[0];
        }
        kout[0] = k0;
        if constexpr (VB > 0)
        {
          vout[0] = v0;
        }
      }
      else
      {
        const U lhs       = kin[0];
        const U rhs       = kin[1];
        const bool keep   = op.equal(lhs, rhs) || op(lhs, rhs);
        V lv{}, rv{};
        if constexpr (VB > 0)
        {
          lv = vin[0];
          rv = vin[1];
        }
        kout[0] = keep ? lhs : rhs;
        kout[1] = keep ? rhs : lhs;
        if constexpr (VB > 0)
        {
          vout[0] = keep ? lv : rv;
          vout[1] = keep ? rv : lv;
        }
      }
    }
    return;
  }

  U keys[I];
  V vals[VB > 0 ? I : 1];
#pragma unroll
  for (int i = 0; i < I; ++i)
  {
    const int x = l * I + i;
    keys[i]     = x < size ? kin[x] : oob;
    if constexpr (VB > 0)
    {
      if (x < size)
      {
        vals[i] = vin[x];
      }
    }
  }
  // past the valid items: the lane's running maximum (its first item excluded)
  {
    U max_key = oob;
#pragma unroll
    for (int i = 1; i < I; ++i)
    {
      if (l * I + i < size)
      {
        max_key = op(max_key, keys[i]) ? keys[i] : max_key;
      }
      else
      {
        keys[i] = max_key;
      }
    }
  }
  // stable odd-even transposition sort inside the lane
  if (l * I < size)
  {
#pragma unroll
    for (int i = 0; i < I; ++i)
    {
#pragma unroll
      for (int j = 1 & i; j < I - 1; j += 2)
      {
        if (op(keys[j + 1], keys[j]))
        {
          const U t = keys[j];
          keys[j]   = keys[j + 1];
          keys[j + 1] = t;
          if constexpr (VB > 0)
          {
            const V tv  = vals[j];
            vals[j]     = vals[j + 1];
            vals[j + 1] = tv;
          }
        }
      }
    }
  }
  // merge rounds through shared memory
#pragma unroll 1
  for (int target = 2; target <= T; target *= 2)
  {
    const int merged = target / 2;
    const int mask   = target - 1;
    __syncwarp(member_mask);
#pragma unroll
    for (int i = 0; i < I; ++i)
    {
      kshared[l * I + i] = keys[i];
    }
    __syncwarp(member_mask);
    const int start  = I * (~mask & l);
    const int span   = I * merged;
    const int diag   = min(size, I * (mask & l));
    const int k1_beg = min(size, start);
    const int k1_end = min(size, k1_beg + span);
    const int k2_beg = k1_end;
    const int k2_end = min(size, k2_beg + span);
    const int n1     = k1_end - k1_beg;
    const int n2     = k2_end - k2_beg;
    int lo           = diag < n2 ? 0 : diag - n2;
    int hi           = min(diag, n1);
    while (lo < hi)
    {
      const int mid = lo + (hi - lo) / 2;
      if (op(kshared[k2_beg + diag - 1 - mid], kshared[k1_beg + mid]))
      {
        hi = mid;
      }
      else
      {
        lo = mid + 1;
      }
    }
    int b1       = k1_beg + lo;
    int b2       = k2_beg + diag - lo;
    const int e1 = k1_end;
    const int e2 = k2_end;
    U key1       = (e1 - b1) != 0 ? kshared[b1] : oob;
    U key2       = (e2 - b2) != 0 ? kshared[b2] : oob;
    int idx[I]; // may point past the valid items for outputs past them (never stored)
#pragma unroll
    for (int i = 0; i < I; ++i)
    {
      const bool p = (b2 < e2) && ((b1 >= e1) || op(key2, key1));
      keys[i]      = p ? key2 : key1;
      idx[i]       = p ? b2++ : b1++;
      if (p)
      {
        key2 = kshared[min(b2, TILE)];
      }
      else
      {
        key1 = kshared[min(b1, TILE)];
      }
    }
    if constexpr (VB > 0)
    {
      __syncwarp(member_mask);
#pragma unroll
      for (int i = 0; i < I; ++i)
      {
        vshared[l * I + i] = vals[i];
      }
      __syncwarp(member_mask);
#pragma unroll
      for (int i = 0; i < I; ++i)
      {
        vals[i] = vshared[min(idx[i], TILE)];
      }
    }
  }
  __syncwarp(member_mask);
#pragma unroll
  for (int i = 0; i < I; ++i)
  {
    const int x = l * I + i;
    if (x < size)
    {
      kout[x] = keys[i];
      if constexpr (VB > 0)
      {
        vout[x] = vals[i];
      }
    }
  }
}

// Persistent: each sub-warp takes segments from `list` until it is exhausted.
template <int KB, int KIND, int VB, int T, int I>
__device__ __forceinline__ void seg_network_body(const SegSortParams& p, const uint32_t* list, uint32_t count_index,
                                                 uint32_t ticket_index)
{
  using L      = NetworkSmem<KB, KIND, VB, T, I>;
  using U      = typename L::U;
  using V      = typename L::V;
  extern __shared__ __align__(128) unsigned char smem[];
  const int warp   = threadIdx.x >> 5;
  const int lane   = threadIdx.x & 31;
  const int group  = lane / T;
  const int l      = lane % T;
  const uint32_t member_mask = (T == 32) ? 0xffffffffu : (((1u << T) - 1u) << (group * T));
  unsigned char* wbase = smem + warp * L::per_warp;
  U* kshared           = reinterpret_cast<U*>(wbase + group * L::kgrp);
  V* vshared           = reinterpret_cast<V*>(wbase + L::GROUPS * L::kgrp + group * L::vgrp);

  const uint32_t count = p.counters[count_index];
  while (true)
  {
    // one ticket per warp covers GROUPS segments
    uint32_t first = 0;
    if (lane == 0)
    {
      first = atomicAdd(p.counters + ticket_index, uint32_t(L::GROUPS));
    }
    first = __shfl_sync(0xffffffffu, first, 0);
    if (first >= count)
    {
      break;
    }
    const uint32_t item = first + group;
    if (item < count)
    {
      const uint32_t s   = list[item];
      const long long b  = load_offset(p.begin_offsets, s, p.offsets_64);
      const int size     = int(load_offset(p.end_offsets, s, p.offsets_64) - b);
      const U* kin = static_cast<const U*>(p.keys_in) + b;
      U* kout      = static_cast<U*>(p.keys_out) + b;
      const V* vin = VB > 0 ? static_cast<const V*>(p.values_in) + b : nullptr;
      V* vout      = VB > 0 ? static_cast<V*>(p.values_out) + b : nullptr;
      if constexpr (KIND >= NET_RADIX)
      {
        // radix order: ascending in the encoded key (the order lives in the codec); the key
        // decoding from all ones sorts last
        const int width = p.end_bit - p.begin_bit;
        const RadixNetworkCompare<KB, KIND - NET_RADIX> op{
          p.codec, p.begin_bit, width >= 8 * KB ? U(~U(0)) : U((U(1) << width) - 1)};
        network_sort_segment<KB, VB, T, I>(
          kin, kout, vin, vout, size, op, decode_key<U>(U(~U(0)), p.codec), kshared, vshared, member_mask, l);
      }
      else
      {
        const NetworkCompare<KB, KIND> op{p.descending != 0};
        network_sort_segment<KB, VB, T, I>(
          kin, kout, vin, vout, size, op, network_oob<KB, KIND>(p.descending != 0), kshared, vshared, member_mask, l);
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------------------
// block class: one CTA per segment, shared-memory LSD passes
// ---------------------------------------------------------------------------------------
template <int KB, int VB, int FP, int TPB, int ITEMS, int BITS = RADIX_BITS>
__device__ __forceinline__ void seg_block_body(const SegSortParams& p, const uint32_t* list, uint32_t count_index,
                                               uint32_t ticket_index)
{
  using U = typename uint_of<KB>::type;
  using V = typename value_word<VB>::type;
  __shared__ uint32_t ticket;
  const uint32_t count = p.counters[count_index];
  while (true)
  {
    __syncthreads();
    if (threadIdx.x == 0)
    {
      ticket = atomicAdd(p.counters + ticket_index, 1u);
    }
    __syncthreads();
    const uint32_t item = ticket;
    if (item >= count)
    {
      break;
    }
    const uint32_t s  = list[item];
    const long long b = load_offset(p.begin_offsets, s, p.offsets_64);
    const uint32_t n  = uint32_t(load_offset(p.end_offsets, s, p.offsets_64) - b);
    // the merge sort orders by the whole key; a bit window takes the radix block sort
    if (seg_block_algo(KB) == SEG_BLOCK_MERGE && p.begin_bit == 0 && p.end_bit == 8 * KB)
    {
      block_merge_sort_body<KB, VB, FP, TPB, ITEMS>(static_cast<const U*>(p.keys_in) + b,
                                                    static_cast<U*>(p.keys_out) + b,
                                                    VB > 0 ? static_cast<const V*>(p.values_in) + b : nullptr,
                                                    VB > 0 ? static_cast<V*>(p.values_out) + b : nullptr,
                                                    n,
                                                    p.codec);
    }
    else
    {
      block_sort_body<KB, VB, FP, TPB, ITEMS, BITS>(static_cast<const U*>(p.keys_in) + b,
                                              static_cast<U*>(p.keys_out) + b,
                                              VB > 0 ? static_cast<const V*>(p.values_in) + b : nullptr,
                                              VB > 0 ? static_cast<V*>(p.values_out) + b : nullptr,
                                              n,
                                              p.begin_bit,
                                              p.end_bit,
                                              p.codec);
    }
  }
}

// ---------------------------------------------------------------------------------------
// device class: all large segments together
// ---------------------------------------------------------------------------------------
// Per-segment digit counts of every pass (one read of the large segments), and the
// clearing of pass 0's look-back rows.
template <int KB, int FP, int TPB>
__device__ __forceinline__ void seg_device_histogram_body(const SegDeviceParams& p)
{
  using U         = typename uint_of<KB>::type;
  constexpr int R = RADIX_DIGITS;
  __shared__ uint32_t sh[SEG_MAX_PASSES * R]; // up to 8 digits plus one split pass
  __shared__ uint32_t ticket;
  // with overlapping segments the lists may be incomplete: do no large-segment work at all
  const uint32_t ntiles = (*p.status & STATUS_SEG_CAPACITY) ? 0u : p.counters[SEG_CTR_DEVICE_TILES];
  const int tid         = threadIdx.x;
  // the whole key in 8-bit digits from bit 0 (no bit window, no split pass): digit q is byte q
  bool bytewise = p.num_passes == KB;
  for (int q = 0; q < p.num_passes; ++q)
  {
    bytewise = bytewise && p.pass_bit[q] == 8 * q && p.pass_bits[q] == 8;
  }
  // keys in flight per thread in the byte-digit loop: 32 bytes
  constexpr int LOADS = KB >= 8 ? 4 : 32 / KB > 8 ? 8 : 32 / KB;

  for (unsigned long long i = blockIdx.x * (unsigned long long) TPB + tid; i < (unsigned long long) ntiles * R;
       i += (unsigned long long) gridDim.x * TPB)
  {
    p.lookback[0][i] = 0u;
  }
  while (true)
  {
    __syncthreads();
    if (tid == 0)
    {
      ticket = atomicAdd(p.counters + SEG_CTR_TICKET_HIST, 1u);
    }
    for (int i = tid; i < p.num_passes * R; i += TPB)
    {
      sh[i] = 0;
    }
    __syncthreads();
    const uint32_t t = ticket;
    if (t >= ntiles)
    {
      break;
    }
    const uint32_t si        = p.tile_segment[t];
    const DeviceSegment seg  = p.device_list[si];
    const uint32_t local     = t - seg.tile_base;
    const uint32_t first     = local * p.device_tile;
    const uint32_t valid     = min(p.device_tile, seg.size - first);
    const U* keys            = static_cast<const U*>(p.keys_in) + seg.begin + first;
    const uint32_t sh_base   = smem_addr(sh);
    if (bytewise)
    {
      // digit q is byte q of the digit source: one byte permute and one address add per pass
      auto count_key = [&](U raw) {
        const U k         = digit_source<U, FP>(encode_key<U>(raw, p.codec));
        const uint32_t lo = uint32_t(k);
        uint32_t hi       = 0;
        if constexpr (KB == 8)
        {
          hi = uint32_t((unsigned long long) k >> 32);
        }
#pragma unroll
        for (int q = 0; q < KB; ++q)
        {
          const uint32_t d = __byte_perm(q < 4 ? lo : hi, 0u, 0x4440u | uint32_t(q & 3));
          asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(sh_base + uint32_t(q * R * 4) + 4u * d));
        }
      };
      // LOADS loads in flight per thread, the tile's ragged end included (a tile is about two
      // such batches per thread: one key at a time, its end would cost a load latency per key)
      for (uint32_t i = tid; i < valid; i += LOADS * TPB)
      {
        U k[LOADS];
#pragma unroll
        for (int j = 0; j < LOADS; ++j)
        {
          if (i + j * TPB < valid)
          {
            k[j] = __ldcs(keys + i + j * TPB);
          }
        }
#pragma unroll
        for (int j = 0; j < LOADS; ++j)
        {
          if (i + j * TPB < valid)
          {
            count_key(k[j]);
          }
        }
      }
    }
    else
    {
      auto count_key = [&](U raw) {
        const U k = encode_key<U>(raw, p.codec);
        for (int q = 0; q < p.num_passes; ++q)
        {
          const uint32_t d = extract_digit<U, FP>(k, p.pass_bit[q], (1u << p.pass_bits[q]) - 1u);
          asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(sh_base + 4u * uint32_t(q * R + int(d))));
        }
      };
      // four loads in flight per thread
      uint32_t i = tid;
      for (; i + 3u * TPB < valid; i += 4u * TPB)
      {
        U k[4];
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
          k[j] = __ldcs(keys + i + j * TPB);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
          count_key(k[j]);
        }
      }
      for (; i < valid; i += TPB)
      {
        count_key(keys[i]);
      }
    }
    __syncthreads();
    for (int i = tid; i < p.num_passes * R; i += TPB)
    {
      if (sh[i] != 0)
      {
        atomicAdd(&p.seg_counts[(size_t) si * p.num_passes * R + i], sh[i]);
      }
    }
  }
}

// Per large segment: digit bases of every pass = segment begin + exclusive digit prefix.
template <int TPB>
__device__ __forceinline__ void seg_device_scan_body(const SegDeviceParams& p)
{
  constexpr int R = RADIX_DIGITS;
  static_assert(TPB == R, "one thread per digit");
  __shared__ uint32_t scratch[8];
  __shared__ uint32_t ticket;
  const uint32_t nseg = (*p.status & STATUS_SEG_CAPACITY) ? 0u : p.counters[SEG_CTR_DEVICE];
  while (true)
  {
    __syncthreads();
    if (threadIdx.x == 0)
    {
      ticket = atomicAdd(p.counters + SEG_CTR_TICKET_SCAN, 1u);
    }
    __syncthreads();
    const uint32_t si = ticket;
    if (si >= nseg)
    {
      break;
    }
    const unsigned long long begin = p.device_list[si].begin;
    for (int q = 0; q < p.num_passes; ++q)
    {
      const size_t row = ((size_t) si * p.num_passes + q) * R;
      const uint32_t c = p.seg_counts[row + threadIdx.x];
      const uint32_t e = digit_exclusive_scan(c, scratch);
      p.seg_bins[row + threadIdx.x] = begin + e;
      named_barrier_256(); // scratch is reused by the next pass's scan
    }
  }
}

// One digit pass over all large segments: CTAs take tiles in ticket order (forward progress:
// a tile only waits on lower tiles of its own segment, already taken by running CTAs).
template <int KB, int VB, int FP, int TPB, int ITEMS>
__device__ __forceinline__ void seg_device_onesweep_body(const SegDeviceParams& dp)
{
  const int pass = dp.pass;
  using L          = OnesweepSmem<KB, VB, TPB, ITEMS>;
  using U          = typename L::U;
  using V          = typename L::V;
  constexpr int NW = L::NW;
  constexpr int R  = RADIX_DIGITS;

  extern __shared__ __align__(128) unsigned char smem[];
  uint32_t* whist   = reinterpret_cast<uint32_t*>(smem + L::whist_off);
  long long* gdelta = reinterpret_cast<long long*>(smem + L::gdelta_off);
  uint32_t* misc    = reinterpret_cast<uint32_t*>(smem + L::misc_off);
  U* kstage         = reinterpret_cast<U*>(smem + L::kstage_off);
  V* vstage         = reinterpret_cast<V*>(smem + L::vstage_off);

  const uint32_t ntiles = (*dp.status & STATUS_SEG_CAPACITY) ? 0u : dp.counters[SEG_CTR_DEVICE_TILES];
  const int tid         = threadIdx.x;
  while (true)
  {
    __syncthreads();
    if (tid == 0)
    {
      misc[0] = atomicAdd(dp.counters + SEG_CTR_TICKET_PASS0 + pass, 1u);
      misc[1] = 0u;
    }
    for (int i = tid; i < NW * R; i += TPB)
    {
      whist[i] = 0;
    }
    __syncthreads();
    const uint32_t t = misc[0];
    if (t >= ntiles)
    {
      break;
    }
    const uint32_t si       = dp.tile_segment[t];
    const DeviceSegment seg = dp.device_list[si];

    OnesweepParams p{};
    p.keys_in         = static_cast<const U*>(dp.keys_src[pass]) + seg.begin;
    p.keys_out        = dp.keys_dst[pass];
    p.values_in       = VB > 0 ? static_cast<const V*>(dp.values_src[pass]) + seg.begin : nullptr;
    p.values_out      = dp.values_dst[pass];
    p.num_items_total = dp.num_items;
    p.portion_items   = seg.size;
    p.portion_tiles   = (seg.size + dp.device_tile - 1) / dp.device_tile;
    p.tile_row_base   = seg.tile_base;
    p.lookback        = dp.lookback[pass & 1];
    p.lookback_next   = (pass + 1 < dp.num_passes) ? dp.lookback[(pass + 1) & 1] : nullptr;
    p.bins            = dp.seg_bins + ((size_t) si * dp.num_passes + pass) * R;
    p.bins_next       = nullptr;
    p.status          = dp.status;
    p.codec           = dp.codec;
    p.current_bit     = dp.pass_bit[pass];
    p.num_bits        = dp.pass_bits[pass];
    p.encode_in       = pass == 0;
    p.decode_out      = pass == dp.num_passes - 1;

    const uint32_t local      = t - seg.tile_base;
    const uint32_t tile_first = local * L::TILE;
    const uint32_t valid      = min(uint32_t(L::TILE), seg.size - tile_first);
    U keys[ITEMS];
    load_tile_keys_global<KB, TPB, ITEMS>(p, p.keys_in, p.encode_in, tile_first, valid, keys);
    onesweep_tile<KB, VB, FP, TPB, ITEMS, true>(p, local, valid, keys, whist, gdelta, misc, kstage, vstage, [&](auto& vals) {
      if constexpr (VB > 0)
      {
        load_tile_values_global<VB, TPB, ITEMS>(p.values_in, tile_first, valid, vals);
      }
    });
  }
}

} // namespace gb300

namespace gb300
{

// ---------------------------------------------------------------------------------------
// Device class, pipelined: the same digit pass over all large segments as
// seg_device_onesweep_body, in the persistent, warp-specialised form of the plain pass
// (onesweep_persistent_impl): one CTA per SM walks the global tile list blockIdx.x,
// blockIdx.x + gridDim.x, ...; 256 look-back threads walk a tile's segment chain while the
// main threads rank it, and a tile is written out one iteration later.
//
// Tiles start anywhere inside a segment, so a tile's keys (and values) rarely start on a
// 16-byte boundary: the bulk copy fetches the 16-byte-aligned range that covers them (up to
// 32 bytes more than the tile) and the tile is read from its offset inside the buffer. The
// one tile whose covering range would reach past the end of the array is read with plain
// loads. A tile's geometry (segment, index inside the segment, keys) is worked out by the
// thread that issues its copy and kept beside its buffer.
//
// Forward progress: tile t waits only on lower tiles of its own segment, which are lower
// global tiles, held by CTAs that are all resident (cooperative launch) and that take their
// tiles in increasing order.
// ---------------------------------------------------------------------------------------
template <int KB, int VB, int TPB, int ITEMS>
struct SegPersistentSmem
{
  using U                   = typename uint_of<KB>::type;
  using V                   = typename value_word<VB>::type;
  static constexpr int MT   = TPB - LOOKBACK_THREADS;
  static constexpr int NW   = MT / 32;
  static constexpr int TILE = MT * ITEMS;
  static constexpr size_t whist_off  = 0;
  static constexpr size_t gdelta_off = whist_off + sizeof(uint32_t) * NW * RADIX_DIGITS;
  static constexpr size_t misc_off   = gdelta_off + sizeof(long long) * RADIX_DIGITS;
  static constexpr size_t geo_off    = misc_off + 128; // 3 slots of SEG_GEO_WORDS words
  static constexpr size_t buf_off    = geo_off + 256;
  static constexpr size_t kbytes     = ((sizeof(U) * TILE + 15) / 16) * 16 + 32; // covering range
  static constexpr size_t vbytes     = VB > 0 ? ((sizeof(V) * TILE + 15) / 16) * 16 + 32 : 0;
  static constexpr size_t buf_bytes  = kbytes + vbytes;
  static constexpr size_t bytes      = buf_off + 3 * buf_bytes;
  static_assert(seg_persistent_smem_for(KB, VB, TPB, ITEMS) == bytes, "host and kernel layouts agree");
};

// geometry words of a tile slot
enum : int
{
  SEG_GEO_LOCAL = 0, // tile index inside its segment
  SEG_GEO_VALID,     // keys in the tile
  SEG_GEO_BASE,      // global tile index of the segment's first tile (its first look-back row)
  SEG_GEO_SEG,       // index into the device-class list
  SEG_GEO_KOFF,      // first key's element offset in the buffer (bulk-copied tiles)
  SEG_GEO_VOFF,
  SEG_GEO_BULK,      // 1: fetched by bulk copy, 0: read with plain loads
  SEG_GEO_BEGIN_LO,  // global index of the tile's first key
  SEG_GEO_BEGIN_HI,
  SEG_GEO_WORDS = 16
};

template <int KB, int VB, int FP, int TPB, int ITEMS>
__device__ __forceinline__ void seg_device_persistent_body(const SegDeviceParams& dp)
{
  using L            = SegPersistentSmem<KB, VB, TPB, ITEMS>;
  using U            = typename L::U;
  using V            = typename L::V;
  constexpr int MT   = L::MT;
  constexpr int NW   = L::NW;
  constexpr int R    = RADIX_DIGITS;
  constexpr int TILE = L::TILE;

  extern __shared__ __align__(128) unsigned char smem[];
  uint32_t* whist   = reinterpret_cast<uint32_t*>(smem + L::whist_off);
  long long* gdelta = reinterpret_cast<long long*>(smem + L::gdelta_off);
  uint32_t* misc    = reinterpret_cast<uint32_t*>(smem + L::misc_off);
  uint64_t* mbar    = reinterpret_cast<uint64_t*>(misc + 16);
  uint32_t* geo     = reinterpret_cast<uint32_t*>(smem + L::geo_off);
  auto kbuf         = [&](int b) {
    return reinterpret_cast<U*>(smem + L::buf_off + size_t(b) * L::buf_bytes);
  };
  auto vbuf = [&](int b) {
    return reinterpret_cast<V*>(smem + L::buf_off + size_t(b) * L::buf_bytes + L::kbytes);
  };

  const int tid         = threadIdx.x;
  const int pass        = dp.pass;
  const uint32_t ntiles = (*dp.status & STATUS_SEG_CAPACITY) ? 0u : dp.counters[SEG_CTR_DEVICE_TILES];
  const U* keys_src     = static_cast<const U*>(dp.keys_src[pass]);
  const V* values_src   = static_cast<const V*>(dp.values_src[pass]);
  const int bit         = dp.pass_bit[pass];
  const uint32_t dmask  = (1u << dp.pass_bits[pass]) - 1u;
  const bool encode_in  = pass == 0;
  const bool decode_out = pass == dp.num_passes - 1;
  uint32_t* lookback      = dp.lookback[pass & 1];
  uint32_t* lookback_next = (pass + 1 < dp.num_passes) ? dp.lookback[(pass + 1) & 1] : nullptr;

  // thread 0: the geometry of tile t (of segment si, seg) into slot b, and its bulk copy when
  // it can have one
  auto issue = [&](uint32_t t, uint32_t si, const DeviceSegment& seg, int b) {
    const uint32_t local    = t - seg.tile_base;
    const uint32_t first    = local * uint32_t(TILE);
    const uint32_t valid    = min(uint32_t(TILE), seg.size - first);
    const unsigned long long begin = seg.begin + first;
    uint32_t* g          = geo + b * SEG_GEO_WORDS;
    g[SEG_GEO_LOCAL]     = local;
    g[SEG_GEO_VALID]     = valid;
    g[SEG_GEO_BASE]      = seg.tile_base;
    g[SEG_GEO_SEG]       = si;
    g[SEG_GEO_BEGIN_LO]  = uint32_t(begin);
    g[SEG_GEO_BEGIN_HI]  = uint32_t(begin >> 32);
    const uintptr_t ka   = reinterpret_cast<uintptr_t>(keys_src + begin);
    const uintptr_t ka0  = ka & ~uintptr_t(15);
    const uint32_t kb    = uint32_t(((ka + uintptr_t(valid) * KB + 15) & ~uintptr_t(15)) - ka0);
    bool bulk            = ka0 + kb <= reinterpret_cast<uintptr_t>(keys_src + dp.num_items);
    uintptr_t va = 0, va0 = 0;
    uint32_t vb = 0;
    if constexpr (VB > 0)
    {
      va   = reinterpret_cast<uintptr_t>(values_src + begin);
      va0  = va & ~uintptr_t(15);
      vb   = uint32_t(((va + uintptr_t(valid) * sizeof(V) + 15) & ~uintptr_t(15)) - va0);
      bulk = bulk && va0 + vb <= reinterpret_cast<uintptr_t>(values_src + dp.num_items);
    }
    g[SEG_GEO_KOFF] = uint32_t(ka - ka0) / KB;
    g[SEG_GEO_VOFF] = VB > 0 ? uint32_t(va - va0) / uint32_t(sizeof(V)) : 0u;
    g[SEG_GEO_BULK] = bulk ? 1u : 0u;
    if (bulk)
    {
      mbar_arrive_expect_tx(&mbar[b], kb + vb);
      bulk_copy_g2s(kbuf(b), reinterpret_cast<const void*>(ka0), kb, &mbar[b]);
      if constexpr (VB > 0)
      {
        bulk_copy_g2s(vbuf(b), reinterpret_cast<const void*>(va0), vb, &mbar[b]);
      }
    }
  };

  if (tid == 0)
  {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_init(&mbar[2], 1);
    mbar_init_fence();
    misc[2] = 0u;
    if (blockIdx.x < ntiles)
    {
      const uint32_t si = dp.tile_segment[blockIdx.x];
      issue(blockIdx.x, si, dp.device_list[si], 0);
    }
  }
  for (int i = tid; i < NW * R; i += TPB)
  {
    whist[i] = 0;
  }
  __syncthreads();

  if (tid < MT)
  {
    // ================================ main threads ================================
    const int warp = tid >> 5;
    const int lane = tid & 31;
    const int wofs = warp * ITEMS * 32 + lane;
    U* kout        = static_cast<U*>(dp.keys_dst[pass]);
    V* vout        = static_cast<V*>(dp.values_dst[pass]);

    // consecutive staging slots of one digit go to consecutive outputs; every store is
    // bounds-checked against the array, so corrupted offsets cannot write outside it
    auto write_out_as = [&](int b, uint32_t valid, auto decode_tag, auto narrow_tag) {
      constexpr bool DECODE              = decltype(decode_tag)::value;
      constexpr bool NARROW              = decltype(narrow_tag)::value;
      const U* ks                        = kbuf(b);
      const V* vs                        = vbuf(b);
      const unsigned long long out_limit = misc[2] != 0u ? 0ull : dp.num_items;
      const int32_t* gdelta32            = reinterpret_cast<const int32_t*>(gdelta);
#pragma unroll
      for (int j = 0; j < ITEMS; ++j)
      {
        const uint32_t s = j * MT + tid;
        if (s < valid)
        {
          const U k        = ks[s];
          const uint32_t d = extract_digit<U, FP>(k, bit, dmask);
          const U out      = DECODE ? decode_key<U>(k, dp.codec) : k;
          if constexpr (NARROW)
          {
            const uint32_t g = uint32_t(gdelta32[2 * d] + int32_t(s));
            if (g < uint32_t(out_limit))
            {
              __stcs(kout + g, out);
              if constexpr (VB > 0)
              {
                __stcs(vout + g, vs[s]);
              }
            }
          }
          else
          {
            const long long g = gdelta[d] + (long long) s;
            if ((unsigned long long) g < out_limit)
            {
              __stcs(kout + g, out);
              if constexpr (VB > 0)
              {
                __stcs(vout + g, vs[s]);
              }
            }
          }
        }
      }
    };
    auto write_out = [&](int b, uint32_t valid) {
      const bool narrow = dp.num_items < (1ull << 31);
      if (decode_out)
      {
        if (narrow)
        {
          write_out_as(b, valid, BoolTag<true>{}, BoolTag<true>{});
        }
        else
        {
          write_out_as(b, valid, BoolTag<true>{}, BoolTag<false>{});
        }
      }
      else
      {
        if (narrow)
        {
          write_out_as(b, valid, BoolTag<false>{}, BoolTag<true>{});
        }
        else
        {
          write_out_as(b, valid, BoolTag<false>{}, BoolTag<false>{});
        }
      }
    };

    uint32_t parity     = 0; // bit b: phase parity to wait for on buffer b
    int buf             = 0;
    int prev_buf        = 0;
    uint32_t prev_valid = 0;
    bool have_prev      = false;
    // Thread 0 looks up the segment of the CTA's tile after next one iteration ahead, in two
    // steps placed where warp 0 waits anyway (tile -> segment index after BH, segment record
    // after BO): the two dependent loads then never delay the tile's histogram, and the
    // barrier behind it, the way a lookup at the bulk copy's issue would.
    uint32_t si_next = 0;
    DeviceSegment seg_next{};
    if (tid == 0 && blockIdx.x + gridDim.x < ntiles)
    {
      si_next  = dp.tile_segment[blockIdx.x + gridDim.x];
      seg_next = dp.device_list[si_next];
    }
    for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x)
    {
      const uint32_t tn  = t + gridDim.x;
      const uint32_t tnn = tn + gridDim.x; // < 2^32: tiles and grid are far below 2^31
      const int nbuf     = buf == 2 ? 0 : buf + 1;
      if (tid == 0 && tn < ntiles)
      {
        fence_proxy_async_smem(); // buffer nbuf was last accessed by the generic proxy
        issue(tn, si_next, seg_next, nbuf);
      }

      // ---- load (encode on the first pass; keys past the tile are all-ones: they rank last) ----
      const uint32_t* g     = geo + buf * SEG_GEO_WORDS;
      const uint32_t valid  = g[SEG_GEO_VALID];
      U keys[ITEMS];
      V vals[VB > 0 ? ITEMS : 1];
      if (g[SEG_GEO_BULK] != 0u)
      {
        const bool data_ok = mbar_wait(&mbar[buf], (parity >> buf) & 1u);
        parity ^= 1u << buf;
        if (!data_ok)
        {
          // the copy never completed: this CTA stores nothing from here on
          atomicOr(dp.status, STATUS_LOOKBACK_TIMEOUT);
          misc[2] = 1u;
        }
        const U* ks = kbuf(buf) + g[SEG_GEO_KOFF];
#pragma unroll
        for (int i = 0; i < ITEMS; ++i)
        {
          const uint32_t idx = uint32_t(wofs + i * 32);
          keys[i]            = idx < valid ? (encode_in ? encode_key<U>(ks[idx], dp.codec) : ks[idx]) : U(~U(0));
        }
        if constexpr (VB > 0)
        {
          const V* vs = vbuf(buf) + g[SEG_GEO_VOFF];
#pragma unroll
          for (int i = 0; i < ITEMS; ++i)
          {
            const uint32_t idx = uint32_t(wofs + i * 32);
            if (idx < valid)
            {
              vals[i] = vs[idx];
            }
          }
        }
      }
      else
      {
        const unsigned long long begin = (unsigned long long) g[SEG_GEO_BEGIN_LO] | ((unsigned long long) g[SEG_GEO_BEGIN_HI] << 32);
        const U* kin                   = keys_src + begin;
#pragma unroll
        for (int i = 0; i < ITEMS; ++i)
        {
          const uint32_t idx = uint32_t(wofs + i * 32);
          keys[i]            = idx < valid ? (encode_in ? encode_key<U>(kin[idx], dp.codec) : kin[idx]) : U(~U(0));
        }
        if constexpr (VB > 0)
        {
          const V* vin = values_src + begin;
#pragma unroll
          for (int i = 0; i < ITEMS; ++i)
          {
            const uint32_t idx = uint32_t(wofs + i * 32);
            if (idx < valid)
            {
              vals[i] = __ldcs(vin + idx);
            }
          }
        }
      }
      // a segment's last tile is partial: warps holding only padding do not count their keys
      // (their rows stay zero; the look-back threads discount only the counted padding)
      const bool live = uint32_t(warp) * uint32_t(ITEMS * 32) < valid;
      if (live)
      {
        warp_histogram<U, FP, ITEMS>(keys, whist + warp * R, bit, dmask);
      }
      if (tid == 0)
      {
        misc[4] = extract_digit<U, FP>(keys[0], bit, dmask);
      }
      asm volatile("bar.arrive 3, %0;" ::"n"(TPB) : "memory"); // BH: counts of t ready
      uint32_t si_nn = 0;
      if (tid == 0 && tnn < ntiles)
      {
        si_nn = dp.tile_segment[tnn];
      }

      // ---- the previous tile goes out while the look-back threads turn t's counts into positions ----
      if (have_prev)
      {
        asm volatile("bar.sync 5, %0;" ::"n"(TPB) : "memory"); // BG: offsets of the previous tile
        write_out(prev_buf, prev_valid);
      }
      asm volatile("bar.sync 4, %0;" ::"n"(TPB) : "memory"); // BO: positions of t in whist
      if (tid == 0 && tnn < ntiles)
      {
        si_next  = si_nn;
        seg_next = dp.device_list[si_nn];
      }

      // ---- rank t, stage it in its own buffer (every main thread read it before BO) ----
      // (padding-only warps rank their keys after every counted one, inside the tile)
      const uint32_t single = misc[3];
      uint32_t pos[ITEMS];
      if (single != 0u)
      {
#pragma unroll
        for (int i = 0; i < ITEMS; ++i)
        {
          pos[i] = uint32_t(wofs + i * 32);
        }
      }
      else
      {
        __syncwarp();
        warp_rank_stable<U, FP, ITEMS>(keys, pos, whist + warp * R, bit, dmask);
      }
      U* ks = kbuf(buf);
#pragma unroll
      for (int i = 0; i < ITEMS; ++i)
      {
        ks[pos[i]] = keys[i];
      }
      if constexpr (VB > 0)
      {
        V* vs = vbuf(buf);
#pragma unroll
        for (int i = 0; i < ITEMS; ++i)
        {
          vs[pos[i]] = vals[i];
        }
      }
      __syncwarp();
      for (int k = lane; k < R; k += 32)
      {
        whist[warp * R + k] = 0u;
      }
      asm volatile("bar.sync 6, %0;" ::"n"(MT) : "memory");
      prev_buf   = buf;
      prev_valid = valid;
      have_prev  = true;
      buf        = nbuf;
    }
    if (have_prev)
    {
      asm volatile("bar.sync 5, %0;" ::"n"(TPB) : "memory"); // BG of the last tile
      write_out(prev_buf, prev_valid);
    }
  }
  else
  {
    // ============================== look-back threads ==============================
    const int d              = tid - MT;
    const uint32_t skip_tile = gb300_fault_skip_tile; // no tile, unless a test withholds one
    int buf                  = 0;
    for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x)
    {
      asm volatile("bar.sync 3, %0;" ::"n"(TPB) : "memory"); // BH
      const uint32_t* g       = geo + buf * SEG_GEO_WORDS;
      const uint32_t valid    = g[SEG_GEO_VALID];
      const uint32_t local    = g[SEG_GEO_LOCAL];
      const uint32_t row_base = g[SEG_GEO_BASE];
      const uint32_t si       = g[SEG_GEO_SEG];
      buf                     = buf == 2 ? 0 : buf + 1;
      // the segment's digit offset, loaded now: its latency hides behind the tile's digit
      // scan and look-back instead of delaying the offsets the main threads wait for
      const unsigned long long seg_base = dp.seg_bins[((size_t) si * dp.num_passes + pass) * R + d];
      uint32_t start;
      const uint32_t total = block_digit_offsets<NW>(whist, misc + 8, &start, d);
      if (uint32_t(d) == misc[4])
      {
        // every real key of the tile has the first key's digit (the counted padding keys, digit
        // dmask, are discounted: the padding of the live warps, whole warps of 32 x ITEMS slots)
        constexpr uint32_t WS  = uint32_t(ITEMS * 32);
        const uint32_t counted = min(uint32_t(TILE), (valid + WS - 1) / WS * WS);
        const uint32_t real    = total - (uint32_t(d) == dmask ? counted - valid : 0u);
        misc[3]             = real == valid ? (1u | (uint32_t(d) << 8)) : 0u;
      }
      uint32_t* col      = lookback + (size_t) row_base * R + d; // this segment's chain, digit d
      const bool publish = t != skip_tile;
      if (publish)
      {
        store_status(col + (size_t) local * R, (local == 0 ? LB_INCLUSIVE : LB_PARTIAL) | total);
      }
      asm volatile("bar.sync 4, %0;" ::"n"(TPB) : "memory"); // BO

      uint32_t excl = 0;
      if (local > 0)
      {
        bool failed = false;
        bool done   = false;
        for (int j = int(local) - 1; !done; j -= PERSISTENT_LOOKBACK_BATCH)
        {
          uint32_t w[PERSISTENT_LOOKBACK_BATCH];
#pragma unroll
          for (int k = 0; k < PERSISTENT_LOOKBACK_BATCH; ++k)
          {
            w[k] = (j - k >= 0) ? load_status(col + (size_t) (j - k) * R) : LB_INCLUSIVE;
          }
#pragma unroll
          for (int k = 0; k < PERSISTENT_LOOKBACK_BATCH; ++k)
          {
            if (!done)
            {
              uint32_t v = w[k];
              if ((v & LB_FLAGS) == LB_EMPTY)
              {
                v = wait_status(col + (size_t) (j - k) * R);
              }
              const uint32_t f = v & LB_FLAGS;
              if (f == LB_ERROR)
              {
                failed = true;
                done   = true;
              }
              else
              {
                excl += v & LB_VALUE;
                done = (f == LB_INCLUSIVE);
              }
            }
          }
        }
        if (publish)
        {
          store_status(col + (size_t) local * R, failed ? LB_ERROR : (LB_INCLUSIVE | (excl + total)));
        }
        if (failed)
        {
          atomicOr(dp.status, STATUS_LOOKBACK_TIMEOUT);
          misc[2] = 1u;
        }
      }
      if (lookback_next != nullptr)
      {
        lookback_next[(size_t) t * R + d] = 0u;
      }
      const unsigned long long base = seg_base + excl;
      gdelta[d]                     = (long long) base - (long long) start;
      asm volatile("bar.arrive 5, %0;" ::"n"(TPB) : "memory"); // BG
    }
  }
}

} // namespace gb300
