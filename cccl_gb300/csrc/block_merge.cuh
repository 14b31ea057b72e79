// Block-wide stable merge sort of one segment of up to TPB * ITEMS keys in shared memory:
// the segmented sort's block classes (and so the learned sort's bucket sort) use it.
//
// The order is the radix sort's: keys compare as their digit source (the encoded, order-
// applied key with -0.0 folded into +0.0) as unsigned integers, and ties keep input order,
// so the result is bit for bit the stable LSD radix sort's (cub/cub/block/block_radix_sort.cuh
// is what the reference's block classes run; cub/cub/block/block_merge_sort.cuh:107-470 is the
// reference's own block merge sort, the same Merge Path steps). Unlike a radix pass, whose
// cost grows with the key width, a merge level costs a few instructions per key whatever the
// width, so 8-byte keys sort in about the time of 4-byte ones.
//
//   1. the segment is loaded coalesced; each key becomes (digit source, 16-bit input index);
//      padding slots get the largest digit source and rank after every real key;
//   2. each thread sorts its ITEMS consecutive pairs in registers (odd-even transposition,
//      stable);
//   3. runs of ITEMS, 2*ITEMS, ... are merged pairwise: each thread finds its split of the
//      two runs by a Merge Path binary search and merges ITEMS outputs serially; merging
//      stops once a run covers every real key;
//   4. keys and values are gathered from the input by index (the input may alias the output:
//      all gathers of an array complete before its first store).
#pragma once

#include "sort_common.cuh"

namespace gb300
{

// Shared arrays are indexed through kpad/ipad: one spare slot per 32 (4-byte keys) or 16
// (8-byte keys, 16-bit indices: per 64) entries, so a warp reading ITEMS-strided slots
// spreads over the banks.
template <int KB>
__device__ __forceinline__ uint32_t kpad(uint32_t x)
{
  return x + (x >> (KB == 8 ? 4 : 5));
}
__device__ __forceinline__ uint32_t ipad(uint32_t x)
{
  return x + 2 * (x >> 6);
}

template <int KB, int TPB, int ITEMS>
struct BlockMergeSmem
{
  using U                   = typename uint_of<KB>::type;
  static constexpr int TILE = TPB * ITEMS;
  static constexpr size_t kslots   = size_t(TILE) + TILE / (KB == 8 ? 16 : 32) + 1;
  static constexpr size_t islots   = size_t(TILE) + 2 * (TILE / 64) + 2;
  static constexpr size_t kbuf_off = 0;
  static constexpr size_t ibuf_off = ((sizeof(U) * kslots + 15) / 16) * 16;
  static constexpr size_t bytes    = ibuf_off + ((2 * islots + 15) / 16) * 16;
};

template <int KB, int VB, int FP, int TPB, int ITEMS>
__device__ __forceinline__ void block_merge_sort_body(
  const void* keys_in, void* keys_out, const void* values_in, void* values_out, uint32_t num_items, const KeyCodec& codec)
{
  using L            = BlockMergeSmem<KB, TPB, ITEMS>;
  using U            = typename L::U;
  using V            = typename value_word<VB>::type;
  constexpr int TILE = L::TILE;
  static_assert((ITEMS & (ITEMS - 1)) == 0 && (TPB & (TPB - 1)) == 0, "power-of-two runs");
  static_assert(TILE <= 65536, "16-bit source indices");

  extern __shared__ __align__(128) unsigned char smem[];
  U* kbuf        = reinterpret_cast<U*>(smem + L::kbuf_off);
  uint16_t* ibuf = reinterpret_cast<uint16_t*>(smem + L::ibuf_off);

  const int tid    = threadIdx.x;
  const uint32_t n = num_items;
  const U* kin     = static_cast<const U*>(keys_in);
  const U PAD      = U(~U(0));

  __syncthreads(); // the previous segment of a persistent CTA is done with shared memory
  for (uint32_t s = tid; s < uint32_t(TILE); s += TPB)
  {
    kbuf[kpad<KB>(s)] = s < n ? digit_source<U, FP>(encode_key<U>(kin[s], codec)) : PAD;
  }
  __syncthreads();

  // 2. per-thread stable sort of ITEMS consecutive pairs
  const uint32_t first = uint32_t(tid) * ITEMS;
  U k[ITEMS];
  uint32_t ix[ITEMS];
#pragma unroll
  for (int i = 0; i < ITEMS; ++i)
  {
    k[i]  = kbuf[kpad<KB>(first + i)];
    ix[i] = first + i;
  }
  if (first < n)
  {
#pragma unroll
    for (int r = 0; r < ITEMS; ++r)
    {
#pragma unroll
      for (int j = r & 1; j + 1 < ITEMS; j += 2)
      {
        if (k[j + 1] < k[j])
        {
          const U tk      = k[j];
          k[j]            = k[j + 1];
          k[j + 1]        = tk;
          const uint32_t ti = ix[j];
          ix[j]           = ix[j + 1];
          ix[j + 1]       = ti;
        }
      }
    }
  }

  // 3. merge levels
  for (uint32_t w = ITEMS; w < n; w *= 2)
  {
    __syncthreads(); // previous level's reads are done
#pragma unroll
    for (int i = 0; i < ITEMS; ++i)
    {
      kbuf[kpad<KB>(first + i)] = k[i];
      ibuf[ipad(first + i)]      = uint16_t(ix[i]);
    }
    __syncthreads();
    const uint32_t start = first & ~(2 * w - 1);
    if (start < n) // groups made only of padding stay as they are
    {
      const uint32_t a0   = start;
      const uint32_t b0   = start + w;
      const uint32_t diag = first - start;
      // Merge Path: number of run-A keys among the first diag outputs (A first on ties)
      uint32_t lo = diag > w ? diag - w : 0;
      uint32_t hi = diag < w ? diag : w;
      while (lo < hi)
      {
        const uint32_t mid = (lo + hi) >> 1;
        if (kbuf[kpad<KB>(b0 + diag - 1 - mid)] < kbuf[kpad<KB>(a0 + mid)])
        {
          hi = mid;
        }
        else
        {
          lo = mid + 1;
        }
      }
      uint32_t ia          = a0 + lo;
      uint32_t ib          = b0 + (diag - lo);
      const uint32_t a_end = a0 + w;
      const uint32_t b_end = b0 + w;
      U ka                 = ia < a_end ? kbuf[kpad<KB>(ia)] : PAD;
      U kb                 = ib < b_end ? kbuf[kpad<KB>(ib)] : PAD;
#pragma unroll
      for (int i = 0; i < ITEMS; ++i)
      {
        const bool take_b = ib < b_end && (ia >= a_end || kb < ka);
        if (take_b)
        {
          k[i]  = kb;
          ix[i] = ibuf[ipad(ib)];
          ++ib;
          kb = ib < b_end ? kbuf[kpad<KB>(ib)] : PAD;
        }
        else
        {
          k[i]  = ka;
          ix[i] = ibuf[ipad(ia)];
          ++ia;
          ka = ia < a_end ? kbuf[kpad<KB>(ia)] : PAD;
        }
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < ITEMS; ++i)
  {
    ibuf[ipad(first + i)] = uint16_t(ix[i]);
  }
  __syncthreads();

  // 4. gather by index; the input may alias the output, so every read of an array ends
  // (barrier) before the first store to it. Keys, then values: half the registers.
  constexpr int PER = (TILE + TPB - 1) / TPB;
  {
    U kt[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j)
    {
      const uint32_t s = j * TPB + tid;
      if (s < n)
      {
        kt[j] = kin[ibuf[ipad(s)]];
      }
    }
    __syncthreads();
    U* kout = static_cast<U*>(keys_out);
#pragma unroll
    for (int j = 0; j < PER; ++j)
    {
      const uint32_t s = j * TPB + tid;
      if (s < n)
      {
        kout[s] = kt[j];
      }
    }
  }
  if constexpr (VB > 0)
  {
    V vt[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j)
    {
      const uint32_t s = j * TPB + tid;
      if (s < n)
      {
        vt[j] = static_cast<const V*>(values_in)[ibuf[ipad(s)]];
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PER; ++j)
    {
      const uint32_t s = j * TPB + tid;
      if (s < n)
      {
        static_cast<V*>(values_out)[s] = vt[j];
      }
    }
  }
}

} // namespace gb300
