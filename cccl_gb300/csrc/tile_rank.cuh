// In-tile digit ranking primitives shared by the onesweep pass and the single-tile sort.
//
// A tile is split into warp segments; in round i lane l of warp w holds the key at
// segment index i*32 + l, so (warp, round, lane) order is source order. Ranking is done
// in three steps (the structure of CUB's BlockRadixRankMatchEarlyCounts,
// cub/cub/block/block_radix_rank.cuh:913-1213, with GB300-specific matching):
//   1. warp_histogram: per-warp digit counts with shared-memory atomics (order-free);
//   2. block_digit_offsets: per-digit totals, an exclusive scan over warps and over
//      digits, leaving in whist[w][d] the tile position where warp w's first digit-d key goes;
//   3. warp_rank_stable: the stable rank of every key among the warp's same-digit keys.
//
// Matching on GB300: match.any.sync executes at about one instruction per 64 cycles per SM
// (measured), so peers are found with one warp ballot per digit bit instead (the
// technique CUB's warp_matcher_t also uses, cub/cub/util_ptx.cuh:407-446), and the
// warp's running digit offset is advanced by the highest peer lane with one shared
// atomic whose result is broadcast with a shuffle.
#pragma once

#include "sort_common.cuh"

namespace gb300
{

__device__ __forceinline__ void named_barrier_256()
{
  asm volatile("bar.sync 1, 256;" ::: "memory");
}

__device__ __forceinline__ uint32_t lanemask_le()
{
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_le;" : "=r"(m));
  return m;
}

// Exclusive prefix over the R digit slots held by one group of R threads (R / 32 whole
// warps; thread d holds digit d's value; R = 256 for 8-bit digits). `scratch` holds 8 words.
// Must be called by exactly that group, and by no other thread of the CTA at the same time
// (named barrier 1).
template <int R = RADIX_DIGITS>
__device__ __forceinline__ uint32_t digit_exclusive_scan(uint32_t v, uint32_t* scratch, int d = threadIdx.x)
{
  static_assert(R % 32 == 0 && R <= 256, "whole warps, at most 8");
  const int lane = d & 31;
  const int w    = d >> 5;
  uint32_t x     = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o)
    {
      x += y;
    }
  }
  if (lane == 31)
  {
    scratch[w] = x;
  }
  asm volatile("bar.sync 1, %0;" ::"n"(R) : "memory");
  uint32_t pre = 0;
#pragma unroll
  for (int j = 0; j < R / 32; ++j)
  {
    pre += (j < w) ? scratch[j] : 0u;
  }
  return pre + x - v;
}

// Lanes whose 8-bit digit equals this lane's: one ballot per bit. Written in PTX so each
// bit costs a bit test into a predicate, the vote, a predicated inversion and an AND
// (measured 1.6x faster on GB300 than the select-based C++ form).
template <int BITS = RADIX_BITS>
__device__ __forceinline__ uint32_t warp_match_digit(uint32_t d)
{
  uint32_t peers = 0xffffffffu;
#pragma unroll
  for (int b = 0; b < BITS; ++b)
  {
    uint32_t bal;
    asm("{\n"
        "  .reg .pred p;\n"
        "  .reg .b32 t;\n"
        "  and.b32 t, %1, %2;\n"
        "  setp.ne.u32 p, t, 0;\n"
        "  vote.ballot.sync.b32 %0, p, 0xffffffff;\n"
        "  @!p not.b32 %0, %0;\n"
        "}\n"
        : "=r"(bal)
        : "r"(d), "r"(1u << b));
    peers &= bal;
  }
  return peers;
}

template <class U, int FP, int ITEMS>
__device__ __forceinline__ void warp_histogram(const U (&keys)[ITEMS], uint32_t* whist_w, int bit, uint32_t dmask)
{
#pragma unroll
  for (int i = 0; i < ITEMS; ++i)
  {
    atomicAdd(&whist_w[extract_digit<U, FP>(keys[i], bit, dmask)], 1u);
  }
}

// One group of R threads (thread d, digit d; R = 256 for 8-bit digits): turns per-warp
// counts whist[w][d] (rows of R) into tile positions (exclusive over digits, then over
// warps). Returns this thread's digit total; *tile_start receives the digit's first position
// in the tile.
template <int NW, int R = RADIX_DIGITS>
__device__ __forceinline__ uint32_t
block_digit_offsets(uint32_t* whist, uint32_t* scratch8, uint32_t* tile_start, int d = threadIdx.x)
{
  uint32_t total = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w)
  {
    const uint32_t c = whist[w * R + d];
    whist[w * R + d] = total;
    total += c;
  }
  const uint32_t start = digit_exclusive_scan<R>(total, scratch8, d);
#pragma unroll
  for (int w = 0; w < NW; ++w)
  {
    whist[w * R + d] += start;
  }
  *tile_start = start;
  return total;
}

// Stable tile positions: pos[i] = whist_w[d] at the time key i is reached, in source order.
// Digits have BITS bits (8 in the digit passes).
template <class U, int FP, int ITEMS, int BITS = RADIX_BITS>
__device__ __forceinline__ void warp_rank_stable(
  const U (&keys)[ITEMS], uint32_t (&pos)[ITEMS], uint32_t* whist_w, int bit, uint32_t dmask)
{
  const int lane    = threadIdx.x & 31;
  const uint32_t le = lanemask_le();
#pragma unroll
  for (int i = 0; i < ITEMS; ++i)
  {
    const uint32_t d      = extract_digit<U, FP>(keys[i], bit, dmask);
    const uint32_t peers  = warp_match_digit<BITS>(d);
    const int leader      = 31 - __clz(peers);
    const uint32_t cnt_le = __popc(peers & le);
    uint32_t base         = 0;
    if (lane == leader)
    {
      base = atomicAdd(&whist_w[d], cnt_le); // cnt_le of the highest peer = the peer count
    }
    // The shuffle completes only after the leader's atomic returned, so the next round's
    // atomics on the same counter are ordered after this one.
    base   = __shfl_sync(0xffffffffu, base, leader);
    pos[i] = base + cnt_le - 1;
  }
}

// Stable tile positions with the peer lanes found through shared memory instead of ballots:
// every lane ORs its lane bit into tbl_w[digit] (one word per digit for the warp), the warp
// re-reads its word to get the lanes sharing its digit, and the highest of them advances the
// digit's running offset and clears the word again. Three shared-memory operations per key
// in place of eight ballots: the ballots run on the integer ALU pipe, which the ballot form
// keeps saturated, these on the load/store pipe. tbl_w (256 words) must be zero on entry and
// is zero again on return. ALT = true ranks every other item (odd i) this way and the rest by
// ballots, splitting the work between the two pipes.
template <class U, int FP, int ITEMS, bool ALT, int FIRST = 0>
__device__ __forceinline__ void warp_rank_stable_table(
  const U (&keys)[ITEMS], uint32_t (&pos)[ITEMS], uint32_t* whist_w, uint32_t* tbl_w, int bit, uint32_t dmask)
{
  const int lane    = threadIdx.x & 31;
  const uint32_t le = lanemask_le();
  const uint32_t me = 1u << lane;
#pragma unroll
  for (int i = FIRST; i < ITEMS; ++i)
  {
    const uint32_t d = extract_digit<U, FP>(keys[i], bit, dmask);
    uint32_t peers;
    if (ALT && (i & 1) == 0)
    {
      peers = warp_match_digit(d);
    }
    else
    {
      volatile uint32_t* slot = tbl_w + d;
      atomicOr(const_cast<uint32_t*>(slot), me);
      __syncwarp();
      peers = *slot;
      __syncwarp(); // every lane has read its word before a leader clears it
    }
    const int leader      = 31 - __clz(peers);
    const uint32_t cnt_le = __popc(peers & le);
    uint32_t base         = 0;
    if (lane == leader)
    {
      base = atomicAdd(&whist_w[d], cnt_le);
      if (!(ALT && (i & 1) == 0))
      {
        tbl_w[d] = 0u;
      }
    }
    base   = __shfl_sync(0xffffffffu, base, leader);
    pos[i] = base + cnt_le - 1;
  }
  __syncwarp(); // the clears are visible before the table is reused
}

// Ranking that picks its form per warp: item 0 is ranked by ballots, and when no lane of it
// has four or more peers (digits spread out, the common case of high-entropy keys) the
// remaining items alternate between ballots and the lane-mask table; otherwise (many equal
// digits, where the table's same-address ORs serialise) they all use ballots.
template <class U, int FP, int ITEMS>
__device__ __forceinline__ void warp_rank_stable_adaptive(
  const U (&keys)[ITEMS], uint32_t (&pos)[ITEMS], uint32_t* whist_w, uint32_t* tbl_w, int bit, uint32_t dmask)
{
  const int lane    = threadIdx.x & 31;
  const uint32_t le = lanemask_le();
  bool spread;
  {
    const uint32_t d      = extract_digit<U, FP>(keys[0], bit, dmask);
    const uint32_t peers  = warp_match_digit(d);
    const int leader      = 31 - __clz(peers);
    const uint32_t cnt_le = __popc(peers & le);
    uint32_t base         = 0;
    if (lane == leader)
    {
      base = atomicAdd(&whist_w[d], cnt_le);
    }
    base   = __shfl_sync(0xffffffffu, base, leader);
    pos[0] = base + cnt_le - 1;
    spread = !__any_sync(0xffffffffu, __popc(peers) >= 4);
  }
  if (spread)
  {
    // item 1 onward: odd items by the table, even ones by ballots
    warp_rank_stable_table<U, FP, ITEMS, true, 1>(keys, pos, whist_w, tbl_w, bit, dmask);
  }
  else
  {
#pragma unroll
    for (int i = 1; i < ITEMS; ++i)
    {
      const uint32_t d      = extract_digit<U, FP>(keys[i], bit, dmask);
      const uint32_t peers  = warp_match_digit(d);
      const int leader      = 31 - __clz(peers);
      const uint32_t cnt_le = __popc(peers & le);
      uint32_t base         = 0;
      if (lane == leader)
      {
        base = atomicAdd(&whist_w[d], cnt_le);
      }
      base   = __shfl_sync(0xffffffffu, base, leader);
      pos[i] = base + cnt_le - 1;
    }
  }
}

// The same two steps for digits computed by the caller (dig[i] < 256), used by passes
// whose digit is not a bit field of the key.
template <int ITEMS>
__device__ __forceinline__ void warp_histogram_digits(const uint32_t (&dig)[ITEMS], uint32_t* whist_w)
{
#pragma unroll
  for (int i = 0; i < ITEMS; ++i)
  {
    atomicAdd(&whist_w[dig[i]], 1u);
  }
}

template <int ITEMS>
__device__ __forceinline__ void
warp_rank_stable_digits(const uint32_t (&dig)[ITEMS], uint32_t (&pos)[ITEMS], uint32_t* whist_w)
{
  const int lane    = threadIdx.x & 31;
  const uint32_t le = lanemask_le();
#pragma unroll
  for (int i = 0; i < ITEMS; ++i)
  {
    const uint32_t d      = dig[i];
    const uint32_t peers  = warp_match_digit(d);
    const int leader      = 31 - __clz(peers);
    const uint32_t cnt_le = __popc(peers & le);
    uint32_t base         = 0;
    if (lane == leader)
    {
      base = atomicAdd(&whist_w[d], cnt_le);
    }
    base   = __shfl_sync(0xffffffffu, base, leader);
    pos[i] = base + cnt_le - 1;
  }
}

// Order-free tile positions (same digit buckets, arbitrary order inside a bucket).
template <class U, int FP, int ITEMS>
__device__ __forceinline__ void warp_rank_unstable(
  const U (&keys)[ITEMS], uint32_t (&pos)[ITEMS], uint32_t* whist_w, int bit, uint32_t dmask)
{
#pragma unroll
  for (int i = 0; i < ITEMS; ++i)
  {
    pos[i] = atomicAdd(&whist_w[extract_digit<U, FP>(keys[i], bit, dmask)], 1u);
  }
}

// Order-free tile positions for a tile whose keys at segment indexes >= valid are padding:
// real keys take their digit's slots, padding keys the slots [valid, TILE) at their own
// index. Padding keys carry the largest digit and come last in source order, so the
// real keys of that digit fill exactly its slots below `valid`.
template <class U, int FP, int ITEMS>
__device__ __forceinline__ void warp_rank_unstable_tail(
  const U (&keys)[ITEMS], uint32_t (&pos)[ITEMS], uint32_t* whist_w, int bit, uint32_t dmask, int wofs, uint32_t valid)
{
#pragma unroll
  for (int i = 0; i < ITEMS; ++i)
  {
    const uint32_t idx = uint32_t(wofs + i * 32);
    pos[i] = idx < valid ? atomicAdd(&whist_w[extract_digit<U, FP>(keys[i], bit, dmask)], 1u) : idx;
  }
}

} // namespace gb300
