// Onesweep digit pass: one stable 8-bit counting-sort pass over one portion of the keys
// (reference roles: cub/cub/agent/agent_radix_sort_onesweep.cuh:152-739 and
// cub/cub/device/dispatch/kernels/kernel_radix_sort.cuh:498-558).
//
// Per tile:
//   1. the tile's keys (and values) are in registers, keys encoded; digits are counted
//      per warp with shared-memory atomics;
//   2. threads [0,256) turn the counts into tile positions and publish the tile's digit
//      counts to the look-back array before any ranking ("early counts"), then walk the
//      look-back array (one digit each, LOOKBACK_BATCH predecessor rows per step) while
//      the other warps already rank their keys;
//   3. every warp ranks its keys stably and scatters them into a digit-sorted staging
//      tile in shared memory;
//   4. the staging tile is written out in order, so each digit's run lands contiguously;
//      values follow the same permutation.
//
// Two kernels run these steps:
//   * onesweep_persistent_body: the main path. One CTA per SM, launched cooperatively, walks
//     tiles blockIdx.x, blockIdx.x + gridDim.x, ...; the next tile's keys and values are
//     fetched into shared memory by a bulk async copy (cp.async.bulk + mbarrier) while the
//     current tile is ranked, so HBM latency is off the critical path. Its threads are
//     split: 256 look-back threads run step 2 while the others rank, and a tile is written
//     out one iteration after it was ranked, so the look-back latency is hidden as well;
//   * onesweep_body (onesweep_tile): CTA-per-tile with dynamic tile ids and plain
//     warp-striped loads; used when the caller's buffers are not 16-byte aligned, and by
//     the segmented sort's device-class pass.
#pragma once

#include "sort_policy.h"
#include "tile_rank.cuh"

namespace gb300
{

template <int KB, int VB, int TPB, int ITEMS>
struct OnesweepSmem
{
  using U                   = typename uint_of<KB>::type;
  using V                   = typename value_word<VB>::type;
  static constexpr int NW   = TPB / 32;
  static constexpr int TILE = TPB * ITEMS;
  static constexpr size_t whist_off  = 0;                                               // [NW][256] u32
  static constexpr size_t gdelta_off = whist_off + sizeof(uint32_t) * NW * RADIX_DIGITS; // [256] i64
  static constexpr size_t misc_off   = gdelta_off + sizeof(long long) * RADIX_DIGITS;   // 128 B
  static constexpr size_t kstage_off = misc_off + 128;
  static constexpr size_t vstage_off = kstage_off + ((sizeof(U) * TILE + 15) / 16) * 16;
  static constexpr size_t bytes      = vstage_off + (VB > 0 ? sizeof(V) * TILE : 0);
};
// misc words: [0] tile id, [1] tile failed (stores disabled), [2] sticky failure of the
// CTA, [3] single-digit tile flag and digit, [8..15] scan scratch, [16..19] two mbarriers
// (persistent kernel).

// Where a pass takes its digits from.
//   RadixDigits: bits [current_bit, current_bit + num_bits) of the encoded key, recomputed
//     wherever needed (histogram, ranking, write-out);
//   ComputedDigits: one digit per key supplied by the caller (a digit that is not a bit
//     field of the key, e.g. a model's bucket id). Padding keys of a partial tile must get
//     digit 255. The digits are staged next to the keys so the write-out reads them back.
struct RadixDigits
{
  static constexpr bool computed = false;
};

template <int ITEMS>
struct ComputedDigits
{
  static constexpr bool computed = true;
  uint32_t d[ITEMS];
  uint8_t* stage; // [TILE] digit of every staging slot
};

// Buffers and encode/decode flags a pass runs with: the launch's, or the ones its pass plan
// gives (see PLAN_* in sort_params.h).
struct PassIO
{
  const void* keys_in; // portion-relative
  void* keys_out;
  const void* values_in;
  void* values_out;
  int encode_in;
  int decode_out;
};

// Resolves the pass's buffers. Returns false when the pass does nothing: gated off, or
// skipped by its plan (its digit is the same for every key), in which case the grid first
// clears this portion's rows of the next pass's look-back buffer, as the pass would have,
// unless the previous pass was skipped too. Passes q and q + 2 share a look-back buffer, so
// after a skipped pass q - 1 the buffer of pass q + 1 is the one pass q - 1 found clean and
// left untouched: the first pass's buffer is cleared by the histogram, the second's by the
// first pass (run or skipped), and a pass that runs clears its successor's as it goes.
template <int KB, int VB>
__device__ __forceinline__ bool resolve_pass(const OnesweepParams& p, PassIO& io)
{
  if (!gate_open(p.gate))
  {
    return false;
  }
  io = PassIO{p.keys_in, p.keys_out, p.values_in, p.values_out, p.encode_in, p.decode_out};
  if (p.plan == nullptr)
  {
    return true;
  }
  const uint32_t w = __ldcg(p.plan);
  if (w & PLAN_SKIP)
  {
    const bool prev_skipped = p.plan_prev != nullptr && (__ldcg(p.plan_prev) & PLAN_SKIP) != 0u;
    if (p.lookback_next != nullptr && !prev_skipped)
    {
      uint32_t* rows                    = p.lookback_next + (size_t) p.tile_row_base * RADIX_DIGITS;
      const unsigned long long words    = (unsigned long long) p.portion_tiles * RADIX_DIGITS;
      const unsigned long long nthreads = (unsigned long long) gridDim.x * blockDim.x;
      for (unsigned long long i = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; i < words; i += nthreads)
      {
        rows[i] = 0u;
      }
    }
    return false;
  }
  const int si = int(w >> PLAN_SRC_SHIFT) & 3;
  const int di = int(w >> PLAN_DST_SHIFT) & 3;
  io.keys_in   = static_cast<const unsigned char*>(p.key_bufs[si]) + p.portion_begin * KB;
  io.keys_out  = const_cast<void*>(p.key_bufs[di]);
  if constexpr (VB > 0)
  {
    io.values_in  = static_cast<const unsigned char*>(p.value_bufs[si]) + p.portion_begin * VB;
    io.values_out = const_cast<void*>(p.value_bufs[di]);
  }
  io.encode_in  = (w & PLAN_ENCODE) != 0u;
  io.decode_out = (w & PLAN_DECODE) != 0u;
  return true;
}

// The same for a kernel that passes its own copy q of the parameters to the pass body.
template <int KB, int VB>
__device__ __forceinline__ bool apply_pass_plan(OnesweepParams& q)
{
  PassIO io;
  if (!resolve_pass<KB, VB>(q, io))
  {
    return false;
  }
  q.keys_in    = io.keys_in;
  q.keys_out   = io.keys_out;
  q.values_in  = io.values_in;
  q.values_out = io.values_out;
  q.encode_in  = io.encode_in;
  q.decode_out = io.decode_out;
  return true;
}

// Decoupled look-back of digit d for `tile` (tile > 0): the sum of the predecessors'
// counts back to the nearest inclusive prefix. BATCH predecessor rows are read per step (one
// L2 round trip): inclusive prefixes spread from tile to tile at about BATCH tiles per round
// trip, which bounds the pass's tile rate when every CTA waits for its walk. `failed` is set
// when a predecessor reported an error or never published (bounded wait).
template <int BATCH = LOOKBACK_BATCH>
__device__ __forceinline__ uint32_t lookback_walk(const OnesweepParams& p, uint32_t tile, int d, bool& failed)
{
  const uint32_t* col = p.lookback + (size_t) p.tile_row_base * RADIX_DIGITS + d;
  uint32_t excl       = 0;
  bool done           = false;
  failed              = false;
  for (int j = int(tile) - 1; !done; j -= BATCH)
  {
    uint32_t w[BATCH];
#pragma unroll
    for (int k = 0; k < BATCH; ++k)
    {
      w[k] = (j - k >= 0) ? load_status(col + (size_t) (j - k) * RADIX_DIGITS) : LB_INCLUSIVE;
    }
#pragma unroll
    for (int k = 0; k < BATCH; ++k)
    {
      if (!done)
      {
        uint32_t v = w[k];
        if ((v & LB_FLAGS) == LB_EMPTY)
        {
          v = wait_status(col + (size_t) (j - k) * RADIX_DIGITS);
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
  return excl;
}

// Per-tile steps 1-4. Preconditions: whist is zero, keys[] hold the tile's encoded keys
// (padding keys of a partial tile are all-ones), misc[1] says whether stores are
// disabled. load_values(vals) is called once after the ranking to fill the values.
template <int KB, int VB, int FP, int TPB, int ITEMS, bool STABLE, class LoadValues, class Digits = RadixDigits>
__device__ __forceinline__ void onesweep_tile(
  const OnesweepParams& p,
  const uint32_t tile,
  const uint32_t valid,
  typename uint_of<KB>::type (&keys)[ITEMS],
  uint32_t* whist,
  long long* gdelta,
  uint32_t* misc,
  typename uint_of<KB>::type* kstage,
  typename value_word<VB>::type* vstage,
  LoadValues&& load_values,
  const Digits& dg = Digits{})
{
  using U            = typename uint_of<KB>::type;
  using V            = typename value_word<VB>::type;
  constexpr int NW   = TPB / 32;
  constexpr int TILE = TPB * ITEMS;
  constexpr int R    = RADIX_DIGITS;
  static_assert(TPB >= R, "the digit-parallel phases need one thread per digit");
  static_assert(STABLE || VB == 0, "pairs need a stable pass");
  static_assert(STABLE || !Digits::computed, "computed digits are ranked stably");

  const int tid        = threadIdx.x;
  const int warp       = tid >> 5;
  const bool full      = valid == uint32_t(TILE);
  const int bit        = p.current_bit;
  const uint32_t dmask = (1u << p.num_bits) - 1u;

  if constexpr (Digits::computed)
  {
    warp_histogram_digits<ITEMS>(dg.d, whist + warp * R);
  }
  else
  {
    warp_histogram<U, FP, ITEMS>(keys, whist + warp * R, bit, dmask);
  }
  if (STABLE && tid == 0)
  {
    if constexpr (Digits::computed)
    {
      misc[4] = dg.d[0];
    }
    else
    {
      misc[4] = extract_digit<U, FP>(keys[0], bit, dmask);
    }
  }
  __syncthreads();

  // ---- tile positions; publish the tile's digit counts; look-back ----
  if (tid < R)
  {
    uint32_t start;
    const uint32_t total = block_digit_offsets<NW>(whist, misc + 8, &start);
    if (STABLE)
    {
      // Short circuit (the reference's TryShortCircuit, agent_radix_sort_onesweep.cuh:386-467):
      // when every real key of the tile has the first key's digit (padding keys carry the
      // largest digit and are discounted), the stable permutation is the identity and the
      // keys go out straight from registers. misc[3] = flag | digit << 8, written by that
      // digit's thread; barrier 1 publishes it to warps 0-7, bar 2 to the rest.
      if (uint32_t(tid) == misc[4])
      {
        const uint32_t pad_digit = Digits::computed ? 255u : dmask;
        const uint32_t real      = total - (uint32_t(tid) == pad_digit ? uint32_t(TILE) - valid : 0u);
        misc[3]                  = real == valid ? (1u | (uint32_t(tid) << 8)) : 0u;
      }
      named_barrier_256();
    }
    uint32_t* lb_row     = p.lookback + (size_t) (p.tile_row_base + tile) * R;
    const bool publish   = tile != gb300_fault_skip_tile; // always, unless a test withholds this tile
    if (publish)
    {
      store_status(lb_row + tid, (tile == 0 ? LB_INCLUSIVE : LB_PARTIAL) | total);
    }
    asm volatile("bar.arrive 2, %0;" ::"n"(TPB) : "memory");

    uint32_t excl = 0;
    bool failed   = false;
    if (tile > 0)
    {
      excl = lookback_walk(p, tile, tid, failed);
      if (publish)
      {
        store_status(lb_row + tid, failed ? LB_ERROR : (LB_INCLUSIVE | (excl + total)));
      }
      if (failed)
      {
        atomicOr(p.status, STATUS_LOOKBACK_TIMEOUT);
        misc[1] = 1u;
      }
    }
    if (p.lookback_next != nullptr)
    {
      p.lookback_next[(size_t) (p.tile_row_base + tile) * R + tid] = 0u;
    }
    const unsigned long long base = p.bins[tid] + excl;
    gdelta[tid]                   = (long long) base - (long long) start;
    if (p.bins_next != nullptr && tile == p.portion_tiles - 1)
    {
      p.bins_next[tid] = base + total;
    }
  }
  else
  {
    asm volatile("bar.sync 2, %0;" ::"n"(TPB) : "memory");
  }

  // (not in the order-free first-pass kernel: ptxas cannot allocate its ballot loop with the
  // extra branch, and that kernel sorts integer keys only, where single-digit tiles are rare)
  const uint32_t single = STABLE ? misc[3] : 0u;
  const unsigned long long out_limit_early = p.num_items_total;
  U* kout                                  = static_cast<U*>(p.keys_out);
  V* vout                                  = static_cast<V*>(p.values_out);
  if (single != 0u)
  {
    // ---- one digit: tile order is the output order ----
    V vals[VB > 0 ? ITEMS : 1];
    if constexpr (VB > 0)
    {
      load_values(vals);
    }
    __syncthreads(); // gdelta written; misc[1] final
    const unsigned long long out_limit = misc[1] != 0u ? 0ull : out_limit_early;
    const long long base               = gdelta[single >> 8];
    const uint32_t wofs                = uint32_t(warp * ITEMS * 32 + (tid & 31));
#pragma unroll
    for (int i = 0; i < ITEMS; ++i)
    {
      const uint32_t s = wofs + i * 32;
      if (full || s < valid)
      {
        const long long g = base + (long long) s;
        if ((unsigned long long) g < out_limit)
        {
          __stcs(kout + g, p.decode_out ? decode_key<U>(keys[i], p.codec) : keys[i]);
          if constexpr (VB > 0)
          {
            __stcs(vout + g, vals[i]);
          }
        }
      }
    }
  }
  else
  {
    // ---- stable ranks, scatter into the staging tile ----
    uint32_t pos[ITEMS];
    __syncwarp(); // reconverge after the divergent look-back before the warp votes
    if constexpr (Digits::computed)
    {
      warp_rank_stable_digits<ITEMS>(dg.d, pos, whist + warp * R);
    }
    else if (STABLE || !full) // a partial tile's padding keys must rank after its real keys
    {
      warp_rank_stable<U, FP, ITEMS>(keys, pos, whist + warp * R, bit, dmask);
    }
    else
    {
      warp_rank_unstable<U, FP, ITEMS>(keys, pos, whist + warp * R, bit, dmask);
    }
#pragma unroll
    for (int i = 0; i < ITEMS; ++i)
    {
      kstage[pos[i]] = keys[i];
    }
    if constexpr (Digits::computed)
    {
#pragma unroll
      for (int i = 0; i < ITEMS; ++i)
      {
        dg.stage[pos[i]] = uint8_t(dg.d[i]);
      }
    }
    if constexpr (VB > 0)
    {
      V vals[ITEMS];
      load_values(vals);
#pragma unroll
      for (int i = 0; i < ITEMS; ++i)
      {
        vstage[pos[i]] = vals[i];
      }
    }
    __syncthreads();

    // ---- write out: consecutive staging slots of one digit go to consecutive outputs.
    // Every store is bounds-checked against the output size, so even corrupted offsets
    // (a look-back that gave up) cannot write outside the caller's buffers.
    const unsigned long long out_limit = misc[1] != 0u ? 0ull : out_limit_early;
    // keys of up to 4 bytes: decode and position width fixed at compile time (as in the
    // persistent kernel's write-out)
    auto write_out = [&](auto decode_tag, auto narrow_tag) {
      constexpr bool DECODE = decltype(decode_tag)::value;
      constexpr bool NARROW = decltype(narrow_tag)::value;
#pragma unroll
      for (int j = 0; j < ITEMS; ++j)
      {
        const uint32_t s = j * TPB + threadIdx.x;
        if (full || s < valid)
        {
          const U k = kstage[s];
          uint32_t d;
          if constexpr (Digits::computed)
          {
            d = dg.stage[s];
          }
          else
          {
            d = extract_digit<U, FP>(k, bit, dmask);
          }
          const U out = KB <= 4 ? (DECODE ? decode_key<U>(k, p.codec) : k)
                                : (p.decode_out ? decode_key<U>(k, p.codec) : k);
          if constexpr (NARROW)
          {
            // positions and deltas fit in 31 bits; a corrupted delta wraps above the limit
            const uint32_t g = uint32_t(reinterpret_cast<const int32_t*>(gdelta)[2 * d] + int32_t(s));
            if (g < uint32_t(out_limit))
            {
              __stcs(kout + g, out);
              if constexpr (VB > 0)
              {
                __stcs(vout + g, vstage[s]);
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
                __stcs(vout + g, vstage[s]);
              }
            }
          }
        }
      }
    };
    if constexpr (KB <= 4)
    {
      const bool narrow = p.num_items_total < (1ull << 31);
      if (p.decode_out)
      {
        if (narrow)
        {
          write_out(BoolTag<true>{}, BoolTag<true>{});
        }
        else
        {
          write_out(BoolTag<true>{}, BoolTag<false>{});
        }
      }
      else
      {
        if (narrow)
        {
          write_out(BoolTag<false>{}, BoolTag<true>{});
        }
        else
        {
          write_out(BoolTag<false>{}, BoolTag<false>{});
        }
      }
    }
    else
    {
      write_out(BoolTag<false>{}, BoolTag<false>{}); // the decode is chosen per key
    }
  }
}

// Loads one tile's keys warp-striped from global memory (coalesced), encoding on the
// first pass; padding keys of a partial tile are all-ones so they rank last.
template <int KB, int TPB, int ITEMS>
__device__ __forceinline__ void load_tile_keys_global(
  const OnesweepParams& p,
  const void* keys_in,
  int encode_in,
  uint32_t tile_first,
  uint32_t valid,
  typename uint_of<KB>::type (&keys)[ITEMS])
{
  using U        = typename uint_of<KB>::type;
  const U* kin   = static_cast<const U*>(keys_in) + tile_first;
  const int wofs = (threadIdx.x >> 5) * ITEMS * 32 + (threadIdx.x & 31);
  if (valid == uint32_t(TPB * ITEMS))
  {
#pragma unroll
    for (int i = 0; i < ITEMS; ++i)
    {
      keys[i] = __ldcs(kin + wofs + i * 32);
    }
  }
  else
  {
#pragma unroll
    for (int i = 0; i < ITEMS; ++i)
    {
      const uint32_t idx = wofs + i * 32;
      keys[i]            = idx < valid ? kin[idx] : U(~U(0));
    }
  }
  if (encode_in)
  {
#pragma unroll
    for (int i = 0; i < ITEMS; ++i)
    {
      const uint32_t idx = wofs + i * 32;
      if (idx < valid)
      {
        keys[i] = encode_key<U>(keys[i], p.codec);
      }
    }
  }
}

template <int VB, int TPB, int ITEMS>
__device__ __forceinline__ void load_tile_values_global(
  const void* values_in, uint32_t tile_first, uint32_t valid, typename value_word<VB>::type (&vals)[ITEMS])
{
  using V        = typename value_word<VB>::type;
  const V* vin   = static_cast<const V*>(values_in) + tile_first;
  const int wofs = (threadIdx.x >> 5) * ITEMS * 32 + (threadIdx.x & 31);
#pragma unroll
  for (int i = 0; i < ITEMS; ++i)
  {
    const uint32_t idx = wofs + i * 32;
    if (idx < valid)
    {
      vals[i] = __ldcs(vin + idx);
    }
  }
}

// ---------------------------------------------------------------------------------------
// CTA-per-tile kernel (dynamic tile ids taken in launch order guarantee forward progress)
// ---------------------------------------------------------------------------------------
template <int KB, int VB, int FP, int TPB, int ITEMS, bool STABLE>
__device__ __forceinline__ void onesweep_body(const OnesweepParams& p)
{
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

  if (!gate_open(p.gate))
  {
    return;
  }
  const int tid = threadIdx.x;
  if (tid == 0)
  {
    misc[0] = atomicAdd(p.tile_counter, 1u);
    misc[1] = 0u;
  }
  for (int i = tid; i < NW * R; i += TPB)
  {
    whist[i] = 0;
  }
  __syncthreads();

  const uint32_t tile       = misc[0];
  const uint32_t tile_first = tile * L::TILE;
  const uint32_t valid      = min(uint32_t(L::TILE), p.portion_items - tile_first);
  U keys[ITEMS];
  load_tile_keys_global<KB, TPB, ITEMS>(p, p.keys_in, p.encode_in, tile_first, valid, keys);
  onesweep_tile<KB, VB, FP, TPB, ITEMS, STABLE>(p, tile, valid, keys, whist, gdelta, misc, kstage, vstage, [&](auto& vals) {
    if constexpr (VB > 0)
    {
      load_tile_values_global<VB, TPB, ITEMS>(p.values_in, tile_first, valid, vals);
    }
  });
}

// ---------------------------------------------------------------------------------------
// Persistent kernel, warp-specialised and pipelined. The CTA has TPB - LOOKBACK_THREADS
// "main" threads, whose tiles hold (TPB - LOOKBACK_THREADS) * ITEMS keys, and
// LOOKBACK_THREADS = 256 look-back threads, one per digit. It walks tiles blockIdx.x,
// blockIdx.x + gridDim.x, ...; iteration i (tile t_i, buffer i % 3):
//
//   main:      prefetch t_(i+1) | load t_i, count digits | BH | write out t_(i-1) after BG |
//              BO | rank t_i, stage it in its own buffer | main barrier
//   look-back: BH | tile positions, publish the tile's counts | BO | walk back, global
//              offsets of t_i | BG
//
// The walk of t_i overlaps the ranking of t_i and the loading of t_(i+1); its result is
// needed only when t_i is written out, one iteration later, so the look-back's L2 round
// trips are off the critical path. Three tile buffers rotate: the input of t_(i+1) (bulk
// copy in flight), the input and then the staging tile of t_i, the staging tile of t_(i-1)
// (being written out).
//
// Named barriers: 1 the look-back threads' digit scan (256); 3 BH, 4 BO, 5 BG (all threads:
// BH main arrive / look-back sync, BO both sync, BG look-back arrive / main sync); 6 main
// threads only. BO is a sync on both sides, so the look-back threads cannot arrive at BG
// for t_(i+1) before the main threads have consumed BG for t_i.
// ---------------------------------------------------------------------------------------
template <int KB, int VB, int TPB, int ITEMS, size_t EXTRA = 0>
struct PersistentSmem
{
  using U                   = typename uint_of<KB>::type;
  using V                   = typename value_word<VB>::type;
  static constexpr int MT   = TPB - LOOKBACK_THREADS; // main threads
  static constexpr int NW   = MT / 32;                // main warps: one digit-counter row each
  static constexpr int TILE = MT * ITEMS;
  static constexpr size_t whist_off  = 0;
  static constexpr size_t gdelta_off = whist_off + sizeof(uint32_t) * NW * RADIX_DIGITS;
  static constexpr size_t misc_off   = gdelta_off + sizeof(long long) * RADIX_DIGITS;
  static constexpr size_t buf_off    = misc_off + 128;
  static constexpr size_t kbytes     = ((sizeof(U) * TILE + 15) / 16) * 16;
  static constexpr size_t vbytes     = VB > 0 ? sizeof(V) * TILE : 0;
  static constexpr size_t buf_bytes  = kbytes + vbytes; // keys, then values; input and staging
  static constexpr size_t extra_off  = buf_off + 3 * buf_bytes; // the pass hook's own region
  static constexpr size_t bytes      = extra_off + EXTRA;
  static_assert(MT >= 32 && MT % 32 == 0, "whole main warps");
};
// misc words: [2] sticky failure of the CTA (its stores are disabled), [3] single-digit
// flag and digit of the tile being ranked, [4] digit of the tile's first key, [8..15] scan
// scratch, [16..21] three mbarriers, [22..31] the pass's buffers and flags (PassIO).

// Pass hook of the persistent kernel: the plain radix pass has none. A hook may fill its
// shared-memory region once per CTA (setup) and supply computed digits per tile.
struct PlainPassHook
{
  template <int ITEMS>
  using digits_t = RadixDigits;
  __device__ __forceinline__ void setup(unsigned char*) const {}
  template <class U, int ITEMS>
  __device__ __forceinline__ void compute(const U (&)[ITEMS], uint32_t, int, RadixDigits&, unsigned char*) const
  {}
};

// FROM_PLAN: the pass's buffers and flags come from the resolved plan (res, kept in the misc
// block) instead of the launch parameters.
template <int KB, int VB, int FP, int TPB, int ITEMS, bool STABLE, class Hook, size_t EXTRA, bool FROM_PLAN>
__device__ __forceinline__ void onesweep_persistent_impl(const OnesweepParams& p, const Hook& hook, const PassIO& res)
{
  using L            = PersistentSmem<KB, VB, TPB, ITEMS, EXTRA>;
  using U            = typename L::U;
  using V            = typename L::V;
  using Digits       = typename Hook::template digits_t<ITEMS>;
  constexpr int MT   = L::MT;
  constexpr int NW   = L::NW;
  constexpr int R    = RADIX_DIGITS;
  constexpr int TILE = L::TILE;
  static_assert(STABLE || VB == 0, "pairs need a stable pass");
  static_assert(STABLE || !Digits::computed, "computed digits are ranked stably");
  // How the stable passes find a key's peer lanes: 0 ballots only; 1 lane-mask tables in
  // shared memory; 2 the two alternating by item; 3 per warp, alternating where the digits
  // are spread out and ballots where many are equal (warp_rank_stable_adaptive). The tables
  // live in the tile's own buffer, so the mode needs all main warps' tables to fit in it.
  // Measured on GB300 (2^28 keys, pass time): u32 keys-only 0.967 ms ballots, 0.944 / 0.905
  // / 0.906 ms modes 1-3; u64+u32 pairs 1.693 / 1.675 / 1.674 / 1.699 ms; u64+u32 pairs of
  // low entropy (AND of 5 words) 1.540 / 2.048 / 1.668 / 1.623 ms. Keys-only passes take
  // mode 3, pairs keep ballots.
#ifndef GB300_RANK_MODE_KEYS
#  define GB300_RANK_MODE_KEYS 3
#endif
#ifndef GB300_RANK_MODE_PAIRS
#  define GB300_RANK_MODE_PAIRS 0
#endif
  constexpr int RANK_MODE   = VB == 0 ? GB300_RANK_MODE_KEYS : GB300_RANK_MODE_PAIRS;
  constexpr bool RANK_TABLE = RANK_MODE != 0 && size_t(NW) * R * 4 <= L::buf_bytes;

  extern __shared__ __align__(128) unsigned char smem[];
  uint32_t* whist   = reinterpret_cast<uint32_t*>(smem + L::whist_off);
  long long* gdelta = reinterpret_cast<long long*>(smem + L::gdelta_off);
  uint32_t* misc    = reinterpret_cast<uint32_t*>(smem + L::misc_off);
  uint64_t* mbar    = reinterpret_cast<uint64_t*>(misc + 16);
  PassIO* io        = reinterpret_cast<PassIO*>(misc + 22); // read where used: no registers held
  static_assert(sizeof(PassIO) <= 10 * sizeof(uint32_t), "PassIO fits misc[22..31]");
  // the pass's buffers and flags: launch parameters, or the plan's from shared memory
  auto keys_in_of = [&]() -> const void* {
    if constexpr (FROM_PLAN)
    {
      return io->keys_in;
    }
    else
    {
      return p.keys_in;
    }
  };
  auto values_in_of = [&]() -> const void* {
    if constexpr (FROM_PLAN)
    {
      return io->values_in;
    }
    else
    {
      return p.values_in;
    }
  };
  auto kbuf         = [&](int b) {
    return reinterpret_cast<U*>(smem + L::buf_off + size_t(b) * L::buf_bytes);
  };
  auto vbuf = [&](int b) {
    return reinterpret_cast<V*>(smem + L::buf_off + size_t(b) * L::buf_bytes + L::kbytes);
  };

  const int tid         = threadIdx.x;
  const uint32_t ntiles = p.portion_tiles;
  const int bit         = p.current_bit;
  const uint32_t dmask  = (1u << p.num_bits) - 1u;
  // full tiles come by bulk copy; the partial last tile is read with plain loads
  const uint32_t nfull = p.portion_items / TILE;
  auto issue           = [&](uint32_t t, int b) {
    mbar_arrive_expect_tx(&mbar[b], uint32_t(TILE * KB + (VB > 0 ? TILE * VB : 0)));
    bulk_copy_g2s(kbuf(b), static_cast<const U*>(keys_in_of()) + (size_t) t * TILE, uint32_t(TILE * KB), &mbar[b]);
    if constexpr (VB > 0)
    {
      bulk_copy_g2s(vbuf(b), static_cast<const V*>(values_in_of()) + (size_t) t * TILE, uint32_t(TILE * VB), &mbar[b]);
    }
  };

  if (tid == 0)
  {
    *io = res;
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_init(&mbar[2], 1);
    mbar_init_fence();
    misc[2] = 0u;
    if (blockIdx.x < nfull)
    {
      issue(blockIdx.x, 0);
    }
  }
  for (int i = tid; i < NW * R; i += TPB)
  {
    whist[i] = 0;
  }
  hook.setup(smem + L::extra_off);
  __syncthreads();

  if (tid < MT)
  {
    // ================================ main threads ================================
    const int warp  = tid >> 5;
    const int lane  = tid & 31;
    const int wofs  = warp * ITEMS * 32 + lane;
    U* kout         = static_cast<U*>(FROM_PLAN ? io->keys_out : p.keys_out);
    V* vout         = static_cast<V*>(FROM_PLAN ? io->values_out : p.values_out);
    uint8_t* dstage = nullptr; // computed digits of the staged tile

    // Consecutive staging slots of one digit go to consecutive outputs. Every store is
    // bounds-checked against the output size, so even corrupted offsets (a look-back that
    // gave up) cannot write outside the caller's buffers.
    // Keys of up to 4 bytes: the loop is specialised at compile time on the decode (last pass
    // only) and on the position width (32-bit when the whole array has fewer than 2^31
    // items). Measured on GB300: u32 keys and f32+u32 passes 4 % faster. 8-byte keys keep
    // one loop with a runtime decode and 64-bit positions: the four copies made their
    // passes 2-4 % slower at 2^28 and 2^30.
#ifndef GB300_WRITE_OUT_SPECIALISED
#  define GB300_WRITE_OUT_SPECIALISED (KB <= 4)
#endif
    auto write_out_as = [&](int b, uint32_t valid, auto decode_tag, auto narrow_tag) {
      constexpr bool DECODE              = decltype(decode_tag)::value;
      constexpr bool NARROW              = decltype(narrow_tag)::value;
      const U* ks                        = kbuf(b);
      const V* vs                        = vbuf(b);
      const bool full                    = valid == uint32_t(TILE);
      const unsigned long long out_limit = misc[2] != 0u ? 0ull : p.num_items_total;
      const int32_t* gdelta32            = reinterpret_cast<const int32_t*>(gdelta); // low words
#pragma unroll
      for (int j = 0; j < ITEMS; ++j)
      {
        const uint32_t s = j * MT + tid;
        if (full || s < valid)
        {
          const U k = ks[s];
          uint32_t d;
          if constexpr (Digits::computed)
          {
            d = dstage[s];
          }
          else
          {
            d = extract_digit<U, FP>(k, bit, dmask);
          }
          const U out = DECODE ? decode_key<U>(k, p.codec) : k;
          if constexpr (NARROW)
          {
            // positions and deltas fit in 31 bits; a corrupted delta wraps above the limit
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
    // the same loop, the decode chosen per key at run time, 64-bit positions
    auto write_out_plain = [&](int b, uint32_t valid, bool decode) {
      const U* ks                        = kbuf(b);
      const V* vs                        = vbuf(b);
      const bool full                    = valid == uint32_t(TILE);
      const unsigned long long out_limit = misc[2] != 0u ? 0ull : p.num_items_total;
#pragma unroll
      for (int j = 0; j < ITEMS; ++j)
      {
        const uint32_t s = j * MT + tid;
        if (full || s < valid)
        {
          const U k = ks[s];
          uint32_t d;
          if constexpr (Digits::computed)
          {
            d = dstage[s];
          }
          else
          {
            d = extract_digit<U, FP>(k, bit, dmask);
          }
          const long long g = gdelta[d] + (long long) s;
          if ((unsigned long long) g < out_limit)
          {
            __stcs(kout + g, decode ? decode_key<U>(k, p.codec) : k);
            if constexpr (VB > 0)
            {
              __stcs(vout + g, vs[s]);
            }
          }
        }
      }
    };
    auto write_out = [&](int b, uint32_t valid) {
      const bool decode = (FROM_PLAN ? io->decode_out : p.decode_out) != 0;
      if constexpr (!(GB300_WRITE_OUT_SPECIALISED))
      {
        write_out_plain(b, valid, decode);
      }
      else
      {
        const bool narrow = p.num_items_total < (1ull << 31);
        if (decode)
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
      }
    };

    uint32_t parity     = 0; // bit b: phase parity to wait for on buffer b
    int buf             = 0;
    int prev_buf        = 0;
    uint32_t prev_valid = 0;
    bool have_prev      = false;
    for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x)
    {
      const uint32_t tn = t + gridDim.x;
      const int nbuf    = buf == 2 ? 0 : buf + 1;
      if (tid == 0 && tn < nfull)
      {
        fence_proxy_async_smem(); // buffer nbuf was last accessed by the generic proxy
        issue(tn, nbuf);
      }

      // ---- load, count digits ----
      U keys[ITEMS];
      V vals[VB > 0 ? ITEMS : 1];
      const uint32_t tile_first = t * TILE;
      const uint32_t valid      = min(uint32_t(TILE), p.portion_items - tile_first);
      if (t < nfull)
      {
        const bool data_ok = mbar_wait(&mbar[buf], (parity >> buf) & 1u);
        parity ^= 1u << buf;
        if (!data_ok)
        {
          // the copy never completed: this CTA stores nothing from here on
          atomicOr(p.status, STATUS_LOOKBACK_TIMEOUT);
          misc[2] = 1u;
        }
        const U* ks = kbuf(buf);
#pragma unroll
        for (int i = 0; i < ITEMS; ++i)
        {
          keys[i] = ks[wofs + i * 32];
        }
        if (FROM_PLAN ? io->encode_in : p.encode_in)
        {
#pragma unroll
          for (int i = 0; i < ITEMS; ++i)
          {
            keys[i] = encode_key<U>(keys[i], p.codec);
          }
        }
        if constexpr (VB > 0)
        {
          const V* vs = vbuf(buf);
#pragma unroll
          for (int i = 0; i < ITEMS; ++i)
          {
            vals[i] = vs[wofs + i * 32];
          }
        }
      }
      else
      {
        load_tile_keys_global<KB, MT, ITEMS>(p, keys_in_of(), FROM_PLAN ? io->encode_in : p.encode_in, tile_first,
                                             valid, keys);
        if constexpr (VB > 0)
        {
          load_tile_values_global<VB, MT, ITEMS>(values_in_of(), tile_first, valid, vals);
        }
      }
      Digits dg;
      hook.template compute<U, ITEMS>(keys, valid, wofs, dg, smem + L::extra_off);
      if constexpr (Digits::computed)
      {
        warp_histogram_digits<ITEMS>(dg.d, whist + warp * R);
        dstage = dg.stage;
      }
      else
      {
        warp_histogram<U, FP, ITEMS>(keys, whist + warp * R, bit, dmask);
      }
      if (tid == 0)
      {
        if constexpr (Digits::computed)
        {
          misc[4] = dg.d[0];
        }
        else
        {
          misc[4] = extract_digit<U, FP>(keys[0], bit, dmask);
        }
      }
      asm volatile("bar.arrive 3, %0;" ::"n"(TPB) : "memory"); // BH: counts of t ready

      // ---- the previous tile goes out while the look-back threads turn t's counts into positions ----
      if (have_prev)
      {
        asm volatile("bar.sync 5, %0;" ::"n"(TPB) : "memory"); // BG: offsets of the previous tile
        write_out(prev_buf, prev_valid);
      }
      asm volatile("bar.sync 4, %0;" ::"n"(TPB) : "memory"); // BO: positions of t in whist

      // ---- rank t, stage it in its own buffer ----
      const uint32_t single = STABLE ? misc[3] : 0u;
      uint32_t pos[ITEMS];
      if (single != 0u)
      {
        // one digit (the reference's TryShortCircuit, agent_radix_sort_onesweep.cuh:386-467):
        // the stable permutation is the identity
#pragma unroll
        for (int i = 0; i < ITEMS; ++i)
        {
          pos[i] = uint32_t(wofs + i * 32);
        }
      }
      else
      {
        __syncwarp();
        if constexpr (Digits::computed)
        {
          warp_rank_stable_digits<ITEMS>(dg.d, pos, whist + warp * R);
        }
        else if constexpr (STABLE && RANK_TABLE)
        {
          // the warp's lane-mask table lives in this tile's own buffer: every main thread
          // read its keys (and values) from it before BO, and nothing is staged into it
          // before the main barrier below
          uint32_t* tbl = reinterpret_cast<uint32_t*>(smem + L::buf_off + size_t(buf) * L::buf_bytes) + warp * R;
#pragma unroll
          for (int k = lane; k < R; k += 32)
          {
            tbl[k] = 0u;
          }
          __syncwarp();
          if constexpr (RANK_MODE == 3)
          {
            warp_rank_stable_adaptive<U, FP, ITEMS>(keys, pos, whist + warp * R, tbl, bit, dmask);
          }
          else
          {
            warp_rank_stable_table<U, FP, ITEMS, RANK_MODE == 2>(keys, pos, whist + warp * R, tbl, bit, dmask);
          }
        }
        else if constexpr (STABLE)
        {
          warp_rank_stable<U, FP, ITEMS>(keys, pos, whist + warp * R, bit, dmask);
        }
        else
        {
          warp_rank_unstable_tail<U, FP, ITEMS>(keys, pos, whist + warp * R, bit, dmask, wofs, valid);
        }
      }
      if constexpr (STABLE && RANK_TABLE && !Digits::computed)
      {
        asm volatile("bar.sync 6, %0;" ::"n"(MT) : "memory"); // every warp has ranked: the tables are dead
      }
      U* ks = kbuf(buf);
#pragma unroll
      for (int i = 0; i < ITEMS; ++i)
      {
        ks[pos[i]] = keys[i];
      }
      if constexpr (Digits::computed)
      {
#pragma unroll
        for (int i = 0; i < ITEMS; ++i)
        {
          dg.stage[pos[i]] = uint8_t(dg.d[i]);
        }
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
      __syncwarp(); // the warp's ranking atomics are done: clear its counter row for the next tile
      for (int k = lane; k < R; k += 32)
      {
        whist[warp * R + k] = 0u;
      }
      // staging of t visible to every main thread; the previous tile's buffer is free for
      // the next prefetch
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
    const int d                = tid - MT; // this thread's digit
    const uint32_t skip_tile   = gb300_fault_skip_tile; // no tile, unless a test withholds one
    const unsigned long long bin_base = p.bins[d]; // the digit's global offset, the same for every tile
    for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x)
    {
      const uint32_t valid = min(uint32_t(TILE), p.portion_items - t * TILE);
      asm volatile("bar.sync 3, %0;" ::"n"(TPB) : "memory"); // BH
      uint32_t start;
      const uint32_t total = block_digit_offsets<NW>(whist, misc + 8, &start, d);
      if (STABLE && uint32_t(d) == misc[4])
      {
        // every real key of the tile has the first key's digit (padding keys carry the
        // largest digit and are discounted)
        const uint32_t pad_digit = Digits::computed ? 255u : dmask;
        const uint32_t real      = total - (uint32_t(d) == pad_digit ? uint32_t(TILE) - valid : 0u);
        misc[3]                  = real == valid ? (1u | (uint32_t(d) << 8)) : 0u;
      }
      uint32_t* lb_row   = p.lookback + (size_t) (p.tile_row_base + t) * R;
      const bool publish = t != skip_tile;
      if (publish)
      {
        store_status(lb_row + d, (t == 0 ? LB_INCLUSIVE : LB_PARTIAL) | total);
      }
      asm volatile("bar.sync 4, %0;" ::"n"(TPB) : "memory"); // BO

      uint32_t excl = 0;
      if (t > 0)
      {
        bool failed = false;
        excl        = lookback_walk<PERSISTENT_LOOKBACK_BATCH>(p, t, d, failed);
        if (publish)
        {
          store_status(lb_row + d, failed ? LB_ERROR : (LB_INCLUSIVE | (excl + total)));
        }
        if (failed)
        {
          atomicOr(p.status, STATUS_LOOKBACK_TIMEOUT);
          misc[2] = 1u;
        }
      }
      if (p.lookback_next != nullptr)
      {
        p.lookback_next[(size_t) (p.tile_row_base + t) * R + d] = 0u;
      }
      const unsigned long long base = bin_base + excl;
      gdelta[d]                     = (long long) base - (long long) start;
      if (p.bins_next != nullptr && t == p.portion_tiles - 1)
      {
        p.bins_next[d] = base + total;
      }
      asm volatile("bar.arrive 5, %0;" ::"n"(TPB) : "memory"); // BG
    }
  }
}

// Persistent pass kernel body: resolves the pass plan (returns at once for a pass that is
// gated off or skipped), then runs the pass with its launch parameters when the plan keeps
// them (every pass of a sort that skips none), else with the plan's buffers.
template <int KB, int VB, int FP, int TPB, int ITEMS, bool STABLE, class Hook = PlainPassHook, size_t EXTRA = 0>
__device__ __forceinline__ void onesweep_persistent_body(const OnesweepParams& p, const Hook& hook = Hook{})
{
  PassIO res;
  if (!resolve_pass<KB, VB>(p, res))
  {
    return; // uniform over the grid
  }
  if constexpr (Hook::template digits_t<ITEMS>::computed)
  {
    // passes with computed digits (the learned partition) have no plan
    onesweep_persistent_impl<KB, VB, FP, TPB, ITEMS, STABLE, Hook, EXTRA, false>(p, hook, res);
    return;
  }
  const bool as_launched = res.keys_in == p.keys_in && res.keys_out == p.keys_out && res.values_in == p.values_in
                        && res.values_out == p.values_out && res.encode_in == p.encode_in
                        && res.decode_out == p.decode_out;
  if (as_launched)
  {
    onesweep_persistent_impl<KB, VB, FP, TPB, ITEMS, STABLE, Hook, EXTRA, false>(p, hook, res);
  }
  else
  {
    onesweep_persistent_impl<KB, VB, FP, TPB, ITEMS, STABLE, Hook, EXTRA, true>(p, hook, res);
  }
}

} // namespace gb300
