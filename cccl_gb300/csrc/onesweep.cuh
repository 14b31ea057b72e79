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
// Two kernels share this tile code:
//   * onesweep_persistent_body: the main path. One CTA per SM, launched cooperatively, walks
//     tiles blockIdx.x, blockIdx.x + gridDim.x, ...; the next tile's keys and values are
//     fetched into shared memory by a bulk async copy (cp.async.bulk + mbarrier) while the
//     current tile is ranked and written, so HBM latency is off the critical path;
//   * onesweep_body: CTA-per-tile with dynamic tile ids and plain warp-striped loads; used
//     when the caller's buffers are not 16-byte aligned.
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
  __syncthreads();

  // ---- tile positions; publish the tile's digit counts; look-back ----
  if (tid < R)
  {
    if (STABLE && tid < 32)
    {
      // Short circuit (the reference's TryShortCircuit, agent_radix_sort_onesweep.cuh:386-467):
      // when every real key of the tile has the tile's first digit, the stable permutation is
      // the identity and the keys go out straight from registers. misc[3] = flag | digit << 8;
      // the barrier inside block_digit_offsets publishes it to warps 0-7, bar 2 to the rest.
      uint32_t d0;
      if constexpr (Digits::computed)
      {
        d0 = dg.d[0];
      }
      else
      {
        d0 = extract_digit<U, FP>(keys[0], bit, dmask);
      }
      d0         = __shfl_sync(0xffffffffu, d0, 0);
      uint32_t c = 0;
      for (int w = tid; w < NW; w += 32)
      {
        c += whist[w * R + d0];
      }
      c = __reduce_add_sync(0xffffffffu, c);
      const uint32_t pad_digit = Digits::computed ? 255u : dmask;
      const uint32_t real_d0   = c - (d0 == pad_digit ? uint32_t(TILE) - valid : 0u);
      if (tid == 0)
      {
        misc[3] = real_d0 == valid ? (1u | (d0 << 8)) : 0u;
      }
    }
    uint32_t start;
    const uint32_t total = block_digit_offsets<NW>(whist, misc + 8, &start);
    uint32_t* lb_row     = p.lookback + (size_t) (p.tile_row_base + tile) * R;
    store_status(lb_row + tid, (tile == 0 ? LB_INCLUSIVE : LB_PARTIAL) | total);
    asm volatile("bar.arrive 2, %0;" ::"n"(TPB) : "memory");

    uint32_t excl = 0;
    bool failed   = false;
    if (tile > 0)
    {
      // Read LOOKBACK_BATCH predecessor rows per step: a sequential walk would cap the
      // pass at one tile per L2 round trip.
      const uint32_t* col = p.lookback + (size_t) p.tile_row_base * R + tid;
      bool done           = false;
      for (int j = int(tile) - 1; !done; j -= LOOKBACK_BATCH)
      {
        uint32_t w[LOOKBACK_BATCH];
#pragma unroll
        for (int k = 0; k < LOOKBACK_BATCH; ++k)
        {
          w[k] = (j - k >= 0) ? load_status(col + (size_t) (j - k) * R) : LB_INCLUSIVE;
        }
#pragma unroll
        for (int k = 0; k < LOOKBACK_BATCH; ++k)
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
      store_status(lb_row + tid, failed ? LB_ERROR : (LB_INCLUSIVE | (excl + total)));
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
        const long long g = gdelta[d] + (long long) s;
        if ((unsigned long long) g < out_limit)
        {
          __stcs(kout + g, p.decode_out ? decode_key<U>(k, p.codec) : k);
          if constexpr (VB > 0)
          {
            __stcs(vout + g, vstage[s]);
          }
        }
      }
    }
  }
}

// Loads one tile's keys warp-striped from global memory (coalesced), encoding on the
// first pass; padding keys of a partial tile are all-ones so they rank last.
template <int KB, int TPB, int ITEMS>
__device__ __forceinline__ void load_tile_keys_global(
  const OnesweepParams& p, uint32_t tile_first, uint32_t valid, typename uint_of<KB>::type (&keys)[ITEMS])
{
  using U        = typename uint_of<KB>::type;
  const U* kin   = static_cast<const U*>(p.keys_in) + tile_first;
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
  if (p.encode_in)
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
  const OnesweepParams& p, uint32_t tile_first, uint32_t valid, typename value_word<VB>::type (&vals)[ITEMS])
{
  using V        = typename value_word<VB>::type;
  const V* vin   = static_cast<const V*>(p.values_in) + tile_first;
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
  load_tile_keys_global<KB, TPB, ITEMS>(p, tile_first, valid, keys);
  onesweep_tile<KB, VB, FP, TPB, ITEMS, STABLE>(p, tile, valid, keys, whist, gdelta, misc, kstage, vstage, [&](auto& vals) {
    if constexpr (VB > 0)
    {
      load_tile_values_global<VB, TPB, ITEMS>(p, tile_first, valid, vals);
    }
  });
}

// ---------------------------------------------------------------------------------------
// Persistent kernel: tiles blockIdx.x + k * gridDim.x, the next tile prefetched into
// shared memory by bulk async copies while the current one is processed.
// ---------------------------------------------------------------------------------------
template <int KB, int VB, int TPB, int ITEMS, size_t EXTRA = 0>
struct PersistentSmem
{
  using U                   = typename uint_of<KB>::type;
  using V                   = typename value_word<VB>::type;
  static constexpr int NW   = TPB / 32;
  static constexpr int TILE = TPB * ITEMS;
  static constexpr size_t whist_off  = 0;
  static constexpr size_t gdelta_off = whist_off + sizeof(uint32_t) * NW * RADIX_DIGITS;
  static constexpr size_t misc_off   = gdelta_off + sizeof(long long) * RADIX_DIGITS;
  static constexpr size_t buf_off    = misc_off + 128;
  static constexpr size_t kbytes     = ((sizeof(U) * TILE + 15) / 16) * 16;
  static constexpr size_t vbytes     = VB > 0 ? sizeof(V) * TILE : 0;
  static constexpr size_t buf_bytes  = kbytes + vbytes; // keys, then values; input and staging
  static constexpr size_t extra_off  = buf_off + 2 * buf_bytes; // the pass hook's own region
  static constexpr size_t bytes      = extra_off + EXTRA;
};

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

template <int KB, int VB, int FP, int TPB, int ITEMS, bool STABLE, class Hook = PlainPassHook, size_t EXTRA = 0>
__device__ __forceinline__ void onesweep_persistent_body(const OnesweepParams& p, const Hook& hook = Hook{})
{
  using L            = PersistentSmem<KB, VB, TPB, ITEMS, EXTRA>;
  using U            = typename L::U;
  using V            = typename L::V;
  constexpr int NW   = L::NW;
  constexpr int R    = RADIX_DIGITS;
  constexpr int TILE = L::TILE;

  extern __shared__ __align__(128) unsigned char smem[];
  uint32_t* whist   = reinterpret_cast<uint32_t*>(smem + L::whist_off);
  long long* gdelta = reinterpret_cast<long long*>(smem + L::gdelta_off);
  uint32_t* misc    = reinterpret_cast<uint32_t*>(smem + L::misc_off);
  uint64_t* mbar    = reinterpret_cast<uint64_t*>(misc + 16);
  auto kbuf         = [&](int b) {
    return reinterpret_cast<U*>(smem + L::buf_off + size_t(b) * L::buf_bytes);
  };
  auto vbuf = [&](int b) {
    return reinterpret_cast<V*>(smem + L::buf_off + size_t(b) * L::buf_bytes + L::kbytes);
  };

  if (!gate_open(p.gate))
  {
    return;
  }
  const int tid         = threadIdx.x;
  const int wofs        = (tid >> 5) * ITEMS * 32 + (tid & 31);
  const uint32_t ntiles = p.portion_tiles;
  // full tiles come by bulk copy; the partial last tile is read with plain loads
  const uint32_t nfull = p.portion_items / TILE;
  auto issue           = [&](uint32_t t, int b) {
    mbar_arrive_expect_tx(&mbar[b], uint32_t(TILE * KB + (VB > 0 ? TILE * VB : 0)));
    bulk_copy_g2s(kbuf(b), static_cast<const U*>(p.keys_in) + (size_t) t * TILE, uint32_t(TILE * KB), &mbar[b]);
    if constexpr (VB > 0)
    {
      bulk_copy_g2s(vbuf(b), static_cast<const V*>(p.values_in) + (size_t) t * TILE, uint32_t(TILE * VB), &mbar[b]);
    }
  };

  if (tid == 0)
  {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_init_fence();
    misc[2] = 0u;
    if (blockIdx.x < nfull)
    {
      issue(blockIdx.x, 0);
    }
  }
  hook.setup(smem + L::extra_off);
  __syncthreads();

  uint32_t parity = 0; // bit b: phase parity to wait for on buffer b
  int cur         = 0;
  for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x, cur ^= 1)
  {
    const uint32_t tn = t + gridDim.x;
    if (tid == 0)
    {
      misc[1] = misc[2];
      if (tn < nfull)
      {
        fence_proxy_async_smem(); // buffer cur^1 was last accessed by the generic proxy
        issue(tn, cur ^ 1);
      }
    }
    for (int i = tid; i < NW * R; i += TPB)
    {
      whist[i] = 0;
    }

    U keys[ITEMS];
    V vals[VB > 0 ? ITEMS : 1];
    const uint32_t tile_first = t * TILE;
    const uint32_t valid      = min(uint32_t(TILE), p.portion_items - tile_first);
    bool data_ok              = true;
    if (t < nfull)
    {
      data_ok = mbar_wait(&mbar[cur], (parity >> cur) & 1u);
      parity ^= 1u << cur;
      const U* ks = kbuf(cur);
#pragma unroll
      for (int i = 0; i < ITEMS; ++i)
      {
        keys[i] = ks[wofs + i * 32];
      }
      if (p.encode_in)
      {
#pragma unroll
        for (int i = 0; i < ITEMS; ++i)
        {
          keys[i] = encode_key<U>(keys[i], p.codec);
        }
      }
      if constexpr (VB > 0)
      {
        const V* vs = vbuf(cur);
#pragma unroll
        for (int i = 0; i < ITEMS; ++i)
        {
          vals[i] = vs[wofs + i * 32];
        }
      }
    }
    else
    {
      load_tile_keys_global<KB, TPB, ITEMS>(p, tile_first, valid, keys);
      if constexpr (VB > 0)
      {
        load_tile_values_global<VB, TPB, ITEMS>(p, tile_first, valid, vals);
      }
    }
    typename Hook::template digits_t<ITEMS> dg;
    hook.template compute<U, ITEMS>(keys, valid, wofs, dg, smem + L::extra_off);
    if (!data_ok)
    {
      // the copy never completed: this CTA stores nothing from here on
      atomicOr(p.status, STATUS_LOOKBACK_TIMEOUT);
      misc[2] = 1u;
      misc[1] = 1u;
    }
    __syncthreads(); // whist zeroed, failure flags set, buffer cur consumed: it becomes the staging tile
    onesweep_tile<KB, VB, FP, TPB, ITEMS, STABLE>(
      p, t, valid, keys, whist, gdelta, misc, kbuf(cur), vbuf(cur), [&](auto& out) {
        if constexpr (VB > 0)
        {
#pragma unroll
          for (int i = 0; i < ITEMS; ++i)
          {
            out[i] = vals[i];
          }
        }
      }, dg);
    __syncthreads(); // staging tile written out; whist/gdelta/misc free for the next tile
  }
}

} // namespace gb300
