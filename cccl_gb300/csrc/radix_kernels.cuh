// Plain-path radix sort kernels for sm_103a: control-block init, all-pass digit
// histogram (with the exclusive scan fused into its last CTA), the onesweep digit pass
// and the single-CTA sort for small inputs.
//
// Algorithm (reference roles, file:line in the reference tree):
//  * histogram of every pass in one read of the keys
//      cub/cub/agent/agent_radix_sort_histogram.cuh:96-285, kernel_radix_sort.cuh:447-473;
//    exclusive sum of each pass's bins  kernel_radix_sort.cuh:563-606;
//  * one stable 8-bit counting-sort pass per digit with decoupled look-back across tiles
//      cub/cub/agent/agent_radix_sort_onesweep.cuh:152-739, kernel_radix_sort.cuh:498-558;
//    stable in-tile ranking with per-warp digit counters and warp match
//      cub/cub/block/block_radix_rank.cuh:913-1213;
//  * small inputs sorted by one CTA  kernel_radix_sort.cuh:330-434.
//
// Differences in how the work is laid out on GB300 (same results):
//  * tiles are staged in up to ~100 KB of dynamic shared memory (CUB caps static shared
//    memory at 48 KB), giving longer same-digit runs in the scatter;
//  * keys stay in the encoded (bit-ordered, order-applied) form between passes, so the
//    encode runs on the first pass's load and the decode on the last pass's store only;
//  * every look-back wait is bounded (wait_status) and reports a status bit instead of
//    spinning forever;
//  * the look-back buffer of the next pass is cleared by the current pass (row per tile),
//    so no memset runs between passes.
#pragma once

#include "sort_policy.h"
#include "tile_rank.cuh"

namespace gb300
{

// ---------------------------------------------------------------------------------------
// init: zero a block of 32-bit words (the per-call control block)
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void init_body(const InitParams& p)
{
  if (!gate_open(p.gate))
  {
    return;
  }
  for (unsigned long long i = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x; i < p.num_words;
       i += (unsigned long long) gridDim.x * blockDim.x)
  {
    p.words[i] = 0u;
  }
}

// The pass plan (plan_pass_words), kept out of line: it runs once per sort, and inlined it
// cost the histogram kernels registers.
__device__ __noinline__ void write_pass_plan(uint32_t* plan, int num_passes, int plan_mode, uint32_t trivial_mask)
{
  plan_pass_words(plan, num_passes, plan_mode, trivial_mask);
}

// Second half of every all-pass histogram kernel: clears pass 0's look-back buffer, adds
// this CTA's shared counts (sh[pass * 256 + digit]) to the global ones, and the last CTA
// to finish writes each pass's exclusive prefix (portion 0's digit bases) and, when asked,
// the pass plan (the PLAN_* words: which passes skip, which buffers the others use).
template <int TPB>
__device__ __forceinline__ void histogram_finish(const HistogramParams& p, const uint32_t* sh)
{
  constexpr int R = RADIX_DIGITS;
  __shared__ uint32_t last_flag;
  __shared__ uint32_t trivial_mask; // bit q: one digit holds every key in pass q
  const int tid = threadIdx.x;
  // clear the look-back buffer of pass 0
  for (unsigned long long i = blockIdx.x * (unsigned long long) TPB + tid; i < p.lookback_words;
       i += (unsigned long long) gridDim.x * TPB)
  {
    p.lookback_clear[i] = 0u;
  }

  __syncthreads();
  for (int i = tid; i < p.num_passes * R; i += TPB)
  {
    if (sh[i] != 0)
    {
      atomicAdd(&p.ctrl->counts[i], (unsigned long long) sh[i]);
    }
  }
  __threadfence();
  __syncthreads();
  if (tid == 0)
  {
    last_flag    = (atomicAdd(&p.ctrl->hist_done, 1u) == gridDim.x - 1) ? 1u : 0u;
    trivial_mask = 0u;
  }
  __syncthreads();
  if (last_flag == 0)
  {
    return;
  }
  __threadfence();
  // one warp per pass: lane l owns digits [8l, 8l+8)
  const int warp = tid >> 5;
  const int lane = tid & 31;
  if (warp < p.num_passes)
  {
    unsigned long long c[8];
    unsigned long long s = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j)
    {
      c[j] = __ldcg(&p.ctrl->counts[warp * R + lane * 8 + j]);
      s += c[j];
    }
    unsigned long long x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o)
      {
        x += y;
      }
    }
    unsigned long long run = x - s;
    unsigned long long* out = p.bins + (size_t) warp * p.num_portions * R;
#pragma unroll
    for (int j = 0; j < 8; ++j)
    {
      out[lane * 8 + j] = run;
      run += c[j];
    }
  }
  if (p.plan == nullptr)
  {
    return;
  }
  // a pass is skippable when one digit holds every key (counts re-read: fewer live registers)
  if (warp < p.num_passes)
  {
    bool all_one_digit = false;
#pragma unroll 1
    for (int j = 0; j < 8; ++j)
    {
      all_one_digit |= __ldcg(&p.ctrl->counts[warp * R + lane * 8 + j]) == p.num_items;
    }
    if (__any_sync(0xffffffffu, all_one_digit) && lane == 0)
    {
      atomicOr(&trivial_mask, 1u << warp);
    }
  }
  __syncthreads();
  if (tid == 0)
  {
    write_pass_plan(p.plan, p.num_passes, p.plan_mode, trivial_mask);
  }
}

// Calls fn(key) once for every key of keys[0, n), spread over the grid: a scalar head up
// to 16-byte alignment and a scalar tail (CTA 0), 16-byte streaming loads in between.
template <int KB, int TPB, class Fn>
__device__ __forceinline__ void histogram_for_each_key(const void* keys_v, unsigned long long n, Fn&& fn)
{
  using U           = typename uint_of<KB>::type;
  constexpr int VEC = 16 / KB;
  const int tid     = threadIdx.x;
  const U* keys     = static_cast<const U*>(keys_v);
  const unsigned long long addr = reinterpret_cast<unsigned long long>(keys);
  unsigned long long head       = ((16 - (addr & 15)) & 15) / KB;
  if (head > n)
  {
    head = n;
  }
  const unsigned long long nvec     = (n - head) / VEC;
  const unsigned long long body_end = head + nvec * VEC;
  if (blockIdx.x == 0)
  {
    for (unsigned long long i = tid; i < head; i += TPB)
    {
      fn(keys[i]);
    }
    for (unsigned long long i = body_end + tid; i < n; i += TPB)
    {
      fn(keys[i]);
    }
  }
  const uint4* vkeys = reinterpret_cast<const uint4*>(keys + head);
  for (unsigned long long v = blockIdx.x * (unsigned long long) TPB + tid; v < nvec;
       v += (unsigned long long) gridDim.x * TPB)
  {
    const uint4 w = __ldcs(vkeys + v);
    U k[VEC];
    memcpy(k, &w, 16);
#pragma unroll
    for (int j = 0; j < VEC; ++j)
    {
      fn(k[j]);
    }
  }
}

// ---------------------------------------------------------------------------------------
// histogram: counts of every pass's digit in one read; the last CTA writes the exclusive
// prefix (global digit bases) of portion 0 for every pass. Also clears pass 0's look-back.
// ---------------------------------------------------------------------------------------
template <int KB, int FP, int TPB>
__device__ __forceinline__ void histogram_body(const HistogramParams& p)
{
  using U         = typename uint_of<KB>::type;
  constexpr int R = RADIX_DIGITS;
  __shared__ uint32_t sh[MAX_PASSES * R];
  if (!gate_open(p.gate))
  {
    return;
  }

  const int tid = threadIdx.x;
  for (int i = tid; i < MAX_PASSES * R; i += TPB)
  {
    sh[i] = 0;
  }
  __syncthreads();

  int shift[MAX_PASSES];
  uint32_t mask[MAX_PASSES];
#pragma unroll
  for (int q = 0; q < MAX_PASSES; ++q)
  {
    const int b  = p.begin_bit + q * RADIX_BITS;
    const int nb = min(RADIX_BITS, p.end_bit - b);
    shift[q]     = b;
    mask[q]      = (q < p.num_passes) ? ((1u << nb) - 1u) : 0u;
  }

  auto count_key = [&](U raw) {
    const U t = encode_key<U>(raw, p.codec);
#pragma unroll
    for (int q = 0; q < MAX_PASSES; ++q)
    {
      if (q < p.num_passes)
      {
        atomicAdd(&sh[q * R + extract_digit<U, FP>(t, shift[q], mask[q])], 1u);
      }
    }
  };

  histogram_for_each_key<KB, TPB>(p.keys, p.num_items, count_key);
  histogram_finish<TPB>(p, sh);
}

// ---------------------------------------------------------------------------------------
// Lane-column histogram: the all-pass digit counts of the plain sort, one CTA per SM.
//
// The reference counts into one shared table per CTA with an atomic per digit
// (cub/cub/agent/agent_radix_sort_histogram.cuh:96-285); on GB300 that is bound by bank
// conflicts among the 32 random addresses of each warp-wide atomic (measured: ~0.4 of HBM).
// Here the counter of (pass q, digit d) for lane l is its own word, laid out so that the 32
// lanes of a warp always hit 32 different banks:
//   byte offset = block(q) << 16 | d << 8 | byte0(q, l)
//   up to 4 passes: block = q >> 1, byte0 = (q & 1) * 128 + l * 4 (32-bit counters)
//   5 to 8 passes:  two passes share 32-bit words, pass 2p in the low and pass 2p + 1 in the
//                   high 16 bits: block = q >> 2, byte0 = ((q >> 1) & 1) * 128 + l * 4
// so one byte permute (digit byte q of the key into byte 1 of a per-lane constant) gives the
// counter's address, and one reduction-add (no return value; 1, or 1 << 16 for the high half)
// counts the key: two instructions per key and pass, all 32 columns conflict-free for every
// pass count. Every CTA of the kernel shares the columns among its warps (the adds are
// atomic). The 16-bit halves are folded into 32-bit totals before they can overflow (every
// warp adds at most one key per lane and counter per key it loads). At the end each row of
// columns is summed by a warp and the totals go to histogram_finish. Keys are streamed with
// four 16-byte loads in flight per thread.
// ---------------------------------------------------------------------------------------
// Encoded key for the counting loops: integer kinds have one mask for both signs (make_codec),
// so their encoding is a single XOR; floating-point kinds pick the mask by the sign bit.
template <class U, int FP>
__device__ __forceinline__ U encode_key_for_count(U x, const KeyCodec& c)
{
  if constexpr (FP == FP_NONE)
  {
    return U(x ^ U(c.fwd_pos));
  }
  else
  {
    return encode_key<U>(x, c);
  }
}

// Counts one key's digits in passes [0, NP): digit q is byte q of t (the key's window,
// shifted down to bit 0), its counter address one byte permute away (see the layout above).
template <class U, int NP>
__device__ __forceinline__ void count_digits_lanes(U t, uint32_t table_base, const uint32_t (&col)[8])
{
  constexpr bool PACKED = NP > 4;
  const uint32_t lo     = uint32_t(t);
  uint32_t hi           = 0;
  if constexpr (sizeof(U) == 8)
  {
    hi = uint32_t((unsigned long long) t >> 32);
  }
#pragma unroll
  for (int q = 0; q < NP; ++q)
  {
    const uint32_t off = __byte_perm(q < 4 ? lo : hi, col[q], 0x7604u | (uint32_t(q & 3) << 4));
    if (PACKED && (q & 1))
    {
      asm volatile("red.shared.add.u32 [%0], 65536;" ::"r"(table_base + off));
    }
    else
    {
      asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(table_base + off));
    }
  }
}

// Column counters of (pass, digit) in the layout above, summed over the 32 columns by one warp
// per row, added to totals[pass * 256 + digit] and cleared. Called by the whole CTA.
template <int TPB, int NP>
__device__ __forceinline__ void histogram_lanes_fold(unsigned char* table, uint32_t* totals)
{
  constexpr int R      = RADIX_DIGITS;
  constexpr bool PACKED = NP > 4;
  constexpr int ROWS   = PACKED ? (NP + 1) / 2 : NP; // word rows: pass pairs, or passes
  const int warp       = threadIdx.x >> 5;
  const int lane       = threadIdx.x & 31;
  for (int r = warp; r < ROWS * R; r += TPB / 32)
  {
    const int q          = r >> 8; // pass (pair, when packed)
    const int d          = r & (R - 1);
    const uint32_t base  = (uint32_t(q >> 1) << 16) | (uint32_t(d) << 8) | (uint32_t(q & 1) * 128u);
    uint32_t* word       = reinterpret_cast<uint32_t*>(table + base + 4u * uint32_t(lane));
    const uint32_t x     = *word;
    *word                = 0u;
    if constexpr (PACKED)
    {
      const uint32_t lo = __reduce_add_sync(0xffffffffu, x & 0xffffu);
      const uint32_t hi = __reduce_add_sync(0xffffffffu, x >> 16);
      if (lane == 0)
      {
        totals[(2 * q) * R + d] += lo;
        if (2 * q + 1 < NP)
        {
          totals[(2 * q + 1) * R + d] += hi;
        }
      }
    }
    else
    {
      const uint32_t total = __reduce_add_sync(0xffffffffu, x);
      if (lane == 0)
      {
        totals[q * R + d] += total;
      }
    }
  }
}

template <int KB, int FP, int TPB, int NP, bool WINDOW>
__device__ __forceinline__ void
histogram_lanes_count(const HistogramParams& p, unsigned char* table, uint32_t table_base, const uint32_t (&col)[8], uint32_t* totals)
{
  using U           = typename uint_of<KB>::type;
  constexpr int VEC = 16 / KB; // keys per 16-byte load
  const int tid     = threadIdx.x;
  const int bb      = p.begin_bit;
  const int wbits   = p.end_bit - p.begin_bit;
  const U wmask     = wbits >= 8 * KB ? U(~U(0)) : U((U(1) << wbits) - U(1));
  auto count_key    = [&](U raw) {
    U t = digit_source<U, FP>(encode_key_for_count<U, FP>(raw, p.codec));
    if constexpr (WINDOW)
    {
      t = U(U(t >> bb) & wmask);
    }
    count_digits_lanes<U, NP>(t, table_base, col);
  };
  const U* keys                 = static_cast<const U*>(p.keys);
  const unsigned long long n    = p.num_items;
  const unsigned long long addr = reinterpret_cast<unsigned long long>(keys);
  unsigned long long head       = ((16 - (addr & 15)) & 15) / KB;
  if (head > n)
  {
    head = n;
  }
  const unsigned long long nvec     = (n - head) / VEC;
  const unsigned long long body_end = head + nvec * VEC;
  if (blockIdx.x == 0)
  {
    for (unsigned long long i = tid; i < head; i += TPB)
    {
      count_key(keys[i]);
    }
    for (unsigned long long i = body_end + tid; i < n; i += TPB)
    {
      count_key(keys[i]);
    }
  }
  const uint4* vkeys              = reinterpret_cast<const uint4*>(keys + head);
  const unsigned long long stride = (unsigned long long) gridDim.x * TPB;
  unsigned long long v            = blockIdx.x * (unsigned long long) TPB + tid;
  auto count_vec                  = [&](const uint4& w) {
    U k[VEC];
    memcpy(k, &w, 16);
#pragma unroll
    for (int j = 0; j < VEC; ++j)
    {
      count_key(k[j]);
    }
  };
  if constexpr (NP <= 4)
  {
    for (; v + 3 * stride < nvec; v += 4 * stride)
    {
      uint4 w[4];
#pragma unroll
      for (int j = 0; j < 4; ++j)
      {
        w[j] = __ldcs(vkeys + v + j * stride);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j)
      {
        count_vec(w[j]);
      }
    }
  }
  else
  {
    // 16-bit counters: the CTA runs its first thread's trip count (the largest of its
    // threads; the others skip what they have not got) and folds the counters every FOLD
    // trips, before any half can pass 65535: a trip adds at most 4 * VEC keys per thread, so
    // 32 warps x 4 * VEC x FOLD, plus the head, tail and remainder keys of a thread (at most
    // 2 + 3 * VEC), stay below 2^16.
    constexpr unsigned FOLD = 32768u / (32u * 4u * VEC) - 1u;
    static_assert(32u * (4u * VEC * FOLD + 2u + 3u * VEC) < 65536u, "16-bit counters fold in time");
    const unsigned long long v0 = blockIdx.x * (unsigned long long) TPB;
    const unsigned long long trips =
      v0 + 3 * stride < nvec ? (nvec - 3 * stride - v0 + 4 * stride - 1) / (4 * stride) : 0ull;
    for (unsigned long long it = 0; it < trips; ++it)
    {
      if (v + 3 * stride < nvec)
      {
        uint4 w[4];
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
          w[j] = __ldcs(vkeys + v + j * stride);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
          count_vec(w[j]);
        }
        v += 4 * stride;
      }
      if ((it + 1) % FOLD == 0u)
      {
        __syncthreads();
        histogram_lanes_fold<TPB, NP>(table, totals);
        __syncthreads();
      }
    }
  }
  for (; v < nvec; v += stride)
  {
    count_vec(__ldcs(vkeys + v));
  }
  __syncthreads();
  histogram_lanes_fold<TPB, NP>(table, totals);
}

template <int KB, int FP, int TPB>
__device__ __forceinline__ void histogram_lanes_body(const HistogramParams& p)
{
  constexpr int R = RADIX_DIGITS;
  extern __shared__ __align__(16) unsigned char table[];
  __shared__ uint32_t sh[MAX_PASSES * R];
  if (!gate_open(p.gate))
  {
    return;
  }
  const int tid  = threadIdx.x;
  const int lane = tid & 31;
  const int P    = p.num_passes;
  const uint32_t table_bytes = uint32_t(histogram_table_bytes(P));
  for (uint32_t i = uint32_t(tid) * 16u; i < table_bytes; i += uint32_t(TPB) * 16u)
  {
    *reinterpret_cast<uint4*>(table + i) = make_uint4(0u, 0u, 0u, 0u);
  }
  for (int i = tid; i < MAX_PASSES * R; i += TPB)
  {
    sh[i] = 0u;
  }
  // byte 0 and byte 2 of every pass's counter offsets for this lane (layout above)
  uint32_t col[8];
  const bool packed = P > 4;
#pragma unroll
  for (int q = 0; q < 8; ++q)
  {
    col[q] = packed ? ((uint32_t(q >> 2) << 16) | (uint32_t((q >> 1) & 1) * 128u + uint32_t(lane) * 4u))
                    : ((uint32_t(q >> 1) << 16) | (uint32_t(q & 1) * 128u + uint32_t(lane) * 4u));
  }
  const uint32_t table_base = smem_addr(table);
  __syncthreads();

  // the pass count is a compile-time constant of the counting loop: a whole key, or a window;
  // the loop leaves the CTA's counts of (pass, digit) in sh
  if (p.begin_bit == 0 && p.end_bit == 8 * KB)
  {
    histogram_lanes_count<KB, FP, TPB, KB, false>(p, table, table_base, col, sh);
  }
  else
  {
    switch (P)
    {
      case 1: histogram_lanes_count<KB, FP, TPB, 1, true>(p, table, table_base, col, sh); break;
      case 2: if constexpr (KB >= 2) { histogram_lanes_count<KB, FP, TPB, 2, true>(p, table, table_base, col, sh); } break;
      case 3: if constexpr (KB >= 4) { histogram_lanes_count<KB, FP, TPB, 3, true>(p, table, table_base, col, sh); } break;
      case 4: if constexpr (KB >= 4) { histogram_lanes_count<KB, FP, TPB, 4, true>(p, table, table_base, col, sh); } break;
      case 5: if constexpr (KB >= 8) { histogram_lanes_count<KB, FP, TPB, 5, true>(p, table, table_base, col, sh); } break;
      case 6: if constexpr (KB >= 8) { histogram_lanes_count<KB, FP, TPB, 6, true>(p, table, table_base, col, sh); } break;
      case 7: if constexpr (KB >= 8) { histogram_lanes_count<KB, FP, TPB, 7, true>(p, table, table_base, col, sh); } break;
      default: if constexpr (KB >= 8) { histogram_lanes_count<KB, FP, TPB, 8, true>(p, table, table_base, col, sh); } break;
    }
  }
  histogram_finish<TPB>(p, sh);
}

// ---------------------------------------------------------------------------------------
// single tile: the whole LSD sort of <= TPB*ITEMS keys inside one CTA
// ---------------------------------------------------------------------------------------
template <int KB, int TPB, int ITEMS>
struct SingleTileSmem
{
  using U              = typename uint_of<KB>::type;
  static constexpr int NW   = TPB / 32;
  static constexpr int TILE = TPB * ITEMS;
  static constexpr size_t whist_off = 0;
  static constexpr size_t misc_off  = whist_off + sizeof(uint32_t) * NW * RADIX_DIGITS;
  static constexpr size_t kbuf_off  = misc_off + 128;
  static constexpr size_t ibuf_off  = kbuf_off + ((2 * sizeof(U) * TILE + 15) / 16) * 16;
  static constexpr size_t bytes     = ibuf_off + 2 * sizeof(uint16_t) * TILE;
};

// Sorts n <= TPB*ITEMS keys (and values) by bits [begin_bit, end_bit) inside one CTA.
// Reads keys_in/values_in, writes keys_out/values_out (which may alias the inputs: all
// reads complete before the first write). Starts with a CTA barrier so a persistent CTA
// can call it for one segment after another.
template <int KB, int VB, int FP, int TPB, int ITEMS, int BITS = RADIX_BITS>
__device__ __forceinline__ void block_sort_body(
  const void* keys_in,
  void* keys_out,
  const void* values_in,
  void* values_out,
  uint32_t num_items,
  int begin_bit,
  int end_bit,
  const KeyCodec& codec)
{
  using L            = SingleTileSmem<KB, TPB, ITEMS>;
  using U            = typename L::U;
  using V            = typename value_word<VB>::type;
  constexpr int NW   = L::NW;
  constexpr int TILE = L::TILE;
  constexpr int R    = 1 << BITS; // digits of one in-shared-memory pass
  static_assert(TPB >= R && BITS >= 5 && BITS <= RADIX_BITS, "one thread per digit, whole warps of digits");
  static_assert(TILE <= 65536, "16-bit source indices");

  extern __shared__ __align__(128) unsigned char smem[];
  uint32_t* whist = reinterpret_cast<uint32_t*>(smem + L::whist_off);
  uint32_t* misc  = reinterpret_cast<uint32_t*>(smem + L::misc_off);
  U* kbuf         = reinterpret_cast<U*>(smem + L::kbuf_off);
  uint16_t* ibuf  = reinterpret_cast<uint16_t*>(smem + L::ibuf_off);

  const int tid    = threadIdx.x;
  const int lane   = tid & 31;
  const int warp   = tid >> 5;
  const uint32_t n = num_items;
  const U* kin     = static_cast<const U*>(keys_in);

  __syncthreads();
  // warps whose keys are all padding keep them in place: they rank after every real key, and
  // their slots are never read, so only the active warps' slots are filled
  const int active_warps = int((n + ITEMS * 32 - 1) / (ITEMS * 32));
  const int filled       = active_warps * ITEMS * 32;
  U kor = U(0), kand = U(~U(0)); // over the real keys' digit sources
  for (int s = tid; s < filled; s += TPB)
  {
    U k = U(~U(0));
    if (uint32_t(s) < n)
    {
      k               = encode_key<U>(kin[s], codec);
      const U src_bits = digit_source<U, FP>(k);
      kor |= src_bits;
      kand &= src_bits;
    }
    kbuf[s] = k;
    ibuf[s] = uint16_t(s);
  }

  // Only bits that differ between two keys need a pass: a digit equal for every key gives
  // the identity permutation. Per-warp OR/AND go through whist before its first use.
  {
    uint32_t v[4] = {uint32_t(kor), uint32_t((unsigned long long) kor >> 32), uint32_t(kand),
                     uint32_t((unsigned long long) kand >> 32)};
    v[0] = __reduce_or_sync(0xffffffffu, v[0]);
    v[1] = __reduce_or_sync(0xffffffffu, v[1]);
    v[2] = __reduce_and_sync(0xffffffffu, v[2]);
    v[3] = __reduce_and_sync(0xffffffffu, v[3]);
    if (lane == 0)
    {
#pragma unroll
      for (int j = 0; j < 4; ++j)
      {
        whist[warp * 4 + j] = v[j];
      }
    }
  }
  __syncthreads();
  unsigned long long vary = 0;
  {
    unsigned long long o = 0, a = ~0ull;
#pragma unroll 1
    for (int w = 0; w < NW; ++w)
    {
      o |= (unsigned long long) whist[w * 4] | ((unsigned long long) whist[w * 4 + 1] << 32);
      a &= (unsigned long long) whist[w * 4 + 2] | ((unsigned long long) whist[w * 4 + 3] << 32);
    }
    const unsigned long long window =
      (end_bit >= 64 ? ~0ull : ((1ull << end_bit) - 1ull)) & ~((1ull << begin_bit) - 1ull);
    vary = (o ^ a) & window & (sizeof(U) == 8 ? ~0ull : 0xffffffffull);
  }
  __syncthreads(); // whist is zeroed by the first pass
  const int lo_bit = vary == 0 ? 0 : __ffsll((long long) vary) - 1;
  const int hi_bit = vary == 0 ? 0 : 64 - __clzll((long long) vary);

  int cur = 0;
  for (int bit = lo_bit; bit < hi_bit; bit += BITS)
  {
    const uint32_t dmask = (1u << min(BITS, hi_bit - bit)) - 1u;
    for (int i = tid; i < NW * R; i += TPB)
    {
      whist[i] = 0;
    }
    __syncthreads();

    const U* src       = kbuf + cur * TILE;
    U* dst             = kbuf + (cur ^ 1) * TILE;
    const uint16_t* is = ibuf + cur * TILE;
    uint16_t* id       = ibuf + (cur ^ 1) * TILE;
    const int wofs     = warp * ITEMS * 32 + lane;

    const bool active = warp < active_warps;
    U keys[ITEMS];
    if (active)
    {
#pragma unroll
      for (int i = 0; i < ITEMS; ++i)
      {
        keys[i] = src[wofs + i * 32];
      }
      warp_histogram<U, FP, ITEMS>(keys, whist + warp * R, bit, dmask);
    }
    __syncthreads();
    if (tid < R)
    {
      uint32_t tstart;
      block_digit_offsets<NW, R>(whist, misc + 8, &tstart);
    }
    __syncthreads();
    if (active)
    {
      uint32_t pos[ITEMS];
      __syncwarp(); // the warp votes below need a converged warp
      warp_rank_stable<U, FP, ITEMS, BITS>(keys, pos, whist + warp * R, bit, dmask);
#pragma unroll
      for (int i = 0; i < ITEMS; ++i)
      {
        dst[pos[i]] = keys[i];
        id[pos[i]]  = is[wofs + i * 32];
      }
    }
    __syncthreads();
    cur ^= 1;
  }

  U* kout              = static_cast<U*>(keys_out);
  const U* kfin        = kbuf + cur * TILE;
  const uint16_t* ifin = ibuf + cur * TILE;
  if constexpr (VB > 0)
  {
    // values may alias their source: gather into registers before any store
    constexpr int PER = (TILE + TPB - 1) / TPB;
    V vtmp[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j)
    {
      const uint32_t s = j * TPB + tid;
      if (s < n)
      {
        vtmp[j] = static_cast<const V*>(values_in)[ifin[s]];
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PER; ++j)
    {
      const uint32_t s = j * TPB + tid;
      if (s < n)
      {
        static_cast<V*>(values_out)[s] = vtmp[j];
      }
    }
  }
  for (uint32_t s = tid; s < n; s += TPB)
  {
    kout[s] = decode_key<U>(kfin[s], codec);
  }
}

template <int KB, int VB, int FP, int TPB, int ITEMS>
__device__ __forceinline__ void single_tile_body(const SingleTileParams& p)
{
  block_sort_body<KB, VB, FP, TPB, ITEMS>(
    p.keys_in, p.keys_out, p.values_in, p.values_out, p.num_items, p.begin_bit, p.end_bit, p.codec);
}

} // namespace gb300

#include "onesweep.cuh"
