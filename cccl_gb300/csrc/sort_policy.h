// Tile configuration of the plain-path kernels per key/value width: the single source
// of truth for both the kernel instantiations and the host dispatcher (grid sizes,
// dynamic shared memory, temp-storage layout). Plain C++, usable from host and device.
//
// The reference's equivalent is the sm_100 onesweep tuning
// (cub/cub/device/dispatch/tuning/tuning_radix_sort.cuh:1743-1800): 384 threads and
// 12..23 items per thread under a 48 KB static shared-memory cap. GB300 kernels here use
// dynamic shared memory, so the staging tile is sized by registers, not by the 48 KB cap.
#pragma once

#include <cstddef>

#include "sort_params.h"

#if defined(__CUDACC__)
#  define GB300_HD __host__ __device__
#else
#  define GB300_HD
#endif

namespace gb300
{

constexpr int ONESWEEP_TPB     = 384; // CTA-per-tile fallback kernel
// Persistent onesweep kernel shape. The GB300_* macros let a tuning build override the
// shipped table (cccl_gb300/build.py passes GB300_TUNE_DEFINES to both compilers).
#ifndef GB300_PERSISTENT_MINB
#  define GB300_PERSISTENT_MINB 1
#endif
constexpr int PERSISTENT_MINB = GB300_PERSISTENT_MINB; // CTAs per SM the registers are sized for

// Threads per CTA of the persistent kernel: LOOKBACK_THREADS look-back threads (one per
// digit) plus the main threads that load, rank and write the tiles. Measured on GB300 with
// the autotuner (2^26 keys, one sort): keys-only runs best with 24 main warps of 14 items,
// pairs with 20 main warps and as many items as three tile buffers leave room for (the
// ranking is latency-bound, so more warps per SM pay until the registers run out).
constexpr int LOOKBACK_THREADS = 256;
GB300_HD constexpr int persistent_tpb(int kb, int vb)
{
#ifdef GB300_PERSISTENT_TPB
  return (void) kb, (void) vb, GB300_PERSISTENT_TPB;
#else
  return (void) kb, vb > 0 ? 896 : 1024;
#endif
}
// Predecessor rows the persistent kernel's look-back threads read per step: they have no
// other work, so they can keep more loads in flight than the CTA-per-tile kernel's.
#ifndef GB300_PERSISTENT_LOOKBACK_BATCH
#  define GB300_PERSISTENT_LOOKBACK_BATCH 8
#endif
constexpr int PERSISTENT_LOOKBACK_BATCH = GB300_PERSISTENT_LOOKBACK_BATCH;
GB300_HD constexpr int persistent_main(int kb, int vb)
{
  return persistent_tpb(kb, vb) - LOOKBACK_THREADS;
}
// Stable merge of two sorted runs (merge_kernels.cuh): one CTA per output tile.
constexpr int MERGE_TPB   = 256;
constexpr int MERGE_ITEMS = 8;
constexpr int MERGE_TILE  = MERGE_TPB * MERGE_ITEMS;
// A and B slices (one tile together) and the merged tile, keys and values each
GB300_HD constexpr size_t merge_smem_bytes(int kb, int vb)
{
  return 2 * size_t(MERGE_TILE) * (size_t(kb) + size_t(vb));
}
constexpr int SINGLE_TILE_TPB  = 512;
constexpr int SINGLE_TILE_ITEMS = 10;
constexpr int HISTOGRAM_TPB    = 512;
// CTAs per SM the CTA-table histogram's registers are sized for (32 registers a thread): it
// is bound by shared-memory atomics, and at 40 registers (three CTAs per SM) it ran 20-40 %
// slower. The plain sort uses the lane-column histogram below; this one serves the
// allocation-free entry point and the learned sort's bucket-id histogram.
constexpr int HISTOGRAM_MINB   = 4;

// Lane-column histogram of the plain sort (histogram_lanes_body): one CTA of 1024 threads per
// SM; every lane owns a column of counters per (pass, digit), so the 32 increments of one warp
// instruction hit 32 different banks. Up to 4 passes: 32-bit counters (32 KB a pass); 5 to 8
// passes: two passes share each 32-bit word as 16-bit halves (32 KB a pair of passes).
constexpr int HISTOGRAM_LANES_TPB = 1024;
GB300_HD constexpr size_t histogram_table_bytes(int passes)
{
  return passes <= 2 ? size_t(65536) : size_t(131072);
}

GB300_HD constexpr int onesweep_items(int kb, int vb)
{
  return vb >= 16 ? 8
       : kb == 8  ? (vb == 0 ? 16 : 12)
       : kb == 4  ? (vb == 0 ? 20 : vb <= 4 ? 16 : 12)
                  : 16;
}

GB300_HD constexpr size_t round16(size_t x)
{
  return (x + 15) / 16 * 16;
}

GB300_HD constexpr size_t value_word_bytes(int vb)
{
  return vb == 0 ? 4 : size_t(vb);
}

// Dynamic shared memory of the onesweep kernel: per-warp digit counters, per-digit
// global deltas, a misc block, the key staging tile and (pairs) the value staging tile.
GB300_HD constexpr size_t onesweep_smem_for(int kb, int vb, int tpb, int items)
{
  return size_t(4) * (tpb / 32) * 256 + size_t(8) * 256 + 128 + round16(size_t(kb) * tpb * items)
       + (vb > 0 ? value_word_bytes(vb) * tpb * items : 0);
}

GB300_HD constexpr size_t onesweep_smem_bytes(int kb, int vb)
{
  return size_t(4) * (ONESWEEP_TPB / 32) * 256 + size_t(8) * 256 + 128
       + round16(size_t(kb) * ONESWEEP_TPB * onesweep_items(kb, vb))
       + (vb > 0 ? value_word_bytes(vb) * ONESWEEP_TPB * onesweep_items(kb, vb) : 0);
}

// Items per main thread of the persistent onesweep kernel: the three tile buffers (keys +
// values) must fit the 227 KB of shared memory next to the per-warp counters.
GB300_HD constexpr int persistent_items_nominal(int kb, int vb)
{
#ifdef GB300_PERSISTENT_ITEMS
  return (void) kb, (void) vb, GB300_PERSISTENT_ITEMS;
#else
  return vb > 0 ? 16 : kb == 8 ? 12 : kb == 4 ? 14 : 16;
#endif
}

GB300_HD constexpr size_t persistent_smem_for(int kb, int vb, int items)
{
  return size_t(4) * (persistent_main(kb, vb) / 32) * 256 + size_t(8) * 256 + 128
       + 3 * (round16(size_t(kb) * persistent_main(kb, vb) * items)
              + (vb > 0 ? value_word_bytes(vb) * persistent_main(kb, vb) * items : 0));
}

// Nominal items, reduced until PERSISTENT_MINB CTAs fit in 227 KB of shared memory.
GB300_HD constexpr int persistent_items(int kb, int vb)
{
  int items = persistent_items_nominal(kb, vb);
  while (items > 1 && persistent_smem_for(kb, vb, items) * PERSISTENT_MINB > size_t(227) * 1024)
  {
    --items;
  }
  return items;
}

GB300_HD constexpr size_t persistent_smem_bytes(int kb, int vb)
{
  return persistent_smem_for(kb, vb, persistent_items(kb, vb));
}

// Keys per tile of the persistent kernel.
GB300_HD constexpr unsigned long long persistent_tile_items(int tpb, int items)
{
  return (unsigned long long) (tpb - LOOKBACK_THREADS) * items;
}

// PLAN_* words of a plain sort's digit passes (see sort_params.h) from the passes whose
// digit is the same for every key (bit q of trivial_mask). Runs on the device (one thread
// of the histogram's last CTA) and on the host (the CPU test of every mask).
GB300_HD inline void plan_pass_words(uint32_t* plan, int num_passes, int plan_mode, uint32_t trivial_mask)
{
  auto popcount = [](uint32_t x) {
    int c = 0;
    for (; x != 0u; x &= x - 1u)
    {
      ++c;
    }
    return c;
  };
  const int P        = num_passes;
  const uint32_t all = (1u << P) - 1u;
  trivial_mask &= all;
  uint32_t run     = ~trivial_mask & all; // passes that run
  const int k0     = popcount(run);
  const bool extra = plan_mode == PLAN_MODE_DOUBLE ? ((k0 & 1) != (P & 1)) : (k0 == 0);
  if (extra)
  {
    run |= trivial_mask & (0u - trivial_mask); // the first skippable pass runs too
  }
  const int k  = popcount(run);
  int j        = 0;
  int prev_dst = 0;
  for (int q = 0; q < P; ++q)
  {
    uint32_t w = PLAN_SKIP;
    if ((run >> q) & 1u)
    {
      int src, dst;
      if (plan_mode == PLAN_MODE_DOUBLE)
      {
        src = j & 1;
        dst = (j + 1) & 1;
      }
      else
      {
        src = j == 0 ? 0 : prev_dst;
        dst = ((k - 1 - j) % 2 == 0) ? 1 : 2; // the last pass writes the output
      }
      w = (uint32_t(src) << PLAN_SRC_SHIFT) | (uint32_t(dst) << PLAN_DST_SHIFT) | (j == 0 ? PLAN_ENCODE : 0u)
        | (j == k - 1 ? PLAN_DECODE : 0u);
      prev_dst = dst;
      ++j;
    }
    plan[q] = w;
  }
}

GB300_HD constexpr int single_tile_capacity()
{
  return SINGLE_TILE_TPB * SINGLE_TILE_ITEMS;
}

GB300_HD constexpr size_t single_tile_smem_bytes(int kb)
{
  return size_t(4) * (SINGLE_TILE_TPB / 32) * 256 + 128 + round16(size_t(2) * kb * single_tile_capacity())
       + size_t(2) * 2 * single_tile_capacity();
}

// Largest input CUB sorts with its single-tile kernel (256 threads x 19 items scaled
// by the dominant type size, tuning_radix_sort.cuh:1833-1841 and scale_reg_bound in
// cub/cub/util_arch.cuh:128-139). Using the same cut keeps the returned DoubleBuffer
// selector identical to CUB's.
GB300_HD constexpr unsigned long long cub_single_tile_limit(int key_bytes, int value_bytes)
{
  const int dom   = key_bytes > value_bytes ? key_bytes : value_bytes;
  const int items = (19 * 4 / (dom > 4 ? dom : 4)) > 1 ? (19 * 4 / (dom > 4 ? dom : 4)) : 1;
  const int t     = ((48 * 1024 / (dom * items)) + 31) / 32 * 32;
  const int tpb   = t < 256 ? t : 256;
  return (unsigned long long) tpb * items;
}

static_assert(cub_single_tile_limit(4, 0) == 4864, "CUB single-tile cut, 4-byte keys");
static_assert(cub_single_tile_limit(8, 4) == 2304, "CUB single-tile cut, 8-byte keys");
static_assert(cub_single_tile_limit(4, 16) == 1024, "CUB single-tile cut, 16-byte values");
static_assert(persistent_smem_bytes(8, 8) * PERSISTENT_MINB <= 227 * 1024
                && persistent_smem_bytes(8, 16) * PERSISTENT_MINB <= 227 * 1024
                && persistent_smem_bytes(4, 16) * PERSISTENT_MINB <= 227 * 1024
                && persistent_smem_bytes(2, 16) * PERSISTENT_MINB <= 227 * 1024,
              "persistent tile buffers exceed shared memory");

} // namespace gb300

// ---- batched segmented sort: size classes ----
namespace gb300
{
// CUB's sub-warp network shapes for cc >= 8.6 (tuning_segmented_sort.cuh:182-195, items
// scaled as cub/cub/util_math.cuh:54-57). They fix the bit-exact NaN placement, so they
// are not tuning knobs here.
GB300_HD constexpr int seg_scale_items(int nominal, int dominant)
{
  return (nominal * 4 / dominant) < 1 ? 1 : (nominal * 4 / dominant) > nominal ? nominal : (nominal * 4 / dominant);
}
GB300_HD constexpr int seg_dominant(int kb, int vb)
{
  return kb > vb ? kb : vb;
}
GB300_HD constexpr int seg_small_threads(int kb, int vb)
{
  return seg_dominant(kb, vb) > 4 ? 8 : 2;
}
GB300_HD constexpr int seg_small_items(int kb, int vb)
{
  return seg_scale_items(seg_dominant(kb, vb) > 4 ? 7 : 9, seg_dominant(kb, vb));
}
GB300_HD constexpr int seg_medium_threads(int, int)
{
  return 16;
}
GB300_HD constexpr int seg_medium_items(int kb, int vb)
{
  return seg_scale_items(seg_dominant(kb, vb) > 4 ? 9 : 7, seg_dominant(kb, vb));
}
constexpr int SEG_PARTITION_THRESHOLD = 500; // dispatch_segmented_sort.cuh:465

// The same networks in radix order (segmented radix sort, learned buckets) are not tied to
// CUB's shapes: 8 lanes x 8 keys and a full warp x 8 keys.
constexpr int SEG_RSMALL_THREADS  = 8;
constexpr int SEG_RSMALL_ITEMS    = 8;
constexpr int SEG_RMEDIUM_THREADS = 32;
constexpr int SEG_RMEDIUM_ITEMS   = 8;

// Block classes (free of the reference): one CTA sorts one segment in shared memory, by a
// stable merge sort or by LSD radix passes; the algorithm and shape per key width come from
// measurements on GB300 (the GB300_SEG_BLOCK_* macros override them in tuning builds).
// Measured (2^28 keys in ~4096-key segments, block_l time): 4-byte keys radix 512x16 4.57 ms,
// with 2 CTAs/SM 3.40 ms, 1024x8 4.41 ms, merge 11.4 ms; 8-byte keys radix 512x16 10.4 ms,
// 2 CTAs/SM 14.2 ms, 1024x8 10.1 ms, merge 14.2 ms.
constexpr int SEG_BLOCK_S_CAP = 2048;
constexpr int SEG_BLOCK_L_CAP = 8192;
constexpr int SEG_BLOCK_RADIX = 0;
constexpr int SEG_BLOCK_MERGE = 1;
GB300_HD constexpr int seg_block_algo(int kb)
{
#ifdef GB300_SEG_BLOCK_ALGO
  return (void) kb, GB300_SEG_BLOCK_ALGO;
#else
  return (void) kb, SEG_BLOCK_RADIX; // measured: radix beats merge for 4- and 8-byte keys too
#endif
}
// CTAs per SM the block-class registers are sized for
GB300_HD constexpr int seg_block_minb(int kb)
{
#ifdef GB300_SEG_BLOCK_MINB
  return (void) kb, GB300_SEG_BLOCK_MINB;
#else
  return kb == 4 ? 2 : 1;
#endif
}
// block_s (256 threads) sized for more CTAs per SM than block_l: its segments are short and
// its CTAs spend most of their time in barriers, so resident CTAs hide each other's waits.
// 4-byte keys with values of up to 4 bytes: 48 registers, five CTAs per SM (64 registers held
// it at four; with 8-byte values 48 registers spill).
GB300_HD constexpr int seg_block_s_minb(int kb, int vb)
{
#ifdef GB300_SEG_BLOCK_S_MINB
  return (void) kb, (void) vb, GB300_SEG_BLOCK_S_MINB;
#else
  return kb == 4 && vb <= 4 ? 5 : seg_block_minb(kb);
#endif
}
GB300_HD constexpr int seg_block_s_items(int kb)
{
  return (void) kb, 8;
}
GB300_HD constexpr int seg_block_l_items(int kb)
{
#ifdef GB300_SEG_BLOCK_L_ITEMS
  return (void) kb, GB300_SEG_BLOCK_L_ITEMS;
#else
  return seg_block_algo(kb) == SEG_BLOCK_MERGE || kb == 8 ? 8 : 16;
#endif
}
// Digit bits of one in-shared-memory radix pass of the block classes (5 to 8): fewer bits
// cost fewer ballots per key and smaller counter rows, more passes. Picked per key width and
// class by the autotuner (cccl_gb300/tuning_gb300.json, group "blockbits"); measured on
// GB300 (block_s / block_l time), 8 / 7 / 6 / 5 bits: f32+i32 0.328 / 0.332 / 0.345 / 0.425
// and 0.676 / 0.708 / 0.751 / 0.869 ms; f64+i64 0.856 / 0.908 / 0.922 / 1.006 and 1.664 /
// 1.812 / 1.853 / 2.078 ms. Eight bits win for both widths and both classes.
GB300_HD constexpr int seg_block_s_bits(int kb)
{
#ifdef GB300_SEG_BLOCK_S_BITS
  return (void) kb, GB300_SEG_BLOCK_S_BITS;
#else
  return (void) kb, 8;
#endif
}
GB300_HD constexpr int seg_block_l_bits(int kb)
{
#ifdef GB300_SEG_BLOCK_L_BITS
  return (void) kb, GB300_SEG_BLOCK_L_BITS;
#else
  return (void) kb, 8;
#endif
}
GB300_HD constexpr int seg_block_s_tpb(int kb)
{
  return SEG_BLOCK_S_CAP / seg_block_s_items(kb);
}
GB300_HD constexpr int seg_block_l_tpb(int kb)
{
  return SEG_BLOCK_L_CAP / seg_block_l_items(kb);
}
// block_xs: segments longer than the medium network's tile and up to 512 keys, one CTA of
// 256 threads x 2 keys each (one thread per digit, as every block pass needs). Small
// registers and shared memory keep eight CTAs resident per SM (four-byte keys), against four
// or five of block_s, whose 2048-key tile would be mostly padding for these segments.
constexpr int SEG_BLOCK_XS_CAP = 512;
GB300_HD constexpr int seg_block_xs_items(int kb)
{
  return (void) kb, 2;
}
GB300_HD constexpr int seg_block_xs_tpb(int kb)
{
  return SEG_BLOCK_XS_CAP / seg_block_xs_items(kb);
}
GB300_HD constexpr int seg_block_xs_minb(int kb)
{
#ifdef GB300_SEG_BLOCK_XS_MINB
  return (void) kb, GB300_SEG_BLOCK_XS_MINB;
#else
  return kb == 8 ? 6 : 8;
#endif
}
constexpr int SEG_NETWORK_TPB   = 256;
// Device-class digit pass (CTA per tile): threads and items per thread; GB300_SEG_PASS_*
// override them in tuning builds. Measured (cccl_gb300/autotune.py, cccl_gb300/tuning_gb300.json,
// lognormal segments of 2^26 keys, seg_pass time per sort): f32+i32 384x16 1.56 (shipped
// before) / 384x12 2.19 / 512x12 1.73 / 1024x8 1.57 ms; f64+i64 384x12 4.93 / 512x12 4.24 /
// 1024x8 4.13 ms (with a few spilled registers, still the fastest).
GB300_HD constexpr int seg_pass_tpb(int kb, int vb)
{
#ifdef GB300_SEG_PASS_TPB
  return (void) kb, (void) vb, GB300_SEG_PASS_TPB;
#else
  return (void) kb, (void) vb, 1024;
#endif
}
GB300_HD constexpr int seg_pass_items(int kb, int vb)
{
#ifdef GB300_SEG_PASS_ITEMS
  return (void) kb, (void) vb, GB300_SEG_PASS_ITEMS;
#else
  return (void) kb, (void) vb, 8;
#endif
}

// Pipelined device-class pass (seg_device_persistent_body): the persistent pass's threads,
// and as many items as three tile buffers with 32 bytes of alignment slack each (keys and
// values) leave room for.
GB300_HD constexpr int seg_ppass_tpb(int kb, int vb)
{
  return persistent_tpb(kb, vb);
}
GB300_HD constexpr size_t seg_persistent_smem_for(int kb, int vb, int tpb, int items)
{
  return size_t(4) * ((tpb - LOOKBACK_THREADS) / 32) * 256 + size_t(8) * 256 + 128 + 256
       + 3 * (round16(size_t(kb) * (tpb - LOOKBACK_THREADS) * items) + 32
              + (vb > 0 ? round16(value_word_bytes(vb) * (tpb - LOOKBACK_THREADS) * items) + 32 : 0));
}
GB300_HD constexpr int seg_ppass_items(int kb, int vb)
{
  // 4-byte keys: capped where the plain pass's item counts spill registers here (the tile
  // geometry and the offset reads take a few more): 14 keys-only and 13 with values spill
#ifdef GB300_SEG_PPASS_ITEMS
  int items = GB300_SEG_PPASS_ITEMS;
#else
  int items = kb == 4 ? (vb == 0 ? 13 : vb == 4 ? 12 : persistent_items_nominal(kb, vb)) : persistent_items_nominal(kb, vb);
#endif
  while (items > 1 && seg_persistent_smem_for(kb, vb, seg_ppass_tpb(kb, vb), items) > size_t(227) * 1024)
  {
    --items;
  }
  return items;
}
GB300_HD constexpr size_t seg_ppass_smem(int kb, int vb)
{
  return seg_persistent_smem_for(kb, vb, seg_ppass_tpb(kb, vb), seg_ppass_items(kb, vb));
}
} // namespace gb300

namespace gb300
{
GB300_HD constexpr size_t seg_network_smem(int kb, int vb, int threads, int items)
{
  return size_t(SEG_NETWORK_TPB / 32) * size_t(32 / threads)
       * (round16(size_t(kb) * (threads * items + 1)) + (vb > 0 ? round16(value_word_bytes(vb) * (threads * items + 1)) : 0));
}
GB300_HD constexpr size_t block_sort_smem(int kb, int tpb, int items)
{
  return size_t(4) * (tpb / 32) * 256 + 128 + round16(size_t(2) * kb * tpb * items) + size_t(2) * 2 * tpb * items;
}
GB300_HD constexpr size_t block_merge_smem(int kb, int tpb, int items)
{
  return round16(size_t(kb) * (size_t(tpb) * items + size_t(tpb) * items / (kb == 8 ? 16 : 32) + 1))
       + round16(size_t(2) * (size_t(tpb) * items + 2 * (size_t(tpb) * items / 64) + 2));
}
GB300_HD constexpr size_t seg_block_smem(int kb, int tpb, int items)
{
  return seg_block_algo(kb) == SEG_BLOCK_MERGE ? block_merge_smem(kb, tpb, items) : block_sort_smem(kb, tpb, items);
}
} // namespace gb300

// ---- learned-partition sort ----
namespace gb300
{
// The partition pass is the persistent onesweep pass plus one shared-memory region: the
// model's tables (knot, slope, intercept per leaf) and the staged digit of every tile slot.
// Shared-memory copy of the model: 16-byte leaves, the cell table, kmin and shift.
GB300_HD constexpr size_t learned_tables_bytes()
{
  return size_t(16) * LEARNED_LEAVES + round16(size_t(LEARNED_CELLS) + 16) + 16;
}

GB300_HD constexpr size_t learned_extra_bytes(int kb, int vb, int items)
{
  return (void) kb, learned_tables_bytes() + round16(size_t(persistent_main(kb, vb)) * items);
}

// Items per main thread of the partition pass before the shared-memory fit: the pass holds
// the computed digits in registers beside the keys, values and positions, so 4-byte keys with
// 4-byte values take 10 (12, the shared-memory bound, spilled 84 bytes per thread).
GB300_HD constexpr int learned_items_nominal(int kb, int vb)
{
  return kb == 4 && vb == 4 && persistent_items_nominal(kb, vb) > 10 ? 10 : persistent_items_nominal(kb, vb);
}

GB300_HD constexpr int learned_items(int kb, int vb)
{
  int items = learned_items_nominal(kb, vb);
  while (items > 1
         && (persistent_smem_for(kb, vb, items) + learned_extra_bytes(kb, vb, items)) * PERSISTENT_MINB
              > size_t(227) * 1024)
  {
    --items;
  }
  return items;
}

GB300_HD constexpr size_t learned_pass_smem(int kb, int vb)
{
  return persistent_smem_for(kb, vb, learned_items(kb, vb)) + learned_extra_bytes(kb, vb, learned_items(kb, vb));
}

constexpr int LEARNED_FIT_TPB    = LEARNED_SAMPLE / LEARNED_LEAVES; // one sample point per thread
// Keys per lane of the bucket-bounds kernel, all loaded before the first is used: 16 for
// 4-byte keys; 8 for 8-byte keys, whose 16 took 82 registers and a quarter of the warps
// (f64 at 2^30: 4.7 against 4.0 ms with one key per lane at a time).
GB300_HD constexpr int learned_bounds_items(int kb)
{
  return kb == 8 ? 8 : 16;
}
// Smallest input the learned path takes; below it the plain radix sort runs.
constexpr unsigned long long LEARNED_MIN_ITEMS = 1ull << 20;
// Target keys per bucket: 2048 or 4096 (learned_bucket_items_log2). 64-key buckets of 8-byte
// keys (one more partition pass, radix-order merge networks of 8 x 8 and 32 x 8 keys)
// measured slower on GB300: f64 + i64 at 2^30, 102 ms against 81 ms.

// Bucket sort of the learned path (one bucket per CTA at a time): buckets
// of up to CAP keys are sorted by one counting pass on their top varying bits with as many
// bins as keys, then every run of equal bins (at most LEARNED_RUN_MAX keys) is ordered by
// comparison. Larger buckets and longer runs go to the segmented radix sort. CAP is twice
// the target bucket size: 2048-key buckets (CAP 4096) unless that costs a partition pass,
// else 4096-key buckets (CAP 8192).
constexpr int LEARNED_RUN_MAX = 32;
// 8 keys per thread: 512 threads for CAP 4096 (two CTAs per SM), 1024 for CAP 8192
GB300_HD constexpr int learned_bucket_tpb(int cap)
{
  return cap / 8;
}
template <int KB, int VB, int CAP>
struct LearnedBucketSmem
{
  static constexpr size_t kraw_off = 0;
  static constexpr size_t vst_off  = round16(size_t(KB) * CAP);
  static constexpr size_t bins_off = vst_off + round16(size_t(VB) * CAP);
  static constexpr size_t perm_off = bins_off + size_t(4) * CAP;
  static constexpr size_t bytes    = perm_off + size_t(2) * CAP;
};
GB300_HD constexpr size_t learned_bucket_smem(int kb, int vb, int cap)
{
  return round16(size_t(kb) * cap) + round16(size_t(vb) * cap) + size_t(4) * cap + size_t(2) * cap;
}
// log2 of the target bucket size for log2n = ceil(log2(num_items)): 2048-key buckets when
// that needs no more partition passes than 4096-key buckets, else 4096.
GB300_HD constexpr int learned_bucket_items_log2(int log2n)
{
#ifdef GB300_LEARNED_ITEMS_LOG2
  if (GB300_LEARNED_ITEMS_LOG2 == 11 || GB300_LEARNED_ITEMS_LOG2 == 12)
  {
    return GB300_LEARNED_ITEMS_LOG2; // tuning builds
  }
#endif
  const int b11 = log2n - 11 < 8 ? 8 : (log2n - 11 > LEARNED_MAX_BUCKET_LOG2 ? LEARNED_MAX_BUCKET_LOG2 : log2n - 11);
  const int b12 = log2n - 12 < 8 ? 8 : (log2n - 12 > LEARNED_MAX_BUCKET_LOG2 ? LEARNED_MAX_BUCKET_LOG2 : log2n - 12);
  return (b11 + 7) / 8 == (b12 + 7) / 8 ? 11 : 12;
}
} // namespace gb300
