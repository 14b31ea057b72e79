// Launch parameter blocks shared by the host dispatcher and the kernels. Every kernel
// takes exactly one of these structs by value, so the driver-API launch packs a single
// argument pointer. Plain C++ only: no CUDA headers, included from host and device code.
#pragma once

#include <cstdint>

namespace gb300
{

constexpr int RADIX_BITS    = 8;
constexpr int RADIX_DIGITS  = 1 << RADIX_BITS;
constexpr int MAX_PASSES    = 8; // 64-bit keys
constexpr uint64_t LOOKBACK_TIMEOUT_NS = 1000000000ull; // 1 s
constexpr int LOOKBACK_BATCH = 8; // predecessor rows read per look-back step

// Status word bits reported by the kernels (OR-ed into SortControl::status).
constexpr uint32_t STATUS_LOOKBACK_TIMEOUT = 1u;
constexpr uint32_t STATUS_BAD_SEGMENT      = 2u; // a segment outside the keys (left unsorted)
constexpr uint32_t STATUS_SEG_CAPACITY     = 4u; // overlapping segments exceeded the plan: large ones skipped

// Bit-order codec. encoded = raw ^ (raw & H ? fwd_neg : fwd_pos);
// raw = encoded ^ (encoded & H ? inv_set : inv_clr). Only the low key-width bits are used.
struct KeyCodec
{
  unsigned long long fwd_pos;
  unsigned long long fwd_neg;
  unsigned long long inv_set;
  unsigned long long inv_clr;
};

// Per-call control block at the start of temp storage; zeroed by the init kernel.
struct SortControl
{
  unsigned long long counts[MAX_PASSES * RADIX_DIGITS]; // all-pass digit histogram
  uint32_t hist_done;                                   // CTAs finished in the histogram
  uint32_t status;                                      // STATUS_* bits
  uint32_t pad[2];
  // followed by tile counters, one per (pass, portion)
};

struct InitParams
{
  uint32_t* words;
  unsigned long long num_words;
};

struct HistogramParams
{
  const void* keys;
  unsigned long long num_items;
  KeyCodec codec;
  int begin_bit;
  int end_bit;
  int num_passes;
  int num_portions;
  SortControl* ctrl;
  unsigned long long* bins;   // [pass][portion][digit], portion 0 written here
  uint32_t* lookback_clear;   // look-back buffer of pass 0, zeroed here
  unsigned long long lookback_words;
};

struct OnesweepParams
{
  const void* keys_in;        // portion-relative
  void* keys_out;             // absolute (whole array)
  const void* values_in;      // portion-relative
  void* values_out;           // absolute
  unsigned long long portion_begin;
  unsigned long long num_items_total; // bound of every output index
  uint32_t portion_items;
  uint32_t portion_tiles;
  uint32_t tile_row_base;     // first look-back row of this portion
  uint32_t pad0;
  uint32_t* lookback;         // [row][digit] for this pass
  uint32_t* lookback_next;    // buffer of the next pass; this pass zeroes its rows
  uint32_t* tile_counter;
  const unsigned long long* bins;   // [digit] global base of this pass and portion
  unsigned long long* bins_next;    // [digit] base of the next portion, or null
  uint32_t* status;
  KeyCodec codec;
  int current_bit;
  int num_bits;
  int encode_in;              // first pass: raw keys are encoded on load
  int decode_out;             // last pass: keys are decoded on store
};

struct SingleTileParams
{
  const void* keys_in;
  void* keys_out;
  const void* values_in;
  void* values_out;
  uint32_t num_items;
  int begin_bit;
  int end_bit;
  int pad0;
  KeyCodec codec;
};

// ---- batched segmented sort ----
constexpr int SEG_MAX_PASSES = 12; // 8-bit digits, plus one split pass to match CUB's buffer parity

struct DeviceSegment
{
  unsigned long long begin;
  uint32_t size;
  uint32_t tile_base;
};

struct SegClassifyParams
{
  const void* begin_offsets;
  const void* end_offsets;
  int offsets_64;
  int partition; // more than 500 segments: small segments get their own network
  unsigned long long num_segments;
  unsigned long long num_items;           // segments reaching past it are rejected
  unsigned long long max_device_segments; // capacity of device_list (temp-storage plan)
  unsigned long long max_tiles;           // capacity of tile_segment
  long long small_tile;
  long long medium_tile;
  long long block_small_cap;
  long long block_large_cap;
  uint32_t device_tile;
  uint32_t pad0;
  uint32_t* counters;
  uint32_t* small_list;
  uint32_t* medium_list;
  uint32_t* block_s_list;
  uint32_t* block_l_list;
  DeviceSegment* device_list;
  uint32_t* tile_segment;
  uint32_t* status;
};

struct SegSortParams
{
  const void* keys_in;
  void* keys_out; // final buffer (may alias keys_in)
  const void* values_in;
  void* values_out;
  const void* begin_offsets;
  const void* end_offsets;
  int offsets_64;
  int descending;
  uint32_t* counters;
  const uint32_t* small_list;
  const uint32_t* medium_list;
  const uint32_t* block_s_list;
  const uint32_t* block_l_list;
  KeyCodec codec;
};

struct SegDeviceParams
{
  const void* keys_in; // original keys (histogram)
  const void* keys_src[SEG_MAX_PASSES];
  void* keys_dst[SEG_MAX_PASSES];
  const void* values_src[SEG_MAX_PASSES];
  void* values_dst[SEG_MAX_PASSES];
  unsigned long long num_items;
  int num_passes;
  int pass; // the pass a pass-kernel launch performs
  int pass_bit[SEG_MAX_PASSES];
  int pass_bits[SEG_MAX_PASSES];
  uint32_t device_tile;
  uint32_t pad0;
  uint32_t* counters;
  const DeviceSegment* device_list;
  const uint32_t* tile_segment;
  uint32_t* seg_counts;
  unsigned long long* seg_bins;
  uint32_t* lookback[2];
  uint32_t* status;
  KeyCodec codec;
};

} // namespace gb300
