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
constexpr uint32_t STATUS_BAD_SEGMENT      = 2u;

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

} // namespace gb300
