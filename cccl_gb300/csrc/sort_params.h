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
constexpr uint64_t LOOKBACK_TIMEOUT_NS = 1000000000ull; // 1 s: the limit of every bounded wait
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

// Per-call control block at the start of temp storage; zeroed by the init kernel. The
// status word comes first: word 0 of every sort's temporary storage is its status word
// (read by cccl_gb300_sort_status).
struct SortControl
{
  uint32_t status;                                      // STATUS_* bits
  uint32_t hist_done;                                   // CTAs finished in the histogram
  uint32_t pad[2];
  unsigned long long counts[MAX_PASSES * RADIX_DIGITS]; // all-pass digit histogram
  uint32_t plan[MAX_PASSES];                            // PLAN_* word of every digit pass
  // followed by tile counters, one per (pass, portion)
};
static_assert(sizeof(uint32_t) * 4 + sizeof(unsigned long long) * MAX_PASSES * RADIX_DIGITS
                  + sizeof(uint32_t) * MAX_PASSES == 16432,
              "SortControl layout");

// Pass plan of a plain sort, one word per digit pass, written by the histogram's last CTA.
// A pass whose digit is the same for every key (one digit holds all n keys) is the identity
// permutation and is skipped; the passes that run take their buffers in turn, the first of
// them encodes and the last decodes. When the passes that run would leave the result in
// another buffer than the one every pass running would (the selector CUB reports), the first
// skippable pass runs as well (a single-digit pass: its tiles are copied in order).
constexpr uint32_t PLAN_SKIP       = 1u << 0;
constexpr uint32_t PLAN_ENCODE     = 1u << 1; // first pass that runs: raw keys are encoded on load
constexpr uint32_t PLAN_DECODE     = 1u << 2; // last pass that runs: keys are decoded on store
constexpr int PLAN_SRC_SHIFT       = 8;       // 2-bit index into OnesweepParams::key_bufs / value_bufs
constexpr int PLAN_DST_SHIFT       = 10;
constexpr int PLAN_MODE_NONE       = 0;       // no plan: every pass runs as launched
constexpr int PLAN_MODE_DOUBLE     = 1;       // buffers {current, alternate}: pass j reads j & 1
constexpr int PLAN_MODE_SEPARATE   = 2;       // buffers {input, output, temporary}: the last pass writes the output

// Optional launch gate of the plain-path kernels: with gate non-null a kernel does its
// work only if (*gate & gate_mask) != 0, a flag an earlier kernel of the same stream set.
struct KernelGate
{
  const uint32_t* gate;
  uint32_t gate_mask;
  uint32_t pad0;
};

// Folds the bits `mask` of a sub-sort's status word into its caller's (one thread).
struct StatusFoldParams
{
  uint32_t* dst;
  const uint32_t* src;
  uint32_t mask;
  uint32_t pad0;
};

// Values of widths the kernels do not carry: sorted as 32-bit indices, then gathered.
constexpr uint32_t VALUES_SKIP = 0xffffffffu; // index of a position the sort did not write

struct ValuesIotaParams
{
  uint32_t* out;
  unsigned long long n;
};

struct ValuesGatherParams
{
  const void* src;
  void* dst;
  const uint32_t* idx;
  unsigned long long n;
  uint32_t width; // bytes per value
  uint32_t word;  // bytes per copy: divides width and both buffers' alignment
};

struct InitParams
{
  uint32_t* words;
  unsigned long long num_words;
  KernelGate gate;
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
  KernelGate gate;
  uint32_t* plan;             // [num_passes] pass plan words to write, or null (no skipping)
  int plan_mode;              // PLAN_MODE_*
  int pad0;
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
  KernelGate gate;
  // Pass plan (null: the pass runs with the buffers above). With a plan the pass reads its
  // PLAN_* word: a skipped pass only clears its rows of lookback_next, and only when the
  // previous pass ran (plan_prev: that pass's word, null for the first pass, which always
  // clears); a pass that runs takes keys_in / keys_out / values_in / values_out from these
  // tables by the word's indices, and encode_in / decode_out from its flags.
  const uint32_t* plan;
  const void* key_bufs[3];    // whole arrays
  const void* value_bufs[3];
  const uint32_t* plan_prev;
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

// Counter words at the start of the segmented sort's temporary storage (zeroed per call).
enum : uint32_t
{
  SEG_CTR_STATUS = 0, // STATUS_* bits: word 0 of the temporary storage, as in every sort
  SEG_CTR_SMALL,      // segments per class
  SEG_CTR_MEDIUM,
  SEG_CTR_BLOCK_S,
  SEG_CTR_BLOCK_L,
  SEG_CTR_DEVICE,
  SEG_CTR_DEVICE_TILES,
  SEG_CTR_TICKET_SMALL,
  SEG_CTR_TICKET_MEDIUM,
  SEG_CTR_TICKET_BLOCK_S,
  SEG_CTR_TICKET_BLOCK_L,
  SEG_CTR_TICKET_HIST,
  SEG_CTR_TICKET_SCAN,
  SEG_CTR_BLOCK_XS, // block class of the shortest segments (256 threads x 2 keys)
  SEG_CTR_TICKET_BLOCK_XS,
  SEG_CTR_TICKET_PASS0, // one per device pass
  SEG_CTR_DEVICE_ITEMS = 30, // u64 (two words, 8-byte aligned): keys in device-class segments
  SEG_CTR_WORDS        = 32
};
static_assert(SEG_CTR_TICKET_PASS0 + SEG_MAX_PASSES <= SEG_CTR_DEVICE_ITEMS, "segmented counter words overlap");

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
  long long block_xs_cap;
  long long block_small_cap;
  long long block_large_cap;
  uint32_t device_tile;
  uint32_t pad0;
  uint32_t* counters;
  uint32_t* small_list;
  uint32_t* medium_list;
  uint32_t* block_xs_list;
  uint32_t* block_s_list;
  uint32_t* block_l_list;
  DeviceSegment* device_list;
  uint32_t* tile_segment;
  uint32_t* status;
  uint32_t* seg_counts; // [max_device_segments][num_passes][256]: a device segment's row is zeroed here
  int num_passes;
  int pad1;
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
  const uint32_t* block_xs_list;
  const uint32_t* block_s_list;
  const uint32_t* block_l_list;
  KeyCodec codec;
  int begin_bit; // key bits the block classes sort by
  int end_bit;
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

// ---- stable merge of two sorted runs (merge_kernels.cuh) ----
struct MergeParams
{
  const void* a_keys; // run A: earlier in the stable order of equal keys
  const void* b_keys;
  const void* a_values; // null for keys-only
  const void* b_values;
  void* out_keys; // na + nb items, A and B merged
  void* out_values;
  unsigned long long na;
  unsigned long long nb;
  KeyCodec codec;
  unsigned long long* splits; // A items before every tile's first output: [tiles + 1]
};

// ---- learned-partition sort ----
constexpr int LEARNED_SAMPLE_LOG2 = 16;  // keys in the model's sample
constexpr int LEARNED_SAMPLE      = 1 << LEARNED_SAMPLE_LOG2;
constexpr int LEARNED_LEAVES      = 256; // linear pieces of the second level
constexpr int LEARNED_MAX_BUCKET_LOG2 = 24;

// Two-level piecewise-linear model of the keys' CDF, in sample ranks. Level one: the sorted
// sample cut into LEARNED_LEAVES leaves of equal sample count, leaf j starting at knot[j]
// (an encoded key); a key belongs to the last leaf whose knot is <= the key. Level two: a
// least-squares line per leaf, rank = slope[j] * (key - knot[j]) + icpt[j], slope >= 0,
// clamped to the leaf's own rank range [j * P, (j + 1) * P] (P = sample / leaves). The
// predicted rank is therefore non-decreasing in the key, whatever the fit.
// Leaf lookup in O(1): the key range [kmin, kmin + LEARNED_CELLS << shift) is cut into
// equal cells; cell_leaf[c] is the leaf of the cell's lowest key, so a key of cell c lies
// in a leaf of [cell_leaf[c], cell_leaf[c + 1]] (a short search only where a cell holds
// several leaves, i.e. where the keys are dense).
constexpr int LEARNED_CELLS_LOG2 = 12;
constexpr int LEARNED_CELLS      = 1 << LEARNED_CELLS_LOG2;

struct LearnedModel
{
  unsigned long long knot[LEARNED_LEAVES];
  float slope[LEARNED_LEAVES];
  float icpt[LEARNED_LEAVES];
  unsigned long long kmin;
  int shift;
  uint32_t route; // LEARNED_ROUTE_*: written after the fit, the gate of both routes' kernels
  unsigned char cell_leaf[LEARNED_CELLS + 16]; // [LEARNED_CELLS + 1] used
};

// Route of one learned sort, chosen on the device from the fitted model and the sorted
// sample s. Each sample key stands for n / 2^16 keys, so a bucket holding more than
// span = ceil(cap * 2^16 / n) sample keys is predicted to exceed cap, the largest bucket the
// bucket sort takes; bucket ids never decrease along s, so bucket(s[i]) == bucket(s[i + span])
// says key i lies in such a bucket. When more than half of the sample does, the partition
// cannot pay and the plain radix sort runs instead (all-equal and near-constant keys, heavy
// duplicates).
constexpr uint32_t LEARNED_ROUTE_LEARNED = 1u;
constexpr uint32_t LEARNED_ROUTE_PLAIN   = 2u;
constexpr int LEARNED_ROUTE_TPB         = 1024; // one CTA, 64 sample keys a thread

struct LearnedRouteParams
{
  const void* sorted_sample;
  LearnedModel* model;
  int bucket_log2;
  int span; // >= 1
};

struct LearnedSampleParams
{
  const void* keys;
  unsigned long long num_items;
  void* sample; // [LEARNED_SAMPLE] encoded keys, -0.0 folded into +0.0
  KeyCodec codec;
};

struct LearnedFitParams
{
  const void* sorted_sample;
  LearnedModel* model;
};
// the cell table (one thread per cell) runs after the fit with the same parameters

// bucket = floor(rank * 2^bucket_log2 / LEARNED_SAMPLE), in [0, 2^bucket_log2)
struct LearnedHistParams
{
  HistogramParams h; // num_passes = partition passes; digit q = bits [8q, 8q+8) of the bucket
  const LearnedModel* model;
  int bucket_log2;
  int pad0;
};

struct LearnedPassParams
{
  OnesweepParams os;
  const LearnedModel* model;
  int bucket_log2;
  int digit_shift; // this pass's digit = (bucket >> digit_shift) & 255
};

// Bucket sort of the learned path: one wide counting pass per bucket in shared memory.
struct LearnedBucketParams
{
  const void* keys_in; // partitioned (raw) keys
  const void* values_in;
  void* keys_out; // may alias keys_in: every bucket is read completely before it is written
  void* values_out;
  const unsigned long long* begins;
  const unsigned long long* ends;
  unsigned long long* rest_ends; // per bucket: ends[b] if the bucket is left to the segmented sort, else begins[b]
  uint32_t* counters;            // [0] bucket ticket, [1] buckets sorted here (zeroed before the launch)
  uint32_t num_buckets;
  uint32_t pad0;
  unsigned long long num_items;  // of the whole array (bounds the L2 prefetches)
  KeyCodec codec;
  KernelGate gate;
};

struct LearnedBoundsParams
{
  const void* keys; // partitioned (raw) keys: bucket ids are non-decreasing along them
  unsigned long long num_items;
  const LearnedModel* model;
  unsigned long long* begins; // [2^bucket_log2], cleared: first index of every non-empty bucket
  unsigned long long* ends;   // [2^bucket_log2], cleared: one past its last index
  KeyCodec codec;
  int bucket_log2;
  int pad0;
  KernelGate gate;
};

} // namespace gb300
