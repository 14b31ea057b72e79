// Host dispatcher of the learned-partition sort: sample -> plain radix sort of the sample
// -> least-squares fit -> digit counts -> stable partition passes on the bucket id -> bucket
// bounds (one read of the partitioned keys) -> bucket sort in shared memory (one wide counting pass per bucket) ->
// batched segmented radix sort of the buckets that one could not take. Inputs it does not take (fewer
// than LEARNED_MIN_ITEMS keys, a partial bit window, buffers that are not 16-byte aligned)
// run the plain radix sort instead; the output and the selector are the plain sort's either way.
#pragma once

#include <cuda.h>

#include <cstddef>
#include <cstdint>

#include "radix_plan.h"
#include "segmented_plan.h"

namespace gb300
{

struct LearnedKernels
{
  CUkernel init;
  CUkernel sample;
  CUkernel fit;
  CUkernel cells;
  CUkernel route; // learned or plain, from the model and the sorted sample
  CUkernel hist;
  CUkernel pass;
  CUkernel bounds;
  CUkernel bucket4k; // bucket sort, up to 4096 keys per bucket
  CUkernel bucket8k; // up to 8192
  CUkernel status_fold; // a sub-sort's error bits into the call's status word
};

// Everything one (key type, value width, order) needs; lives in the build result.
struct LearnedSetup
{
  uint32_t magic;
  int32_t key_bytes;
  int32_t value_bytes;
  int32_t key_kind;
  int32_t pass_tpb;
  int32_t pass_items;
  uint64_t pass_smem;
  RadixPolicy plain_pol; // the plain sort of these types (fallback)
  RadixKernels plain_ks;
  RadixPolicy sample_pol; // keys-only sort of the encoded sample (unsigned keys)
  RadixKernels sample_ks;
  SegmentedPolicy seg_pol; // bucket sort
  SegmentedKernels seg_ks;
  LearnedKernels lk;
  int32_t route_policy; // LEARNED_POLICY_*
  int32_t reserved0;
};

// Host-side route policy of a build (cccl_gb300_learned_sort_set_route).
constexpr int LEARNED_POLICY_COST_MODEL = 0; // learned only where its byte count predicts a win
constexpr int LEARNED_POLICY_ALWAYS     = 1; // learned wherever the input qualifies

// Where the pieces of one call live in its temporary storage.
struct LearnedTempPlan
{
  bool learned; // false: the plain radix sort runs (plain_bytes of temp)
  int bucket_log2;
  int bucket_cap; // largest bucket the shared-memory bucket sort takes (twice the target size)
  int passes;
  uint64_t tile_items, portion_items, num_portions;
  size_t ctrl_off, ctrl_bytes, bins_off, lookback_off, lookback_words;
  size_t model_off, sample_off, sample_temp_off, sample_temp_bytes, bounds_off;
  size_t keys_tmp_off, values_tmp_off, seg_off, seg_bytes;
  // n >= 2^30: a bucket may reach the segmented sort's 2^30-key limit; a plain radix sort of
  // the partitioned keys, gated on the segmented sort's bad-segment flag, then redoes the sort
  size_t fallback_off, fallback_bytes;
  // the plain route: the plain radix sort of the input, gated on the route word. Without
  // overwrite its alternate key/value buffers are the learned passes' (keys_tmp_off and
  // values_tmp_off point into this region): only one of the two routes runs
  size_t plain_off, plain_bytes;
  size_t total_bytes;
};

LearnedTempPlan plan_learned_temp(const LearnedSetup& s, const RadixCall& call);

// Counters a caller can read back after a run (synchronously) from the temp storage.
struct LearnedStats
{
  int learned;
  int bucket_log2;
  int partition_passes;
  uint32_t block_buckets;  // buckets sorted in shared memory (network and block classes)
  uint32_t device_buckets; // buckets handed to the plain radix passes
  uint64_t device_items;   // keys in those buckets
};

void learned_sort_dispatch(const LearnedSetup& s, const RadixCall& call, int* selector);
LearnedStats learned_sort_stats(const LearnedSetup& s, const RadixCall& call);

} // namespace gb300
