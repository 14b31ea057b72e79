// Host dispatcher of the batched segmented sort: temporary-storage plan, digit-pass plan
// that lands the result in the buffer CUB's DeviceSegmentedSort would use, and the launch
// sequence init -> classify -> class kernels -> large-segment passes.
#pragma once

#include <cuda.h>

#include <cstddef>
#include <cstdint>

#include "sort_params.h"

namespace gb300
{

struct SegmentedPolicy
{
  uint32_t magic;
  int32_t key_bytes;
  int32_t value_bytes;
  int32_t key_kind;
  int32_t small_threads;
  int32_t small_items;
  int32_t medium_threads;
  int32_t medium_items;
  int32_t block_s_cap;
  int32_t block_l_cap;
  int32_t block_s_tpb;
  int32_t block_l_tpb;
  int32_t pass_tpb;
  int32_t pass_items;
  uint64_t network_small_smem;
  uint64_t network_medium_smem;
  uint64_t network_rsmall_smem; // radix-order networks
  uint64_t network_rmedium_smem;
  uint64_t block_s_smem;
  uint64_t block_l_smem;
  uint64_t pass_smem;
  int32_t ppass_tpb; // pipelined device-class pass (buffers 16-byte aligned)
  int32_t ppass_items;
  uint64_t ppass_smem;
  int32_t gather_value_bytes; // > 0: the caller's values have this width, sorted as 32-bit indices
  int32_t pad0;
};

SegmentedPolicy make_segmented_policy(int key_bytes, int value_bytes, int key_kind);

// Kernels resolved from the library (names in segmented_sort_abi.cpp).
enum SegKernel : int
{
  SK_INIT = 0,
  SK_CLASSIFY,
  SK_SMALL,
  SK_MEDIUM,
  SK_BLOCK_S,
  SK_BLOCK_L,
  SK_HIST,
  SK_SCAN,
  SK_PASS,
  SK_RSMALL,  // the networks in radix order (segmented radix sort, learned buckets)
  SK_RMEDIUM,
  SK_PPASS,   // the pipelined device-class pass
  SK_BLOCK_XS, // block class of the shortest segments
  SK_COUNT
};

struct SegmentedKernels
{
  CUkernel k[SK_COUNT];
};

// Kernel names of one (key width, value width, key kind) in the segmented image.
void segmented_kernel_names(int kb, int vb, int kind, bool descending, char (&names)[SK_COUNT][64]);

struct SegmentedCall
{
  void* keys[2];   // [0] = current (input), [1] = alternate (output)
  void* values[2]; // null for keys-only
  uint64_t num_items;
  uint64_t num_segments;
  const void* begin_offsets;
  const void* end_offsets;
  int offsets_64;
  bool overwrite;
  bool descending;
  void* d_temp_storage;
  size_t* temp_storage_bytes;
  CUstream stream;
  int target; // buffer index that receives the result; -1: the one CUB's dispatch picks
  // DeviceSegmentedRadixSort semantics: every segment is radix-sorted (no merge networks)
  // by bits [begin_bit, end_bit), and the buffer follows that dispatch's pass count
  bool radix_only;
  int begin_bit;
  int end_bit;
};

// Runs (or sizes, when d_temp_storage is null) one segmented sort; writes the selector
// CUB's dispatch leaves in the caller's DoubleBuffer. Throws cuda_error on failure.
void segmented_sort_dispatch(const SegmentedPolicy& pol, const SegmentedKernels& ks, const SegmentedCall& call,
                             int* selector);

} // namespace gb300
