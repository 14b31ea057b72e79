// Host dispatcher of the plain radix sort: temporary-storage plan, buffer ping-pong,
// selector bookkeeping and the launch sequence init -> histogram -> onesweep passes.
#pragma once

#include <cuda.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "sort_params.h"

namespace gb300
{

// Tile configuration stored in the build result's runtime_policy (plain data, part of
// the serialized blob).
struct RadixPolicy
{
  uint32_t magic;
  int32_t key_bytes;
  int32_t value_bytes;
  int32_t key_kind;
  int32_t onesweep_tpb;
  int32_t onesweep_items;
  int32_t single_tile_tpb;
  int32_t single_tile_items;
  int32_t histogram_tpb;
  int32_t persistent_tpb;
  int32_t persistent_items;
  int32_t gather_value_bytes; // > 0: the caller's values have this width, sorted as 32-bit indices
  int32_t reserved[4];
  uint64_t onesweep_smem;
  uint64_t single_tile_smem;
  uint64_t persistent_smem;
};

RadixPolicy make_radix_policy(int key_bytes, int value_bytes, int key_kind);

struct RadixKernels
{
  CUkernel init;
  CUkernel histogram;
  CUkernel onesweep;       // persistent pass kernel (bulk-copy prefetch, cooperative launch)
  CUkernel onesweep_first; // its order-free variant for pass 0 of integer keys-only sorts (may be == onesweep)
  CUkernel onesweep_dyn;   // CTA-per-tile pass kernel for buffers that are not 16-byte aligned
  CUkernel single_tile;
};

// Kernel names of one (key width, value width, key kind) in the radix image.
struct RadixKernelNames
{
  std::string init, histogram, onesweep, onesweep_first, onesweep_dyn, single_tile;
};
RadixKernelNames radix_kernel_names(int key_bytes, int value_bytes, int key_kind, bool descending);

struct RadixCall
{
  void* keys[2];   // [0] = current (input), [1] = alternate (output)
  void* values[2]; // null for keys-only
  uint64_t num_items;
  int begin_bit;
  int end_bit;
  bool overwrite;
  bool descending;
  void* d_temp_storage;
  size_t* temp_storage_bytes;
  CUstream stream;
  KernelGate gate; // null: always run; else the kernels run only if the flag is set (onesweep path only)
  uint32_t* status_word; // null: the call's own status word (word 0 of its temp storage); else
                         // where its kernels report (a sort run inside another reports there)
};

// Byte layout of the temporary storage of one call.
struct RadixTempPlan
{
  int num_passes;
  uint64_t tile_items;
  uint64_t portion_items;
  uint64_t num_portions;
  uint64_t total_tiles;
  size_t ctrl_off, ctrl_bytes;
  size_t bins_off;
  size_t lookback_off, lookback_words; // two buffers of lookback_words each
  size_t keys_tmp_off, values_tmp_off;
  size_t total_bytes;
};

RadixTempPlan plan_radix_temp(
  const RadixPolicy& pol, uint64_t num_items, int begin_bit, int end_bit, bool need_tmp, bool persistent);

// Runs (or sizes, when d_temp_storage is null) one sort. Writes the DoubleBuffer
// selector CUB would report. Throws cuda_error on failure.
void radix_sort_dispatch(const RadixPolicy& pol, const RadixKernels& ks, const RadixCall& call, int* selector);

} // namespace gb300
