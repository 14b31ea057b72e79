// extern "C" entry kernels of the plain path for one key width (KEY_BYTES must be
// defined by the including translation unit). The unmangled names are what the host
// resolves with cuLibraryGetKernel; see kernel_names.h for the naming scheme.
#pragma once

#include "radix_kernels.cuh"
#include "gather_kernels.cuh"
#include "merge_kernels.cuh"
#include "sort_policy.h"

#define GB300_CAT_(a, b) a##b
#define GB300_CAT(a, b)  GB300_CAT_(a, b)

#define GB300_ONESWEEP(KB, VB, FP, SUF)                                                                           \
  static_assert(gb300::OnesweepSmem<KB, VB, gb300::ONESWEEP_TPB, gb300::onesweep_items(KB, VB)>::bytes          \
                  == gb300::onesweep_smem_bytes(KB, VB),                                                        \
                "onesweep shared-memory layout mismatch");                                                      \
  static_assert(gb300::PersistentSmem<KB, VB, gb300::persistent_tpb(KB, VB), gb300::persistent_items(KB, VB)>::bytes    \
                  == gb300::persistent_smem_bytes(KB, VB),                                                      \
                "persistent onesweep shared-memory layout mismatch");                                           \
  extern "C" __global__ void __launch_bounds__(gb300::ONESWEEP_TPB)                                             \
    gb300_onesweep_dyn_k##KB##_v##VB##_##SUF(const gb300::OnesweepParams p)                                     \
  {                                                                                                             \
    gb300::OnesweepParams q = p;                                                                                \
    if (gb300::apply_pass_plan<KB, VB>(q))                                                                      \
    {                                                                                                           \
      gb300::onesweep_body<KB, VB, FP, gb300::ONESWEEP_TPB, gb300::onesweep_items(KB, VB), true>(q);            \
    }                                                                                                           \
  }                                                                                                             \
  extern "C" __global__ void __launch_bounds__(gb300::persistent_tpb(KB, VB), gb300::PERSISTENT_MINB)                                        \
    gb300_onesweep_k##KB##_v##VB##_##SUF(const gb300::OnesweepParams p)                                         \
  {                                                                                                             \
    gb300::onesweep_persistent_body<KB, VB, FP, gb300::persistent_tpb(KB, VB), gb300::persistent_items(KB, VB), true>(p); \
  }

// First pass of a full-width integer keys-only sort: equal digits may land in any order
// inside their bucket, because keys equal in that digit are ordered by the later (stable)
// passes and fully equal integer keys are indistinguishable.
#define GB300_ONESWEEP_FIRST(KB)                                                                                  \
  extern "C" __global__ void __launch_bounds__(gb300::persistent_tpb(KB, 0), gb300::PERSISTENT_MINB)                                   \
    gb300_onesweep_first_k##KB##_v0_i(const gb300::OnesweepParams p)                                            \
  {                                                                                                             \
    gb300::onesweep_persistent_body<KB, 0, false, gb300::persistent_tpb(KB, 0), gb300::persistent_items(KB, 0), false>(p); \
  }

#define GB300_SINGLE_TILE(KB, VB, FP, SUF)                                                                        \
  extern "C" __global__ void __launch_bounds__(gb300::SINGLE_TILE_TPB)                                          \
    gb300_single_tile_k##KB##_v##VB##_##SUF(const gb300::SingleTileParams p)                                    \
  {                                                                                                             \
    gb300::single_tile_body<KB, VB, FP, gb300::SINGLE_TILE_TPB, gb300::SINGLE_TILE_ITEMS>(p);                   \
  }

#define GB300_HISTOGRAM(KB, FP, SUF)                                                                              \
  extern "C" __global__ void __launch_bounds__(gb300::HISTOGRAM_LANES_TPB, 1)                                   \
    gb300_histogram_k##KB##_##SUF(const gb300::HistogramParams p)                                               \
  {                                                                                                             \
    gb300::histogram_lanes_body<KB, FP, gb300::HISTOGRAM_LANES_TPB>(p);                                         \
  }

// Single-tile kernels of descending floating-point sorts: CUB's single tile folds -0.0 into
// +0.0 before ordering (see digit_source), unlike its onesweep passes.
#define GB300_SINGLE_TILE_DESC_FP(KB)                   \
  GB300_SINGLE_TILE(KB, 0, gb300::FP_BLOCK_DESC, fd)    \
  GB300_SINGLE_TILE(KB, 1, gb300::FP_BLOCK_DESC, fd)    \
  GB300_SINGLE_TILE(KB, 2, gb300::FP_BLOCK_DESC, fd)    \
  GB300_SINGLE_TILE(KB, 4, gb300::FP_BLOCK_DESC, fd)    \
  GB300_SINGLE_TILE(KB, 8, gb300::FP_BLOCK_DESC, fd)    \
  GB300_SINGLE_TILE(KB, 16, gb300::FP_BLOCK_DESC, fd)

#define GB300_ALL_VALUES(KB, FP, SUF)  \
  GB300_ONESWEEP(KB, 0, FP, SUF)       \
  GB300_ONESWEEP(KB, 1, FP, SUF)       \
  GB300_ONESWEEP(KB, 2, FP, SUF)       \
  GB300_ONESWEEP(KB, 4, FP, SUF)       \
  GB300_ONESWEEP(KB, 8, FP, SUF)       \
  GB300_ONESWEEP(KB, 16, FP, SUF)      \
  GB300_SINGLE_TILE(KB, 0, FP, SUF)    \
  GB300_SINGLE_TILE(KB, 1, FP, SUF)    \
  GB300_SINGLE_TILE(KB, 2, FP, SUF)    \
  GB300_SINGLE_TILE(KB, 4, FP, SUF)    \
  GB300_SINGLE_TILE(KB, 8, FP, SUF)    \
  GB300_SINGLE_TILE(KB, 16, FP, SUF)   \
  GB300_HISTOGRAM(KB, FP, SUF)         \
  GB300_MERGE_ALL_VALUES(KB, FP, SUF)

extern "C" __global__ void __launch_bounds__(256) gb300_init(const gb300::InitParams p)
{
  gb300::init_body(p);
}
