// extern "C" entry kernels of the learned-partition sort for one key width. The host
// resolves them by these names (see learned_sort_abi.cpp). Integer kinds share kernels:
// the order lives in the runtime key codec.
#pragma once

#include "learned_kernels.cuh"
#include "sort_policy.h"

extern "C" __global__ void __launch_bounds__(256) gb300_init(const gb300::InitParams p)
{
  gb300::init_body(p);
}

extern "C" __global__ void __launch_bounds__(32) gb300_status_fold(const gb300::StatusFoldParams p)
{
  if (threadIdx.x == 0 && blockIdx.x == 0)
  {
    const uint32_t bits = __ldcg(p.src) & p.mask;
    if (bits != 0u)
    {
      atomicOr(p.dst, bits);
    }
  }
}

#define GB300_LEARNED_PASS(KB, VB, FP, FS)                                                                        \
  static_assert(gb300::PersistentSmem<KB, VB, gb300::persistent_tpb(KB, VB), gb300::learned_items(KB, VB),        \
                                      gb300::learned_extra_bytes(KB, VB, gb300::learned_items(KB, VB))>::bytes    \
                  == gb300::learned_pass_smem(KB, VB),                                                          \
                "learned pass shared-memory layout mismatch");                                                  \
  extern "C" __global__ void __launch_bounds__(gb300::persistent_tpb(KB, VB), gb300::PERSISTENT_MINB)            \
    gb300_learned_pass_k##KB##_v##VB##_##FS(const gb300::LearnedPassParams p)                                   \
  {                                                                                                             \
    gb300::learned_pass_body<KB, VB, FP>(p);                                                                    \
  }

// bucket sort kernels: CAP keys at most per bucket
#define GB300_LEARNED_BUCKET(KB, VB, FP, FS, CAP)                                                                 \
  static_assert(gb300::LearnedBucketSmem<KB, VB, CAP>::bytes == gb300::learned_bucket_smem(KB, VB, CAP),         \
                "learned bucket shared-memory layout mismatch");                                                \
  extern "C" __global__ void __launch_bounds__(gb300::learned_bucket_tpb(CAP), 65536 / 64 / gb300::learned_bucket_tpb(CAP)) \
    gb300_learned_bucket##CAP##_k##KB##_v##VB##_##FS(const gb300::LearnedBucketParams p)                        \
  {                                                                                                             \
    gb300::learned_bucket_body<KB, VB, FP, gb300::learned_bucket_tpb(CAP), CAP>(p);                             \
  }

#define GB300_LEARNED(KB, FP, FS)                                                                                 \
  extern "C" __global__ void __launch_bounds__(256) gb300_learned_sample_k##KB##_##FS(                          \
    const gb300::LearnedSampleParams p)                                                                         \
  {                                                                                                             \
    gb300::learned_sample_body<KB, FP>(p);                                                                      \
  }                                                                                                             \
  extern "C" __global__ void __launch_bounds__(gb300::HISTOGRAM_TPB) gb300_learned_hist_k##KB##_##FS(           \
    const gb300::LearnedHistParams p)                                                                           \
  {                                                                                                             \
    gb300::learned_hist_body<KB, FP, gb300::HISTOGRAM_TPB>(p);                                                  \
  }                                                                                                             \
  extern "C" __global__ void __launch_bounds__(gb300::LEARNED_ROUTE_TPB) gb300_learned_route_k##KB##_##FS(      \
    const gb300::LearnedRouteParams p)                                                                          \
  {                                                                                                             \
    gb300::learned_route_body<KB, FP>(p);                                                                       \
  }                                                                                                             \
  extern "C" __global__ void __launch_bounds__(256) gb300_learned_bounds_k##KB##_##FS(                          \
    const gb300::LearnedBoundsParams p)                                                                         \
  {                                                                                                             \
    gb300::learned_bounds_body<KB, FP>(p);                                                                      \
  }                                                                                                             \
  GB300_LEARNED_PASS(KB, 0, FP, FS)                                                                             \
  GB300_LEARNED_PASS(KB, 4, FP, FS)                                                                             \
  GB300_LEARNED_PASS(KB, 8, FP, FS)                                                                             \
  GB300_LEARNED_BUCKET(KB, 0, FP, FS, 8192)                                                                  \
  GB300_LEARNED_BUCKET(KB, 4, FP, FS, 8192)                                                                  \
  GB300_LEARNED_BUCKET(KB, 8, FP, FS, 8192)                                                                  \
  GB300_LEARNED_BUCKET(KB, 0, FP, FS, 4096)                                                                  \
  GB300_LEARNED_BUCKET(KB, 4, FP, FS, 4096)                                                                  \
  GB300_LEARNED_BUCKET(KB, 8, FP, FS, 4096)

#define GB300_LEARNED_FIT(KB)                                                                                     \
  extern "C" __global__ void __launch_bounds__(gb300::LEARNED_FIT_TPB) gb300_learned_fit_k##KB(                 \
    const gb300::LearnedFitParams p)                                                                            \
  {                                                                                                             \
    gb300::learned_fit_body<KB>(p);                                                                             \
  }                                                                                                             \
  extern "C" __global__ void __launch_bounds__(256) gb300_learned_cells_k##KB(const gb300::LearnedFitParams p)  \
  {                                                                                                             \
    gb300::learned_cells_body<KB>(p);                                                                           \
  }
