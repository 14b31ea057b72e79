// extern "C" entry kernels of the batched segmented sort for one key width. The host
// resolves them by these names (see segmented_plan.cpp).
#pragma once

#include "segmented_kernels.cuh"
#include "gather_kernels.cuh"
#include "sort_policy.h"

extern "C" __global__ void __launch_bounds__(256) gb300_init(const gb300::InitParams p)
{
  gb300::init_body(p);
}

extern "C" __global__ void __launch_bounds__(256) gb300_seg_classify(const gb300::SegClassifyParams p)
{
  gb300::seg_classify_body(p);
}

extern "C" __global__ void __launch_bounds__(256) gb300_seg_scan(const gb300::SegDeviceParams p)
{
  gb300::seg_device_scan_body<256>(p);
}

// merge-network kernels: KIND 0 unsigned (u), 1 signed (i), 2 floating point (f)
#define GB300_SEG_NETWORK(KB, KIND, KS, VB)                                                                          \
  static_assert(gb300::NetworkSmem<KB, KIND, VB, gb300::seg_small_threads(KB, VB), gb300::seg_small_items(KB, VB)>::per_warp \
                    * (gb300::SEG_NETWORK_TPB / 32)                                                                   \
                  == gb300::seg_network_smem(KB, VB, gb300::seg_small_threads(KB, VB), gb300::seg_small_items(KB, VB)), \
                "network smem");                                                                                     \
  extern "C" __global__ void __launch_bounds__(gb300::SEG_NETWORK_TPB)                                               \
    gb300_seg_small_k##KB##_v##VB##_##KS(const gb300::SegSortParams p)                                               \
  {                                                                                                                  \
    gb300::seg_network_body<KB, KIND, VB, gb300::seg_small_threads(KB, VB), gb300::seg_small_items(KB, VB)>(         \
      p, p.small_list, gb300::SEG_CTR_SMALL, gb300::SEG_CTR_TICKET_SMALL);                                           \
  }                                                                                                                  \
  extern "C" __global__ void __launch_bounds__(gb300::SEG_NETWORK_TPB)                                               \
    gb300_seg_medium_k##KB##_v##VB##_##KS(const gb300::SegSortParams p)                                              \
  {                                                                                                                  \
    gb300::seg_network_body<KB, KIND, VB, gb300::seg_medium_threads(KB, VB), gb300::seg_medium_items(KB, VB)>(       \
      p, p.medium_list, gb300::SEG_CTR_MEDIUM, gb300::SEG_CTR_TICKET_MEDIUM);                                        \
  }

// radix kernels (integer kinds share them: the order lives in the runtime key codec)
#define GB300_SEG_RADIX(KB, FP, FS, VB)                                                                              \
  static_assert(gb300::seg_block_algo(KB) != gb300::SEG_BLOCK_MERGE                                                  \
                  || gb300::BlockMergeSmem<KB, gb300::seg_block_l_tpb(KB), gb300::seg_block_l_items(KB)>::bytes      \
                       == gb300::block_merge_smem(KB, gb300::seg_block_l_tpb(KB), gb300::seg_block_l_items(KB)),     \
                "block merge shared-memory layout");                                                                 \
  extern "C" __global__ void __launch_bounds__(gb300::seg_block_xs_tpb(KB), gb300::seg_block_xs_minb(KB))            \
    gb300_seg_block_xs_k##KB##_v##VB##_##FS(const gb300::SegSortParams p)                                            \
  {                                                                                                                  \
    gb300::seg_block_body<KB, VB, FP, gb300::seg_block_xs_tpb(KB), gb300::seg_block_xs_items(KB),                    \
                          gb300::seg_block_s_bits(KB)>(                                                            \
      p, p.block_xs_list, gb300::SEG_CTR_BLOCK_XS, gb300::SEG_CTR_TICKET_BLOCK_XS);                                  \
  }                                                                                                                  \
  extern "C" __global__ void __launch_bounds__(gb300::seg_block_s_tpb(KB), gb300::seg_block_s_minb(KB, VB))              \
    gb300_seg_block_s_k##KB##_v##VB##_##FS(const gb300::SegSortParams p)                                             \
  {                                                                                                                  \
    gb300::seg_block_body<KB, VB, FP, gb300::seg_block_s_tpb(KB), gb300::seg_block_s_items(KB),               \
                          gb300::seg_block_s_bits(KB)>(                                                            \
      p, p.block_s_list, gb300::SEG_CTR_BLOCK_S, gb300::SEG_CTR_TICKET_BLOCK_S);                                     \
  }                                                                                                                  \
  extern "C" __global__ void __launch_bounds__(gb300::seg_block_l_tpb(KB), gb300::seg_block_minb(KB))              \
    gb300_seg_block_l_k##KB##_v##VB##_##FS(const gb300::SegSortParams p)                                             \
  {                                                                                                                  \
    gb300::seg_block_body<KB, VB, FP, gb300::seg_block_l_tpb(KB), gb300::seg_block_l_items(KB),               \
                          gb300::seg_block_l_bits(KB)>(                                                            \
      p, p.block_l_list, gb300::SEG_CTR_BLOCK_L, gb300::SEG_CTR_TICKET_BLOCK_L);                                     \
  }                                                                                                                  \
  extern "C" __global__ void __launch_bounds__(gb300::seg_pass_tpb(KB, VB))                                         \
    gb300_seg_pass_k##KB##_v##VB##_##FS(const gb300::SegDeviceParams p)                                              \
  {                                                                                                                  \
    gb300::seg_device_onesweep_body<KB, VB, FP, gb300::seg_pass_tpb(KB, VB), gb300::seg_pass_items(KB, VB)>(p);      \
  }                                                                                                                  \
  extern "C" __global__ void __launch_bounds__(gb300::seg_ppass_tpb(KB, VB), 1)                                     \
    gb300_seg_ppass_k##KB##_v##VB##_##FS(const gb300::SegDeviceParams p)                                             \
  {                                                                                                                  \
    gb300::seg_device_persistent_body<KB, VB, FP, gb300::seg_ppass_tpb(KB, VB), gb300::seg_ppass_items(KB, VB)>(p);  \
  }

#define GB300_SEG_HIST(KB, FP, FS)                                                                                   \
  extern "C" __global__ void __launch_bounds__(gb300::HISTOGRAM_TPB)                                                 \
    gb300_seg_hist_k##KB##_##FS(const gb300::SegDeviceParams p)                                                      \
  {                                                                                                                  \
    gb300::seg_device_histogram_body<KB, FP, gb300::HISTOGRAM_TPB>(p);                                               \
  }

// radix-order networks: KIND = NET_RADIX + FP mode, their own shapes
#define GB300_SEG_RNETWORK(KB, KIND, KS, VB)                                                                         \
  extern "C" __global__ void __launch_bounds__(gb300::SEG_NETWORK_TPB)                                               \
    gb300_seg_small_k##KB##_v##VB##_##KS(const gb300::SegSortParams p)                                               \
  {                                                                                                                  \
    gb300::seg_network_body<KB, KIND, VB, gb300::SEG_RSMALL_THREADS, gb300::SEG_RSMALL_ITEMS>(                        \
      p, p.small_list, gb300::SEG_CTR_SMALL, gb300::SEG_CTR_TICKET_SMALL);                                           \
  }                                                                                                                  \
  extern "C" __global__ void __launch_bounds__(gb300::SEG_NETWORK_TPB)                                               \
    gb300_seg_medium_k##KB##_v##VB##_##KS(const gb300::SegSortParams p)                                              \
  {                                                                                                                  \
    gb300::seg_network_body<KB, KIND, VB, gb300::SEG_RMEDIUM_THREADS, gb300::SEG_RMEDIUM_ITEMS>(                      \
      p, p.medium_list, gb300::SEG_CTR_MEDIUM, gb300::SEG_CTR_TICKET_MEDIUM);                                        \
  }
#define GB300_SEG_RNET_VALUES(KB, KIND, KS) GB300_SEG_RNETWORK(KB, KIND, KS, 0) GB300_SEG_RNETWORK(KB, KIND, KS, 4) GB300_SEG_RNETWORK(KB, KIND, KS, 8)

#define GB300_SEG_VALUES(KB, FP, FS, ...) GB300_SEG_RADIX(KB, FP, FS, 0) GB300_SEG_RADIX(KB, FP, FS, 4) GB300_SEG_RADIX(KB, FP, FS, 8)
#define GB300_SEG_NET_VALUES(KB, KIND, KS) GB300_SEG_NETWORK(KB, KIND, KS, 0) GB300_SEG_NETWORK(KB, KIND, KS, 4) GB300_SEG_NETWORK(KB, KIND, KS, 8)
