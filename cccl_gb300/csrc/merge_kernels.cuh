// Stable merge of two sorted runs in the radix sort's order (the merge step of the sort across
// GPUs: every rank receives one sorted run from every rank and merges them pairwise, the role of
// the reference's k-way merge, cudax/include/cuda/experimental/__multi_gpu/algorithm/sort/hss/
// merge_k_way.h). Included by the radix images.
//
// Two kernels per merge. The split kernel runs one thread per tile boundary (every
// MERGE_TPB x MERGE_ITEMS outputs): a merge-path search in global memory finds how many of
// A's items precede that output (A's keys come first among equal keys: the runs are in rank
// order); thousands of these searches run at once, so their latency overlaps. The merge kernel
// then takes one output tile per CTA: it loads the tile's slices of A and B into shared memory,
// every thread finds its own diagonal inside the tile, merges MERGE_ITEMS outputs serially into
// a staging buffer, and the tile is stored coalesced. Keys are compared by their sortable images
// (the encoding of the sort, -0.0 folded into +0.0), so equal images keep A before B.
#pragma once

#include "sort_common.cuh"
#include "sort_params.h"
#include "sort_policy.h"

namespace gb300
{

// splits[t] = A items among the first min(t * MERGE_TILE, na + nb) outputs
template <int KB, int FP>
__device__ __forceinline__ void merge_split_body(const MergeParams& p)
{
  using U = typename uint_of<KB>::type;
  const U* ak                    = static_cast<const U*>(p.a_keys);
  const U* bk                    = static_cast<const U*>(p.b_keys);
  const unsigned long long na    = p.na, nb = p.nb, n = na + nb;
  const unsigned long long tiles = (n + MERGE_TILE - 1) / MERGE_TILE;
  const unsigned long long t     = blockIdx.x * (unsigned long long) blockDim.x + threadIdx.x;
  if (t > tiles)
  {
    return;
  }
  auto img                    = [&](U x) { return digit_source<U, FP>(encode_key<U>(x, p.codec)); };
  const unsigned long long o  = t * MERGE_TILE < n ? t * MERGE_TILE : n;
  unsigned long long lo       = o > nb ? o - nb : 0ull;
  unsigned long long hi       = o < na ? o : na;
  while (lo < hi)
  {
    const unsigned long long mid = (lo + hi) >> 1;
    if (img(ak[mid]) <= img(bk[o - 1 - mid]))
    {
      lo = mid + 1;
    }
    else
    {
      hi = mid;
    }
  }
  p.splits[t] = lo;
}

template <int KB, int VB, int FP>
__device__ __forceinline__ void merge_pair_body(const MergeParams& p)
{
  using U = typename uint_of<KB>::type;
  using V = typename value_word<VB>::type;
  extern __shared__ __align__(16) unsigned char smem[];
  U* sk             = reinterpret_cast<U*>(smem);                              // [A slice | B slice]
  U* ok             = reinterpret_cast<U*>(smem + size_t(MERGE_TILE) * KB);    // merged tile
  V* sv             = reinterpret_cast<V*>(smem + 2 * size_t(MERGE_TILE) * KB);
  V* ov             = sv + MERGE_TILE;

  const U* ak = static_cast<const U*>(p.a_keys);
  const U* bk = static_cast<const U*>(p.b_keys);
  const V* av = static_cast<const V*>(p.a_values);
  const V* bv = static_cast<const V*>(p.b_values);
  U* outk     = static_cast<U*>(p.out_keys);
  V* outv     = static_cast<V*>(p.out_values);
  const unsigned long long na = p.na, nb = p.nb, n = na + nb;
  auto img    = [&](U x) { return digit_source<U, FP>(encode_key<U>(x, p.codec)); };

  const unsigned long long o0 = (unsigned long long) blockIdx.x * MERGE_TILE;
  if (o0 >= n)
  {
    return; // uniform over the CTA
  }
  const unsigned long long o1 = o0 + MERGE_TILE < n ? o0 + MERGE_TILE : n;
  const unsigned long long a0 = p.splits[blockIdx.x], a1 = p.splits[blockIdx.x + 1];
  const unsigned long long b0 = o0 - a0, b1 = o1 - a1;
  const int la = int(a1 - a0), lb = int(b1 - b0), len = la + lb;
  for (int i = threadIdx.x; i < len; i += MERGE_TPB)
  {
    if (i < la)
    {
      sk[i] = ak[a0 + i];
      if constexpr (VB > 0)
      {
        sv[i] = av[a0 + i];
      }
    }
    else
    {
      sk[i] = bk[b0 + (i - la)];
      if constexpr (VB > 0)
      {
        sv[i] = bv[b0 + (i - la)];
      }
    }
  }
  __syncthreads();
  // this thread's MERGE_ITEMS outputs start on diagonal d of the tile
  const U* sa = sk;
  const U* sb = sk + la;
  const int d = min(int(threadIdx.x) * MERGE_ITEMS, len);
  int lo      = d > lb ? d - lb : 0;
  int hi      = d < la ? d : la;
  while (lo < hi)
  {
    const int mid = (lo + hi) >> 1;
    if (img(sa[mid]) <= img(sb[d - 1 - mid]))
    {
      lo = mid + 1;
    }
    else
    {
      hi = mid;
    }
  }
  int ia = lo, ib = d - lo;
#pragma unroll
  for (int k = 0; k < MERGE_ITEMS; ++k)
  {
    const int pos = d + k;
    if (pos < len)
    {
      const bool take_a = ib >= lb || (ia < la && img(sa[ia]) <= img(sb[ib]));
      const int src     = take_a ? ia : la + ib;
      ok[pos]           = sk[src];
      if constexpr (VB > 0)
      {
        ov[pos] = sv[src];
      }
      ia += take_a ? 1 : 0;
      ib += take_a ? 0 : 1;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < len; i += MERGE_TPB)
  {
    outk[o0 + i] = ok[i];
    if constexpr (VB > 0)
    {
      outv[o0 + i] = ov[i];
    }
  }
}

} // namespace gb300

#define GB300_MERGE(KB, VB, FP, SUF)                                                                              \
  extern "C" __global__ void __launch_bounds__(gb300::MERGE_TPB)                                                \
    gb300_merge_k##KB##_v##VB##_##SUF(const gb300::MergeParams p)                                               \
  {                                                                                                             \
    gb300::merge_pair_body<KB, VB, FP>(p);                                                                      \
  }

#define GB300_MERGE_ALL_VALUES(KB, FP, SUF)                                                                       \
  extern "C" __global__ void __launch_bounds__(256) gb300_merge_split_k##KB##_##SUF(const gb300::MergeParams p)  \
  {                                                                                                             \
    gb300::merge_split_body<KB, FP>(p);                                                                         \
  }                                                                                                             \
  GB300_MERGE(KB, 0, FP, SUF)               \
  GB300_MERGE(KB, 1, FP, SUF)               \
  GB300_MERGE(KB, 2, FP, SUF)               \
  GB300_MERGE(KB, 4, FP, SUF)               \
  GB300_MERGE(KB, 8, FP, SUF)               \
  GB300_MERGE(KB, 16, FP, SUF)
