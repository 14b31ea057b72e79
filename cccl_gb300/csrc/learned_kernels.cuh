// Learned-partition sort kernels for sm_103a (no reference counterpart: a new form of the
// sort beside CUB's plain radix sort, with the same output bit for bit).
//
//   sample  : LEARNED_SAMPLE keys at jittered, evenly spaced positions, encoded;
//   (the sample is sorted by the plain radix sort, which gives every sample key its rank)
//   fit     : one CTA per leaf fits rank ~ key by least squares over the leaf's sample points;
//   hist    : one read of the keys: bucket of every key, digit counts of every partition pass;
//   pass    : the persistent onesweep pass with the bucket id's digits in place of key bits
//             (stable, so after the passes the keys are grouped by bucket in input order);
//   bounds  : first index of every bucket, from one read of the partitioned keys.
// The buckets are then sorted as segments by the batched segmented sort; a bucket too large
// for a block sort goes to its plain radix passes.
//
// Exactness does not depend on the model: the bucket id is non-decreasing in the encoded
// key (the -0.0 rule applied first, so -0.0 and +0.0 share a bucket), the partition is
// stable and every bucket is sorted stably by the full key, so the result is the stable
// sort of the input by the encoded key, i.e. CUB's.
#pragma once

#include "radix_kernels.cuh"

namespace gb300
{

template <class U>
struct alignas(16) LearnedLeaf
{
  U knot;
  float slope;
  float icpt;
};

// Shared-memory copy of the model for one sort (layout size: learned_tables_bytes()). Each
// leaf's line is stored in buckets rather than sample ranks: slope and intercept times
// scale = buckets / sample keys, a power of two, so the product is exact.
template <class U>
struct LearnedTables
{
  LearnedLeaf<U> leaf[LEARNED_LEAVES];
  unsigned char cell_leaf[LEARNED_CELLS + 16];
  U kmin;
  int shift;
};

// 2^bucket_log2 buckets per 2^LEARNED_SAMPLE_LOG2 sample ranks
__device__ __forceinline__ float learned_scale(int bucket_log2)
{
  return exp2f(float(bucket_log2 - LEARNED_SAMPLE_LOG2)); // a power of two: exact
}

template <class U>
__device__ __forceinline__ void learned_load_tables(const LearnedModel* m, LearnedTables<U>* t, int bucket_log2)
{
  const float scale = learned_scale(bucket_log2);
  for (int i = threadIdx.x; i < LEARNED_LEAVES; i += blockDim.x)
  {
    t->leaf[i].knot  = U(m->knot[i]);
    t->leaf[i].slope = m->slope[i] * scale;
    t->leaf[i].icpt  = m->icpt[i] * scale;
  }
  const uint32_t* src = reinterpret_cast<const uint32_t*>(m->cell_leaf);
  uint32_t* dst       = reinterpret_cast<uint32_t*>(t->cell_leaf);
  for (int i = threadIdx.x; i < (LEARNED_CELLS + 16) / 4; i += blockDim.x)
  {
    dst[i] = src[i];
  }
  if (threadIdx.x == 0)
  {
    t->kmin  = U(m->kmin);
    t->shift = m->shift;
  }
}

__device__ __forceinline__ float learned_to_float(uint32_t x)
{
  return __uint2float_rn(x);
}

__device__ __forceinline__ float learned_to_float(unsigned long long x)
{
  return __ull2float_rn(x);
}

// Leaf of an encoded key: the last leaf whose knot is <= the key, searched only among the
// leaves of the key's cell (the first leaf if no knot is <= the key).
template <class U>
__device__ __forceinline__ int learned_leaf(U k, const LearnedTables<U>& t)
{
  const U d        = k > t.kmin ? U(k - t.kmin) : U(0);
  const U c_wide   = d >> t.shift;
  const uint32_t c = c_wide < U(LEARNED_CELLS - 1) ? uint32_t(c_wide) : uint32_t(LEARNED_CELLS - 1);
  int j            = t.cell_leaf[c];
  int span         = int(t.cell_leaf[c + 1]) - j;
  while (span > 0)
  {
    const int half = (span + 1) >> 1;
    if (t.leaf[j + half].knot <= k)
    {
      j += half;
      span -= half;
    }
    else
    {
      span = half - 1;
    }
  }
  return j;
}

// Bucket of an encoded key: floor(clamp(rank, j * P, (j + 1) * P) * scale) for the predicted
// sample rank of leaf j (P = sample keys per leaf). The tables hold the line times scale, a
// power of two, so fmaf gives rank * scale exactly; the leaf's bucket range
// [j * P * scale, (j + 1) * P * scale] is integral (at least 256 buckets), so the clamp is
// applied after the truncation, in integers, with the same result. Every step is
// non-decreasing in the key: the leaf lookup, the conversion of (key - knot) to float, the
// fused multiply-add with a slope >= 0, the truncation (negative ranks give 0) and the
// clamp to the leaf's range (leaf j's top equals leaf j+1's bottom).
template <class U, int FP>
__device__ __forceinline__ uint32_t learned_bucket(U enc, const LearnedTables<U>& t, int range_log2, uint32_t bmax)
{
  const U k               = digit_source<U, FP>(enc);
  const int j             = learned_leaf<U>(k, t);
  const LearnedLeaf<U> lf = t.leaf[j];
  const float x           = k > lf.knot ? learned_to_float(U(k - lf.knot)) : 0.0f;
  const uint32_t lo       = uint32_t(j) << range_log2;
  uint32_t b              = __float2uint_rz(fmaf(lf.slope, x, lf.icpt));
  b                       = min(max(b, lo), lo + (1u << range_log2));
  return b < bmax ? b : bmax;
}

// learned_bucket for N keys at once, step by step across the keys: every phase (the cell
// table, each step of the leaf search, the leaf line) issues its shared-memory reads for all
// N keys before using any, so their latencies overlap instead of adding up key after key.
// The search takes the same halving steps as learned_leaf (a cell's span is below 256, so at
// most 8), and the bucket is the same value. Used by the model histogram, which streams the
// keys (2^30 f64: 4.96 -> 4.34 ms on the lognormal/uniform mix, 3.91 -> 2.95 ms on sorted-then-
// reversed keys); in the partition pass it made no difference (35.2 -> 35.8 ms), and the pass
// keeps the key-by-key form, which needs fewer registers.
template <class U, int FP, int N>
__device__ __forceinline__ void
learned_bucket_batch(const U (&enc)[N], uint32_t (&out)[N], const LearnedTables<U>& t, int range_log2, uint32_t bmax)
{
  U k[N];
  int j[N];
  int span[N];
#pragma unroll
  for (int i = 0; i < N; ++i)
  {
    k[i]             = digit_source<U, FP>(enc[i]);
    const U d        = k[i] > t.kmin ? U(k[i] - t.kmin) : U(0);
    const U c_wide   = d >> t.shift;
    const uint32_t c = c_wide < U(LEARNED_CELLS - 1) ? uint32_t(c_wide) : uint32_t(LEARNED_CELLS - 1);
    j[i]             = t.cell_leaf[c];
    span[i]          = int(t.cell_leaf[c + 1]) - j[i];
  }
#pragma unroll
  for (int step = 0; step < 8; ++step)
  {
    bool more = false;
#pragma unroll
    for (int i = 0; i < N; ++i)
    {
      if (span[i] > 0)
      {
        const int half = (span[i] + 1) >> 1;
        if (t.leaf[j[i] + half].knot <= k[i])
        {
          j[i] += half;
          span[i] -= half;
        }
        else
        {
          span[i] = half - 1;
        }
        more |= span[i] > 0;
      }
    }
    if (!more)
    {
      break;
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i)
  {
    const LearnedLeaf<U> lf = t.leaf[j[i]];
    const float x           = k[i] > lf.knot ? learned_to_float(U(k[i] - lf.knot)) : 0.0f;
    const uint32_t lo       = uint32_t(j[i]) << range_log2;
    uint32_t b              = __float2uint_rz(fmaf(lf.slope, x, lf.icpt));
    b                       = min(max(b, lo), lo + (1u << range_log2));
    out[i]                  = b < bmax ? b : bmax;
  }
}

// log2 of the buckets in one leaf's rank range: (sample / leaves) * scale
__host__ __device__ constexpr int learned_range_log2(int bucket_log2)
{
  return bucket_log2 - (LEARNED_SAMPLE_LOG2 - 8);
}
static_assert(LEARNED_SAMPLE / LEARNED_LEAVES == 256, "leaf rank range of 2^8 sample keys");

// ---------------------------------------------------------------------------------------
// sample: thread i takes one key from [i*n/S, (i+1)*n/S) at a hashed offset
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t learned_mix(uint32_t x)
{
  // integer finaliser (xorshift-multiply), only to decorrelate the offsets from the input
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

template <int KB, int FP>
__device__ __forceinline__ void learned_sample_body(const LearnedSampleParams& p)
{
  using U            = typename uint_of<KB>::type;
  const uint32_t i   = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= uint32_t(LEARNED_SAMPLE))
  {
    return;
  }
  const unsigned long long n  = p.num_items;
  const unsigned long long lo = ((unsigned long long) i * n) >> LEARNED_SAMPLE_LOG2;
  const unsigned long long hi = ((unsigned long long) (i + 1) * n) >> LEARNED_SAMPLE_LOG2;
  const unsigned long long w  = hi > lo ? hi - lo : 1;
  unsigned long long pos      = lo + learned_mix(i) % w;
  pos                         = pos < n ? pos : n - 1;
  const U raw                 = static_cast<const U*>(p.keys)[pos];
  static_cast<U*>(p.sample)[i] = digit_source<U, FP>(encode_key<U>(raw, p.codec));
}

// ---------------------------------------------------------------------------------------
// fit: CTA j, thread t holds sample point j*P + t (P = LEARNED_FIT_TPB); centred least
// squares in double precision
// ---------------------------------------------------------------------------------------
template <int TPB>
__device__ __forceinline__ double learned_block_sum(double v, double* scratch)
{
  const int lane = threadIdx.x & 31;
  const int w    = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1)
  {
    v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  __syncthreads(); // scratch reuse across calls
  if (lane == 0)
  {
    scratch[w] = v;
  }
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < TPB / 32; ++k)
  {
    s += scratch[k];
  }
  return s;
}

template <int KB>
__device__ __forceinline__ void learned_fit_body(const LearnedFitParams& p)
{
  using U             = typename uint_of<KB>::type;
  constexpr int P     = LEARNED_FIT_TPB;
  __shared__ double scratch[P / 32];
  const int j         = blockIdx.x;
  const U* s          = static_cast<const U*>(p.sorted_sample);
  const uint32_t idx  = uint32_t(j) * P + threadIdx.x;
  const U knot        = s[uint32_t(j) * P];
  const double x      = double(s[idx] - knot); // sorted: s[idx] >= knot
  const double y      = double(idx);
  const double mx     = learned_block_sum<P>(x, scratch) / P;
  const double my     = learned_block_sum<P>(y, scratch) / P;
  const double sxx    = learned_block_sum<P>((x - mx) * (x - mx), scratch);
  const double sxy    = learned_block_sum<P>((x - mx) * (y - my), scratch);
  if (threadIdx.x == 0)
  {
    double slope = sxx > 0.0 ? sxy / sxx : 0.0;
    if (!(slope >= 0.0) || !isfinite(slope))
    {
      slope = 0.0;
    }
    double icpt = my - slope * mx;
    if (!isfinite(icpt))
    {
      icpt = my;
    }
    p.model->knot[j]  = (unsigned long long) knot;
    p.model->slope[j] = float(slope);
    p.model->icpt[j]  = float(icpt);
  }
}

// ---------------------------------------------------------------------------------------
// cells: thread c finds the leaf of cell c's lowest key (c = LEARNED_CELLS: of the largest
// key); thread 0 also stores kmin and the cell width
// ---------------------------------------------------------------------------------------
template <int KB>
__device__ __forceinline__ void learned_cells_body(const LearnedFitParams& p)
{
  using U          = typename uint_of<KB>::type;
  const U* s       = static_cast<const U*>(p.sorted_sample);
  const U kmin     = s[0];
  const U width    = U(s[LEARNED_SAMPLE - 1] - kmin);
  const int bits   = width == 0 ? 0 : (KB == 8 ? 64 - __clzll((long long) width) : 32 - __clz(uint32_t(width)));
  const int shift  = bits > LEARNED_CELLS_LOG2 ? bits - LEARNED_CELLS_LOG2 : 0;
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c == 0)
  {
    p.model->kmin  = (unsigned long long) kmin;
    p.model->shift = shift;
  }
  if (c > uint32_t(LEARNED_CELLS))
  {
    return;
  }
  // lowest key of the cell, saturated at the top of the key range
  const U off    = U(c) << shift;
  const bool sat = (shift >= 8 * KB) || ((U(c) << shift) >> shift) != U(c) || U(kmin + off) < kmin;
  const U lo_key = sat ? U(~U(0)) : U(kmin + off);
  int j          = 0;
#pragma unroll 1
  for (int st = LEARNED_LEAVES / 2; st >= 1; st >>= 1)
  {
    if (U(p.model->knot[j + st]) <= lo_key)
    {
      j += st;
    }
  }
  p.model->cell_leaf[c] = (unsigned char) j;
}

// ---------------------------------------------------------------------------------------
// route: one CTA over the sorted sample. Counts the sample keys that lie in a bucket
// predicted to overflow and sets the route (LEARNED_ROUTE_*, see sort_params.h).
// ---------------------------------------------------------------------------------------
template <int KB, int FP>
__device__ __forceinline__ void learned_route_body(const LearnedRouteParams& p)
{
  using U = typename uint_of<KB>::type;
  constexpr int PER = LEARNED_SAMPLE / LEARNED_ROUTE_TPB;
  __shared__ LearnedTables<U> tables;
  __shared__ uint32_t in_large;
  learned_load_tables<U>(p.model, &tables, p.bucket_log2);
  if (threadIdx.x == 0)
  {
    in_large = 0u;
  }
  __syncthreads();
  const U* s           = static_cast<const U*>(p.sorted_sample);
  const int range_log2 = learned_range_log2(p.bucket_log2);
  const uint32_t bmax  = (1u << p.bucket_log2) - 1u;
  uint32_t count       = 0;
  for (int j = 0; j < PER; ++j)
  {
    const int i = int(threadIdx.x) * PER + j;
    if (i + p.span < LEARNED_SAMPLE)
    {
      const uint32_t b0 = learned_bucket<U, FP>(s[i], tables, range_log2, bmax);
      const uint32_t b1 = learned_bucket<U, FP>(s[i + p.span], tables, range_log2, bmax);
      count += b0 == b1 ? 1u : 0u;
    }
  }
  count = __reduce_add_sync(0xffffffffu, count);
  if ((threadIdx.x & 31) == 0)
  {
    atomicAdd(&in_large, count);
  }
  __syncthreads();
  if (threadIdx.x == 0)
  {
    p.model->route = 2u * in_large > uint32_t(LEARNED_SAMPLE) ? LEARNED_ROUTE_PLAIN : LEARNED_ROUTE_LEARNED;
  }
}

// ---------------------------------------------------------------------------------------
// hist: digit counts of every partition pass in one read of the keys
// ---------------------------------------------------------------------------------------
template <int KB, int FP, int TPB>
__device__ __forceinline__ void learned_hist_body(const LearnedHistParams& p)
{
  using U         = typename uint_of<KB>::type;
  constexpr int R = RADIX_DIGITS;
  __shared__ uint32_t sh[MAX_PASSES * R];
  __shared__ LearnedTables<U> tables;
  if (!gate_open(p.h.gate))
  {
    return;
  }

  for (int i = threadIdx.x; i < MAX_PASSES * R; i += TPB)
  {
    sh[i] = 0;
  }
  learned_load_tables<U>(p.model, &tables, p.bucket_log2);
  __syncthreads();

  const int range_log2 = learned_range_log2(p.bucket_log2);
  const uint32_t bmax  = (1u << p.bucket_log2) - 1u;
  const int passes     = p.h.num_passes;
  auto count_bucket    = [&](uint32_t b) {
#pragma unroll
    for (int q = 0; q < MAX_PASSES; ++q)
    {
      if (q < passes)
      {
        atomicAdd(&sh[q * R + ((b >> (8 * q)) & 255u)], 1u);
      }
    }
  };
  auto count_key = [&](U raw) {
    count_bucket(learned_bucket<U, FP>(encode_key<U>(raw, p.h.codec), tables, range_log2, bmax));
  };
  // the keys of several 16-byte loads (8 keys) are evaluated together (learned_bucket_batch),
  // so the loads and the model's table reads of those keys are in flight at once
  constexpr int VEC   = 16 / KB;
  constexpr int LOADS = 8 / VEC;
  const U* keys     = static_cast<const U*>(p.h.keys);
  const unsigned long long n    = p.h.num_items;
  const unsigned long long addr = reinterpret_cast<unsigned long long>(keys);
  unsigned long long head       = ((16 - (addr & 15)) & 15) / KB;
  head                          = head > n ? n : head;
  const unsigned long long nvec     = (n - head) / VEC;
  const unsigned long long body_end = head + nvec * VEC;
  if (blockIdx.x == 0)
  {
    for (unsigned long long i = threadIdx.x; i < head; i += TPB)
    {
      count_key(keys[i]);
    }
    for (unsigned long long i = body_end + threadIdx.x; i < n; i += TPB)
    {
      count_key(keys[i]);
    }
  }
  const uint4* vkeys              = reinterpret_cast<const uint4*>(keys + head);
  const unsigned long long stride = (unsigned long long) gridDim.x * TPB;
  unsigned long long v            = blockIdx.x * (unsigned long long) TPB + threadIdx.x;
  for (; v + (LOADS - 1) * stride < nvec; v += LOADS * stride)
  {
    uint4 w[LOADS];
#pragma unroll
    for (int g = 0; g < LOADS; ++g)
    {
      w[g] = __ldcs(vkeys + v + g * stride);
    }
    U k[LOADS * VEC];
    memcpy(k, w, sizeof(w));
#pragma unroll
    for (int i = 0; i < LOADS * VEC; ++i)
    {
      k[i] = encode_key<U>(k[i], p.h.codec);
    }
    uint32_t b[LOADS * VEC];
    learned_bucket_batch<U, FP, LOADS * VEC>(k, b, tables, range_log2, bmax);
#pragma unroll
    for (int i = 0; i < LOADS * VEC; ++i)
    {
      count_bucket(b[i]);
    }
  }
  for (; v < nvec; v += stride)
  {
    const uint4 w = __ldcs(vkeys + v);
    U k[VEC];
    memcpy(k, &w, 16);
#pragma unroll
    for (int i = 0; i < VEC; ++i)
    {
      count_key(k[i]);
    }
  }
  histogram_finish<TPB>(p.h, sh);
}

// ---------------------------------------------------------------------------------------
// pass: hook of the persistent onesweep pass that supplies the bucket id's digit
// ---------------------------------------------------------------------------------------
template <class U, int FP>
struct LearnedPassHook
{
  const LearnedModel* model;
  int bucket_log2;
  uint32_t bmax;
  int shift;

  template <int ITEMS>
  using digits_t = ComputedDigits<ITEMS>;

  static constexpr size_t tables_bytes = learned_tables_bytes();
  static_assert(sizeof(LearnedTables<U>) <= learned_tables_bytes(), "learned tables layout");

  __device__ __forceinline__ void setup(unsigned char* extra) const
  {
    learned_load_tables<U>(model, reinterpret_cast<LearnedTables<U>*>(extra), bucket_log2);
  }

  template <class K, int ITEMS>
  __device__ __forceinline__ void
  compute(const K (&keys)[ITEMS], uint32_t valid, int wofs, ComputedDigits<ITEMS>& dg, unsigned char* extra) const
  {
    const auto& t        = *reinterpret_cast<const LearnedTables<U>*>(extra);
    const int range_log2 = learned_range_log2(bucket_log2);
    dg.stage             = extra + tables_bytes;
#pragma unroll
    for (int i = 0; i < ITEMS; ++i)
    {
      const uint32_t idx = uint32_t(wofs + i * 32);
      dg.d[i] = idx < valid ? (learned_bucket<U, FP>(keys[i], t, range_log2, bmax) >> shift) & 255u : 255u;
    }
  }
};

template <int KB, int VB, int FP>
__device__ __forceinline__ void learned_pass_body(const LearnedPassParams& p)
{
  using U             = typename uint_of<KB>::type;
  constexpr int TPB   = persistent_tpb(KB, VB);
  constexpr int ITEMS = learned_items(KB, VB);
  constexpr size_t EXTRA = learned_extra_bytes(KB, VB, ITEMS);
  const LearnedPassHook<U, FP> hook{p.model, p.bucket_log2, (1u << p.bucket_log2) - 1u, p.digit_shift};
  onesweep_persistent_body<KB, VB, FP, TPB, ITEMS, true, LearnedPassHook<U, FP>, EXTRA>(p.os, hook);
}

// ---------------------------------------------------------------------------------------
// bounds: one read of the partitioned keys (bucket ids never decrease along them); where the
// bucket id changes from a to b at index i, begins[b] = ends[a] = i, and the last key's bucket
// ends at n. Empty buckets keep the zeros they were cleared to (begin == end). Warp w covers keys
// [w * 32 * ITEMS, (w + 1) * 32 * ITEMS), lane l the keys l, l + 32, ...; the bucket of the
// key before each comes from the neighbouring lane. A warp's keys are all loaded before the
// first is used (ITEMS = learned_bounds_items: as many loads in flight as registers allow);
// a chunk whose first and last keys share the bucket of the key before it is skipped unread.
// ---------------------------------------------------------------------------------------

template <int KB, int FP>
__device__ __forceinline__ void learned_bounds_body(const LearnedBoundsParams& p)
{
  using U = typename uint_of<KB>::type;
  if (!gate_open(p.gate))
  {
    return;
  }
  __shared__ LearnedTables<U> tables;
  learned_load_tables<U>(p.model, &tables, p.bucket_log2);
  __syncthreads();

  const unsigned long long n   = p.num_items;
  const int range_log2         = learned_range_log2(p.bucket_log2);
  const uint32_t bmax          = (1u << p.bucket_log2) - 1;
  const U* keys                = static_cast<const U*>(p.keys);
  const int lane               = threadIdx.x & 31;
  const unsigned long long warps_total = (unsigned long long) gridDim.x * (blockDim.x >> 5);
  constexpr int ITEMS                  = learned_bounds_items(KB);
  const unsigned long long chunk       = 32ull * ITEMS;
  auto bucket_at = [&](unsigned long long i) {
    return learned_bucket<U, FP>(encode_key<U>(keys[i], p.codec), tables, range_log2, bmax);
  };
  for (unsigned long long w = blockIdx.x * (unsigned long long) (blockDim.x >> 5) + (threadIdx.x >> 5);
       w * chunk < n; w += warps_total)
  {
    const unsigned long long first = w * chunk;
    const unsigned long long last  = (first + chunk < n ? first + chunk : n) - 1;
    // Buckets of the key before the chunk (none before index 0), of its first and of its
    // last key, one lane each. Bucket ids never decrease along the keys, so when the three
    // agree no bucket starts or ends inside the chunk and its keys need not be read.
    long long probe = -1;
    if (lane < 3 && !(lane == 0 && first == 0))
    {
      probe = (long long) bucket_at(lane == 0 ? first - 1 : lane == 1 ? first : last);
    }
    long long carry      = __shfl_sync(0xffffffffu, probe, 0);
    const long long b_lo = __shfl_sync(0xffffffffu, probe, 1);
    const long long b_hi = __shfl_sync(0xffffffffu, probe, 2);
    if (carry == b_lo && b_lo == b_hi && last != n - 1)
    {
      continue;
    }
    // the chunk's keys are loaded before any is used, so their loads overlap
    U k[ITEMS];
#pragma unroll
    for (int it = 0; it < ITEMS; ++it)
    {
      const unsigned long long i = first + (unsigned long long) it * 32 + lane;
      k[it]                      = i < n ? __ldcs(keys + i) : U(0);
    }
#pragma unroll
    for (int it = 0; it < ITEMS; ++it)
    {
      const unsigned long long i = first + (unsigned long long) it * 32 + lane;
      const bool valid           = i < n;
      const long long b          = valid ? (long long) learned_bucket<U, FP>(encode_key<U>(k[it], p.codec), tables, range_log2, bmax) : -2ll;
      long long prev             = __shfl_up_sync(0xffffffffu, b, 1);
      if (lane == 0)
      {
        prev = carry;
      }
      carry = __shfl_sync(0xffffffffu, b, 31);
      if (valid && b != prev)
      {
        p.begins[b] = i; // a bucket starts here
        if (prev >= 0)
        {
          p.ends[prev] = i; // and the one before it ends
        }
      }
      if (i == n - 1)
      {
        p.ends[b] = n;
      }
    }
  }
}

// ---------------------------------------------------------------------------------------
// bucket sort: per bucket of n <= CAP keys, one counting pass on the top varying bits of
// the ordering key t = digit_source(encode(key)) with 2^ceil(log2 n) bins, then the keys of
// every bin ordered by (t, index in the bucket). Since t - min is split by its top bits,
// bin order is t order; ranking a key among its bin by (t, index) makes the whole stable.
// The partition passes keep equal keys in input order, so the index in the bucket is the
// tie-break the plain sort uses. A bucket whose largest bin holds more than RUN_MAX keys
// is left to the segmented radix sort (rest_ends[b] = ends[b]).
//
// Every thread keeps its PER keys in registers from load to the final placement, and the
// values wait in shared memory in input order (all loads of a bucket precede all of its
// stores, so the output may alias the input); shared memory also holds the ordering keys
// for the comparisons, the bins (start | count << 16 after the scan) and, for bins of two
// or more keys, their members' indices. The sorted keys are assembled in shared memory,
// the values gathered through the input index of every sorted slot, and both stored with
// coalesced writes: scattered 4- and 8-byte stores cost one L1 transaction each and were
// the kernel's bottleneck.
// ---------------------------------------------------------------------------------------
template <int KB, int VB, int FP, int TPB, int CAP>
__device__ __forceinline__ void learned_bucket_body(const LearnedBucketParams& p)
{
  using U            = typename uint_of<KB>::type;
  using V            = typename value_word<VB>::type;
  using L            = LearnedBucketSmem<KB, VB, CAP>;
  constexpr int NW   = TPB / 32;
  constexpr int PER  = CAP / TPB; // keys per thread
  static_assert(CAP % TPB == 0 && CAP < 65536, "16-bit bin fields and indices");
  if (!gate_open(p.gate))
  {
    return;
  }

  extern __shared__ __align__(16) unsigned char smem[];
  U* kraw        = reinterpret_cast<U*>(smem + L::kraw_off);
  V* vst         = reinterpret_cast<V*>(smem + L::vst_off);
  uint32_t* bins = reinterpret_cast<uint32_t*>(smem + L::bins_off);
  uint16_t* perm = reinterpret_cast<uint16_t*>(smem + L::perm_off);
  static_assert(NW <= 32, "one warp combines the per-warp values");
  __shared__ unsigned long long range[2]; // min and max ordering key of the bucket
  __shared__ uint32_t scan_w[NW], run_w[NW];
  __shared__ unsigned long long bucket[3]; // id, begin, end

  const int tid  = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const U* kin   = static_cast<const U*>(p.keys_in);
  const V* vin   = static_cast<const V*>(p.values_in);
  U* kout        = static_cast<U*>(p.keys_out);
  V* vout        = static_cast<V*>(p.values_out);
  auto key_of    = [&](U k) {
    return digit_source<U, FP>(encode_key<U>(k, p.codec));
  };

  // Thread 0 takes the next bucket's ticket and bounds while the current one is sorted, and
  // has the bulk-copy unit prefetch its keys and values into L2.
  uint32_t nb_id              = 0;
  unsigned long long nb_begin = 0, nb_end = 0;
  auto fetch_next             = [&]() {
    nb_id    = atomicAdd(p.counters, 1u);
    nb_begin = nb_id < p.num_buckets ? p.begins[nb_id] : 0ull;
    nb_end   = nb_id < p.num_buckets ? p.ends[nb_id] : 0ull;
    if (nb_end > nb_begin && nb_end - nb_begin <= (unsigned long long) CAP)
    {
      // 16-byte aligned sub-range inside the arrays (which start 16-byte aligned)
      const unsigned long long kb0 = (nb_begin * KB) & ~15ull;
      const unsigned long long kb1 = min(nb_end * KB + 15, p.num_items * KB) & ~15ull;
      if (kb1 > kb0)
      {
        bulk_prefetch_l2(static_cast<const unsigned char*>(p.keys_in) + kb0, uint32_t(kb1 - kb0));
      }
      if constexpr (VB > 0)
      {
        const unsigned long long vb0 = (nb_begin * VB) & ~15ull;
        const unsigned long long vb1 = min(nb_end * VB + 15, p.num_items * VB) & ~15ull;
        if (vb1 > vb0)
        {
          bulk_prefetch_l2(static_cast<const unsigned char*>(p.values_in) + vb0, uint32_t(vb1 - vb0));
        }
      }
    }
  };
  if (tid == 0)
  {
    fetch_next();
  }
  while (true)
  {
    if (tid == 0)
    {
      bucket[0] = nb_id;
      bucket[1] = nb_begin;
      bucket[2] = nb_end;
      range[0]  = ~0ull;
      range[1]  = 0ull;
    }
    __syncthreads();
    const uint32_t b             = uint32_t(bucket[0]);
    const unsigned long long beg = bucket[1];
    const unsigned long long end = bucket[2];
    if (b >= p.num_buckets)
    {
      break;
    }
    if (tid == 0)
    {
      fetch_next();
    }
    const uint32_t n = end > beg ? uint32_t(min(end - beg, (unsigned long long) CAP + 1)) : 0u;
    if (n <= 1 || n > uint32_t(CAP))
    {
      // empty and single-key buckets need no ordering; large ones go to the segmented sort
      if (tid == 0)
      {
        p.rest_ends[b] = n > uint32_t(CAP) ? end : beg;
        if (n == 1 && p.keys_out != p.keys_in)
        {
          kout[beg] = kin[beg];
          if constexpr (VB > 0)
          {
            vout[beg] = vin[beg];
          }
        }
      }
      __syncthreads(); // bucket[] is read by everyone before thread 0 takes the next ticket
      continue;
    }
    const int s       = 32 - __clz(n - 1); // bins = 2^s >= n
    const uint32_t nb = 1u << s;
    // Rows of slots that hold keys: slot j of every thread is empty for j >= rows. Buckets
    // average half of CAP, so every per-slot loop below skips the empty rows (a CTA-uniform
    // branch) instead of running them predicated off.
    const int rows = int((n + TPB - 1) / TPB);

    // ---- load (registers and shared memory); clear the bins; range of the ordering keys ----
    // keys in registers, values in shared memory in input order (vst[i])
    U kr[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j)
    {
      const uint32_t i = tid + j * TPB;
      if (j < rows && i < n)
      {
        kr[j] = kin[beg + i];
        if constexpr (VB > 0)
        {
          vst[i] = vin[beg + i];
        }
      }
    }
    // at least 4 bins, so that the scan below works on whole 16-byte groups (the extra bins
    // stay empty: no key maps to them)
    const uint32_t nb4 = nb > 4u ? nb : 4u;
    for (uint32_t i = tid; i < nb4; i += TPB)
    {
      bins[i] = 0u;
    }
    // kraw holds the ordering keys t until the comparisons are done, then the raw keys of
    // the sorted bucket
    U lo = U(~U(0)), hi = U(0);
#pragma unroll
    for (int j = 0; j < PER; ++j)
    {
      const uint32_t i = tid + j * TPB;
      if (j < rows && i < n)
      {
        const U t = key_of(kr[j]);
        kraw[i]   = t;
        lo        = t < lo ? t : lo;
        hi        = t > hi ? t : hi;
      }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1)
    {
      const U a = __shfl_xor_sync(0xffffffffu, lo, o);
      const U c = __shfl_xor_sync(0xffffffffu, hi, o);
      lo        = a < lo ? a : lo;
      hi        = c > hi ? c : hi;
    }
    if (lane == 0)
    {
      atomicMin(&range[0], (unsigned long long) lo);
      atomicMax(&range[1], (unsigned long long) hi);
    }
    __syncthreads();
    lo = U(range[0]);
    hi = U(range[1]);

    bool sorted_here = true;
    if (lo == hi)
    {
      // one ordering key: input order is the stable order
#pragma unroll
      for (int j = 0; j < PER; ++j)
      {
        const uint32_t i = tid + j * TPB;
        if (j < rows && i < n)
        {
          kout[beg + i] = kr[j];
          if constexpr (VB > 0)
          {
            vout[beg + i] = vst[i]; // this thread's own slot
          }
        }
      }
    }
    else
    {
      const U width   = U(hi - lo);
      const int wbits = KB == 8 ? 64 - __clzll((long long) width) : 32 - __clz(uint32_t(width));
      const int shift = wbits > s ? wbits - s : 0;
      uint32_t sub[PER];
#pragma unroll
      for (int j = 0; j < PER; ++j)
      {
        const uint32_t i = tid + j * TPB;
        if (j < rows && i < n)
        {
          sub[j] = uint32_t(U(kraw[i] - lo) >> shift); // this thread's own slot
          atomicAdd(&bins[sub[j]], 1u);
        }
      }
      __syncthreads();
      // longest run; exclusive scan of the bins. Thread t owns the 16-byte groups
      // [t*gper, (t+1)*gper) of 4 bins each, read and written as uint4: scalar accesses at a
      // stride of `per` words put 4 to 8 lanes on one bank.
      const uint32_t groups = nb4 / 4u;
      const uint32_t gper   = (groups + TPB - 1) / TPB;
      const uint32_t first  = tid * gper;
      uint4* bins4          = reinterpret_cast<uint4*>(bins);
      uint32_t run = 0, sum = 0;
      for (uint32_t j = 0; j < gper; ++j)
      {
        if (first + j < groups)
        {
          const uint4 c = bins4[first + j];
          run           = max(max(run, max(c.x, c.y)), max(c.z, c.w));
          sum += c.x + c.y + c.z + c.w;
        }
      }
      uint32_t x = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1)
      {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
        {
          x += y;
        }
      }
      run = __reduce_max_sync(0xffffffffu, run);
      if (lane == 31)
      {
        scan_w[warp] = x;
        run_w[warp]  = run;
      }
      __syncthreads();
      // every warp combines the warp totals itself: lane l holds warp l's
      const uint32_t tw = lane < NW ? scan_w[lane] : 0u;
      uint32_t pw       = tw;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1)
      {
        const uint32_t y = __shfl_up_sync(0xffffffffu, pw, o);
        if (lane >= o)
        {
          pw += y;
        }
      }
      const uint32_t base    = __shfl_sync(0xffffffffu, pw - tw, warp);
      const uint32_t longest = __reduce_max_sync(0xffffffffu, lane < NW ? run_w[lane] : 0u);
      if (longest > uint32_t(LEARNED_RUN_MAX))
      {
        sorted_here = false; // uniform across the CTA
      }
      else
      {
        // bins[x] = start | count << 16
        uint32_t acc = base + x - sum;
        for (uint32_t j = 0; j < gper; ++j)
        {
          if (first + j < groups)
          {
            const uint4 c = bins4[first + j];
            uint4 o;
            o.x = acc | (c.x << 16);
            acc += c.x;
            o.y = acc | (c.y << 16);
            acc += c.y;
            o.z = acc | (c.z << 16);
            acc += c.z;
            o.w = acc | (c.w << 16);
            acc += c.w;
            bins4[first + j] = o;
          }
        }
        __syncthreads();
        // a key alone in its bin is placed; the others take a member slot of their bin (the
        // start field counts up; the count field is unchanged)
        uint32_t pos[PER];
#pragma unroll
        for (int j = 0; j < PER; ++j)
        {
          const uint32_t i = tid + j * TPB;
          pos[j]           = 0xffffffffu;
          if (j < rows && i < n)
          {
            const uint32_t w = bins[sub[j]];
            if ((w >> 16) == 1u)
            {
              pos[j] = w & 0xffffu;
            }
            else
            {
              perm[atomicAdd(&bins[sub[j]], 1u) & 0xffffu] = uint16_t(i);
            }
          }
        }
        __syncthreads();
        // rank the others among their bin's members by (t, index); bins[x] = end | count << 16
#pragma unroll
        for (int j = 0; j < PER; ++j)
        {
          const uint32_t i = tid + j * TPB;
          if (j < rows && i < n && pos[j] == 0xffffffffu)
          {
            const uint32_t w  = bins[sub[j]];
            const uint32_t b1 = w & 0xffffu;
            const uint32_t b0 = b1 - (w >> 16);
            uint32_t rank     = 0;
            if (shift == 0)
            {
              // a bin holds one ordering key: the index alone decides
              for (uint32_t r = b0; r < b1; ++r)
              {
                rank += perm[r] < i ? 1u : 0u;
              }
            }
            else
            {
              const U ti = kraw[i];
              for (uint32_t r = b0; r < b1; ++r)
              {
                const uint32_t m = perm[r];
                const U tm       = kraw[m];
                rank += (tm < ti || (tm == ti && m < i)) ? 1u : 0u;
              }
            }
            pos[j] = b0 + rank;
          }
        }
        __syncthreads(); // every comparison read of kraw and perm is done
        // sorted keys in shared memory, and for every sorted slot the input index of its
        // key (perm, free after the ranking), which gathers the values; coalesced stores
#pragma unroll
        for (int j = 0; j < PER; ++j)
        {
          const uint32_t i = tid + j * TPB;
          if (j < rows && i < n)
          {
            kraw[pos[j]] = kr[j];
            if constexpr (VB > 0)
            {
              perm[pos[j]] = uint16_t(i);
            }
          }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PER; ++j)
        {
          const uint32_t q = tid + j * TPB;
          if (j < rows && q < n)
          {
            kout[beg + q] = kraw[q];
            if constexpr (VB > 0)
            {
              vout[beg + q] = vst[perm[q]];
            }
          }
        }
      }
    }
    if (tid == 0)
    {
      p.rest_ends[b] = sorted_here ? beg : end;
      if (sorted_here)
      {
        atomicAdd(p.counters + 1, 1u);
      }
    }
    __syncthreads(); // shared buffers and bucket[] free for the next bucket
  }
}

} // namespace gb300
