// Host dispatcher of the learned-partition sort (see learned_plan.h).
//
// No reference counterpart: it is a second form of DeviceRadixSort::SortKeys/SortPairs with
// the same result and the same DoubleBuffer selector as the plain sort
// (cub/cub/device/dispatch/dispatch_radix_sort.cuh:1698-1948 leaves the result of a
// full-width sort of k-byte keys after k 8-bit passes, i.e. in the current buffer when k is
// even). Bucket count: about 2^learned_bucket_items_log2 keys per bucket (2048 or 4096, sorted
// in shared memory); the partition needs
// ceil(log2(buckets) / 8) stable passes.
#include "learned_plan.h"

#include <algorithm>
#include <cstddef>

#include "abi_common.h"
#include "sort_policy.h"

namespace gb300
{

namespace
{
uint64_t ceil_div(uint64_t a, uint64_t b)
{
  return (a + b - 1) / b;
}

int ceil_log2(uint64_t x)
{
  int l = 0;
  while ((1ull << l) < x)
  {
    ++l;
  }
  return l;
}

bool aligned16(const void* p)
{
  return (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}

// Stand-in buffers for size queries: 256-byte aligned, never dereferenced.
void* fake_ptr(int i)
{
  return reinterpret_cast<void*>(uintptr_t(256) * uintptr_t(i + 1));
}

SegmentedCall bucket_sort_call(const LearnedSetup& s, const RadixCall& c, const LearnedTempPlan& t)
{
  SegmentedCall sc{};
  sc.keys[0]       = fake_ptr(0);
  sc.keys[1]       = fake_ptr(1);
  sc.values[0]     = (s.value_bytes > 0 && c.values[0] != nullptr) ? fake_ptr(2) : nullptr;
  sc.values[1]     = sc.values[0] != nullptr ? fake_ptr(3) : nullptr;
  sc.num_items     = c.num_items;
  sc.num_segments  = 1ull << t.bucket_log2;
  sc.begin_offsets = fake_ptr(4);
  sc.end_offsets   = fake_ptr(5);
  sc.offsets_64    = 1;
  sc.overwrite     = true;
  sc.descending    = c.descending;
  sc.stream        = c.stream;
  sc.target        = 0;
  // radix order in every bucket: the merge networks of small segments compare floats as
  // floats (NaN placement), the plain sort orders bit patterns
  sc.radix_only    = true;
  sc.begin_bit     = 0;
  sc.end_bit       = 8 * s.key_bytes;
  return sc;
}
} // namespace

LearnedTempPlan plan_learned_temp(const LearnedSetup& s, const RadixCall& c)
{
  LearnedTempPlan t{};
  const int kb        = s.key_bytes;
  const int vb        = s.value_bytes;
  const bool has_vals = vb > 0 && c.values[0] != nullptr;
  const bool aligned  = aligned16(c.keys[0]) && aligned16(c.keys[1])
                    && (!has_vals || (aligned16(c.values[0]) && aligned16(c.values[1])));
  t.learned = c.num_items >= LEARNED_MIN_ITEMS && c.begin_bit == 0 && c.end_bit == 8 * kb && aligned
           && (kb == 4 || kb == 8) && (vb == 0 || vb == 4 || vb == 8);
  if (!t.learned)
  {
    return t;
  }
  const uint64_t n = c.num_items;
  const int items_log2 = learned_bucket_items_log2(ceil_log2(n));
  t.bucket_log2        = std::clamp(ceil_log2(n) - items_log2, 8, LEARNED_MAX_BUCKET_LOG2);
  t.bucket_cap         = 2 << items_log2;
  t.passes         = (t.bucket_log2 + RADIX_BITS - 1) / RADIX_BITS;
  // Cost model. The learned route moves about (partition passes + 1 bucket-sort pass) times
  // 2 (K + V) bytes per key, the plain sort K passes of the same (8-bit digits of a K-byte
  // key), and the learned kernels ran at about 0.7 of the plain passes' bandwidth on GB300
  // (model evaluation per key, in-shared-memory bucket sort). So it takes the learned route
  // only when (passes + 1) / 0.7 < K: 8-byte keys (3 + 1 against 8 passes), never 4-byte keys
  // (2 + 1 against 4). Inputs it sends to the plain sort cost nothing extra.
  if (s.route_policy == LEARNED_POLICY_COST_MODEL && (t.passes + 1) * 10 >= kb * 7)
  {
    t         = LearnedTempPlan{};
    t.learned = false;
    return t;
  }
  t.tile_items     = persistent_tile_items(s.pass_tpb, s.pass_items);
  t.portion_items  = ((1ull << 30) - 1) / t.tile_items * t.tile_items; // 30-bit look-back counts
  t.num_portions   = ceil_div(n, t.portion_items);
  const uint64_t lookback_rows = ceil_div(n, t.tile_items) + t.num_portions;

  size_t off   = 0;
  t.ctrl_off   = off;
  t.ctrl_bytes = align_up(sizeof(SortControl) + 4 * size_t(t.passes) * t.num_portions, 256);
  off += t.ctrl_bytes;
  t.bins_off = off;
  off += align_up(8 * size_t(t.passes) * t.num_portions * RADIX_DIGITS, 256);
  t.lookback_off   = off;
  t.lookback_words = size_t(lookback_rows) * RADIX_DIGITS;
  off += align_up(2 * 4 * t.lookback_words, 256);
  t.model_off = off;
  off += align_up(sizeof(LearnedModel), 256);
  t.sample_off = off;
  off += 2 * align_up(size_t(LEARNED_SAMPLE) * kb, 256);
  t.sample_temp_off   = off;
  t.sample_temp_bytes = plan_radix_temp(s.sample_pol, LEARNED_SAMPLE, 0, 8 * kb, false, true).total_bytes;
  off += align_up(t.sample_temp_bytes, 256);
  t.bounds_off = off;
  off += 256 + align_up(3 * 8 * (size_t(1) << t.bucket_log2), 256); // counters; begins, ends, rest_ends
  // The plain route's temporary storage. Without overwrite it holds alternate key and value
  // buffers of n items, which the learned passes use as their own (only one route runs).
  {
    const RadixTempPlan pt = plan_radix_temp(s.plain_pol, n, 0, 8 * kb, !c.overwrite, true);
    t.plain_off            = off;
    t.plain_bytes          = pt.total_bytes;
    t.keys_tmp_off         = t.plain_off + pt.keys_tmp_off;
    t.values_tmp_off       = t.plain_off + pt.values_tmp_off;
    off += align_up(t.plain_bytes, 256);
  }
  t.seg_off = off;
  // the buffer the bucket sort must land in changes its pass count: size for both
  t.seg_bytes = 0;
  for (int target = 0; target < 2; ++target)
  {
    SegmentedCall sc      = bucket_sort_call(s, c, t);
    size_t bytes          = 0;
    sc.d_temp_storage     = nullptr;
    sc.temp_storage_bytes = &bytes;
    sc.target             = target;
    int sel               = 0;
    segmented_sort_dispatch(s.seg_pol, s.seg_ks, sc, &sel);
    t.seg_bytes = std::max(t.seg_bytes, bytes);
  }
  off += align_up(t.seg_bytes, 256);
  t.fallback_off   = off;
  t.fallback_bytes = 0;
  if (n >= (1ull << 30))
  {
    t.fallback_bytes = plan_radix_temp(s.plain_pol, n, 0, 8 * kb, true, true).total_bytes;
    off += align_up(t.fallback_bytes, 256);
  }
  t.total_bytes = off;
  return t;
}

void learned_sort_dispatch(const LearnedSetup& s, const RadixCall& c, int* selector)
{
  *selector             = 0;
  const LearnedTempPlan t = plan_learned_temp(s, c);
  if (!t.learned)
  {
    radix_sort_dispatch(s.plain_pol, s.plain_ks, c, selector);
    return;
  }
  if (c.d_temp_storage == nullptr)
  {
    *c.temp_storage_bytes = t.total_bytes;
    return;
  }
  const int kb        = s.key_bytes;
  const int vb        = s.value_bytes;
  const bool has_vals = vb > 0 && c.values[0] != nullptr;
  const uint64_t n    = c.num_items;
  if (*c.temp_storage_bytes < t.total_bytes)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "temp storage is smaller than the size query returned");
  }
  if ((reinterpret_cast<uintptr_t>(c.d_temp_storage) & 255) != 0)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "temp storage is not 256-byte aligned");
  }
  if (c.keys[0] == nullptr || c.keys[1] == nullptr || (has_vals && c.values[1] == nullptr))
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "key/value buffer is null");
  }
  if (vb > 0 && !has_vals)
  {
    // the kernels of a pairs build move values unconditionally
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "the build sorts pairs but the values are null");
  }

  auto* base          = static_cast<unsigned char*>(c.d_temp_storage);
  auto* ctrl          = reinterpret_cast<SortControl*>(base + t.ctrl_off);
  auto* tile_ctrs     = reinterpret_cast<uint32_t*>(base + t.ctrl_off + sizeof(SortControl));
  auto* bins          = reinterpret_cast<unsigned long long*>(base + t.bins_off);
  uint32_t* lb[2]     = {reinterpret_cast<uint32_t*>(base + t.lookback_off),
                         reinterpret_cast<uint32_t*>(base + t.lookback_off) + t.lookback_words};
  auto* model         = reinterpret_cast<LearnedModel*>(base + t.model_off);
  void* sample[2]     = {base + t.sample_off, base + t.sample_off + align_up(size_t(LEARNED_SAMPLE) * kb, 256)};
  auto* bucket_ctrs   = reinterpret_cast<uint32_t*>(base + t.bounds_off);
  auto* begins        = reinterpret_cast<unsigned long long*>(base + t.bounds_off + 256);
  auto* ends          = begins + (size_t(1) << t.bucket_log2);
  auto* rest_ends     = ends + (size_t(1) << t.bucket_log2);

  void* keys_tmp      = base + t.keys_tmp_off;
  void* values_tmp    = base + t.values_tmp_off;
  const KeyCodec codec = make_codec(s.key_kind, kb, c.descending);
  const int sms        = sm_count();
  const int plain_passes = int(ceil_div(uint64_t(8 * kb), RADIX_BITS));
  const int final_sel    = plain_passes & 1; // the plain sort's selector

  // 1. zero the control block
  {
    InitParams p{};
    p.words     = reinterpret_cast<uint32_t*>(ctrl);
    p.num_words = t.ctrl_bytes / 4;
    launch("learned_init", s.lk.init, unsigned(std::min<uint64_t>(ceil_div(p.num_words, 256), 1024)), 256, 0,
           c.stream, p);
  }
  // 2. sample, 3. its plain radix sort (exact ranks), 4. least-squares fit per leaf and the
  // cell table of the leaf lookup
  {
    LearnedSampleParams p{};
    p.keys      = c.keys[0];
    p.num_items = n;
    p.sample    = sample[0];
    p.codec     = codec;
    launch("learned_sample", s.lk.sample, unsigned(LEARNED_SAMPLE / 256), 256, 0, c.stream, p);
  }
  int ssel = 0;
  {
    RadixCall sc{};
    sc.keys[0]            = sample[0];
    sc.keys[1]            = sample[1];
    sc.num_items          = LEARNED_SAMPLE;
    sc.begin_bit          = 0;
    sc.end_bit            = 8 * kb;
    sc.overwrite          = true;
    sc.descending         = false;
    sc.d_temp_storage     = base + t.sample_temp_off;
    size_t bytes          = t.sample_temp_bytes;
    sc.temp_storage_bytes = &bytes;
    sc.stream             = c.stream;
    sc.status_word        = &ctrl->status;
    radix_sort_dispatch(s.sample_pol, s.sample_ks, sc, &ssel);
  }
  {
    LearnedFitParams p{};
    p.sorted_sample = sample[ssel];
    p.model         = model;
    launch("learned_fit", s.lk.fit, unsigned(LEARNED_LEAVES), unsigned(LEARNED_FIT_TPB), 0, c.stream, p);
    launch("learned_cells", s.lk.cells, unsigned(ceil_div(LEARNED_CELLS + 1, 256)), 256, 0, c.stream, p);
  }
  // 4b. the route: the learned kernels below run only on LEARNED_ROUTE_LEARNED, the plain
  // sort at the end only on LEARNED_ROUTE_PLAIN (a flag on the device: no host sync)
  {
    LearnedRouteParams p{};
    p.sorted_sample = sample[ssel];
    p.model         = model;
    p.bucket_log2   = t.bucket_log2;
    p.span          = int(std::max<uint64_t>(1, ceil_div(uint64_t(t.bucket_cap) * LEARNED_SAMPLE, n)));
    launch("learned_route", s.lk.route, 1, unsigned(LEARNED_ROUTE_TPB), 0, c.stream, p);
  }
  const KernelGate learned_gate{&model->route, LEARNED_ROUTE_LEARNED, 0};
  const KernelGate plain_gate{&model->route, LEARNED_ROUTE_PLAIN, 0};
  // 5. digit counts of every partition pass (and pass 0's look-back cleared)
  {
    LearnedHistParams p{};
    p.h.keys           = c.keys[0];
    p.h.num_items      = n;
    p.h.codec          = codec;
    p.h.begin_bit      = 0;
    p.h.end_bit        = t.bucket_log2;
    p.h.num_passes     = t.passes;
    p.h.num_portions   = int(t.num_portions);
    p.h.ctrl           = ctrl;
    p.h.bins           = bins;
    p.h.lookback_clear = lb[0];
    p.h.lookback_words = t.lookback_words;
    p.h.gate           = learned_gate;
    p.model            = model;
    p.bucket_log2      = t.bucket_log2;
    const uint64_t want = ceil_div(n, uint64_t(HISTOGRAM_TPB) * (16 / kb) * 4);
    const unsigned grid = unsigned(std::max<uint64_t>(1, std::min<uint64_t>(want, uint64_t(sms) * 4)));
    launch("learned_hist", s.lk.hist, grid, unsigned(HISTOGRAM_TPB), 0, c.stream, p);
  }
  // 6. stable partition passes on the bucket id, low digit first
  const int P = t.passes;
  void* ksrc[MAX_PASSES];
  void* kdst[MAX_PASSES];
  void* vsrc[MAX_PASSES];
  void* vdst[MAX_PASSES];
  for (int q = 0; q < P; ++q)
  {
    if (c.overwrite)
    {
      ksrc[q] = c.keys[q & 1];
      kdst[q] = c.keys[(q + 1) & 1];
      vsrc[q] = c.values[q & 1];
      vdst[q] = c.values[(q + 1) & 1];
    }
    else
    {
      const bool to_tmp = ((P - 1 - q) % 2) == 0; // the last pass lands in the temp buffers
      kdst[q]           = to_tmp ? keys_tmp : c.keys[1];
      vdst[q]           = to_tmp ? values_tmp : c.values[1];
      ksrc[q]           = q == 0 ? c.keys[0] : kdst[q - 1];
      vsrc[q]           = q == 0 ? c.values[0] : vdst[q - 1];
    }
  }
  const uint64_t tiles_per_portion = t.portion_items / t.tile_items;
  const unsigned pass_grid_cap = unsigned(sms * occupancy(s.lk.pass, s.pass_tpb, s.pass_smem));
  for (int q = 0; q < P; ++q)
  {
    for (uint64_t pi = 0; pi < t.num_portions; ++pi)
    {
      const uint64_t first = pi * t.portion_items;
      const uint64_t items = std::min<uint64_t>(n - first, t.portion_items);
      LearnedPassParams lp{};
      OnesweepParams& op  = lp.os;
      op.keys_in          = static_cast<const unsigned char*>(ksrc[q]) + first * kb;
      op.keys_out         = kdst[q];
      op.values_in        = has_vals ? static_cast<const unsigned char*>(vsrc[q]) + first * vb : nullptr;
      op.values_out       = has_vals ? vdst[q] : nullptr;
      op.portion_begin    = first;
      op.num_items_total  = n;
      op.portion_items    = uint32_t(items);
      op.portion_tiles    = uint32_t(ceil_div(items, t.tile_items));
      op.tile_row_base    = uint32_t(pi * tiles_per_portion);
      op.lookback         = lb[q & 1];
      op.lookback_next    = (q + 1 < P) ? lb[(q + 1) & 1] : nullptr;
      op.tile_counter     = tile_ctrs + (size_t(q) * t.num_portions + pi);
      op.bins             = bins + (size_t(q) * t.num_portions + pi) * RADIX_DIGITS;
      op.bins_next        = (pi + 1 < t.num_portions) ? bins + (size_t(q) * t.num_portions + pi + 1) * RADIX_DIGITS : nullptr;
      op.status           = &ctrl->status;
      op.codec            = codec;
      op.current_bit      = q * RADIX_BITS;
      op.num_bits         = std::min(RADIX_BITS, t.bucket_log2 - q * RADIX_BITS);
      op.encode_in        = q == 0;
      op.decode_out       = q == P - 1;
      op.gate             = learned_gate;
      lp.model            = model;
      lp.bucket_log2      = t.bucket_log2;
      lp.digit_shift      = q * RADIX_BITS;
      const unsigned grid = std::min<unsigned>(op.portion_tiles, pass_grid_cap);
      launch_cooperative("learned_pass", s.lk.pass, grid, unsigned(s.pass_tpb), s.pass_smem, c.stream, lp);
    }
  }
  void* part_keys = kdst[P - 1];
  void* part_vals = has_vals ? vdst[P - 1] : nullptr;
  // 7. begin and end of every bucket, from one read of the partitioned keys. The counters and
  // all three bound arrays are cleared on either route: on the plain route every bucket stays
  // empty, so the segmented sort below has nothing to do
  {
    InitParams z{};
    z.words     = bucket_ctrs; // the counters, begins, ends and rest_ends
    z.num_words = 64 + 6 * (uint64_t(1) << t.bucket_log2);
    launch("learned_init", s.lk.init, unsigned(std::min<uint64_t>(ceil_div(z.num_words, 256), uint64_t(sms) * 8)),
           256, 0, c.stream, z);
    LearnedBoundsParams p{};
    p.keys        = part_keys;
    p.num_items   = n;
    p.model       = model;
    p.begins      = begins;
    p.ends        = ends;
    p.codec       = codec;
    p.bucket_log2 = t.bucket_log2;
    p.gate        = learned_gate;
    const uint64_t warps = ceil_div(n, 32ull * learned_bounds_items(kb));
    const unsigned grid  = unsigned(std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(warps, 8), uint64_t(sms) * 16)));
    launch("learned_bounds", s.lk.bounds, grid, 256, 0, c.stream, p);
  }
  // 8. every bucket sorted as a segment; the result lands where the plain sort puts it
  {
    void* final_keys  = c.overwrite ? c.keys[final_sel] : c.keys[1];
    void* other_keys  = part_keys == c.keys[0] ? c.keys[1] : part_keys == c.keys[1] ? c.keys[0] : c.keys[1];
    void* other_vals  = nullptr;
    if (has_vals)
    {
      other_vals = part_vals == c.values[0] ? c.values[1] : part_vals == c.values[1] ? c.values[0] : c.values[1];
    }
    // 8a. buckets of up to bucket_cap keys: one wide counting pass each, in shared memory
    {
      LearnedBucketParams bp{};
      bp.keys_in     = part_keys;
      bp.values_in   = part_vals;
      bp.keys_out    = final_keys;
      bp.values_out  = has_vals ? (final_keys == part_keys ? part_vals : other_vals) : nullptr;
      bp.begins      = begins;
      bp.ends        = ends;
      bp.rest_ends   = rest_ends;
      bp.counters    = bucket_ctrs;
      bp.num_buckets = uint32_t(1u << t.bucket_log2);
      bp.num_items   = n;
      bp.codec       = codec;
      bp.gate        = learned_gate;
      const CUkernel k    = t.bucket_cap == 4096 ? s.lk.bucket4k : s.lk.bucket8k;
      const int tpb       = learned_bucket_tpb(t.bucket_cap);
      const size_t smem   = learned_bucket_smem(kb, vb, t.bucket_cap);
      const unsigned grid = unsigned(sms * occupancy(k, tpb, smem));
      launch("learned_bucket", k, grid, unsigned(tpb), smem, c.stream, bp);
    }
    // 8b. the rest (larger buckets, buckets with long runs of equal top bits): segmented radix sort
    SegmentedCall sc      = bucket_sort_call(s, c, t);
    sc.keys[0]            = part_keys;
    sc.keys[1]            = other_keys;
    sc.values[0]          = part_vals;
    sc.values[1]          = other_vals;
    sc.begin_offsets      = begins;
    sc.end_offsets        = rest_ends;
    sc.target             = final_keys == part_keys ? 0 : 1;
    sc.d_temp_storage     = base + t.seg_off;
    size_t bytes          = t.seg_bytes;
    sc.temp_storage_bytes = &bytes;
    int seg_sel           = 0;
    segmented_sort_dispatch(s.seg_pol, s.seg_ks, sc, &seg_sel);
    // its errors are the call's; a bucket too large for it is not (step 9 sorts it)
    {
      StatusFoldParams fp{};
      fp.dst  = &ctrl->status;
      fp.src  = reinterpret_cast<const uint32_t*>(base + t.seg_off) + SEG_CTR_STATUS;
      fp.mask = ~STATUS_BAD_SEGMENT;
      launch("learned_status", s.lk.status_fold, 1, 32, 0, c.stream, fp);
    }
    // 9. a bucket of 2^30 or more keys was left unsorted: a stable sort of the partitioned
    // keys equals the stable sort of the input (the partition keeps equal keys in order),
    // so the plain radix sort of them into the final buffer finishes the job
    if (t.fallback_bytes > 0)
    {
      RadixCall fc{};
      fc.keys[0]            = part_keys;
      fc.keys[1]            = final_keys;
      fc.values[0]          = part_vals;
      fc.values[1]          = has_vals ? (c.overwrite ? c.values[final_sel] : c.values[1]) : nullptr;
      fc.num_items          = n;
      fc.begin_bit          = 0;
      fc.end_bit            = 8 * kb;
      fc.overwrite          = false;
      fc.descending         = c.descending;
      fc.d_temp_storage     = base + t.fallback_off;
      size_t fbytes         = t.fallback_bytes;
      fc.temp_storage_bytes = &fbytes;
      fc.stream             = c.stream;
      fc.gate.gate          = reinterpret_cast<const uint32_t*>(base + t.seg_off) + SEG_CTR_STATUS;
      fc.gate.gate_mask     = STATUS_BAD_SEGMENT;
      fc.status_word        = &ctrl->status;
      int fsel              = 0;
      radix_sort_dispatch(s.plain_pol, s.plain_ks, fc, &fsel);
    }
  }
  // 10. the plain route: the plain radix sort of the input, where the learned sort puts its
  // result (the same buffer and selector)
  {
    RadixCall pc{};
    pc.keys[0]            = c.keys[0];
    pc.keys[1]            = c.keys[1];
    pc.values[0]          = has_vals ? c.values[0] : nullptr;
    pc.values[1]          = has_vals ? c.values[1] : nullptr;
    pc.num_items          = n;
    pc.begin_bit          = 0;
    pc.end_bit            = 8 * kb;
    pc.overwrite          = c.overwrite;
    pc.descending         = c.descending;
    pc.d_temp_storage     = base + t.plain_off;
    size_t pbytes         = t.plain_bytes;
    pc.temp_storage_bytes = &pbytes;
    pc.stream             = c.stream;
    pc.gate               = plain_gate;
    pc.status_word        = &ctrl->status;
    int psel              = 0;
    radix_sort_dispatch(s.plain_pol, s.plain_ks, pc, &psel);
  }
  *selector = final_sel;
}

LearnedStats learned_sort_stats(const LearnedSetup& s, const RadixCall& c)
{
  LearnedStats st{};
  const LearnedTempPlan t = plan_learned_temp(s, c);
  st.learned              = t.learned ? 1 : 0;
  if (!t.learned || c.d_temp_storage == nullptr)
  {
    return st;
  }
  st.bucket_log2      = t.bucket_log2;
  st.partition_passes = t.passes;
  uint32_t route      = 0;
  check(cuMemcpyDtoH(&route,
                     CUdeviceptr(static_cast<unsigned char*>(c.d_temp_storage) + t.model_off + offsetof(LearnedModel, route)),
                     sizeof(route)),
        "cuMemcpyDtoH(learned route)");
  if (route != LEARNED_ROUTE_LEARNED)
  {
    st.learned = 0; // the model sent this input to the plain radix sort
    return st;
  }
  uint32_t w[SEG_CTR_WORDS];
  check(cuMemcpyDtoH(w, CUdeviceptr(static_cast<unsigned char*>(c.d_temp_storage) + t.seg_off), sizeof(w)),
        "cuMemcpyDtoH(learned stats)");
  uint32_t bucket_ctrs[2];
  check(cuMemcpyDtoH(bucket_ctrs, CUdeviceptr(static_cast<unsigned char*>(c.d_temp_storage) + t.bounds_off),
                     sizeof(bucket_ctrs)),
        "cuMemcpyDtoH(learned stats)");
  st.block_buckets = bucket_ctrs[1] + w[SEG_CTR_SMALL] + w[SEG_CTR_MEDIUM] + w[SEG_CTR_BLOCK_XS] + w[SEG_CTR_BLOCK_S] + w[SEG_CTR_BLOCK_L];
  st.device_buckets = w[SEG_CTR_DEVICE];
  std::memcpy(&st.device_items, &w[SEG_CTR_DEVICE_ITEMS], sizeof(st.device_items));
  return st;
}

} // namespace gb300
