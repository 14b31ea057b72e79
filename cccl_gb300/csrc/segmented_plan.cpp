// Host dispatcher of the batched segmented sort (see segmented_plan.h).
//
// Reference: cub/cub/device/dispatch/dispatch_segmented_sort.cuh
//   temp-storage layout and size query            :459-574
//   buffer routing, final selector                :579-669, :722-746
//   partitioning threshold (> 500 segments)       :465
// The large-segment passes use 8-bit digits (CUB uses 6-bit ones); when the caller allows
// overwriting, the pass count is adjusted by splitting one digit so the result lands in the
// same buffer CUB's 6-bit pass count selects, and the returned selector is CUB's.
#include "segmented_plan.h"

#include <algorithm>
#include <cstdio>
#include <string>

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
} // namespace

void segmented_kernel_names(int kb, int vb, int kind, bool descending, char (&names)[SK_COUNT][64])
{
  // descending float radix classes fold -0.0 into +0.0 before ordering, as CUB's block-radix
  // paths do (FP_BLOCK_DESC); over whole keys the order is the same as the onesweep folding
  const std::string fs  = kind == KIND_FLOAT ? (descending ? "fd" : "f") : "i";
  const std::string kv  = "k" + std::to_string(kb) + "_v" + std::to_string(vb) + "_";
  const std::string net = kv + (kind == KIND_FLOAT ? "f" : kind == KIND_SIGNED ? "i" : "u");
  const std::string rad = kv + fs;
  const std::string n[SK_COUNT] = {
    "gb300_init",
    "gb300_seg_classify",
    "gb300_seg_small_" + net,
    "gb300_seg_medium_" + net,
    "gb300_seg_block_s_" + rad,
    "gb300_seg_block_l_" + rad,
    "gb300_seg_hist_k" + std::to_string(kb) + "_" + fs,
    "gb300_seg_scan",
    "gb300_seg_pass_" + rad,
    "gb300_seg_small_" + kv + "r" + fs,
    "gb300_seg_medium_" + kv + "r" + fs,
    "gb300_seg_ppass_" + rad,
    "gb300_seg_block_xs_" + rad};
  for (int i = 0; i < SK_COUNT; ++i)
  {
    std::snprintf(names[i], sizeof(names[i]), "%s", n[i].c_str());
  }
}

SegmentedPolicy make_segmented_policy(int kb, int vb, int kind)
{
  SegmentedPolicy p{};
  p.key_bytes           = kb;
  p.value_bytes         = vb;
  p.key_kind            = kind;
  p.small_threads       = seg_small_threads(kb, vb);
  p.small_items         = seg_small_items(kb, vb);
  p.medium_threads      = seg_medium_threads(kb, vb);
  p.medium_items        = seg_medium_items(kb, vb);
  p.block_s_cap         = SEG_BLOCK_S_CAP;
  p.block_l_cap         = SEG_BLOCK_L_CAP;
  p.pass_tpb            = seg_pass_tpb(kb, vb);
  p.pass_items          = seg_pass_items(kb, vb);
  p.network_small_smem  = seg_network_smem(kb, vb, p.small_threads, p.small_items);
  p.network_medium_smem = seg_network_smem(kb, vb, p.medium_threads, p.medium_items);
  p.network_rsmall_smem  = seg_network_smem(kb, vb, SEG_RSMALL_THREADS, SEG_RSMALL_ITEMS);
  p.network_rmedium_smem = seg_network_smem(kb, vb, SEG_RMEDIUM_THREADS, SEG_RMEDIUM_ITEMS);
  p.block_s_tpb         = seg_block_s_tpb(kb);
  p.block_l_tpb         = seg_block_l_tpb(kb);
  p.block_s_smem        = seg_block_smem(kb, seg_block_s_tpb(kb), seg_block_s_items(kb));
  p.block_l_smem        = seg_block_smem(kb, seg_block_l_tpb(kb), seg_block_l_items(kb));
  p.pass_smem           = onesweep_smem_for(kb, vb, seg_pass_tpb(kb, vb), seg_pass_items(kb, vb));
  p.ppass_tpb           = seg_ppass_tpb(kb, vb);
  p.ppass_items         = seg_ppass_items(kb, vb);
  p.ppass_smem          = seg_ppass_smem(kb, vb);
  return p;
}

void segmented_sort_dispatch(const SegmentedPolicy& pol, const SegmentedKernels& ks, const SegmentedCall& c,
                             int* selector)
{
  const int kb        = pol.key_bytes;
  const int vb        = pol.value_bytes;
  const bool has_vals = vb > 0 && c.values[0] != nullptr;
  const uint64_t n    = c.num_items;
  const uint64_t nseg = c.num_segments;
  *selector           = 0;
  if (c.d_temp_storage != nullptr && c.num_items > 0 && vb > 0 && c.values[0] == nullptr)
  {
    // the kernels of a pairs build move values unconditionally
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "the build sorts pairs but the values are null");
  }

  // ---- digit passes of the large segments and the buffer that receives the result ----
  // DeviceSegmentedSort: CUB's large segments take ceil(key bits / 6) passes (4-bit digits
  // for 1-byte keys). DeviceSegmentedRadixSort (dispatch_segmented_radix_sort.cuh:734-745 and
  // :519-526): max(ceil(window / R), 1) passes, R = 6 (5 for 1-byte keys), and the result is
  // in the output buffer whenever overwriting is not allowed.
  const int begin_bit = c.radix_only ? c.begin_bit : 0;
  const int end_bit   = c.radix_only ? c.end_bit : 8 * kb;
  if (begin_bit < 0 || end_bit > 8 * kb || begin_bit > end_bit)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "begin_bit/end_bit outside the key");
  }
  if (c.radix_only && begin_bit == end_bit && c.overwrite)
  {
    // nothing to sort and the caller takes the current buffer (dispatch_segmented_radix_sort.cuh:541)
    if (c.d_temp_storage == nullptr)
    {
      *c.temp_storage_bytes = 1;
    }
    return;
  }
  const int cub_passes = c.radix_only
                         ? std::max<int>(int(ceil_div(uint64_t(end_bit - begin_bit), kb > 1 ? 6 : 5)), 1)
                         : int(ceil_div(uint64_t(8 * kb), kb > 1 ? 6 : 4));
  const int target = c.target >= 0 ? c.target : c.overwrite ? (cub_passes & 1) : 1;
  int bit[SEG_MAX_PASSES];
  int bits[SEG_MAX_PASSES];
  int passes = 0;
  for (int b = begin_bit; b < end_bit; b += RADIX_BITS)
  {
    bit[passes]  = b;
    bits[passes] = std::min(RADIX_BITS, end_bit - b);
    ++passes;
  }
  if (passes == 0)
  {
    // an empty window still moves every large segment once (a 0-bit pass is a copy)
    bit[0]  = begin_bit;
    bits[0] = 0;
    passes  = 1;
  }
  if (c.overwrite && (passes & 1) != target)
  {
    // split the last digit into two passes (one may have 0 bits): the parity now matches
    const int w      = bits[passes - 1];
    bits[passes - 1] = (w + 1) / 2;
    bit[passes]      = bit[passes - 1] + (w + 1) / 2;
    bits[passes]     = w / 2;
    ++passes;
  }

  // ---- temporary storage ----
  // The pipelined pass bulk-copies 16-byte-aligned ranges of the pass buffers, so it needs
  // aligned buffers (the temporary ones are); otherwise the CTA-per-tile pass runs. The
  // tile size follows the kernel.
  auto aligned16 = [](const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; };
  const bool pipelined = aligned16(c.keys[0]) && aligned16(c.keys[1])
                      && (!has_vals || (aligned16(c.values[0]) && aligned16(c.values[1])));
  const uint64_t ptile     = uint64_t(pol.ppass_tpb - LOOKBACK_THREADS) * pol.ppass_items;
  const uint64_t ctile     = uint64_t(pol.pass_tpb) * pol.pass_items;
  const uint64_t pass_tile = pipelined ? ptile : ctile;
  const uint64_t max_dev   = std::min<uint64_t>(nseg, n / (uint64_t(pol.block_l_cap) + 1));
  // tile lists and look-back rows sized for the smaller tile of the two pass kernels, so the
  // size a caller queried is enough whichever kernel the buffers' alignment selects
  const uint64_t max_tiles = ceil_div(n, std::min(ptile, ctile)) + max_dev;
  const bool need_tmp      = !c.overwrite && passes > 1 && max_dev > 0;

  size_t off               = 0;
  const size_t ctrl_off    = off;
  off += align_up(4 * SEG_CTR_WORDS, 256);
  const size_t zero_bytes  = off; // the control block is zeroed per call (classify clears the counts rows it uses)
  const size_t counts_off  = off;
  off += align_up(4 * size_t(max_dev) * passes * RADIX_DIGITS, 256);
  const size_t lists_off   = off;
  off += 5 * align_up(4 * size_t(nseg), 256); // one segment list per block or network class
  const size_t dev_off     = off;
  off += align_up(sizeof(DeviceSegment) * size_t(max_dev), 256);
  const size_t tseg_off    = off;
  off += align_up(4 * size_t(max_tiles), 256);
  const size_t bins_off    = off;
  off += align_up(8 * size_t(max_dev) * passes * RADIX_DIGITS, 256);
  const size_t lb_off      = off;
  const size_t lb_words    = size_t(max_tiles) * RADIX_DIGITS;
  off += align_up(2 * 4 * lb_words, 256);
  const size_t ktmp_off    = off;
  if (need_tmp)
  {
    off += align_up(size_t(n) * kb, 256);
  }
  const size_t vtmp_off = off;
  if (need_tmp && has_vals)
  {
    off += align_up(size_t(n) * vb, 256);
  }
  const size_t total = std::max<size_t>(off, 1);

  if (c.d_temp_storage == nullptr)
  {
    *c.temp_storage_bytes = total;
    return;
  }
  if (n == 0 || nseg == 0)
  {
    // nothing runs: word 0 (the status word) still reads "no error" for a status query
    if (*c.temp_storage_bytes >= 4)
    {
      check(cuMemsetD32Async(CUdeviceptr(c.d_temp_storage), 0u, 1, c.stream), "cuMemsetD32Async(status)");
    }
    return;
  }
  if (*c.temp_storage_bytes < total)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "temp storage is smaller than the size query returned");
  }
  if ((reinterpret_cast<uintptr_t>(c.d_temp_storage) & 255) != 0)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "temp storage is not 256-byte aligned");
  }
  for (int i = 0; i < 2; ++i)
  {
    if (c.keys[i] == nullptr || (reinterpret_cast<uintptr_t>(c.keys[i]) % kb) != 0
        || (has_vals && (c.values[i] == nullptr || (reinterpret_cast<uintptr_t>(c.values[i]) % vb) != 0)))
    {
      throw cuda_error(CUDA_ERROR_INVALID_VALUE, "key/value buffers must be non-null and element aligned");
    }
  }
  if (c.begin_offsets == nullptr || c.end_offsets == nullptr)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "segment offsets are null");
  }

  auto* base     = static_cast<unsigned char*>(c.d_temp_storage);
  auto* counters = reinterpret_cast<uint32_t*>(base + ctrl_off);
  uint32_t* status = counters + SEG_CTR_STATUS;
  auto* lists    = reinterpret_cast<uint32_t*>(base + lists_off);
  const size_t list_stride = align_up(4 * size_t(nseg), 256) / 4;
  auto* dev_list = reinterpret_cast<DeviceSegment*>(base + dev_off);
  auto* tseg     = reinterpret_cast<uint32_t*>(base + tseg_off);
  auto* counts   = reinterpret_cast<uint32_t*>(base + counts_off);
  auto* bins     = reinterpret_cast<unsigned long long*>(base + bins_off);
  uint32_t* lb[2] = {reinterpret_cast<uint32_t*>(base + lb_off), reinterpret_cast<uint32_t*>(base + lb_off) + lb_words};
  void* ktmp     = base + ktmp_off;
  void* vtmp     = base + vtmp_off;

  const KeyCodec codec = make_codec(pol.key_kind, kb, c.descending);
  const int sms        = sm_count();
  void* final_keys     = c.keys[target];
  void* final_vals     = has_vals ? c.values[target] : nullptr;

  // 1. zero the counters and the per-segment digit counts
  {
    InitParams p{};
    p.words     = counters;
    p.num_words = zero_bytes / 4;
    launch("seg_init", ks.k[SK_INIT], unsigned(std::min<uint64_t>(ceil_div(p.num_words, 256), 4096)), 256, 0, c.stream,
           p);
  }
  // 2. size classes, on the device
  {
    SegClassifyParams p{};
    p.begin_offsets   = c.begin_offsets;
    p.end_offsets     = c.end_offsets;
    p.offsets_64      = c.offsets_64;
    p.partition       = c.radix_only || nseg > uint64_t(SEG_PARTITION_THRESHOLD);
    p.num_segments    = nseg;
    p.num_items       = n;
    p.max_device_segments = max_dev;
    p.max_tiles       = max_tiles;
    p.small_tile      = c.radix_only ? SEG_RSMALL_THREADS * SEG_RSMALL_ITEMS : pol.small_threads * pol.small_items;
    p.medium_tile     = c.radix_only ? SEG_RMEDIUM_THREADS * SEG_RMEDIUM_ITEMS : pol.medium_threads * pol.medium_items;
    p.block_xs_cap    = SEG_BLOCK_XS_CAP;
    p.block_small_cap = pol.block_s_cap;
    p.block_large_cap = pol.block_l_cap;
    p.device_tile     = uint32_t(pass_tile);
    p.counters        = counters;
    p.small_list      = lists;
    p.medium_list     = lists + list_stride;
    p.block_s_list    = lists + 2 * list_stride;
    p.block_l_list    = lists + 3 * list_stride;
    p.block_xs_list   = lists + 4 * list_stride;
    p.device_list     = dev_list;
    p.tile_segment    = tseg;
    p.status          = status;
    p.seg_counts      = counts;
    p.num_passes      = passes;
    launch("seg_classify", ks.k[SK_CLASSIFY], unsigned(std::min<uint64_t>(ceil_div(nseg, 256), uint64_t(sms) * 8)), 256,
           0, c.stream, p);
  }
  // 3. warp and block classes: straight from the input into the final buffer
  {
    SegSortParams p{};
    p.keys_in       = c.keys[0];
    p.keys_out      = final_keys;
    p.values_in     = has_vals ? c.values[0] : nullptr;
    p.values_out    = final_vals;
    p.begin_offsets = c.begin_offsets;
    p.end_offsets   = c.end_offsets;
    p.offsets_64    = c.offsets_64;
    p.descending    = c.descending ? 1 : 0;
    p.counters      = counters;
    p.small_list    = lists;
    p.medium_list   = lists + list_stride;
    p.block_s_list  = lists + 2 * list_stride;
    p.block_l_list  = lists + 3 * list_stride;
    p.block_xs_list = lists + 4 * list_stride;
    p.codec         = codec;
    p.begin_bit     = begin_bit;
    p.end_bit       = end_bit;
    // radix order: the same networks comparing digit sources (every segment count)
    const CUkernel small        = c.radix_only ? ks.k[SK_RSMALL] : ks.k[SK_SMALL];
    const CUkernel medium       = c.radix_only ? ks.k[SK_RMEDIUM] : ks.k[SK_MEDIUM];
    const uint64_t small_smem   = c.radix_only ? pol.network_rsmall_smem : pol.network_small_smem;
    const uint64_t medium_smem  = c.radix_only ? pol.network_rmedium_smem : pol.network_medium_smem;
    if (c.radix_only || nseg > uint64_t(SEG_PARTITION_THRESHOLD))
    {
      launch("seg_small", small, unsigned(sms * occupancy(small, SEG_NETWORK_TPB, small_smem)), SEG_NETWORK_TPB,
             small_smem, c.stream, p);
    }
    launch("seg_medium", medium, unsigned(sms * occupancy(medium, SEG_NETWORK_TPB, medium_smem)), SEG_NETWORK_TPB,
           medium_smem, c.stream, p);
    const int xs_tpb       = seg_block_xs_tpb(kb);
    const uint64_t xs_smem = seg_block_smem(kb, xs_tpb, seg_block_xs_items(kb));
    launch("seg_block_xs", ks.k[SK_BLOCK_XS], unsigned(sms * occupancy(ks.k[SK_BLOCK_XS], xs_tpb, xs_smem)),
           unsigned(xs_tpb), xs_smem, c.stream, p);
    launch("seg_block_s", ks.k[SK_BLOCK_S], unsigned(sms * occupancy(ks.k[SK_BLOCK_S], pol.block_s_tpb, pol.block_s_smem)),
           unsigned(pol.block_s_tpb), pol.block_s_smem, c.stream, p);
    launch("seg_block_l", ks.k[SK_BLOCK_L], unsigned(sms * occupancy(ks.k[SK_BLOCK_L], pol.block_l_tpb, pol.block_l_smem)),
           unsigned(pol.block_l_tpb), pol.block_l_smem, c.stream, p);
  }
  // 4. device class: every large segment together, one launch per digit pass
  if (max_dev > 0)
  {
    SegDeviceParams p{};
    p.keys_in     = c.keys[0];
    p.num_items   = n;
    p.num_passes  = passes;
    p.device_tile = uint32_t(pass_tile);
    p.counters    = counters;
    p.device_list = dev_list;
    p.tile_segment = tseg;
    p.seg_counts  = counts;
    p.seg_bins    = bins;
    p.lookback[0] = lb[0];
    p.lookback[1] = lb[1];
    p.status      = status;
    p.codec       = codec;
    for (int q = 0; q < passes; ++q)
    {
      p.pass_bit[q]  = bit[q];
      p.pass_bits[q] = bits[q];
      void* kd;
      void* vd;
      if (c.overwrite)
      {
        kd = c.keys[(q + 1) & 1];
        vd = has_vals ? c.values[(q + 1) & 1] : nullptr;
      }
      else
      {
        const bool to_out = ((passes - 1 - q) % 2) == 0;
        kd                = to_out ? c.keys[1] : ktmp;
        vd                = has_vals ? (to_out ? c.values[1] : vtmp) : nullptr;
      }
      p.keys_dst[q]   = kd;
      p.values_dst[q] = vd;
      p.keys_src[q]   = q == 0 ? c.keys[0] : p.keys_dst[q - 1];
      p.values_src[q] = has_vals ? (q == 0 ? c.values[0] : p.values_dst[q - 1]) : nullptr;
    }
    // one shared table per tile. A lane-column form (one CTA per SM over a contiguous range
    // of tiles, counters flushed when the segment changes) measured slower on C3: 0.461 ms
    // against 0.282 ms (the flushes of 1024 rows per segment change dominate)
    launch("seg_hist", ks.k[SK_HIST], unsigned(sms * 4), HISTOGRAM_TPB, 0, c.stream, p);
    launch("seg_scan", ks.k[SK_SCAN], unsigned(sms * 4), 256, 0, c.stream, p);
    if (pipelined)
    {
      // persistent: every CTA resident (a tile waits on lower tiles of its segment)
      const unsigned grid = unsigned(sms * occupancy(ks.k[SK_PPASS], pol.ppass_tpb, pol.ppass_smem));
      for (int q = 0; q < passes; ++q)
      {
        p.pass = q;
        launch_cooperative("seg_pass", ks.k[SK_PPASS], grid, unsigned(pol.ppass_tpb), pol.ppass_smem, c.stream, p);
      }
    }
    else
    {
      const unsigned pass_grid = unsigned(sms * occupancy(ks.k[SK_PASS], pol.pass_tpb, pol.pass_smem));
      for (int q = 0; q < passes; ++q)
      {
        p.pass = q;
        launch("seg_pass", ks.k[SK_PASS], pass_grid, unsigned(pol.pass_tpb), pol.pass_smem, c.stream, p);
      }
    }
  }
  *selector = target;
}

} // namespace gb300
