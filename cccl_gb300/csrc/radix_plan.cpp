// Host dispatcher of the plain radix sort (see radix_plan.h).
//
// Reference: cub/cub/device/dispatch/dispatch_radix_sort.cuh
//   special cases        :1950-2003 (empty input / begin_bit == end_bit / single tile)
//   copy                 :1364-1420 (begin_bit == end_bit without overwrite)
//   single tile          :1307-1362 (selector flips once)
//   onesweep driver      :1698-1948 (temp plan, portions, pass loop, buffer ping-pong)
// The selector values written here are the ones CUB's dispatch leaves in the caller's
// DoubleBuffer, so code that routes on the selector behaves identically.
#include "radix_plan.h"

#include <algorithm>

#include "abi_common.h"
#include "sort_policy.h"

namespace gb300
{

RadixPolicy make_radix_policy(int key_bytes, int value_bytes, int key_kind)
{
  RadixPolicy p{};
  p.key_bytes         = key_bytes;
  p.value_bytes       = value_bytes;
  p.key_kind          = key_kind;
  p.onesweep_tpb      = ONESWEEP_TPB;
  p.onesweep_items    = onesweep_items(key_bytes, value_bytes);
  p.single_tile_tpb   = SINGLE_TILE_TPB;
  p.single_tile_items = SINGLE_TILE_ITEMS;
  p.histogram_tpb     = HISTOGRAM_LANES_TPB;
  p.onesweep_smem     = onesweep_smem_bytes(key_bytes, value_bytes);
  p.persistent_tpb    = persistent_tpb(key_bytes, value_bytes);
  p.persistent_items  = persistent_items(key_bytes, value_bytes);
  p.persistent_smem   = persistent_smem_bytes(key_bytes, value_bytes);
  p.single_tile_smem  = single_tile_smem_bytes(key_bytes);
  return p;
}

RadixKernelNames radix_kernel_names(int kb, int vb, int kind, bool descending)
{
  const std::string kv = "k" + std::to_string(kb) + "_v" + std::to_string(vb) + "_" + (kind == KIND_FLOAT ? "f" : "i");
  RadixKernelNames n;
  n.init      = "gb300_init";
  n.histogram = "gb300_histogram_k" + std::to_string(kb) + "_" + (kind == KIND_FLOAT ? "f" : "i");
  n.onesweep  = "gb300_onesweep_" + kv;
  n.onesweep_dyn = "gb300_onesweep_dyn_" + kv;
  // integer keys-only sorts have an order-free first-pass kernel
  n.onesweep_first = (vb == 0 && kind != KIND_FLOAT) ? "gb300_onesweep_first_" + kv : n.onesweep;
  // descending float sorts: CUB's single tile folds -0.0 into +0.0 before ordering (FP_BLOCK_DESC)
  n.single_tile = "gb300_single_tile_" + (kind == KIND_FLOAT && descending ? kv + "d" : kv);
  return n;
}

static uint64_t ceil_div(uint64_t a, uint64_t b)
{
  return (a + b - 1) / b;
}

RadixTempPlan
plan_radix_temp(const RadixPolicy& pol, uint64_t n, int begin_bit, int end_bit, bool need_tmp, bool persistent)
{
  RadixTempPlan t{};
  t.num_passes    = int(ceil_div(uint64_t(end_bit - begin_bit), RADIX_BITS));
  t.tile_items    = persistent ? persistent_tile_items(pol.persistent_tpb, pol.persistent_items)
                               : uint64_t(pol.onesweep_tpb) * pol.onesweep_items;
  // Look-back words carry a 30-bit count, so one launch covers < 2^30 keys.
  t.portion_items = ((1ull << 30) - 1) / t.tile_items * t.tile_items;
  t.num_portions  = ceil_div(n, t.portion_items);
  t.total_tiles   = ceil_div(n, t.tile_items);
  // Look-back rows are sized for the smaller tile of the two pass kernels, so the size a
  // caller queried is enough whichever kernel the buffers' alignment selects.
  const uint64_t min_tile = std::min<uint64_t>(persistent_tile_items(pol.persistent_tpb, pol.persistent_items),
                                               uint64_t(pol.onesweep_tpb) * pol.onesweep_items);
  const uint64_t lookback_rows = ceil_div(n, min_tile) + t.num_portions;

  size_t off     = 0;
  t.ctrl_off     = off;
  t.ctrl_bytes   = align_up(sizeof(SortControl) + 4 * size_t(t.num_passes) * t.num_portions, 256);
  off += t.ctrl_bytes;
  t.bins_off = off;
  off += align_up(8 * size_t(t.num_passes) * t.num_portions * RADIX_DIGITS, 256);
  t.lookback_off   = off;
  t.lookback_words = size_t(lookback_rows) * RADIX_DIGITS;
  off += align_up(2 * 4 * t.lookback_words, 256);
  t.keys_tmp_off = off;
  if (need_tmp)
  {
    off += align_up(size_t(n) * pol.key_bytes, 256);
  }
  t.values_tmp_off = off;
  if (need_tmp && pol.value_bytes > 0)
  {
    off += align_up(size_t(n) * pol.value_bytes, 256);
  }
  t.total_bytes = off;
  return t;
}

static bool aligned16(const void* p)
{
  return (reinterpret_cast<uintptr_t>(p) & 15u) == 0;
}

// Paths that use no temporary storage still leave word 0 of a caller's buffer (the status
// word the onesweep path reports into) reading "no error", so that a status query after any
// call reads that call's status, not an earlier one's.
static void clear_status_word(const RadixCall& c)
{
  if (c.status_word == nullptr && c.d_temp_storage != nullptr && *c.temp_storage_bytes >= 4)
  {
    check(cuMemsetD32Async(CUdeviceptr(c.d_temp_storage), 0u, 1, c.stream), "cuMemsetD32Async(status)");
  }
}

static void check_aligned(const void* p, size_t a, const char* what)
{
  if (p != nullptr && (reinterpret_cast<uintptr_t>(p) % a) != 0)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, std::string(what) + " is not aligned to its element size");
  }
}

void radix_sort_dispatch(const RadixPolicy& pol, const RadixKernels& ks, const RadixCall& c, int* selector)
{
  const int kb         = pol.key_bytes;
  const int vb         = pol.value_bytes;
  const bool has_vals  = vb > 0 && c.values[0] != nullptr;
  const uint64_t n     = c.num_items;
  *selector            = 0;
  if (c.d_temp_storage != nullptr && c.num_items > 0 && vb > 0 && c.values[0] == nullptr)
  {
    // the kernels of a pairs build move values unconditionally
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "the build sorts pairs but the values are null");
  }

  if (c.begin_bit < 0 || c.end_bit > 8 * kb || c.begin_bit > c.end_bit)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "begin_bit/end_bit outside the key");
  }
  if (vb > 0 && c.values[0] != nullptr && c.values[1] == nullptr)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "values output is null");
  }
  // empty problem, or nothing to sort and the caller accepts the input buffer as result
  if (n == 0 || (c.begin_bit == c.end_bit && c.overwrite))
  {
    if (c.d_temp_storage == nullptr)
    {
      *c.temp_storage_bytes = 1;
    }
    else
    {
      clear_status_word(c);
    }
    return;
  }
  for (int i = 0; i < 2; ++i)
  {
    check_aligned(c.keys[i], size_t(kb), "key buffer");
    if (has_vals)
    {
      check_aligned(c.values[i], size_t(vb), "value buffer");
    }
  }
  if (c.keys[0] == nullptr || c.keys[1] == nullptr)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "key buffer is null");
  }

  const KeyCodec codec = make_codec(pol.key_kind, kb, c.descending);
  if (c.gate.gate != nullptr && (c.begin_bit == c.end_bit || n <= cub_single_tile_limit(kb, vb)))
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "a gated sort must take the onesweep path");
  }

  if (c.begin_bit == c.end_bit)
  {
    if (c.d_temp_storage == nullptr)
    {
      *c.temp_storage_bytes = 1;
      return;
    }
    clear_status_word(c);
    check(cuMemcpyAsync(CUdeviceptr(c.keys[1]), CUdeviceptr(c.keys[0]), n * kb, c.stream), "cuMemcpyAsync(keys)");
    if (has_vals)
    {
      check(cuMemcpyAsync(CUdeviceptr(c.values[1]), CUdeviceptr(c.values[0]), n * vb, c.stream),
            "cuMemcpyAsync(values)");
    }
    *selector = 1;
    return;
  }

  if (n <= cub_single_tile_limit(kb, vb))
  {
    if (c.d_temp_storage == nullptr)
    {
      *c.temp_storage_bytes = 1;
      return;
    }
    SingleTileParams p{};
    p.keys_in    = c.keys[0];
    p.keys_out   = c.keys[1];
    p.values_in  = has_vals ? c.values[0] : nullptr;
    p.values_out = has_vals ? c.values[1] : nullptr;
    p.num_items  = uint32_t(n);
    p.begin_bit  = c.begin_bit;
    p.end_bit    = c.end_bit;
    p.codec      = codec;
    clear_status_word(c);
    launch("single_tile", ks.single_tile, 1, unsigned(pol.single_tile_tpb), pol.single_tile_smem, c.stream, p);
    *selector = 1;
    return;
  }

  const int passes    = int(ceil_div(uint64_t(c.end_bit - c.begin_bit), RADIX_BITS));
  const bool need_tmp = !c.overwrite && passes > 1;
  // The persistent kernel bulk-copies tiles straight from the pass inputs, which needs
  // 16-byte aligned buffers; otherwise every pass uses the CTA-per-tile kernel.
  const bool persistent = aligned16(c.keys[0]) && aligned16(c.keys[1])
                       && (!has_vals || (aligned16(c.values[0]) && aligned16(c.values[1])));
  const RadixTempPlan t = plan_radix_temp(pol, n, c.begin_bit, c.end_bit, need_tmp, persistent);
  if (c.d_temp_storage == nullptr)
  {
    *c.temp_storage_bytes = t.total_bytes;
    return;
  }
  if (*c.temp_storage_bytes < t.total_bytes)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "temp storage is smaller than the size query returned");
  }
  check_aligned(c.d_temp_storage, 256, "temp storage");

  auto* base       = static_cast<unsigned char*>(c.d_temp_storage);
  auto* ctrl       = reinterpret_cast<SortControl*>(base + t.ctrl_off);
  auto* tile_ctrs  = reinterpret_cast<uint32_t*>(base + t.ctrl_off + sizeof(SortControl));
  auto* bins       = reinterpret_cast<unsigned long long*>(base + t.bins_off);
  uint32_t* lb[2]  = {reinterpret_cast<uint32_t*>(base + t.lookback_off),
                      reinterpret_cast<uint32_t*>(base + t.lookback_off) + t.lookback_words};
  void* keys_tmp   = base + t.keys_tmp_off;
  void* values_tmp = base + t.values_tmp_off;

  // 1. zero the control block (histogram counters, tile counters, status)
  {
    InitParams p{};
    p.words     = reinterpret_cast<uint32_t*>(ctrl);
    p.num_words = t.ctrl_bytes / 4;
    p.gate      = c.gate;
    const unsigned grid = unsigned(std::min<uint64_t>(ceil_div(p.num_words, 256), 1024));
    launch("init", ks.init, grid, 256, 0, c.stream, p);
  }
  // 2. all-pass histogram + exclusive scan (+ clears pass 0's look-back)
  {
    HistogramParams p{};
    p.keys           = c.keys[0];
    p.num_items      = n;
    p.codec          = codec;
    p.begin_bit      = c.begin_bit;
    p.end_bit        = c.end_bit;
    p.num_passes     = passes;
    p.num_portions   = int(t.num_portions);
    p.ctrl           = ctrl;
    p.bins           = bins;
    p.lookback_clear = lb[0];
    p.lookback_words = t.lookback_words;
    p.gate           = c.gate;
    // the pass plan: passes whose digit is the same for every key are skipped
    p.plan      = ctrl->plan;
    p.plan_mode = c.overwrite ? PLAN_MODE_DOUBLE : PLAN_MODE_SEPARATE;
    // one lane-column CTA per SM (fewer for small inputs: four 16-byte loads per thread)
    const uint64_t want = ceil_div(n, uint64_t(HISTOGRAM_LANES_TPB) * (16 / kb) * 4);
    const unsigned grid = unsigned(std::max<uint64_t>(1, std::min<uint64_t>(want, uint64_t(sm_count()))));
    launch("histogram", ks.histogram, grid, unsigned(HISTOGRAM_LANES_TPB), histogram_table_bytes(passes), c.stream, p);
  }
  // 3. one onesweep launch per (pass, portion)
  void* kdst[MAX_PASSES];
  void* vdst[MAX_PASSES];
  void* ksrc[MAX_PASSES];
  void* vsrc[MAX_PASSES];
  for (int p = 0; p < passes; ++p)
  {
    if (c.overwrite)
    {
      ksrc[p] = c.keys[p & 1];
      kdst[p] = c.keys[(p + 1) & 1];
      vsrc[p] = c.values[p & 1];
      vdst[p] = c.values[(p + 1) & 1];
    }
    else
    {
      const bool to_out = ((passes - 1 - p) % 2) == 0;
      kdst[p]           = to_out ? c.keys[1] : keys_tmp;
      vdst[p]           = to_out ? c.values[1] : values_tmp;
      ksrc[p]           = p == 0 ? c.keys[0] : kdst[p - 1];
      vsrc[p]           = p == 0 ? c.values[0] : vdst[p - 1];
    }
  }
  const uint64_t tiles_per_portion = t.portion_items / t.tile_items;
  // buffer tables of the pass plan (PLAN_MODE_DOUBLE: {current, alternate};
  // PLAN_MODE_SEPARATE: {input, output, temporary})
  const void* key_bufs[3]   = {c.keys[0], c.keys[1], c.overwrite ? nullptr : keys_tmp};
  const void* value_bufs[3] = {has_vals ? c.values[0] : nullptr, has_vals ? c.values[1] : nullptr,
                               (c.overwrite || !has_vals) ? nullptr : values_tmp};
  for (int p = 0; p < passes; ++p)
  {
    const int bit = c.begin_bit + p * RADIX_BITS;
    for (uint64_t q = 0; q < t.num_portions; ++q)
    {
      const uint64_t first = q * t.portion_items;
      const uint64_t items = std::min<uint64_t>(n - first, t.portion_items);
      OnesweepParams op{};
      op.keys_in       = static_cast<const unsigned char*>(ksrc[p]) + first * kb;
      op.keys_out      = kdst[p];
      op.values_in     = has_vals ? static_cast<const unsigned char*>(vsrc[p]) + first * vb : nullptr;
      op.values_out    = has_vals ? vdst[p] : nullptr;
      op.portion_begin = first;
      op.num_items_total = n;
      op.portion_items = uint32_t(items);
      op.portion_tiles = uint32_t(ceil_div(items, t.tile_items));
      op.tile_row_base = uint32_t(q * tiles_per_portion);
      op.lookback      = lb[p & 1];
      op.lookback_next = (p + 1 < passes) ? lb[(p + 1) & 1] : nullptr;
      op.tile_counter  = tile_ctrs + (size_t(p) * t.num_portions + q);
      op.bins          = bins + (size_t(p) * t.num_portions + q) * RADIX_DIGITS;
      op.bins_next     = (q + 1 < t.num_portions) ? bins + (size_t(p) * t.num_portions + q + 1) * RADIX_DIGITS : nullptr;
      op.status        = c.status_word != nullptr ? c.status_word : &ctrl->status;
      op.codec         = codec;
      op.current_bit   = bit;
      op.num_bits      = std::min(RADIX_BITS, c.end_bit - bit);
      op.encode_in     = p == 0;
      op.decode_out    = p == passes - 1;
      op.gate          = c.gate;
      op.plan          = &ctrl->plan[p];
      op.plan_prev     = p > 0 ? &ctrl->plan[p - 1] : nullptr;
      for (int b = 0; b < 3; ++b)
      {
        op.key_bufs[b]   = key_bufs[b];
        op.value_bufs[b] = value_bufs[b];
      }
      if (persistent)
      {
        const bool order_free =
          p == 0 && !has_vals && pol.key_kind != KIND_FLOAT && c.begin_bit == 0 && c.end_bit == 8 * kb;
        const CUkernel k    = order_free ? ks.onesweep_first : ks.onesweep;
        const unsigned grid = unsigned(std::min<uint64_t>(
          op.portion_tiles, uint64_t(sm_count()) * occupancy(k, pol.persistent_tpb, pol.persistent_smem)));
        launch_cooperative("onesweep", k, grid, unsigned(pol.persistent_tpb), pol.persistent_smem, c.stream, op);
      }
      else
      {
        launch("onesweep", ks.onesweep_dyn, op.portion_tiles, unsigned(pol.onesweep_tpb), pol.onesweep_smem, c.stream,
               op);
      }
    }
  }
  *selector = passes & 1;
}

} // namespace gb300
