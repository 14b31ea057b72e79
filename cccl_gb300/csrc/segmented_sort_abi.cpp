// C ABI of the batched segmented sort: cccl_device_segmented_sort_{build,build_ex,compile,
// load,link_ltoir,serialize,deserialize,cleanup}, the run entry cccl_device_segmented_sort and
// cccl_gb300_segmented_radix_sort (DeviceSegmentedRadixSort semantics, same build).
//
// Reference interface: c/parallel/include/cccl/c/segmented_sort.h:27-139, implemented in
// c/parallel/src/segmented_sort.cu (run :859-985: null selector rejected :875-881, keys and
// values must be pointers, offsets through iterators :916-917).
#include <cccl/c/segmented_sort.h>
#include <cccl_gb300/segmented_radix_sort.h>

#include <memory>

#include "abi_common.h"
#include "offset_iterators.h"
#include "segmented_plan.h"
#include "value_gather.h"
#include "sort_policy.h"

using namespace gb300;

namespace
{

constexpr uint32_t SEG_POLICY_MAGIC = 0x53425047u; // "GPBS"
constexpr uint32_t SEG_TABLE_MAGIC  = 0x54425047u; // "GPBT"
constexpr uint32_t ALGO_SEGMENTED   = 8u;          // CCCL_SERIALIZATION_ALGO_SEGMENTED_SORT

// Names (and, once loaded, handles) of every kernel the run needs; kept in the build
// result's partition_runtime_policy slot, which the reference uses for its partition policy.
struct SegKernelTable
{
  uint32_t magic;
  char names[SK_COUNT][64];
  CUkernel handles[SK_COUNT];
  // begin and end offsets given as iterators: their evaluation kernels, compiled at build
  // time (null: both are pointers; an entry without an image is a pointer)
  OffsetIteratorKernel* offsets;
};

void free_offsets(SegKernelTable* tab)
{
  if (tab != nullptr && tab->offsets != nullptr)
  {
    free_offset_iterator(tab->offsets[0]);
    free_offset_iterator(tab->offsets[1]);
    delete[] tab->offsets;
    tab->offsets = nullptr;
  }
}

bool keys_only(const cccl_iterator_t& values)
{
  return values.type == CCCL_POINTER && values.state == nullptr;
}

void free_result(cccl_device_segmented_sort_build_result_t* b)
{
  delete[] static_cast<char*>(b->payload);
  b->payload = nullptr;
  std::free(b->runtime_policy);
  b->runtime_policy = nullptr;
  free_offsets(static_cast<SegKernelTable*>(b->partition_runtime_policy));
  std::free(b->partition_runtime_policy);
  b->partition_runtime_policy = nullptr;
  for (char** p :
       {&b->segmented_sort_fallback_kernel_lowered_name,
        &b->segmented_sort_kernel_small_lowered_name,
        &b->segmented_sort_kernel_large_lowered_name,
        &b->three_way_partition_init_kernel_lowered_name,
        &b->three_way_partition_kernel_lowered_name})
  {
    delete[] *p;
    *p = nullptr;
  }
}

// The run of both entry points; radix_only selects DeviceSegmentedRadixSort's semantics.
CUresult segmented_run(const char* who,
                       cccl_device_segmented_sort_build_result_t build,
                       void* d_temp_storage,
                       size_t* temp_storage_bytes,
                       cccl_iterator_t d_keys_in,
                       cccl_iterator_t d_keys_out,
                       cccl_iterator_t d_values_in,
                       cccl_iterator_t d_values_out,
                       uint64_t num_items,
                       uint64_t num_segments,
                       cccl_iterator_t start_offset_in,
                       cccl_iterator_t end_offset_in,
                       bool radix_only,
                       int begin_bit,
                       int end_bit,
                       bool is_overwrite_okay,
                       int* selector,
                       CUstream stream)
{
  if (selector == nullptr)
  {
    fflush(stderr);
    printf("\nERROR in %s(): selector cannot be nullptr\n", who);
    fflush(stdout);
    return CUDA_ERROR_UNKNOWN;
  }
  if (d_keys_in.type != CCCL_POINTER || d_keys_out.type != CCCL_POINTER || d_values_in.type != CCCL_POINTER
      || d_values_out.type != CCCL_POINTER)
  {
    fflush(stderr);
    printf("\nERROR in %s(): keys and values must be pointers\n", who);
    fflush(stdout);
    return CUDA_ERROR_UNKNOWN;
  }
  const bool iter_begin = start_offset_in.type == CCCL_ITERATOR;
  const bool iter_end   = end_offset_in.type == CCCL_ITERATOR;
  if ((iter_begin || iter_end)
      && (build.partition_runtime_policy == nullptr
          || static_cast<const SegKernelTable*>(build.partition_runtime_policy)->offsets == nullptr
          || (iter_begin && static_cast<const SegKernelTable*>(build.partition_runtime_policy)->offsets[0].kernel == nullptr)
          || (iter_end && static_cast<const SegKernelTable*>(build.partition_runtime_policy)->offsets[1].kernel == nullptr)))
  {
    printf("\nERROR in %s(): segment offsets are iterators, but the build compiled pointer offsets\n", who);
    return CUDA_ERROR_NOT_SUPPORTED;
  }
  const size_t osz = start_offset_in.value_type.size;
  if ((osz != 4 && osz != 8) || end_offset_in.value_type.size != osz || temp_storage_bytes == nullptr)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  try
  {
    context_guard ctx;
    if (build.runtime_policy == nullptr || build.runtime_policy_size != sizeof(SegmentedPolicy)
        || static_cast<const SegmentedPolicy*>(build.runtime_policy)->magic != SEG_POLICY_MAGIC
        || build.partition_runtime_policy == nullptr || build.library == nullptr)
    {
      return CUDA_ERROR_NOT_INITIALIZED;
    }
    const auto& pol = *static_cast<const SegmentedPolicy*>(build.runtime_policy);
    const auto& tab = *static_cast<const SegKernelTable*>(build.partition_runtime_policy);
    SegmentedKernels ks{};
    for (int i = 0; i < SK_COUNT; ++i)
    {
      ks.k[i] = tab.handles[i];
    }
    SegmentedCall call{};
    // offsets given as iterators are evaluated, in their own type, into arrays at the tail
    // of the temporary storage (the sort's own part, with its status word, stays at the
    // front); the sort reads those like pointers
    const int n_iter       = int(iter_begin) + int(iter_end);
    const size_t off_bytes = n_iter > 0 ? align_up(size_t(num_segments) * osz, 16) : 0;
    const size_t tail      = n_iter * off_bytes;
    const bool sizing      = d_temp_storage == nullptr;
    if (!sizing && *temp_storage_bytes < tail)
    {
      throw cuda_error(CUDA_ERROR_INVALID_VALUE, "temp storage is smaller than the size query returned");
    }
    auto* tbase        = static_cast<unsigned char*>(d_temp_storage);
    size_t inner_bytes = sizing ? 0 : (*temp_storage_bytes - tail) / 16 * 16;
    void* offsets[2]   = {start_offset_in.state, end_offset_in.state};
    for (int e = 0, slot = 0; e < 2; ++e)
    {
      const cccl_iterator_t& oit = e == 0 ? start_offset_in : end_offset_in;
      if (oit.type != CCCL_ITERATOR)
      {
        continue;
      }
      // placeholders while sizing: aligned and non-null, never read
      offsets[e] = sizing ? reinterpret_cast<void*>(uintptr_t(256) * (e + 1))
                          : static_cast<void*>(tbase + inner_bytes + slot * off_bytes);
      if (!sizing)
      {
        if (tab.offsets[e].value_size != osz)
        {
          throw cuda_error(CUDA_ERROR_INVALID_VALUE, "offset iterator type differs from the one the build compiled");
        }
        evaluate_offset_iterator(tab.offsets[e], oit, num_segments, offsets[e], stream);
      }
      ++slot;
    }
    call.keys[0]            = d_keys_in.state;
    call.keys[1]            = d_keys_out.state;
    call.values[0]          = d_values_in.state;
    call.values[1]          = d_values_out.state;
    call.num_items          = num_items;
    call.num_segments       = num_segments;
    call.begin_offsets      = offsets[0];
    call.end_offsets        = offsets[1];
    call.offsets_64         = osz == 8 ? 1 : 0;
    call.overwrite          = is_overwrite_okay;
    call.descending         = build.order == CCCL_DESCENDING;
    call.d_temp_storage     = d_temp_storage;
    call.temp_storage_bytes = n_iter == 0 ? temp_storage_bytes : &inner_bytes;
    call.stream             = stream;
    call.target             = -1;
    call.radix_only         = radix_only;
    call.begin_bit          = begin_bit;
    call.end_bit            = end_bit;
    int sel                 = 0;
    if (pol.gather_value_bytes > 0 && call.values[0] != nullptr)
    {
      sort_with_gathered_values(
        build.library, uint32_t(pol.gather_value_bytes), call.values, num_items, is_overwrite_okay, true,
        call.d_temp_storage, call.temp_storage_bytes, stream,
        [&](void* const idx[2], void* temp, size_t* bytes, int* s) {
          SegmentedCall inner      = call;
          inner.values[0]          = idx[0];
          inner.values[1]          = idx[1];
          inner.d_temp_storage     = temp;
          inner.temp_storage_bytes = bytes;
          segmented_sort_dispatch(pol, ks, inner, s);
        },
        &sel);
    }
    else
    {
      segmented_sort_dispatch(pol, ks, call, &sel);
    }
    if (n_iter > 0 && sizing)
    {
      *temp_storage_bytes = align_up(inner_bytes, 16) + tail;
    }
    *selector = sel;
    return CUDA_SUCCESS;
  }
  catch (const std::exception& e)
  {
    return report(who, e);
  }
}

} // namespace

extern "C" {

CCCL_C_API CUresult cccl_device_segmented_sort_compile(
  cccl_device_segmented_sort_build_result_t* build,
  cccl_sort_order_t sort_order,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_values_in,
  cccl_iterator_t begin_offset_in,
  cccl_iterator_t end_offset_in,
  int cc_major,
  int cc_minor,
  const char*,
  const char*,
  const char*,
  const char*,
  cccl_build_config*)
try
{
  if (build == nullptr || (sort_order != CCCL_ASCENDING && sort_order != CCCL_DESCENDING))
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  if (cc_major * 10 + cc_minor != 103)
  {
    printf("\nERROR in cccl_device_segmented_sort_compile(): kernels are built for sm_103a only (requested %d.%d)\n",
           cc_major,
           cc_minor);
    return CUDA_ERROR_NOT_SUPPORTED;
  }
  int kind = 0, kb = 0;
  if (!key_kind_of(d_keys_in.value_type.type, kind, kb) || d_keys_in.value_type.size != size_t(kb))
  {
    printf("\nERROR in cccl_device_segmented_sort_compile(): unsupported key type\n");
    return CUDA_ERROR_NOT_SUPPORTED;
  }
  const size_t user_value = keys_only(d_values_in) ? 0 : d_values_in.value_type.size;
  if (!keys_only(d_values_in) && (user_value == 0 || user_value > (size_t(1) << 20)))
  {
    printf("\nERROR in cccl_device_segmented_sort_compile(): value size %zu is not supported\n", user_value);
    return CUDA_ERROR_NOT_SUPPORTED;
  }
  // the kernels carry 4- and 8-byte values; other widths (custom types) travel as 32-bit
  // indices and are gathered afterwards
  const bool gathered = !(user_value == 0 || user_value == 4 || user_value == 8);
  const size_t vb     = gathered ? 4 : user_value;
  const image_ref img = segmented_image(kb);
  std::unique_ptr<char[]> payload(new char[img.size]);
  std::memcpy(payload.get(), img.data, img.size);

  auto* pol = static_cast<SegmentedPolicy*>(std::malloc(sizeof(SegmentedPolicy)));
  auto* tab = static_cast<SegKernelTable*>(std::calloc(1, sizeof(SegKernelTable)));
  if (pol == nullptr || tab == nullptr)
  {
    std::free(pol);
    std::free(tab);
    return CUDA_ERROR_OUT_OF_MEMORY;
  }
  *pol       = make_segmented_policy(kb, int(vb), kind);
  pol->magic = SEG_POLICY_MAGIC;
  pol->gather_value_bytes = gathered ? int32_t(user_value) : 0;
  tab->magic = SEG_TABLE_MAGIC;
  segmented_kernel_names(kb, int(vb), kind, sort_order == CCCL_DESCENDING, tab->names);
  if (begin_offset_in.type == CCCL_ITERATOR || end_offset_in.type == CCCL_ITERATOR)
  {
    try
    {
      tab->offsets = new OffsetIteratorKernel[2]{};
      if (begin_offset_in.type == CCCL_ITERATOR)
      {
        compile_offset_iterator(begin_offset_in, &end_offset_in, cc_major, cc_minor, tab->offsets[0]);
      }
      if (end_offset_in.type == CCCL_ITERATOR)
      {
        compile_offset_iterator(end_offset_in, &begin_offset_in, cc_major, cc_minor, tab->offsets[1]);
      }
    }
    catch (...)
    {
      free_offsets(tab);
      std::free(pol);
      std::free(tab);
      throw;
    }
  }

  cccl_device_segmented_sort_build_result_t r{};
  r.cc                            = cc_major * 10 + cc_minor;
  r.payload                       = payload.release();
  r.payload_size                  = img.size;
  r.payload_kind                  = CCCL_PAYLOAD_CUBIN;
  r.key_type                      = d_keys_in.value_type;
  r.offset_type                   = begin_offset_in.value_type;
  r.runtime_policy                = pol;
  r.runtime_policy_size           = sizeof(SegmentedPolicy);
  r.partition_runtime_policy      = tab;
  r.partition_runtime_policy_size = sizeof(SegKernelTable);
  r.order                         = sort_order;
  r.segmented_sort_fallback_kernel_lowered_name = dup_cstr(tab->names[SK_PASS]);
  r.segmented_sort_kernel_small_lowered_name    = dup_cstr(tab->names[SK_SMALL]);
  r.segmented_sort_kernel_large_lowered_name    = dup_cstr(tab->names[SK_BLOCK_L]);
  r.three_way_partition_init_kernel_lowered_name = dup_cstr(tab->names[SK_INIT]);
  r.three_way_partition_kernel_lowered_name      = dup_cstr(tab->names[SK_CLASSIFY]);
  *build                                         = r;
  return CUDA_SUCCESS;
}
catch (const std::exception& e)
{
  return report("cccl_device_segmented_sort_compile", e);
}

CCCL_C_API CUresult cccl_device_segmented_sort_load(cccl_device_segmented_sort_build_result_t* build)
try
{
  if (build == nullptr || build->payload == nullptr || build->payload_size == 0
      || build->payload_kind != CCCL_PAYLOAD_CUBIN || build->partition_runtime_policy == nullptr
      || build->partition_runtime_policy_size != sizeof(SegKernelTable)
      || static_cast<SegKernelTable*>(build->partition_runtime_policy)->magic != SEG_TABLE_MAGIC)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  const CUresult st = cuLibraryLoadData(&build->library, build->payload, nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (st != CUDA_SUCCESS)
  {
    return st;
  }
  auto* tab = static_cast<SegKernelTable*>(build->partition_runtime_policy);
  try
  {
    for (int i = 0; i < SK_COUNT; ++i)
    {
      check(cuLibraryGetKernel(&tab->handles[i], build->library, tab->names[i]), tab->names[i]);
    }
    if (tab->offsets != nullptr)
    {
      load_offset_iterator(tab->offsets[0]);
      load_offset_iterator(tab->offsets[1]);
    }
  }
  catch (...)
  {
    if (tab->offsets != nullptr)
    {
      for (int e = 0; e < 2; ++e)
      {
        if (tab->offsets[e].library != nullptr)
        {
          cuLibraryUnload(tab->offsets[e].library);
          tab->offsets[e].library = nullptr;
          tab->offsets[e].kernel  = nullptr;
        }
      }
    }
    cuLibraryUnload(build->library);
    build->library = nullptr;
    throw;
  }
  build->segmented_sort_fallback_kernel  = tab->handles[SK_PASS];
  build->segmented_sort_kernel_small     = tab->handles[SK_SMALL];
  build->segmented_sort_kernel_large     = tab->handles[SK_BLOCK_L];
  build->three_way_partition_init_kernel = tab->handles[SK_INIT];
  build->three_way_partition_kernel      = tab->handles[SK_CLASSIFY];
  return CUDA_SUCCESS;
}
catch (const std::exception& e)
{
  return report("cccl_device_segmented_sort_load", e);
}

CCCL_C_API CUresult cccl_device_segmented_sort_build_ex(
  cccl_device_segmented_sort_build_result_t* build,
  cccl_sort_order_t sort_order,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_values_in,
  cccl_iterator_t begin_offset_in,
  cccl_iterator_t end_offset_in,
  int cc_major,
  int cc_minor,
  const char* cub_path,
  const char* thrust_path,
  const char* libcudacxx_path,
  const char* ctk_path,
  cccl_build_config* config)
{
  CUresult r = cccl_device_segmented_sort_compile(
    build,
    sort_order,
    d_keys_in,
    d_values_in,
    begin_offset_in,
    end_offset_in,
    cc_major,
    cc_minor,
    cub_path,
    thrust_path,
    libcudacxx_path,
    ctk_path,
    config);
  if (r != CUDA_SUCCESS)
  {
    return r;
  }
  r = cccl_device_segmented_sort_load(build);
  if (r != CUDA_SUCCESS)
  {
    cccl_device_segmented_sort_cleanup(build);
  }
  return r;
}

CCCL_C_API CUresult cccl_device_segmented_sort_build(
  cccl_device_segmented_sort_build_result_t* build,
  cccl_sort_order_t sort_order,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_values_in,
  cccl_iterator_t begin_offset_in,
  cccl_iterator_t end_offset_in,
  int cc_major,
  int cc_minor,
  const char* cub_path,
  const char* thrust_path,
  const char* libcudacxx_path,
  const char* ctk_path)
{
  return cccl_device_segmented_sort_build_ex(
    build,
    sort_order,
    d_keys_in,
    d_values_in,
    begin_offset_in,
    end_offset_in,
    cc_major,
    cc_minor,
    cub_path,
    thrust_path,
    libcudacxx_path,
    ctk_path,
    nullptr);
}

CCCL_C_API CUresult cccl_device_segmented_sort(
  cccl_device_segmented_sort_build_result_t build,
  void* d_temp_storage,
  size_t* temp_storage_bytes,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_keys_out,
  cccl_iterator_t d_values_in,
  cccl_iterator_t d_values_out,
  uint64_t num_items,
  uint64_t num_segments,
  cccl_iterator_t start_offset_in,
  cccl_iterator_t end_offset_in,
  bool is_overwrite_okay,
  int* selector,
  CUstream stream)
{
  return segmented_run("cccl_device_segmented_sort", build, d_temp_storage, temp_storage_bytes, d_keys_in, d_keys_out,
                       d_values_in, d_values_out, num_items, num_segments, start_offset_in, end_offset_in, false, 0, 0,
                       is_overwrite_okay, selector, stream);
}

CCCL_GB300_API CUresult cccl_gb300_segmented_radix_sort(
  cccl_device_segmented_sort_build_result_t build,
  void* d_temp_storage,
  size_t* temp_storage_bytes,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_keys_out,
  cccl_iterator_t d_values_in,
  cccl_iterator_t d_values_out,
  uint64_t num_items,
  uint64_t num_segments,
  cccl_iterator_t start_offset_in,
  cccl_iterator_t end_offset_in,
  int begin_bit,
  int end_bit,
  bool is_overwrite_okay,
  int* selector,
  CUstream stream)
{
  return segmented_run("cccl_gb300_segmented_radix_sort", build, d_temp_storage, temp_storage_bytes, d_keys_in,
                       d_keys_out, d_values_in, d_values_out, num_items, num_segments, start_offset_in, end_offset_in,
                       true, begin_bit, end_bit, is_overwrite_okay, selector, stream);
}

CCCL_C_API CUresult cccl_device_segmented_sort_link_ltoir(
  cccl_device_segmented_sort_build_result_t* build, const void**, const size_t*, size_t)
{
  // The payload is a finished cubin: there is no LTO-IR stage to link into.
  if (build == nullptr || build->payload == nullptr || build->payload_size == 0
      || build->payload_kind != CCCL_PAYLOAD_LTOIR)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  return CUDA_ERROR_NOT_SUPPORTED;
}

CCCL_C_API CUresult cccl_device_segmented_sort_serialize(
  const cccl_device_segmented_sort_build_result_t* b, void** out_buf, size_t* out_size)
try
{
  if (b == nullptr || out_buf == nullptr || out_size == nullptr)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  if (b->payload == nullptr || b->payload_size == 0 || b->runtime_policy == nullptr
      || b->partition_runtime_policy == nullptr)
  {
    *out_buf  = nullptr;
    *out_size = 0;
    return CUDA_ERROR_INVALID_VALUE;
  }
  SegKernelTable tab = *static_cast<const SegKernelTable*>(b->partition_runtime_policy);
  for (auto& h : tab.handles)
  {
    h = nullptr; // handles belong to a loaded library; never serialized
  }
  const OffsetIteratorKernel* offs = tab.offsets;
  tab.offsets                      = nullptr;
  blob_writer w;
  write_header(w, ALGO_SEGMENTED, b->payload_kind, b->cc);
  w.type_info(b->key_type);
  w.type_info(b->offset_type);
  w.pod<uint32_t>(uint32_t(b->order));
  w.blob(b->payload, b->payload_size);
  w.blob(b->runtime_policy, b->runtime_policy_size);
  w.blob(&tab, sizeof(tab));
  w.cstr(b->segmented_sort_fallback_kernel_lowered_name);
  w.cstr(b->segmented_sort_kernel_small_lowered_name);
  w.cstr(b->segmented_sort_kernel_large_lowered_name);
  w.cstr(b->three_way_partition_init_kernel_lowered_name);
  w.cstr(b->three_way_partition_kernel_lowered_name);
  // offset iterators: their evaluation images and state layouts
  w.pod<uint32_t>(offs != nullptr ? 2u : 0u);
  for (int e = 0; offs != nullptr && e < 2; ++e)
  {
    w.blob(offs[e].cubin, offs[e].cubin_size);
    w.pod<uint64_t>(offs[e].state_size);
    w.pod<uint64_t>(offs[e].state_alignment);
    w.pod<uint64_t>(offs[e].value_size);
  }
  w.release(out_buf, out_size);
  return CUDA_SUCCESS;
}
catch (const std::exception& e)
{
  return report("cccl_device_segmented_sort_serialize", e);
}

CCCL_C_API CUresult
cccl_device_segmented_sort_deserialize(cccl_device_segmented_sort_build_result_t* build, const void* buf, size_t size)
try
{
  if (build == nullptr || buf == nullptr || size == 0)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  blob_reader rd{static_cast<const unsigned char*>(buf), size};
  const blob_header h = read_header(rd, ALGO_SEGMENTED);
  cccl_device_segmented_sort_build_result_t r{};
  r.cc           = h.cc;
  r.payload_kind = cccl_payload_kind_t(h.payload_kind);
  r.key_type     = rd.type_info();
  r.offset_type  = rd.type_info();
  r.order        = cccl_sort_order_t(rd.pod<uint32_t>());
  if (r.order != CCCL_ASCENDING && r.order != CCCL_DESCENDING)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "serialization blob: invalid sort order");
  }
  std::unique_ptr<char[]> payload(static_cast<char*>(rd.blob_new(&r.payload_size)));
  size_t pol_size = 0, tab_size = 0;
  std::unique_ptr<char[]> pol_bytes(static_cast<char*>(rd.blob_new(&pol_size)));
  std::unique_ptr<char[]> tab_bytes(static_cast<char*>(rd.blob_new(&tab_size)));
  if (r.payload_size == 0 || pol_size != sizeof(SegmentedPolicy) || tab_size != sizeof(SegKernelTable))
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "serialization blob: size mismatch");
  }
  auto* pol = static_cast<SegmentedPolicy*>(std::malloc(sizeof(SegmentedPolicy)));
  auto* tab = static_cast<SegKernelTable*>(std::malloc(sizeof(SegKernelTable)));
  if (pol == nullptr || tab == nullptr)
  {
    std::free(pol);
    std::free(tab);
    return CUDA_ERROR_OUT_OF_MEMORY;
  }
  std::memcpy(pol, pol_bytes.get(), sizeof(SegmentedPolicy));
  std::memcpy(tab, tab_bytes.get(), sizeof(SegKernelTable));
  if (pol->magic != SEG_POLICY_MAGIC || tab->magic != SEG_TABLE_MAGIC)
  {
    std::free(pol);
    std::free(tab);
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "serialization blob: bad policy");
  }
  for (auto& name : tab->names)
  {
    name[sizeof(name) - 1] = '\0';
  }
  for (auto& hd : tab->handles)
  {
    hd = nullptr;
  }
  tab->offsets = nullptr;
  std::unique_ptr<char[]> names[5];
  try
  {
    for (auto& n : names)
    {
      n.reset(rd.cstr_new());
    }
    const uint32_t n_offsets = rd.pod<uint32_t>();
    if (n_offsets != 0 && n_offsets != 2)
    {
      throw cuda_error(CUDA_ERROR_INVALID_VALUE, "serialization blob: bad offset iterator count");
    }
    if (n_offsets == 2)
    {
      tab->offsets = new OffsetIteratorKernel[2]{};
      for (int e = 0; e < 2; ++e)
      {
        size_t bytes = 0;
        std::unique_ptr<char[]> img(static_cast<char*>(rd.blob_new(&bytes)));
        OffsetIteratorKernel& k = tab->offsets[e];
        k.state_size            = rd.pod<uint64_t>();
        k.state_alignment       = rd.pod<uint64_t>();
        k.value_size            = rd.pod<uint64_t>();
        if (bytes > 0)
        {
          if (k.state_size == 0 || k.state_size > MAX_OFFSET_STATE_BYTES || (k.value_size != 4 && k.value_size != 8))
          {
            throw cuda_error(CUDA_ERROR_INVALID_VALUE, "serialization blob: bad offset iterator");
          }
          k.cubin = std::malloc(bytes);
          if (k.cubin == nullptr)
          {
            throw cuda_error(CUDA_ERROR_OUT_OF_MEMORY, "offset iterator image");
          }
          std::memcpy(k.cubin, img.get(), bytes);
          k.cubin_size = bytes;
        }
      }
    }
  }
  catch (...)
  {
    free_offsets(tab);
    std::free(pol);
    std::free(tab);
    throw;
  }
  r.payload                                      = payload.release();
  r.runtime_policy                               = pol;
  r.runtime_policy_size                          = sizeof(SegmentedPolicy);
  r.partition_runtime_policy                     = tab;
  r.partition_runtime_policy_size                = sizeof(SegKernelTable);
  r.segmented_sort_fallback_kernel_lowered_name  = names[0].release();
  r.segmented_sort_kernel_small_lowered_name     = names[1].release();
  r.segmented_sort_kernel_large_lowered_name     = names[2].release();
  r.three_way_partition_init_kernel_lowered_name = names[3].release();
  r.three_way_partition_kernel_lowered_name      = names[4].release();
  *build                                         = r;
  return CUDA_SUCCESS;
}
catch (const std::exception& e)
{
  return report("cccl_device_segmented_sort_deserialize", e);
}

CCCL_C_API CUresult cccl_device_segmented_sort_cleanup(cccl_device_segmented_sort_build_result_t* b)
try
{
  if (b == nullptr)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  free_result(b);
  if (b->library != nullptr)
  {
    check(cuLibraryUnload(b->library), "cuLibraryUnload");
    b->library = nullptr;
  }
  return CUDA_SUCCESS;
}
catch (const std::exception& e)
{
  return report("cccl_device_segmented_sort_cleanup", e);
}

} // extern "C"
