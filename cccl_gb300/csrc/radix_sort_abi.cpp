// C ABI of the plain radix sort: cccl_device_radix_sort_{build,build_ex,compile,load,
// link_ltoir,serialize,deserialize,cleanup} and the run entry cccl_device_radix_sort.
//
// Reference interface: c/parallel/include/cccl/c/radix_sort.h:27-143, implemented in
// c/parallel/src/radix_sort.cu (compile :221-472, load :474-539, run :582-698,
// cleanup :730-770, serialize/deserialize :816-947). The host dispatch follows CUB's
// onesweep driver (cub/cub/device/dispatch/dispatch_radix_sort.cuh:1698-1948) and its
// special cases (:1950-2003): empty input, begin_bit == end_bit, single tile.
#include <cccl/c/radix_sort.h>
#include <cccl/c/serialization.h>
#include <cccl_gb300/merge_runs.h>

#include <algorithm>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "abi_common.h"
#include "radix_plan.h"
#include "value_gather.h"
#include "sort_policy.h"

using namespace gb300;

namespace
{

constexpr uint32_t POLICY_MAGIC = 0x52425047u; // "GPBR"

bool is_keys_only(const cccl_iterator_t& values)
{
  return values.type == CCCL_POINTER && values.state == nullptr;
}

bool has_decomposer(const cccl_op_t& op)
{
  return op.name != nullptr && op.name[0] != '\0';
}

void free_names(cccl_device_radix_sort_build_result_t* b)
{
  for (char** p :
       {&b->single_tile_kernel_lowered_name,
        &b->upsweep_kernel_lowered_name,
        &b->alt_upsweep_kernel_lowered_name,
        &b->scan_bins_kernel_lowered_name,
        &b->downsweep_kernel_lowered_name,
        &b->alt_downsweep_kernel_lowered_name,
        &b->histogram_kernel_lowered_name,
        &b->exclusive_sum_kernel_lowered_name,
        &b->init_bins_and_counters_kernel_lowered_name,
        &b->init_lookback_kernel_lowered_name,
        &b->onesweep_kernel_lowered_name})
  {
    delete[] *p;
    *p = nullptr;
  }
}

const RadixPolicy& policy_of(const cccl_device_radix_sort_build_result_t& b)
{
  if (b.runtime_policy == nullptr || b.runtime_policy_size != sizeof(RadixPolicy)
      || static_cast<const RadixPolicy*>(b.runtime_policy)->magic != POLICY_MAGIC)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "build result has no valid runtime policy");
  }
  return *static_cast<const RadixPolicy*>(b.runtime_policy);
}

} // namespace

extern "C" {

CCCL_C_API void cccl_serialization_buffer_free(void* buf)
{
  std::free(buf);
}

CCCL_C_API CUresult cccl_device_radix_sort_compile(
  cccl_device_radix_sort_build_result_t* build,
  cccl_sort_order_t sort_order,
  cccl_iterator_t input_keys_it,
  cccl_iterator_t input_values_it,
  cccl_op_t decomposer,
  const char* /*decomposer_return_type*/,
  int cc_major,
  int cc_minor,
  const char* /*cub_path*/,
  const char* /*thrust_path*/,
  const char* /*libcudacxx_path*/,
  const char* /*ctk_path*/,
  cccl_build_config* /*config*/)
try
{
  if (build == nullptr)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  if (sort_order != CCCL_ASCENDING && sort_order != CCCL_DESCENDING)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  if (has_decomposer(decomposer))
  {
    printf("\nERROR in cccl_device_radix_sort_compile(): custom key decomposers are not supported\n");
    return CUDA_ERROR_NOT_SUPPORTED;
  }
  if (cc_major * 10 + cc_minor != 103)
  {
    printf("\nERROR in cccl_device_radix_sort_compile(): kernels are built for sm_103a only (requested %d.%d)\n",
           cc_major,
           cc_minor);
    return CUDA_ERROR_NOT_SUPPORTED;
  }
  int kind = 0, key_bytes = 0;
  if (!key_kind_of(input_keys_it.value_type.type, kind, key_bytes)
      || input_keys_it.value_type.size != size_t(key_bytes))
  {
    printf("\nERROR in cccl_device_radix_sort_compile(): unsupported key type\n");
    return CUDA_ERROR_NOT_SUPPORTED;
  }
  const bool keys_only    = is_keys_only(input_values_it);
  const size_t user_value = keys_only ? 0 : input_values_it.value_type.size;
  if (!keys_only && (user_value == 0 || user_value > (size_t(1) << 20)))
  {
    printf("\nERROR in cccl_device_radix_sort_compile(): value size %zu is not supported\n", user_value);
    return CUDA_ERROR_NOT_SUPPORTED;
  }
  // widths the kernels do not carry travel as 32-bit indices and are gathered afterwards
  const bool gathered     = !supported_value_bytes(user_value);
  const size_t value_size = gathered ? 4 : user_value;

  const image_ref img = radix_image(key_bytes);
  std::unique_ptr<char[]> payload(new char[img.size]);
  std::memcpy(payload.get(), img.data, img.size);

  auto* pol        = static_cast<RadixPolicy*>(std::malloc(sizeof(RadixPolicy)));
  if (pol == nullptr)
  {
    return CUDA_ERROR_OUT_OF_MEMORY;
  }
  *pol = make_radix_policy(key_bytes, int(value_size), kind);
  pol->magic              = POLICY_MAGIC;
  pol->gather_value_bytes = gathered ? int32_t(user_value) : 0;

  const RadixKernelNames names = radix_kernel_names(key_bytes, int(value_size), kind, sort_order == CCCL_DESCENDING);
  const std::string& one   = names.onesweep;
  const std::string& dyn   = names.onesweep_dyn;
  const std::string& first = names.onesweep_first;
  const std::string& st    = names.single_tile;
  const std::string& his   = names.histogram;
  const std::string& ini   = names.init;

  cccl_device_radix_sort_build_result_t r{};
  r.cc                   = cc_major * 10 + cc_minor;
  r.payload              = payload.release();
  r.payload_size         = img.size;
  r.payload_kind         = CCCL_PAYLOAD_CUBIN;
  r.key_type             = input_keys_it.value_type;
  r.value_type           = input_values_it.value_type;
  r.order                = sort_order;
  r.runtime_policy       = pol;
  r.runtime_policy_size  = sizeof(RadixPolicy);
  r.single_tile_kernel_lowered_name            = dup_cstr(st);
  r.upsweep_kernel_lowered_name                = dup_cstr(his);
  r.alt_upsweep_kernel_lowered_name            = dup_cstr(his);
  r.scan_bins_kernel_lowered_name              = dup_cstr(his);
  r.downsweep_kernel_lowered_name              = dup_cstr(dyn);
  r.alt_downsweep_kernel_lowered_name          = dup_cstr(first);
  r.histogram_kernel_lowered_name              = dup_cstr(his);
  r.exclusive_sum_kernel_lowered_name          = dup_cstr(his);
  r.init_bins_and_counters_kernel_lowered_name = dup_cstr(ini);
  r.init_lookback_kernel_lowered_name          = dup_cstr(ini);
  r.onesweep_kernel_lowered_name               = dup_cstr(one);
  *build                                       = r;
  return CUDA_SUCCESS;
}
catch (const std::exception& e)
{
  return report("cccl_device_radix_sort_compile", e);
}

CCCL_C_API CUresult cccl_device_radix_sort_load(cccl_device_radix_sort_build_result_t* build)
try
{
  auto invalid = [](const char* n) {
    return n == nullptr || n[0] == '\0';
  };
  if (build == nullptr || build->payload == nullptr || build->payload_size == 0
      || build->payload_kind != CCCL_PAYLOAD_CUBIN || invalid(build->single_tile_kernel_lowered_name)
      || invalid(build->upsweep_kernel_lowered_name) || invalid(build->alt_upsweep_kernel_lowered_name)
      || invalid(build->scan_bins_kernel_lowered_name) || invalid(build->downsweep_kernel_lowered_name)
      || invalid(build->alt_downsweep_kernel_lowered_name) || invalid(build->histogram_kernel_lowered_name)
      || invalid(build->exclusive_sum_kernel_lowered_name)
      || invalid(build->init_bins_and_counters_kernel_lowered_name)
      || invalid(build->init_lookback_kernel_lowered_name) || invalid(build->onesweep_kernel_lowered_name))
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  const CUresult st = cuLibraryLoadData(&build->library, build->payload, nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (st != CUDA_SUCCESS)
  {
    return st;
  }
  try
  {
    auto get = [&](CUkernel* k, const char* name) {
      check(cuLibraryGetKernel(k, build->library, name), name);
    };
    get(&build->single_tile_kernel, build->single_tile_kernel_lowered_name);
    get(&build->upsweep_kernel, build->upsweep_kernel_lowered_name);
    get(&build->alt_upsweep_kernel, build->alt_upsweep_kernel_lowered_name);
    get(&build->scan_bins_kernel, build->scan_bins_kernel_lowered_name);
    get(&build->downsweep_kernel, build->downsweep_kernel_lowered_name);
    get(&build->alt_downsweep_kernel, build->alt_downsweep_kernel_lowered_name);
    get(&build->histogram_kernel, build->histogram_kernel_lowered_name);
    get(&build->exclusive_sum_kernel, build->exclusive_sum_kernel_lowered_name);
    get(&build->init_bins_and_counters_kernel, build->init_bins_and_counters_kernel_lowered_name);
    get(&build->init_lookback_kernel, build->init_lookback_kernel_lowered_name);
    get(&build->onesweep_kernel, build->onesweep_kernel_lowered_name);
  }
  catch (...)
  {
    cuLibraryUnload(build->library);
    build->library = nullptr;
    throw;
  }
  return CUDA_SUCCESS;
}
catch (const std::exception& e)
{
  return report("cccl_device_radix_sort_load", e);
}

CCCL_C_API CUresult cccl_device_radix_sort_build_ex(
  cccl_device_radix_sort_build_result_t* build,
  cccl_sort_order_t sort_order,
  cccl_iterator_t input_keys_it,
  cccl_iterator_t input_values_it,
  cccl_op_t decomposer,
  const char* decomposer_return_type,
  int cc_major,
  int cc_minor,
  const char* cub_path,
  const char* thrust_path,
  const char* libcudacxx_path,
  const char* ctk_path,
  cccl_build_config* config)
{
  CUresult r = cccl_device_radix_sort_compile(
    build,
    sort_order,
    input_keys_it,
    input_values_it,
    decomposer,
    decomposer_return_type,
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
  r = cccl_device_radix_sort_load(build);
  if (r != CUDA_SUCCESS)
  {
    cccl_device_radix_sort_cleanup(build);
  }
  return r;
}

CCCL_C_API CUresult cccl_device_radix_sort_build(
  cccl_device_radix_sort_build_result_t* build,
  cccl_sort_order_t sort_order,
  cccl_iterator_t input_keys_it,
  cccl_iterator_t input_values_it,
  cccl_op_t decomposer,
  const char* decomposer_return_type,
  int cc_major,
  int cc_minor,
  const char* cub_path,
  const char* thrust_path,
  const char* libcudacxx_path,
  const char* ctk_path)
{
  return cccl_device_radix_sort_build_ex(
    build,
    sort_order,
    input_keys_it,
    input_values_it,
    decomposer,
    decomposer_return_type,
    cc_major,
    cc_minor,
    cub_path,
    thrust_path,
    libcudacxx_path,
    ctk_path,
    nullptr);
}

CCCL_C_API CUresult cccl_device_radix_sort(
  cccl_device_radix_sort_build_result_t build,
  void* d_temp_storage,
  size_t* temp_storage_bytes,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_keys_out,
  cccl_iterator_t d_values_in,
  cccl_iterator_t d_values_out,
  cccl_op_t decomposer,
  uint64_t num_items,
  int begin_bit,
  int end_bit,
  bool is_overwrite_okay,
  int* selector,
  CUstream stream)
{
  if (d_keys_in.type != CCCL_POINTER || d_keys_out.type != CCCL_POINTER || d_values_in.type != CCCL_POINTER
      || d_values_out.type != CCCL_POINTER)
  {
    fflush(stderr);
    printf("\nERROR in cccl_device_radix_sort(): radix sort input must be a pointer\n");
    fflush(stdout);
    return CUDA_ERROR_UNKNOWN;
  }
  if (temp_storage_bytes == nullptr || selector == nullptr)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  if (has_decomposer(decomposer))
  {
    return CUDA_ERROR_NOT_SUPPORTED;
  }
  try
  {
    context_guard ctx;
    const RadixPolicy& pol = policy_of(build);
    if (build.library == nullptr || build.onesweep_kernel == nullptr)
    {
      return CUDA_ERROR_NOT_INITIALIZED;
    }
    RadixKernels ks{build.init_bins_and_counters_kernel,
                    build.histogram_kernel,
                    build.onesweep_kernel,
                    build.alt_downsweep_kernel,
                    build.downsweep_kernel,
                    build.single_tile_kernel};
    RadixCall call{};
    call.keys[0]          = d_keys_in.state;
    call.keys[1]          = d_keys_out.state;
    call.values[0]        = d_values_in.state;
    call.values[1]        = d_values_out.state;
    call.num_items        = num_items;
    call.begin_bit        = begin_bit;
    call.end_bit          = end_bit;
    call.overwrite        = is_overwrite_okay;
    call.descending       = build.order == CCCL_DESCENDING;
    call.d_temp_storage   = d_temp_storage;
    call.temp_storage_bytes = temp_storage_bytes;
    call.stream           = stream;
    int sel               = 0;
    if (pol.gather_value_bytes > 0 && call.values[0] != nullptr)
    {
      sort_with_gathered_values(
        build.library, uint32_t(pol.gather_value_bytes), call.values, num_items, is_overwrite_okay, false,
        d_temp_storage, temp_storage_bytes, stream,
        [&](void* const idx[2], void* temp, size_t* bytes, int* s) {
          RadixCall inner      = call;
          inner.values[0]      = idx[0];
          inner.values[1]      = idx[1];
          inner.d_temp_storage = temp;
          inner.temp_storage_bytes = bytes;
          radix_sort_dispatch(pol, ks, inner, s);
        },
        &sel);
    }
    else
    {
      radix_sort_dispatch(pol, ks, call, &sel);
    }
    *selector = sel;
    return CUDA_SUCCESS;
  }
  catch (const std::exception& e)
  {
    return report("cccl_device_radix_sort", e);
  }
}

CCCL_C_API CUresult cccl_device_radix_sort_link_ltoir(
  cccl_device_radix_sort_build_result_t* build, const void** input_blobs, const size_t* input_sizes, size_t num_inputs)
{
  // The payload is a finished cubin: there is no LTO-IR stage to link into.
  (void) input_blobs;
  (void) input_sizes;
  (void) num_inputs;
  if (build == nullptr || build->payload == nullptr || build->payload_size == 0
      || build->payload_kind != CCCL_PAYLOAD_LTOIR)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  return CUDA_ERROR_NOT_SUPPORTED;
}

CCCL_C_API CUresult
cccl_device_radix_sort_serialize(const cccl_device_radix_sort_build_result_t* b, void** out_buf, size_t* out_size)
try
{
  if (b == nullptr || out_buf == nullptr || out_size == nullptr)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  if (b->payload == nullptr || b->payload_size == 0 || b->runtime_policy == nullptr || b->runtime_policy_size == 0)
  {
    *out_buf  = nullptr;
    *out_size = 0;
    return CUDA_ERROR_INVALID_VALUE;
  }
  blob_writer w;
  write_header(w, 7u /* CCCL_SERIALIZATION_ALGO_RADIX_SORT */, b->payload_kind, b->cc);
  w.type_info(b->key_type);
  w.type_info(b->value_type);
  w.pod<uint32_t>(uint32_t(b->order));
  w.blob(b->payload, b->payload_size);
  w.blob(b->runtime_policy, b->runtime_policy_size);
  w.cstr(b->single_tile_kernel_lowered_name);
  w.cstr(b->upsweep_kernel_lowered_name);
  w.cstr(b->alt_upsweep_kernel_lowered_name);
  w.cstr(b->scan_bins_kernel_lowered_name);
  w.cstr(b->downsweep_kernel_lowered_name);
  w.cstr(b->alt_downsweep_kernel_lowered_name);
  w.cstr(b->histogram_kernel_lowered_name);
  w.cstr(b->exclusive_sum_kernel_lowered_name);
  w.cstr(b->init_bins_and_counters_kernel_lowered_name);
  w.cstr(b->init_lookback_kernel_lowered_name);
  w.cstr(b->onesweep_kernel_lowered_name);
  w.release(out_buf, out_size);
  return CUDA_SUCCESS;
}
catch (const std::exception& e)
{
  return report("cccl_device_radix_sort_serialize", e);
}

CCCL_C_API CUresult
cccl_device_radix_sort_deserialize(cccl_device_radix_sort_build_result_t* build, const void* buf, size_t size)
try
{
  if (build == nullptr || buf == nullptr || size == 0)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  blob_reader rd{static_cast<const unsigned char*>(buf), size};
  const blob_header h = read_header(rd, 7u);
  cccl_device_radix_sort_build_result_t r{};
  r.cc         = h.cc;
  r.payload_kind = cccl_payload_kind_t(h.payload_kind);
  r.key_type   = rd.type_info();
  r.value_type = rd.type_info();
  r.order      = cccl_sort_order_t(rd.pod<uint32_t>());
  if (r.order != CCCL_ASCENDING && r.order != CCCL_DESCENDING)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "serialization blob: invalid sort order");
  }
  std::unique_ptr<char[]> payload(static_cast<char*>(rd.blob_new(&r.payload_size)));
  if (r.payload_size == 0)
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "serialization blob: empty payload");
  }
  size_t pol_size = 0;
  std::unique_ptr<char[]> pol_bytes(static_cast<char*>(rd.blob_new(&pol_size)));
  if (pol_size != sizeof(RadixPolicy))
  {
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "serialization blob: policy size mismatch");
  }
  auto* pol = static_cast<RadixPolicy*>(std::malloc(sizeof(RadixPolicy)));
  if (pol == nullptr)
  {
    return CUDA_ERROR_OUT_OF_MEMORY;
  }
  std::memcpy(pol, pol_bytes.get(), sizeof(RadixPolicy));
  if (pol->magic != POLICY_MAGIC)
  {
    std::free(pol);
    throw cuda_error(CUDA_ERROR_INVALID_VALUE, "serialization blob: bad policy");
  }
  std::unique_ptr<char[]> names[11];
  for (auto& n : names)
  {
    n.reset(rd.cstr_new());
  }
  r.payload                                    = payload.release();
  r.runtime_policy                             = pol;
  r.runtime_policy_size                        = sizeof(RadixPolicy);
  r.single_tile_kernel_lowered_name            = names[0].release();
  r.upsweep_kernel_lowered_name                = names[1].release();
  r.alt_upsweep_kernel_lowered_name            = names[2].release();
  r.scan_bins_kernel_lowered_name              = names[3].release();
  r.downsweep_kernel_lowered_name              = names[4].release();
  r.alt_downsweep_kernel_lowered_name          = names[5].release();
  r.histogram_kernel_lowered_name              = names[6].release();
  r.exclusive_sum_kernel_lowered_name          = names[7].release();
  r.init_bins_and_counters_kernel_lowered_name = names[8].release();
  r.init_lookback_kernel_lowered_name          = names[9].release();
  r.onesweep_kernel_lowered_name               = names[10].release();
  *build                                       = r;
  return CUDA_SUCCESS;
}
catch (const std::exception& e)
{
  return report("cccl_device_radix_sort_deserialize", e);
}

CCCL_C_API CUresult cccl_device_radix_sort_cleanup(cccl_device_radix_sort_build_result_t* b)
try
{
  if (b == nullptr)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  delete[] static_cast<char*>(b->payload);
  b->payload = nullptr;
  std::free(b->runtime_policy);
  b->runtime_policy = nullptr;
  free_names(b);
  if (b->library != nullptr)
  {
    check(cuLibraryUnload(b->library), "cuLibraryUnload");
    b->library = nullptr;
  }
  return CUDA_SUCCESS;
}
catch (const std::exception& e)
{
  return report("cccl_device_radix_sort_cleanup", e);
}

// Stable merge of sorted runs (include/cccl_gb300/merge_runs.h): rounds of pairwise merges,
// ping-ponging between the output and one buffer of temporary storage so that the last
// round writes the output.
CCCL_C_API CUresult cccl_gb300_merge_sorted_runs(
  cccl_device_radix_sort_build_result_t build,
  void* d_temp_storage,
  size_t* temp_storage_bytes,
  cccl_iterator_t d_keys_in,
  cccl_iterator_t d_keys_out,
  cccl_iterator_t d_values_in,
  cccl_iterator_t d_values_out,
  const uint64_t* run_offsets,
  int num_runs,
  CUstream stream)
try
{
  if (d_keys_in.type != CCCL_POINTER || d_keys_out.type != CCCL_POINTER || d_values_in.type != CCCL_POINTER
      || d_values_out.type != CCCL_POINTER)
  {
    return CUDA_ERROR_UNKNOWN;
  }
  if (temp_storage_bytes == nullptr || run_offsets == nullptr || num_runs < 1 || run_offsets[0] != 0)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  for (int r = 0; r < num_runs; ++r)
  {
    if (run_offsets[r + 1] < run_offsets[r])
    {
      return CUDA_ERROR_INVALID_VALUE;
    }
  }
  context_guard ctx;
  const RadixPolicy& pol = policy_of(build);
  if (build.library == nullptr)
  {
    return CUDA_ERROR_NOT_INITIALIZED;
  }
  const bool has_values = d_values_in.state != nullptr;
  if (has_values && (pol.gather_value_bytes > 0 || d_values_out.state == nullptr))
  {
    return pol.gather_value_bytes > 0 ? CUDA_ERROR_NOT_SUPPORTED : CUDA_ERROR_INVALID_VALUE;
  }
  const int kb         = pol.key_bytes;
  const int vb         = has_values ? pol.value_bytes : 0;
  const uint64_t n     = run_offsets[num_runs];
  const size_t kbytes  = align_up(size_t(n) * kb, 256);
  const size_t vbytes  = align_up(size_t(n) * vb, 256);
  const uint64_t max_tiles = (n + MERGE_TILE - 1) / MERGE_TILE + 1; // of any pair in any round
  const size_t need    = std::max<size_t>(1, kbytes + vbytes + align_up(size_t(max_tiles + 1) * 8, 256));
  if (d_temp_storage == nullptr)
  {
    *temp_storage_bytes = need;
    return CUDA_SUCCESS;
  }
  if (*temp_storage_bytes < need)
  {
    return CUDA_ERROR_INVALID_VALUE;
  }
  if (n == 0)
  {
    return CUDA_SUCCESS;
  }
  auto overlap = [](const void* a, const void* b, size_t bytes) {
    const auto x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
    return x < y + bytes && y < x + bytes;
  };
  if (overlap(d_keys_in.state, d_keys_out.state, size_t(n) * kb)
      || (has_values && overlap(d_values_in.state, d_values_out.state, size_t(n) * vb)))
  {
    return CUDA_ERROR_INVALID_VALUE; // the rounds read the inputs while writing the output
  }
  auto* tmp       = static_cast<unsigned char*>(d_temp_storage);
  auto* out_keys  = static_cast<unsigned char*>(d_keys_out.state);
  auto* out_vals  = static_cast<unsigned char*>(d_values_out.state);
  const auto* src_keys = static_cast<const unsigned char*>(d_keys_in.state);
  const auto* src_vals = static_cast<const unsigned char*>(d_values_in.state);
  int rounds = 0;
  while ((1 << rounds) < num_runs)
  {
    ++rounds;
  }
  if (rounds == 0)
  {
    check(cuMemcpyAsync(CUdeviceptr(out_keys), CUdeviceptr(src_keys), size_t(n) * kb, stream), "cuMemcpyAsync(keys)");
    if (has_values)
    {
      check(cuMemcpyAsync(CUdeviceptr(out_vals), CUdeviceptr(src_vals), size_t(n) * vb, stream), "cuMemcpyAsync(values)");
    }
    return CUDA_SUCCESS;
  }
  const std::string name = "gb300_merge_k" + std::to_string(kb) + "_v" + std::to_string(vb) + "_"
                         + (pol.key_kind == KIND_FLOAT ? "f" : "i");
  const std::string split_name = "gb300_merge_split_k" + std::to_string(kb) + "_" + (pol.key_kind == KIND_FLOAT ? "f" : "i");
  CUkernel merge = nullptr;
  CUkernel split = nullptr;
  check(cuLibraryGetKernel(&merge, build.library, name.c_str()), "cuLibraryGetKernel(merge)");
  check(cuLibraryGetKernel(&split, build.library, split_name.c_str()), "cuLibraryGetKernel(merge split)");
  auto* splits = reinterpret_cast<unsigned long long*>(tmp + kbytes + vbytes);
  const KeyCodec codec = make_codec(pol.key_kind, kb, build.order == CCCL_DESCENDING);
  const size_t smem    = merge_smem_bytes(kb, vb);
  std::vector<std::pair<uint64_t, uint64_t>> runs; // [begin, end)
  for (int r = 0; r < num_runs; ++r)
  {
    runs.emplace_back(run_offsets[r], run_offsets[r + 1]);
  }
  // an odd round count starts in the output, an even one in the temporary buffer
  bool to_out = (rounds & 1) != 0;
  for (int round = 0; round < rounds; ++round)
  {
    unsigned char* dk = to_out ? out_keys : tmp;
    unsigned char* dv = to_out ? out_vals : tmp + kbytes;
    std::vector<std::pair<uint64_t, uint64_t>> next;
    for (size_t j = 0; j < runs.size(); j += 2)
    {
      const uint64_t a = runs[j].first;
      if (j + 1 == runs.size())
      {
        // the odd run out moves unchanged
        const uint64_t len = runs[j].second - a;
        if (len > 0)
        {
          check(cuMemcpyAsync(CUdeviceptr(dk + a * kb), CUdeviceptr(src_keys + a * kb), size_t(len) * kb, stream),
                "cuMemcpyAsync(keys)");
          if (has_values)
          {
            check(cuMemcpyAsync(CUdeviceptr(dv + a * vb), CUdeviceptr(src_vals + a * vb), size_t(len) * vb, stream),
                  "cuMemcpyAsync(values)");
          }
        }
        next.push_back(runs[j]);
        continue;
      }
      const uint64_t b = runs[j + 1].first, e = runs[j + 1].second;
      MergeParams mp{};
      mp.a_keys     = src_keys + a * kb;
      mp.b_keys     = src_keys + b * kb;
      mp.a_values   = has_values ? src_vals + a * vb : nullptr;
      mp.b_values   = has_values ? src_vals + b * vb : nullptr;
      mp.out_keys   = dk + a * kb;
      mp.out_values = has_values ? dv + a * vb : nullptr;
      mp.na         = b - a;
      mp.nb         = e - b;
      mp.codec      = codec;
      mp.splits     = splits;
      const uint64_t tiles = (e - a + MERGE_TILE - 1) / MERGE_TILE;
      if (tiles > 0)
      {
        // the pairs of a round run one after another on the stream, so they share the splits
        launch("merge_split", split, unsigned((tiles + 1 + 255) / 256), 256u, 0, stream, mp);
        launch("merge", merge, unsigned(tiles), unsigned(MERGE_TPB), smem, stream, mp);
      }
      next.emplace_back(a, e);
    }
    runs     = std::move(next);
    src_keys = dk;
    src_vals = dv;
    to_out   = !to_out;
  }
  return CUDA_SUCCESS;
}
catch (const std::exception& e)
{
  return report("cccl_gb300_merge_sorted_runs", e);
}

} // extern "C"
