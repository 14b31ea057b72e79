// Runs the reference's own CPU sort reference (radix_sort_reference in
// cub/test/catch2_radix_sort_helper.cuh:270-310, built on get_striped_keys/get_permutation
// :174-268 and cub::Traits from cub/cub/util_type.cuh) on binary inputs, to produce the
// golden vectors that pin the oracle. Built by oracle/Makefile into oracle/_ref/; never
// part of the library.
//
// usage: ref_pin <key_type> <value_bytes> <n> <begin_bit> <end_bit> <descending> <in.bin> <out.bin>
//   in.bin  = n keys, then (value_bytes > 0) n values
//   out.bin = n sorted keys, then n values
#include <cuda_fp16.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <vector>

#include "catch2_radix_sort_helper.cuh"

template <int N>
struct value_blob
{
  unsigned char b[N];
};

template <class K, int VB>
static int run(uint64_t n, int begin_bit, int end_bit, bool desc, const std::vector<char>& in, std::ofstream& out)
{
  c2h::host_vector<K> hk(n);
  std::memcpy(thrust::raw_pointer_cast(hk.data()), in.data(), n * sizeof(K));
  c2h::device_vector<K> dk(hk);
  if constexpr (VB == 0)
  {
    c2h::host_vector<K> r = radix_sort_reference(dk, desc, begin_bit, end_bit);
    out.write(reinterpret_cast<const char*>(thrust::raw_pointer_cast(r.data())), n * sizeof(K));
  }
  else
  {
    using V = value_blob<VB>;
    c2h::host_vector<V> hv(n);
    std::memcpy(thrust::raw_pointer_cast(hv.data()), in.data() + n * sizeof(K), n * VB);
    c2h::device_vector<V> dv(hv);
    auto r = radix_sort_reference(dk, dv, desc, begin_bit, end_bit);
    out.write(reinterpret_cast<const char*>(thrust::raw_pointer_cast(r.first.data())), n * sizeof(K));
    out.write(reinterpret_cast<const char*>(thrust::raw_pointer_cast(r.second.data())), n * VB);
  }
  return 0;
}

template <class K>
static int by_value(int vb, uint64_t n, int b, int e, bool d, const std::vector<char>& in, std::ofstream& out)
{
  switch (vb)
  {
    case 0:
      return run<K, 0>(n, b, e, d, in, out);
    case 4:
      return run<K, 4>(n, b, e, d, in, out);
    case 8:
      return run<K, 8>(n, b, e, d, in, out);
    default:
      return 2;
  }
}

int main(int argc, char** argv)
{
  if (argc != 9)
  {
    std::fprintf(stderr, "usage: ref_pin key_type value_bytes n begin end desc in out\n");
    return 1;
  }
  const int kt   = std::atoi(argv[1]);
  const int vb   = std::atoi(argv[2]);
  const uint64_t n = std::strtoull(argv[3], nullptr, 10);
  const int b    = std::atoi(argv[4]);
  const int e    = std::atoi(argv[5]);
  const bool d   = std::atoi(argv[6]) != 0;
  std::ifstream fin(argv[7], std::ios::binary);
  std::vector<char> in((std::istreambuf_iterator<char>(fin)), std::istreambuf_iterator<char>());
  std::ofstream out(argv[8], std::ios::binary);
  switch (kt) // cccl_type_enum codes
  {
    case 0:
      return by_value<int8_t>(vb, n, b, e, d, in, out);
    case 1:
      return by_value<int16_t>(vb, n, b, e, d, in, out);
    case 2:
      return by_value<int32_t>(vb, n, b, e, d, in, out);
    case 3:
      return by_value<int64_t>(vb, n, b, e, d, in, out);
    case 4:
      return by_value<uint8_t>(vb, n, b, e, d, in, out);
    case 5:
      return by_value<uint16_t>(vb, n, b, e, d, in, out);
    case 6:
      return by_value<uint32_t>(vb, n, b, e, d, in, out);
    case 7:
      return by_value<uint64_t>(vb, n, b, e, d, in, out);
    case 8:
      return by_value<__half>(vb, n, b, e, d, in, out);
    case 9:
      return by_value<float>(vb, n, b, e, d, in, out);
    case 10:
      return by_value<double>(vb, n, b, e, d, in, out);
    default:
      return 3;
  }
}
