// Minimal stand-ins for the reference's c2h/Catch2 test harness, so that the reference's
// CPU sort reference (cub/test/catch2_radix_sort_helper.cuh) compiles on its own.
// Written for the oracle pin; no reference code is copied here.
#pragma once
#include <algorithm>
#include <cassert>
#include <cstdint>
#include <thrust/execution_policy.h>
#include <cstdio>
#include <cstdlib>
#define REQUIRE(x)                                                  \
  do                                                                \
  {                                                                 \
    if (!(x))                                                       \
    {                                                               \
      std::fprintf(stderr, "requirement failed: %s\n", #x);         \
      std::abort();                                                 \
    }                                                               \
  } while (0)
#include <c2h/vector.h>
namespace c2h
{
template <class... Ts>
struct type_list
{};
// declared only: referenced by helper templates the pin never instantiates
struct seed_t
{
  std::uint64_t value;
};
template <class... Ts>
void gen(Ts&&...);
inline const auto& device_policy = thrust::host;
} // namespace c2h
