// Device-side building blocks shared by the sort kernels: key bit-ordering, digit
// extraction, launch parameter blocks and the bounded look-back wait.
//
// Semantics follow CUB's radix sort exactly:
//  * keys are mapped to an unsigned bit order before ranking (cub/cub/util_type.cuh:893-963
//    Traits<T>::TwiddleIn/TwiddleOut), then bit-inverted for descending order
//    (cub/cub/block/radix_rank_sort_operations.cuh:536-575 RadixSortTwiddle);
//  * for floating-point keys the bit-ordered -0.0 is treated as +0.0 only when a digit is
//    extracted (radix_rank_sort_operations.cuh:43-80, ShiftDigitExtractor::Digit :124-127),
//    so +-0 compare equal, stay stable, and keep their own bit patterns in the output.
#pragma once

#include <cstdint>

#include "sort_params.h"

// Test hooks of the bounded waits, one copy per kernel image. With the defaults they change
// nothing. A test (cccl_gb300_testing_set_wait_fault) may name one tile of every digit pass
// whose look-back counts are then never published, and shorten the wait limit, so that the
// successors' waits run out, the pass reports STATUS_LOOKBACK_TIMEOUT and its kernels still
// return (no GPU hang: every wait below gives up after gb300_wait_limit_ns). Global-namespace
// variables keep their plain names as symbols, which is how the host finds them.
__device__ uint32_t gb300_fault_skip_tile = 0xffffffffu;
__device__ unsigned long long gb300_wait_limit_ns = gb300::LOOKBACK_TIMEOUT_NS;

namespace gb300
{

// Compile-time flag carried by a value (for generic lambdas).
template <bool B>
struct BoolTag
{
  static constexpr bool value = B;
};

template <int BYTES>
struct uint_of;
template <>
struct uint_of<1>
{
  using type = uint8_t;
};
template <>
struct uint_of<2>
{
  using type = uint16_t;
};
template <>
struct uint_of<4>
{
  using type = uint32_t;
};
template <>
struct uint_of<8>
{
  using type = unsigned long long;
};

// Opaque value payloads are moved as words of their own size.
template <int BYTES>
struct value_word
{
  using type = typename uint_of<BYTES>::type;
};
template <>
struct value_word<16>
{
  using type = uint4;
};
template <>
struct value_word<0>
{
  using type = uint32_t; // unused (keys-only)
};

template <class U>
__device__ __forceinline__ constexpr U high_bit()
{
  return U(U(1) << (8 * sizeof(U) - 1));
}

// Forward map raw key bits -> sortable unsigned bits (order already applied).
template <class U>
__device__ __forceinline__ U encode_key(U x, const KeyCodec& c)
{
  return U(x ^ U((x & high_bit<U>()) ? c.fwd_neg : c.fwd_pos));
}

// Inverse map sortable bits -> raw key bits.
template <class U>
__device__ __forceinline__ U decode_key(U t, const KeyCodec& c)
{
  return U(t ^ U((t & high_bit<U>()) ? c.inv_set : c.inv_clr));
}

// False when the kernel is gated off (see KernelGate).
__device__ __forceinline__ bool gate_open(const KernelGate& g)
{
  return g.gate == nullptr || (__ldcg(g.gate) & g.gate_mask) != 0u;
}

// Key modes (the FP template argument) and the digit source of an encoded key:
//   FP_NONE: integer keys, the encoded key itself;
//   FP_ONESWEEP: -0.0 and +0.0 both take the encoded pattern 0x80..0, in either order. CUB's
//     onesweep complements descending keys after twiddling and then folds the twiddled -0.0
//     pattern (cub/cub/block/radix_rank_sort_operations.cuh:43-80);
//   FP_BLOCK_DESC: descending sorts of CUB's block-radix paths (single tile, segmented radix
//     sort), which fold -0.0 into +0.0 before ordering: in the complemented key both zeros
//     take +0.0's pattern 0x7f..f.
// Over the whole key the two give one order (the patterns are adjacent); under a bit window
// the zeros' window bits differ, and each path must match its CUB counterpart.
constexpr int FP_NONE       = 0;
constexpr int FP_ONESWEEP   = 1;
constexpr int FP_BLOCK_DESC = 2;

template <class U, int FP>
__device__ __forceinline__ U digit_source(U t)
{
  if constexpr (FP == FP_ONESWEEP)
  {
    return (t == U(~high_bit<U>())) ? high_bit<U>() : t;
  }
  else if constexpr (FP == FP_BLOCK_DESC)
  {
    return (t == high_bit<U>()) ? U(~high_bit<U>()) : t;
  }
  else
  {
    return t;
  }
}

template <class U, int FP>
__device__ __forceinline__ uint32_t extract_digit(U t, int bit, uint32_t mask)
{
  return uint32_t(digit_source<U, FP>(t) >> bit) & mask;
}

__device__ __forceinline__ uint32_t lanemask_lt()
{
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ uint64_t global_timer_ns()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Look-back status word: bits 31..30 = flag, bits 29..0 = digit count.
constexpr uint32_t LB_EMPTY     = 0u;
constexpr uint32_t LB_PARTIAL   = 1u << 30;
constexpr uint32_t LB_INCLUSIVE = 2u << 30;
constexpr uint32_t LB_ERROR     = 3u << 30;
constexpr uint32_t LB_FLAGS     = 3u << 30;
constexpr uint32_t LB_VALUE     = (1u << 30) - 1;

__device__ __forceinline__ uint32_t load_status(const uint32_t* p)
{
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void store_status(uint32_t* p, uint32_t v)
{
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Waits until the status word is non-empty. Gives up after gb300_wait_limit_ns (1 s unless a
// test shortened it) and returns LB_ERROR, so a stuck predecessor can never hang the GPU.
__device__ __forceinline__ uint32_t wait_status(const uint32_t* p)
{
  uint32_t v = load_status(p);
  if ((v & LB_FLAGS) != LB_EMPTY)
  {
    return v;
  }
  const uint64_t start = global_timer_ns();
  uint32_t spins       = 0;
  while (true)
  {
    v = load_status(p);
    if ((v & LB_FLAGS) != LB_EMPTY)
    {
      return v;
    }
    if (++spins > 32)
    {
      __nanosleep(64);
      if (global_timer_ns() - start > gb300_wait_limit_ns)
      {
        return LB_ERROR;
      }
    }
  }
}

} // namespace gb300

// ---- bulk async copies global -> shared with mbarrier completion (sm_90+) ----
namespace gb300
{

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_init_fence()
{
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses before later
// async-proxy (bulk copy) accesses.
__device__ __forceinline__ void fence_proxy_async_smem()
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// 1-D bulk copy; dst/src 16-byte aligned, bytes a multiple of 16.
// L2 prefetch of [src, src + bytes) by the bulk-copy unit (src 16-byte aligned, bytes a
// multiple of 16); no completion to wait for.
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes)
{
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                 smem_addr(dst)),
               "l"(src),
               "r"(bytes),
               "r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile("{\n"
               "  .reg .pred p;\n"
               "  mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
               "  selp.u32 %0, 1, 0, p;\n"
               "}\n"
               : "=r"(ok)
               : "r"(smem_addr(bar)), "r"(parity)
               : "memory");
  return ok != 0;
}

// Waits for the barrier phase with the given parity to complete; gives up after
// gb300_wait_limit_ns and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity)
{
  if (mbar_try_wait(bar, parity))
  {
    return true;
  }
  const uint64_t start = global_timer_ns();
  while (!mbar_try_wait(bar, parity))
  {
    if (global_timer_ns() - start > gb300_wait_limit_ns)
    {
      return false;
    }
  }
  return true;
}

} // namespace gb300
