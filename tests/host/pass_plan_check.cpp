// Checks plan_pass_words (the plain sort's pass plan, cccl_gb300/csrc/sort_policy.h) for every
// pass count, buffer mode and set of skippable passes. Prints one line per failure and exits
// non-zero if any. Built and run by tests/test_pass_plan.py.
#include <cstdint>
#include <cstdio>
#include <initializer_list>

#include "sort_policy.h"

using namespace gb300;

namespace
{
int failures = 0;

void fail(int P, int mode, uint32_t mask, const char* what)
{
  if (failures < 20)
  {
    std::printf("P=%d mode=%d trivial=0x%02x: %s\n", P, mode, mask, what);
  }
  ++failures;
}

void check(int P, int mode, uint32_t mask)
{
  uint32_t plan[MAX_PASSES] = {};
  plan_pass_words(plan, P, mode, mask);
  int k = 0, extra = 0, first = -1, last = -1, prev_dst = -1;
  bool chain_ok = true;
  for (int q = 0; q < P; ++q)
  {
    const uint32_t w    = plan[q];
    const bool trivial  = (mask >> q) & 1u;
    if (w & PLAN_SKIP)
    {
      if (!trivial)
      {
        fail(P, mode, mask, "a pass with several digits is skipped");
      }
      if (w != PLAN_SKIP)
      {
        fail(P, mode, mask, "a skipped pass carries other flags");
      }
      continue;
    }
    extra += trivial ? 1 : 0;
    const int src = int(w >> PLAN_SRC_SHIFT) & 3;
    const int dst = int(w >> PLAN_DST_SHIFT) & 3;
    if (src == dst)
    {
      fail(P, mode, mask, "a pass reads and writes the same buffer");
    }
    if (mode == PLAN_MODE_DOUBLE)
    {
      if (src != (k & 1) || dst != ((k + 1) & 1))
      {
        chain_ok = false;
      }
    }
    else
    {
      if ((k == 0 && src != 0) || (k > 0 && src != prev_dst) || dst == 0)
      {
        chain_ok = false;
      }
      if (dst == 2 && P < 2)
      {
        fail(P, mode, mask, "the temporary buffer is used by a one-pass sort");
      }
    }
    if (((w & PLAN_ENCODE) != 0) != (k == 0))
    {
      fail(P, mode, mask, "encode is not on the first pass that runs");
    }
    if (first < 0)
    {
      first = q;
    }
    last     = q;
    prev_dst = dst;
    ++k;
  }
  if (!chain_ok)
  {
    fail(P, mode, mask, "the passes that run do not hand their buffers on in turn");
  }
  if (last >= 0 && !(plan[last] & PLAN_DECODE))
  {
    fail(P, mode, mask, "decode is not on the last pass that runs");
  }
  for (int q = 0; q < P; ++q)
  {
    if (q != last && (plan[q] & PLAN_DECODE))
    {
      fail(P, mode, mask, "decode on a pass that is not the last to run");
    }
  }
  int nontrivial = 0;
  for (int q = 0; q < P; ++q)
  {
    nontrivial += ((mask >> q) & 1u) ? 0 : 1;
  }
  if (mode == PLAN_MODE_DOUBLE)
  {
    // the result must land in buffer P & 1, where running every pass puts it
    if ((k & 1) != (P & 1))
    {
      fail(P, mode, mask, "the result lands in the other buffer");
    }
    if (extra != ((nontrivial & 1) != (P & 1) ? 1 : 0))
    {
      fail(P, mode, mask, "a skippable pass runs without need, or none runs when needed");
    }
  }
  else
  {
    if (k == 0)
    {
      fail(P, mode, mask, "no pass writes the output");
    }
    else if (prev_dst != 1)
    {
      fail(P, mode, mask, "the last pass does not write the output");
    }
    if (extra != (nontrivial == 0 ? 1 : 0))
    {
      fail(P, mode, mask, "a skippable pass runs without need, or none runs when needed");
    }
  }
  // look-back buffers (passes q and q + 2 share one): every pass that runs must find its
  // rows clean. Restated from resolve_pass (onesweep.cuh): the histogram clears the first
  // pass's buffer, a pass that runs uses its own and clears its successor's, a skipped pass
  // clears its successor's only when the previous pass ran (or it is the first pass).
  bool dirty[2] = {true, true}; // left by an earlier sort in the same temporary storage
  dirty[0]      = false;
  for (int q = 0; q < P; ++q)
  {
    const bool has_next = q + 1 < P;
    if (!(plan[q] & PLAN_SKIP))
    {
      if (dirty[q & 1])
      {
        fail(P, mode, mask, "a pass that runs finds its look-back rows dirty");
      }
      dirty[q & 1] = true;
      if (has_next)
      {
        dirty[(q + 1) & 1] = false;
      }
    }
    else
    {
      const bool prev_skipped = q > 0 && (plan[q - 1] & PLAN_SKIP);
      if (has_next && !prev_skipped)
      {
        dirty[(q + 1) & 1] = false;
      }
    }
  }
  if (extra == 1 && first >= 0)
  {
    // the extra pass is the first skippable one
    for (int q = 0; q < P; ++q)
    {
      if ((mask >> q) & 1u)
      {
        if (plan[q] & PLAN_SKIP)
        {
          fail(P, mode, mask, "the extra pass is not the first skippable one");
        }
        break;
      }
    }
  }
}
} // namespace

int main()
{
  int cases = 0;
  for (int P = 1; P <= MAX_PASSES; ++P)
  {
    for (int mode : {PLAN_MODE_DOUBLE, PLAN_MODE_SEPARATE})
    {
      for (uint32_t mask = 0; mask < (1u << P); ++mask)
      {
        check(P, mode, mask);
        ++cases;
      }
    }
  }
  std::printf("%d cases, %d failures\n", cases, failures);
  return failures == 0 ? 0 : 1;
}
