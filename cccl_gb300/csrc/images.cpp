// Accessors for the sm_103a cubins linked into the library. The bytes are placed by
// the build step (cccl_gb300/build.py writes an .incbin stub next to this file's object).
#include <atomic>

#include <cccl_gb300/sort_trace.h>

#include "abi_common.h"

extern "C" {
extern const unsigned char gb300_img_radix_k1[], gb300_img_radix_k1_end[];
extern const unsigned char gb300_img_radix_k2[], gb300_img_radix_k2_end[];
extern const unsigned char gb300_img_radix_k4[], gb300_img_radix_k4_end[];
extern const unsigned char gb300_img_radix_k8[], gb300_img_radix_k8_end[];
extern const unsigned char gb300_img_seg_k1[], gb300_img_seg_k1_end[];
extern const unsigned char gb300_img_seg_k2[], gb300_img_seg_k2_end[];
extern const unsigned char gb300_img_seg_k4[], gb300_img_seg_k4_end[];
extern const unsigned char gb300_img_seg_k8[], gb300_img_seg_k8_end[];
extern const unsigned char gb300_img_learned_k4[], gb300_img_learned_k4_end[];
extern const unsigned char gb300_img_learned_k8[], gb300_img_learned_k8_end[];
}

namespace gb300
{

image_ref radix_image(int key_bytes)
{
  switch (key_bytes)
  {
    case 1:
      return {gb300_img_radix_k1, size_t(gb300_img_radix_k1_end - gb300_img_radix_k1)};
    case 2:
      return {gb300_img_radix_k2, size_t(gb300_img_radix_k2_end - gb300_img_radix_k2)};
    case 4:
      return {gb300_img_radix_k4, size_t(gb300_img_radix_k4_end - gb300_img_radix_k4)};
    case 8:
      return {gb300_img_radix_k8, size_t(gb300_img_radix_k8_end - gb300_img_radix_k8)};
    default:
      throw cuda_error(CUDA_ERROR_NOT_SUPPORTED, "no kernels for this key width");
  }
}

image_ref segmented_image(int key_bytes)
{
  switch (key_bytes)
  {
    case 1:
      return {gb300_img_seg_k1, size_t(gb300_img_seg_k1_end - gb300_img_seg_k1)};
    case 2:
      return {gb300_img_seg_k2, size_t(gb300_img_seg_k2_end - gb300_img_seg_k2)};
    case 4:
      return {gb300_img_seg_k4, size_t(gb300_img_seg_k4_end - gb300_img_seg_k4)};
    case 8:
      return {gb300_img_seg_k8, size_t(gb300_img_seg_k8_end - gb300_img_seg_k8)};
    default:
      throw cuda_error(CUDA_ERROR_NOT_SUPPORTED, "no segmented kernels for this key width");
  }
}

image_ref learned_image(int key_bytes)
{
  switch (key_bytes)
  {
    case 4:
      return {gb300_img_learned_k4, size_t(gb300_img_learned_k4_end - gb300_img_learned_k4)};
    case 8:
      return {gb300_img_learned_k8, size_t(gb300_img_learned_k8_end - gb300_img_learned_k8)};
    default:
      throw cuda_error(CUDA_ERROR_NOT_SUPPORTED, "the learned sort takes 4- and 8-byte keys");
  }
}

} // namespace gb300

namespace
{
std::atomic<gb300::launch_observer_fn> g_observer{nullptr};
std::atomic<void*> g_observer_user{nullptr};
} // namespace

void gb300::notify_launch(const char* role, int phase, CUstream stream)
{
  if (auto fn = g_observer.load(std::memory_order_acquire))
  {
    fn(g_observer_user.load(std::memory_order_relaxed), role, phase, stream);
  }
}

extern "C" CCCL_GB300_API void cccl_gb300_set_launch_observer(cccl_gb300_launch_observer_t observer, void* user)
{
  g_observer_user.store(user, std::memory_order_relaxed);
  g_observer.store(observer, std::memory_order_release);
}
