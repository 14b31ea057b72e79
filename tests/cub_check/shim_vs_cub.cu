// Runs the same sorts through CUB (the CUDA toolkit's CCCL headers) and through the
// library's cub-compatible shim (include/cccl_gb300/cub_shim.h) and compares every output
// byte and every DoubleBuffer selector. Exit status 0 when all cases match.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_segmented_radix_sort.cuh>
#include <cub/device/device_segmented_sort.cuh>

#include <cccl_gb300/cub_shim.h>

#include <cstdio>
#include <cstring>
#include <vector>

namespace shim = cccl_gb300::cub;

#define CK(x)                                                                   \
  do                                                                            \
  {                                                                             \
    cudaError_t err_ = (x);                                                     \
    if (err_ != cudaSuccess)                                                    \
    {                                                                           \
      std::printf("CUDA error %d (%s) at %s:%d\n", int(err_), cudaGetErrorString(err_), __FILE__, __LINE__); \
      std::exit(2);                                                             \
    }                                                                           \
  } while (0)

static unsigned long long lcg_state = 0x9E3779B97F4A7C15ull;
static unsigned long long next64()
{
  lcg_state = lcg_state * 6364136223846793005ull + 1442695040888963407ull;
  unsigned long long x = lcg_state;
  x ^= x >> 29;
  x *= 0xBF58476D1CE4E5B9ull;
  x ^= x >> 32;
  return x;
}

template <class T>
std::vector<T> random_bits(size_t n)
{
  std::vector<T> v(n);
  for (auto& x : v)
  {
    unsigned long long r = next64();
    std::memcpy(&x, &r, sizeof(T));
  }
  return v;
}

// floats with +-0, +-inf, NaNs of both signs and payloads, denormals sprinkled in
template <class F, class U>
std::vector<F> special_floats(size_t n)
{
  std::vector<F> v(n);
  const int mant       = sizeof(F) == 4 ? 23 : 52;
  const U sign         = U(1) << (8 * sizeof(F) - 1);
  const U exp_all      = ((U(1) << (8 * sizeof(F) - 1 - mant)) - 1) << mant;
  const U pats[]       = {0, sign, exp_all, exp_all | sign, exp_all | (U(1) << (mant - 1)),
                          exp_all | (U(1) << (mant - 1)) | sign, exp_all | 1, 1, 1 | sign};
  for (size_t i = 0; i < n; ++i)
  {
    const unsigned long long r = next64();
    if ((r & 63) == 0)
    {
      std::memcpy(&v[i], &pats[(r >> 8) % 9], sizeof(F));
    }
    else
    {
      v[i] = F(double(static_cast<long long>((r >> 11) % 2000001) - 1000000) * 1e-3);
    }
  }
  return v;
}

template <class T>
T* to_dev(const std::vector<T>& h)
{
  T* d = nullptr;
  CK(cudaMalloc(&d, sizeof(T) * (h.size() ? h.size() : 1)));
  CK(cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
  return d;
}

template <class T>
std::vector<T> from_dev(const T* d, size_t n)
{
  std::vector<T> h(n);
  CK(cudaMemcpy(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost));
  return h;
}

template <class T>
bool same(const char* name, const char* what, const std::vector<T>& a, const std::vector<T>& b)
{
  if (a.size() == b.size() && std::memcmp(a.data(), b.data(), sizeof(T) * a.size()) == 0)
  {
    return true;
  }
  size_t i = 0;
  while (i < a.size() && std::memcmp(&a[i], &b[i], sizeof(T)) == 0)
  {
    ++i;
  }
  std::printf("FAIL %s: %s differ at index %zu of %zu\n", name, what, i, a.size());
  return false;
}

static int failures = 0;

// Runs the size query and the sort with temp storage for one callable.
template <class F>
void run(F&& f)
{
  size_t bytes = 0;
  CK(f(nullptr, bytes));
  void* tmp = nullptr;
  CK(cudaMalloc(&tmp, bytes ? bytes : 1));
  CK(f(tmp, bytes));
  CK(cudaDeviceSynchronize());
  CK(cudaFree(tmp));
}

template <class K, class V, bool DESC>
void pairs_case(const char* name, const std::vector<K>& hk, const std::vector<V>& hv, int b, int e)
{
  const size_t n = hk.size();
  K *ki = to_dev(hk), *ko_c = to_dev(hk), *ko_s = to_dev(hk);
  V *vi = to_dev(hv), *vo_c = to_dev(hv), *vo_s = to_dev(hv);
  run([&](void* t, size_t& s) {
    return DESC ? cub::DeviceRadixSort::SortPairsDescending(t, s, ki, ko_c, vi, vo_c, n, b, e)
                : cub::DeviceRadixSort::SortPairs(t, s, ki, ko_c, vi, vo_c, n, b, e);
  });
  run([&](void* t, size_t& s) {
    return DESC ? shim::DeviceRadixSort::SortPairsDescending(t, s, ki, ko_s, vi, vo_s, n, b, e)
                : shim::DeviceRadixSort::SortPairs(t, s, ki, ko_s, vi, vo_s, n, b, e);
  });
  bool ok = same(name, "keys", from_dev(ko_c, n), from_dev(ko_s, n)) && same(name, "values", from_dev(vo_c, n), from_dev(vo_s, n));
  std::printf("%s %s\n", ok ? "PASS" : "FAIL", name);
  failures += !ok;
  for (void* p : {(void*) ki, (void*) ko_c, (void*) ko_s, (void*) vi, (void*) vo_c, (void*) vo_s})
  {
    cudaFree(p);
  }
}

template <class K, bool DESC>
void keys_db_case(const char* name, const std::vector<K>& hk, int b, int e)
{
  const size_t n = hk.size();
  K *a_c = to_dev(hk), *b_c = to_dev(hk), *a_s = to_dev(hk), *b_s = to_dev(hk);
  cub::DoubleBuffer<K> dc(a_c, b_c);
  shim::DoubleBuffer<K> ds(a_s, b_s);
  run([&](void* t, size_t& s) {
    return DESC ? cub::DeviceRadixSort::SortKeysDescending(t, s, dc, n, b, e) : cub::DeviceRadixSort::SortKeys(t, s, dc, n, b, e);
  });
  run([&](void* t, size_t& s) {
    return DESC ? shim::DeviceRadixSort::SortKeysDescending(t, s, ds, n, b, e) : shim::DeviceRadixSort::SortKeys(t, s, ds, n, b, e);
  });
  bool ok = dc.selector == ds.selector;
  if (!ok)
  {
    std::printf("FAIL %s: selector %d vs %d\n", name, dc.selector, ds.selector);
  }
  ok = ok && same(name, "keys", from_dev(dc.Current(), n), from_dev(ds.Current(), n));
  std::printf("%s %s\n", ok ? "PASS" : "FAIL", name);
  failures += !ok;
  for (void* p : {(void*) a_c, (void*) b_c, (void*) a_s, (void*) b_s})
  {
    cudaFree(p);
  }
}

template <class K, class V>
void pairs_db_case(const char* name, const std::vector<K>& hk, const std::vector<V>& hv)
{
  const size_t n = hk.size();
  K *a_c = to_dev(hk), *b_c = to_dev(hk), *a_s = to_dev(hk), *b_s = to_dev(hk);
  V *x_c = to_dev(hv), *y_c = to_dev(hv), *x_s = to_dev(hv), *y_s = to_dev(hv);
  cub::DoubleBuffer<K> kc(a_c, b_c);
  cub::DoubleBuffer<V> vc(x_c, y_c);
  shim::DoubleBuffer<K> ks(a_s, b_s);
  shim::DoubleBuffer<V> vs(x_s, y_s);
  run([&](void* t, size_t& s) { return cub::DeviceRadixSort::SortPairs(t, s, kc, vc, n); });
  run([&](void* t, size_t& s) { return shim::DeviceRadixSort::SortPairs(t, s, ks, vs, n); });
  bool ok = kc.selector == ks.selector && vc.selector == vs.selector;
  if (!ok)
  {
    std::printf("FAIL %s: selector %d vs %d\n", name, kc.selector, ks.selector);
  }
  ok = ok && same(name, "keys", from_dev(kc.Current(), n), from_dev(ks.Current(), n))
    && same(name, "values", from_dev(vc.Current(), n), from_dev(vs.Current(), n));
  std::printf("%s %s\n", ok ? "PASS" : "FAIL", name);
  failures += !ok;
  for (void* p : {(void*) a_c, (void*) b_c, (void*) a_s, (void*) b_s, (void*) x_c, (void*) y_c, (void*) x_s, (void*) y_s})
  {
    cudaFree(p);
  }
}

template <class O>
void random_segments(size_t n, std::vector<O>& begin, std::vector<O>& end)
{
  size_t at = 0;
  while (at < n)
  {
    const unsigned long long r = next64();
    size_t len                  = (r & 3) == 0 ? 0 : size_t(1) << ((r >> 2) % 15);
    len                         = len + ((r >> 8) % (len + 1));
    if (at + len > n)
    {
      len = n - at;
    }
    begin.push_back(O(at));
    end.push_back(O(at + len));
    at += len;
  }
}

template <class K, class V, class O, bool DESC>
void segmented_pairs_case(const char* name, const std::vector<K>& hk, const std::vector<V>& hv)
{
  const size_t n = hk.size();
  std::vector<O> hb, he;
  random_segments(n, hb, he);
  const size_t ns = hb.size();
  O *db = to_dev(hb), *de = to_dev(he);
  K *ki = to_dev(hk), *ko_c = to_dev(hk), *ko_s = to_dev(hk);
  V *vi = to_dev(hv), *vo_c = to_dev(hv), *vo_s = to_dev(hv);
  run([&](void* t, size_t& s) {
    return DESC ? cub::DeviceSegmentedSort::StableSortPairsDescending(t, s, ki, ko_c, vi, vo_c, n, ns, db, de)
                : cub::DeviceSegmentedSort::StableSortPairs(t, s, ki, ko_c, vi, vo_c, n, ns, db, de);
  });
  run([&](void* t, size_t& s) {
    return DESC ? shim::DeviceSegmentedSort::StableSortPairsDescending(t, s, ki, ko_s, vi, vo_s, n, ns, db, de)
                : shim::DeviceSegmentedSort::StableSortPairs(t, s, ki, ko_s, vi, vo_s, n, ns, db, de);
  });
  bool ok = same(name, "keys", from_dev(ko_c, n), from_dev(ko_s, n)) && same(name, "values", from_dev(vo_c, n), from_dev(vo_s, n));
  std::printf("%s %s (%zu segments)\n", ok ? "PASS" : "FAIL", name, ns);
  failures += !ok;
  for (void* p : {(void*) db, (void*) de, (void*) ki, (void*) ko_c, (void*) ko_s, (void*) vi, (void*) vo_c, (void*) vo_s})
  {
    cudaFree(p);
  }
}

template <class K, class O>
void segmented_keys_db_case(const char* name, const std::vector<K>& hk)
{
  const size_t n = hk.size();
  std::vector<O> hb, he;
  random_segments(n, hb, he);
  const size_t ns = hb.size();
  O *db = to_dev(hb), *de = to_dev(he);
  K *a_c = to_dev(hk), *b_c = to_dev(hk), *a_s = to_dev(hk), *b_s = to_dev(hk);
  cub::DoubleBuffer<K> dc(a_c, b_c);
  shim::DoubleBuffer<K> ds(a_s, b_s);
  run([&](void* t, size_t& s) { return cub::DeviceSegmentedSort::SortKeysDescending(t, s, dc, n, ns, db, de); });
  run([&](void* t, size_t& s) { return shim::DeviceSegmentedSort::SortKeysDescending(t, s, ds, n, ns, db, de); });
  bool ok = dc.selector == ds.selector;
  if (!ok)
  {
    std::printf("FAIL %s: selector %d vs %d\n", name, dc.selector, ds.selector);
  }
  // positions outside every segment are not written by either: compare the current buffers
  ok = ok && same(name, "keys", from_dev(dc.Current(), n), from_dev(ds.Current(), n));
  std::printf("%s %s (%zu segments)\n", ok ? "PASS" : "FAIL", name, ns);
  failures += !ok;
  for (void* p : {(void*) db, (void*) de, (void*) a_c, (void*) b_c, (void*) a_s, (void*) b_s})
  {
    cudaFree(p);
  }
}

template <class K, class V, class O, bool DESC>
void segmented_radix_pairs_case(const char* name, const std::vector<K>& hk, const std::vector<V>& hv, int b, int e)
{
  const size_t n = hk.size();
  std::vector<O> hb, he;
  random_segments(n, hb, he);
  const size_t ns = hb.size();
  O *db = to_dev(hb), *de = to_dev(he);
  K *ki = to_dev(hk), *ko_c = to_dev(hk), *ko_s = to_dev(hk);
  V *vi = to_dev(hv), *vo_c = to_dev(hv), *vo_s = to_dev(hv);
  run([&](void* t, size_t& s) {
    return DESC ? cub::DeviceSegmentedRadixSort::SortPairsDescending(t, s, ki, ko_c, vi, vo_c, n, ns, db, de, b, e)
                : cub::DeviceSegmentedRadixSort::SortPairs(t, s, ki, ko_c, vi, vo_c, n, ns, db, de, b, e);
  });
  run([&](void* t, size_t& s) {
    return DESC ? shim::DeviceSegmentedRadixSort::SortPairsDescending(t, s, ki, ko_s, vi, vo_s, n, ns, db, de, b, e)
                : shim::DeviceSegmentedRadixSort::SortPairs(t, s, ki, ko_s, vi, vo_s, n, ns, db, de, b, e);
  });
  bool ok = same(name, "keys", from_dev(ko_c, n), from_dev(ko_s, n)) && same(name, "values", from_dev(vo_c, n), from_dev(vo_s, n));
  std::printf("%s %s (%zu segments)\n", ok ? "PASS" : "FAIL", name, ns);
  failures += !ok;
  for (void* p : {(void*) db, (void*) de, (void*) ki, (void*) ko_c, (void*) ko_s, (void*) vi, (void*) vo_c, (void*) vo_s})
  {
    cudaFree(p);
  }
}

template <class K, class O, bool DESC>
void segmented_radix_keys_db_case(const char* name, const std::vector<K>& hk, int b, int e)
{
  const size_t n = hk.size();
  std::vector<O> hb, he;
  random_segments(n, hb, he);
  const size_t ns = hb.size();
  O *db = to_dev(hb), *de = to_dev(he);
  K *a_c = to_dev(hk), *b_c = to_dev(hk), *a_s = to_dev(hk), *b_s = to_dev(hk);
  cub::DoubleBuffer<K> dc(a_c, b_c);
  shim::DoubleBuffer<K> ds(a_s, b_s);
  run([&](void* t, size_t& s) {
    return DESC ? cub::DeviceSegmentedRadixSort::SortKeysDescending(t, s, dc, n, ns, db, de, b, e)
                : cub::DeviceSegmentedRadixSort::SortKeys(t, s, dc, n, ns, db, de, b, e);
  });
  run([&](void* t, size_t& s) {
    return DESC ? shim::DeviceSegmentedRadixSort::SortKeysDescending(t, s, ds, n, ns, db, de, b, e)
                : shim::DeviceSegmentedRadixSort::SortKeys(t, s, ds, n, ns, db, de, b, e);
  });
  bool ok = dc.selector == ds.selector;
  if (!ok)
  {
    std::printf("FAIL %s: selector %d vs %d\n", name, dc.selector, ds.selector);
  }
  ok = ok && same(name, "keys", from_dev(dc.Current(), n), from_dev(ds.Current(), n));
  std::printf("%s %s (%zu segments)\n", ok ? "PASS" : "FAIL", name, ns);
  failures += !ok;
  for (void* p : {(void*) db, (void*) de, (void*) a_c, (void*) b_c, (void*) a_s, (void*) b_s})
  {
    cudaFree(p);
  }
}

int main()
{
  {
    auto k = random_bits<unsigned long long>((1u << 22) + 77);
    std::vector<unsigned> v(k.size());
    for (size_t i = 0; i < v.size(); ++i)
    {
      v[i] = unsigned(i);
    }
    pairs_case<unsigned long long, unsigned, false>("SortPairs u64+u32", k, v, 0, 64);
    pairs_case<unsigned long long, unsigned, false>("SortPairs u64+u32 bits 8..40", k, v, 8, 40);
  }
  {
    auto k = special_floats<float, unsigned>(3000017);
    std::vector<unsigned long long> v(k.size());
    for (size_t i = 0; i < v.size(); ++i)
    {
      v[i] = i;
    }
    pairs_case<float, unsigned long long, true>("SortPairsDescending f32+u64", k, v, 0, 32);
  }
  keys_db_case<int, false>("SortKeys i32 DoubleBuffer", random_bits<int>(1000003), 0, 32);
  keys_db_case<double, true>("SortKeysDescending f64 DoubleBuffer", special_floats<double, unsigned long long>(777777), 0, 64);
  keys_db_case<double, false>("SortKeys f64 bits 3..50", special_floats<double, unsigned long long>(65537), 3, 50);
  keys_db_case<__half, false>("SortKeys f16 DoubleBuffer", random_bits<__half>(123457), 0, 16);
  // descending float keys under a bit window: the single tile and the onesweep passes order the
  // zeros differently in CUB itself
  keys_db_case<float, true>("SortKeysDescending f32 bits 3..29 single tile", special_floats<float, unsigned>(4000), 3, 29);
  keys_db_case<float, true>("SortKeysDescending f32 bits 3..29 onesweep", special_floats<float, unsigned>(300001), 3, 29);
  keys_db_case<double, true>("SortKeysDescending f64 bits 0..50 single tile", special_floats<double, unsigned long long>(2000), 0, 50);
  {
    auto k = random_bits<unsigned>(4000);
    std::vector<unsigned char> v(k.size());
    for (size_t i = 0; i < v.size(); ++i)
    {
      v[i] = (unsigned char) i;
    }
    pairs_db_case<unsigned, unsigned char>("SortPairs u32+u8 DoubleBuffer single tile", k, v);
  }
  {
    auto k = special_floats<float, unsigned>(2000003);
    std::vector<int> v(k.size());
    for (size_t i = 0; i < v.size(); ++i)
    {
      v[i] = int(i);
    }
    segmented_pairs_case<float, int, int, false>("DeviceSegmentedSort StableSortPairs f32+i32", k, v);
    segmented_pairs_case<float, int, int, true>("DeviceSegmentedSort StableSortPairsDescending f32+i32", k, v);
  }
  segmented_keys_db_case<unsigned long long, long long>("DeviceSegmentedSort SortKeysDescending u64 DoubleBuffer",
                                                        random_bits<unsigned long long>(1500001));
  {
    auto k = special_floats<float, unsigned>(2000003);
    std::vector<int> v(k.size());
    for (size_t i = 0; i < v.size(); ++i)
    {
      v[i] = int(i);
    }
    segmented_radix_pairs_case<float, int, int, false>("DeviceSegmentedRadixSort SortPairs f32+i32", k, v, 0, 32);
    segmented_radix_pairs_case<float, int, int, true>("DeviceSegmentedRadixSort SortPairsDescending f32+i32 bits 3..29", k, v, 3, 29);
  }
  segmented_radix_keys_db_case<unsigned long long, long long, false>(
    "DeviceSegmentedRadixSort SortKeys u64 DoubleBuffer bits 4..44", random_bits<unsigned long long>(1500001), 4, 44);
  segmented_radix_keys_db_case<double, int, true>(
    "DeviceSegmentedRadixSort SortKeysDescending f64 DoubleBuffer", special_floats<double, unsigned long long>(900001), 0, 64);
  segmented_radix_keys_db_case<unsigned, int, false>(
    "DeviceSegmentedRadixSort SortKeys u32 DoubleBuffer empty window", random_bits<unsigned>(300001), 7, 7);
  std::printf("%d failure(s)\n", failures);
  return failures == 0 ? 0 : 1;
}
