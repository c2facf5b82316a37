// CUB comparison arm for the benchmark (never linked into libb200prims.so).
//
// RAJA's CUDA back-end computes scans and sorts by calling CUB:
//   impl::scan::exclusive      -> cub::DeviceScan::ExclusiveScan   (policy/cuda/scan.hpp:199-235)
//   impl::sort::stable/unstable -> cub::DeviceRadixSort::SortKeys   (policy/cuda/sort.hpp:92-160)
//   impl::sort::*_pairs        -> cub::DeviceRadixSort::SortPairs  (policy/cuda/sort.hpp:380-460)
// Sorts use CUB's out-of-place form (input preserved, alternate buffer in
// the temp storage), the same work as the library's *_copy sorts that the
// benchmark times.  RAJA's own form (a DoubleBuffer over the user's array
// plus a pool buffer) runs the same digit passes.
// This file times those same CUB calls (CCCL from the CUDA toolkit) on the
// benchmark's shapes, so the library's own scan and sort have "the kernel a
// RAJA user gets today" beside them.  Scratch (CUB temp storage) is
// allocated once in cub_arm_setup and excluded from the timed calls, as
// RAJA's pooled allocator makes it nearly free after the first call.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

namespace {
void* g_temp = nullptr;
size_t g_temp_bytes = 0;
char g_err[256];

int note(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return 0;
  std::snprintf(g_err, sizeof(g_err), "%s: %s", what, cudaGetErrorString(e));
  return 1;
}

template <class F>
size_t need(F f) {
  size_t b = 0;
  f(nullptr, b);
  return b;
}
}  // namespace

extern "C" {

const char* cub_arm_error() { return g_err; }

// Allocate CUB temp storage large enough for every call below at n items.
int cub_arm_setup(size_t n) {
  const int ni = static_cast<int>(n);
  size_t b = 0, t;
  t = need([&](void* p, size_t& s) {
    cub::DeviceScan::ExclusiveScan(p, s, (const int64_t*)nullptr, (int64_t*)nullptr,
                                   ::cuda::std::plus<int64_t>{}, int64_t(0), ni);
  });
  b = t > b ? t : b;
  t = need([&](void* p, size_t& s) {
    cub::DeviceRadixSort::SortKeys(p, s, (const uint32_t*)nullptr, (uint32_t*)nullptr, ni);
  });
  b = t > b ? t : b;
  t = need([&](void* p, size_t& s) {
    cub::DeviceRadixSort::SortKeys(p, s, (const uint64_t*)nullptr, (uint64_t*)nullptr, ni);
  });
  b = t > b ? t : b;
  t = need([&](void* p, size_t& s) {
    cub::DeviceRadixSort::SortPairs(p, s, (const float*)nullptr, (float*)nullptr,
                                    (const int32_t*)nullptr, (int32_t*)nullptr, ni);
  });
  b = t > b ? t : b;
  if (g_temp && g_temp_bytes >= b) return 0;
  if (g_temp) cudaFree(g_temp);
  g_temp = nullptr;
  g_temp_bytes = 0;
  if (note(cudaMalloc(&g_temp, b), "cudaMalloc(cub temp)")) return 1;
  g_temp_bytes = b;
  return 0;
}

void cub_arm_teardown() {
  if (g_temp) cudaFree(g_temp);
  g_temp = nullptr;
  g_temp_bytes = 0;
}

size_t cub_arm_temp_bytes() { return g_temp_bytes; }

// RAJA's exclusive scan with operators::plus and init 0 (scan.hpp:213-226)
int cub_exclusive_scan_i64(const int64_t* in, int64_t* out, size_t n, cudaStream_t s) {
  size_t b = g_temp_bytes;
  return note(cub::DeviceScan::ExclusiveScan(g_temp, b, in, out, ::cuda::std::plus<int64_t>{},
                                             int64_t(0), static_cast<int>(n), s),
              "DeviceScan::ExclusiveScan");
}

int cub_sort_keys_u32(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t s) {
  size_t b = g_temp_bytes;
  return note(cub::DeviceRadixSort::SortKeys(g_temp, b, in, out, static_cast<int>(n), 0, 32, s),
              "DeviceRadixSort::SortKeys<u32>");
}

int cub_sort_keys_u64(const uint64_t* in, uint64_t* out, size_t n, cudaStream_t s) {
  size_t b = g_temp_bytes;
  return note(cub::DeviceRadixSort::SortKeys(g_temp, b, in, out, static_cast<int>(n), 0, 64, s),
              "DeviceRadixSort::SortKeys<u64>");
}

int cub_sort_pairs_f32_i32(const float* kin, float* kout, const int32_t* vin, int32_t* vout,
                           size_t n, cudaStream_t s) {
  size_t b = g_temp_bytes;
  return note(cub::DeviceRadixSort::SortPairs(g_temp, b, kin, kout, vin, vout,
                                              static_cast<int>(n), 0, 32, s),
              "DeviceRadixSort::SortPairs<f32,i32>");
}

}  // extern "C"
