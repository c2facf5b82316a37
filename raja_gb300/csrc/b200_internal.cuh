// Internal definitions shared by the libb200prims translation units.
//
// Host side: error reporting, per-device properties, per-stream scratch
// arenas, the device status word and the launch-timing instrumentation
// (runtime.cu).  Device side: memory-ordering helpers, bounded waits, warp
// utilities and 16-byte vector types.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <cstring>

#include "../../include/b200prims.h"

namespace b200 {

// ------------------------------------------------------------------ host

// Record a failure message for b200_last_error_string() and return `code`.
int fail(int code, const char* fmt, ...);
// Map a CUDA error to B200_ERR_CUDA (or B200_OK for cudaSuccess).
int cuda_check(cudaError_t e, const char* what);
// Clear the message of the calling thread (called on success paths).
void clear_error();

// Devices a process may use (the per-device tables are this long).
constexpr int kMaxDevices = 64;

struct DeviceProps {
  int device = -1;
  int sms = 0;
  int cc_major = 0;
  int cc_minor = 0;
  int max_threads_per_sm = 0;
  size_t smem_per_block_optin = 0;
  size_t smem_per_sm = 0;
};
// Properties of the current device (cached after the first query).
int device_props(DeviceProps* out);

// Device status word of the current device: kernels OR an error code into
// it when a bounded wait gives up; b200_stream_synchronize() reads it.
int status_word(uint32_t** out);

// Polling bound for device waits (b200_set_spin_limit).
uint32_t spin_limit();

// Per-(device, stream) scratch arena.  The returned pointer stays valid for
// work enqueued on `stream` until the next scratch() call on that stream.
// `zeroed_counters` points at a small region (kCounterBytes) that was
// zeroed when the arena was created; kernels that use it must leave it
// zeroed when they finish (self-resetting tickets).
constexpr size_t kCounterBytes = 4096;
int scratch(cudaStream_t stream, size_t bytes, void** out,
            uint32_t** zeroed_counters);

// Launch-timing instrumentation (b200_prof_*).
bool prof_on();
void prof_begin(cudaStream_t s, const char* name, void** token);
void prof_end(cudaStream_t s, void* token);

// Round x up to a multiple of a.
inline size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Carve successive aligned sub-buffers out of one scratch allocation.
struct Carver {
  char* base;
  size_t off = 0;
  explicit Carver(void* p) : base(static_cast<char*>(p)) {}
  template <class T>
  T* take(size_t count) {
    off = round_up(off, 256);
    T* p = reinterpret_cast<T*>(base + off);
    off += count * sizeof(T);
    return p;
  }
};
// Size that a Carver sequence needs (same rounding as Carver::take).
struct Sizer {
  size_t off = 0;
  template <class T>
  void take(size_t count) {
    off = round_up(off, 256);
    off += count * sizeof(T);
  }
  size_t bytes() const { return round_up(off, 256); }
};

// Launch `kern` with instrumentation and error checking.
#define B200_LAUNCH(name, kern, grid, block, smem, stream, ...)              \
  do {                                                                       \
    void* _b200_tok = nullptr;                                               \
    if (::b200::prof_on()) ::b200::prof_begin((stream), (name), &_b200_tok); \
    kern<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);                \
    cudaError_t _b200_e = cudaGetLastError();                                \
    if (_b200_tok) ::b200::prof_end((stream), _b200_tok);                    \
    if (_b200_e != cudaSuccess) return ::b200::cuda_check(_b200_e, (name));  \
  } while (0)

#define B200_CUDA(call)                                          \
  do {                                                           \
    cudaError_t _b200_e = (call);                                \
    if (_b200_e != cudaSuccess) return ::b200::cuda_check(_b200_e, #call); \
  } while (0)

#define B200_TRY(call)                 \
  do {                                 \
    int _b200_rc = (call);             \
    if (_b200_rc != B200_OK) return _b200_rc; \
  } while (0)

// Once-per-(kernel, device) launch setup: the dynamic shared-memory opt-in
// (a per-device function attribute) and the resident blocks per SM.  Each
// kernel keeps one `static KernelSetup`; concurrent first calls from
// several host threads may both run the setup, which is idempotent.
struct KernelSetup {
  std::atomic<int> bps[kMaxDevices] = {};   // 0 until the device's first launch
};
template <class K>
int kernel_setup(KernelSetup& ks, const DeviceProps& props, K kern, int block, size_t dyn_smem,
                 int* bps) {
  int v = ks.bps[props.device].load(std::memory_order_acquire);
  if (v == 0) {
    if (dyn_smem > 0)
      B200_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(dyn_smem)));
    int b = 0;
    B200_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, block, dyn_smem));
    v = b > 0 ? b : 1;
    ks.bps[props.device].store(v, std::memory_order_release);
  }
  *bps = v;
  return B200_OK;
}

// Dynamic shared-memory opt-in, once per device, for a kernel whose size
// varies per launch: set to the largest size it is ever launched with, so
// that concurrent launches of different sizes never race on the attribute.
struct SmemOptIn {
  std::atomic<bool> done[kMaxDevices] = {};
};
template <class K>
int smem_optin(SmemOptIn& so, const DeviceProps& props, K kern, size_t max_smem) {
  if (!so.done[props.device].load(std::memory_order_acquire)) {
    B200_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(max_smem)));
    so.done[props.device].store(true, std::memory_order_release);
  }
  return B200_OK;
}

// ---------------------------------------------------------------- device

// Error codes ORed into the status word (bit positions name the waiter).
// The word is mapped host memory that the host clears with an atomic
// exchange, so kernels set bits with system-scope atomics.
constexpr uint32_t kStatusScanTimeout = 1u << 0;
constexpr uint32_t kStatusSortTimeout = 1u << 1;
constexpr uint32_t kStatusSegTimeout = 1u << 2;
constexpr uint32_t kStatusTmaTimeout = 1u << 3;

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_acquire64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release64(uint64_t* p, uint64_t v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed64(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}
__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// Shuffle an arbitrary trivially-copyable value (size multiple of 4).
template <class T>
__device__ __forceinline__ T shfl_xor_any(const T& v, int mask) {
  static_assert(sizeof(T) % 4 == 0, "shuffle type size");
  constexpr int W = sizeof(T) / 4;
  uint32_t w[W];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int i = 0; i < W; ++i) w[i] = __shfl_xor_sync(0xffffffffu, w[i], mask);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}
template <class T>
__device__ __forceinline__ T shfl_up_any(const T& v, int delta) {
  static_assert(sizeof(T) % 4 == 0, "shuffle type size");
  constexpr int W = sizeof(T) / 4;
  uint32_t w[W];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int i = 0; i < W; ++i) w[i] = __shfl_up_sync(0xffffffffu, w[i], delta);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}
template <class T>
__device__ __forceinline__ T shfl_idx_any(const T& v, int src) {
  static_assert(sizeof(T) % 4 == 0, "shuffle type size");
  constexpr int W = sizeof(T) / 4;
  uint32_t w[W];
  memcpy(w, &v, sizeof(T));
#pragma unroll
  for (int i = 0; i < W; ++i) w[i] = __shfl_sync(0xffffffffu, w[i], src);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}

// 16-byte vector of element type T.
template <class T>
struct alignas(16) Vec16 {
  static constexpr int N = 16 / sizeof(T);
  T v[N];
};

template <class T>
__device__ __forceinline__ Vec16<T> ld_vec_stream(const T* p) {
  // Streaming read-only load: data is touched once, keep it out of L1.
  Vec16<T> r;
  uint4 u = __ldcs(reinterpret_cast<const uint4*>(p));
  memcpy(&r, &u, 16);
  return r;
}
template <class T>
__device__ __forceinline__ Vec16<T> ld_vec(const T* p) {
  Vec16<T> r;
  uint4 u = __ldg(reinterpret_cast<const uint4*>(p));
  memcpy(&r, &u, 16);
  return r;
}
template <class T>
__device__ __forceinline__ void st_vec(T* p, const Vec16<T>& r) {
  uint4 u;
  memcpy(&u, &r, 16);
  *reinterpret_cast<uint4*>(p) = u;
}
template <class T>
__device__ __forceinline__ void st_vec_stream(T* p, const Vec16<T>& r) {
  uint4 u;
  memcpy(&u, &r, 16);
  __stcs(reinterpret_cast<uint4*>(p), u);
}

// ---- TMA bulk copies (cp.async.bulk) completed on an mbarrier.
// Addresses must be 16-byte aligned and sizes multiples of 16 bytes.
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
// make mbarrier initialisation visible to the async (TMA) proxy
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_load_1d(void* dst_smem, const void* src, uint32_t bytes,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst_smem)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// Bring `bytes` (a multiple of 16, from a 16-byte aligned address) into
// L2 without waiting for them.
__device__ __forceinline__ void prefetch_l2_bulk(const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tma_store_1d(void* dst, const void* src_smem, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
               "r"(smem_addr(src_smem)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_store_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// wait until at most N committed bulk stores still read shared memory
template <int N>
__device__ __forceinline__ void tma_store_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
template <int N>
__device__ __forceinline__ void tma_store_wait_all() {
  asm volatile("cp.async.bulk.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
  return ok != 0;
}
// Bounded wait for an mbarrier phase; false when the bound ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i <= limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// Drain wait after a bounded wait gave up: a bulk copy from valid global
// memory always completes, so this waits for it to land before the block
// reuses or releases its shared memory.  Its bound is fixed and large,
// independent of b200_set_spin_limit, so lowering that limit cannot let a
// block exit with a copy still writing into shared memory.
constexpr uint32_t kDrainPolls = 1u << 28;
__device__ __forceinline__ void mbar_drain(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < kDrainPolls; ++i)
    if (mbar_try_wait(bar, parity)) return;
}

// Error-free transformations (Knuth TwoSum, FMA-based TwoProd).
template <class F>
__device__ __forceinline__ void two_sum(F a, F b, F& s, F& e) {
  s = a + b;
  F bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = a * b;
  e = fmaf(a, b, -p);
}
__device__ __forceinline__ void two_prod(double a, double b, double& p, double& e) {
  p = a * b;
  e = fma(a, b, -p);
}

}  // namespace b200
