// Runtime glue of libb200prims: error strings, device properties, the
// device status word, per-stream scratch arenas and launch timing.
//
// Replaces the reference's CUDA runtime layer for the primitive path:
// the device property cache and occupancy helpers
// (policy/cuda/MemUtils_CUDA.hpp:173-181, 401-499), the reducer and
// scan/sort memory pools (MemUtils_CUDA.hpp:69-167, util/basic_mempool.hpp)
// and the stream synchronisation bookkeeping (MemUtils_CUDA.hpp:205-269).
// The pools are replaced by one grow-only arena per (device, stream): work
// on one stream is ordered, so a call can reuse the previous call's scratch
// without any host synchronisation, and growth uses the stream-ordered
// allocator (cudaMallocAsync / cudaFreeAsync).
#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>
#include <atomic>

#include "b200_internal.cuh"

namespace b200 {

namespace {
thread_local std::string t_last_error;
std::mutex g_mu;
DeviceProps g_props[kMaxDevices];
uint32_t* g_status[kMaxDevices] = {};       // device address of the status word
uint32_t* g_status_host[kMaxDevices] = {};  // its host address (mapped pinned memory)
std::atomic<uint32_t> g_spin_limit{0};
constexpr uint32_t kDefaultSpinLimit = 1u << 22;  // ~0.4 s of polling

struct Arena {
  void* ptr = nullptr;
  size_t cap = 0;
  uint32_t* counters = nullptr;  // separate, zeroed at creation
};
std::map<std::pair<int, cudaStream_t>, Arena> g_arenas;

// ---- launch timing
std::atomic<bool> g_prof{false};
struct ProfRec {
  const char* name;
  cudaEvent_t a, b;
};
std::vector<ProfRec> g_pending;
std::vector<cudaEvent_t> g_event_pool;
struct ProfTotal {
  uint64_t launches = 0;
  double ms = 0.0;
};
std::map<std::string, ProfTotal> g_totals;
}  // namespace

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_last_error = buf;
  return code;
}

void clear_error() { t_last_error.clear(); }

int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return B200_OK;
  if (e == cudaErrorMemoryAllocation)
    return fail(B200_ERR_NOMEM, "%s: %s", what, cudaGetErrorString(e));
  return fail(B200_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int device_props(DeviceProps* out) {
  int dev = 0;
  B200_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(B200_ERR_ARG, "device %d out of range", dev);
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_props[dev].device == dev) {
      *out = g_props[dev];
      return B200_OK;
    }
  }
  DeviceProps p;
  p.device = dev;
  B200_CUDA(cudaDeviceGetAttribute(&p.sms, cudaDevAttrMultiProcessorCount, dev));
  B200_CUDA(cudaDeviceGetAttribute(&p.cc_major, cudaDevAttrComputeCapabilityMajor, dev));
  B200_CUDA(cudaDeviceGetAttribute(&p.cc_minor, cudaDevAttrComputeCapabilityMinor, dev));
  B200_CUDA(cudaDeviceGetAttribute(&p.max_threads_per_sm,
                                   cudaDevAttrMaxThreadsPerMultiProcessor, dev));
  int v = 0;
  B200_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  p.smem_per_block_optin = static_cast<size_t>(v);
  B200_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  p.smem_per_sm = static_cast<size_t>(v);
  std::lock_guard<std::mutex> lk(g_mu);
  g_props[dev] = p;
  *out = p;
  return B200_OK;
}

// The status word lives in mapped pinned host memory: kernels OR error bits
// into it through its device address (only when a bounded wait gives up),
// and a host thread reads it directly once the stream has synchronised.
// Reading a device word instead costs a copy-engine operation (about 3 us
// more per synchronisation on GB300).
namespace {
int status_words(uint32_t** dev_out, uint32_t** host_out) {
  int dev = 0;
  B200_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(B200_ERR_ARG, "device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_status[dev]) {
    void* h = nullptr;
    B200_CUDA(cudaHostAlloc(&h, 256, cudaHostAllocMapped | cudaHostAllocPortable));
    std::memset(h, 0, 256);
    void* d = nullptr;
    B200_CUDA(cudaHostGetDevicePointer(&d, h, 0));
    g_status_host[dev] = static_cast<uint32_t*>(h);
    g_status[dev] = static_cast<uint32_t*>(d);
  }
  if (dev_out) *dev_out = g_status[dev];
  if (host_out) *host_out = g_status_host[dev];
  return B200_OK;
}
}  // namespace

int status_word(uint32_t** out) { return status_words(out, nullptr); }

uint32_t spin_limit() {
  uint32_t v = g_spin_limit.load();
  return v ? v : kDefaultSpinLimit;
}

int scratch(cudaStream_t stream, size_t bytes, void** out, uint32_t** counters) {
  int dev = 0;
  B200_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_mu);
  Arena& a = g_arenas[std::make_pair(dev, stream)];
  if (!a.counters) {
    uint32_t* c = nullptr;
    cudaError_t e = cudaMalloc(&c, kCounterBytes);
    if (e != cudaSuccess) return cuda_check(e, "scratch counters");
    e = cudaMemset(c, 0, kCounterBytes);
    if (e != cudaSuccess) return cuda_check(e, "scratch counters memset");
    a.counters = c;
  }
  if (bytes > a.cap) {
    // Grow geometrically; the old buffer is released in stream order, after
    // the work already enqueued on this stream that may still use it.
    size_t cap = bytes;
    if (cap < 2 * a.cap) cap = 2 * a.cap;
    cap = round_up(cap, 1 << 20);
    void* p = nullptr;
    cudaError_t e = cudaMallocAsync(&p, cap, stream);
    if (e != cudaSuccess) return cuda_check(e, "scratch arena");
    if (a.ptr) cudaFreeAsync(a.ptr, stream);
    a.ptr = p;
    a.cap = cap;
  }
  *out = a.ptr;
  if (counters) *counters = a.counters;
  return B200_OK;
}

bool prof_on() { return g_prof.load(std::memory_order_relaxed); }

void prof_begin(cudaStream_t s, const char* name, void** token) {
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEvent_t ev[2];
  for (int i = 0; i < 2; ++i) {
    if (!g_event_pool.empty()) {
      ev[i] = g_event_pool.back();
      g_event_pool.pop_back();
    } else if (cudaEventCreate(&ev[i]) != cudaSuccess) {
      *token = nullptr;
      return;
    }
  }
  cudaEventRecord(ev[0], s);
  g_pending.push_back(ProfRec{name, ev[0], ev[1]});
  *token = reinterpret_cast<void*>(g_pending.size());
}

void prof_end(cudaStream_t s, void* token) {
  std::lock_guard<std::mutex> lk(g_mu);
  size_t i = reinterpret_cast<size_t>(token);
  if (i == 0 || i > g_pending.size()) return;
  cudaEventRecord(g_pending[i - 1].b, s);
}

}  // namespace b200

using namespace b200;

extern "C" {

int b200_abi_version(void) { return B200_ABI_VERSION; }

const char* b200_last_error_string(void) { return t_last_error.c_str(); }

int b200_stream_synchronize(b200_stream_t stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  uint32_t* host = nullptr;
  B200_TRY(status_words(nullptr, &host));
  // Only this stream is waited for; the word itself is shared by all
  // streams of the device, so an error raised by another stream's kernel
  // before this point is reported here too.
  B200_CUDA(cudaStreamSynchronize(s));
  const uint32_t h = __atomic_exchange_n(host, 0u, __ATOMIC_ACQ_REL);
  if (h != 0) {
    return fail(B200_ERR_TIMEOUT,
                "a bounded device wait gave up (status 0x%x: %s%s%s)", h,
                (h & kStatusScanTimeout) ? "scan look-back " : "",
                (h & kStatusSortTimeout) ? "sort look-back " : "",
                (h & kStatusSegTimeout) ? "batched/segmented look-back " : "");
  }
  return B200_OK;
}

int b200_status_word_address(const uint32_t** out) {
  if (!out) return fail(B200_ERR_ARG, "b200_status_word_address: null out");
  uint32_t* host = nullptr;
  B200_TRY(status_words(nullptr, &host));
  *out = host;
  return B200_OK;
}

int b200_set_spin_limit(uint64_t limit) {
  if (limit > 0xffffffffull) limit = 0xffffffffull;
  g_spin_limit.store(static_cast<uint32_t>(limit));
  return B200_OK;
}

int b200_device_info(int* sm_count, int* cc_major, int* cc_minor) {
  DeviceProps p;
  B200_TRY(device_props(&p));
  if (sm_count) *sm_count = p.sms;
  if (cc_major) *cc_major = p.cc_major;
  if (cc_minor) *cc_minor = p.cc_minor;
  return B200_OK;
}

int b200_release_scratch(void) {
  int dev = 0;
  B200_CUDA(cudaGetDevice(&dev));
  B200_CUDA(cudaDeviceSynchronize());
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto it = g_arenas.begin(); it != g_arenas.end();) {
    if (it->first.first == dev) {
      if (it->second.ptr) cudaFree(it->second.ptr);
      if (it->second.counters) cudaFree(it->second.counters);
      it = g_arenas.erase(it);
    } else {
      ++it;
    }
  }
  return B200_OK;
}

int b200_prof_enable(int enable) {
  g_prof.store(enable != 0);
  return B200_OK;
}

int b200_prof_reset(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& r : g_pending) {
    cudaEventSynchronize(r.b);
    g_event_pool.push_back(r.a);
    g_event_pool.push_back(r.b);
  }
  g_pending.clear();
  g_totals.clear();
  return B200_OK;
}

int b200_prof_read(char* names, size_t name_stride, uint64_t* launches,
                   double* total_ms, int cap) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& r : g_pending) {
    if (cudaEventSynchronize(r.b) != cudaSuccess) continue;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      ProfTotal& t = g_totals[r.name];
      t.launches += 1;
      t.ms += ms;
    }
    g_event_pool.push_back(r.a);
    g_event_pool.push_back(r.b);
  }
  g_pending.clear();
  int i = 0;
  for (auto& kv : g_totals) {
    if (i >= cap) break;
    if (names && name_stride > 0) {
      snprintf(names + static_cast<size_t>(i) * name_stride, name_stride, "%s",
               kv.first.c_str());
    }
    if (launches) launches[i] = kv.second.launches;
    if (total_ms) total_ms[i] = kv.second.ms;
    ++i;
  }
  return i;
}

}  // extern "C"
