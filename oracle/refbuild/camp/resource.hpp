// Clean-room camp subset (test infrastructure): the host resource, a
// type-erased resource and event, and EventProxy -- enough for RAJA's
// sequential and OpenMP policies, which run synchronously on the host.
#ifndef CAMP_SUBSET_RESOURCE_HPP
#define CAMP_SUBSET_RESOURCE_HPP

#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <type_traits>
#if defined(__CUDACC__)
#include <cuda_runtime.h>
#endif

#include "camp/helpers.hpp"

namespace camp
{
namespace resources
{
inline namespace v1
{
// Ordered so that the larger value is the more specific (device) platform.
enum class Platform { undefined = 0, host = 1, cuda = 2, omp_target = 4, hip = 8, sycl = 16 };

enum class MemoryAccess { Unknown, Device, Pinned, Managed };

// Host work completes before the call returns, so host events are always
// complete.
struct HostEvent {
  bool check() const { return true; }
  void wait() const {}
};

class Event
{
public:
  Event() = default;
  template <typename E, typename = typename std::enable_if<!std::is_same<decay<E>, Event>::value>::type>
  Event(E&&)
  {
  }
  bool check() const { return true; }
  void wait() const {}
};

class Host
{
public:
  Host(int = 0) {}
  static Host get_default() { return Host(); }
  Platform get_platform() const { return Platform::host; }
  HostEvent get_event() { return HostEvent(); }
  Event get_event_erased() { return Event(HostEvent()); }
  void wait() {}
  void wait_for(Event*) {}
  template <typename T>
  T* allocate(size_t n, MemoryAccess = MemoryAccess::Device)
  {
    return static_cast<T*>(std::malloc(sizeof(T) * n));
  }
  void* calloc(size_t bytes, MemoryAccess = MemoryAccess::Device) { return std::calloc(1, bytes); }
  void deallocate(void* p, MemoryAccess = MemoryAccess::Device) { std::free(p); }
  void memcpy(void* dst, const void* src, size_t bytes) { std::memcpy(dst, src, bytes); }
  void memset(void* p, int val, size_t bytes) { std::memset(p, val, bytes); }
  bool operator==(Host const&) const { return true; }
  bool operator!=(Host const&) const { return false; }
};

// Type-erased resource: wraps any resource value and reports its platform.
class Resource
{
  struct Base {
    virtual ~Base() = default;
    virtual Platform platform() const = 0;
    virtual void wait() = 0;
    virtual const void* raw() const = 0;
    virtual const std::type_info& type() const = 0;
    virtual void* alloc(size_t bytes, MemoryAccess ma) = 0;
    virtual void dealloc(void* p, MemoryAccess ma) = 0;
    virtual void copy(void* dst, const void* src, size_t bytes) = 0;
    virtual void set(void* p, int v, size_t bytes) = 0;
  };
  template <typename R>
  struct Holder : Base {
    R r;
    explicit Holder(R rr) : r(rr) {}
    Platform platform() const override { return r.get_platform(); }
    void wait() override { r.wait(); }
    const void* raw() const override { return &r; }
    const std::type_info& type() const override { return typeid(R); }
    void* alloc(size_t bytes, MemoryAccess ma) override { return r.template allocate<char>(bytes, ma); }
    void dealloc(void* p, MemoryAccess ma) override { r.deallocate(p, ma); }
    void copy(void* dst, const void* src, size_t bytes) override { r.memcpy(dst, src, bytes); }
    void set(void* p, int v, size_t bytes) override { r.memset(p, v, bytes); }
  };
  std::shared_ptr<Base> m;

public:
  template <typename R,
            typename = typename std::enable_if<!std::is_same<decay<R>, Resource>::value>::type,
            typename = decltype(val<decay<R>&>().get_platform())>
  Resource(R&& r) : m(std::make_shared<Holder<decay<R>>>(static_cast<R&&>(r)))
  {
  }
  Platform get_platform() const { return m->platform(); }
  void wait() { m->wait(); }
  template <typename T>
  T* allocate(size_t n, MemoryAccess ma = MemoryAccess::Device)
  {
    return static_cast<T*>(m->alloc(sizeof(T) * n, ma));
  }
  void deallocate(void* p, MemoryAccess ma = MemoryAccess::Device) { m->dealloc(p, ma); }
  void memcpy(void* dst, const void* src, size_t bytes) { m->copy(dst, src, bytes); }
  void memset(void* p, int v, size_t bytes) { m->set(p, v, bytes); }
  Event get_event() { return Event(); }
  Event get_event_erased() { return Event(); }
  template <typename R>
  R get() const
  {
    if (m->type() != typeid(R)) throw std::runtime_error("Resource: wrong type requested");
    return *static_cast<const R*>(m->raw());
  }
  template <typename R>
  R* try_get()
  {
    return m->type() == typeid(R) ? const_cast<R*>(static_cast<const R*>(m->raw())) : nullptr;
  }
};

template <typename Res>
struct EventProxy {
  using native_event = decltype(val<Res&>().get_event());
  EventProxy(Res r) : res(r) {}
  EventProxy(EventProxy&&) = default;
  EventProxy& operator=(EventProxy&&) = default;
  native_event get() { return res.get_event(); }
  operator native_event() { return res.get_event(); }
  template <typename E = Event,
            typename = typename std::enable_if<!std::is_same<E, native_event>::value>::type>
  operator E()
  {
    return E(res.get_event());
  }
  Res res;
};

#if defined(__CUDACC__)
// A CUDA stream on the current device, with the part of camp's Cuda
// resource interface the b200 policies use (get_stream, get_default,
// get_platform, wait, stream-ordered memory helpers).
class Cuda
{
public:
  Cuda() : s(nullptr) {}
  explicit Cuda(cudaStream_t st) : s(st) {}
  static Cuda get_default() { return Cuda(); }
  static Cuda CudaFromStream(cudaStream_t st, int = 0) { return Cuda(st); }
  Platform get_platform() const { return Platform::cuda; }
  cudaStream_t get_stream() const { return s; }
  Event get_event() { return Event(); }
  Event get_event_erased() { return Event(); }
  void wait() { cudaStreamSynchronize(s); }
  void wait_for(Event*) {}
  template <typename T>
  T* allocate(size_t n, MemoryAccess = MemoryAccess::Device)
  {
    void* p = nullptr;
    cudaMallocAsync(&p, sizeof(T) * n, s);
    return static_cast<T*>(p);
  }
  void deallocate(void* p, MemoryAccess = MemoryAccess::Device) { cudaFreeAsync(p, s); }
  void memcpy(void* dst, const void* src, size_t bytes)
  {
    cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, s);
  }
  void memset(void* p, int v, size_t bytes) { cudaMemsetAsync(p, v, bytes, s); }
  bool operator==(Cuda const& o) const { return s == o.s; }

private:
  cudaStream_t s;
};
#endif

template <typename Res>
struct is_resource : std::false_type {
};
template <>
struct is_resource<Host> : std::true_type {
};
template <>
struct is_resource<Resource> : std::true_type {
};
}  // namespace v1
}  // namespace resources
}  // namespace camp

#endif
