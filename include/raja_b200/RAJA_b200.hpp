// RAJA_b200.hpp -- the b200 policy family for RAJA's data-parallel
// primitive path on GB300 (sm_103a).
//
//   RAJA::b200_exec<BLOCK, Async>   forall over range / strided / list /
//                                   IndexSet segments (replaces cuda_exec,
//                                   policy/cuda/forall.hpp:554-706); BLOCK 0
//                                   tunes block size and elements per thread
//                                   on line (b200::tune)
//   RAJA::b200_reduce               ReduceSum/Min/Max/MinLoc/MaxLoc/BitOr/
//                                   BitAnd captured in device lambdas
//                                   (replaces cuda_reduce,
//                                   policy/cuda/reduce.hpp:968-1378)
//   expt::Reduce / ReduceLoc        forall params (policy/cuda/params/reduce.hpp)
//   scans, sorts                    impl::scan / impl::sort overloads that
//                                   forward to libb200prims (replace the CUB
//                                   wrappers policy/cuda/scan.hpp, sort.hpp)
//   RAJA::b200_multi_reduce         MultiReduceSum/Min/Max/BitOr/BitAnd
//                                   (policy/cuda/multi_reduce.hpp)
//   RAJA::b200_atomic               RAJA's atomic family (policy/cuda/atomic.hpp)
//   RAJA::b200_work<BLOCK>          WorkGroup runner: b200_unordered runs
//                                   every loop in one persistent launch with
//                                   captured reducers combined inside it;
//                                   ordered / reverse_ordered launch per loop
//                                   (policy/cuda/WorkGroup/WorkRunner.hpp);
//                                   BLOCK 0 tunes the tile shape per group
//   RAJA::b200_synchronize          RAJA::synchronize<> target
//   RAJA::resources::Cuda           stream resource for the b200 policies:
//                                   forall / scan / sort / WorkGroup::run
//                                   take it first and return EventProxy
//
// With an installed RAJA, include this header before RAJA/RAJA.hpp (it
// includes RAJA/RAJA.hpp itself): RAJA's front-ends reach the b200
// overloads through qualified calls that see only earlier declarations.
// With raja_compat, include it after RAJA/RAJA.hpp.  Lambda loop bodies
// stay templated and are compiled into the application with nvcc
// --extended-lambda; fixed-type work goes through the C ABI in b200prims.h.
// Errors throw std::runtime_error, as RAJA's CUDA back-end does
// (policy/cuda/raja_cudaerrchk.hpp:116-137).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "../b200prims.h"

// Host-and-device functions of this header.  RAJA's own RAJA_HOST_DEVICE
// is empty in an installed RAJA configured without its CUDA back-end, which
// the b200 policies do not need.
#if defined(__CUDACC__)
#define B200_HOST_DEVICE __host__ __device__
#else
#define B200_HOST_DEVICE
#endif

#if !defined(RAJA_COMPAT_FRONTEND)
// An installed RAJA.  RAJA's scan and sort front-ends call impl::scan:: and
// impl::sort:: by qualified name, which finds only the overloads declared
// before those front-ends, so this header comes before RAJA/RAJA.hpp: it
// includes the parts of RAJA its declarations need, declares the b200
// overloads, and then includes RAJA/RAJA.hpp itself (RAJA's own back-ends
// sit at the same place inside RAJA/RAJA.hpp).
#if defined(RAJA_scan_HPP) || defined(RAJA_sort_HPP) || defined(RAJA_pattern_atomic_HPP)
#error "include raja_b200/RAJA_b200.hpp before RAJA/RAJA.hpp (it adds impl::scan / impl::sort / atomic overloads)"
#endif
// RAJA's policy-generic atomics (atomicAdd<Policy>(acc, v) and the rest)
// call RAJA::atomicAdd(Policy{}, acc, v) by qualified name
// (pattern/atomic.hpp:113-118), so the b200_atomic forms are declared here,
// ahead of every RAJA header; they are defined with the other atomics below.
namespace RAJA {
struct b200_atomic;
template <typename T> B200_HOST_DEVICE inline T atomicLoad(b200_atomic, T* acc);
template <typename T> B200_HOST_DEVICE inline void atomicStore(b200_atomic, T* acc, T v);
template <typename T> B200_HOST_DEVICE inline T atomicAdd(b200_atomic, T* acc, T v);
template <typename T> B200_HOST_DEVICE inline T atomicSub(b200_atomic, T* acc, T v);
template <typename T> B200_HOST_DEVICE inline T atomicMin(b200_atomic, T* acc, T v);
template <typename T> B200_HOST_DEVICE inline T atomicMax(b200_atomic, T* acc, T v);
template <typename T> B200_HOST_DEVICE inline T atomicInc(b200_atomic, T* acc);
template <typename T> B200_HOST_DEVICE inline T atomicInc(b200_atomic, T* acc, T val);
template <typename T> B200_HOST_DEVICE inline T atomicDec(b200_atomic, T* acc);
template <typename T> B200_HOST_DEVICE inline T atomicDec(b200_atomic, T* acc, T val);
template <typename T> B200_HOST_DEVICE inline T atomicAnd(b200_atomic, T* acc, T v);
template <typename T> B200_HOST_DEVICE inline T atomicOr(b200_atomic, T* acc, T v);
template <typename T> B200_HOST_DEVICE inline T atomicXor(b200_atomic, T* acc, T v);
template <typename T> B200_HOST_DEVICE inline T atomicExchange(b200_atomic, T* acc, T v);
template <typename T> B200_HOST_DEVICE inline T atomicCAS(b200_atomic, T* acc, T compare, T v);
}  // namespace RAJA
#include "RAJA/config.hpp"
#include "RAJA/policy/PolicyBase.hpp"
#include "RAJA/util/Operators.hpp"
#include "RAJA/util/resource.hpp"
#include "RAJA/pattern/reduce.hpp"
#include "RAJA/pattern/multi_reduce.hpp"
#include "RAJA/pattern/atomic.hpp"
#endif

#if defined(RAJA_ENABLE_NVTX)
#include <nvtx3/nvToolsExt.h>
#endif

namespace RAJA {

// ------------------------------------------------------------ policies
// On an installed RAJA the exec policy carries RAJA's policy traits (a
// CUDA-platform forall policy, as the reference's cuda_exec does), so that
// RAJA's front-ends accept it; raja_compat needs none.
#if defined(RAJA_COMPAT_FRONTEND)
template <int BLOCK = 256, bool Async = false>
struct b200_exec {
  static constexpr int block_size = BLOCK;
  static constexpr bool async = Async;
};
template <int BLOCK = 256, bool Async = false>
struct b200_work {};
// order policy of the one-launch WorkGroup runner (the compat front-end's
// own unordered)
using b200_unordered = unordered;
#else
template <int BLOCK = 256, bool Async = false>
struct b200_exec : make_policy_pattern_launch_platform_t<Policy::cuda, Pattern::forall,
                                                         (Async ? Launch::async : Launch::sync),
                                                         Platform::cuda> {
  static constexpr int block_size = BLOCK;
  static constexpr bool async = Async;
};
// WorkGroup exec policy (as cuda_work, policy/cuda/policy.hpp:384-389)
template <int BLOCK = 256, bool Async = false>
struct b200_work : make_policy_pattern_launch_platform_t<Policy::cuda, Pattern::workgroup_exec,
                                                         (Async ? Launch::async : Launch::sync),
                                                         Platform::cuda> {};
// Order policy of the one-launch WorkGroup runner: every loop in one
// persistent launch (RAJA's own unordered CUDA order policy is
// unordered_cuda_loop_y_block_iter_x_threadblock_average,
// policy/cuda/policy.hpp:395-400).
struct b200_unordered : make_policy_pattern_platform_t<Policy::cuda, Pattern::workgroup_order, Platform::cuda> {};
#endif
template <int BLOCK = 256>
using b200_exec_async = b200_exec<BLOCK, true>;
struct b200_reduce {};
struct b200_multi_reduce {};
struct b200_atomic {};
struct b200_synchronize {};

namespace b200 {

// Stream used by b200 policies (the legacy default stream unless set).
inline cudaStream_t& stream() {
  static thread_local cudaStream_t s = nullptr;
  return s;
}

inline void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
inline void check(int rc, const char* what) {
  if (rc != B200_OK)
    throw std::runtime_error(std::string(what) + ": " + b200_last_error_string());
}
// Wait for the b200 stream and surface device-side errors (bounded waits
// that gave up), like res.wait() + cudaErrchk.
inline void wait() { check(b200_stream_synchronize(stream()), "b200 synchronize"); }

// Devices a process may use (per-device caches are this long).
constexpr int kMaxDevices = 64;

inline int current_device_index() {
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) throw std::runtime_error("b200: device index out of range");
  return dev;
}

// SM count of the current device, queried once per device.
inline int sm_count() {
  static std::atomic<int> n[kMaxDevices] = {};
  const int dev = current_device_index();
  int v = n[dev].load(std::memory_order_acquire);
  if (v == 0) {
    check_cuda(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev), "sm count");
    n[dev].store(v, std::memory_order_release);
  }
  return v;
}

namespace detail {

// Launch context read by reducer copy constructors while forall_impl makes
// the launch copy of the loop body (the role of RAJA's tl_status,
// policy/cuda/MemUtils_CUDA.hpp:379-394).
struct LaunchCtx {
  bool active = false;
  unsigned grid = 0;
  cudaStream_t stream = nullptr;
  unsigned long long launch_id = 0;  // new for every launch copy
};
inline LaunchCtx& ctx() {
  static thread_local LaunchCtx c;
  return c;
}

// WorkGroup capture (host): while a b200 WorkPool copies an enqueued loop
// body, each captured b200 reducer gets a slot for that loop -- one
// partial per (tile, warp) of the loop, in device memory -- an accumulator
// cell in mapped pinned memory, and a fold entry.  After each run's loop
// launches, one fold launch adds every entry's partials in (tile, warp)
// order and folds the loop's result into the cell (runs fold in stream
// order, so no host work is needed per run).  The pool's registry owns the
// slots, cells and entries and records an event behind the last run on
// each stream; a reducer's get() waits for those events and reads its cell.
constexpr size_t kWgCellBytes = 32;  // value (at most 24 bytes), then a "has a value" word at byte 28
// Device code that adds `count` partials in index order and folds the
// result into a cell (one per reducer kind).  Its address sits in the
// 16 bytes in front of a slot's partials, stored there on the device by the
// warp that writes partial 0 of each run.
using wg_fold_fn = void (*)(const void* parts, unsigned count, void* cell);
constexpr size_t kWgSlotHeader = 16;
struct WgFold {
  const void* parts;  // the loop's partials: tile-major, one per warp of the block
  void* cell;         // device address of the reducer's cell
  long long loop;     // the loop's index in its group
};
struct WgRegistry {
  std::vector<void*> blocks;       // device memory of the slots
  std::vector<void*> host_blocks;  // mapped pinned memory of the cells
  std::vector<WgFold> folds;       // one per (captured reducer, loop), in capture order
  unsigned char* cell_host = nullptr;
  unsigned char* cell_dev = nullptr;
  size_t cells_left = 0;
  std::mutex m;
  // per stream a run went to: an event recorded behind its last run, and
  // whether that run has been waited for
  struct RunMark {
    cudaStream_t stream;
    cudaEvent_t event;
    bool pending;
  };
  std::vector<RunMark> marks;
  WgRegistry() = default;
  WgRegistry(const WgRegistry&) = delete;
  WgRegistry& operator=(const WgRegistry&) = delete;
  ~WgRegistry() {
    for (void* b : blocks) cudaFree(b);
    for (void* b : host_blocks) cudaFreeHost(b);
    for (const RunMark& r : marks) cudaEventDestroy(r.event);
  }
  // A zeroed cell (host and device addresses), from 64 KB pinned chunks.
  void new_cell(unsigned char** host, unsigned char** dev) {
    std::lock_guard<std::mutex> g(m);
    if (cells_left == 0) {
      constexpr size_t chunk = 65536;
      void* h = nullptr;
      check_cuda(cudaHostAlloc(&h, chunk, cudaHostAllocMapped), "WorkGroup reducer cells");
      host_blocks.push_back(h);
      void* d = nullptr;
      check_cuda(cudaHostGetDevicePointer(&d, h, 0), "WorkGroup reducer cells");
      std::memset(h, 0, chunk);
      cell_host = static_cast<unsigned char*>(h);
      cell_dev = static_cast<unsigned char*>(d);
      cells_left = chunk / kWgCellBytes;
    }
    *host = cell_host;
    *dev = cell_dev;
    cell_host += kWgCellBytes;
    cell_dev += kWgCellBytes;
    --cells_left;
  }
  // Before a run's launches on stream s: when loops captured reducers, the
  // run follows every earlier run on other streams (runs of one group share
  // the reducers' partials, and fold into the cells in order).
  // Runs issued while s is being captured into a graph are left out: the
  // graph's launches are ordered by the caller, and the reducers' cells are
  // read after the caller has synchronised the graph's stream.
  void order_after_runs(cudaStream_t s) {
    std::lock_guard<std::mutex> g(m);
    if (blocks.empty() || capturing(s)) return;
    for (const RunMark& r : marks)
      if (r.stream != s) check_cuda(cudaStreamWaitEvent(s, r.event, 0), "WorkGroup run order");
  }
  // After a run's launches on stream s (the events outlive the stream).
  void ran_on(cudaStream_t s) {
    std::lock_guard<std::mutex> g(m);
    if (blocks.empty() || capturing(s)) return;
    auto it = std::find_if(marks.begin(), marks.end(), [s](const RunMark& r) { return r.stream == s; });
    if (it == marks.end()) {
      cudaEvent_t e = nullptr;
      check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "WorkGroup run event");
      marks.push_back(RunMark{s, e, false});
      it = marks.end() - 1;
    }
    check_cuda(cudaEventRecord(it->event, s), "WorkGroup run event");
    it->pending = true;
  }
  static bool capturing(cudaStream_t s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone;
  }
  // Wait for every run issued so far.
  void wait_runs() {
    std::lock_guard<std::mutex> g(m);
    for (RunMark& r : marks) {
      if (!r.pending) continue;
      check_cuda(cudaEventSynchronize(r.event), "WorkGroup reducer wait");
      r.pending = false;
    }
  }
};
struct WgCaptureCtx {
  bool active = false;
  std::shared_ptr<WgRegistry> reg;
  long long nslots = 0;               // partials the loop being captured needs (most over the tile shapes)
  long long loop = 0;                 // its index in the group
  unsigned long long capture_id = 0;  // new for every enqueue
};
inline WgCaptureCtx& wg_capture() {
  static thread_local WgCaptureCtx c;
  return c;
}


// Grid for a kernel that always runs `block` threads: one block per
// `block` x `items` elements, capped at the resident blocks of the whole
// GPU (the loop grid-strides beyond that).  The occupancy query runs once per (kernel,
// device), as RAJA's CUDA back-end caches it after the first launch.
template <auto Kernel>
inline unsigned grid_for(int block, long long len, int items = 1) {
  static std::atomic<long long> resident[kMaxDevices] = {};
  const int dev = current_device_index();
  long long cap = resident[dev].load(std::memory_order_acquire);
  if (cap == 0) {
    int bps = 0;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, Kernel, block, 0), "occupancy");
    cap = (long long)sm_count() * (bps > 0 ? bps : 1);
    resident[dev].store(cap, std::memory_order_release);
  }
  const long long per = (long long)block * (items > 0 ? items : 1);
  long long g = (len + per - 1) / per;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return unsigned(g);
}

// ---- device combine helpers (block reduce + last-block ticket)
// Threads and blocks are numbered linearly (x fastest), so the helpers
// serve 1-D forall launches and the 1-3-D grids of RAJA::launch alike.
__device__ inline unsigned lin_tid() { return threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z); }
__device__ inline unsigned lin_nthreads() { return blockDim.x * blockDim.y * blockDim.z; }
__device__ inline unsigned lin_bid() { return blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z); }
__device__ inline unsigned lin_nblocks() { return gridDim.x * gridDim.y * gridDim.z; }

template <class T>
__device__ inline T shfl_down_t(const T& v, int o, unsigned mask) {
  static_assert(sizeof(T) % 4 == 0, "reducer value size");
  unsigned w[sizeof(T) / 4];
  memcpy(w, &v, sizeof(T));
  for (int i = 0; i < int(sizeof(T) / 4); ++i) w[i] = __shfl_down_sync(mask, w[i], o);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}
// Fold the first `valid` lanes of this warp into lane 0.  `present` lanes
// of the warp exist (a block's last warp may be partial) and all of them
// take part in the shuffles.
template <class T, class Merge>
__device__ inline T warp_fold(T v, int lane, int valid, int present, Merge merge) {
  const unsigned mask = present >= 32 ? 0xffffffffu : ((1u << present) - 1u);
  for (int o = 16; o > 0; o >>= 1) {
    const T other = shfl_down_t(v, o, mask);
    if (lane + o < valid) v = merge(v, other);
  }
  return v;
}

template <class T, class Merge>
__device__ inline T block_reduce(T v, Merge merge) {
  static_assert(alignof(T) <= 16, "reducer values are aligned to at most 16 bytes");
  // typed views of byte buffers need the alignment of T (values up to 16 B)
  __shared__ __align__(16) unsigned char sh_raw[32 * sizeof(T) + 16];
  T* sh = reinterpret_cast<T*>(sh_raw);
  const int tid = int(lin_tid()), nt = int(lin_nthreads());
  const int lane = tid & 31, warp = tid >> 5, nw = (nt + 31) >> 5;
  const int present = nt - warp * 32 < 32 ? nt - warp * 32 : 32;
  v = warp_fold(v, lane, present, present, merge);
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  if (warp == 0) v = warp_fold(sh[lane < nw ? lane : 0], lane, nw, present, merge);
  __syncthreads();
  return v;  // valid in thread 0
}

template <class T>
struct DevSlot {
  T* partials;        // one per block
  unsigned* ticket;   // zero before the launch; the last block re-zeroes it
  T* result;          // written by the last block
};

// Read a value another block wrote in this kernel (bypass L1).
template <class T>
__device__ inline T ld_cg(const T* p) {
  static_assert(sizeof(T) % 4 == 0, "reducer value size");
  unsigned w[sizeof(T) / 4];
  const unsigned* q = reinterpret_cast<const unsigned*>(p);
  for (int i = 0; i < int(sizeof(T) / 4); ++i) w[i] = __ldcg(q + i);
  T r;
  memcpy(&r, w, sizeof(T));
  return r;
}

// Block reduce, publish one partial per block, and let the last block to
// take the ticket fold all partials (reduce.hpp:133-214 restated).
template <class T, class Merge>
__device__ inline void grid_combine(const DevSlot<T>& s, T v, Merge merge) {
  __shared__ bool last;
  const unsigned tid = lin_tid(), nt = lin_nthreads(), nb = lin_nblocks();
  v = block_reduce(v, merge);
  if (tid == 0) {
    s.partials[lin_bid()] = v;
    __threadfence();
    last = ::atomicAdd(s.ticket, 1u) == nb - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // thread t folds partials t, t + nt, ...; the threads holding partials
  // are a prefix 0 .. min(nb, nt) - 1, so only those merge below
  T r = v;
  for (unsigned b = tid; b < nb; b += nt) {
    const T p = ld_cg(s.partials + b);
    r = b == tid ? p : merge(r, p);
  }
  __shared__ __align__(16) unsigned char fin_raw[32 * sizeof(T) + 16];
  T* fin = reinterpret_cast<T*>(fin_raw);
  const int lane = int(tid & 31), warp = int(tid >> 5);
  const int holders = int(nb < nt ? nb : nt);
  const int present = int(nt) - warp * 32 < 32 ? int(nt) - warp * 32 : 32;
  int valid = holders - warp * 32;
  valid = valid < 0 ? 0 : (valid > 32 ? 32 : valid);
  r = warp_fold(r, lane, valid, present, merge);
  if (lane == 0 && valid > 0) fin[warp] = r;
  __syncthreads();
  if (tid == 0) {
    T acc = fin[0];
    for (int w = 1; w * 32 < holders; ++w) acc = merge(acc, fin[w]);
    *s.result = acc;
    *s.ticket = 0u;
  }
}

// The device context of a WorkGroup run: per warp of the block, the slot
// its reducer partials go to for the tile being run (tile of the loop x
// warps per block + warp).  Lane 0 of the warp writes it before the loop
// body runs and reads it in the reducers' combine, so no barrier is needed.
__device__ __forceinline__ long long* wg_warp_slots() {
  __shared__ long long slots[32];
  return slots;
}

// Fold count partials in index order with every thread of the block
// (thread t takes t, t + nthreads, ...; then a fixed tree): the result,
// valid in thread 0, depends only on the partials and the block shape.
template <class T, class Merge>
__device__ inline T fold_partials(const T* parts, unsigned count, Merge merge) {
  const unsigned tid = lin_tid(), nt = lin_nthreads();
  T r{};
  for (unsigned b = tid; b < count; b += nt) {
    const T p = ld_cg(parts + b);
    r = b == tid ? p : merge(r, p);
  }
  __shared__ __align__(16) unsigned char fold_raw[32 * sizeof(T) + 16];
  T* fin = reinterpret_cast<T*>(fold_raw);
  const int lane = int(tid & 31), warp = int(tid >> 5);
  const int holders = int(count < nt ? count : nt);
  const int present = int(nt) - warp * 32 < 32 ? int(nt) - warp * 32 : 32;
  int valid = holders - warp * 32;
  valid = valid < 0 ? 0 : (valid > 32 ? 32 : valid);
  r = warp_fold(r, lane, valid, present, merge);
  if (lane == 0 && valid > 0) fin[warp] = r;
  __syncthreads();
  T acc = fin[0];
  if (tid == 0)
    for (int w = 1; w * 32 < holders; ++w) acc = merge(acc, fin[w]);
  __syncthreads();
  return acc;
}

// A WorkGroup reducer's fold: add the loop's partials of this run in index
// order (tile, then warp) and fold the result into the reducer's cell.  The
// cell is mapped host memory; the runs of one group fold in stream order.
template <class K>
__device__ void wg_fold(const void* parts, unsigned count, void* cell_v) {
  using V = typename K::V;
  static_assert(sizeof(V) <= 24, "reducer value larger than a WorkGroup cell");
  auto merge = [](V a, V b) { return K::merge(a, b); };
  const V r = fold_partials(static_cast<const V*>(parts), count, merge);
  if (lin_tid() == 0) {
    unsigned char* cell = static_cast<unsigned char*>(cell_v);
    volatile unsigned* has = reinterpret_cast<volatile unsigned*>(cell + 28);
    V acc = r;
    if (*has != 0u) {
      V prev;
      memcpy(&prev, cell, sizeof(V));
      acc = merge(prev, r);
    }
    memcpy(cell, &acc, sizeof(V));
    __threadfence_system();
    *has = 1u;
  }
}
// Stream-ordered pool of the current device for the C++ layer's per-launch
// device memory (reducer partials, IndexSet tables).  Its release threshold
// is unbounded: the device's default pool returns freed memory at every
// synchronisation, and re-mapping it cost ~100 us per call on GB300.
inline cudaMemPool_t launch_pool() {
  static std::atomic<cudaMemPool_t> pools[kMaxDevices] = {};
  static std::mutex mu;
  const int dev = current_device_index();
  cudaMemPool_t p = pools[dev].load(std::memory_order_acquire);
  if (!p) {
    std::lock_guard<std::mutex> lk(mu);
    p = pools[dev].load(std::memory_order_relaxed);
    if (!p) {
      cudaMemPoolProps props{};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      check_cuda(cudaMemPoolCreate(&p, &props), "launch memory pool");
      uint64_t keep = ~uint64_t(0);
      check_cuda(cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep), "launch memory pool");
      pools[dev].store(p, std::memory_order_release);
    }
  }
  return p;
}
inline void* launch_alloc(size_t bytes, cudaStream_t s, const char* what) {
  void* p = nullptr;
  check_cuda(cudaMallocFromPoolAsync(&p, bytes, launch_pool(), s), what);
  return p;
}

// A reducer result cell: 32 bytes of mapped pinned host memory.  The last
// block of the launch stores the result through `dev`; the host reads
// `host` after synchronising the stream, with no copy.
struct ResultCell {
  void* host = nullptr;
  void* dev = nullptr;
};
struct CellPool {
  std::mutex mu;
  std::vector<ResultCell> free;
};
inline CellPool& cell_pool() {
  static CellPool* pool = new CellPool;  // never destroyed: cells may be read until exit
  return *pool;
}
inline ResultCell acquire_cell() {
  CellPool& pool = cell_pool();
  std::lock_guard<std::mutex> lk(pool.mu);
  if (pool.free.empty()) {
    constexpr size_t kCells = 256, kCell = 32;
    void* h = nullptr;
    check_cuda(cudaHostAlloc(&h, kCells * kCell, cudaHostAllocMapped | cudaHostAllocPortable), "reducer result cells");
    void* d = nullptr;
    check_cuda(cudaHostGetDevicePointer(&d, h, 0), "reducer result cells");
    for (size_t i = kCells; i-- > 0;)
      pool.free.push_back(ResultCell{static_cast<char*>(h) + i * kCell, static_cast<char*>(d) + i * kCell});
  }
  const ResultCell c = pool.free.back();
  pool.free.pop_back();
  return c;
}
inline void release_cell(const ResultCell& c) {
  if (!c.host) return;
  CellPool& pool = cell_pool();
  std::lock_guard<std::mutex> lk(pool.mu);
  pool.free.push_back(c);
}

// Memory behind one launch's reducer slot.
struct SlotMem {
  void* block = nullptr;  // partials and ticket (launch pool)
  ResultCell cell;        // the result
};
template <class T>
inline T read_cell(const ResultCell& c) {
  static_assert(sizeof(T) <= 32, "reducer value larger than a result cell");
  T v;
  std::memcpy(&v, c.host, sizeof(T));
  return v;
}

// Allocate one launch's slot on the stream: partials and ticket in device
// memory, the result in a mapped host cell.
template <class T>
inline DevSlot<T> alloc_slot(unsigned grid, cudaStream_t s, SlotMem* mem) {
  const size_t pbytes = ((size_t(grid) * sizeof(T) + 255) / 256) * 256;
  mem->block = launch_alloc(pbytes + 256, s, "reducer slot");
  char* b = static_cast<char*>(mem->block);
  check_cuda(cudaMemsetAsync(b + pbytes, 0, sizeof(unsigned), s), "reducer ticket");
  mem->cell = acquire_cell();
  return DevSlot<T>{reinterpret_cast<T*>(b), reinterpret_cast<unsigned*>(b + pbytes), static_cast<T*>(mem->cell.dev)};
}

// ---- ValLoc with lowest-index tie-break (device merges)
template <class T, class I>
struct VLoc {
  T val;
  I loc;
};

// Reducer kinds: how to combine values
template <class T>
struct SumK {
  using V = T;
  B200_HOST_DEVICE static V ident() { return T(0); }
  B200_HOST_DEVICE static V merge(V a, V b) { return a + b; }
  static V fold_init(V a, V b) { return a + b; }
};
template <class T>
struct MinK {
  using V = T;
  B200_HOST_DEVICE static V ident() { return operators::limits<T>::max(); }
  B200_HOST_DEVICE static V merge(V a, V b) { return (b < a) ? b : a; }
  static V fold_init(V a, V b) { return (b < a) ? b : a; }
};
template <class T>
struct MaxK {
  using V = T;
  B200_HOST_DEVICE static V ident() { return operators::limits<T>::min(); }
  B200_HOST_DEVICE static V merge(V a, V b) { return (a < b) ? b : a; }
  static V fold_init(V a, V b) { return (a < b) ? b : a; }
};
template <class T>
struct OrK {
  using V = T;
  B200_HOST_DEVICE static V ident() { return T(0); }
  B200_HOST_DEVICE static V merge(V a, V b) { return a | b; }
  static V fold_init(V a, V b) { return a | b; }
};
template <class T>
struct AndK {
  using V = T;
  B200_HOST_DEVICE static V ident() { return T(~T(0)); }
  B200_HOST_DEVICE static V merge(V a, V b) { return a & b; }
  static V fold_init(V a, V b) { return a & b; }
};
template <class T, class I, bool MIN>
struct LocK {
  using V = VLoc<T, I>;
  B200_HOST_DEVICE static V ident() {
    return V{MIN ? operators::limits<T>::max() : operators::limits<T>::min(), I(-1)};
  }
  // device merges: strictly better value wins, equal values keep the
  // lowest location -- the order a sequential loop would have produced
  B200_HOST_DEVICE static V merge(V a, V b) {
    const bool better = MIN ? (b.val < a.val) : (a.val < b.val);
    if (better || (b.val == a.val && b.loc < a.loc && !(a.loc == I(-1)))) return b;
    return a;
  }
  // folding a launch result into the reducer's value: the earlier value
  // wins ties (operators::minimum / maximum, util/Operators.hpp:555-591)
  static V fold_init(V a, V b) { return (MIN ? (b.val < a.val) : (a.val < b.val)) ? b : a; }
};

// Device-capturable reducer.  The user's object (original) keeps the init
// value and the list of launch results still to fold; the launch copy made
// inside forall_impl gets a fresh device slot; the per-thread device copy
// accumulates privately and its destructor runs the block + grid combine
// (reduce.hpp:1047-1124 restated with a last-block ticket).
template <class K>
class DevReducer {
 public:
  using V = typename K::V;

 protected:
  struct Pending {
    SlotMem mem;
    cudaStream_t stream;
  };
  struct Shared {
    V init;
    std::vector<Pending> pending;
    // The slot of the launch being copied: copying a __host__ __device__
    // lambda's closure copy-constructs its captures more than once, and
    // every such copy of one launch must share one slot.
    unsigned long long slot_launch = 0;
    DevSlot<V> slot{nullptr, nullptr, nullptr};
    // likewise for the WorkGroup capture of one enqueued loop
    unsigned long long slot_capture = 0;
    DevSlot<V> wg_slot{nullptr, nullptr, nullptr};
    // the WorkGroup accumulator cells this reducer folds at get()
    std::vector<unsigned char*> wg_cells;
    std::vector<std::shared_ptr<WgRegistry>> wg_regs;
  };
  Shared* shared_ = nullptr;
  bool original_ = false;
  bool launch_copy_ = false;
  bool owner_ = false;
  bool wg_ = false;  // a WorkGroup loop's copy: per-warp partials, folded after the run
  DevSlot<V> slot_{nullptr, nullptr, nullptr};
  mutable V val_;

  // The combine of a WorkGroup loop's reducer: each warp of a tile stores
  // its partial in its slot; the run's fold launch adds them (wg_fold).
  __device__ void wg_combine(V v) const;

 public:
  explicit DevReducer(V init) : shared_(new Shared{init, {}}), original_(true), val_(K::ident()) {}

  B200_HOST_DEVICE DevReducer(const DevReducer& o) : val_(K::ident()) {
#if defined(__CUDA_ARCH__)
    // per-thread copy of the launch copy: owns the combine
    slot_ = o.slot_;
    owner_ = o.launch_copy_;
    wg_ = o.wg_;
#else
    shared_ = o.shared_;
    LaunchCtx& c = ctx();
    WgCaptureCtx& w = wg_capture();
    if (w.active && !o.launch_copy_ && w.nslots == 0) {
      // an empty loop never runs: no slot, the reducer keeps its value
      slot_ = o.slot_;
      launch_copy_ = false;
    } else if (w.active && !o.launch_copy_) {
      if (shared_->slot_capture != w.capture_id) {
        static_assert(alignof(V) <= kWgSlotHeader, "reducer values are aligned to at most 16 bytes");
        const size_t pbytes = kWgSlotHeader + size_t(w.nslots) * sizeof(V);
        void* blk = nullptr;
        check_cuda(cudaMalloc(&blk, pbytes), "WorkGroup reducer slot");
        {
          std::lock_guard<std::mutex> g(w.reg->m);
          w.reg->blocks.push_back(blk);  // owned by the registry before anything else can throw
        }
        V* parts = reinterpret_cast<V*>(static_cast<char*>(blk) + kWgSlotHeader);
        unsigned char *cell_host = nullptr, *cell_dev = nullptr;
        w.reg->new_cell(&cell_host, &cell_dev);
        {
          std::lock_guard<std::mutex> g(w.reg->m);
          w.reg->folds.push_back(WgFold{parts, cell_dev, w.loop});
        }
        shared_->wg_slot = DevSlot<V>{parts, nullptr, reinterpret_cast<V*>(cell_dev)};
        shared_->wg_cells.push_back(cell_host);
        if (std::find(shared_->wg_regs.begin(), shared_->wg_regs.end(), w.reg) == shared_->wg_regs.end())
          shared_->wg_regs.push_back(w.reg);
        shared_->slot_capture = w.capture_id;
      }
      slot_ = shared_->wg_slot;
      wg_ = true;
      launch_copy_ = true;
    } else if (c.active && !o.launch_copy_) {
      if (shared_->slot_launch != c.launch_id) {
        SlotMem mem;
        shared_->slot = alloc_slot<V>(c.grid, c.stream, &mem);
        shared_->slot_launch = c.launch_id;
        shared_->pending.push_back(Pending{mem, c.stream});
      }
      slot_ = shared_->slot;
      launch_copy_ = true;
    } else {
      slot_ = o.slot_;
      launch_copy_ = o.launch_copy_;
      wg_ = o.wg_;
    }
#endif
  }
  DevReducer& operator=(const DevReducer&) = delete;

  B200_HOST_DEVICE ~DevReducer() {
#if defined(__CUDA_ARCH__)
    if (owner_) {
      if (wg_) wg_combine(val_);
      else grid_combine(slot_, val_, [](V a, V b) { return K::merge(a, b); });
    }
#else
    if (original_) {
      try {
        fold();
      } catch (...) {
      }
      delete shared_;
    }
#endif
  }

  B200_HOST_DEVICE void combine(const V& v) const { val_ = K::merge(val_, v); }

  // Fold the pending launch results into init, in launch order, then the
  // accumulator cells of WorkGroup loops that captured this reducer.  One
  // synchronisation per stream with pending launches or runs (other
  // streams are not waited for); the results are then read from their host
  // cells.
  V fold() const {
    if (!shared_) return V{};
    std::vector<Pending>& pend = shared_->pending;
    std::vector<cudaStream_t> waited;
    for (const Pending& p : pend) {
      if (std::find(waited.begin(), waited.end(), p.stream) != waited.end()) continue;
      check_cuda(cudaStreamSynchronize(p.stream), "reducer wait");
      waited.push_back(p.stream);
    }
    for (const Pending& p : pend) {
      shared_->init = K::fold_init(shared_->init, read_cell<V>(p.mem.cell));
      release_cell(p.mem.cell);
      if (p.mem.block) cudaFreeAsync(p.mem.block, p.stream);
    }
    pend.clear();
    for (const auto& r : shared_->wg_regs) r->wait_runs();
    for (unsigned char* c : shared_->wg_cells) {
      volatile unsigned* has = reinterpret_cast<volatile unsigned*>(c + 28);
      if (*has == 0u) continue;
      V v;
      std::memcpy(&v, c, sizeof(V));
      shared_->init = K::fold_init(shared_->init, v);
      *has = 0u;  // folded: the next run starts the cell afresh
    }
    return shared_->init;
  }
  void reset_value(V v) {
    fold();
    shared_->init = v;
  }
};

template <class K>
__device__ void DevReducer<K>::wg_combine(V v) const {
  // WorkGroup launches are 1-D with whole warps
  const int lane = int(threadIdx.x & 31);
  v = warp_fold(v, lane, 32, 32, [](V a, V b) { return K::merge(a, b); });
  if (lane == 0) {
    const long long slot = wg_warp_slots()[threadIdx.x >> 5];
    slot_.partials[slot] = v;
    if (slot == 0)  // once per run: the fold the run's fold launch calls
      *reinterpret_cast<wg_fold_fn*>(reinterpret_cast<char*>(slot_.partials) - kWgSlotHeader) = wg_fold<K>;
  }
}

}  // namespace detail
}  // namespace b200

// ------------------------------------------------------------- reducers
template <typename T>
class ReduceSum<b200_reduce, T> : public b200::detail::DevReducer<b200::detail::SumK<T>> {
  using B = b200::detail::DevReducer<b200::detail::SumK<T>>;

 public:
  explicit ReduceSum(T init = T(0)) : B(init) {}
  B200_HOST_DEVICE ReduceSum(const ReduceSum& o) : B(o) {}
  B200_HOST_DEVICE const ReduceSum& operator+=(T v) const { this->val_ += v; return *this; }
  T get() const { return this->fold(); }
  operator T() const { return get(); }
  void reset(T v) { this->reset_value(v); }
};
template <typename T>
class ReduceMin<b200_reduce, T> : public b200::detail::DevReducer<b200::detail::MinK<T>> {
  using B = b200::detail::DevReducer<b200::detail::MinK<T>>;

 public:
  explicit ReduceMin(T init = operators::limits<T>::max()) : B(init) {}
  B200_HOST_DEVICE ReduceMin(const ReduceMin& o) : B(o) {}
  B200_HOST_DEVICE const ReduceMin& min(T v) const { this->combine(v); return *this; }
  T get() const { return this->fold(); }
  operator T() const { return get(); }
  void reset(T v) { this->reset_value(v); }
};
template <typename T>
class ReduceMax<b200_reduce, T> : public b200::detail::DevReducer<b200::detail::MaxK<T>> {
  using B = b200::detail::DevReducer<b200::detail::MaxK<T>>;

 public:
  explicit ReduceMax(T init = operators::limits<T>::min()) : B(init) {}
  B200_HOST_DEVICE ReduceMax(const ReduceMax& o) : B(o) {}
  B200_HOST_DEVICE const ReduceMax& max(T v) const { this->combine(v); return *this; }
  T get() const { return this->fold(); }
  operator T() const { return get(); }
  void reset(T v) { this->reset_value(v); }
};
template <typename T>
class ReduceBitOr<b200_reduce, T> : public b200::detail::DevReducer<b200::detail::OrK<T>> {
  using B = b200::detail::DevReducer<b200::detail::OrK<T>>;

 public:
  explicit ReduceBitOr(T init = T(0)) : B(init) {}
  B200_HOST_DEVICE ReduceBitOr(const ReduceBitOr& o) : B(o) {}
  B200_HOST_DEVICE const ReduceBitOr& operator|=(T v) const { this->val_ |= v; return *this; }
  T get() const { return this->fold(); }
  operator T() const { return get(); }
  void reset(T v) { this->reset_value(v); }
};
template <typename T>
class ReduceBitAnd<b200_reduce, T> : public b200::detail::DevReducer<b200::detail::AndK<T>> {
  using B = b200::detail::DevReducer<b200::detail::AndK<T>>;

 public:
  explicit ReduceBitAnd(T init = T(~T(0))) : B(init) {}
  B200_HOST_DEVICE ReduceBitAnd(const ReduceBitAnd& o) : B(o) {}
  B200_HOST_DEVICE const ReduceBitAnd& operator&=(T v) const { this->val_ &= v; return *this; }
  T get() const { return this->fold(); }
  operator T() const { return get(); }
  void reset(T v) { this->reset_value(v); }
};
// MinLoc / MaxLoc: the first extreme (lowest location among equal values),
// and the init pair wins ties (pattern/detail/reduce.hpp:287-358).
template <typename T, typename I>
class ReduceMinLoc<b200_reduce, T, I>
    : public b200::detail::DevReducer<b200::detail::LocK<T, I, true>> {
  using K = b200::detail::LocK<T, I, true>;
  using B = b200::detail::DevReducer<K>;

 public:
  ReduceMinLoc(T init, I idx) : B(typename K::V{init, idx}) {}
  B200_HOST_DEVICE ReduceMinLoc(const ReduceMinLoc& o) : B(o) {}
  B200_HOST_DEVICE const ReduceMinLoc& minloc(T v, I l) const {
    if (v < this->val_.val || (v == this->val_.val && l < this->val_.loc)) this->val_ = {v, l};
    return *this;
  }
  T get() const { return this->fold().val; }
  I getLoc() const { return this->fold().loc; }
  operator T() const { return get(); }
  void reset(T v, I l) { this->reset_value(typename K::V{v, l}); }
};
template <typename T, typename I>
class ReduceMaxLoc<b200_reduce, T, I>
    : public b200::detail::DevReducer<b200::detail::LocK<T, I, false>> {
  using K = b200::detail::LocK<T, I, false>;
  using B = b200::detail::DevReducer<K>;

 public:
  ReduceMaxLoc(T init, I idx) : B(typename K::V{init, idx}) {}
  B200_HOST_DEVICE ReduceMaxLoc(const ReduceMaxLoc& o) : B(o) {}
  B200_HOST_DEVICE const ReduceMaxLoc& maxloc(T v, I l) const {
    if (this->val_.val < v || (v == this->val_.val && l < this->val_.loc)) this->val_ = {v, l};
    return *this;
  }
  T get() const { return this->fold().val; }
  I getLoc() const { return this->fold().loc; }
  operator T() const { return get(); }
  void reset(T v, I l) { this->reset_value(typename K::V{v, l}); }
};

// ------------------------------------------------------------- autotuner
// b200_exec<0> and b200_work<0> choose their launch shape (threads per
// block, elements per thread) on line.  The first calls of a kernel -- per
// device and per power-of-two size class for forall, per instantiated group
// for WorkGroup -- cycle through the candidate shapes, each call bracketed
// by a pair of CUDA events on its stream; once every candidate has
// kSamples timings, the shape with the least time per element serves every
// later call.  Every call does its whole work with the shape it is given,
// so tuning never repeats or skips a loop body; floating-point reductions
// may round differently from one shape to another until the choice is
// made.  Calls made while their stream is being captured into a graph are
// not timed (they take the best shape so far).  A fixed BLOCK > 0 is never
// tuned.
namespace b200 {
namespace tune {

struct Shape {
  int block;
  int items;
};
constexpr int kSamples = 3;
// forall: the 256-thread, one-element-per-thread shape first (the default
// until timings arrive)
constexpr Shape kForallShapes[] = {{256, 1}, {128, 1}, {128, 4}, {256, 4}, {256, 16},
                                   {512, 1}, {512, 4}, {1024, 1}, {1024, 4}};
// WorkGroup tiles of block x items elements
constexpr Shape kWorkShapes[] = {{256, 8}, {128, 4}, {128, 8}, {128, 16}, {128, 32}, {256, 4},
                                 {256, 16}, {256, 32}, {512, 2}, {512, 4}, {512, 8}, {512, 16}};

struct Report {
  std::string name;
  int device;
  int size_class;  // floor(log2(elements)) for forall, -1 for a WorkGroup
  bool settled;
  Shape best;
  int candidates;
  int timed_calls;
};

class Tuner {
 public:
  struct Ticket {
    int cand = 0;
    cudaEvent_t start = nullptr, stop = nullptr;
  };
  Tuner(std::string name, int device, int size_class, const Shape* shapes, int n)
      : name_(std::move(name)), device_(device), class_(size_class), shapes_(shapes, shapes + n),
        samples_(n), inflight_(n, 0) {}
  ~Tuner() {
    for (auto& p : pending_) {
      cudaEventDestroy(p.t.start);
      cudaEventDestroy(p.t.stop);
    }
    for (cudaEvent_t e : free_) cudaEventDestroy(e);
  }
  Tuner(const Tuner&) = delete;
  Tuner& operator=(const Tuner&) = delete;

  Shape shape(int cand) const { return shapes_[size_t(cand)]; }

  // The candidate for the next call, with its start event recorded when the
  // call is to be timed.
  Ticket begin(cudaStream_t s) {
    std::lock_guard<std::mutex> g(m_);
    harvest();
    Ticket t;
    if (best_ >= 0) {
      t.cand = best_;
      return t;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
      t.cand = best_so_far();
      return t;
    }
    const int n = int(shapes_.size());
    for (int k = 0; k < n; ++k) {
      const int c = (next_ + k) % n;
      if (int(samples_[size_t(c)].size()) + inflight_[size_t(c)] < kSamples) {
        next_ = (c + 1) % n;
        t.cand = c;
        t.start = event();
        t.stop = event();
        check_cuda(cudaEventRecord(t.start, s), "b200 tuner event");
        ++inflight_[size_t(c)];
        return t;
      }
    }
    t.cand = best_so_far();  // every candidate issued; timings still in flight
    return t;
  }
  // After the call's launches: record the stop event of a timed call.
  void end(Ticket& t, cudaStream_t s, long long work) {
    if (!t.start) return;
    std::lock_guard<std::mutex> g(m_);
    const cudaError_t e = cudaEventRecord(t.stop, s);
    if (e != cudaSuccess) {
      --inflight_[size_t(t.cand)];
      free_.push_back(t.start);
      free_.push_back(t.stop);
      check_cuda(e, "b200 tuner event");
    }
    pending_.push_back(Pending{t, work > 0 ? work : 1});
    ++timed_;
  }
  // A call that threw between begin and end.
  void abandon(Ticket& t) {
    if (!t.start) return;
    std::lock_guard<std::mutex> g(m_);
    --inflight_[size_t(t.cand)];
    free_.push_back(t.start);
    free_.push_back(t.stop);
  }
  Report report() {
    std::lock_guard<std::mutex> g(m_);
    harvest();
    const int b = best_ >= 0 ? best_ : best_so_far();
    return Report{name_, device_, class_, best_ >= 0, shapes_[size_t(b)], int(shapes_.size()), timed_};
  }

 private:
  struct Pending {
    Ticket t;
    long long work;
  };
  cudaEvent_t event() {
    if (!free_.empty()) {
      cudaEvent_t e = free_.back();
      free_.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    check_cuda(cudaEventCreate(&e), "b200 tuner event");
    return e;
  }
  // Collect the timings whose stop event has completed (never waits).
  void harvest() {
    for (size_t i = 0; i < pending_.size();) {
      Pending& p = pending_[i];
      const cudaError_t q = cudaEventQuery(p.t.stop);
      if (q == cudaErrorNotReady) {
        ++i;
        continue;
      }
      float ms = 0.f;
      if (q == cudaSuccess && cudaEventElapsedTime(&ms, p.t.start, p.t.stop) == cudaSuccess)
        samples_[size_t(p.t.cand)].push_back(double(ms) / double(p.work));
      else
        (void)cudaGetLastError();  // a failed timing is dropped; the call reported its own errors
      --inflight_[size_t(p.t.cand)];
      free_.push_back(p.t.start);
      free_.push_back(p.t.stop);
      pending_[i] = pending_.back();
      pending_.pop_back();
    }
    if (best_ >= 0) return;
    for (const auto& v : samples_)
      if (int(v.size()) < kSamples) return;
    best_ = best_so_far();
  }
  // The candidate with the least time per element among those timed (the
  // fastest of each candidate's samples), else the first.
  int best_so_far() const {
    int b = -1;
    double bt = 0.0;
    for (size_t c = 0; c < samples_.size(); ++c) {
      if (samples_[c].empty()) continue;
      const double t = *std::min_element(samples_[c].begin(), samples_[c].end());
      if (b < 0 || t < bt) {
        b = int(c);
        bt = t;
      }
    }
    return b < 0 ? 0 : b;
  }

  std::mutex m_;
  std::string name_;
  int device_, class_;
  std::vector<Shape> shapes_;
  std::vector<std::vector<double>> samples_;
  std::vector<int> inflight_;
  std::vector<Pending> pending_;
  std::vector<cudaEvent_t> free_;
  int best_ = -1, next_ = 0, timed_ = 0;
};

// Every tuner made so far, for reports.
struct Registry {
  std::mutex m;
  std::vector<std::weak_ptr<Tuner>> all;
};
inline Registry& registry() {
  static Registry* r = new Registry;  // outlives static tuners at exit
  return *r;
}
inline std::shared_ptr<Tuner> make_tuner(std::string name, int device, int size_class, const Shape* shapes,
                                         int n) {
  auto t = std::make_shared<Tuner>(std::move(name), device, size_class, shapes, n);
  Registry& r = registry();
  std::lock_guard<std::mutex> g(r.m);
  r.all.push_back(t);
  return t;
}
// The state of every live tuner: its candidates, timed calls and the shape
// it uses now (the chosen one once settled).
inline std::vector<Report> reports() {
  std::vector<std::shared_ptr<Tuner>> live;
  {
    Registry& r = registry();
    std::lock_guard<std::mutex> g(r.m);
    std::vector<std::weak_ptr<Tuner>> keep;
    for (auto& w : r.all)
      if (auto t = w.lock()) {
        live.push_back(t);
        keep.push_back(w);
      }
    r.all.swap(keep);
  }
  std::vector<Report> out;
  for (auto& t : live) out.push_back(t->report());
  return out;
}

inline int size_class(long long n) {
  int c = 0;
  while (c < 62 && (n >> (c + 1)) > 0) ++c;
  return c;
}
// The tuner of one forall kernel family (Tag) for this device and size.
template <class Tag>
inline Tuner& forall_tuner(const char* name, long long len) {
  static std::mutex m;
  static std::map<std::pair<int, int>, std::shared_ptr<Tuner>>* tab =
      new std::map<std::pair<int, int>, std::shared_ptr<Tuner>>;  // kept to exit
  const int dev = current_device_index(), cls = size_class(len);
  std::lock_guard<std::mutex> g(m);
  auto& t = (*tab)[{dev, cls}];
  if (!t) t = make_tuner(name, dev, cls, kForallShapes, int(sizeof(kForallShapes) / sizeof(kForallShapes[0])));
  return *t;
}

template <class F>
inline void with_block(int block, F&& f) {
  switch (block) {
    case 128: f(std::integral_constant<int, 128>{}); break;
    case 512: f(std::integral_constant<int, 512>{}); break;
    case 1024: f(std::integral_constant<int, 1024>{}); break;
    default: f(std::integral_constant<int, 256>{}); break;
  }
}

// Run launch(integral_constant<int, block>, items) with BLOCK's fixed shape
// (one element per thread up to the resident grid), or, for BLOCK == 0,
// with the shape that Tag's tuner gives this call.
template <int BLOCK, class Tag, class F>
inline void shaped_launch(const char* name, long long len, cudaStream_t s, F&& launch) {
  if constexpr (BLOCK > 0) {
    launch(std::integral_constant<int, BLOCK>{}, 1);
  } else {
    Tuner& t = forall_tuner<Tag>(name, len);
    Tuner::Ticket tk = t.begin(s);
    const Shape sh = t.shape(tk.cand);
    try {
      with_block(sh.block, [&](auto B) { launch(B, sh.items); });
    } catch (...) {
      t.abandon(tk);
      throw;
    }
    t.end(tk, s, len);
  }
}
template <int Family, class... Ts>
struct Tag {};

}  // namespace tune
}  // namespace b200

// ---------------------------------------------------------------- forall
namespace b200 {
namespace detail {

template <int BLOCK, class Body, class T>
__global__ void __launch_bounds__(BLOCK) forall_range_kernel(Body body_in, T begin, long long len) {
  Body body(body_in);  // per-thread copy: reducers privatise here
  const long long stride = (long long)gridDim.x * BLOCK;
  for (long long i = (long long)blockIdx.x * BLOCK + threadIdx.x; i < len; i += stride)
    body(T(begin + T(i)));
}
template <int BLOCK, class Body, class T>
__global__ void __launch_bounds__(BLOCK)
forall_stride_kernel(Body body_in, T begin, T step, long long len) {
  Body body(body_in);
  const long long stride = (long long)gridDim.x * BLOCK;
  for (long long i = (long long)blockIdx.x * BLOCK + threadIdx.x; i < len; i += stride)
    body(T(begin + T(i) * step));
}
template <int BLOCK, class Body, class T>
__global__ void __launch_bounds__(BLOCK) forall_list_kernel(Body body_in, const T* idx, long long len) {
  Body body(body_in);
  const long long stride = (long long)gridDim.x * BLOCK;
  for (long long i = (long long)blockIdx.x * BLOCK + threadIdx.x; i < len; i += stride) body(idx[i]);
}
// Every segment of an IndexSet in one launch, whatever the mix of range,
// strided and list segments: a table holds each segment's parameters, and
// a prefix of segment lengths maps the flat iteration k to (segment,
// offset).  Index k of a segment is base + k * step (a range has step 1);
// a list segment keeps the address of its indices in base and kListStep
// (no stride a segment can have) in step.  An IndexSet of range segments
// only keeps just the bases (8 bytes a segment instead of 16).
constexpr long long kListStep = -9223372036854775807LL - 1;  // the most negative long long
struct SegDesc {
  long long base;
  long long step;
};
// Largest s in [lo, nseg) with prefix[s] <= k, given prefix[lo] <= k < prefix[nseg].
__device__ inline int seg_search(const long long* __restrict__ prefix, int lo, int nseg, long long k) {
  int hi = nseg;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (prefix[mid] <= k) lo = mid;
    else hi = mid;
  }
  return lo;
}
// Block b runs a contiguous slice of the flat iterations; each thread
// finds the segment of its first iteration by binary search and follows
// its later ones (BLOCK apart) by walking forward a few segments, or by a
// search of the rest of the table when the walk gets long.
template <int BLOCK, bool RANGES, class Body, class T>
__global__ void __launch_bounds__(BLOCK)
forall_indexset_kernel(Body body_in, const void* descs, const long long* __restrict__ prefix, int nseg,
                       long long total) {
  // No early return: a captured reducer's combine (in the destructor of
  // `body`) holds block barriers, which every thread of a warp must reach
  // at the same point.
  Body body(body_in);
  const long long rows = (total + BLOCK - 1) / BLOCK;
  const long long per = (rows + gridDim.x - 1) / gridDim.x * BLOCK;  // iterations per block
  const long long b0 = (long long)blockIdx.x * per;
  const long long b1 = b0 + per < total ? b0 + per : total;
  long long k = b0 + threadIdx.x;
  int s = k < b1 ? seg_search(prefix, 0, nseg, k) : 0;
  long long lo = prefix[s], hi = prefix[s + 1];
  for (; k < b1; k += BLOCK) {
    if (k >= hi) {
      int steps = 0;
      do {
        ++s;
        lo = hi;
        hi = prefix[s + 1];
      } while (k >= hi && ++steps < 8);
      if (k >= hi) {
        s = seg_search(prefix, s, nseg, k);
        lo = prefix[s];
        hi = prefix[s + 1];
      }
    }
    const long long off = k - lo;
    if constexpr (RANGES) {
      body(T(static_cast<const long long*>(descs)[s] + off));
    } else {
      const SegDesc d = static_cast<const SegDesc*>(descs)[s];
      body(d.step == kListStep ? reinterpret_cast<const T*>(d.base)[off] : T(d.base + off * d.step));
    }
  }
}

// Minimal tuple usable in device code.
template <class... Ts>
struct DTuple;
template <>
struct DTuple<> {};
template <class T, class... Ts>
struct DTuple<T, Ts...> {
  T head;
  DTuple<Ts...> tail;
};
template <size_t I, class T, class... Ts>
B200_HOST_DEVICE auto& dget(DTuple<T, Ts...>& t) {
  if constexpr (I == 0) return t.head;
  else return dget<I - 1>(t.tail);
}
template <size_t I, class T, class... Ts>
B200_HOST_DEVICE const auto& dget(const DTuple<T, Ts...>& t) {
  if constexpr (I == 0) return t.head;
  else return dget<I - 1>(t.tail);
}

// Make the launch copy of the body with the context active, so captured
// b200 reducers get their device slots for this grid.
template <class Body>
struct LaunchCopy {
  Body body;
  static Body make(const Body& b, unsigned grid, cudaStream_t s) {
    LaunchCtx& c = ctx();
    c.active = true;
    c.grid = grid;
    c.stream = s;
    ++c.launch_id;
    try {
      Body copy(b);
      c.active = false;
      return copy;
    } catch (...) {
      c.active = false;
      throw;
    }
  }
};

template <bool Async>
inline void finish(const char* what) {
  check_cuda(cudaGetLastError(), what);
  if (!Async) wait();
}

// Host staging of small per-launch tables (IndexSet segment tables) in
// pinned memory, so that their copy to the device is a plain asynchronous
// DMA (a copy from pageable memory first stages through the driver).  A
// ring of four grow-only buffers per host thread; an event behind the last
// copy out of a buffer says when it may be rewritten, so a thread blocks
// only when four copies are still queued.
class PinnedStage {
 public:
  static constexpr int kSlots = 4;
  ~PinnedStage() {
    for (Slot& sl : slots_) {
      if (sl.done) cudaEventDestroy(sl.done);
      if (sl.p) cudaFreeHost(sl.p);
    }
  }
  // A buffer of at least `bytes` whose previous copy has completed.
  unsigned char* get(size_t bytes) {
    Slot& sl = slots_[next_];
    if (sl.pending) {
      check_cuda(cudaEventSynchronize(sl.done), "pinned staging");
      sl.pending = false;
    }
    if (bytes > sl.cap) {
      if (sl.p) cudaFreeHost(sl.p);
      sl.p = nullptr;
      sl.cap = 0;
      check_cuda(cudaHostAlloc(reinterpret_cast<void**>(&sl.p), bytes, cudaHostAllocDefault), "pinned staging");
      sl.cap = bytes;
    }
    return sl.p;
  }
  // After the copy out of the buffer get() returned was issued on stream s.
  void copied(cudaStream_t s) {
    Slot& sl = slots_[next_];
    if (!sl.done) check_cuda(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming), "pinned staging");
    check_cuda(cudaEventRecord(sl.done, s), "pinned staging");
    sl.pending = true;
    next_ = (next_ + 1) % kSlots;
  }

 private:
  struct Slot {
    unsigned char* p = nullptr;
    size_t cap = 0;
    cudaEvent_t done = nullptr;
    bool pending = false;
  };
  Slot slots_[kSlots];
  int next_ = 0;
};
inline PinnedStage& pinned_stage() {
  static thread_local PinnedStage st;
  return st;
}

// Layout of an IndexSet's table, the same on the host and the device: the
// segment descriptors (SegDesc, or the bases alone for RANGES; padded to
// 256 bytes), then the running lengths (nseg + 1 entries).  Returns the
// total bytes; *desc_bytes is the padded descriptor part.
template <bool RANGES>
inline size_t seg_table_bytes(int nseg, size_t* desc_bytes) {
  const size_t each = RANGES ? sizeof(long long) : sizeof(SegDesc);
  *desc_bytes = ((size_t(nseg) * each + 255) / 256) * 256;
  return *desc_bytes + (size_t(nseg) + 1) * sizeof(long long);
}

// One launch over the segments of an IndexSet whose table (built by the
// caller in the pinned stage buffer `host`) holds nseg descriptors and
// their running lengths: one copy to launch-pool memory on the b200
// stream, freed behind the launch.
template <int BLOCK, bool Async, bool RANGES, class T, class Body>
void indexset_launch(const unsigned char* host, int nseg, size_t desc_bytes, size_t bytes, long long total,
                     Body&& body) {
  using B = std::decay_t<Body>;
  if (total == 0) return;
  cudaStream_t s = stream();
  void* tbl = launch_alloc(bytes, s, "indexset table");
  check_cuda(cudaMemcpyAsync(tbl, host, bytes, cudaMemcpyHostToDevice, s), "indexset table");
  pinned_stage().copied(s);
  const void* d_desc = tbl;
  long long* d_prefix = reinterpret_cast<long long*>(static_cast<char*>(tbl) + desc_bytes);
  tune::shaped_launch<BLOCK, tune::Tag<3, B, T>>("forall indexset", total, s, [&](auto NB, int items) {
    auto k = forall_indexset_kernel<NB(), RANGES, B, T>;
    const unsigned g = grid_for<forall_indexset_kernel<NB(), RANGES, B, T>>(NB(), total, items);
    B lb = LaunchCopy<B>::make(body, g, s);
    k<<<g, NB(), 0, s>>>(lb, d_desc, d_prefix, nseg, total);
  });
  check_cuda(cudaGetLastError(), "b200 forall indexset");
  check_cuda(cudaFreeAsync(tbl, s), "indexset table");
  if (!Async) wait();
}

}  // namespace detail
}  // namespace b200

// --------------------------------------------------------- kernel names
// A RAJA::Name param on a b200 loop or launch opens an NVTX range of that
// name around the launch when built with RAJA_ENABLE_NVTX (as the CUDA
// back-end does, policy/cuda/params/kernel_name.hpp:33-70), and is kept as
// the thread's last kernel name either way.
namespace b200 {
inline const char*& last_kernel_name() {
  static thread_local const char* n = nullptr;
  return n;
}
class NameScope {
 public:
  explicit NameScope(const char* n) : on_(n != nullptr) {
    if (!on_) return;
    last_kernel_name() = n;
#if defined(RAJA_ENABLE_NVTX)
    nvtxRangePushA(n);
#endif
  }
  NameScope(NameScope&& o) noexcept : on_(o.on_) { o.on_ = false; }
  NameScope(const NameScope&) = delete;
  NameScope& operator=(const NameScope&) = delete;
  ~NameScope() {
#if defined(RAJA_ENABLE_NVTX)
    if (on_) nvtxRangePop();
#endif
  }

 private:
  bool on_;
};
}  // namespace b200
template <int BLOCK, bool Async>
b200::NameScope kernel_name_scope(const b200_exec<BLOCK, Async>&, const char* n) {
  return b200::NameScope(n);
}

#if defined(RAJA_COMPAT_FRONTEND)
// ------------------------------------------------------------ resources
// resources::Cuda for the b200 policies: a CUDA stream on one device, with
// the interface of camp's Cuda resource as RAJA uses it (allocate /
// deallocate / memcpy / memset in stream order, get_event, wait, wait_for;
// test/unit/resource/tests/*.hpp).  A default-constructed resource takes
// the next stream of a per-device pool of 16 (blocking streams, so work on
// the legacy default stream still orders with them); get_default() is the
// thread's current b200 stream (the legacy default stream unless changed);
// CudaFromStream wraps a stream the caller owns.  While a call runs on a
// resource, the b200 policies launch on its stream.
namespace resources {

class CudaEvent {
 public:
  explicit CudaEvent(cudaStream_t s) {
    cudaEvent_t e = nullptr;
    b200::check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
    ev_ = std::shared_ptr<CUevent_st>(e, [](cudaEvent_t x) { cudaEventDestroy(x); });
    b200::check_cuda(cudaEventRecord(e, s), "cudaEventRecord");
  }
  bool check() const { return cudaEventQuery(ev_.get()) == cudaSuccess; }
  void wait() const { b200::check_cuda(cudaEventSynchronize(ev_.get()), "cudaEventSynchronize"); }
  cudaEvent_t getCudaEvent_t() const { return ev_.get(); }

 private:
  std::shared_ptr<CUevent_st> ev_;
};

class Cuda {
 public:
  static constexpr int kPoolSize = 16;
  Cuda() : Cuda(-1) {}
  explicit Cuda(int group, int device = current_device()) : dev_(device) {
    static std::atomic<unsigned> next{0};
    const unsigned k = group >= 0 ? unsigned(group) % kPoolSize : next.fetch_add(1) % kPoolSize;
    s_ = pool(device)[k];
  }
  static Cuda get_default() { return CudaFromStream(b200::stream()); }
  static Cuda CudaFromStream(cudaStream_t s, int device = current_device()) {
    Cuda c(s, device);
    return c;
  }
  cudaStream_t get_stream() const { return s_; }
  int get_device() const { return dev_; }
  Platform get_platform() const { return Platform::cuda; }

  template <typename T>
  T* allocate(size_t n, MemoryAccess ma = MemoryAccess::Device) {
    void* p = nullptr;
    const size_t bytes = n * sizeof(T);
    if (ma == MemoryAccess::Pinned)
      b200::check_cuda(cudaMallocHost(&p, bytes), "resources::Cuda::allocate (pinned)");
    else if (ma == MemoryAccess::Managed)
      b200::check_cuda(cudaMallocManaged(&p, bytes), "resources::Cuda::allocate (managed)");
    else
      b200::check_cuda(cudaMalloc(&p, bytes), "resources::Cuda::allocate");
    return static_cast<T*>(p);
  }
  void* calloc(size_t bytes, MemoryAccess ma = MemoryAccess::Device) {
    void* p = allocate<char>(bytes, ma);
    memset(p, 0, bytes);
    return p;
  }
  // The kind of memory is read from the pointer, so a pointer from any of
  // the three kinds of allocate() is freed correctly.
  void deallocate(void* p, MemoryAccess = MemoryAccess::Unknown) {
    if (!p) return;
    cudaPointerAttributes a{};
    b200::check_cuda(cudaPointerGetAttributes(&a, p), "resources::Cuda::deallocate");
    if (a.type == cudaMemoryTypeHost)
      b200::check_cuda(cudaFreeHost(p), "cudaFreeHost");
    else
      b200::check_cuda(cudaFree(p), "cudaFree");
  }
  void memcpy(void* dst, const void* src, size_t bytes) {
    if (bytes) b200::check_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, s_), "resources::Cuda::memcpy");
  }
  void memset(void* p, int v, size_t bytes) {
    if (bytes) b200::check_cuda(cudaMemsetAsync(p, v, bytes, s_), "resources::Cuda::memset");
  }
  CudaEvent get_event() { return CudaEvent(s_); }
  Event get_event_erased() { return Event{CudaEvent(s_)}; }
  // Waits for the stream and reports device-side errors of the b200
  // kernels (bounded waits that gave up), like res.wait() + cudaErrchk.
  void wait() { b200::check(b200_stream_synchronize(s_), "resources::Cuda::wait"); }
  // A CUDA event becomes a stream dependency; any other event is waited
  // for on the host.
  void wait_for(Event* e) {
    if (const CudaEvent* ce = e->try_get<CudaEvent>())
      b200::check_cuda(cudaStreamWaitEvent(s_, ce->getCudaEvent_t(), 0), "cudaStreamWaitEvent");
    else
      e->wait();
  }
  friend bool operator==(const Cuda& a, const Cuda& b) { return a.s_ == b.s_ && a.dev_ == b.dev_; }
  friend bool operator!=(const Cuda& a, const Cuda& b) { return !(a == b); }

 private:
  Cuda(cudaStream_t s, int device) : s_(s), dev_(device) {}
  static int current_device() {
    int d = 0;
    b200::check_cuda(cudaGetDevice(&d), "cudaGetDevice");
    return d;
  }
  static const cudaStream_t* pool(int device) {
    static std::mutex mu;
    static std::vector<std::vector<cudaStream_t>> pools;
    std::lock_guard<std::mutex> lock(mu);
    if (int(pools.size()) <= device) pools.resize(device + 1);
    auto& p = pools[device];
    if (p.empty()) {
      int cur = 0;
      b200::check_cuda(cudaGetDevice(&cur), "cudaGetDevice");
      if (cur != device) b200::check_cuda(cudaSetDevice(device), "cudaSetDevice");
      p.resize(kPoolSize);
      for (auto& s : p) b200::check_cuda(cudaStreamCreate(&s), "cudaStreamCreate");
      if (cur != device) b200::check_cuda(cudaSetDevice(cur), "cudaSetDevice");
    }
    return p.data();
  }
  cudaStream_t s_ = nullptr;
  int dev_ = 0;
};

// Binding: the b200 policies read the thread's current stream; the guard
// sets it to the resource's stream and restores the previous one.
class StreamBinding {
 public:
  explicit StreamBinding(cudaStream_t s) : prev_(b200::stream()) { b200::stream() = s; }
  StreamBinding(StreamBinding&& o) noexcept : prev_(o.prev_), active_(o.active_) { o.active_ = false; }
  StreamBinding(const StreamBinding&) = delete;
  StreamBinding& operator=(const StreamBinding&) = delete;
  ~StreamBinding() {
    if (active_) b200::stream() = prev_;
  }

 private:
  cudaStream_t prev_;
  bool active_ = true;
};
inline StreamBinding bind_resource(Cuda& r) { return StreamBinding(r.get_stream()); }

template <>
struct is_resource<Cuda> : std::true_type {};
template <int BLOCK, bool Async>
struct get_resource<b200_exec<BLOCK, Async>> {
  using type = Cuda;
};
template <int BLOCK, bool Async>
struct get_resource<b200_work<BLOCK, Async>> {
  using type = Cuda;
};

}  // namespace resources

template <int BLOCK, bool Async, class Body, class T>
void forall_impl(b200_exec<BLOCK, Async>, const TypedRangeSegment<T>& r, Body&& body) {
  using B = std::decay_t<Body>;
  const long long len = (long long)stripIndexType(r.size());
  if (len <= 0) return;
  cudaStream_t s = b200::stream();
  b200::tune::shaped_launch<BLOCK, b200::tune::Tag<0, B, T>>("forall range", len, s, [&](auto NB, int items) {
    auto k = b200::detail::forall_range_kernel<NB(), B, T>;
    const unsigned g = b200::detail::grid_for<b200::detail::forall_range_kernel<NB(), B, T>>(NB(), len, items);
    B lb = b200::detail::LaunchCopy<B>::make(body, g, s);
    k<<<g, NB(), 0, s>>>(lb, r.b, len);
  });
  b200::detail::finish<Async>("b200 forall");
}
template <int BLOCK, bool Async, class Body, class T>
void forall_impl(b200_exec<BLOCK, Async>, const TypedRangeStrideSegment<T>& r, Body&& body) {
  using B = std::decay_t<Body>;
  const long long len = (long long)stripIndexType(r.size());
  if (len <= 0) return;
  cudaStream_t s = b200::stream();
  b200::tune::shaped_launch<BLOCK, b200::tune::Tag<1, B, T>>("forall strided", len, s, [&](auto NB, int items) {
    auto k = b200::detail::forall_stride_kernel<NB(), B, T>;
    const unsigned g = b200::detail::grid_for<b200::detail::forall_stride_kernel<NB(), B, T>>(NB(), len, items);
    B lb = b200::detail::LaunchCopy<B>::make(body, g, s);
    k<<<g, NB(), 0, s>>>(lb, r.b, r.s, len);
  });
  b200::detail::finish<Async>("b200 forall");
}
template <int BLOCK, bool Async, class Body, class T>
void forall_impl(b200_exec<BLOCK, Async>, const TypedListSegment<T>& l, Body&& body) {
  using B = std::decay_t<Body>;
  const long long len = (long long)l.size();
  if (len <= 0) return;
  cudaStream_t s = b200::stream();
  b200::tune::shaped_launch<BLOCK, b200::tune::Tag<2, B, T>>("forall list", len, s, [&](auto NB, int items) {
    auto k = b200::detail::forall_list_kernel<NB(), B, T>;
    const unsigned g = b200::detail::grid_for<b200::detail::forall_list_kernel<NB(), B, T>>(NB(), len, items);
    B lb = b200::detail::LaunchCopy<B>::make(body, g, s);
    k<<<g, NB(), 0, s>>>(lb, l.data, len);
  });
  b200::detail::finish<Async>("b200 forall");
}
// IndexSet: one launch covers every segment, whatever the mix of range,
// strided and list segments (the reference launches each segment
// separately, policy/cuda/forall.hpp:675-706).  Segments with zero length
// take no iterations; the segment table lives in launch-pool memory for the
// duration of the launch.
namespace b200 {
namespace detail {
template <class T, class Seg>
inline bool seg_desc(const Seg& g, SegDesc* d, long long* len) {
  using G = std::decay_t<Seg>;
  if constexpr (std::is_same<G, TypedRangeSegment<T>>::value) {
    *len = (long long)stripIndexType(g.size());
    *d = SegDesc{(long long)g.b, 1};
    return true;
  } else if constexpr (std::is_same<G, TypedRangeStrideSegment<T>>::value) {
    *len = (long long)stripIndexType(g.size());
    *d = SegDesc{(long long)g.b, *len > 1 ? (long long)g.s : 1};
    return true;
  } else if constexpr (std::is_same<G, TypedListSegment<T>>::value) {
    *len = (long long)g.size();
    *d = SegDesc{(long long)reinterpret_cast<intptr_t>(g.data), kListStep};
    return true;
  } else {
    return false;  // another segment type: run per segment
  }
}
}  // namespace detail
}  // namespace b200

template <int BLOCK, bool Async, class Body, class... Segs>
void forall_impl(b200_exec<BLOCK, Async> pol, const TypedIndexSet<Segs...>& is, Body&& body) {
  using T = typename TypedIndexSet<Segs...>::value_type;
  const auto& segs = is.segments();
  const int nseg = int(segs.size());
  if (nseg == 0) return;
  constexpr bool kRanges = (std::is_same<Segs, TypedRangeSegment<T>>::value && ...);
  size_t db = 0;
  const size_t bytes = b200::detail::seg_table_bytes<kRanges>(nseg, &db);
  unsigned char* h = b200::detail::pinned_stage().get(bytes);
  long long* prefix = reinterpret_cast<long long*>(h + db);
  long long acc = 0;
  prefix[0] = 0;
  if constexpr (kRanges) {
    auto* base = reinterpret_cast<long long*>(h);
    for (int i = 0; i < nseg; ++i) {
      std::visit([&](const auto& g) {
        base[i] = (long long)g.b;
        acc += (long long)stripIndexType(g.size());
      }, segs[i]);
      prefix[i + 1] = acc;
    }
  } else {
    auto* desc = reinterpret_cast<b200::detail::SegDesc*>(h);
    bool table_ok = true;
    for (int i = 0; i < nseg && table_ok; ++i) {
      long long len = 0;
      table_ok = std::visit([&](const auto& g) { return b200::detail::seg_desc<T>(g, &desc[i], &len); }, segs[i]);
      acc += len;
      prefix[i + 1] = acc;
    }
    if (!table_ok) {
      for (const auto& v : segs) std::visit([&](const auto& g) { forall_impl(pol, g, body); }, v);
      return;
    }
  }
  b200::detail::indexset_launch<BLOCK, Async, kRanges, T>(h, nseg, db, bytes, acc, std::forward<Body>(body));
}

// ------------------------------------------------------ forall with params
namespace b200 {
namespace detail {

// The K (kind) of an expt reducer param, from its operator.
template <class R>
struct ParamKind;
template <template <class, class, class> class Op, class T, class VOp>
struct ParamKind<expt::detail::Reducer<Op<T, T, T>, T, VOp>> {
  using type = typename std::conditional<
      std::is_same<Op<T, T, T>, operators::plus<T, T, T>>::value, SumK<T>,
      typename std::conditional<
          std::is_same<Op<T, T, T>, operators::minimum<T, T, T>>::value, MinK<T>,
          typename std::conditional<
              std::is_same<Op<T, T, T>, operators::maximum<T, T, T>>::value, MaxK<T>,
              typename std::conditional<std::is_same<Op<T, T, T>, operators::bit_or<T, T, T>>::value,
                                        OrK<T>, AndK<T>>::type>::type>::type>::type;
  static T to_target(typename type::V v) { return v; }
  static B200_HOST_DEVICE typename type::V from_valop(const VOp& v) { return v.val; }
};
template <class T, class I, class Op, class VOp>
struct ParamKind<expt::detail::ReducerLoc<T, I, Op, VOp>> {
  static constexpr bool is_min =
      std::is_same<Op, operators::minimum<expt::ValLoc<T, I>, expt::ValLoc<T, I>, expt::ValLoc<T, I>>>::value;
  using type = LocK<T, I, is_min>;
  static expt::ValLoc<T, I> to_target(typename type::V v) { return expt::ValLoc<T, I>(v.val, v.loc); }
  static B200_HOST_DEVICE typename type::V from_valop(const VOp& v) { return {v.val.val, v.val.loc}; }
};

template <class R, class VOp>
__device__ inline void combine_param(const DevSlot<typename ParamKind<R>::type::V>& slot, const VOp& v) {
  using K = typename ParamKind<R>::type;
  grid_combine(slot, ParamKind<R>::from_valop(v), [](typename K::V a, typename K::V b) { return K::merge(a, b); });
}

// Any segment kind: element i is RAJA::detail::seg_at(seg, i).
template <int BLOCK, class Body, class Seg, class... R, size_t... I>
__device__ inline void params_body(Body& body, const Seg& seg, long long len,
                                   const DTuple<DevSlot<typename ParamKind<R>::type::V>...>& slots,
                                   std::index_sequence<I...>) {
  DTuple<typename R::valop_type...> vals{};
  const long long stride = (long long)gridDim.x * BLOCK;
  for (long long i = (long long)blockIdx.x * BLOCK + threadIdx.x; i < len; i += stride)
    body(::RAJA::detail::seg_at(seg, Index_type(i)), dget<I>(vals)...);
  (combine_param<R>(dget<I>(slots), dget<I>(vals)), ...);
}

template <int BLOCK, class Body, class Seg, class... R>
__global__ void __launch_bounds__(BLOCK)
forall_params_kernel(Body body, Seg seg, long long len,
                     DTuple<DevSlot<typename ParamKind<R>::type::V>...> slots) {
  params_body<BLOCK, Body, Seg, R...>(body, seg, len, slots, std::index_sequence_for<R...>{});
}

}  // namespace detail
}  // namespace b200

// Wait for the launch on stream s and fold its results into the targets in
// parameter order: *target = op(*target, result).  One synchronisation
// covers the launch; the results (host cells, one per parameter in `mem`)
// and the status word (mapped host memory) are then read directly.
// Returns false, with the targets untouched, when a bounded device wait
// gave up; b200::wait() then reports it.
template <class... Red>
bool resolve_params(const b200::detail::SlotMem* mem, cudaStream_t s, Red&... reds) {
  const uint32_t* status = nullptr;
  b200::check(b200_status_word_address(&status), "b200 status word");
  b200::check_cuda(cudaStreamSynchronize(s), "param result");
  if (__atomic_load_n(status, __ATOMIC_ACQUIRE) != 0) return false;
  size_t i = 0;
  auto take = [&](auto& red) {
    using RK = b200::detail::ParamKind<std::decay_t<decltype(red)>>;
    red.combineTarget(RK::to_target(b200::detail::read_cell<typename RK::type::V>(mem[i++].cell)));
  };
  (take(reds), ...);
  return true;
}
// Return the slot memory of a finished launch: cells to their pool, device
// blocks to the launch pool in the stream's order.
inline void release_slots(const b200::detail::SlotMem* mem, size_t n, cudaStream_t s) {
  for (size_t i = 0; i < n; ++i) {
    b200::detail::release_cell(mem[i].cell);
    if (mem[i].block) cudaFreeAsync(mem[i].block, s);
  }
}

template <int BLOCK, bool Async, class Seg, class Body, class... Red,
          class = decltype(::RAJA::detail::seg_len(std::declval<const Seg&>()))>
void forall_params_impl(b200_exec<BLOCK, Async>, const Seg& r, Body&& body, Red&... reds) {
  using B = std::decay_t<Body>;
  using Slots = b200::detail::DTuple<b200::detail::DevSlot<typename b200::detail::ParamKind<Red>::type::V>...>;
  const long long len = (long long)::RAJA::detail::seg_len(r);
  cudaStream_t s = b200::stream();
  b200::detail::SlotMem mem[sizeof...(Red) + 1];
  b200::tune::shaped_launch<BLOCK, b200::tune::Tag<4, B, Seg, Red...>>(
      "forall params", len > 0 ? len : 1, s, [&](auto NB, int items) {
        auto k = b200::detail::forall_params_kernel<NB(), B, Seg, Red...>;
        const unsigned g = b200::detail::grid_for<b200::detail::forall_params_kernel<NB(), B, Seg, Red...>>(
            NB(), len > 0 ? len : 1, items);
        size_t bi = 0;
        Slots slots{b200::detail::alloc_slot<typename b200::detail::ParamKind<Red>::type::V>(g, s, &mem[bi++])...};
        k<<<g, NB(), 0, s>>>(body, r, len, slots);
      });
  b200::check_cuda(cudaGetLastError(), "b200 forall params");
  // param_resolve waits for the kernel, as the reference does
  const bool ok = resolve_params(mem, s, reds...);
  release_slots(mem, sizeof...(Red), s);
  if (!ok) b200::wait();  // reports the device status and throws
}

// ---------------------------------------------------------------- launch
// RAJA::launch on the b200 policies (replaces cuda_launch_t and the CUDA
// loop policies, policy/cuda/launch.hpp): one kernel of Teams x Threads
// with LaunchParams::shared_mem_size bytes of dynamic shared memory; each
// loop policy maps a segment onto one kind of index:
//   b200_thread_{x,y,z}_{direct,loop}   threadIdx   (team-local)
//   b200_block_{x,y,z}_{direct,loop}    blockIdx
//   b200_global_{x,y,z}_{direct,loop}   blockIdx * blockDim + threadIdx
//   b200_flatten_block_threads_{xy,xyz}_{direct,loop}
//                                       threads of a team numbered x-first
// "direct" runs index i on the i-th position if i < length; "loop" strides
// by the number of positions.  The *_direct_unchecked names of the
// reference map to the checked direct forms (same results whenever the
// unchecked form is valid).  A host-compiled loop body runs sequentially.
template <bool Async = false, int NUM_THREADS = 0>
struct b200_launch_t {};
template <bool Async, int NUM_THREADS>
b200::NameScope kernel_name_scope(const b200_launch_t<Async, NUM_THREADS>&, const char* n) {
  return b200::NameScope(n);
}

template <int KIND, int D, bool LOOP>
struct b200_loop_pol {};
namespace b200 {
namespace launch {
enum Kind { kThread = 0, kBlock = 1, kGlobal = 2, kFlatThreads = 3 };
struct Pos {
  Index_type id;  // this thread's position
  Index_type n;   // number of positions
};
__device__ inline unsigned tid3(int d) { return d == 0 ? threadIdx.x : (d == 1 ? threadIdx.y : threadIdx.z); }
__device__ inline unsigned tdim3(int d) { return d == 0 ? blockDim.x : (d == 1 ? blockDim.y : blockDim.z); }
__device__ inline unsigned bid3(int d) { return d == 0 ? blockIdx.x : (d == 1 ? blockIdx.y : blockIdx.z); }
__device__ inline unsigned bdim3(int d) { return d == 0 ? gridDim.x : (d == 1 ? gridDim.y : gridDim.z); }
template <int KIND, int D>
__device__ inline Pos pos() {
  if constexpr (KIND == kThread) {
    return {Index_type(tid3(D)), Index_type(tdim3(D))};
  } else if constexpr (KIND == kBlock) {
    return {Index_type(bid3(D)), Index_type(bdim3(D))};
  } else if constexpr (KIND == kGlobal) {
    return {Index_type(bid3(D)) * tdim3(D) + tid3(D), Index_type(bdim3(D)) * tdim3(D)};
  } else {
    static_assert(D == 2 || D == 3, "flattened threads over xy or xyz");
    const Index_type xy = Index_type(threadIdx.x) + Index_type(blockDim.x) * threadIdx.y;
    if constexpr (D == 2) return {xy, Index_type(blockDim.x) * blockDim.y};
    else return {xy + Index_type(blockDim.x) * blockDim.y * threadIdx.z,
                 Index_type(blockDim.x) * blockDim.y * blockDim.z};
  }
}
}  // namespace launch
}  // namespace b200

#define RAJA_B200_LOOP_POLS(NAME, KIND, D)                                \
  using b200_##NAME##_direct = b200_loop_pol<KIND, D, false>;            \
  using b200_##NAME##_direct_unchecked = b200_loop_pol<KIND, D, false>;  \
  using b200_##NAME##_loop = b200_loop_pol<KIND, D, true>;
RAJA_B200_LOOP_POLS(thread_x, 0, 0)
RAJA_B200_LOOP_POLS(thread_y, 0, 1)
RAJA_B200_LOOP_POLS(thread_z, 0, 2)
RAJA_B200_LOOP_POLS(block_x, 1, 0)
RAJA_B200_LOOP_POLS(block_y, 1, 1)
RAJA_B200_LOOP_POLS(block_z, 1, 2)
RAJA_B200_LOOP_POLS(global_x, 2, 0)
RAJA_B200_LOOP_POLS(global_y, 2, 1)
RAJA_B200_LOOP_POLS(global_z, 2, 2)
RAJA_B200_LOOP_POLS(flatten_block_threads_xy, 3, 2)
RAJA_B200_LOOP_POLS(flatten_block_threads_xyz, 3, 3)
#undef RAJA_B200_LOOP_POLS
using b200_global_thread_x = b200_global_x_direct;
using b200_global_thread_y = b200_global_y_direct;
using b200_global_thread_z = b200_global_z_direct;

template <int KIND, int D, bool LOOP, typename SEGMENT>
struct LoopExecute<b200_loop_pol<KIND, D, LOOP>, SEGMENT> {
  template <typename BODY>
  B200_HOST_DEVICE static void exec(const LaunchContext& ctx, const SEGMENT& seg, const BODY& body) {
#if defined(__CUDA_ARCH__)
    (void)ctx;
    const b200::launch::Pos p = b200::launch::pos<KIND, D>();
    const Index_type n = detail::seg_len(seg);
    if (LOOP) {
      for (Index_type k = p.id; k < n; k += p.n) body(detail::seg_at(seg, k));
    } else if (p.id < n) {
      body(detail::seg_at(seg, p.id));
    }
#else
    LoopExecute<seq_exec, SEGMENT>::exec(ctx, seg, body);
#endif
  }
};
template <int KIND, int D, bool LOOP, typename SEGMENT>
struct LoopICountExecute<b200_loop_pol<KIND, D, LOOP>, SEGMENT> {
  template <typename BODY>
  B200_HOST_DEVICE static void exec(const LaunchContext& ctx, const SEGMENT& seg, const BODY& body) {
#if defined(__CUDA_ARCH__)
    (void)ctx;
    using I = std::decay_t<decltype(detail::seg_at(seg, 0))>;
    const b200::launch::Pos p = b200::launch::pos<KIND, D>();
    const Index_type n = detail::seg_len(seg);
    if (LOOP) {
      for (Index_type k = p.id; k < n; k += p.n) body(detail::seg_at(seg, k), I(k));
    } else if (p.id < n) {
      body(detail::seg_at(seg, p.id), I(p.id));
    }
#else
    LoopICountExecute<seq_exec, SEGMENT>::exec(ctx, seg, body);
#endif
  }
};
template <int KIND, int D, bool LOOP, typename SEGMENT>
struct TileExecute<b200_loop_pol<KIND, D, LOOP>, SEGMENT> {
  template <typename TILE_T, typename BODY>
  B200_HOST_DEVICE static void exec(const LaunchContext& ctx, TILE_T ts, const SEGMENT& seg, const BODY& body) {
#if defined(__CUDA_ARCH__)
    (void)ctx;
    const b200::launch::Pos p = b200::launch::pos<KIND, D>();
    const Index_type t = Index_type(ts), nt = (detail::seg_len(seg) + t - 1) / t;
    if (LOOP) {
      for (Index_type k = p.id; k < nt; k += p.n) body(detail::seg_tile(seg, t, k));
    } else if (p.id < nt) {
      body(detail::seg_tile(seg, t, p.id));
    }
#else
    TileExecute<seq_exec, SEGMENT>::exec(ctx, ts, seg, body);
#endif
  }
};
template <int KIND, int D, bool LOOP, typename SEGMENT>
struct TileTCountExecute<b200_loop_pol<KIND, D, LOOP>, SEGMENT> {
  template <typename TILE_T, typename BODY>
  B200_HOST_DEVICE static void exec(const LaunchContext& ctx, TILE_T ts, const SEGMENT& seg, const BODY& body) {
#if defined(__CUDA_ARCH__)
    (void)ctx;
    using I = std::decay_t<decltype(detail::seg_at(seg, 0))>;
    const b200::launch::Pos p = b200::launch::pos<KIND, D>();
    const Index_type t = Index_type(ts), nt = (detail::seg_len(seg) + t - 1) / t;
    if (LOOP) {
      for (Index_type k = p.id; k < nt; k += p.n) body(detail::seg_tile(seg, t, k), I(k));
    } else if (p.id < nt) {
      body(detail::seg_tile(seg, t, p.id), I(p.id));
    }
#else
    TileTCountExecute<seq_exec, SEGMENT>::exec(ctx, ts, seg, body);
#endif
  }
};

namespace b200 {
namespace detail {
// Every launch kernel names the dynamic shared memory the same way.
#define RAJA_B200_LAUNCH_SMEM extern __shared__ __align__(16) unsigned char b200_launch_smem[]

template <class Body>
__global__ void launch_kernel(Body body_in) {
  RAJA_B200_LAUNCH_SMEM;
  Body body(body_in);  // per-thread copy: captured reducers privatise here
  LaunchContext ctx;
  ctx.shared_mem_ptr = b200_launch_smem;
  body(ctx);
}
template <int NT, class Body>
__global__ void __launch_bounds__(NT) launch_kernel_nt(Body body_in) {
  RAJA_B200_LAUNCH_SMEM;
  Body body(body_in);
  LaunchContext ctx;
  ctx.shared_mem_ptr = b200_launch_smem;
  body(ctx);
}
template <class Body, class... R, size_t... I>
__device__ inline void launch_params_body(Body& body, const DTuple<DevSlot<typename ParamKind<R>::type::V>...>& slots,
                                          std::index_sequence<I...>) {
  RAJA_B200_LAUNCH_SMEM;
  LaunchContext ctx;
  ctx.shared_mem_ptr = b200_launch_smem;
  DTuple<typename R::valop_type...> vals{};
  body(ctx, dget<I>(vals)...);
  (combine_param<R>(dget<I>(slots), dget<I>(vals)), ...);
}
template <int NT, class Body, class... R>
__global__ void __launch_bounds__(NT > 0 ? NT : 1024)
launch_params_kernel(Body body_in, DTuple<DevSlot<typename ParamKind<R>::type::V>...> slots) {
  Body body(body_in);
  launch_params_body<Body, R...>(body, slots, std::index_sequence_for<R...>{});
}
#undef RAJA_B200_LAUNCH_SMEM

struct LaunchShape {
  dim3 grid, block;
  size_t smem;
  unsigned blocks;
  bool empty;
};
template <int NT, class Kernel>
inline LaunchShape launch_shape(const LaunchParams& p, Kernel k) {
  LaunchShape sh;
  const int* t = p.teams.value;
  const int* th = p.threads.value;
  sh.empty = t[0] <= 0 || t[1] <= 0 || t[2] <= 0 || th[0] <= 0 || th[1] <= 0 || th[2] <= 0;
  if (sh.empty) return sh;
  sh.grid = dim3(unsigned(t[0]), unsigned(t[1]), unsigned(t[2]));
  sh.block = dim3(unsigned(th[0]), unsigned(th[1]), unsigned(th[2]));
  const long long nthreads = (long long)th[0] * th[1] * th[2];
  if (nthreads > 1024 || (NT > 0 && nthreads > NT))
    throw std::runtime_error("b200 launch: " + std::to_string(nthreads) + " threads per team exceed the policy's " +
                             std::to_string(NT > 0 ? NT : 1024));
  sh.blocks = sh.grid.x * sh.grid.y * sh.grid.z;
  sh.smem = p.shared_mem_size ? p.shared_mem_size + kLaunchSharedSlack : 0;
  if (sh.smem > 48 * 1024)
    check_cuda(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sh.smem)),
               "b200 launch shared memory");
  return sh;
}
}  // namespace detail
}  // namespace b200

template <bool Async, int NT>
struct LaunchExecute<b200_launch_t<Async, NT>> {
  template <typename Res, typename Body>
  static void exec(Res, const LaunchParams& p, const Body& body) {
    using B = std::decay_t<Body>;
    void (*k)(B) = NT > 0 ? b200::detail::launch_kernel_nt<(NT > 0 ? NT : 1), B> : b200::detail::launch_kernel<B>;
    const b200::detail::LaunchShape sh = b200::detail::launch_shape<NT>(p, k);
    if (sh.empty) return;
    cudaStream_t s = b200::stream();
    B lb = b200::detail::LaunchCopy<B>::make(body, sh.blocks, s);
    k<<<sh.grid, sh.block, sh.smem, s>>>(lb);
    b200::detail::finish<Async>("b200 launch");
  }
  template <typename Res, typename Body, typename... Red>
  static void exec_params(Res, const LaunchParams& p, const Body& body, Red&... reds) {
    using B = std::decay_t<Body>;
    using Slots = b200::detail::DTuple<b200::detail::DevSlot<typename b200::detail::ParamKind<Red>::type::V>...>;
    auto k = b200::detail::launch_params_kernel<NT, B, Red...>;
    const b200::detail::LaunchShape sh = b200::detail::launch_shape<NT>(p, k);
    if (sh.empty) return;
    cudaStream_t s = b200::stream();
    b200::detail::SlotMem mem[sizeof...(Red) + 1];
    size_t bi = 0;
    Slots slots{b200::detail::alloc_slot<typename b200::detail::ParamKind<Red>::type::V>(sh.blocks, s, &mem[bi++])...};
    B lb = b200::detail::LaunchCopy<B>::make(body, sh.blocks, s);
    k<<<sh.grid, sh.block, sh.smem, s>>>(lb, slots);
    b200::check_cuda(cudaGetLastError(), "b200 launch params");
    // the targets are combined after the kernel, as in the reference
    const bool ok = resolve_params(mem, s, reds...);
    release_slots(mem, sizeof...(Red), s);
    if (!ok) b200::wait();  // reports the device status and throws
  }
};

namespace resources {
template <bool Async, int NT>
struct get_resource<b200_launch_t<Async, NT>> {
  using type = Cuda;
};
}  // namespace resources

#endif  // RAJA_COMPAT_FRONTEND

// ----------------------------------------------------------------- scans
namespace b200 {
namespace detail {
template <class F, class T>
constexpr int scan_op() {
  return std::is_same<F, operators::plus<T>>::value
             ? B200_OP_SUM
             : (std::is_same<F, operators::minimum<T>>::value
                    ? B200_OP_MIN
                    : (std::is_same<F, operators::maximum<T>>::value ? B200_OP_MAX : -1));
}
template <class T>
inline int scan_incl(const T* in, T* out, size_t n, int op, cudaStream_t s);
template <class T>
inline int scan_excl(const T* in, T* out, size_t n, int op, T init, cudaStream_t s);
#define B200_SCAN_BIND(SUF, T)                                                              \
  template <>                                                                               \
  inline int scan_incl<T>(const T* in, T* out, size_t n, int op, cudaStream_t s) {          \
    return b200_scan_inclusive_##SUF(in, out, n, op, s);                                    \
  }                                                                                         \
  template <>                                                                               \
  inline int scan_excl<T>(const T* in, T* out, size_t n, int op, T init, cudaStream_t s) {  \
    return b200_scan_exclusive_##SUF(in, out, n, op, init, s);                              \
  }
B200_SCAN_BIND(i32, int32_t)
B200_SCAN_BIND(i64, int64_t)
B200_SCAN_BIND(u32, uint32_t)
B200_SCAN_BIND(u64, uint64_t)
#undef B200_SCAN_BIND
// long long / unsigned long long: the 64-bit entry points (a distinct type
// from int64_t / uint64_t on LP64 hosts)
#define B200_SCAN_BIND_LL(SUF, T, C)                                                         \
  template <>                                                                                \
  inline int scan_incl<T>(const T* in, T* out, size_t n, int op, cudaStream_t s) {           \
    return b200_scan_inclusive_##SUF(reinterpret_cast<const C*>(in), reinterpret_cast<C*>(out), n, op, s); \
  }                                                                                          \
  template <>                                                                                \
  inline int scan_excl<T>(const T* in, T* out, size_t n, int op, T init, cudaStream_t s) {   \
    return b200_scan_exclusive_##SUF(reinterpret_cast<const C*>(in), reinterpret_cast<C*>(out), n, op, \
                                     C(init), s);                                            \
  }
static_assert(sizeof(long long) == 8, "64-bit long long");
#if !defined(_WIN32)
B200_SCAN_BIND_LL(i64, long long, int64_t)
B200_SCAN_BIND_LL(u64, unsigned long long, uint64_t)
#endif
#undef B200_SCAN_BIND_LL
template <>
inline int scan_incl<float>(const float* in, float* out, size_t n, int op, cudaStream_t s) {
  return b200_scan_inclusive_f32(in, out, n, op, B200_MODE_NAIVE, s);
}
template <>
inline int scan_incl<double>(const double* in, double* out, size_t n, int op, cudaStream_t s) {
  return b200_scan_inclusive_f64(in, out, n, op, B200_MODE_NAIVE, s);
}
template <>
inline int scan_excl<float>(const float* in, float* out, size_t n, int op, float init, cudaStream_t s) {
  return b200_scan_exclusive_f32(in, out, n, op, init, B200_MODE_NAIVE, s);
}
template <>
inline int scan_excl<double>(const double* in, double* out, size_t n, int op, double init,
                             cudaStream_t s) {
  return b200_scan_exclusive_f64(in, out, n, op, init, B200_MODE_NAIVE, s);
}
}  // namespace detail
}  // namespace b200

#if defined(RAJA_COMPAT_FRONTEND)
// policy/cuda/scan.hpp:141-235 (CUB DeviceScan) replaced by libb200prims.
template <int BLOCK, bool Async, typename T, typename F>
void scan_inclusive(b200_exec<BLOCK, Async>, const T* b, const T* e, T* out, F) {
  constexpr int op = b200::detail::scan_op<F, T>();
  static_assert(op >= 0, "b200 scans take operators::plus / minimum / maximum");
  b200::check(b200::detail::scan_incl<T>(b, out, size_t(e - b), op, b200::stream()), "b200 inclusive_scan");
  if (!Async) b200::wait();
}
template <int BLOCK, bool Async, typename T, typename F>
void scan_exclusive(b200_exec<BLOCK, Async>, const T* b, const T* e, T* out, F, T v) {
  constexpr int op = b200::detail::scan_op<F, T>();
  static_assert(op >= 0, "b200 scans take operators::plus / minimum / maximum");
  b200::check(b200::detail::scan_excl<T>(b, out, size_t(e - b), op, v, b200::stream()),
              "b200 exclusive_scan");
  if (!Async) b200::wait();
}

#endif  // RAJA_COMPAT_FRONTEND

// ----------------------------------------------------------------- sorts
// policy/cuda/sort.hpp:92-653 (CUB DeviceRadixSort) replaced by the
// stable radix sort of libb200prims; unstable forms forward to it.
namespace b200d {
template <class K>
inline int keys(K* k, size_t n, int desc, cudaStream_t s);
#define B200_SORT_BIND(SUF, K)                                                       \
  template <>                                                                        \
  inline int keys<K>(K * k, size_t n, int desc, cudaStream_t s) {                    \
    return b200_sort_keys_##SUF(k, n, desc, s);                                      \
  }
B200_SORT_BIND(u32, uint32_t)
B200_SORT_BIND(u64, uint64_t)
B200_SORT_BIND(i32, int32_t)
B200_SORT_BIND(i64, int64_t)
B200_SORT_BIND(f32, float)
B200_SORT_BIND(f64, double)
#undef B200_SORT_BIND
template <>
inline int keys<long long>(long long* k, size_t n, int desc, cudaStream_t s) {
  return b200_sort_keys_i64(reinterpret_cast<int64_t*>(k), n, desc, s);
}
template <>
inline int keys<unsigned long long>(unsigned long long* k, size_t n, int desc, cudaStream_t s) {
  return b200_sort_keys_u64(reinterpret_cast<uint64_t*>(k), n, desc, s);
}
// Values travel with their keys as bit patterns, so every trivially
// copyable 4- or 8-byte value type sorts through the 32- or 64-bit value
// entry of its key type.
template <class K, int VB>
inline int pairs_bits(K* k, void* v, size_t n, int desc, cudaStream_t s);
#define B200_PAIRS_BITS(K, SUF32, SUF64)                                                         \
  template <>                                                                                   \
  inline int pairs_bits<K, 4>(K * k, void* v, size_t n, int desc, cudaStream_t s) {             \
    return b200_sort_pairs_##SUF32(k, static_cast<int32_t*>(v), n, desc, s);                    \
  }                                                                                             \
  template <>                                                                                   \
  inline int pairs_bits<K, 8>(K * k, void* v, size_t n, int desc, cudaStream_t s) {             \
    return b200_sort_pairs_##SUF64(k, static_cast<int64_t*>(v), n, desc, s);                    \
  }
B200_PAIRS_BITS(uint32_t, u32_i32, u32_i64)
B200_PAIRS_BITS(int32_t, i32_i32, i32_i64)
B200_PAIRS_BITS(float, f32_i32, f32_i64)
B200_PAIRS_BITS(uint64_t, u64_i32, u64_i64)
B200_PAIRS_BITS(int64_t, i64_i32, i64_i64)
B200_PAIRS_BITS(double, f64_i32, f64_i64)
#undef B200_PAIRS_BITS
template <class K, class V>
inline int pairs(K* k, V* v, size_t n, int desc, cudaStream_t s) {
  static_assert(std::is_trivially_copyable<V>::value && (sizeof(V) == 4 || sizeof(V) == 8),
                "b200 sort_pairs takes trivially copyable 4- or 8-byte values");
  using KK = typename std::conditional<
      std::is_same<K, long long>::value, int64_t,
      typename std::conditional<std::is_same<K, unsigned long long>::value, uint64_t, K>::type>::type;
  return pairs_bits<KK, int(sizeof(V))>(reinterpret_cast<KK*>(k), static_cast<void*>(v), n, desc, s);
}
template <class C, class T>
constexpr int desc_of() {
  static_assert(std::is_same<C, operators::less<T>>::value || std::is_same<C, operators::greater<T>>::value,
                "b200 sorts take operators::less or operators::greater");
  return std::is_same<C, operators::greater<T>>::value ? 1 : 0;
}
}  // namespace b200d

#if defined(RAJA_COMPAT_FRONTEND)
template <int BLOCK, bool Async, typename T, typename C>
void sort_stable(b200_exec<BLOCK, Async>, T* b, T* e, C) {
  b200::check(b200d::keys<T>(b, size_t(e - b), b200d::desc_of<C, T>(), b200::stream()), "b200 sort");
  if (!Async) b200::wait();
}
template <int BLOCK, bool Async, typename T, typename C>
void sort_unstable(b200_exec<BLOCK, Async> p, T* b, T* e, C c) { sort_stable(p, b, e, c); }
template <int BLOCK, bool Async, typename K, typename V, typename C>
void sort_stable_pairs(b200_exec<BLOCK, Async>, K* kb, K* ke, V* vb, C) {
  b200::check(b200d::pairs<K, V>(kb, vb, size_t(ke - kb), b200d::desc_of<C, K>(), b200::stream()),
              "b200 sort_pairs");
  if (!Async) b200::wait();
}
template <int BLOCK, bool Async, typename K, typename V, typename C>
void sort_unstable_pairs(b200_exec<BLOCK, Async> p, K* kb, K* ke, V* vb, C c) {
  sort_stable_pairs(p, kb, ke, vb, c);
}

#endif  // RAJA_COMPAT_FRONTEND

// ------------------------------------------------------------- WorkGroup
// b200_work: enqueued loops (range segment + trivially copyable device
// lambda) are kept as (function pointer, body bytes, range).  The unordered
// runner executes every loop in one persistent launch over fixed-size
// tiles of all loops (load-balanced whatever the lengths); the ordered
// runners launch the loops one after another, as the reference's ordered
// CUDA runner does (policy/cuda/WorkGroup/WorkRunner.hpp:38-162).
namespace b200 {
namespace detail {
using wg_fn = void (*)(const void* body, long long begin, long long lo, long long hi);

// One tile of one loop.  Every thread runs with its own copy of the body,
// so captured b200 reducers accumulate privately; the copies' destructors
// (all threads of the block, at the end of the tile) combine them.
template <class Body>
__device__ void wg_run(const void* body, long long begin, long long lo, long long hi) {
  const Body b(*static_cast<const Body*>(body));
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) b(Index_type(begin + i));
}
// Device address of wg_run<Body>, read once per loop-body type by a
// one-thread kernel (Dispatcher.hpp:43-48 does the same).
template <class Body>
__global__ void wg_get_fn(wg_fn* out) {
  *out = wg_run<Body>;
}
// The address is per device, so it is cached per device.
template <class Body>
inline wg_fn wg_fn_of() {
  static std::atomic<wg_fn> cache[kMaxDevices] = {};
  const int dev = current_device_index();
  wg_fn fp = cache[dev].load(std::memory_order_acquire);
  if (!fp) {
    wg_fn* d = nullptr;
    check_cuda(cudaMalloc(&d, sizeof(wg_fn)), "WorkPool dispatcher");
    wg_get_fn<Body><<<1, 1>>>(d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(&fp, d, sizeof(fp), cudaMemcpyDeviceToHost);
    cudaFree(d);
    check_cuda(e, "WorkPool dispatcher");
    cache[dev].store(fp, std::memory_order_release);
  }
  return fp;
}

struct WgLoop {
  wg_fn fn;
  long long begin;
  long long len;
  size_t body_off;
};
constexpr int kWgItems = 8;  // elements per thread of a fixed-BLOCK WorkGroup tile

// All loops in one launch over tiles of `tile` elements: prefix[l] is the
// first tile of loop l (prefix[nloops] the tile count), and block b runs
// tiles b, b + grid, ...; a tile finds its loop by binary search.  Nothing
// is shared between the warps of a block (each warp's reducer partials go
// to their own slot), so the kernel has no barrier.
// The loop bodies are reached through device function pointers, which
// makes the kernels take a full register budget unless it is capped: at
// 32 registers a thread, 2048 threads fit on an SM and twice as many
// elements are in flight as at the default 64.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, 2048 / BLOCK)
wg_kernel(const long long* prefix, int nloops, long long tile, const WgLoop* loops,
          const unsigned char* bodies) {
  static_assert(BLOCK % 32 == 0 && BLOCK <= 1024, "b200_work blocks are whole warps");
  long long* slots = wg_warp_slots();
  const int warp = int(threadIdx.x >> 5);
  const long long ntiles = prefix[nloops];
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    int lo = 0, hi = nloops;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (prefix[mid] <= t) lo = mid;
      else hi = mid;
    }
    const WgLoop lp = loops[lo];
    const long long k = t - prefix[lo];
    if ((threadIdx.x & 31) == 0) slots[warp] = k * (BLOCK / 32) + warp;
    const long long a = k * tile;
    lp.fn(bodies + lp.body_off, lp.begin, a, a + tile < lp.len ? a + tile : lp.len);
  }
}
// One loop per launch (the ordered runners): block b runs tile b.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, 2048 / BLOCK)
wg_one_kernel(const WgLoop* loops, int which, long long tile, const unsigned char* bodies) {
  static_assert(BLOCK % 32 == 0 && BLOCK <= 1024, "b200_work blocks are whole warps");
  const WgLoop lp = loops[which];
  const int warp = int(threadIdx.x >> 5);
  if ((threadIdx.x & 31) == 0) wg_warp_slots()[warp] = (long long)blockIdx.x * (BLOCK / 32) + warp;
  const long long lo = (long long)blockIdx.x * tile;
  const long long hi = lo + tile < lp.len ? lo + tile : lp.len;
  lp.fn(bodies + lp.body_off, lp.begin, lo, hi);
}
// The reducers' folds of a run, one block per (reducer, loop): the loop has
// prefix[l + 1] - prefix[l] tiles at the run's tile size, each with `warps`
// partials.
__global__ void __launch_bounds__(256)
wg_fold_kernel(const WgFold* folds, const long long* prefix, int warps) {
  const WgFold f = folds[blockIdx.x];
  const long long count = (prefix[f.loop + 1] - prefix[f.loop]) * warps;
  const wg_fold_fn fn = *reinterpret_cast<const wg_fold_fn*>(static_cast<const char*>(f.parts) - kWgSlotHeader);
  fn(f.parts, unsigned(count), f.cell);
}
// The tile shapes a b200_work<BLOCK> group runs with: BLOCK x kWgItems, or
// for BLOCK == 0 the tuner's candidates.
template <int BLOCK>
inline std::vector<tune::Shape> wg_shapes() {
  if constexpr (BLOCK > 0) {
    return {tune::Shape{BLOCK, kWgItems}};
  } else {
    return std::vector<tune::Shape>(std::begin(tune::kWorkShapes), std::end(tune::kWorkShapes));
  }
}
// Reducer partials a loop of `len` elements needs: one per (tile, warp),
// the most over the group's tile shapes.
template <int BLOCK>
inline long long wg_slots(long long len) {
  long long m = 0;
  for (const tune::Shape& sh : wg_shapes<BLOCK>()) {
    const long long tile = (long long)sh.block * sh.items;
    const long long n = (len + tile - 1) / tile * (sh.block / 32);
    if (n > m) m = n;
  }
  return m;
}

// The loops of one b200 WorkGroup: capture at enqueue, upload on the first
// run, one persistent launch per unordered run (or one launch per loop for
// the ordered runners).  Shared by RAJA's WorkGroup (through a
// detail::WorkRunner specialisation) and the compat front-end's.
enum WgOrder { kWgUnordered = 0, kWgOrdered = 1, kWgReverse = 2 };

template <int BLOCK>
class WgCore {
 public:
  WgCore() = default;
  WgCore(const WgCore&) = delete;
  WgCore& operator=(const WgCore&) = delete;
  // A moved-from core is empty with a fresh registry, ready for new loops.
  WgCore(WgCore&& o) noexcept { swap(o); }
  WgCore& operator=(WgCore&& o) noexcept {
    swap(o);
    return *this;
  }
  ~WgCore() { free_device(); }

  // Capture loop [begin, begin + len): the body is copied once here, with
  // the capture context active so that captured b200 reducers take a slot
  // of this loop in the registry, and its bytes move to device memory at
  // the first run.
  template <typename Body>
  void enqueue(long long begin, long long len, const Body& body) {
    static_assert(std::is_copy_constructible<Body>::value, "b200_work loop bodies are copied");
    const wg_fn fp = wg_fn_of<Body>();
    WgCaptureCtx& w = wg_capture();
    w.active = true;
    w.reg = reg_;
    w.nslots = wg_slots<BLOCK>(len);
    w.loop = (long long)loops_.size();
    ++w.capture_id;
    alignas(Body) unsigned char raw[sizeof(Body)];
    try {
      ::new (raw) Body(body);  // the capture copy: stays as bytes, never destroyed
    } catch (...) {
      w.active = false;
      w.reg.reset();
      throw;
    }
    w.active = false;
    w.reg.reset();
    const size_t off = (bytes_.size() + 15) / 16 * 16;
    bytes_.resize(off + sizeof(Body));
    std::memcpy(bytes_.data() + off, raw, sizeof(Body));
    loops_.push_back(WgLoop{fp, begin, len, off});
    uploaded_ = false;
  }
  void reserve(size_t n, size_t bytes) {
    loops_.reserve(n);
    bytes_.reserve(bytes);
  }
  size_t num_loops() const { return loops_.size(); }

  // Launch every loop on stream s (uploading the loops the first time).
  void run(cudaStream_t s, WgOrder order) {
    if (loops_.empty()) return;
    if (!uploaded_) upload();
    reg_->order_after_runs(s);
    char* d = static_cast<char*>(dev_);
    auto* loops = reinterpret_cast<const WgLoop*>(d + loops_off_);
    auto* bodies = reinterpret_cast<const unsigned char*>(d + bodies_off_);
    // the tile shape of this run: the fixed one, or the tuner's
    tune::Tuner::Ticket tk;
    if (tuner_) tk = tuner_->begin(s);
    const size_t si = size_t(tk.cand);
    const tune::Shape sh = shapes_[si];
    const long long tile = (long long)sh.block * sh.items;
    auto* prefix = reinterpret_cast<const long long*>(d + prefix_off_[si]);
    const int nloops = int(loops_.size());
    try {
      tune::with_block(sh.block, [&](auto NB) {
        if (order == kWgUnordered) {
          if (ntiles_[si] > 0) {
            auto k = wg_kernel<NB()>;
            const unsigned g = grid_for<wg_kernel<NB()>>(NB(), ntiles_[si] * NB());
            k<<<g, NB(), 0, s>>>(prefix, nloops, tile, loops, bodies);
          }
        } else {
          // one launch per loop, in (reverse) enqueue order: block b runs tile b
          auto k = wg_one_kernel<NB()>;
          for (int i = 0; i < nloops; ++i) {
            const int which = order == kWgReverse ? nloops - 1 - i : i;
            const long long nt = (loops_[size_t(which)].len + tile - 1) / tile;
            if (nt > 0) k<<<unsigned(nt), NB(), 0, s>>>(loops, which, tile, bodies);
          }
        }
        // the captured reducers' partials of this run, into their cells
        if (nfolds_ > 0)
          wg_fold_kernel<<<unsigned(nfolds_), 256, 0, s>>>(reinterpret_cast<const WgFold*>(d + folds_off_),
                                                           prefix, NB() / 32);
      });
      check_cuda(cudaGetLastError(), "WorkGroup run");
    } catch (...) {
      if (tuner_) tuner_->abandon(tk);
      throw;
    }
    if (tuner_) tuner_->end(tk, s, elements_);
    // reducers captured by the loops read their cells after this run
    reg_->ran_on(s);
  }

  // The tuner's state for b200_work<0> (candidates, timed runs, the shape
  // in use); a fixed BLOCK reports its one shape as settled.
  tune::Report tuning() const {
    if (tuner_) return tuner_->report();
    const std::vector<tune::Shape> sh = wg_shapes<BLOCK>();
    return tune::Report{"WorkGroup", -1, -1, true, sh[0], 1, 0};
  }

  // Forget the loops and free their device storage (reducers keep the
  // registry, and with it their cells, alive).
  void clear() {
    free_device();
    loops_.clear();
    bytes_.clear();
    {
      std::lock_guard<std::mutex> g(reg_->m);
      reg_->folds.clear();
    }
    uploaded_ = false;
    tuner_.reset();
  }

 private:
  void swap(WgCore& o) noexcept {
    std::swap(loops_, o.loops_);
    std::swap(bytes_, o.bytes_);
    std::swap(reg_, o.reg_);
    std::swap(dev_, o.dev_);
    std::swap(uploaded_, o.uploaded_);
    std::swap(loops_off_, o.loops_off_);
    std::swap(bodies_off_, o.bodies_off_);
    std::swap(folds_off_, o.folds_off_);
    std::swap(nfolds_, o.nfolds_);
    std::swap(elements_, o.elements_);
    std::swap(shapes_, o.shapes_);
    std::swap(prefix_off_, o.prefix_off_);
    std::swap(ntiles_, o.ntiles_);
    std::swap(tuner_, o.tuner_);
  }
  void free_device() {
    if (dev_) cudaFree(dev_);
    dev_ = nullptr;
  }
  // Loops, bodies, the reducers' fold entries and, per tile shape, the
  // loops' first tiles, in one device allocation.
  void upload() {
    free_device();
    shapes_ = wg_shapes<BLOCK>();
    auto round = [](size_t b) { return (b + 255) / 256 * 256; };
    std::vector<long long> prefix;
    prefix_off_.clear();
    ntiles_.clear();
    elements_ = 0;
    for (const auto& l : loops_) elements_ += l.len;
    const size_t off = round(loops_.size() * sizeof(WgLoop));
    for (const tune::Shape& sh : shapes_) {
      const long long tile = (long long)sh.block * sh.items;
      const size_t first = prefix.size();
      long long acc = 0;
      for (const auto& l : loops_) {
        prefix.push_back(acc);
        acc += (l.len + tile - 1) / tile;
      }
      prefix.push_back(acc);
      prefix_off_.push_back(off + first * sizeof(long long));
      ntiles_.push_back(acc);
    }
    std::vector<WgFold> folds;
    {
      std::lock_guard<std::mutex> g(reg_->m);
      folds = reg_->folds;
    }
    nfolds_ = folds.size();
    loops_off_ = 0;
    bodies_off_ = round(off + prefix.size() * sizeof(long long));
    folds_off_ = round(bodies_off_ + bytes_.size());
    check_cuda(cudaMalloc(&dev_, folds_off_ + folds.size() * sizeof(WgFold) + 16), "WorkGroup storage");
    char* d = static_cast<char*>(dev_);
    check_cuda(cudaMemcpy(d + loops_off_, loops_.data(), loops_.size() * sizeof(WgLoop), cudaMemcpyHostToDevice),
               "WorkGroup loops");
    check_cuda(cudaMemcpy(d + off, prefix.data(), prefix.size() * sizeof(long long), cudaMemcpyHostToDevice),
               "WorkGroup tiles");
    if (!bytes_.empty())
      check_cuda(cudaMemcpy(d + bodies_off_, bytes_.data(), bytes_.size(), cudaMemcpyHostToDevice),
                 "WorkGroup bodies");
    if (!folds.empty())
      check_cuda(cudaMemcpy(d + folds_off_, folds.data(), folds.size() * sizeof(WgFold), cudaMemcpyHostToDevice),
                 "WorkGroup reducer folds");
    tuner_.reset();
    if (shapes_.size() > 1)
      tuner_ = tune::make_tuner("WorkGroup", current_device_index(), -1, shapes_.data(), int(shapes_.size()));
    uploaded_ = true;
  }

  std::vector<WgLoop> loops_;
  std::vector<unsigned char> bytes_;
  std::shared_ptr<WgRegistry> reg_ = std::make_shared<WgRegistry>();
  void* dev_ = nullptr;
  bool uploaded_ = false;
  size_t loops_off_ = 0, bodies_off_ = 0, folds_off_ = 0;
  size_t nfolds_ = 0;
  long long elements_ = 0;
  std::vector<tune::Shape> shapes_;
  std::vector<size_t> prefix_off_;  // per shape
  std::vector<long long> ntiles_;   // per shape
  std::shared_ptr<tune::Tuner> tuner_;
};

}  // namespace detail
}  // namespace b200

#if defined(RAJA_COMPAT_FRONTEND)
template <int BLOCK, bool Async, typename ORDER, typename STORAGE, typename DISPATCH, typename Index, typename Alloc>
class WorkGroup<WorkGroupPolicy<b200_work<BLOCK, Async>, ORDER, STORAGE, DISPATCH>, Index, xargs<>, Alloc>;

// The compat front-end's WorkPool / WorkGroup on b200_work: plugin hooks
// and resources around the shared core.
namespace b200 {
namespace detail {
template <class ORDER>
constexpr WgOrder wg_order() {
  return std::is_same<ORDER, unordered>::value ? kWgUnordered
                                               : (std::is_same<ORDER, reverse_ordered>::value ? kWgReverse : kWgOrdered);
}
}  // namespace detail
}  // namespace b200

template <int BLOCK, bool Async, typename ORDER, typename STORAGE, typename DISPATCH, typename Index, typename Alloc>
class WorkPool<WorkGroupPolicy<b200_work<BLOCK, Async>, ORDER, STORAGE, DISPATCH>, Index, xargs<>, Alloc> {
 public:
  using policy = WorkGroupPolicy<b200_work<BLOCK, Async>, ORDER, STORAGE, DISPATCH>;
  using group_type = WorkGroup<policy, Index, xargs<>, Alloc>;
  WorkPool() = default;
  template <typename A>
  explicit WorkPool(const A&) {}  // the allocator: device storage comes from cudaMalloc
  // Loop bodies are device lambdas whose captures are plain data or b200
  // reducers (captured reducers take a slot of this loop, so their per-loop
  // combine runs inside the group's launch).
  template <typename T, typename Body>
  void enqueue(TypedRangeSegment<T> seg, Body body) {
    // with plugins registered, the capture hooks bracket the body copy
    // (pattern/WorkGroup.hpp:287-296)
    const bool hooks = !util::PluginRegistry::empty();
    const util::PluginContext ctx(Platform::cuda, std::string());
    if (hooks) util::callPreCapturePlugins(ctx);
    m_core.enqueue((long long)seg.b, (long long)seg.size(), body);
    if (hooks) util::callPostCapturePlugins(ctx);
  }
  void reserve(size_t n, size_t bytes) { m_core.reserve(n, bytes); }
  size_t num_loops() const { return m_core.num_loops(); }
  group_type instantiate() { return group_type(std::move(m_core)); }

 private:
  b200::detail::WgCore<BLOCK> m_core;
};

template <int BLOCK, bool Async, typename ORDER, typename STORAGE, typename DISPATCH, typename Index, typename Alloc>
class WorkGroup<WorkGroupPolicy<b200_work<BLOCK, Async>, ORDER, STORAGE, DISPATCH>, Index, xargs<>, Alloc> {
 public:
  using policy = WorkGroupPolicy<b200_work<BLOCK, Async>, ORDER, STORAGE, DISPATCH>;
  WorkGroup() = default;
  explicit WorkGroup(b200::detail::WgCore<BLOCK>&& core) : m_core(std::move(core)) {}
  WorkGroup(const WorkGroup&) = delete;
  WorkGroup(WorkGroup&&) noexcept = default;
  WorkGroup& operator=(WorkGroup&&) noexcept = default;
  using resource_type = resources::Cuda;
  WorkSite<policy, Index, xargs<>, Alloc> run() { return run(resource_type::get_default()); }
  // The loops run on the resource's stream (pattern/WorkGroup.hpp:357-370).
  WorkSite<policy, Index, xargs<>, Alloc> run(resource_type r) {
    WorkSite<policy, Index, xargs<>, Alloc> site(r);
    if (m_core.num_loops() == 0) return site;
    auto bound = bind_resource(r);
    // with plugins registered, the launch hooks bracket the run
    // (pattern/WorkGroup.hpp:515-528)
    const bool hooks = !util::PluginRegistry::empty();
    const util::PluginContext ctx(Platform::cuda, std::string());
    if (hooks) util::callPreLaunchPlugins(ctx);
    m_core.run(b200::stream(), b200::detail::wg_order<ORDER>());
    if (!Async) b200::wait();
    if (hooks) util::callPostLaunchPlugins(ctx);
    return site;
  }
  void clear() {}
  b200::tune::Report tuning() const { return m_core.tuning(); }

 private:
  b200::detail::WgCore<BLOCK> m_core;
};

// ----------------------------------------------------------- synchronize
template <>
inline void synchronize<b200_synchronize>() {
  b200::check_cuda(cudaDeviceSynchronize(), "synchronize");
  b200::wait();
}

#endif  // RAJA_COMPAT_FRONTEND

// --------------------------------------------------------------- atomics
// b200_atomic: CUDA atomics in device code (min / max of floating types by
// compare-and-swap with the `<` rule), GCC __atomic builtins on the host.
// Each returns the value before the operation, as the reference's
// cuda_atomic does (policy/cuda/atomic.hpp).
namespace b200 {
namespace atom {
template <typename T>
using Word = std::conditional_t<sizeof(T) == 4, unsigned int, unsigned long long>;
template <typename T>
B200_HOST_DEVICE inline Word<T> bits(T v) {
  Word<T> w;
  memcpy(&w, &v, sizeof(T));
  return w;
}
template <typename T>
B200_HOST_DEVICE inline T from_bits(Word<T> w) {
  T v;
  memcpy(&v, &w, sizeof(T));
  return v;
}
// generic read-modify-write by compare-and-swap: new value = f(old)
template <typename T, typename F>
B200_HOST_DEVICE inline T rmw(T* acc, F f) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte atomics");
  Word<T>* p = reinterpret_cast<Word<T>*>(acc);
#ifdef __CUDA_ARCH__
  Word<T> cur = *reinterpret_cast<volatile Word<T>*>(p);
  while (true) {
    const Word<T> nv = bits<T>(f(from_bits<T>(cur)));
    const Word<T> prev = ::atomicCAS(p, cur, nv);
    if (prev == cur) return from_bits<T>(cur);
    cur = prev;
  }
#else
  Word<T> cur = __atomic_load_n(p, __ATOMIC_RELAXED);
  while (true) {
    const Word<T> nv = bits<T>(f(from_bits<T>(cur)));
    if (__atomic_compare_exchange_n(p, &cur, nv, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED))
      return from_bits<T>(cur);
  }
#endif
}
}  // namespace atom
}  // namespace b200

template <typename T>
B200_HOST_DEVICE inline T atomicLoad(b200_atomic, T* acc) {
  return b200::atom::rmw(acc, [](T o) { return o; });
}
template <typename T>
B200_HOST_DEVICE inline void atomicStore(b200_atomic, T* acc, T v) {
  b200::atom::rmw(acc, [v](T) { return v; });
}
template <typename T>
B200_HOST_DEVICE inline T atomicAdd(b200_atomic, T* acc, T v) {
#ifdef __CUDA_ARCH__
  if constexpr (std::is_same<T, int>::value || std::is_same<T, unsigned>::value ||
                std::is_same<T, unsigned long long>::value || std::is_same<T, float>::value ||
                std::is_same<T, double>::value)
    return ::atomicAdd(acc, v);
#endif
  return b200::atom::rmw(acc, [v](T o) { return T(o + v); });
}
template <typename T>
B200_HOST_DEVICE inline T atomicSub(b200_atomic, T* acc, T v) {
  return b200::atom::rmw(acc, [v](T o) { return T(o - v); });
}
template <typename T>
B200_HOST_DEVICE inline T atomicMin(b200_atomic, T* acc, T v) {
#ifdef __CUDA_ARCH__
  if constexpr (std::is_same<T, int>::value || std::is_same<T, unsigned>::value ||
                std::is_same<T, long long>::value || std::is_same<T, unsigned long long>::value)
    return ::atomicMin(acc, v);
#endif
  return b200::atom::rmw(acc, [v](T o) { return v < o ? v : o; });
}
template <typename T>
B200_HOST_DEVICE inline T atomicMax(b200_atomic, T* acc, T v) {
#ifdef __CUDA_ARCH__
  if constexpr (std::is_same<T, int>::value || std::is_same<T, unsigned>::value ||
                std::is_same<T, long long>::value || std::is_same<T, unsigned long long>::value)
    return ::atomicMax(acc, v);
#endif
  return b200::atom::rmw(acc, [v](T o) { return o < v ? v : o; });
}
template <typename T>
B200_HOST_DEVICE inline T atomicInc(b200_atomic, T* acc) {
  return atomicAdd(b200_atomic{}, acc, T(1));
}
template <typename T>
B200_HOST_DEVICE inline T atomicInc(b200_atomic, T* acc, T val) {
  return b200::atom::rmw(acc, [val](T o) { return val <= o ? T(0) : T(o + T(1)); });
}
template <typename T>
B200_HOST_DEVICE inline T atomicDec(b200_atomic, T* acc) {
  return atomicSub(b200_atomic{}, acc, T(1));
}
template <typename T>
B200_HOST_DEVICE inline T atomicDec(b200_atomic, T* acc, T val) {
  return b200::atom::rmw(acc, [val](T o) { return (o == T(0) || val < o) ? val : T(o - T(1)); });
}
template <typename T>
B200_HOST_DEVICE inline T atomicAnd(b200_atomic, T* acc, T v) {
  return b200::atom::rmw(acc, [v](T o) { return T(o & v); });
}
template <typename T>
B200_HOST_DEVICE inline T atomicOr(b200_atomic, T* acc, T v) {
  return b200::atom::rmw(acc, [v](T o) { return T(o | v); });
}
template <typename T>
B200_HOST_DEVICE inline T atomicXor(b200_atomic, T* acc, T v) {
  return b200::atom::rmw(acc, [v](T o) { return T(o ^ v); });
}
template <typename T>
B200_HOST_DEVICE inline T atomicExchange(b200_atomic, T* acc, T v) {
  return b200::atom::rmw(acc, [v](T) { return v; });
}
template <typename T>
B200_HOST_DEVICE inline T atomicCAS(b200_atomic, T* acc, T compare, T v) {
#ifdef __CUDA_ARCH__
  using W = b200::atom::Word<T>;
  return b200::atom::from_bits<T>(::atomicCAS(reinterpret_cast<W*>(acc), b200::atom::bits(compare),
                                              b200::atom::bits(v)));
#else
  auto w = b200::atom::bits(compare);
  __atomic_compare_exchange_n(reinterpret_cast<b200::atom::Word<T>*>(acc), &w,
                              b200::atom::bits(v), false, __ATOMIC_RELAXED, __ATOMIC_RELAXED);
  return b200::atom::from_bits<T>(w);
#endif
}

// ---------------------------------------------------------- multi reduce
// MultiReduce{Sum,Min,Max,BitOr,BitAnd}<b200_multi_reduce, T>: the bins
// live in device memory, initialised to the op's identity; device code
// combines into them with b200_atomic operations (the reference's
// cuda_multi_reduce_atomic global path, policy/cuda/multi_reduce.hpp:
// 208-470); get() waits for the b200 stream, reads them back and folds
// them into the host-side init values.  Copies share the bins.  For binned
// reductions over arrays, the library's b200_multi_reduce_* entry points
// privatize the bins in shared memory.
namespace b200 {
namespace detail {
template <typename T, typename Op>
class DevMultiReduce {
 public:
  using value_type = T;
  DevMultiReduce(size_t num_bins, T init) { setup(std::vector<T>(num_bins, init)); }
  explicit DevMultiReduce(size_t num_bins) : DevMultiReduce(num_bins, Op::ident()) {}
  template <typename Container, typename = decltype(std::declval<const Container&>().begin())>
  explicit DevMultiReduce(const Container& c) {
    setup(std::vector<T>(c.begin(), c.end()));
  }
  // copies (the loop body's capture, on the host and on the device) share
  // the bins and own nothing
  B200_HOST_DEVICE DevMultiReduce(const DevMultiReduce& o)
      : st_(o.st_), dev_(o.dev_), n_(o.n_), owner_(false) {}
  DevMultiReduce& operator=(const DevMultiReduce&) = delete;
  B200_HOST_DEVICE ~DevMultiReduce() {
#if !defined(__CUDA_ARCH__)
    release();
#endif
  }
  size_t size() const { return n_; }
  T get(size_t bin) const {
    sync();
    return st_->host.at(bin);
  }
  template <typename Container>
  void get_all(Container& c) const {
    sync();
    size_t b = 0;
    for (auto& v : c) v = st_->host[b++];
  }
  void reset() { reset(n_, Op::ident()); }
  void reset(size_t num_bins, T init = Op::ident()) {
    release();
    setup(std::vector<T>(num_bins, init));
  }
  B200_HOST_DEVICE void combine(size_t bin, T v) const { Op::atomic(dev_ + bin, v); }

 private:
  struct State {
    std::vector<T> init, host;
    T* dev = nullptr;
  };
  void setup(std::vector<T> init) {
    n_ = init.size();
    st_ = new State();
    owner_ = true;
    check_cuda(cudaMalloc(&st_->dev, std::max<size_t>(n_, 1) * sizeof(T)), "multi reduce bins");
    dev_ = st_->dev;
    std::vector<T> id(n_, Op::ident());
    check_cuda(cudaMemcpy(dev_, id.data(), n_ * sizeof(T), cudaMemcpyHostToDevice), "multi reduce bins");
    st_->host = init;
    st_->init = std::move(init);
  }
  void release() {
    if (owner_ && st_) {
      cudaFree(st_->dev);
      delete st_;
    }
    st_ = nullptr;
    owner_ = false;
  }
  void sync() const {
    wait();
    std::vector<T> d(n_);
    check_cuda(cudaMemcpy(d.data(), dev_, n_ * sizeof(T), cudaMemcpyDeviceToHost), "multi reduce get");
    for (size_t b = 0; b < n_; ++b) {
      T v = st_->init[b];
      Op::fold(v, d[b]);
      st_->host[b] = v;
    }
  }
  State* st_ = nullptr;
  T* dev_ = nullptr;
  size_t n_ = 0;
  bool owner_ = false;
};

template <typename T> struct DMrSum {
  static T ident() { return T(0); }
  B200_HOST_DEVICE static void atomic(T* p, T v) { atomicAdd(b200_atomic{}, p, v); }
  static void fold(T& a, T v) { a += v; }
};
template <typename T> struct DMrMin {
  static T ident() { return operators::limits<T>::max(); }
  B200_HOST_DEVICE static void atomic(T* p, T v) { atomicMin(b200_atomic{}, p, v); }
  static void fold(T& a, T v) { if (v < a) a = v; }
};
template <typename T> struct DMrMax {
  static T ident() { return operators::limits<T>::min(); }
  B200_HOST_DEVICE static void atomic(T* p, T v) { atomicMax(b200_atomic{}, p, v); }
  static void fold(T& a, T v) { if (a < v) a = v; }
};
template <typename T> struct DMrOr {
  static T ident() { return T(0); }
  B200_HOST_DEVICE static void atomic(T* p, T v) { atomicOr(b200_atomic{}, p, v); }
  static void fold(T& a, T v) { a |= v; }
};
template <typename T> struct DMrAnd {
  static T ident() { return T(~T(0)); }
  B200_HOST_DEVICE static void atomic(T* p, T v) { atomicAnd(b200_atomic{}, p, v); }
  static void fold(T& a, T v) { a &= v; }
};
}  // namespace detail
}  // namespace b200

#define RAJA_B200_MULTI_REDUCER(CLS, OPK, METHOD)                                               \
  template <typename T>                                                                         \
  class CLS<b200_multi_reduce, T> : public b200::detail::DevMultiReduce<T, b200::detail::OPK<T>> { \
    using B = b200::detail::DevMultiReduce<T, b200::detail::OPK<T>>;                            \
                                                                                                \
   public:                                                                                      \
    using B::B;                                                                                 \
    struct reference {                                                                          \
      const B* mr;                                                                              \
      size_t bin;                                                                               \
      B200_HOST_DEVICE const reference& METHOD(T v) const {                                     \
        mr->combine(bin, v);                                                                    \
        return *this;                                                                           \
      }                                                                                         \
      T get() const { return mr->get(bin); }                                                    \
    };                                                                                          \
    B200_HOST_DEVICE reference operator[](size_t bin) const { return reference{this, bin}; }    \
  };
RAJA_B200_MULTI_REDUCER(MultiReduceSum, DMrSum, operator+=)
RAJA_B200_MULTI_REDUCER(MultiReduceMin, DMrMin, min)
RAJA_B200_MULTI_REDUCER(MultiReduceMax, DMrMax, max)
RAJA_B200_MULTI_REDUCER(MultiReduceBitOr, DMrOr, operator|=)
RAJA_B200_MULTI_REDUCER(MultiReduceBitAnd, DMrAnd, operator&=)
#undef RAJA_B200_MULTI_REDUCER

}  // namespace RAJA

#if !defined(RAJA_COMPAT_FRONTEND)
// an installed RAJA: the reference's own extension points
#include "RAJA_b200_extension_points.hpp"
#endif
