// Batched loops: WorkGroup-style fusion of many uneven loops into one
// persistent launch, segmented scans and segmented sorts over the same
// segment plan, and CUDA-graph helpers for repeated sweeps.
//
// Reference: WorkGroup runners (pattern/WorkGroup/WorkRunner.hpp:159-333)
// issue one forall launch per enqueued loop (ordered) or one launch with
// grid = (ceil(avg_len / BLOCK), num_loops) that grid-strides each loop over
// an average-sized x extent (policy/cuda/WorkGroup/WorkRunner.hpp:223-407),
// and the unordered runner does not support reducers (:323-329).  IndexSet
// segments are launched one by one (policy/cuda/forall.hpp:675-706), and
// RAJA has no segmented scan/sort: the composition is one scan or sort call
// per segment (pattern/scan.hpp, pattern/sort.hpp).
//
// GB300 design: a plan (built once, like WorkPool::instantiate) cuts every
// loop into fixed-size tiles and stores tile -> loop tables in device
// memory.  A persistent grid (SM count x resident blocks) walks the tiles;
// every tile has the same size (only each loop's last tile is short), so
// the load is balanced whatever the length distribution.  Per-loop
// reductions are fused: each warp keeps a compensated partial across the
// tiles of one loop and stores it when its block moves to the next loop;
// a second small launch adds each loop's warp partials in a fixed order,
// so the result is deterministic.  The tile size and block size are
// autotuned per plan by timing the candidates.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "b200_internal.cuh"

struct b200_batch_plan_s {
  int device = -1;
  int nloops = 0;
  int64_t total = 0;
  std::vector<int64_t> lens;       // host copy
  std::vector<int64_t> offsets;    // host prefix (nloops + 1)
  int64_t* d_lens = nullptr;
  int64_t* d_offsets = nullptr;
  // tiling (depends on the tile size)
  int tile = 0;
  int block = 0;
  int64_t ntiles = 0;
  int32_t* d_tile_loop = nullptr;  // ntiles
  int64_t* d_loop_tile0 = nullptr; // nloops + 1
  double* d_tile_part = nullptr;   // ntiles x 16 warp partials of the runs
  int variant = -1;                // autotuned kernel variant (-1: default)
  // segmented sort classification
  std::vector<int> big_segments;   // segments longer than the block sort
  int32_t* d_small = nullptr;      // ids of the small segments: the warp-sized ones first
  int nsmall = 0;
  int ntiny = 0;                   // small segments of at most SEG_WARP_CAP keys
  // long segments sorted together as (segment << 32 | key) in one 64-bit
  // sort (set when there are several and they are short enough)
  bool big_packed = false;
  int64_t big_total = 0;           // keys in the long segments
  int64_t* d_big_off = nullptr;    // nbig + 1 running lengths of the long segments
  int64_t* d_big_src = nullptr;    // nbig offsets of the long segments in the keys
  uint64_t* d_big_buf = nullptr;   // big_total packed keys
};

struct b200_graph_s {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace b200 {
namespace {

// ----------------------------------------------------- kernel variants
struct Variant {
  int block;
  int items;  // elements per thread per tile
};
constexpr Variant kVariants[] = {{256, 8}, {256, 16}, {512, 8}, {128, 16}, {256, 4}};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);
constexpr int kDefaultVariant = 0;

bool log_on() {
  const char* e = getenv("B200_LOG");
  return e && e[0] == '1';
}

// block reduction of doubles (fixed shape)
template <int BLOCK>
__device__ __forceinline__ double block_sum(double v, double* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = (lane < BLOCK / 32) ? sh[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  __syncthreads();
  return v;
}

// Body of one tile: y += a*x over [lo, hi) of one loop; returns the
// thread's compensated partial of the updated y.  When x and y share their
// offset from a 16-byte boundary (the loops of one flat array do), the tile
// runs as a scalar head of 0-3 elements up to that boundary, 16-byte
// vectors, and a scalar tail of 0-3 elements, so loops that start at any
// element offset, and each loop's short last tile, stay on the vector
// path.  Otherwise the tile runs scalar.
template <int BLOCK, int ITEMS>
__device__ __forceinline__ double tile_axpy_sum(float a, const float* __restrict__ x,
                                                float* __restrict__ y, int64_t lo, int64_t hi,
                                                bool comp) {
  float s = 0.f, c = 0.f;
  auto add = [&](float r) {
    if (comp) {
      float t, e2;
      two_sum(s, r, t, e2);
      s = t;
      c += e2;
    } else {
      s += r;
    }
  };
  const int tid = threadIdx.x;
  constexpr int VN = 4;
  const uintptr_t ax = reinterpret_cast<uintptr_t>(x + lo), ay = reinterpret_cast<uintptr_t>(y + lo);
  if ((((ax ^ ay) & 15) == 0) && ((ax & 3) == 0)) {
    const int64_t n = hi - lo;
    const int64_t h0 = int64_t(((16 - (ax & 15)) & 15) >> 2);  // elements before the boundary
    const int64_t nh = h0 < n ? h0 : n;
    const int64_t vb = lo + nh;                 // first vector element
    const int64_t nv = (hi - vb) / VN;          // whole vectors in the tile
    const int64_t tb = vb + nv * VN;            // first tail element
    float4 vx[ITEMS / VN], vy[ITEMS / VN];
#pragma unroll
    for (int j = 0; j < ITEMS / VN; ++j) {
      const int64_t v = int64_t(j) * BLOCK + tid;
      if (v < nv) {
        vx[j] = __ldcs(reinterpret_cast<const float4*>(x + vb + v * VN));
        vy[j] = __ldcs(reinterpret_cast<const float4*>(y + vb + v * VN));
      }
    }
    if (tid < nh) {
      const float r = y[lo + tid] + a * x[lo + tid];
      y[lo + tid] = r;
      add(r);
    }
#pragma unroll
    for (int j = 0; j < ITEMS / VN; ++j) {
      const int64_t v = int64_t(j) * BLOCK + tid;
      if (v < nv) {
        float4 r;
        r.x = vy[j].x + a * vx[j].x;
        r.y = vy[j].y + a * vx[j].y;
        r.z = vy[j].z + a * vx[j].z;
        r.w = vy[j].w + a * vx[j].w;
        __stcs(reinterpret_cast<float4*>(y + vb + v * VN), r);
        add(r.x);
        add(r.y);
        add(r.z);
        add(r.w);
      }
    }
    if (tid < hi - tb) {
      const float r = y[tb + tid] + a * x[tb + tid];
      y[tb + tid] = r;
      add(r);
    }
  } else {
    for (int64_t i = lo + tid; i < hi; i += BLOCK) {
      const float r = y[i] + a * x[i];
      y[i] = r;
      add(r);
    }
  }
  return double(s) + double(c);
}

// L2 prefetch of the whole 16-byte granules inside [b, e): never a byte
// outside the range.
__device__ __forceinline__ void prefetch_l2_inside(const float* b, const float* e) {
  const uintptr_t s = (reinterpret_cast<uintptr_t>(b) + 15) & ~uintptr_t(15);
  const uintptr_t f = reinterpret_cast<uintptr_t>(e) & ~uintptr_t(15);
  if (f > s) prefetch_l2_bulk(reinterpret_cast<const void*>(s), uint32_t(f - s));
}

// Warps per block of the largest batched variant: the run partials hold
// one slot per (tile, warp) of it.
constexpr int kMaxBatchWarps = 16;

// All loops in one launch.  Each block takes a contiguous run of the tile
// table (tiles are equal-sized, so the runs are balanced), prefetches the
// next tile's descriptor, and keeps its partial sum in registers across the
// tiles of one loop.  When the loop changes, each warp reduces its lanes'
// partials and stores them in the slot (first tile of the run, warp): no
// fences, tickets or block barriers inside the loop.  batched_fold_kernel
// then adds each loop's slots in run and warp order, so the sums are
// deterministic for a given tiling.
template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK)
batched_axpy_sum_kernel(const int32_t* __restrict__ tile_loop,
                        const int64_t* __restrict__ loop_tile0,
                        const int64_t* __restrict__ loop_len, int64_t ntiles, float a,
                        const float* const* __restrict__ xs, float* const* __restrict__ ys,
                        double* __restrict__ run_part, int comp) {
  constexpr int TILE = BLOCK * ITEMS;
  static_assert(BLOCK / 32 <= kMaxBatchWarps, "one run slot per warp");
  const int64_t per = (ntiles + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = int64_t(blockIdx.x) * per;
  const int64_t b1 = b0 + per < ntiles ? b0 + per : ntiles;
  if (b0 >= b1) return;                            // block-uniform
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  auto flush = [&](double v, int64_t r0) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) run_part[r0 * kMaxBatchWarps + warp] = v;
  };
  int cur = -1;                                    // loop of the running partial
  int64_t run0 = b0, t0 = 0, len = 0;
  const float* x = nullptr;
  float* y = nullptr;
  double acc = 0.0;
  int nxt = tile_loop[b0];
  for (int64_t t = b0; t < b1; ++t) {
    const int loop = nxt;
    if (t + 1 < b1) nxt = tile_loop[t + 1];         // one tile ahead
    if (loop != cur) {                             // block-uniform
      if (cur >= 0) flush(acc, run0);
      cur = loop;
      run0 = t;
      acc = 0.0;
      t0 = loop_tile0[loop];
      len = loop_len[loop];
      x = xs[loop];
      y = ys[loop];
    }
    const int64_t lo = (t - t0) * TILE;
    const int64_t hi = min(lo + TILE, len);
    if (threadIdx.x == 0 && t + 1 < b1 && nxt == loop) {
      // the block's next tile, same loop: into L2 while this one runs
      const int64_t hi2 = min(hi + TILE, len);
      prefetch_l2_inside(x + hi, x + hi2);
      prefetch_l2_inside(y + hi, y + hi2);
    }
    acc += tile_axpy_sum<BLOCK, ITEMS>(a, x, y, lo, hi, comp != 0);
  }
  flush(acc, run0);
}

// Each loop's sum from its run partials.  The loop's runs start at its
// first tile and at every block boundary (multiple of `per`, the tiles per
// block of the main launch) inside it; a run's slots are added in warp
// order.  A loop with no tile sums to 0.
__global__ void __launch_bounds__(256)
batched_fold_kernel(const int64_t* __restrict__ loop_tile0, int nloops, int64_t per, int warps,
                    const double* __restrict__ run_part, double* __restrict__ sums) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nloops) return;
  const int64_t T0 = loop_tile0[l], T1 = loop_tile0[l + 1];
  double q = 0.0;
  for (int64_t r0 = T0; r0 < T1; r0 = (r0 / per + 1) * per)
    for (int w = 0; w < warps; ++w) q += run_part[r0 * kMaxBatchWarps + w];
  sums[l] = q;
}

// One fused axpy + sum over a single loop (the per-loop launch that the
// ordered WorkGroup runner issues, with its reduction).
template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK)
loop_axpy_sum_kernel(float a, const float* __restrict__ x, float* __restrict__ y, int64_t n,
                     double* __restrict__ out, double* __restrict__ part,
                     uint32_t* __restrict__ ticket, int comp) {
  constexpr int TILE = BLOCK * ITEMS;
  __shared__ double sh[32];
  __shared__ bool last;
  double acc = 0.0;
  const int64_t ntiles = (n + TILE - 1) / TILE;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t lo = t * TILE;
    acc += tile_axpy_sum<BLOCK, ITEMS>(a, x, y, lo, min(lo + TILE, n), comp != 0);
  }
  acc = block_sum<BLOCK>(acc, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = acc;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double q = 0.0;
  for (int k = threadIdx.x; k < int(gridDim.x); k += BLOCK) q += __ldcg(part + k);
  q = block_sum<BLOCK>(q, sh);
  if (threadIdx.x == 0) {
    *out = q;
    *ticket = 0u;
  }
}

template <int BLOCK, int ITEMS>
int launch_batched(b200_batch_plan_s* p, float a, const float* const* xs, float* const* ys,
                   double* sums, int comp, cudaStream_t s) {
  static KernelSetup ks;
  DeviceProps props;
  B200_TRY(device_props(&props));
  int bps = 0;
  B200_TRY(kernel_setup(ks, props, batched_axpy_sum_kernel<BLOCK, ITEMS>, BLOCK, 0, &bps));
  int64_t grid = int64_t(props.sms) * bps;
  if (grid > p->ntiles) grid = p->ntiles;
  if (grid < 1) grid = 1;
  B200_LAUNCH("b200_batched_axpy_sum", (batched_axpy_sum_kernel<BLOCK, ITEMS>), unsigned(grid),
              BLOCK, 0, s, p->d_tile_loop, p->d_loop_tile0, p->d_lens, p->ntiles, a, xs, ys,
              p->d_tile_part, comp);
  const int64_t per = (p->ntiles + grid - 1) / grid;  // tiles per block, as the kernel splits them
  B200_LAUNCH("b200_batched_fold", batched_fold_kernel, unsigned((p->nloops + 255) / 256), 256, 0, s,
              p->d_loop_tile0, p->nloops, per, BLOCK / 32, p->d_tile_part, sums);
  return B200_OK;
}

int dispatch_batched(int v, b200_batch_plan_s* p, float a, const float* const* xs,
                     float* const* ys, double* sums, int comp, cudaStream_t s) {
  switch (v) {
    case 0: return launch_batched<256, 8>(p, a, xs, ys, sums, comp, s);
    case 1: return launch_batched<256, 16>(p, a, xs, ys, sums, comp, s);
    case 2: return launch_batched<512, 8>(p, a, xs, ys, sums, comp, s);
    case 3: return launch_batched<128, 16>(p, a, xs, ys, sums, comp, s);
    case 4: return launch_batched<256, 4>(p, a, xs, ys, sums, comp, s);
    default: return fail(B200_ERR_ARG, "bad batched variant %d", v);
  }
}

void free_tiling(b200_batch_plan_s* p) {
  cudaFree(p->d_tile_loop);
  cudaFree(p->d_loop_tile0);
  cudaFree(p->d_tile_part);
  p->d_tile_loop = nullptr;
  p->d_loop_tile0 = nullptr;
  p->d_tile_part = nullptr;
  p->ntiles = 0;
}

// (Re)build the tile tables for a tile size.
int build_tiling(b200_batch_plan_s* p, int tile) {
  if (p->tile == tile && p->d_tile_loop) return B200_OK;
  free_tiling(p);
  std::vector<int64_t> t0(p->nloops + 1, 0);
  for (int i = 0; i < p->nloops; ++i) t0[i + 1] = t0[i] + (p->lens[i] + tile - 1) / tile;
  const int64_t nt = t0[p->nloops];
  std::vector<int32_t> tl(size_t(std::max<int64_t>(nt, 1)), 0);
  for (int i = 0; i < p->nloops; ++i)
    for (int64_t k = t0[i]; k < t0[i + 1]; ++k) tl[k] = i;
  B200_CUDA(cudaMalloc(&p->d_tile_loop, tl.size() * sizeof(int32_t)));
  B200_CUDA(cudaMalloc(&p->d_loop_tile0, t0.size() * sizeof(int64_t)));
  B200_CUDA(cudaMalloc(&p->d_tile_part, tl.size() * kMaxBatchWarps * sizeof(double)));
  B200_CUDA(cudaMemcpy(p->d_tile_loop, tl.data(), tl.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  B200_CUDA(cudaMemcpy(p->d_loop_tile0, t0.data(), t0.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
  p->tile = tile;
  p->ntiles = nt;
  return B200_OK;
}

int check_plan(b200_batch_plan_s* p, const char* name) {
  if (!p) return fail(B200_ERR_ARG, "%s: null plan", name);
  int dev = 0;
  B200_CUDA(cudaGetDevice(&dev));
  if (dev != p->device) return fail(B200_ERR_ARG, "%s: plan belongs to device %d", name, p->device);
  return B200_OK;
}

// ------------------------------------------------------ segmented scan
// Inclusive / exclusive sum scan that restarts at every segment head.
// Element i's segment comes from a binary search of the first element a
// thread owns in the offsets, then a forward walk.  The carried value is
// (flag, sum): (f1,a) + (f2,b) = (f1|f2, f2 ? b : a+b).
constexpr int SSB = 256;      // threads
constexpr int SSI = 16;       // items per thread
constexpr int SST = SSB * SSI;

struct SegVal {
  uint32_t flag;
  int32_t v;
};
__device__ __forceinline__ SegVal seg_comb(SegVal a, SegVal b) {
  return {a.flag | b.flag, b.flag ? b.v : int32_t(uint32_t(a.v) + uint32_t(b.v))};
}

__device__ __forceinline__ int64_t seg_of(const int64_t* __restrict__ off, int nseg, int64_t i) {
  // largest s with off[s] <= i
  int lo = 0, hi = nseg;  // off[0] = 0 <= i < off[nseg]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= i) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ int pad32(int e) { return e + (e >> 5); }

template <bool EXCL>
__global__ void __launch_bounds__(SSB)
segscan_kernel(const int32_t* in, int32_t* out, int64_t n, const int64_t* __restrict__ off, int nseg,
               uint32_t* flags, SegVal* aggs, SegVal* incls, uint32_t* tile_counter,
               uint32_t* status, uint32_t spin_limit) {
  // one padding word per 32 keeps both the coalesced and the per-thread
  // views of the tile free of bank conflicts
  __shared__ int32_t sm[SST + SST / 32];
  __shared__ SegVal sh_w[SSB / 32];
  __shared__ SegVal sh_prefix;
  __shared__ uint32_t sh_tile;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) sh_tile = atomicAdd(tile_counter, 1u);
  __syncthreads();
  const int64_t tile = sh_tile;
  const int64_t base = tile * SST;
  for (int e = tid; e < SST; e += SSB) {
    const int64_t i = base + e;
    sm[pad32(e)] = (i < n) ? in[i] : 0;
  }
  __syncthreads();
  // head flags of my items: binary search of the first, then walk forward
  const int64_t first = base + int64_t(tid) * SSI;
  SegVal loc[SSI];
  uint32_t heads = 0;
  {
    int64_t s = first < n ? seg_of(off, nseg, first) : 0;
    int64_t next = __ldg(off + s + 1);
#pragma unroll
    for (int k = 0; k < SSI; ++k) {
      const int64_t i = first + k;
      uint32_t head = 0;
      if (i < n) {
        while (i >= next && s + 1 < nseg) {  // also skips empty segments
          ++s;
          next = __ldg(off + s + 1);
        }
        head = (i == __ldg(off + s)) ? 1u : 0u;
      }
      heads |= head << k;
      const SegVal v{head, (i < n) ? sm[pad32(tid * SSI + k)] : 0};
      loc[k] = (k == 0) ? v : seg_comb(loc[k - 1], v);
    }
  }
  // warp scan of thread totals
  SegVal inc = loc[SSI - 1];
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    SegVal other;
    other.flag = __shfl_up_sync(0xffffffffu, inc.flag, o);
    other.v = __shfl_up_sync(0xffffffffu, inc.v, o);
    if (lane >= o) inc = seg_comb(other, inc);
  }
  SegVal lane_excl;
  lane_excl.flag = __shfl_up_sync(0xffffffffu, inc.flag, 1);
  lane_excl.v = __shfl_up_sync(0xffffffffu, inc.v, 1);
  if (lane == 31) sh_w[warp] = inc;
  __syncthreads();
  SegVal tile_agg = sh_w[0];
  SegVal warp_excl{0u, 0};
#pragma unroll
  for (int w = 1; w < SSB / 32; ++w) {
    if (w == warp) warp_excl = tile_agg;
    tile_agg = seg_comb(tile_agg, sh_w[w]);
  }
  SegVal tp;
  if (warp == 0) tp = lane_excl;
  else tp = (lane == 0) ? warp_excl : seg_comb(warp_excl, lane_excl);
  if (tid == 0) tp = SegVal{0u, 0};

  // look-back (warp 0), bounded like the plain scan
  if (warp == 0) {
    SegVal prefix{0u, 0};
    if (tile == 0) {
      if (lane == 0) {
        incls[0] = tile_agg;
        st_release(flags, 2u);
      }
    } else {
      if (lane == 0) {
        aggs[tile] = tile_agg;
        st_release(flags + tile, 1u);
      }
      int64_t pred = tile - 1;
      SegVal acc{0u, 0};
      bool timed_out = false;
      while (true) {
        const int64_t t = pred - lane;
        uint32_t f = (t >= 0) ? ld_acquire(flags + t) : 2u;
        uint32_t spins = 0;
        while (!__all_sync(0xffffffffu, f != 0)) {
          if (f == 0) f = ld_acquire(flags + t);
          if (++spins > spin_limit) { timed_out = true; break; }
          if (spins > 8) __nanosleep(64);
        }
        timed_out = __any_sync(0xffffffffu, timed_out);
        if (timed_out) break;
        const uint32_t im = __ballot_sync(0xffffffffu, f == 2u);
        const int stop = im ? (__ffs(im) - 1) : 32;
        SegVal v{0u, 0};
        if (lane < stop) { v.flag = __ldcg(&aggs[t].flag); v.v = __ldcg(&aggs[t].v); }
        else if (lane == stop) { v.flag = __ldcg(&incls[t].flag); v.v = __ldcg(&incls[t].v); }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          SegVal other;
          other.flag = __shfl_sync(0xffffffffu, v.flag, (lane + o) & 31);
          other.v = __shfl_sync(0xffffffffu, v.v, (lane + o) & 31);
          if (lane + o < 32) v = seg_comb(other, v);
        }
        SegVal window;
        window.flag = __shfl_sync(0xffffffffu, v.flag, 0);
        window.v = __shfl_sync(0xffffffffu, v.v, 0);
        acc = seg_comb(window, acc);
        if (im) break;
        pred -= 32;
      }
      if (timed_out && lane == 0) atomicOr_system(status, kStatusSegTimeout);
      prefix = acc;
      if (lane == 0) {
        incls[tile] = seg_comb(prefix, tile_agg);
        st_release(flags + tile, 2u);
      }
    }
    if (lane == 0) sh_prefix = prefix;
  }
  __syncthreads();
  const SegVal P = seg_comb(sh_prefix, tp);
#pragma unroll
  for (int k = 0; k < SSI; ++k) {
    int32_t r;
    if (EXCL) {
      // value through the previous element of the same segment; 0 at a head
      const SegVal before = (k == 0) ? P : seg_comb(P, loc[k - 1]);
      r = ((heads >> k) & 1u) ? 0 : before.v;
    } else {
      r = seg_comb(P, loc[k]).v;
    }
    sm[pad32(tid * SSI + k)] = r;
  }
  __syncthreads();
  for (int e = tid; e < SST; e += SSB) {
    const int64_t i = base + e;
    if (i < n) out[i] = sm[pad32(e)];
  }
}

// ------------------------------------------------------ segmented sort
// Segments up to SEG_CAP keys are sorted with a bitonic network in shared
// memory (padded to a power of two with the largest key): one warp per
// segment up to SEG_WARP_CAP keys, one block per longer one; longer
// segments go to the onesweep radix sort.  Several long
// segments of moderate length are sorted together: each key becomes
// (segment << 32 | key) -- the key inverted for a descending sort -- and
// one stable 64-bit sort leaves every segment's keys, in order, in that
// segment's own range of the packed array (passes whose digit is zero for
// every key, the top ones, run as plain copies).  That is about a dozen
// launches instead of six per long segment.
constexpr int SEG_CAP = 4096;
constexpr int SEG_BLOCK = 256;
constexpr int SEG_WARP_CAP = 256;  // segments up to this long are sorted by one warp each
constexpr int64_t SEG_PACK_MEAN = int64_t(1) << 18;  // long segments at most this long on average are packed

__device__ __forceinline__ int big_seg_of(const int64_t* __restrict__ off, int nbig, int64_t e) {
  int lo = 0, hi = nbig;  // off[0] = 0 <= e < off[nbig]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= e) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <bool DESC>
__global__ void __launch_bounds__(256)
segsort_pack_kernel(const uint32_t* __restrict__ keys, const int64_t* __restrict__ off,
                    const int64_t* __restrict__ src, int nbig, int64_t total, uint64_t* __restrict__ packed) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += stride) {
    const int sid = big_seg_of(off, nbig, e);
    const uint32_t k = keys[src[sid] + (e - off[sid])];
    packed[e] = (uint64_t(uint32_t(sid)) << 32) | uint64_t(DESC ? ~k : k);
  }
}

// Back to the keys: the sort left segment sid's keys at [off[sid], off[sid+1]).
template <bool DESC>
__global__ void __launch_bounds__(256)
segsort_unpack_kernel(uint32_t* __restrict__ keys, const int64_t* __restrict__ off,
                      const int64_t* __restrict__ src, int64_t total, const uint64_t* __restrict__ packed) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += stride) {
    const uint64_t v = packed[e];
    const uint32_t sid = uint32_t(v >> 32);
    const uint32_t k = uint32_t(v);
    keys[src[sid] + (e - off[sid])] = DESC ? ~k : k;
  }
}

template <bool DESC>
__global__ void __launch_bounds__(SEG_BLOCK)
segsort_small_kernel(uint32_t* keys, const int64_t* __restrict__ off,
                     const int32_t* __restrict__ seg_ids, int nsmall) {
  __shared__ uint32_t sm[SEG_CAP];
  for (int b = blockIdx.x; b < nsmall; b += gridDim.x) {
    const int sid = seg_ids[b];
    const int64_t lo = off[sid];
    const int len = int(off[sid + 1] - lo);
    int p2 = 1;
    while (p2 < len) p2 <<= 1;
    const uint32_t pad = DESC ? 0u : 0xffffffffu;
    for (int i = threadIdx.x; i < p2; i += SEG_BLOCK) sm[i] = (i < len) ? keys[lo + i] : pad;
    __syncthreads();
    for (int k = 2; k <= p2; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = threadIdx.x; i < p2 / 2; i += SEG_BLOCK) {
          // i-th compare-exchange pair of this stage
          const int lo_i = 2 * j * (i / j) + (i % j);
          const int hi_i = lo_i + j;
          const bool up = ((lo_i & k) == 0) != DESC;
          const uint32_t a = sm[lo_i], c = sm[hi_i];
          if ((a > c) == up) {
            sm[lo_i] = c;
            sm[hi_i] = a;
          }
        }
        __syncthreads();
      }
    }
    for (int i = threadIdx.x; i < len; i += SEG_BLOCK) keys[lo + i] = sm[i];
    __syncthreads();
  }
}

// Segments of at most SEG_WARP_CAP keys: one warp each, eight per block,
// the same bitonic network in the warp's own slice of shared memory with
// warp barriers between the stages.
template <bool DESC>
__global__ void __launch_bounds__(SEG_BLOCK)
segsort_warp_kernel(uint32_t* keys, const int64_t* __restrict__ off,
                    const int32_t* __restrict__ seg_ids, int ntiny) {
  constexpr int WPB = SEG_BLOCK / 32;
  __shared__ uint32_t sm[WPB][SEG_WARP_CAP];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t* w = sm[warp];
  const int nw = int(gridDim.x) * WPB;
  for (int b = int(blockIdx.x) * WPB + warp; b < ntiny; b += nw) {  // warp-uniform
    const int sid = seg_ids[b];
    const int64_t lo = off[sid];
    const int len = int(off[sid + 1] - lo);
    int p2 = 1;
    while (p2 < len) p2 <<= 1;
    const uint32_t pad = DESC ? 0u : 0xffffffffu;
    for (int i = lane; i < p2; i += 32) w[i] = (i < len) ? keys[lo + i] : pad;
    __syncwarp();
    for (int k = 2; k <= p2; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = lane; i < p2 / 2; i += 32) {
          const int lo_i = 2 * j * (i / j) + (i % j);
          const int hi_i = lo_i + j;
          const bool up = ((lo_i & k) == 0) != DESC;
          const uint32_t x = w[lo_i], y = w[hi_i];
          if ((x > y) == up) {
            w[lo_i] = y;
            w[hi_i] = x;
          }
        }
        __syncwarp();
      }
    }
    for (int i = lane; i < len; i += 32) keys[lo + i] = w[i];
    __syncwarp();
  }
}

}  // namespace
}  // namespace b200

using namespace b200;

extern "C" {

int b200_batch_plan_create(const int64_t* lens, int nloops, b200_batch_plan* out) {
  if (!out) return fail(B200_ERR_ARG, "b200_batch_plan_create: null out");
  *out = nullptr;
  if (nloops < 0 || (nloops > 0 && !lens)) return fail(B200_ERR_ARG, "b200_batch_plan_create: bad loops");
  auto* p = new b200_batch_plan_s();
  B200_CUDA(cudaGetDevice(&p->device));
  p->nloops = nloops;
  p->lens.assign(lens, lens + nloops);
  p->offsets.assign(size_t(nloops) + 1, 0);
  for (int i = 0; i < nloops; ++i) {
    if (lens[i] < 0) {
      delete p;
      return fail(B200_ERR_ARG, "b200_batch_plan_create: negative length at %d", i);
    }
    p->offsets[i + 1] = p->offsets[i] + lens[i];
  }
  p->total = p->offsets[nloops];
  int rc = B200_OK;
  auto ck = [&](cudaError_t e, const char* w) { if (rc == B200_OK && e != cudaSuccess) rc = cuda_check(e, w); };
  const size_t nl = size_t(std::max(nloops, 1));
  ck(cudaMalloc(&p->d_lens, nl * sizeof(int64_t)), "plan lens");
  ck(cudaMalloc(&p->d_offsets, (nl + 1) * sizeof(int64_t)), "plan offsets");
  if (rc == B200_OK && nloops > 0) {
    ck(cudaMemcpy(p->d_lens, p->lens.data(), nloops * sizeof(int64_t), cudaMemcpyHostToDevice), "plan lens copy");
  }
  ck(cudaMemcpy(p->d_offsets, p->offsets.data(), (size_t(nloops) + 1) * sizeof(int64_t),
                cudaMemcpyHostToDevice), "plan offsets copy");
  std::vector<int32_t> small, mid;
  for (int i = 0; i < nloops; ++i) {
    if (lens[i] <= 1) continue;
    if (lens[i] <= SEG_WARP_CAP) small.push_back(i);
    else if (lens[i] <= SEG_CAP) mid.push_back(i);
    else p->big_segments.push_back(i);
  }
  p->ntiny = int(small.size());
  small.insert(small.end(), mid.begin(), mid.end());
  p->nsmall = int(small.size());
  for (int sid : p->big_segments) p->big_total += lens[sid];
  const int nbig = int(p->big_segments.size());
  p->big_packed = nbig >= 2 && p->big_total <= int64_t(nbig) * SEG_PACK_MEAN;
  if (rc == B200_OK && p->big_packed) {
    std::vector<int64_t> boff(static_cast<size_t>(nbig) + 1, 0), bsrc(static_cast<size_t>(nbig), 0);
    for (int j = 0; j < nbig; ++j) {
      boff[j + 1] = boff[j] + lens[p->big_segments[j]];
      bsrc[j] = p->offsets[p->big_segments[j]];
    }
    ck(cudaMalloc(&p->d_big_off, boff.size() * sizeof(int64_t)), "plan long segments");
    ck(cudaMalloc(&p->d_big_src, bsrc.size() * sizeof(int64_t)), "plan long segments");
    ck(cudaMalloc(&p->d_big_buf, size_t(p->big_total) * sizeof(uint64_t)), "plan long segments");
    if (rc == B200_OK) {
      ck(cudaMemcpy(p->d_big_off, boff.data(), boff.size() * sizeof(int64_t), cudaMemcpyHostToDevice),
         "plan long segments copy");
      ck(cudaMemcpy(p->d_big_src, bsrc.data(), bsrc.size() * sizeof(int64_t), cudaMemcpyHostToDevice),
         "plan long segments copy");
    }
  }
  ck(cudaMalloc(&p->d_small, std::max<size_t>(small.size(), 1) * sizeof(int32_t)), "plan small");
  if (rc == B200_OK && !small.empty())
    ck(cudaMemcpy(p->d_small, small.data(), small.size() * sizeof(int32_t), cudaMemcpyHostToDevice),
       "plan small copy");
  if (rc == B200_OK) rc = build_tiling(p, kVariants[kDefaultVariant].block * kVariants[kDefaultVariant].items);
  if (rc != B200_OK) {
    b200_batch_plan_destroy(p);
    return rc;
  }
  p->variant = kDefaultVariant;
  *out = p;
  clear_error();
  return B200_OK;
}

int b200_batch_plan_destroy(b200_batch_plan p) {
  if (!p) return B200_OK;
  free_tiling(p);
  cudaFree(p->d_lens);
  cudaFree(p->d_offsets);
  cudaFree(p->d_small);
  cudaFree(p->d_big_off);
  cudaFree(p->d_big_src);
  cudaFree(p->d_big_buf);
  delete p;
  return B200_OK;
}

int b200_batch_plan_info(b200_batch_plan p, int64_t* total, int64_t* ntiles, int* tile, int* block) {
  if (!p) return fail(B200_ERR_ARG, "b200_batch_plan_info: null plan");
  if (total) *total = p->total;
  if (ntiles) *ntiles = p->ntiles;
  if (tile) *tile = p->tile;
  if (block) *block = p->variant >= 0 ? kVariants[p->variant].block : 0;
  return B200_OK;
}

const int64_t* b200_batch_plan_offsets(b200_batch_plan p) { return p ? p->d_offsets : nullptr; }

int b200_batch_plan_set_shape(b200_batch_plan p, int block, int items) {
  B200_TRY(check_plan(p, "b200_batch_plan_set_shape"));
  for (int v = 0; v < kNumVariants; ++v) {
    if (kVariants[v].block != block || kVariants[v].items != items) continue;
    B200_TRY(build_tiling(p, block * items));
    p->variant = v;
    clear_error();
    return B200_OK;
  }
  return fail(B200_ERR_ARG, "b200_batch_plan_set_shape: %d x %d is not a batched shape", block, items);
}

int b200_batched_axpy_sum_f32(b200_batch_plan p, float a, const float* const* xs,
                              float* const* ys, double* sums, int mode, b200_stream_t stream) {
  B200_TRY(check_plan(p, "b200_batched_axpy_sum_f32"));
  if (p->nloops == 0) return B200_OK;
  if (!xs || !ys || !sums) return fail(B200_ERR_ARG, "b200_batched_axpy_sum_f32: null pointer");
  if (mode & ~(B200_MODE_COMPENSATED | B200_MODE_DETERMINISTIC))
    return fail(B200_ERR_ARG, "b200_batched_axpy_sum_f32: unknown mode %d", mode);
  if (p->ntiles == 0) {
    // every loop is empty: its sum is zero
    B200_CUDA(cudaMemsetAsync(sums, 0, p->nloops * sizeof(double), static_cast<cudaStream_t>(stream)));
    return B200_OK;
  }
  const Variant v = kVariants[p->variant];
  B200_TRY(build_tiling(p, v.block * v.items));
  // loops of length zero have no tile: the fold writes their sums as zero
  B200_TRY(dispatch_batched(p->variant, p, a, xs, ys, sums, (mode & B200_MODE_COMPENSATED) ? 1 : 0,
                            static_cast<cudaStream_t>(stream)));
  clear_error();
  return B200_OK;
}

int b200_batch_autotune_axpy_sum_f32(b200_batch_plan p, float a, const float* const* xs,
                                     float* const* ys, double* sums, int mode,
                                     b200_stream_t stream) {
  B200_TRY(check_plan(p, "b200_batch_autotune_axpy_sum_f32"));
  if (p->nloops == 0 || p->total == 0) return B200_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaEvent_t e0, e1;
  B200_CUDA(cudaEventCreate(&e0));
  B200_CUDA(cudaEventCreate(&e1));
  const int comp = (mode & B200_MODE_COMPENSATED) ? 1 : 0;
  float best = 1e30f;
  int best_v = kDefaultVariant;
  for (int v = 0; v < kNumVariants; ++v) {
    B200_TRY(build_tiling(p, kVariants[v].block * kVariants[v].items));
    B200_TRY(dispatch_batched(v, p, a, xs, ys, sums, comp, s));  // warm-up
    B200_CUDA(cudaEventRecord(e0, s));
    for (int r = 0; r < 3; ++r) B200_TRY(dispatch_batched(v, p, a, xs, ys, sums, comp, s));
    B200_CUDA(cudaEventRecord(e1, s));
    B200_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    B200_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (log_on()) fprintf(stderr, "[b200] batched variant block=%d items=%d: %.4f ms\n",
                          kVariants[v].block, kVariants[v].items, ms / 3);
    if (ms < best) { best = ms; best_v = v; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  p->variant = best_v;
  B200_TRY(build_tiling(p, kVariants[best_v].block * kVariants[best_v].items));
  if (log_on()) fprintf(stderr, "[b200] batched autotune chose block=%d items=%d\n",
                        kVariants[best_v].block, kVariants[best_v].items);
  clear_error();
  return B200_OK;
}

int b200_loop_axpy_sum_f32(float a, const float* x, float* y, size_t n, double* sum, int mode,
                           b200_stream_t stream) {
  const char* name = "b200_loop_axpy_sum_f32";
  if (!sum) return fail(B200_ERR_ARG, "%s: null sum", name);
  if (n > 0 && (!x || !y)) return fail(B200_ERR_ARG, "%s: null pointer", name);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  constexpr int BLOCK = 256, ITEMS = 8, TILE = BLOCK * ITEMS;
  static KernelSetup ks;
  DeviceProps props;
  B200_TRY(device_props(&props));
  int bps = 0;
  B200_TRY(kernel_setup(ks, props, loop_axpy_sum_kernel<BLOCK, ITEMS>, BLOCK, 0, &bps));
  int64_t grid = (int64_t(n) + TILE - 1) / TILE;
  if (grid > int64_t(props.sms) * bps) grid = int64_t(props.sms) * bps;
  if (grid < 1) grid = 1;
  void* scr = nullptr;
  uint32_t* counters = nullptr;
  B200_TRY(scratch(s, size_t(grid) * sizeof(double), &scr, &counters));
  B200_LAUNCH(name, (loop_axpy_sum_kernel<BLOCK, ITEMS>), unsigned(grid), BLOCK, 0, s, a, x, y,
              int64_t(n), sum, static_cast<double*>(scr), counters + 1,
              (mode & B200_MODE_COMPENSATED) ? 1 : 0);
  clear_error();
  return B200_OK;
}

int b200_loops_axpy_sum_f32(int nloops, const int64_t* lens_host, float a, const float* const* xs_host,
                            float* const* ys_host, double* sums, int mode, b200_stream_t stream) {
  const char* name = "b200_loops_axpy_sum_f32";
  if (nloops < 0) return fail(B200_ERR_ARG, "%s: nloops=%d", name, nloops);
  if (nloops > 0 && (!lens_host || !xs_host || !ys_host || !sums))
    return fail(B200_ERR_ARG, "%s: null pointer", name);
  for (int i = 0; i < nloops; ++i) {
    if (lens_host[i] < 0) return fail(B200_ERR_ARG, "%s: loop %d has length %lld", name, i, (long long)lens_host[i]);
    B200_TRY(b200_loop_axpy_sum_f32(a, xs_host[i], ys_host[i], size_t(lens_host[i]), sums + i, mode, stream));
  }
  clear_error();
  return B200_OK;
}

static int segscan(const char* name, bool excl, b200_batch_plan p, const int32_t* in, int32_t* out,
                   b200_stream_t stream) {
  B200_TRY(check_plan(p, name));
  const int64_t n = p->total;
  if (n == 0) return B200_OK;
  if (!in || !out) return fail(B200_ERR_ARG, "%s: null pointer", name);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t tiles = (n + SST - 1) / SST;
  Sizer z;
  z.take<uint32_t>(size_t(tiles) + 64);
  z.take<SegVal>(size_t(tiles));
  z.take<SegVal>(size_t(tiles));
  void* scr = nullptr;
  B200_TRY(scratch(s, z.bytes(), &scr, nullptr));
  Carver cv(scr);
  uint32_t* flags = cv.take<uint32_t>(size_t(tiles) + 64);
  SegVal* aggs = cv.take<SegVal>(size_t(tiles));
  SegVal* incls = cv.take<SegVal>(size_t(tiles));
  uint32_t* status = nullptr;
  B200_TRY(status_word(&status));
  B200_CUDA(cudaMemsetAsync(flags, 0, (size_t(tiles) + 64) * sizeof(uint32_t), s));
  if (excl)
    B200_LAUNCH(name, segscan_kernel<true>, unsigned(tiles), SSB, 0, s, in, out, n, p->d_offsets,
                p->nloops, flags, aggs, incls, flags + tiles, status, spin_limit());
  else
    B200_LAUNCH(name, segscan_kernel<false>, unsigned(tiles), SSB, 0, s, in, out, n, p->d_offsets,
                p->nloops, flags, aggs, incls, flags + tiles, status, spin_limit());
  clear_error();
  return B200_OK;
}

int b200_segmented_scan_inclusive_i32(b200_batch_plan p, const int32_t* in, int32_t* out,
                                      b200_stream_t stream) {
  return segscan("b200_segmented_scan_inclusive_i32", false, p, in, out, stream);
}
int b200_segmented_scan_exclusive_i32(b200_batch_plan p, const int32_t* in, int32_t* out,
                                      b200_stream_t stream) {
  return segscan("b200_segmented_scan_exclusive_i32", true, p, in, out, stream);
}

int b200_segmented_sort_keys_u32(b200_batch_plan p, uint32_t* keys, int descending,
                                 b200_stream_t stream) {
  const char* name = "b200_segmented_sort_keys_u32";
  B200_TRY(check_plan(p, name));
  if (p->total == 0) return B200_OK;
  if (!keys) return fail(B200_ERR_ARG, "%s: null keys", name);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->ntiny > 0) {
    DeviceProps props;
    B200_TRY(device_props(&props));
    const int grid = std::min((p->ntiny + SEG_BLOCK / 32 - 1) / (SEG_BLOCK / 32), props.sms * 8);
    if (descending)
      B200_LAUNCH(name, segsort_warp_kernel<true>, grid, SEG_BLOCK, 0, s, keys, p->d_offsets, p->d_small,
                  p->ntiny);
    else
      B200_LAUNCH(name, segsort_warp_kernel<false>, grid, SEG_BLOCK, 0, s, keys, p->d_offsets, p->d_small,
                  p->ntiny);
  }
  if (p->nsmall > p->ntiny) {
    DeviceProps props;
    B200_TRY(device_props(&props));
    const int nmid = p->nsmall - p->ntiny;
    const int grid = std::min(nmid, props.sms * 8);
    if (descending)
      B200_LAUNCH(name, segsort_small_kernel<true>, grid, SEG_BLOCK, 0, s, keys, p->d_offsets,
                  p->d_small + p->ntiny, nmid);
    else
      B200_LAUNCH(name, segsort_small_kernel<false>, grid, SEG_BLOCK, 0, s, keys, p->d_offsets,
                  p->d_small + p->ntiny, nmid);
  }
  if (p->big_packed) {
    DeviceProps props;
    B200_TRY(device_props(&props));
    const int nbig = int(p->big_segments.size());
    const unsigned grid = unsigned(std::min<int64_t>((p->big_total + 255) / 256, int64_t(props.sms) * 8));
    if (descending)
      B200_LAUNCH(name, segsort_pack_kernel<true>, grid, 256, 0, s, keys, p->d_big_off, p->d_big_src, nbig,
                  p->big_total, p->d_big_buf);
    else
      B200_LAUNCH(name, segsort_pack_kernel<false>, grid, 256, 0, s, keys, p->d_big_off, p->d_big_src, nbig,
                  p->big_total, p->d_big_buf);
    B200_TRY(b200_sort_keys_u64(p->d_big_buf, size_t(p->big_total), 0, stream));
    if (descending)
      B200_LAUNCH(name, segsort_unpack_kernel<true>, grid, 256, 0, s, keys, p->d_big_off, p->d_big_src,
                  p->big_total, p->d_big_buf);
    else
      B200_LAUNCH(name, segsort_unpack_kernel<false>, grid, 256, 0, s, keys, p->d_big_off, p->d_big_src,
                  p->big_total, p->d_big_buf);
  } else {
    for (int sid : p->big_segments) {
      B200_TRY(b200_sort_keys_u32(keys + p->offsets[sid], size_t(p->lens[sid]), descending, stream));
    }
  }
  clear_error();
  return B200_OK;
}

// ---------------------------------------------------------------- graphs
int b200_graph_capture_begin(b200_stream_t stream) {
  B200_CUDA(cudaStreamBeginCapture(static_cast<cudaStream_t>(stream), cudaStreamCaptureModeThreadLocal));
  return B200_OK;
}

int b200_graph_capture_end(b200_stream_t stream, b200_graph* out) {
  if (!out) return fail(B200_ERR_ARG, "b200_graph_capture_end: null out");
  auto* g = new b200_graph_s();
  cudaError_t e = cudaStreamEndCapture(static_cast<cudaStream_t>(stream), &g->graph);
  if (e != cudaSuccess) {
    delete g;
    return cuda_check(e, "cudaStreamEndCapture");
  }
  e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g->graph);
    delete g;
    return cuda_check(e, "cudaGraphInstantiate");
  }
  *out = g;
  return B200_OK;
}

int b200_graph_launch(b200_graph g, b200_stream_t stream) {
  if (!g) return fail(B200_ERR_ARG, "b200_graph_launch: null graph");
  B200_CUDA(cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(stream)));
  return B200_OK;
}

int b200_graph_destroy(b200_graph g) {
  if (!g) return B200_OK;
  cudaGraphExecDestroy(g->exec);
  cudaGraphDestroy(g->graph);
  delete g;
  return B200_OK;
}

}  // extern "C"
