// Histogram (binned atomic reduction, MultiReduceSum with a +1 body).
//
// Reference: policy/cuda/multi_reduce.hpp -- per-block shared-memory
// atomics with replication (:128-191, :476-660) flushed to global atomics
// (:80-100), or global atomics only (:208-470).
//
// GB300 design: a persistent grid (SM count x resident blocks) streams the
// input with 16-byte loads.  Each block keeps private 32-bit counters in
// shared memory for as many bins as fit (up to ~56K bins with the 227 KB
// opt-in); bins beyond that go straight to global 64-bit atomics.  Small
// histograms are replicated R ways, interleaved so that lanes of one warp
// that hit the same bin land on different banks and addresses.  Large
// histograms use one copy and plain shared atomics: a warp-wide vote to
// aggregate equal bins (__match_any_sync) costs ~80 cycles per warp on this
// GPU, more than the few replays a Zipf head causes.  At the end each block
// adds its non-zero counters into the global 64-bit counts.
#include "b200_internal.cuh"

namespace b200 {
namespace {

constexpr int HBLOCK = 1024;

__device__ __forceinline__ void count_one(uint32_t* sh, int R, int rsel, uint32_t v,
                                          uint32_t sbins, unsigned long long* gcounts,
                                          bool valid) {
  if (valid) {
    if (v < sbins) atomicAdd(sh + size_t(v) * R + rsel, 1u);
    else atomicAdd(gcounts + v, 1ull);
  }
}

__global__ void __launch_bounds__(HBLOCK)
hist_kernel(const int32_t* __restrict__ x, size_t n, uint32_t nbins, uint32_t sbins, int R,
            int vec_ok, unsigned long long* __restrict__ gcounts) {
  extern __shared__ uint32_t sh[];
  const int tid = threadIdx.x;
  for (size_t i = tid; i < size_t(sbins) * R; i += HBLOCK) sh[i] = 0;
  __syncthreads();
  const int rsel = (tid & 31) % R;
  const size_t gt = size_t(blockIdx.x) * HBLOCK + tid;
  const size_t nt = size_t(gridDim.x) * HBLOCK;
  size_t done = 0;
  if (vec_ok) {
    const size_t nvec = n / 4;
    constexpr int U = 4;
    size_t v = gt;
    for (; v + (U - 1) * nt < nvec; v += U * nt) {
      int4 q[U];
#pragma unroll
      for (int u = 0; u < U; ++u) q[u] = __ldcs(reinterpret_cast<const int4*>(x) + v + u * nt);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const uint32_t e[4] = {uint32_t(q[u].x), uint32_t(q[u].y), uint32_t(q[u].z), uint32_t(q[u].w)};
#pragma unroll
        for (int k = 0; k < 4; ++k) count_one(sh, R, rsel, e[k], sbins, gcounts, e[k] < nbins);
      }
    }
    for (; v < nvec; v += nt) {
      const int4 q = __ldcs(reinterpret_cast<const int4*>(x) + v);
      const uint32_t e[4] = {uint32_t(q.x), uint32_t(q.y), uint32_t(q.z), uint32_t(q.w)};
#pragma unroll
      for (int k = 0; k < 4; ++k) count_one(sh, R, rsel, e[k], sbins, gcounts, e[k] < nbins);
    }
    done = nvec * 4;
  }
  // scalar remainder (or the whole input when unaligned)
  for (size_t i = done + gt; i < n; i += nt) {
    const uint32_t v = uint32_t(x[i]);
    count_one(sh, R, rsel, v, sbins, gcounts, v < nbins);
  }
  __syncthreads();
  // flush: every block starts at its own offset in the bin range (warp
  // aligned), so the blocks, which finish together, do not all hit the
  // same global counters at the same time
  const uint32_t off = uint32_t((size_t(blockIdx.x) * sbins / gridDim.x) & ~size_t(31));
  for (uint32_t k = tid; k < sbins; k += HBLOCK) {
    uint32_t b = k + off;
    if (b >= sbins) b -= sbins;
    uint32_t c = 0;
    for (int r = 0; r < R; ++r) c += sh[size_t(b) * R + r];
    if (c) atomicAdd(gcounts + b, (unsigned long long)c);
  }
}

}  // namespace
}  // namespace b200

using namespace b200;

extern "C" int b200_histogram_i32(const int32_t* x, size_t n, int32_t nbins, uint64_t* counts,
                                  b200_stream_t stream) {
  const char* name = "b200_histogram_i32";
  if (nbins <= 0) return fail(B200_ERR_ARG, "%s: nbins=%d must be positive", name, nbins);
  if (!counts) return fail(B200_ERR_ARG, "%s: null counts", name);
  if (n == 0) { clear_error(); return B200_OK; }
  if (!x) return fail(B200_ERR_ARG, "%s: null input", name);
  if (reinterpret_cast<uintptr_t>(counts) % 8) return fail(B200_ERR_ARG, "%s: counts not 8-byte aligned", name);
  DeviceProps p;
  B200_TRY(device_props(&p));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // shared counters: up to 8 lane-interleaved replicas while they fit,
  // otherwise one copy of as many bins as fit
  const size_t cap_words = (p.smem_per_block_optin > 4096 ? p.smem_per_block_optin - 4096 : 0) / 4;
  int R = 8;
  while (R > 1 && size_t(nbins) * R > cap_words) R >>= 1;
  uint32_t sbins = uint32_t(nbins);
  if (size_t(sbins) * R > cap_words) sbins = uint32_t(cap_words / R);
  const size_t smem = size_t(sbins) * R * 4;
  static SmemOptIn so;
  B200_TRY(smem_optin(so, p, hist_kernel, cap_words * 4));
  int bps = 0;
  B200_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, hist_kernel, HBLOCK, smem));
  if (bps < 1) bps = 1;
  size_t grid = size_t(p.sms) * bps;
  const size_t need = (n / 4 + HBLOCK - 1) / HBLOCK + 1;
  if (grid > need) grid = need;
  const bool vec_ok = reinterpret_cast<uintptr_t>(x) % 16 == 0;
  auto* gc = reinterpret_cast<unsigned long long*>(counts);
  B200_LAUNCH("b200_histogram", hist_kernel, (unsigned)grid, HBLOCK, smem, s, x, n, uint32_t(nbins),
              sbins, R, int(vec_ok), gc);
  clear_error();
  return B200_OK;
}
