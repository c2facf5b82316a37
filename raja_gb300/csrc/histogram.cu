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
// histograms aggregate within the warp first (__match_any_sync): one
// shared atomic per distinct bin per warp instruction, so the heavy head of
// a Zipf distribution does not serialise on one address.  At the end each
// block adds its non-zero counters into the global 64-bit counts.
#include "b200_internal.cuh"

namespace b200 {
namespace {

constexpr int HBLOCK = 512;

template <bool AGG>
__device__ __forceinline__ void count_one(uint32_t* sh, int R, int rsel, uint32_t v,
                                          uint32_t nbins, uint32_t sbins,
                                          unsigned long long* gcounts, bool valid) {
  if (AGG) {
    // warp aggregation; invalid lanes use unique keys that never match
    const uint32_t key = valid ? v : (0x80000000u | threadIdx.x);
    const uint32_t peers = __match_any_sync(0xffffffffu, key);
    if (valid && (threadIdx.x & 31) == __ffs(peers) - 1) {
      const uint32_t c = __popc(peers);
      if (v < sbins) atomicAdd(sh + v, c);
      else atomicAdd(gcounts + v, (unsigned long long)c);
    }
  } else {
    if (valid) {
      if (v < sbins) atomicAdd(sh + size_t(v) * R + rsel, 1u);
      else atomicAdd(gcounts + v, 1ull);
    }
  }
  (void)nbins;
}

template <bool AGG>
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
    // all lanes of a warp run the same number of iterations (for the match)
    const size_t wstart = gt - (tid & 31);
    for (size_t vb = wstart * 1; vb < nvec; vb += nt * U) {
      int4 q[U];
      bool ok[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const size_t vi = vb + size_t(u) * nt + (tid & 31);
        ok[u] = vi < nvec;
        q[u] = ok[u] ? __ldcs(reinterpret_cast<const int4*>(x) + vi) : make_int4(0, 0, 0, 0);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const uint32_t e[4] = {uint32_t(q[u].x), uint32_t(q[u].y), uint32_t(q[u].z), uint32_t(q[u].w)};
#pragma unroll
        for (int k = 0; k < 4; ++k)
          count_one<AGG>(sh, R, rsel, e[k], nbins, sbins, gcounts, ok[u] && e[k] < nbins);
      }
    }
    done = nvec * 4;
  }
  // scalar remainder (or the whole input when unaligned)
  {
    const size_t rem = n - done;
    const size_t wstart = gt - (tid & 31);
    for (size_t b = wstart; b < rem; b += nt) {
      const size_t i = b + (tid & 31);
      const bool ok = i < rem;
      const uint32_t v = ok ? uint32_t(x[done + i]) : 0u;
      count_one<AGG>(sh, R, rsel, v, nbins, sbins, gcounts, ok && v < nbins);
    }
  }
  __syncthreads();
  for (uint32_t b = tid; b < sbins; b += HBLOCK) {
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
  const size_t cap_words = (p.smem_per_block_optin > 4096 ? p.smem_per_block_optin - 4096 : 0) / 4;
  const bool agg = nbins > 2048;
  int R = 1;
  uint32_t sbins;
  if (!agg) {
    R = 8;
    while (R > 1 && size_t(nbins) * R > cap_words) R >>= 1;
    sbins = uint32_t(nbins);
    if (size_t(sbins) * R > cap_words) sbins = uint32_t(cap_words / R);
  } else {
    sbins = uint32_t(size_t(nbins) < cap_words ? size_t(nbins) : cap_words);
  }
  const size_t smem = size_t(sbins) * R * 4;
  int bps = 0;
  if (agg) {
    B200_CUDA(cudaFuncSetAttribute(hist_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    B200_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, hist_kernel<true>, HBLOCK, smem));
  } else {
    B200_CUDA(cudaFuncSetAttribute(hist_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    B200_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, hist_kernel<false>, HBLOCK, smem));
  }
  if (bps < 1) bps = 1;
  size_t grid = size_t(p.sms) * bps;
  const size_t need = (n / 4 + HBLOCK - 1) / HBLOCK + 1;
  if (grid > need) grid = need;
  const bool vec_ok = reinterpret_cast<uintptr_t>(x) % 16 == 0;
  auto* gc = reinterpret_cast<unsigned long long*>(counts);
  if (agg)
    B200_LAUNCH("b200_histogram_agg", hist_kernel<true>, (unsigned)grid, HBLOCK, smem, s, x, n,
                uint32_t(nbins), sbins, R, int(vec_ok), gc);
  else
    B200_LAUNCH("b200_histogram_rep", hist_kernel<false>, (unsigned)grid, HBLOCK, smem, s, x, n,
                uint32_t(nbins), sbins, R, int(vec_ok), gc);
  clear_error();
  return B200_OK;
}
