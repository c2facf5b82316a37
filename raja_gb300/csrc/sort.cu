// LSD radix sort (keys and key/value pairs), ascending or descending.
//
// Reference: impl::sort::{stable, unstable, stable_pairs, unstable_pairs}
// (policy/cuda/sort.hpp:92-653) -> cub::DeviceRadixSort::SortKeys /
// SortPairs (+ Descending) over all sizeof(K)*8 bits, with two N-sized pool
// allocations and a copy-back memcpy when the result lands in the
// alternate buffer.  Unstable sorts forward to the stable ones
// (sort.hpp:276-321, 600-653).
//
// GB300 design (onesweep, Adinets & Merrill, "Onesweep: A Faster Least
// Significant Digit Radix Sort for GPUs", 2022):
//   1. hist_kernel: one read of the keys builds the 256-bin histogram of
//      every 8-bit digit position at once (warp-aggregated shared atomics,
//      so skewed digits such as float exponents do not serialise);
//   2. bins_kernel: exclusive scan of each histogram -> global digit bases;
//   3. one onesweep_kernel per digit: a tile of 256 threads x 16 keys is
//      loaded with coalesced warp-striped reads, ranked in registers with
//      warp-level multisplit (__match_any_sync), its per-digit counts are
//      published and a per-digit decoupled look-back over predecessor tiles
//      yields the global offsets; keys (then values) are scattered through
//      shared memory into digit order and written out in runs, so the
//      global stores coalesce.
// Each pass reads and writes every key once; there is no separate upsweep.
// Look-back waits are bounded (device status word, no trap).  Keys are
// mapped to order-preserving unsigned bit patterns on the first pass and
// mapped back on the last: signed integers flip the sign bit, floats flip
// the sign bit (non-negative) or every bit (negative), descending order
// inverts all bits -- which also keeps equal keys in input order.
#include <type_traits>

#include "b200_internal.cuh"

namespace b200 {
namespace {

constexpr int RB = 256;       // threads per tile
constexpr int KPT = 16;       // keys per thread
constexpr int TILE = RB * KPT;
constexpr int RADIX = 256;
constexpr int WARPS = RB / 32;

template <class K>
struct KeyBits {
  using U = typename std::conditional<sizeof(K) == 4, uint32_t, uint64_t>::type;
  static constexpr U SIGN = U(1) << (sizeof(K) * 8 - 1);
  static __device__ __forceinline__ U raw(K k) {
    U u;
    memcpy(&u, &k, sizeof(K));
    return u;
  }
  static __device__ __forceinline__ K cook(U u) {
    K k;
    memcpy(&k, &u, sizeof(K));
    return k;
  }
  // order-preserving map to unsigned
  static __device__ __forceinline__ U to_ord(K k, bool desc) {
    U u = raw(k);
    if (std::is_floating_point<K>::value) u = (u & SIGN) ? U(~u) : U(u ^ SIGN);
    else if (std::is_signed<K>::value) u ^= SIGN;
    return desc ? U(~u) : u;
  }
  static __device__ __forceinline__ K from_ord(U u, bool desc) {
    if (desc) u = ~u;
    if (std::is_floating_point<K>::value) u = (u & SIGN) ? U(u ^ SIGN) : U(~u);
    else if (std::is_signed<K>::value) u ^= SIGN;
    return cook(u);
  }
};

// Status word: 2 flag bits on top, running count below.
template <class ST>
struct Status {
  static constexpr int SHIFT = sizeof(ST) * 8 - 2;
  static constexpr ST AGG = ST(1) << SHIFT;
  static constexpr ST INCL = ST(2) << SHIFT;
  static constexpr ST MASK = (ST(1) << SHIFT) - 1;
};

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// ------------------------------------------------------------ histogram
template <class K, int P>
__global__ void __launch_bounds__(RB)
hist_kernel(const K* __restrict__ keys, size_t n, int desc, uint32_t* __restrict__ hist) {
  using KB = KeyBits<K>;
  using U = typename KB::U;
  __shared__ uint32_t sh[P][RADIX];
  for (int i = threadIdx.x; i < P * RADIX; i += RB) (&sh[0][0])[i] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const size_t warp_global = (size_t(blockIdx.x) * RB + threadIdx.x) >> 5;
  const size_t nwarps = (size_t(gridDim.x) * RB) >> 5;
  // Each warp takes 32 consecutive keys per step; all lanes iterate
  // together so the warp-wide match below always sees the full warp.
  for (size_t b = warp_global * 32; b < n; b += nwarps * 32) {
    const size_t i = b + lane;
    const bool valid = i < n;
    const U u = valid ? KB::to_ord(keys[i], desc != 0) : U(0);
#pragma unroll
    for (int p = 0; p < P; ++p) {
      const uint32_t d = valid ? uint32_t((u >> (8 * p)) & 0xff) : uint32_t(RADIX + lane);
      const uint32_t peers = __match_any_sync(0xffffffffu, d);
      if (valid && lane == __ffs(peers) - 1) atomicAdd(&sh[p][d], uint32_t(__popc(peers)));
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < P * RADIX; i += RB) {
    const uint32_t c = (&sh[0][0])[i];
    if (c) atomicAdd(hist + i, c);
  }
}

// Exclusive scan of each pass's histogram -> digit bases.
template <int P>
__global__ void __launch_bounds__(RADIX) bins_kernel(const uint32_t* __restrict__ hist,
                                                     uint32_t* __restrict__ bins) {
  __shared__ uint32_t wsum[RADIX / 32];
  const int d = threadIdx.x, lane = d & 31, w = d >> 5;
  for (int p = 0; p < P; ++p) {
    const uint32_t c = hist[p * RADIX + d];
    uint32_t inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    uint32_t off = 0;
    for (int i = 0; i < w; ++i) off += wsum[i];
    bins[p * RADIX + d] = off + inc - c;
    __syncthreads();
  }
}

// ------------------------------------------------------------- onesweep
template <class K, class V, class ST>
struct SweepSmem {
  using U = typename KeyBits<K>::U;
  static constexpr size_t KV = sizeof(U) > sizeof(V) ? sizeof(U) : sizeof(V);
  alignas(16) unsigned char kv[TILE * KV];   // keys, then values, in digit order
  uint32_t whist[WARPS][RADIX];              // per-warp digit counters / offsets
  ST gdst[RADIX];                            // global dst = gdst[d] + local position
  uint32_t wtot[WARPS];
  uint32_t tile;
};

template <class K, class V, bool HAS_V, class ST>
__global__ void __launch_bounds__(RB)
onesweep_kernel(const K* __restrict__ kin, K* __restrict__ kout, const V* __restrict__ vin,
                V* __restrict__ vout, size_t n, int shift, int first, int last, int desc,
                const uint32_t* __restrict__ bins, ST* __restrict__ status,
                uint32_t* __restrict__ tile_counter, uint32_t* __restrict__ err,
                uint32_t spin_limit) {
  using KB = KeyBits<K>;
  using U = typename KB::U;
  using S = Status<ST>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SweepSmem<K, V, ST>& sm = *reinterpret_cast<SweepSmem<K, V, ST>*>(smem_raw);
  U* skeys = reinterpret_cast<U*>(sm.kv);
  V* svals = reinterpret_cast<V*>(sm.kv);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < WARPS * RADIX; i += RB) (&sm.whist[0][0])[i] = 0;
  if (tid == 0) sm.tile = atomicAdd(tile_counter, 1u);
  __syncthreads();
  const size_t tile = sm.tile;
  const size_t tbase = tile * TILE;
  const size_t wbase = tbase + size_t(warp) * (32 * KPT);

  // ---- load keys (warp-striped, coalesced); padding keys sort last
  U u[KPT];
#pragma unroll
  for (int k = 0; k < KPT; ++k) {
    const size_t i = wbase + size_t(k) * 32 + lane;
    if (i < n) {
      const K key = kin[i];
      u[k] = first ? KB::to_ord(key, desc != 0) : KB::raw(key);
    } else {
      u[k] = ~U(0);
    }
  }
  // values are loaded up front so their latency overlaps the ranking
  V v[HAS_V ? KPT : 1];
  if (HAS_V) {
#pragma unroll
    for (int k = 0; k < KPT; ++k) {
      const size_t i = wbase + size_t(k) * 32 + lane;
      v[k] = (i < n) ? vin[i] : V(0);
    }
  }

  // ---- warp-level multisplit ranking
  uint32_t pos[KPT];
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int k = 0; k < KPT; ++k) {
    const uint32_t d = uint32_t((u[k] >> shift) & 0xff);
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t prior = sm.whist[warp][d];
    __syncwarp();
    if (lane == 31 - __clz(peers)) sm.whist[warp][d] = prior + __popc(peers);
    __syncwarp();
    pos[k] = prior + __popc(peers & lt);
  }
  __syncthreads();

  // ---- per-digit counts: thread d owns digit d
  const int d = tid;
  uint32_t cnt = 0;
#pragma unroll
  for (int w = 0; w < WARPS; ++w) {
    const uint32_t c = sm.whist[w][d];
    sm.whist[w][d] = cnt;  // exclusive offset of warp w inside digit d
    cnt += c;
  }

  // publish this tile's count for digit d
  ST* my_status = status + tile * RADIX + d;
  if (tile == 0) st_relaxed(my_status, ST(S::INCL | (ST(bins[d]) + cnt)));
  else st_relaxed(my_status, ST(S::AGG | ST(cnt)));

  // block exclusive scan of the counts -> local digit starts
  uint32_t inc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) sm.wtot[warp] = inc;
  __syncthreads();
  uint32_t lstart = inc - cnt;
  for (int w = 0; w < warp; ++w) lstart += sm.wtot[w];

  // ---- decoupled look-back for digit d
  ST gstart;
  if (tile == 0) {
    gstart = ST(bins[d]);
  } else {
    ST acc = 0;
    long long t = (long long)tile - 1;
    uint32_t spins = 0;
    while (true) {
      const ST s = ld_relaxed(status + size_t(t) * RADIX + d);
      const ST flag = s & ~S::MASK;
      if (flag == 0) {
        if (++spins > spin_limit) {
          atomicOr(err, kStatusSortTimeout);
          break;
        }
        if (spins > 8) __nanosleep(32);
        continue;
      }
      acc += s & S::MASK;
      if (flag == S::INCL) break;
      --t;
      if (t < 0) break;  // unreachable: tile 0 publishes INCL
    }
    gstart = acc;
    st_relaxed(my_status, ST(S::INCL | (acc + cnt)));
  }
  sm.gdst[d] = gstart - ST(lstart);
#pragma unroll
  for (int w = 0; w < WARPS; ++w) sm.whist[w][d] += lstart;
  __syncthreads();

  // ---- scatter keys into digit order in shared memory
#pragma unroll
  for (int k = 0; k < KPT; ++k) {
    const uint32_t dk = uint32_t((u[k] >> shift) & 0xff);
    pos[k] += sm.whist[warp][dk];
    skeys[pos[k]] = u[k];
  }
  __syncthreads();

  // ---- write keys out in runs
  ST dst[KPT];
#pragma unroll
  for (int j = 0; j < KPT; ++j) {
    const int i = j * RB + tid;
    const U uk = skeys[i];
    const uint32_t dk = uint32_t((uk >> shift) & 0xff);
    dst[j] = sm.gdst[dk] + ST(i);
    if (dst[j] < n) kout[dst[j]] = last ? KB::from_ord(uk, desc != 0) : KB::cook(uk);
  }

  if (HAS_V) {
    __syncthreads();  // keys fully read from shared memory
#pragma unroll
    for (int k = 0; k < KPT; ++k) svals[pos[k]] = v[k];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
      const int i = j * RB + tid;
      if (dst[j] < n) vout[dst[j]] = svals[i];
    }
  }
}

struct NoVal {};

template <class K, class V, bool HAS_V>
int run_sort(const char* name, const K* kin, K* kout, const V* vin, V* vout, size_t n, int desc,
             b200_stream_t stream) {
  using U = typename KeyBits<K>::U;
  constexpr int P = sizeof(K);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (n >= (size_t(1) << 32)) return fail(B200_ERR_ARG, "%s: n=%zu exceeds 2^32-1", name, n);
  if (n > 0 && (!kin || !kout || (HAS_V && (!vin || !vout))))
    return fail(B200_ERR_ARG, "%s: null pointer", name);
  if (n <= 1) {
    if (n == 1 && kin != kout) B200_CUDA(cudaMemcpyAsync(kout, kin, sizeof(K), cudaMemcpyDefault, s));
    if (HAS_V && n == 1 && vin != vout)
      B200_CUDA(cudaMemcpyAsync(vout, vin, sizeof(V), cudaMemcpyDefault, s));
    clear_error();
    return B200_OK;
  }
  const size_t tiles = (n + TILE - 1) / TILE;
  const bool wide = n >= (size_t(1) << 30);
  const size_t st_bytes = wide ? sizeof(uint64_t) : sizeof(uint32_t);
  Sizer z;
  z.take<K>(n);                                    // alternate keys
  if (HAS_V) z.take<V>(n);                         // alternate values
  z.take<uint32_t>(P * RADIX);                     // bins
  // zeroed region: hist, tile counters, status words
  z.take<unsigned char>(P * RADIX * 4 + 64 * 4 + size_t(P) * tiles * RADIX * st_bytes);
  void* scr = nullptr;
  B200_TRY(scratch(s, z.bytes(), &scr, nullptr));
  Carver cv(scr);
  K* kalt = cv.take<K>(n);
  V* valt = HAS_V ? cv.take<V>(n) : nullptr;
  uint32_t* bins = cv.take<uint32_t>(P * RADIX);
  const size_t zbytes = P * RADIX * 4 + 64 * 4 + size_t(P) * tiles * RADIX * st_bytes;
  unsigned char* zr = cv.take<unsigned char>(zbytes);
  uint32_t* hist = reinterpret_cast<uint32_t*>(zr);
  uint32_t* counters = hist + P * RADIX;
  void* status = counters + 64;
  B200_CUDA(cudaMemsetAsync(zr, 0, zbytes, s));
  uint32_t* err = nullptr;
  B200_TRY(status_word(&err));

  DeviceProps props;
  B200_TRY(device_props(&props));
  {
    size_t g = size_t(props.sms) * 4;
    const size_t need = (n + RB - 1) / RB;
    if (g > need) g = need;
    B200_LAUNCH("b200_sort_hist", (hist_kernel<K, P>), (unsigned)g, RB, 0, s, kin, n, desc, hist);
  }
  B200_LAUNCH("b200_sort_bins", bins_kernel<P>, 1, RADIX, 0, s, hist, bins);

  using VV = typename std::conditional<HAS_V, V, uint32_t>::type;
  const uint32_t lim = spin_limit();
  // launch names carry key/value widths so timings separate per shape
  const char* sweep_name =
      !HAS_V ? (sizeof(K) == 4 ? "b200_onesweep_k32" : "b200_onesweep_k64")
             : (sizeof(K) == 4 ? (sizeof(VV) == 4 ? "b200_onesweep_k32_v32" : "b200_onesweep_k32_v64")
                               : (sizeof(VV) == 4 ? "b200_onesweep_k64_v32" : "b200_onesweep_k64_v64"));
  for (int p = 0; p < P; ++p) {
    const K* src = (p == 0) ? kin : ((p & 1) ? kalt : kout);
    K* dstk = (p & 1) ? kout : kalt;
    const VV* vsrc = nullptr;
    VV* vdst = nullptr;
    if (HAS_V) {
      vsrc = reinterpret_cast<const VV*>((p == 0) ? vin : ((p & 1) ? valt : vout));
      vdst = reinterpret_cast<VV*>((p & 1) ? vout : valt);
    }
    const int first = p == 0, last = p == P - 1;
    if (wide) {
      using SM = SweepSmem<K, VV, uint64_t>;
      auto kern = onesweep_kernel<K, VV, HAS_V, uint64_t>;
      static bool attr64 = false;
      if (!attr64) {
        B200_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(SM))));
        attr64 = true;
      }
      uint64_t* st = static_cast<uint64_t*>(status) + size_t(p) * tiles * RADIX;
      B200_LAUNCH(sweep_name, kern, (unsigned)tiles, RB, sizeof(SM), s, src, dstk, vsrc,
                  vdst, n, 8 * p, first, last, desc, bins + p * RADIX, st, counters + p, err, lim);
    } else {
      using SM = SweepSmem<K, VV, uint32_t>;
      auto kern = onesweep_kernel<K, VV, HAS_V, uint32_t>;
      static bool attr32 = false;
      if (!attr32) {
        B200_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(SM))));
        attr32 = true;
      }
      uint32_t* st = static_cast<uint32_t*>(status) + size_t(p) * tiles * RADIX;
      B200_LAUNCH(sweep_name, kern, (unsigned)tiles, RB, sizeof(SM), s, src, dstk, vsrc,
                  vdst, n, 8 * p, first, last, desc, bins + p * RADIX, st, counters + p, err, lim);
    }
  }
  static_assert(P % 2 == 0, "even number of digit passes ends in the home buffer");
  (void)sizeof(U);
  clear_error();
  return B200_OK;
}

template <class K>
int sort_keys(const char* name, const K* in, K* out, size_t n, int desc, b200_stream_t s) {
  return run_sort<K, uint32_t, false>(name, in, out, nullptr, nullptr, n, desc, s);
}
template <class K, class V>
int sort_pairs(const char* name, const K* kin, K* kout, const V* vin, V* vout, size_t n, int desc,
               b200_stream_t s) {
  return run_sort<K, V, true>(name, kin, kout, vin, vout, n, desc, s);
}

}  // namespace
}  // namespace b200

using namespace b200;

extern "C" {

#define B200_SORT_KEYS(SUF, K)                                                                 \
  int b200_sort_keys_##SUF(K* keys, size_t n, int desc, b200_stream_t s) {                     \
    return sort_keys<K>("b200_sort_keys_" #SUF, keys, keys, n, desc, s);                       \
  }
B200_SORT_KEYS(u32, uint32_t)
B200_SORT_KEYS(u64, uint64_t)
B200_SORT_KEYS(i32, int32_t)
B200_SORT_KEYS(i64, int64_t)
B200_SORT_KEYS(f32, float)
B200_SORT_KEYS(f64, double)
#undef B200_SORT_KEYS

int b200_sort_keys_copy_u32(const uint32_t* in, uint32_t* out, size_t n, int desc, b200_stream_t s) {
  return sort_keys<uint32_t>("b200_sort_keys_copy_u32", in, out, n, desc, s);
}
int b200_sort_keys_copy_u64(const uint64_t* in, uint64_t* out, size_t n, int desc, b200_stream_t s) {
  return sort_keys<uint64_t>("b200_sort_keys_copy_u64", in, out, n, desc, s);
}
int b200_sort_keys_copy_f32(const float* in, float* out, size_t n, int desc, b200_stream_t s) {
  return sort_keys<float>("b200_sort_keys_copy_f32", in, out, n, desc, s);
}

#define B200_SORT_PAIRS(SUF, K, V)                                                             \
  int b200_sort_pairs_##SUF(K* keys, V* vals, size_t n, int desc, b200_stream_t s) {           \
    return sort_pairs<K, V>("b200_sort_pairs_" #SUF, keys, keys, vals, vals, n, desc, s);      \
  }
B200_SORT_PAIRS(u32_i32, uint32_t, int32_t)
B200_SORT_PAIRS(u32_u32, uint32_t, uint32_t)
B200_SORT_PAIRS(i32_i32, int32_t, int32_t)
B200_SORT_PAIRS(f32_i32, float, int32_t)
B200_SORT_PAIRS(u64_i32, uint64_t, int32_t)
B200_SORT_PAIRS(u64_i64, uint64_t, int64_t)
B200_SORT_PAIRS(i64_i64, int64_t, int64_t)
B200_SORT_PAIRS(f64_i64, double, int64_t)
B200_SORT_PAIRS(f64_i32, double, int32_t)
#undef B200_SORT_PAIRS

int b200_sort_pairs_copy_f32_i32(const float* kin, const int32_t* vin, float* kout,
                                 int32_t* vout, size_t n, int desc, b200_stream_t s) {
  return sort_pairs<float, int32_t>("b200_sort_pairs_copy_f32_i32", kin, kout, vin, vout, n, desc, s);
}
int b200_sort_pairs_copy_u32_i32(const uint32_t* kin, const int32_t* vin, uint32_t* kout,
                                 int32_t* vout, size_t n, int desc, b200_stream_t s) {
  return sort_pairs<uint32_t, int32_t>("b200_sort_pairs_copy_u32_i32", kin, kout, vin, vout, n,
                                       desc, s);
}

}  // extern "C"
