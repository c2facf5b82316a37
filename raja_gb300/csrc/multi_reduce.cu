// Binned reductions: MultiReduce{Sum,Min,Max,BitOr,BitAnd}.
//
// Reference: pattern/multi_reduce.hpp:68-190 (the front-end classes),
// pattern/detail/multi_reduce.hpp:172-402 (combine per bin with the op's
// rule), policy/cuda/multi_reduce.hpp:80-690 (CUDA: shared-memory atomics
// with replication flushed to global atomics, or global atomics only) and
// policy/sequential/multi_reduce.hpp:135 (seq: in index order).
//
// out[b] = op(out[b], vals[i]) over every i with bins[i] == b, bins outside
// [0, nbins) skipped.  out holds the initial values (the MultiReduce
// constructor's init) and is accumulated into, like b200_histogram_i32.
//
// GB300 design: the histogram kernel's structure with a value per element.
// A persistent grid streams bins and values; each block keeps private
// accumulators for as many bins as fit in shared memory, combined with
// shared-memory atomics, and the rest go straight to global atomics.  At
// the end each block flushes its touched bins with global atomics, from a
// staggered offset.  Floating-point min / max accumulate order-preserving
// integer keys (NaN never enters, as with `if (v < val) val = v`; -0.0
// orders below +0.0) and flush with a compare-and-swap loop on the value.
// Integer and bit results are exact and order-independent; floating-point
// sums depend on the atomic order, as the reference's CUDA policy does.
#include <algorithm>
#include <climits>
#include <type_traits>

#include "b200_internal.cuh"

namespace b200 {
namespace {

constexpr int MBLOCK = 512;

template <class T>
struct Bits;
template <> struct Bits<float> { using I = int32_t; };
template <> struct Bits<double> { using I = long long; };

// order-preserving signed key of a float / double
template <class F>
__device__ __forceinline__ typename Bits<F>::I fkey(F v) {
  using I = typename Bits<F>::I;
  I b;
  memcpy(&b, &v, sizeof(F));
  constexpr I low = I((~std::make_unsigned_t<I>(0)) >> 1);
  return b ^ ((b >> (sizeof(I) * 8 - 1)) & low);
}
template <class F>
__device__ __forceinline__ F fval(typename Bits<F>::I k) {
  using I = typename Bits<F>::I;
  constexpr I low = I((~std::make_unsigned_t<I>(0)) >> 1);
  const I b = k ^ ((k >> (sizeof(I) * 8 - 1)) & low);
  F v;
  memcpy(&v, &b, sizeof(F));
  return v;
}

// global atomics on the caller's values
__device__ __forceinline__ void g_add(int32_t* p, int32_t v) { atomicAdd(p, v); }
__device__ __forceinline__ void g_add(uint32_t* p, uint32_t v) { atomicAdd(p, v); }
__device__ __forceinline__ void g_add(int64_t* p, int64_t v) {
  atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
}
__device__ __forceinline__ void g_add(uint64_t* p, uint64_t v) {
  atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
}
__device__ __forceinline__ void g_add(float* p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ void g_add(double* p, double v) { atomicAdd(p, v); }

template <class T> __device__ __forceinline__ void g_min(T* p, T v) { atomicMin(p, v); }
template <class T> __device__ __forceinline__ void g_max(T* p, T v) { atomicMax(p, v); }
template <> __device__ __forceinline__ void g_min(int64_t* p, int64_t v) {
  atomicMin(reinterpret_cast<long long*>(p), (long long)v);
}
template <> __device__ __forceinline__ void g_max(int64_t* p, int64_t v) {
  atomicMax(reinterpret_cast<long long*>(p), (long long)v);
}
template <> __device__ __forceinline__ void g_min(uint64_t* p, uint64_t v) {
  atomicMin(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
}
template <> __device__ __forceinline__ void g_max(uint64_t* p, uint64_t v) {
  atomicMax(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
}
// floats: `if (v < cur) cur = v` (resp. cur < v) by compare-and-swap
template <class F, bool MIN>
__device__ __forceinline__ void g_fext(F* p, F v) {
  using I = typename Bits<F>::I;
  using UI = std::conditional_t<sizeof(F) == 4, unsigned int, unsigned long long>;
  UI* q = reinterpret_cast<UI*>(p);
  UI cur = *q;
  while (true) {
    F c;
    memcpy(&c, &cur, sizeof(F));
    if (!(MIN ? (v < c) : (c < v))) return;
    UI nv;
    memcpy(&nv, &v, sizeof(F));
    const UI prev = atomicCAS(q, cur, nv);
    if (prev == cur) return;
    cur = prev;
  }
  (void)sizeof(I);
}
template <> __device__ __forceinline__ void g_min(float* p, float v) { g_fext<float, true>(p, v); }
template <> __device__ __forceinline__ void g_max(float* p, float v) { g_fext<float, false>(p, v); }
template <> __device__ __forceinline__ void g_min(double* p, double v) { g_fext<double, true>(p, v); }
template <> __device__ __forceinline__ void g_max(double* p, double v) { g_fext<double, false>(p, v); }

template <class T>
using UBits = std::conditional_t<sizeof(T) == 4, unsigned int, unsigned long long>;
template <class T> __device__ __forceinline__ void g_or(T* p, T v) {
  atomicOr(reinterpret_cast<UBits<T>*>(p), UBits<T>(v));
}
template <class T> __device__ __forceinline__ void g_and(T* p, T v) {
  atomicAnd(reinterpret_cast<UBits<T>*>(p), UBits<T>(v));
}

// ---------------------------------------------------------------- ops
// S: the shared-memory accumulator type; ident: its identity; lift: value
// -> S (false: the value does not take part, e.g. a NaN); s_combine: the
// shared atomic; flush: the global combine of a non-identity S.
template <class T>
struct OpSum {
  using S = T;
  static __device__ S ident() { return S(0); }
  static __device__ bool lift(T v, S& s) { s = v; return true; }
  static __device__ void s_combine(S* p, S v) { g_add(p, v); }
  static __device__ void flush(T* out, S s) { g_add(out, s); }
  static __device__ bool is_ident(S s) { return s == S(0); }
};
template <class T, bool MIN>
struct OpExt {
  static constexpr bool FP = std::is_floating_point<T>::value;
  using S = std::conditional_t<FP, typename Bits<std::conditional_t<FP, T, float>>::I, T>;
  static __device__ S lo() {
    if constexpr (std::is_same<S, int32_t>::value) return INT32_MIN;
    else if constexpr (std::is_same<S, long long>::value) return LLONG_MIN;
    else if constexpr (std::is_same<S, int64_t>::value) return INT64_MIN;
    else return S(0);
  }
  static __device__ S hi() { return ~S(0) > S(0) ? ~S(0) : S(~lo()); }
  static __device__ S ident() { return MIN ? hi() : lo(); }
  static __device__ bool lift(T v, S& s) {
    if constexpr (FP) {
      if (v != v) return false;  // NaN never enters
      s = fkey<T>(v);
    } else {
      s = v;
    }
    return true;
  }
  static __device__ void s_combine(S* p, S v) {
    if (MIN) g_min(p, v);
    else g_max(p, v);
  }
  static __device__ void flush(T* out, S s) {
    if constexpr (FP) {
      if (MIN) g_min(out, fval<T>(s));
      else g_max(out, fval<T>(s));
    } else {
      if (MIN) g_min(out, s);
      else g_max(out, s);
    }
  }
  static __device__ bool is_ident(S s) { return s == ident(); }
};
template <class T, bool OR>
struct OpBit {
  using S = T;
  static __device__ S ident() { return OR ? S(0) : S(~S(0)); }
  static __device__ bool lift(T v, S& s) { s = v; return true; }
  static __device__ void s_combine(S* p, S v) {
    if (OR) g_or(p, v);
    else g_and(p, v);
  }
  static __device__ void flush(T* out, S s) {
    if (OR) g_or(out, s);
    else g_and(out, s);
  }
  static __device__ bool is_ident(S s) { return s == ident(); }
};

template <class T> using OpMin = OpExt<T, true>;
template <class T> using OpMax = OpExt<T, false>;
template <class T> using OpOr = OpBit<T, true>;
template <class T> using OpAnd = OpBit<T, false>;

template <class Op, class T>
__global__ void __launch_bounds__(MBLOCK)
multi_reduce_kernel(const int32_t* __restrict__ bins, const T* __restrict__ vals, size_t n,
                    uint32_t nbins, uint32_t sbins, T* __restrict__ out) {
  using S = typename Op::S;
  extern __shared__ __align__(16) unsigned char mr_raw[];
  S* sh = reinterpret_cast<S*>(mr_raw);
  const int tid = threadIdx.x;
  for (uint32_t b = tid; b < sbins; b += MBLOCK) sh[b] = Op::ident();
  __syncthreads();
  const size_t nt = size_t(gridDim.x) * MBLOCK;
  for (size_t i = size_t(blockIdx.x) * MBLOCK + tid; i < n; i += nt) {
    const uint32_t b = uint32_t(__ldcs(bins + i));
    if (b >= nbins) continue;  // negative bins wrap to large values
    S s;
    if (!Op::lift(__ldcs(vals + i), s)) continue;
    if (b < sbins) Op::s_combine(sh + b, s);
    else Op::flush(out + b, s);
  }
  __syncthreads();
  const uint32_t off = uint32_t((size_t(blockIdx.x) * sbins / gridDim.x) & ~size_t(31));
  for (uint32_t k = tid; k < sbins; k += MBLOCK) {
    uint32_t b = k + off;
    if (b >= sbins) b -= sbins;
    const S s = sh[b];
    if (!Op::is_ident(s)) Op::flush(out + b, s);
  }
}

template <class Op, class T>
int run_multi_reduce(const char* name, const int32_t* bins, const T* vals, size_t n,
                     int32_t nbins, T* out, b200_stream_t stream) {
  using S = typename Op::S;
  if (nbins <= 0) return fail(B200_ERR_ARG, "%s: nbins=%d must be positive", name, nbins);
  if (!out) return fail(B200_ERR_ARG, "%s: null output", name);
  if (reinterpret_cast<uintptr_t>(out) % sizeof(T))
    return fail(B200_ERR_ARG, "%s: output not %zu-byte aligned", name, sizeof(T));
  if (n == 0) { clear_error(); return B200_OK; }
  if (!bins || !vals) return fail(B200_ERR_ARG, "%s: null input", name);
  DeviceProps p;
  B200_TRY(device_props(&p));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t cap = (p.smem_per_block_optin > 4096 ? p.smem_per_block_optin - 4096 : 0) / sizeof(S);
  const uint32_t sbins = uint32_t(std::min<size_t>(size_t(nbins), cap));
  const size_t smem = size_t(sbins) * sizeof(S);
  auto kern = multi_reduce_kernel<Op, T>;
  static SmemOptIn so;
  B200_TRY(smem_optin(so, p, kern, cap * sizeof(S)));
  int bps = 0;
  B200_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, MBLOCK, smem));
  if (bps < 1) bps = 1;
  size_t grid = size_t(p.sms) * bps;
  const size_t need = (n + MBLOCK - 1) / MBLOCK;
  if (grid > need) grid = need;
  B200_LAUNCH(name, kern, (unsigned)grid, MBLOCK, smem, s, bins, vals, n, uint32_t(nbins), sbins,
              out);
  clear_error();
  return B200_OK;
}

}  // namespace
}  // namespace b200

using namespace b200;

extern "C" {

#define B200_MR(OP, SUF, T, OPT)                                                                   \
  int b200_multi_reduce_##OP##_##SUF(const int32_t* bins, const T* vals, size_t n, int32_t nbins, \
                                     T* out, b200_stream_t s) {                                   \
    return run_multi_reduce<OPT, T>("b200_multi_reduce_" #OP "_" #SUF, bins, vals, n, nbins, out,  \
                                    s);                                                           \
  }
#define B200_MR_ALL(SUF, T)                       \
  B200_MR(sum, SUF, T, OpSum<T>)                  \
  B200_MR(min, SUF, T, OpMin<T>)                  \
  B200_MR(max, SUF, T, OpMax<T>)
B200_MR_ALL(i32, int32_t)
B200_MR_ALL(i64, int64_t)
B200_MR_ALL(u32, uint32_t)
B200_MR_ALL(u64, uint64_t)
B200_MR_ALL(f32, float)
B200_MR_ALL(f64, double)
#define B200_MR_BIT(SUF, T)                       \
  B200_MR(bitor, SUF, T, OpOr<T>)                 \
  B200_MR(bitand, SUF, T, OpAnd<T>)
B200_MR_BIT(i32, int32_t)
B200_MR_BIT(i64, int64_t)
B200_MR_BIT(u32, uint32_t)
B200_MR_BIT(u64, uint64_t)
#undef B200_MR_BIT
#undef B200_MR_ALL
#undef B200_MR

}  // extern "C"
