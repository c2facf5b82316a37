// Reducers: ReduceSum / dot / Min / Max / MinLoc / MaxLoc / BitOr / BitAnd.
//
// Reference: policy/cuda/reduce.hpp -- per-thread accumulation inside the
// forall body, warp-shuffle block reduce (intrinsics.hpp:383-470) and a
// last-block grid combine driven by an atomicInc ticket
// (reduce.hpp:133-214), followed by a host-side combine of pinned tally
// slots (reduce.hpp:1128-1149).
//
// GB300 design: one streaming kernel per reduction.  The index space is cut
// into fixed chunks of 256 threads x 64 bytes; each thread issues four
// independent 16-byte loads per chunk (8 for dot) so that ~128 KB per SM is
// in flight, enough to cover HBM3e latency.  Blocks are sized to fill every
// SM (occupancy x SM count).  Each block reduces with a fixed butterfly over
// warp shuffles and shared memory, writes one partial, and the last block to
// take a ticket combines the partials in index order and writes the result
// to device memory -- no host round trip, no pinned tally.
//
// Floating-point sums support three modes (B200_MODE_*):
//   naive         -- accumulate in the element type (the reference's rule);
//   compensated   -- FP32 input: per-thread cascaded TwoSum in FP32 (three
//                    levels, so the per-element work stays on the FP32
//                    pipes), double-double across threads and blocks; FP64
//                    input: per-thread TwoSum and double-double throughout;
//   deterministic -- one partial per fixed chunk, combined in a fixed tree:
//                    the result depends on (n, data) only, not on the grid.
// Min/Max(/Loc) carry the element index and break ties by the lowest index,
// which makes them bit-identical to seq_exec's first-wins rule
// (util/Operators.hpp:555-591, pattern/detail/reduce.hpp:127-179).
#include <cfloat>
#include <climits>
#include <mutex>
#include <type_traits>
#include <utility>

#include "b200_internal.cuh"

namespace b200 {
namespace {

constexpr int RBLOCK = 256;
constexpr int F64_DADD = 1;  // of 8 elements, added on the FP64 pipe by the FP64 sum (0-4 measured)

template <class T>
struct Chunk {
  static constexpr int VN = 16 / sizeof(T);      // elements per 16-byte vector
  static constexpr int NV = 4;                   // vectors per thread per chunk
  static constexpr int ITEMS = VN * NV;          // elements per thread per chunk
  static constexpr size_t SIZE = size_t(RBLOCK) * ITEMS;
};

// Read a value written by another block in this kernel (bypass L1).
template <class P>
__device__ __forceinline__ P ld_cg_any(const P* p) {
  static_assert(sizeof(P) % 4 == 0, "partial size");
  constexpr int W = sizeof(P) / 4;
  uint32_t w[W];
  const uint32_t* q = reinterpret_cast<const uint32_t*>(p);
#pragma unroll
  for (int i = 0; i < W; ++i) w[i] = __ldcg(q + i);
  P r;
  memcpy(&r, w, sizeof(P));
  return r;
}

template <class T>
struct Lim;
template <> struct Lim<float> { static __device__ float hi() { return FLT_MAX; } static __device__ float lo() { return -FLT_MAX; } };
template <> struct Lim<int32_t> { static __device__ int32_t hi() { return INT_MAX; } static __device__ int32_t lo() { return INT_MIN; } };
template <> struct Lim<int64_t> { static __device__ int64_t hi() { return LLONG_MAX; } static __device__ int64_t lo() { return LLONG_MIN; } };
template <> struct Lim<uint32_t> { static __device__ uint32_t hi() { return UINT_MAX; } static __device__ uint32_t lo() { return 0u; } };
template <> struct Lim<uint64_t> { static __device__ uint64_t hi() { return ULLONG_MAX; } static __device__ uint64_t lo() { return 0ull; } };

struct OutPtrs {
  void* val;
  int64_t* idx;
};

// ----------------------------------------------------------------- ops
// Each op defines: T, Acc (per thread), Part (across threads and blocks),
// identity(), add(acc, v, i) (or add2 for dot), to_part, part_identity,
// merge_part(earlier, later), store.  Each thread's Acc becomes a Part
// before the block reduction.

// Naive floating-point sum / dot: accumulate in T.
template <class TT>
struct SumNaive {
  using T = TT;
  using Acc = T;
  using Part = T;
  static __device__ Acc identity() { return T(0); }
  static __device__ void add(Acc& a, T v, int64_t) { a += v; }
  static __device__ void add2(Acc& a, T x, T y) { a = fma(x, y, a); }
  static __device__ Acc merge(Acc a, Acc b) { return a + b; }
  static __device__ Part to_part(Acc a) { return a; }
  static __device__ Part part_identity() { return T(0); }
  static __device__ Part merge_part(Part a, Part b) { return a + b; }
  static __device__ void store(OutPtrs o, Part p) { *static_cast<double*>(o.val) = double(p); }
};

// FP64 sum that takes most per-element work off GB300's FP64 pipe (about
// 1.6 DADD per clock per SM, below what HBM delivers).  Of each thread's
// 8-element chunk, D elements are added in FP64 as usual; the mantissas of
// the others are aligned to their largest exponent and summed exactly in
// int64 on the integer pipes (53 bits placed at bits 59..7, so six terms
// cannot overflow and only bits below 2^(emax-59) are dropped), then the
// int64 sum is converted, scaled by a power of two and added once.  That
// is at least as accurate as adding the elements one by one in FP64.
// Chunks holding an infinity or NaN take the plain FP64 path, so IEEE
// propagation is the reference's.
template <int D>
struct SumF64Aligned : SumNaive<double> {
  static constexpr bool CHUNKED = true;
  static __device__ __forceinline__ void add_chunk(double& a, const Vec16<double>* v, size_t,
                                                   size_t) {
    constexpr int M = 8 - D;  // elements taken by the integer path
    double xs[8];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      xs[2 * j] = v[j].v[0];
      xs[2 * j + 1] = v[j].v[1];
    }
    uint64_t b[M];
    int e[M];
    int emax = 1;
#pragma unroll
    for (int i = 0; i < M; ++i) {
      b[i] = uint64_t(__double_as_longlong(xs[D + i]));
      e[i] = int(uint32_t(b[i] >> 52) & 0x7ffu);
      emax = max(emax, e[i]);
    }
    if (emax == 0x7ff) {  // infinity or NaN in the chunk
#pragma unroll
      for (int i = 0; i < 8; ++i) a += xs[i];
      return;
    }
#pragma unroll
    for (int i = 0; i < D; ++i) a += xs[i];
    long long s = 0;
#pragma unroll
    for (int i = 0; i < M; ++i) {
      const uint64_t mant = (b[i] & 0x000fffffffffffffull) | (e[i] ? (1ull << 52) : 0ull);
      const int sh = min(emax - max(e[i], 1), 63);  // subnormals sit at exponent 1
      const long long t = (long long)((mant << 7) >> sh);
      s += ((long long)b[i] < 0) ? -t : t;
    }
    // value = s * 2^(emax - 1075 - 7); a power of two is exact to multiply
    a += (emax >= 60) ? double(s) * __longlong_as_double((long long)(emax - 59) << 52)
                      : scalbn(double(s), emax - 1082);
  }
};

template <class T>
struct Pair { T s, c; };
struct Trip { float s, c, cc; };
struct DD { double hi, lo; };

// Double-double sum (two_sum of the leading parts, trailing parts added,
// then renormalised so that |lo| <= ulp(hi) / 2).
__device__ __forceinline__ DD dd_add(DD a, DD b) {
  double s, e;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  const double hi = s + e;
  return {hi, e - (hi - s)};
}

// Compensated FP32 sum / dot: cascaded TwoSum per thread in FP32,
// double-double across threads and blocks.
struct SumCompF32 {
  using T = float;
  using Acc = Trip;
  using Part = DD;
  static __device__ Acc identity() { return {0.f, 0.f, 0.f}; }
  // Cascaded compensation: the rounding error of the running sum goes into
  // a compensated second level, whose own error is accumulated in a third.
  static __device__ void add(Acc& a, float v, int64_t) {
    float s, e, c, e2;
    two_sum(a.s, v, s, e);
    two_sum(a.c, e, c, e2);
    a.s = s;
    a.c = c;
    a.cc += e2;
  }
  static __device__ void add2(Acc& a, float x, float y) {
    float p, ep, s, es, c1, e1, c2, e2;
    two_prod(x, y, p, ep);  // x*y = p + ep exactly
    two_sum(a.s, p, s, es);
    two_sum(a.c, es, c1, e1);
    two_sum(c1, ep, c2, e2);
    a.s = s;
    a.c = c2;
    a.cc += e1 + e2;
  }
  // The first two levels become one double-double exactly (two_sum in
  // double), the third is added in double-double; from here on every
  // combine is double-double.
  static __device__ Part to_part(Acc a) {
    double hi, lo;
    two_sum(double(a.s), double(a.c), hi, lo);
    return dd_add({hi, lo}, {double(a.cc), 0.0});
  }
  static __device__ Part part_identity() { return {0.0, 0.0}; }
  static __device__ Part merge_part(Part a, Part b) { return dd_add(a, b); }
  static __device__ void store(OutPtrs o, Part p) { *static_cast<double*>(o.val) = p.hi + p.lo; }
};

// Compensated FP64 sum / dot: double-double style accumulation throughout.
struct SumCompF64 {
  using T = double;
  using Acc = Pair<double>;
  using Part = Pair<double>;
  static __device__ Acc identity() { return {0.0, 0.0}; }
  static __device__ void add(Acc& a, double v, int64_t) {
    double s, e;
    two_sum(a.s, v, s, e);
    a.s = s;
    a.c += e;
  }
  static __device__ void add2(Acc& a, double x, double y) {
    double p, ep, s, es;
    two_prod(x, y, p, ep);
    two_sum(a.s, p, s, es);
    a.s = s;
    a.c += ep + es;
  }
  static __device__ Acc merge(Acc a, Acc b) {
    double s, e;
    two_sum(a.s, b.s, s, e);
    return {s, a.c + b.c + e};
  }
  static __device__ Part to_part(Acc a) { return a; }
  static __device__ Part part_identity() { return {0.0, 0.0}; }
  static __device__ Part merge_part(Part a, Part b) { return merge(a, b); }
  static __device__ void store(OutPtrs o, Part p) { *static_cast<double*>(o.val) = p.s + p.c; }
};

// Integer sum with two's-complement wrap-around.
template <class TT>
struct SumInt {
  using T = TT;
  using U = typename std::make_unsigned<T>::type;
  using Acc = U;
  using Part = U;
  static __device__ Acc identity() { return U(0); }
  static __device__ void add(Acc& a, T v, int64_t) { a += U(v); }
  static __device__ void add2(Acc& a, T x, T y) { a += U(x) * U(y); }
  static __device__ Acc merge(Acc a, Acc b) { return a + b; }
  static __device__ Part to_part(Acc a) { return a; }
  static __device__ Part part_identity() { return U(0); }
  static __device__ Part merge_part(Part a, Part b) { return a + b; }
  static __device__ void store(OutPtrs o, Part p) { *static_cast<T*>(o.val) = T(p); }
};

template <class T>
struct ValIdx {
  T v;
  int64_t i;
};

// Min / Max with location; ties resolve to the lowest index.
template <class TT, bool MIN, bool WITH_LOC>
struct Extremum {
  using T = TT;
  using Acc = ValIdx<T>;
  using Part = Acc;
  static __device__ bool better(T cand, T cur) { return MIN ? (cand < cur) : (cur < cand); }
  static __device__ Acc identity() { return {MIN ? Lim<T>::hi() : Lim<T>::lo(), -1}; }
  static __device__ void add(Acc& a, T v, int64_t i) {
    // Indices reach a thread in ascending order: strict comparison keeps
    // the first occurrence.
    if (better(v, a.v)) { a.v = v; a.i = i; }
  }
  static __device__ void add2(Acc&, T, T) {}
  static __device__ Acc merge(Acc a, Acc b) {
    if (better(b.v, a.v) || (b.v == a.v && b.i < a.i)) return b;
    return a;
  }
  static __device__ Part to_part(Acc a) { return a; }
  static __device__ Part part_identity() { return identity(); }
  static __device__ Part merge_part(Part a, Part b) { return merge(a, b); }
  static __device__ void store(OutPtrs o, Part p) {
    *static_cast<T*>(o.val) = p.v;
    if (WITH_LOC) *o.idx = p.i;
  }
};

// FP64 Min / Max with location, compared on the integer pipes.  GB300's
// FP64 unit retires far fewer DSETP than the HBM stream delivers doubles,
// so each double is mapped to an order-preserving int64 key instead: the
// bits of negative values except the sign are inverted and one is added,
// which also folds -0.0 onto +0.0 (they compare equal, as with
// operator<).  NaNs are skipped (operator< never selects them): a chunk is
// tested once for an all-ones exponent, and only chunks holding an
// infinity or a NaN take the per-element test.  Per thread only the key
// and the index are carried; the value's bits are rebuilt from the key when
// the thread's result becomes a partial, except for a zero winner, whose
// bits are read back from the input so that -0.0 keeps its sign.  Ties
// resolve to the lowest index as above.
template <bool MIN, bool WITH_LOC>
struct ExtremumF64 {
  using T = double;
  static constexpr bool CHUNKED = true;
  struct Acc {
    long long key;
    long long i;
  };
  struct Part {
    long long key;
    long long i;
    long long bits;
  };
  static __device__ __forceinline__ long long key_of(long long b) {
    const long long s = b >> 63;  // 0 or -1
    return (b ^ (s & 0x7fffffffffffffffll)) - s;
  }
  static __device__ __forceinline__ bool is_nan(long long b) {
    return (b & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
  }
  static __device__ __forceinline__ long long ident_bits() {
    return __double_as_longlong(MIN ? DBL_MAX : -DBL_MAX);
  }
  static __device__ __forceinline__ bool better(long long k, long long than) {
    return MIN ? (k < than) : (than < k);
  }
  static __device__ Acc identity() { return {key_of(ident_bits()), -1}; }
  static __device__ void add(Acc& a, double v, int64_t i) {
    const long long b = __double_as_longlong(v);
    if (is_nan(b)) return;
    const long long k = key_of(b);
    if (better(k, a.key)) { a.key = k; a.i = i; }
  }
  static __device__ void add2(Acc&, double, double) {}
  // Elements (j, k) of the chunk sit at e0 + j * stride + k, in index order.
  static __device__ __forceinline__ void add_chunk(Acc& a, const Vec16<double>* v, size_t e0,
                                                   size_t stride) {
    long long b[8];
    bool special = false;
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        b[2 * j + k] = __double_as_longlong(v[j].v[k]);
        special |= (uint32_t(b[2 * j + k] >> 32) & 0x7ff00000u) == 0x7ff00000u;
      }
    if (special) {
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int k = 0; k < 2; ++k) add(a, v[j].v[k], int64_t(e0 + j * stride + k));
      return;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const long long key = key_of(b[2 * j + k]);
        if (better(key, a.key)) { a.key = key; a.i = (long long)(e0 + j * stride + k); }
      }
  }
  // The bits of the winner from its key: key_of is one-to-one except that
  // +0.0 and -0.0 both map to key 0, so only a zero winner is read back
  // from the input (to keep its sign).
  static __device__ __forceinline__ long long bits_of_key(long long k) {
    return k >= 0 ? k : ((k - 1) ^ 0x7fffffffffffffffll);
  }
  static __device__ Part to_part_x(Acc a, const double* x) {
    if (a.i < 0) return {a.key, a.i, ident_bits()};
    return {a.key, a.i, a.key != 0 ? bits_of_key(a.key) : __double_as_longlong(x[a.i])};
  }
  static __device__ Part part_identity() { return {key_of(ident_bits()), -1, ident_bits()}; }
  static __device__ Part merge_part(Part a, Part b) {
    if (better(b.key, a.key) || (b.key == a.key && b.i < a.i)) return b;
    return a;
  }
  static __device__ void store(OutPtrs o, Part p) {
    *static_cast<double*>(o.val) = __longlong_as_double(p.bits);
    if (WITH_LOC) *o.idx = p.i;
  }
};

template <class TT, bool OR>
struct BitOp {
  using T = TT;
  using Acc = T;
  using Part = T;
  static __device__ Acc identity() { return OR ? T(0) : T(~T(0)); }
  static __device__ void add(Acc& a, T v, int64_t) { a = OR ? (a | v) : (a & v); }
  static __device__ void add2(Acc&, T, T) {}
  static __device__ Acc merge(Acc a, Acc b) { return OR ? (a | b) : (a & b); }
  static __device__ Part to_part(Acc a) { return a; }
  static __device__ Part part_identity() { return identity(); }
  static __device__ Part merge_part(Part a, Part b) { return merge(a, b); }
  static __device__ void store(OutPtrs o, Part p) { *static_cast<T*>(o.val) = p; }
};

// Ops whose thread result reads the input back to become a partial.
template <class Op, class = void>
struct HasToPartX : std::false_type {};
template <class Op>
struct HasToPartX<Op, decltype(void(Op::to_part_x(std::declval<typename Op::Acc>(),
                                                  std::declval<const typename Op::T*>())))>
    : std::true_type {};
template <class Op>
__device__ __forceinline__ typename Op::Part part_of(typename Op::Acc a, const typename Op::T* x) {
  if constexpr (HasToPartX<Op>::value) return Op::to_part_x(a, x);
  else return Op::to_part(a);
}

// Ops that reduce a whole chunk of a thread's full-vector loads at once.
template <class Op, class = void>
struct IsChunked : std::false_type {};
template <class Op>
struct IsChunked<Op, typename std::enable_if<Op::CHUNKED>::type> : std::true_type {};

// Fixed-shape block reduction: butterfly inside each warp, then warp 0
// combines the warp results in warp order.  Result valid in thread 0.
template <class X, class F>
__device__ __forceinline__ X block_reduce(X v, X ident, F merge, X* sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = merge(v, shfl_xor_any(v, o));
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = (lane < RBLOCK / 32) ? sh[lane] : ident;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = merge(v, shfl_xor_any(v, o));
  }
  __syncthreads();
  return v;
}

template <class Op, bool DOT>
__global__ void __launch_bounds__(RBLOCK)
reduce_kernel(const typename Op::T* __restrict__ x, const typename Op::T* __restrict__ y,
              size_t n, int vec_ok, int det, typename Op::Part* __restrict__ parts,
              unsigned int* ticket, OutPtrs out) {
  using T = typename Op::T;
  using Acc = typename Op::Acc;
  using Part = typename Op::Part;
  using C = Chunk<T>;
  __shared__ Part sh_part[32];
  __shared__ bool am_last;

  const int tid = threadIdx.x;
  const size_t nchunks = (n + C::SIZE - 1) / C::SIZE;
  Acc acc = Op::identity();

  for (size_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const size_t base = c * C::SIZE;
    if (det) acc = Op::identity();
    if (vec_ok && base + C::SIZE <= n) {
      Vec16<T> vx[C::NV], vy[C::NV];
#pragma unroll
      for (int j = 0; j < C::NV; ++j) {
        const size_t e = base + (size_t(j) * RBLOCK + tid) * C::VN;
        vx[j] = ld_vec(x + e);
        if (DOT) vy[j] = ld_vec(y + e);
      }
      if constexpr (!DOT && IsChunked<Op>::value) {
        Op::add_chunk(acc, vx, base + size_t(tid) * C::VN, size_t(RBLOCK) * C::VN);
      } else {
#pragma unroll
        for (int j = 0; j < C::NV; ++j) {
          const size_t e = base + (size_t(j) * RBLOCK + tid) * C::VN;
#pragma unroll
          for (int k = 0; k < C::VN; ++k) {
            if (DOT) Op::add2(acc, vx[j].v[k], vy[j].v[k]);
            else Op::add(acc, vx[j].v[k], int64_t(e + k));
          }
        }
      }
    } else {
      // Same element-to-thread mapping (and, for chunked ops, the same
      // chunk arithmetic on full chunks) as the vector path, so the
      // deterministic mode does not depend on pointer alignment.
      bool chunk_done = false;
      if constexpr (!DOT && IsChunked<Op>::value) {
        if (base + C::SIZE <= n) {
          Vec16<T> vx[C::NV];
#pragma unroll
          for (int j = 0; j < C::NV; ++j) {
            const size_t e = base + (size_t(j) * RBLOCK + tid) * C::VN;
#pragma unroll
            for (int k = 0; k < C::VN; ++k) vx[j].v[k] = x[e + k];
          }
          Op::add_chunk(acc, vx, base + size_t(tid) * C::VN, size_t(RBLOCK) * C::VN);
          chunk_done = true;
        }
      }
      if (!chunk_done) {
#pragma unroll
        for (int j = 0; j < C::NV; ++j) {
          const size_t e = base + (size_t(j) * RBLOCK + tid) * C::VN;
#pragma unroll
          for (int k = 0; k < C::VN; ++k) {
            if (e + k < n) {
              if (DOT) Op::add2(acc, x[e + k], y[e + k]);
              else Op::add(acc, x[e + k], int64_t(e + k));
            }
          }
        }
      }
    }
    if (det) {
      const Part r = block_reduce(part_of<Op>(acc, x), Op::part_identity(),
                                  [](Part a, Part b) { return Op::merge_part(a, b); }, sh_part);
      if (tid == 0) parts[c] = r;
    }
  }
  if (!det) {
    const Part r = block_reduce(part_of<Op>(acc, x), Op::part_identity(),
                                [](Part a, Part b) { return Op::merge_part(a, b); }, sh_part);
    if (tid == 0) parts[blockIdx.x] = r;
  }

  // Last-block combine (reduce.hpp:133-214 restated): publish, take a
  // ticket, and let the final block fold the partials in index order.
  if (tid == 0) {
    __threadfence();
    unsigned int prev = atomicAdd(ticket, 1u);
    am_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  const size_t nparts = det ? nchunks : size_t(gridDim.x);
  Part p = Op::part_identity();
  for (size_t i = tid; i < nparts; i += RBLOCK) p = Op::merge_part(p, ld_cg_any(parts + i));
  p = block_reduce(p, Op::part_identity(), [](Part a, Part b) { return Op::merge_part(a, b); }, sh_part);
  if (tid == 0) {
    Op::store(out, p);
    *ticket = 0u;  // leave the ticket zeroed for the next call on this stream
  }
}

template <class Op, bool DOT>
int grid_for(size_t n, int* grid) {
  static KernelSetup ks;
  DeviceProps props;
  B200_TRY(device_props(&props));
  int blocks_per_sm = 0;
  B200_TRY(kernel_setup(ks, props, reduce_kernel<Op, DOT>, RBLOCK, 0, &blocks_per_sm));
  const size_t nchunks = (n + Chunk<typename Op::T>::SIZE - 1) / Chunk<typename Op::T>::SIZE;
  size_t g = size_t(props.sms) * size_t(blocks_per_sm);
  if (g > nchunks) g = nchunks;
  if (g < 1) g = 1;
  *grid = int(g);
  return B200_OK;
}

template <class Op, bool DOT>
int run_reduce(const char* name, const typename Op::T* x, const typename Op::T* y, size_t n,
               bool det, OutPtrs out, b200_stream_t stream) {
  using T = typename Op::T;
  if (!out.val) return fail(B200_ERR_ARG, "%s: null output pointer", name);
  if (n > 0 && (!x || (DOT && !y))) return fail(B200_ERR_ARG, "%s: null input pointer", name);
  if (n >= (size_t(1) << 40)) return fail(B200_ERR_ARG, "%s: n=%zu too large", name, n);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int grid = 1;
  B200_TRY((grid_for<Op, DOT>(n, &grid)));
  const size_t nchunks = (n + Chunk<T>::SIZE - 1) / Chunk<T>::SIZE;
  const size_t nparts = det ? (nchunks > 0 ? nchunks : 1) : size_t(grid);
  void* scr = nullptr;
  uint32_t* counters = nullptr;
  B200_TRY(scratch(s, nparts * sizeof(typename Op::Part), &scr, &counters));
  const bool vec_ok = (reinterpret_cast<uintptr_t>(x) % 16 == 0) &&
                      (!DOT || reinterpret_cast<uintptr_t>(y) % 16 == 0);
  B200_LAUNCH(name, (reduce_kernel<Op, DOT>), grid, RBLOCK, 0, s, x, y, n, int(vec_ok),
              int(det), static_cast<typename Op::Part*>(scr), counters, out);
  clear_error();
  return B200_OK;
}

template <class T>
int sum_fp(const char* name, const T* x, const T* y, size_t n, int mode, double* out,
           b200_stream_t stream) {
  if (mode & ~(B200_MODE_COMPENSATED | B200_MODE_DETERMINISTIC))
    return fail(B200_ERR_ARG, "%s: unknown mode %d", name, mode);
  const bool det = (mode & B200_MODE_DETERMINISTIC) != 0;
  OutPtrs o{out, nullptr};
  if (mode & B200_MODE_COMPENSATED) {
    using Op = typename std::conditional<std::is_same<T, float>::value, SumCompF32, SumCompF64>::type;
    return y ? run_reduce<Op, true>(name, x, y, n, det, o, stream)
             : run_reduce<Op, false>(name, x, y, n, det, o, stream);
  }
  using Naive = typename std::conditional<std::is_same<T, double>::value, SumF64Aligned<F64_DADD>,
                                          SumNaive<T>>::type;
  return y ? run_reduce<SumNaive<T>, true>(name, x, y, n, det, o, stream)
           : run_reduce<Naive, false>(name, x, y, n, det, o, stream);
}

template <class T>
int sum_int(const char* name, const T* x, size_t n, int mode, T* out, b200_stream_t stream) {
  if (mode & ~(B200_MODE_COMPENSATED | B200_MODE_DETERMINISTIC))
    return fail(B200_ERR_ARG, "%s: unknown mode %d", name, mode);
  // Integer sums are exact modulo 2^bits in every mode.
  return run_reduce<SumInt<T>, false>(name, x, nullptr, n, false, OutPtrs{out, nullptr}, stream);
}

}  // namespace
}  // namespace b200

using namespace b200;

extern "C" {

int b200_reduce_sum_f32(const float* x, size_t n, int mode, double* out, b200_stream_t s) {
  return sum_fp<float>("b200_reduce_sum_f32", x, nullptr, n, mode, out, s);
}
int b200_reduce_sum_f64(const double* x, size_t n, int mode, double* out, b200_stream_t s) {
  return sum_fp<double>("b200_reduce_sum_f64", x, nullptr, n, mode, out, s);
}
int b200_dot_f32(const float* x, const float* y, size_t n, int mode, double* out, b200_stream_t s) {
  if (n > 0 && !y) return fail(B200_ERR_ARG, "b200_dot_f32: null y");
  return sum_fp<float>("b200_dot_f32", x, y ? y : x, n, mode, out, s);
}
int b200_dot_f64(const double* x, const double* y, size_t n, int mode, double* out, b200_stream_t s) {
  if (n > 0 && !y) return fail(B200_ERR_ARG, "b200_dot_f64: null y");
  return sum_fp<double>("b200_dot_f64", x, y ? y : x, n, mode, out, s);
}
int b200_reduce_sum_i32(const int32_t* x, size_t n, int mode, int32_t* out, b200_stream_t s) {
  return sum_int<int32_t>("b200_reduce_sum_i32", x, n, mode, out, s);
}
int b200_reduce_sum_i64(const int64_t* x, size_t n, int mode, int64_t* out, b200_stream_t s) {
  return sum_int<int64_t>("b200_reduce_sum_i64", x, n, mode, out, s);
}
int b200_reduce_sum_u32(const uint32_t* x, size_t n, int mode, uint32_t* out, b200_stream_t s) {
  return sum_int<uint32_t>("b200_reduce_sum_u32", x, n, mode, out, s);
}
int b200_reduce_sum_u64(const uint64_t* x, size_t n, int mode, uint64_t* out, b200_stream_t s) {
  return sum_int<uint64_t>("b200_reduce_sum_u64", x, n, mode, out, s);
}

#define B200_MINMAX(NAME, T, MIN)                                                        \
  int b200_reduce_##NAME(const T* x, size_t n, T* out, b200_stream_t s) {                \
    return run_reduce<Extremum<T, MIN, false>, false>("b200_reduce_" #NAME, x, nullptr, n, \
                                                      false, OutPtrs{out, nullptr}, s);  \
  }
#define B200_MINMAX_F64(NAME, MIN)                                                        \
  int b200_reduce_##NAME(const double* x, size_t n, double* out, b200_stream_t s) {        \
    return run_reduce<ExtremumF64<MIN, false>, false>("b200_reduce_" #NAME, x, nullptr, n,  \
                                                      false, OutPtrs{out, nullptr}, s);    \
  }
B200_MINMAX(min_f32, float, true)
B200_MINMAX_F64(min_f64, true)
B200_MINMAX(min_i32, int32_t, true)
B200_MINMAX(min_i64, int64_t, true)
B200_MINMAX(min_u32, uint32_t, true)
B200_MINMAX(min_u64, uint64_t, true)
B200_MINMAX(max_f32, float, false)
B200_MINMAX_F64(max_f64, false)
B200_MINMAX(max_i32, int32_t, false)
B200_MINMAX(max_i64, int64_t, false)
B200_MINMAX(max_u32, uint32_t, false)
B200_MINMAX(max_u64, uint64_t, false)
#undef B200_MINMAX

#define B200_LOC(NAME, T, MIN)                                                            \
  int b200_reduce_##NAME(const T* x, size_t n, T* val, int64_t* idx, b200_stream_t s) {   \
    if (!idx) return fail(B200_ERR_ARG, "b200_reduce_" #NAME ": null index pointer");      \
    return run_reduce<Extremum<T, MIN, true>, false>("b200_reduce_" #NAME, x, nullptr, n,  \
                                                     false, OutPtrs{val, idx}, s);        \
  }
B200_LOC(minloc_f32, float, true)
#define B200_LOC_F64(NAME, MIN)                                                           \
  int b200_reduce_##NAME(const double* x, size_t n, double* val, int64_t* idx,              \
                         b200_stream_t s) {                                                 \
    if (!idx) return fail(B200_ERR_ARG, "b200_reduce_" #NAME ": null index pointer");       \
    return run_reduce<ExtremumF64<MIN, true>, false>("b200_reduce_" #NAME, x, nullptr, n,   \
                                                     false, OutPtrs{val, idx}, s);         \
  }
B200_LOC_F64(minloc_f64, true)
B200_LOC(minloc_i32, int32_t, true)
B200_LOC(minloc_i64, int64_t, true)
B200_LOC(maxloc_f32, float, false)
B200_LOC_F64(maxloc_f64, false)
B200_LOC(maxloc_i32, int32_t, false)
B200_LOC(maxloc_i64, int64_t, false)
#undef B200_LOC

#define B200_BIT(NAME, T, OR)                                                             \
  int b200_reduce_##NAME(const T* x, size_t n, T* out, b200_stream_t s) {                 \
    return run_reduce<BitOp<T, OR>, false>("b200_reduce_" #NAME, x, nullptr, n, false,     \
                                           OutPtrs{out, nullptr}, s);                     \
  }
B200_BIT(bitor_i32, int32_t, true)
B200_BIT(bitor_i64, int64_t, true)
B200_BIT(bitor_u32, uint32_t, true)
B200_BIT(bitor_u64, uint64_t, true)
B200_BIT(bitand_i32, int32_t, false)
B200_BIT(bitand_i64, int64_t, false)
B200_BIT(bitand_u32, uint32_t, false)
B200_BIT(bitand_u64, uint64_t, false)
#undef B200_BIT

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free FP64 sum.
//
// Some callers cannot let a library allocate device memory.  A host whose
// memory manager owns the whole GPU -- it reserves all of HBM up front and
// hands out slices itself -- has no room for a second allocator.  A
// latency-critical loop cannot afford the allocator calls, which may
// synchronise the device.  b200_reduce_sum_f64_noalloc serves both: it is
// b200_reduce_sum_f64 with its scratch (the per-block partials and the
// completion ticket) taken from the file-scope device array below instead
// of the per-stream arena.  The caller still passes the input and the
// output.  It calls no cudaMalloc, cudaFree or other allocating routine.
// It runs the same kernel, grid and chunk mapping as b200_reduce_sum_f64,
// so the two return identical bits for the same input and mode.
//
// Limits: the array holds kNoAllocParts partials of up to 16 bytes.  The
// naive and compensated modes use one partial per block and fit on any
// GPU; the deterministic mode uses one partial per 2048-element chunk, so
// it accepts n <= kNoAllocParts * 2048 and rejects larger n.
//
// The array exists once per GPU that loads the library and stays resident
// until the process exits.  Every call on that GPU shares it and it keeps
// the last call's contents, so the ticket is cleared before each launch.
// Calls that overlap on the GPU (issued on different streams without
// ordering between them) race on the array and give wrong results.
namespace {
constexpr size_t kNoAllocParts = 8192;
constexpr size_t kNoAllocPartBytes = kNoAllocParts * 16;
constexpr size_t kNoAllocBytes = kNoAllocPartBytes + 256;  // partials, then the ticket
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_addr[64] = {};

// Device address of g_noalloc_scratch on the current device.  In host code
// the symbol is only a stand-in, so its address is looked up once per
// device (with that device current) on the first call there.
int noalloc_scratch(unsigned char** out) {
  int dev = 0;
  B200_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(B200_ERR_ARG, "device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_check(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_addr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_noalloc_addr[dev]);
  return B200_OK;
}

template <class Op>
int run_reduce_noalloc(const char* name, const double* x, size_t n, bool det, double* out,
                       b200_stream_t stream) {
  if (!out) return fail(B200_ERR_ARG, "%s: null output pointer", name);
  if (n > 0 && !x) return fail(B200_ERR_ARG, "%s: null input pointer", name);
  if (n >= (size_t(1) << 40)) return fail(B200_ERR_ARG, "%s: n=%zu too large", name, n);
  static_assert(sizeof(typename Op::Part) <= 16, "partials fit the 16-byte slots");
  const size_t chunk = Chunk<double>::SIZE;
  const size_t nchunks = (n + chunk - 1) / chunk;
  if (det && nchunks > kNoAllocParts)
    return fail(B200_ERR_ARG,
                "%s: n=%zu exceeds the deterministic-mode maximum of %zu elements "
                "(%zu partials of static scratch)",
                name, n, kNoAllocParts * chunk, kNoAllocParts);
  int grid = 1;
  B200_TRY((grid_for<Op, false>(n, &grid)));
  if (size_t(grid) > kNoAllocParts) grid = int(kNoAllocParts);
  unsigned char* base = nullptr;
  B200_TRY(noalloc_scratch(&base));
  auto* parts = reinterpret_cast<typename Op::Part*>(base);
  auto* ticket = reinterpret_cast<unsigned int*>(base + kNoAllocPartBytes);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  B200_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned int), s));
  const bool vec_ok = reinterpret_cast<uintptr_t>(x) % 16 == 0;
  B200_LAUNCH(name, (reduce_kernel<Op, false>), grid, RBLOCK, 0, s, x, x, n, int(vec_ok), int(det),
              parts, ticket, OutPtrs{out, nullptr});
  clear_error();
  return B200_OK;
}
}  // namespace

extern "C" int b200_reduce_sum_f64_noalloc(const double* x, size_t n, int mode, double* out,
                                           b200_stream_t stream) {
  const char* name = "b200_reduce_sum_f64_noalloc";
  if (mode & ~(B200_MODE_COMPENSATED | B200_MODE_DETERMINISTIC))
    return fail(B200_ERR_ARG, "%s: unknown mode %d", name, mode);
  const bool det = (mode & B200_MODE_DETERMINISTIC) != 0;
  if (mode & B200_MODE_COMPENSATED) return run_reduce_noalloc<SumCompF64>(name, x, n, det, out, stream);
  // the same Op as b200_reduce_sum_f64 (exponent-aligned int64 chunk sums),
  // so both entry points give the same bits for the same input and mode
  return run_reduce_noalloc<SumF64Aligned<F64_DADD>>(name, x, n, det, out, stream);
}
