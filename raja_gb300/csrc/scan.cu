// Inclusive / exclusive scans (in place when in == out).
//
// Reference: impl::scan::{inclusive,exclusive}[_inplace]
// (policy/cuda/scan.hpp:45-235) -> cub::DeviceScan with a temp-size query,
// a pool allocation and a sync; seq semantics in
// policy/sequential/scan.hpp:43-153 (left fold; exclusive writes init
// first, then init op x0, ...).
//
// GB300 design: one single-pass kernel with decoupled look-back (Merrill &
// Garland, "Single-pass Parallel Prefix Scan with Decoupled Look-back",
// NVIDIA TR 2016).  A tile is 256 threads x 64 bytes.  Tiles take their id
// from an atomic counter in launch order, so every predecessor of a tile
// has already started and will publish its aggregate without waiting on
// anything: the look-back always terminates.  It is still bounded -- after
// spin_limit polls the tile gives up, ORs a code into the device status
// word and finishes, so a broken invariant can never hang the GPU.
// Global traffic is one coalesced 16-byte read and one 16-byte write per
// element group; tiles are transposed through an XOR-swizzled shared
// buffer so every thread scans 64 contiguous bytes without bank conflicts.
// The look-back is done by one warp that inspects 32 predecessors at once.
#include <cfloat>
#include <climits>
#include <type_traits>

#include "b200_internal.cuh"

namespace b200 {
namespace {

constexpr int SBLOCK = 256;
constexpr int SWARPS = SBLOCK / 32;
constexpr uint32_t FLAG_AGG = 1, FLAG_INCL = 2;

template <class T>
struct Tile {
  static constexpr int VN = 16 / sizeof(T);
  static constexpr int ITEMS = 64 / sizeof(T);
  static constexpr int SIZE = SBLOCK * ITEMS;
};

template <class T>
struct Inf;
template <> struct Inf<float> { static __device__ float hi() { return __int_as_float(0x7f800000); } static __device__ float lo() { return __int_as_float(0xff800000); } };
template <> struct Inf<double> { static __device__ double hi() { return __longlong_as_double(0x7ff0000000000000ll); } static __device__ double lo() { return __longlong_as_double(0xfff0000000000000ll); } };
template <> struct Inf<int32_t> { static __device__ int32_t hi() { return INT_MAX; } static __device__ int32_t lo() { return INT_MIN; } };
template <> struct Inf<int64_t> { static __device__ int64_t hi() { return LLONG_MAX; } static __device__ int64_t lo() { return LLONG_MIN; } };
template <> struct Inf<uint32_t> { static __device__ uint32_t hi() { return UINT_MAX; } static __device__ uint32_t lo() { return 0u; } };
template <> struct Inf<uint64_t> { static __device__ uint64_t hi() { return ULLONG_MAX; } static __device__ uint64_t lo() { return 0ull; } };

template <class T>
struct PairT { T s, c; };

// ------------------------------------------------------------ scan ops
// Local: within-tile value; Carry: cross-tile value (look-back).

// Integer sum, wrap-around (exact modulo 2^bits like the seq fold).
template <class TT>
struct ScanSumInt {
  using T = TT;
  using U = typename std::make_unsigned<T>::type;
  using Local = U;
  using Carry = U;
  static __device__ Local ident() { return U(0); }
  static __device__ Local lift(T x) { return U(x); }
  static __device__ Local comb(Local a, Local b) { return a + b; }
  static __device__ Carry cident() { return U(0); }
  static __device__ Carry ccomb(Carry a, Carry b) { return a + b; }
  static __device__ Carry to_carry(Local a) { return a; }
  static __device__ Carry from_init(T v) { return U(v); }
  static __device__ T out_local(Local l) { return T(l); }
  static __device__ T out(Carry p, Local l) { return T(p + l); }
  static __device__ T out_prefix(Carry p) { return T(p); }
};

// Min / max with RAJA's operator: (rhs < lhs) ? rhs : lhs (min) and
// (lhs < rhs) ? rhs : lhs (max).  +-inf are exact identities for every
// non-NaN input.
template <class TT, bool MIN>
struct ScanMinMax {
  using T = TT;
  using Local = T;
  using Carry = T;
  static __device__ T op(T a, T b) { return MIN ? ((b < a) ? b : a) : ((a < b) ? b : a); }
  static __device__ Local ident() { return MIN ? Inf<T>::hi() : Inf<T>::lo(); }
  static __device__ Local lift(T x) { return x; }
  static __device__ Local comb(Local a, Local b) { return op(a, b); }
  static __device__ Carry cident() { return ident(); }
  static __device__ Carry ccomb(Carry a, Carry b) { return op(a, b); }
  static __device__ Carry to_carry(Local a) { return a; }
  static __device__ Carry from_init(T v) { return v; }
  static __device__ T out_local(Local l) { return l; }
  static __device__ T out(Carry p, Local l) { return op(p, l); }
  static __device__ T out_prefix(Carry p) { return p; }
};

// Naive floating-point sum (element precision).  -0.0 is the identity so
// that a leading -0.0 survives bit for bit.
template <class TT>
struct ScanSumFP {
  using T = TT;
  using Local = T;
  using Carry = T;
  static __device__ Local ident() { return T(-0.0); }
  static __device__ Local lift(T x) { return x; }
  static __device__ Local comb(Local a, Local b) { return a + b; }
  static __device__ Carry cident() { return T(-0.0); }
  static __device__ Carry ccomb(Carry a, Carry b) { return a + b; }
  static __device__ Carry to_carry(Local a) { return a; }
  static __device__ Carry from_init(T v) { return v; }
  static __device__ T out_local(Local l) { return l; }
  static __device__ T out(Carry p, Local l) { return p + l; }
  static __device__ T out_prefix(Carry p) { return p; }
};

// Compensated FP32 sum: TwoSum pairs inside the tile, FP64 carry between
// tiles.  The carry is applied per element as a float-float pair, so the
// per-element work stays on the FP32 pipes.
struct ScanSumCompF32 {
  using T = float;
  using Local = PairT<float>;
  using Carry = double;
  static __device__ Local ident() { return {-0.0f, 0.0f}; }
  static __device__ Local lift(float x) { return {x, 0.0f}; }
  static __device__ Local comb(Local a, Local b) {
    float s, e;
    two_sum(a.s, b.s, s, e);
    return {s, a.c + b.c + e};
  }
  static __device__ Carry cident() { return -0.0; }
  static __device__ Carry ccomb(Carry a, Carry b) { return a + b; }
  static __device__ Carry to_carry(Local a) { return double(a.s) + double(a.c); }
  static __device__ Carry from_init(float v) { return double(v); }
  static __device__ float out_local(Local l) { return l.s + l.c; }
  static __device__ float out(Carry p, Local l) {
    // p as float-float (hi, lo), then hi + l.s with TwoSum.
    const float hi = float(p);
    const float lo = float(p - double(hi));
    float s, e;
    two_sum(hi, l.s, s, e);
    return s + (e + (lo + l.c));
  }
  static __device__ float out_prefix(Carry p) { return float(p); }
};

// Compensated FP64 sum: double-double throughout.
struct ScanSumCompF64 {
  using T = double;
  using Local = PairT<double>;
  using Carry = PairT<double>;
  static __device__ Local ident() { return {-0.0, 0.0}; }
  static __device__ Local lift(double x) { return {x, 0.0}; }
  static __device__ Local comb(Local a, Local b) {
    double s, e;
    two_sum(a.s, b.s, s, e);
    return {s, a.c + b.c + e};
  }
  static __device__ Carry cident() { return ident(); }
  static __device__ Carry ccomb(Carry a, Carry b) { return comb(a, b); }
  static __device__ Carry to_carry(Local a) { return a; }
  static __device__ Carry from_init(double v) { return {v, 0.0}; }
  static __device__ double out_local(Local l) { return l.s + l.c; }
  static __device__ double out(Carry p, Local l) {
    Local r = comb(p, l);
    return r.s + r.c;
  }
  static __device__ double out_prefix(Carry p) { return p.s + p.c; }
};

// Carry folded with a thread-local prefix (once per thread).
template <class Op>
__device__ __forceinline__ typename Op::Carry fold_local(typename Op::Carry p, typename Op::Local l) {
  return Op::ccomb(p, Op::to_carry(l));
}
template <>
__device__ __forceinline__ double fold_local<ScanSumCompF32>(double p, PairT<float> l) {
  return p + (double(l.s) + double(l.c));
}

// XOR swizzle of 16-byte granules within groups of eight: conflict-free
// for both the warp-striped (global side) and per-thread (scan side) views.
template <class T>
__device__ __forceinline__ int swz(int e) {
  constexpr int VN = 16 / sizeof(T);
  const int g = e / VN;
  return ((g ^ ((g >> 3) & 7)) * VN) + (e % VN);
}

template <class P>
__device__ __forceinline__ P ld_cg_val(const P* p) {
  static_assert(sizeof(P) % 4 == 0, "carry size");
  constexpr int W = sizeof(P) / 4;
  uint32_t w[W];
  const uint32_t* q = reinterpret_cast<const uint32_t*>(p);
#pragma unroll
  for (int i = 0; i < W; ++i) w[i] = __ldcg(q + i);
  P r;
  memcpy(&r, w, sizeof(P));
  return r;
}

template <class Op, bool EXCL>
__global__ void __launch_bounds__(SBLOCK)
scan_kernel(const typename Op::T* in, typename Op::T* out, size_t n, typename Op::T init,
            int vec_ok, uint32_t* flags, typename Op::Carry* aggs, typename Op::Carry* incls,
            uint32_t* tile_counter, uint32_t* status, uint32_t spin_limit) {
  using T = typename Op::T;
  using Local = typename Op::Local;
  using Carry = typename Op::Carry;
  constexpr int VN = Tile<T>::VN, ITEMS = Tile<T>::ITEMS, TS = Tile<T>::SIZE;
  __shared__ __align__(16) T sm[TS];
  __shared__ Local sh_warp[SWARPS];
  __shared__ Carry sh_prefix;
  __shared__ uint32_t sh_tile;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) sh_tile = atomicAdd(tile_counter, 1u);
  __syncthreads();
  const size_t tile = sh_tile;
  const size_t base = tile * TS;
  const bool full = base + TS <= n;

  // ---- load the tile (coalesced) into swizzled shared memory
  if (full && vec_ok) {
#pragma unroll
    for (int j = 0; j < ITEMS / VN; ++j) {
      const int g = j * SBLOCK + tid;
      Vec16<T> v = ld_vec_stream(in + base + size_t(g) * VN);
      *reinterpret_cast<Vec16<T>*>(&sm[swz<T>(g * VN)]) = v;
    }
  } else {
    for (int e = tid; e < TS; e += SBLOCK) {
      const size_t i = base + e;
      sm[swz<T>(e)] = (i < n) ? in[i] : T(0);
    }
  }
  __syncthreads();

  // ---- per-thread sequential scan of 64 contiguous bytes
  Local loc[ITEMS];
  const int first = tid * ITEMS;
  {
    T xs[ITEMS];
#pragma unroll
    for (int q = 0; q < ITEMS / VN; ++q) {
      // 16-byte shared reads: conflict-free under the swizzle
      const Vec16<T> v = *reinterpret_cast<const Vec16<T>*>(&sm[swz<T>(first + q * VN)]);
#pragma unroll
      for (int k = 0; k < VN; ++k) xs[q * VN + k] = v.v[k];
    }
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      const size_t i = base + first + k;
      const Local v = (i < n) ? Op::lift(xs[k]) : Op::ident();
      loc[k] = (k == 0) ? v : Op::comb(loc[k - 1], v);
    }
  }

  // ---- warp inclusive scan of thread totals
  Local tot = loc[ITEMS - 1];
  Local inc = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    Local other = shfl_up_any(inc, o);
    if (lane >= o) inc = Op::comb(other, inc);
  }
  Local lane_excl = shfl_up_any(inc, 1);
  if (lane == 31) sh_warp[warp] = inc;
  __syncthreads();

  // ---- block: warp prefix and tile aggregate
  Local tile_agg = sh_warp[0];
  Local warp_excl = Op::ident();
#pragma unroll
  for (int w = 1; w < SWARPS; ++w) {
    if (w == warp) warp_excl = tile_agg;
    tile_agg = Op::comb(tile_agg, sh_warp[w]);
  }
  // thread prefix inside the tile (absent for thread 0)
  const bool has_tp = tid != 0;
  Local tp;
  if (warp == 0) tp = lane_excl;
  else tp = (lane == 0) ? warp_excl : Op::comb(warp_excl, lane_excl);

  // ---- publish and look back (warp 0)
  if (warp == 0) {
    Carry prefix = Op::cident();
    bool have = false;
    if (tile == 0) {
      if (EXCL) { prefix = Op::from_init(init); have = true; }
      if (lane == 0) {
        incls[0] = have ? Op::ccomb(prefix, Op::to_carry(tile_agg)) : Op::to_carry(tile_agg);
        st_release(flags, FLAG_INCL);
      }
    } else {
      if (lane == 0) {
        aggs[tile] = Op::to_carry(tile_agg);
        st_release(flags + tile, FLAG_AGG);
      }
      long long pred = (long long)tile - 1;
      Carry acc = Op::cident();
      bool timed_out = false;
      while (true) {
        const long long t = pred - lane;
        uint32_t f = (t >= 0) ? ld_acquire(flags + t) : FLAG_INCL;
        uint32_t spins = 0;
        while (!__all_sync(0xffffffffu, f != 0)) {
          if (f == 0) f = ld_acquire(flags + t);
          if (++spins > spin_limit) { timed_out = true; break; }
          if (spins > 8) __nanosleep(64);
        }
        timed_out = __any_sync(0xffffffffu, timed_out);
        if (timed_out) break;
        const uint32_t im = __ballot_sync(0xffffffffu, f == FLAG_INCL);
        const int stop = im ? (__ffs(im) - 1) : 32;
        Carry v = Op::cident();
        if (lane < stop) v = ld_cg_val(aggs + t);
        else if (lane == stop) v = ld_cg_val(incls + t);
        // ordered combine: higher lane = earlier tile
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          Carry other = shfl_idx_any(v, (lane + o) & 31);
          if (lane + o < 32) v = Op::ccomb(other, v);
        }
        const Carry window = shfl_idx_any(v, 0);
        acc = Op::ccomb(window, acc);
        if (im) break;
        pred -= 32;
      }
      if (timed_out && lane == 0) atomicOr(status, kStatusScanTimeout);
      prefix = acc;
      have = true;
      if (lane == 0) {
        incls[tile] = Op::ccomb(prefix, Op::to_carry(tile_agg));
        st_release(flags + tile, FLAG_INCL);
      }
    }
    if (lane == 0) sh_prefix = prefix;
    (void)have;
  }
  __syncthreads();

  // ---- combine prefixes and write outputs into shared memory
  const bool tile_has_prefix = EXCL || tile > 0;
  Carry P = sh_prefix;
  bool hasP = tile_has_prefix;
  if (has_tp) {
    if (hasP) P = fold_local<Op>(P, tp);
    else P = Op::to_carry(tp);
    hasP = true;
  }
#pragma unroll
  for (int q = 0; q < ITEMS / VN; ++q) {
    Vec16<T> v;
#pragma unroll
    for (int kk = 0; kk < VN; ++kk) {
      const int k = q * VN + kk;
      T r;
      if (EXCL) r = (k == 0) ? Op::out_prefix(P) : Op::out(P, loc[k - 1]);
      else r = hasP ? Op::out(P, loc[k]) : Op::out_local(loc[k]);
      v.v[kk] = r;
    }
    *reinterpret_cast<Vec16<T>*>(&sm[swz<T>(first + q * VN)]) = v;
  }
  __syncthreads();

  // ---- store the tile (coalesced)
  if (full && vec_ok) {
#pragma unroll
    for (int j = 0; j < ITEMS / VN; ++j) {
      const int g = j * SBLOCK + tid;
      Vec16<T> v = *reinterpret_cast<const Vec16<T>*>(&sm[swz<T>(g * VN)]);
      st_vec_stream(out + base + size_t(g) * VN, v);
    }
  } else {
    for (int e = tid; e < TS; e += SBLOCK) {
      const size_t i = base + e;
      if (i < n) out[i] = sm[swz<T>(e)];
    }
  }
}

template <class Op, bool EXCL>
int run_scan(const char* name, const typename Op::T* in, typename Op::T* out, size_t n,
             typename Op::T init, b200_stream_t stream) {
  using T = typename Op::T;
  using Carry = typename Op::Carry;
  if (n == 0) { clear_error(); return B200_OK; }
  if (!in || !out) return fail(B200_ERR_ARG, "%s: null pointer", name);
  if (n >= (size_t(1) << 40)) return fail(B200_ERR_ARG, "%s: n=%zu too large", name, n);
  if (in != out && ((in < out && in + n > out) || (out < in && out + n > in)))
    return fail(B200_ERR_ARG, "%s: input and output overlap partially", name);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t tiles = (n + Tile<T>::SIZE - 1) / Tile<T>::SIZE;
  Sizer z;
  z.take<uint32_t>(tiles + 64);  // flags + tile counter
  z.take<Carry>(tiles);
  z.take<Carry>(tiles);
  void* scr = nullptr;
  B200_TRY(scratch(s, z.bytes(), &scr, nullptr));
  Carver cv(scr);
  uint32_t* flags = cv.take<uint32_t>(tiles + 64);
  Carry* aggs = cv.take<Carry>(tiles);
  Carry* incls = cv.take<Carry>(tiles);
  uint32_t* counter = flags + tiles;
  uint32_t* status = nullptr;
  B200_TRY(status_word(&status));
  B200_CUDA(cudaMemsetAsync(flags, 0, (tiles + 64) * sizeof(uint32_t), s));
  const bool vec_ok = reinterpret_cast<uintptr_t>(in) % 16 == 0 &&
                      reinterpret_cast<uintptr_t>(out) % 16 == 0;
  B200_LAUNCH(name, (scan_kernel<Op, EXCL>), (unsigned)tiles, SBLOCK, 0, s, in, out, n, init,
              int(vec_ok), flags, aggs, incls, counter, status, spin_limit());
  clear_error();
  return B200_OK;
}

template <class T>
int scan_int(const char* name, bool excl, const T* in, T* out, size_t n, int op, T init,
             b200_stream_t s) {
  switch (op) {
    case B200_OP_SUM:
      return excl ? run_scan<ScanSumInt<T>, true>(name, in, out, n, init, s)
                  : run_scan<ScanSumInt<T>, false>(name, in, out, n, init, s);
    case B200_OP_MIN:
      return excl ? run_scan<ScanMinMax<T, true>, true>(name, in, out, n, init, s)
                  : run_scan<ScanMinMax<T, true>, false>(name, in, out, n, init, s);
    case B200_OP_MAX:
      return excl ? run_scan<ScanMinMax<T, false>, true>(name, in, out, n, init, s)
                  : run_scan<ScanMinMax<T, false>, false>(name, in, out, n, init, s);
    default:
      return fail(B200_ERR_ARG, "%s: unknown op %d", name, op);
  }
}

template <class T>
int scan_fp(const char* name, bool excl, const T* in, T* out, size_t n, int op, T init, int mode,
            b200_stream_t s) {
  if (mode & ~(B200_MODE_COMPENSATED | B200_MODE_DETERMINISTIC))
    return fail(B200_ERR_ARG, "%s: unknown mode %d", name, mode);
  if (op == B200_OP_SUM && (mode & B200_MODE_COMPENSATED)) {
    using Op = typename std::conditional<std::is_same<T, float>::value, ScanSumCompF32,
                                         ScanSumCompF64>::type;
    return excl ? run_scan<Op, true>(name, in, out, n, init, s)
                : run_scan<Op, false>(name, in, out, n, init, s);
  }
  switch (op) {
    case B200_OP_SUM:
      return excl ? run_scan<ScanSumFP<T>, true>(name, in, out, n, init, s)
                  : run_scan<ScanSumFP<T>, false>(name, in, out, n, init, s);
    case B200_OP_MIN:
      return excl ? run_scan<ScanMinMax<T, true>, true>(name, in, out, n, init, s)
                  : run_scan<ScanMinMax<T, true>, false>(name, in, out, n, init, s);
    case B200_OP_MAX:
      return excl ? run_scan<ScanMinMax<T, false>, true>(name, in, out, n, init, s)
                  : run_scan<ScanMinMax<T, false>, false>(name, in, out, n, init, s);
    default:
      return fail(B200_ERR_ARG, "%s: unknown op %d", name, op);
  }
}

}  // namespace
}  // namespace b200

using namespace b200;

extern "C" {

#define B200_SCAN_INT(SUF, T)                                                                  \
  int b200_scan_inclusive_##SUF(const T* in, T* out, size_t n, int op, b200_stream_t s) {      \
    return scan_int<T>("b200_scan_inclusive_" #SUF, false, in, out, n, op, T(0), s);           \
  }                                                                                            \
  int b200_scan_exclusive_##SUF(const T* in, T* out, size_t n, int op, T init,                 \
                                b200_stream_t s) {                                             \
    return scan_int<T>("b200_scan_exclusive_" #SUF, true, in, out, n, op, init, s);            \
  }
B200_SCAN_INT(i32, int32_t)
B200_SCAN_INT(i64, int64_t)
B200_SCAN_INT(u32, uint32_t)
B200_SCAN_INT(u64, uint64_t)
#undef B200_SCAN_INT

int b200_scan_inclusive_f32(const float* in, float* out, size_t n, int op, int mode,
                            b200_stream_t s) {
  return scan_fp<float>("b200_scan_inclusive_f32", false, in, out, n, op, 0.f, mode, s);
}
int b200_scan_inclusive_f64(const double* in, double* out, size_t n, int op, int mode,
                            b200_stream_t s) {
  return scan_fp<double>("b200_scan_inclusive_f64", false, in, out, n, op, 0.0, mode, s);
}
int b200_scan_exclusive_f32(const float* in, float* out, size_t n, int op, float init, int mode,
                            b200_stream_t s) {
  return scan_fp<float>("b200_scan_exclusive_f32", true, in, out, n, op, init, mode, s);
}
int b200_scan_exclusive_f64(const double* in, double* out, size_t n, int op, double init,
                            int mode, b200_stream_t s) {
  return scan_fp<double>("b200_scan_exclusive_f64", true, in, out, n, op, init, mode, s);
}

// Self-test of the bounded wait: one block is launched as tile 1 of a scan
// whose tile 0 never runs, so its look-back polls a flag that nothing sets
// until the spin limit, then records kStatusScanTimeout and returns.  The
// next b200_stream_synchronize() must report B200_ERR_TIMEOUT.
int b200_selftest_scan_timeout(b200_stream_t stream) {
  using Op = ScanSumInt<int32_t>;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = 2 * size_t(Tile<int32_t>::SIZE);
  Sizer z;
  z.take<int32_t>(n);
  z.take<uint32_t>(64);
  z.take<uint32_t>(64);
  z.take<uint32_t>(64);
  void* scr = nullptr;
  B200_TRY(scratch(s, z.bytes(), &scr, nullptr));
  Carver cv(scr);
  int32_t* data = cv.take<int32_t>(n);
  uint32_t* flags = cv.take<uint32_t>(64);
  uint32_t* aggs = cv.take<uint32_t>(64);
  uint32_t* incls = cv.take<uint32_t>(64);
  uint32_t* status = nullptr;
  B200_TRY(status_word(&status));
  B200_CUDA(cudaMemsetAsync(data, 0, n * sizeof(int32_t), s));
  B200_CUDA(cudaMemsetAsync(flags, 0, 64 * sizeof(uint32_t), s));
  const uint32_t one = 1;  // the tile counter: the block takes tile id 1
  B200_CUDA(cudaMemcpyAsync(flags + 32, &one, sizeof(one), cudaMemcpyHostToDevice, s));
  B200_CUDA(cudaStreamSynchronize(s));  // `one` lives on this stack frame
  uint32_t lim = spin_limit();
  if (lim > (1u << 16)) lim = 1u << 16;
  B200_LAUNCH("b200_selftest_scan_timeout", (scan_kernel<Op, false>), 1, SBLOCK, 0, s, data, data,
              n, 0, 1, flags, aggs, incls, flags + 32, status, lim);
  clear_error();
  return B200_OK;
}

}  // extern "C"
