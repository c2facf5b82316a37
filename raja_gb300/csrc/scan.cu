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
// NVIDIA TR 2016).  A tile is 256 threads x 128 bytes.  Tiles take their id
// from an atomic counter in launch order, so every predecessor of a tile
// has already started and will publish its aggregate without waiting on
// anything: the look-back always terminates.  It is still bounded -- after
// spin_limit polls the tile gives up, ORs a code into the device status
// word and finishes, so a broken invariant can never hang the GPU.
// Global traffic is one TMA bulk read and one coalesced 16-byte write per
// element group.  A block also prefetches into L2 the tile that will be
// claimed one SM's worth of tiles later, so a block's own TMA load is
// mostly an L2 read and less of its life goes to waiting for its tile.  A tile's status (flag + carry) is published with plain
// relaxed stores and no fences: the carry is cut into 32-bit pieces, each
// stored in a 64-bit word beside a copy of the flag, and a reader accepts a
// status only when every word carries the same non-zero flag -- a torn read
// (words from the aggregate and the inclusive publication, or not yet
// written) shows up as a flag mismatch and is polled again.  Warp 0 does
// the look-back, LBJ predecessors per lane per poll, with a short sleep
// between polls so that the waiting tiles do not flood the L2 slices that
// hold the status words.
#include <cfloat>
#include <climits>
#include <type_traits>

#include "b200_internal.cuh"

namespace b200 {
namespace {

constexpr int SBLOCK = 256;
constexpr int SWARPS = SBLOCK / 32;
constexpr uint32_t FLAG_AGG = 1, FLAG_INCL = 2;

// A tile is 256 threads x G 16-byte granules.  Thread t owns granules
// j*256 + t (j = 0..G-1): consecutive threads touch consecutive granules,
// so both the TMA-filled shared buffer and the global stores are accessed
// without bank conflicts and fully coalesced, with no transposition.
// Tiles are 64 KB (G = 16); the compensated sums, whose in-tile values are
// pairs, use 32 KB tiles to stay within the register budget.  Large tiles matter
// here: each tile pays one look-back of a few L2 round trips, and the
// bytes in flight per SM (three 64 KB tiles) set the bandwidth.
template <class Op>
struct Tile {
  using T = typename Op::T;
  static constexpr int VN = 16 / sizeof(T);   // elements per granule
  static constexpr int G = sizeof(typename Op::Local) > sizeof(T) ? 8 : 16;  // granules per thread
  static constexpr int ITEMS = G * VN;
  static constexpr int SIZE = SBLOCK * ITEMS;
  static constexpr int PT = G * SWARPS / 32;  // prefix-table entries per lane
};
constexpr int LBJ = 1;          // predecessors each look-back lane inspects per poll
constexpr int LB_SLEEP_NS = 64; // pause between polls of a window that is not ready

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

// ---------------------------------------------------- tile status words
// Word = (flag << 32) | 32-bit piece of the carry; NW words per tile.
template <class Carry>
struct StatusWords {
  static_assert(sizeof(Carry) % 4 == 0 && sizeof(Carry) <= 16, "carry size");
  static constexpr int NW = sizeof(Carry) / 4;

  static __device__ __forceinline__ void publish(uint64_t* w, uint32_t flag, const Carry& v) {
    uint32_t piece[NW];
    memcpy(piece, &v, sizeof(Carry));
    const uint64_t f = uint64_t(flag) << 32;
    if (NW == 1) {
      asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(w), "l"(f | piece[0]) : "memory");
    } else {
#pragma unroll
      for (int i = 0; i < NW; i += 2)
        asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(w + i),
                     "l"(f | piece[i]), "l"(f | piece[(i + 1) % NW]) : "memory");
    }
  }
  // The tile's flag if every word agrees on it, else 0 (not ready).
  static __device__ __forceinline__ uint32_t poll(const uint64_t* w, Carry& v) {
    uint64_t x[NW + (NW & 1)];
    if (NW == 1) {
      asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(x[0]) : "l"(w) : "memory");
    } else {
#pragma unroll
      for (int i = 0; i < NW; i += 2)
        asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];"
                     : "=l"(x[i]), "=l"(x[i + 1]) : "l"(w + i) : "memory");
    }
    uint32_t flag = uint32_t(x[0] >> 32);
    uint32_t piece[NW];
#pragma unroll
    for (int i = 0; i < NW; ++i) {
      if (uint32_t(x[i] >> 32) != flag) flag = 0;
      piece[i] = uint32_t(x[i]);
    }
    memcpy(&v, piece, sizeof(Carry));
    return flag;
  }
};

// Per-tile working set of a block besides the tile itself.
template <class Op>
struct ScanWork {
  using Local = typename Op::Local;
  Local wsum[SWARPS];                        // warp totals over the whole tile
  Local wtot[Tile<Op>::G * SWARPS];          // warp totals, sub-tile major
  Local pref[Tile<Op>::G * SWARPS];          // their exclusive prefix in the tile
  typename Op::Carry prefix;                 // the tile's carry-in
};

template <class Op>
struct ScanSmem {
  using T = typename Op::T;
  alignas(128) T stage[Tile<Op>::SIZE];      // the tile, filled by one TMA bulk copy
  ScanWork<Op> work;
  uint64_t bar;
  uint32_t tile;
};

// One tile per block.  Tiles take their id from an atomic counter in
// launch order, so every predecessor of a tile has already started and
// publishes its aggregate without waiting on anything: the look-back
// always terminates.  The tile arrives by one TMA bulk copy (cp.async.bulk
// completed on an mbarrier) straight into shared memory, so no registers
// stage it and five or more blocks fit per SM: while one block waits in its
// look-back, the others keep HBM busy.
// Resident blocks per SM the register budget is cut for: three 64 KB
// tiles fill the shared memory; four 32 KB ones for the compensated sums.
template <class Op>
constexpr int scan_min_blocks() { return Tile<Op>::G == 16 ? 3 : 4; }

// Scan one tile held in shared memory (st) and write its outputs: thread
// totals and the tile aggregate, published at once; the decoupled
// look-back (warp 0) beside the sub-tile scans and the prefix table (warp
// 1); then carry-in + prefixes applied as the outputs are stored.
template <class Op, bool EXCL>
__device__ __forceinline__ void scan_tile(ScanWork<Op>& sm, const typename Op::T* st, size_t tile, size_t n,
                                          typename Op::T init, int vec_out, typename Op::T* out,
                                          uint64_t* words, uint32_t* status, uint32_t spin_limit) {
  using T = typename Op::T;
  using Local = typename Op::Local;
  using Carry = typename Op::Carry;
  constexpr int VN = Tile<Op>::VN, G = Tile<Op>::G, TS = Tile<Op>::SIZE, PT = Tile<Op>::PT;
  static_assert(G * SWARPS == 32 * PT, "prefix table: PT entries per lane of warp 1");
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const size_t base = tile * TS;
  const bool full = base + TS <= n;
  {
    using SW = StatusWords<Carry>;
    // ---- granule totals (registers) and the tile aggregate: thread
    // totals, warp totals, then warp 0 folds the eight warps
    Local lex[G];
#pragma unroll
    for (int j = 0; j < G; ++j) {
      const int g = j * SBLOCK + tid;
      const Vec16<T> v = *reinterpret_cast<const Vec16<T>*>(&st[g * VN]);
      Local tot = Op::ident();
#pragma unroll
      for (int k = 0; k < VN; ++k) {
        const Local x = (full || base + size_t(g) * VN + k < n) ? Op::lift(v.v[k]) : Op::ident();
        tot = (k == 0) ? x : Op::comb(tot, x);
      }
      lex[j] = tot;
    }
    {
      Local tt = lex[0];
#pragma unroll
      for (int j = 1; j < G; ++j) tt = Op::comb(tt, lex[j]);
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const Local other = shfl_up_any(tt, o);
        if (lane >= o) tt = Op::comb(other, tt);
      }
      if (lane == 31) sm.wsum[warp] = tt;
    }
    __syncthreads();

    // ---- warp 0 publishes the aggregate at once and issues the first
    // look-back poll; its latency is hidden behind the sub-tile scans
    Carry tile_agg = Op::cident();
    long long pred = (long long)tile - 1;
    Carry lbv[LBJ];
    uint32_t lbf[LBJ];
    auto load_window = [&](long long t0) {
#pragma unroll
      for (int j = 0; j < LBJ; ++j) {
        if (t0 - j >= 0) {
          lbf[j] = SW::poll(words + (t0 - j) * SW::NW, lbv[j]);
        } else {  // before tile 0: never reached past tile 0's inclusive prefix
          lbf[j] = FLAG_INCL;
          lbv[j] = Op::cident();
        }
      }
    };
    if (warp == 0) {
      Local wt = (lane < SWARPS) ? sm.wsum[lane] : Op::ident();
#pragma unroll
      for (int o = 1; o < SWARPS; o <<= 1) {
        const Local other = shfl_up_any(wt, o);
        if (lane >= o) wt = Op::comb(other, wt);
      }
      tile_agg = Op::to_carry(shfl_idx_any(wt, SWARPS - 1));
      if (tile == 0) {
        if (lane == 0) {
          SW::publish(words, FLAG_INCL,
                      EXCL ? Op::ccomb(Op::from_init(init), tile_agg) : tile_agg);
          sm.prefix = EXCL ? Op::from_init(init) : Op::cident();
        }
      } else {
        if (lane == 0) SW::publish(words + tile * SW::NW, FLAG_AGG, tile_agg);
        load_window(pred - (long long)lane * LBJ);
      }
    }

    // ---- per-sub-tile warp scans: lex[j] becomes the lane's exclusive
    // prefix inside its warp's slice of sub-tile j
#pragma unroll
    for (int j = 0; j < G; ++j) {
      Local inc = lex[j];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const Local other = shfl_up_any(inc, o);
        if (lane >= o) inc = Op::comb(other, inc);
      }
      lex[j] = shfl_up_any(inc, 1);
      if (lane == 31) sm.wtot[j * SWARPS + warp] = inc;
    }
    __syncthreads();

    if (warp == 1) {
      // ---- prefix table of the warp totals (sub-tile major): lane q
      // holds entries q*PT .. q*PT+PT-1
      Local e[PT];
#pragma unroll
      for (int i = 0; i < PT; ++i) e[i] = sm.wtot[PT * lane + i];
      Local pin = e[0];
#pragma unroll
      for (int i = 1; i < PT; ++i) pin = Op::comb(pin, e[i]);
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const Local other = shfl_up_any(pin, o);
        if (lane >= o) pin = Op::comb(other, pin);
      }
      Local run = shfl_up_any(pin, 1);
#pragma unroll
      for (int i = 0; i < PT; ++i) {
        if (lane == 0 && i == 0) {
          sm.pref[0] = Op::ident();
          run = e[0];
        } else {
          sm.pref[PT * lane + i] = run;
          run = Op::comb(run, e[i]);
        }
      }
    } else if (warp == 0 && tile > 0) {
      // ---- decoupled look-back.  Lane q inspects tiles pred - q*LBJ - j
      // (j = 0..LBJ-1), nearest first; the window is folded up to the
      // nearest inclusive prefix, or wholly, and then the next window
      // further back is inspected.
      Carry acc = Op::cident();
      bool timed_out = false;
      while (true) {
        const long long t0 = pred - (long long)lane * LBJ;
        uint32_t spins = 0;
        int stop, jstop;
        while (true) {
          jstop = LBJ;
#pragma unroll
          for (int j = LBJ - 1; j >= 0; --j)
            if (lbf[j] == FLAG_INCL) jstop = j;
          const uint32_t im = __ballot_sync(0xffffffffu, jstop < LBJ);
          stop = im ? (__ffs(im) - 1) : 32;
          // every tile from the nearest one to the first inclusive prefix
          // must have published
          const int need = (lane < stop) ? LBJ - 1 : (lane == stop ? jstop : -1);
          bool ok = true;
#pragma unroll
          for (int j = 0; j < LBJ; ++j)
            if (j <= need) ok = ok && (lbf[j] != 0);
          if (__all_sync(0xffffffffu, ok)) break;
          if (++spins > spin_limit) {
            timed_out = true;
            break;
          }
          __nanosleep(LB_SLEEP_NS);
#pragma unroll
          for (int j = 0; j < LBJ; ++j)
            if (lbf[j] == 0) lbf[j] = SW::poll(words + (t0 - j) * SW::NW, lbv[j]);
        }
        if (timed_out) break;  // warp-uniform
        // fold this lane's share of the window, earliest tile first
        const int need = (lane < stop) ? LBJ - 1 : (lane == stop ? jstop : -1);
        Carry x = Op::cident();
        bool any = false;
#pragma unroll
        for (int j = LBJ - 1; j >= 0; --j)
          if (j <= need) {
            x = any ? Op::ccomb(x, lbv[j]) : lbv[j];
            any = true;
          }
        // ordered combine across lanes: a higher lane holds earlier tiles
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const Carry other = shfl_idx_any(x, (lane + o) & 31);
          if (lane + o < 32) x = Op::ccomb(other, x);
        }
        acc = Op::ccomb(shfl_idx_any(x, 0), acc);
        if (stop < 32) break;
        pred -= 32 * LBJ;
        load_window(pred - (long long)lane * LBJ);
      }
      if (lane == 0) {
        if (timed_out) atomicOr_system(status, kStatusScanTimeout);
        SW::publish(words + tile * SW::NW, FLAG_INCL, Op::ccomb(acc, tile_agg));
        sm.prefix = acc;
      }
    }
    __syncthreads();

    // ---- outputs: carry-in + prefix of earlier sub-tiles and warps + lane
    // prefix + running scan of the granule, stored straight from registers
    const Carry TP = sm.prefix;
    const bool tile_has = EXCL || tile > 0;
#pragma unroll
    for (int j = 0; j < G; ++j) {
      const int g = j * SBLOCK + tid;
      bool has_tp = true;
      Local tp;
      if (j == 0 && warp == 0) {
        has_tp = lane > 0;
        tp = lex[0];
      } else {
        const Local pw = sm.pref[j * SWARPS + warp];
        tp = (lane > 0) ? Op::comb(pw, lex[j]) : pw;
      }
      Carry P = TP;
      bool hasP = tile_has;
      if (has_tp) {
        P = hasP ? fold_local<Op>(TP, tp) : Op::to_carry(tp);
        hasP = true;
      }
      const Vec16<T> v = *reinterpret_cast<const Vec16<T>*>(&st[g * VN]);
      Vec16<T> o;
      Local run = Op::ident();
#pragma unroll
      for (int k = 0; k < VN; ++k) {
        const Local x = (full || base + size_t(g) * VN + k < n) ? Op::lift(v.v[k]) : Op::ident();
        if (EXCL) o.v[k] = (k == 0) ? Op::out_prefix(P) : Op::out(P, run);
        run = (k == 0) ? x : Op::comb(run, x);
        if (!EXCL) o.v[k] = hasP ? Op::out(P, run) : Op::out_local(run);
      }
      T* dst = out + base + size_t(g) * VN;
      if (full && vec_out) {
        st_vec_stream(dst, o);
      } else {
#pragma unroll
        for (int k = 0; k < VN; ++k)
          if (base + size_t(g) * VN + k < n) dst[k] = o.v[k];
      }
    }
  }
}

template <class Op, bool EXCL>
__global__ void __launch_bounds__(SBLOCK, scan_min_blocks<Op>())
scan_kernel(const typename Op::T* in, typename Op::T* out, size_t n, typename Op::T init,
            int tma_ok, int vec_out, uint64_t* words, uint32_t* tile_counter,
            uint32_t* status, uint32_t spin_limit, uint32_t pf_tiles) {
  using T = typename Op::T;
  constexpr int TS = Tile<Op>::SIZE;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  ScanSmem<Op>& sm = *reinterpret_cast<ScanSmem<Op>*>(smem_raw);
  const int tid = threadIdx.x;
  T* st = sm.stage;
  if (tid == 0) {
    sm.tile = atomicAdd(tile_counter, 1u);
    mbar_init(&sm.bar, 1);
    fence_mbar_init();
    const size_t b0 = size_t(sm.tile) * TS;
    if (tma_ok && b0 + TS <= n) {
      mbar_arrive_expect_tx(&sm.bar, TS * sizeof(T));
      tma_load_1d(st, in + b0, TS * sizeof(T), &sm.bar);
    }
    // the tile a block will claim about one generation of resident blocks
    // later: into L2 now, so that its TMA load is an L2 read
    const size_t pb = b0 + size_t(pf_tiles) * TS;
    if (pf_tiles && tma_ok && pb + TS <= n) prefetch_l2_bulk(in + pb, TS * sizeof(T));
  }
  __syncthreads();
  const size_t tile = sm.tile;
  const size_t base = tile * TS;
  if (tma_ok && base + TS <= n) {
    if (!mbar_wait(&sm.bar, 0, spin_limit)) {
      if (tid == 0) atomicOr_system(status, kStatusTmaTimeout);
      mbar_drain(&sm.bar, 0);  // let the copy land before the block goes on
    }
  } else {
    for (int e = tid; e < TS; e += SBLOCK) st[e] = (base + e < n) ? in[base + e] : T(0);
    __syncthreads();
  }
  scan_tile<Op, EXCL>(sm.work, st, tile, n, init, vec_out, out, words, status, spin_limit);
}

template <class Op, bool EXCL>
int launch_scan(const char* name, unsigned grid, cudaStream_t s, const typename Op::T* in,
                typename Op::T* out, size_t n, typename Op::T init, int tma_ok, int vec_out,
                uint64_t* words, uint32_t* counter, uint32_t* status, uint32_t lim) {
  auto kern = scan_kernel<Op, EXCL>;
  static KernelSetup ks;
  DeviceProps props;
  B200_TRY(device_props(&props));
  int bps = 0;
  B200_TRY(kernel_setup(ks, props, kern, SBLOCK, sizeof(ScanSmem<Op>), &bps));
  // L2 prefetch distance: one tile per SM.  Measured on GB300 for the
  // int64 exclusive scan at 2^28 (64 KB tiles): none 0.815 ms; 152 tiles
  // 0.689; 304 0.690; 456 0.75; 608 and more 0.91-0.97 (prefetched lines
  // are evicted, or crowd out the demand loads, before their tile is claimed).
  const uint32_t pf = uint32_t(props.sms);
  B200_LAUNCH(name, kern, grid, SBLOCK, sizeof(ScanSmem<Op>), s, in, out, n, init, tma_ok, vec_out,
              words, counter, status, lim, pf);
  return B200_OK;
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
  const size_t tiles = (n + Tile<Op>::SIZE - 1) / Tile<Op>::SIZE;
  constexpr size_t NW = StatusWords<Carry>::NW;
  const size_t nwords = tiles * NW + 16;  // status words + the tile counter
  Sizer z;
  z.take<uint64_t>(nwords);
  void* scr = nullptr;
  B200_TRY(scratch(s, z.bytes(), &scr, nullptr));
  Carver cv(scr);
  uint64_t* words = cv.take<uint64_t>(nwords);
  uint32_t* counter = reinterpret_cast<uint32_t*>(words + tiles * NW);
  uint32_t* status = nullptr;
  B200_TRY(status_word(&status));
  B200_CUDA(cudaMemsetAsync(words, 0, nwords * sizeof(uint64_t), s));
  const int tma_ok = reinterpret_cast<uintptr_t>(in) % 16 == 0;
  const int vec_out = reinterpret_cast<uintptr_t>(out) % 16 == 0;
  B200_TRY((launch_scan<Op, EXCL>(name, unsigned(tiles), s, in, out, n, init, tma_ok, vec_out,
                                   words, counter, status, spin_limit())));
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
  const size_t n = 2 * size_t(Tile<Op>::SIZE);
  Sizer z;
  z.take<int32_t>(n);
  z.take<uint64_t>(64);
  void* scr = nullptr;
  B200_TRY(scratch(s, z.bytes(), &scr, nullptr));
  Carver cv(scr);
  int32_t* data = cv.take<int32_t>(n);
  uint64_t* words = cv.take<uint64_t>(64);
  uint32_t* counter = reinterpret_cast<uint32_t*>(words + 32);
  uint32_t* status = nullptr;
  B200_TRY(status_word(&status));
  B200_CUDA(cudaMemsetAsync(data, 0, n * sizeof(int32_t), s));
  B200_CUDA(cudaMemsetAsync(words, 0, 64 * sizeof(uint64_t), s));
  const uint32_t one = 1;  // the tile counter: the block takes tile id 1
  B200_CUDA(cudaMemcpyAsync(counter, &one, sizeof(one), cudaMemcpyHostToDevice, s));
  B200_CUDA(cudaStreamSynchronize(s));  // `one` lives on this stack frame
  uint32_t lim = spin_limit();
  if (lim > (1u << 16)) lim = 1u << 16;
  B200_TRY((launch_scan<Op, false>("b200_selftest_scan_timeout", 1, s, data, data, n, 0, 1, 1,
                                   words, counter, status, lim)));
  clear_error();
  return B200_OK;
}

}  // extern "C"
