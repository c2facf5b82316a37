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
//      every 8-bit digit position at once (per-warp shared counters); it
//      also zeroes the first pass's look-back status words;
//   2. bins_kernel: exclusive scan of each histogram -> global digit bases;
//   3. one onesweep_kernel per digit: a tile of 384 threads x 16-24 keys is
//      loaded by one TMA bulk copy (the block also prefetches into L2 the
//      tile claimed one SM's worth of tiles later, so most loads are L2
//      reads), ranked in registers with a
//      warp-level multisplit built from eight ballots per key (on this GPU
//      __match_any_sync costs ~80 cycles per warp, the ballots a few), its
//      per-digit counts are published before the ranking (early counts) and
//      a per-digit decoupled look-back (eight predecessors per poll) yields
//      the global offsets; the keys' tile positions are scattered into
//      digit order in shared memory and keys and values are written out in
//      runs, so the global stores coalesce.  Each pass
//      zeroes its tiles' rows of the next pass's status words (two
//      ping-pong buffers instead of one per pass).
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

constexpr int RB = 256;       // threads per block of the histogram kernel
constexpr int RADIX = 256;
constexpr int WARPS = RB / 32;
// Threads and keys per thread of a onesweep tile, by shape, measured on
// GB300 at 2^28: 384 threads with 24 keys each for 32-bit keys alone (9216
// per tile) and 16 each otherwise (6144 per tile, three blocks per SM for
// 64-bit keys).  256 threads x 28 / 24 keys is 1% slower for 64-bit keys
// and pairs; 512 threads leave two blocks per SM and are 20% slower.  The
// first RADIX threads own one digit each in the per-digit phase.
template <class K, bool HAS_V>
struct SweepShape {
  static constexpr int RB = 384;
  static constexpr int WARPS = RB / 32;
  static constexpr int KPT = (sizeof(K) == 4 && !HAS_V) ? 24 : 16;
  static constexpr int TILE = RB * KPT;
  static_assert(RB >= RADIX && RB % 32 == 0 && KPT % 4 == 0, "whole digit warps, four digits per register");
};

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
  // Raw key whose first-pass ordered form (desc applied) is all ones, so
  // that padding sorts last.
  static __device__ __forceinline__ K pad(bool desc) {
    return from_ord(U(~U(0)), desc);
  }
  static __device__ __forceinline__ K from_ord(U u, bool desc) {
    if (desc) u = ~u;
    if (std::is_floating_point<K>::value) u = (u & SIGN) ? U(u ^ SIGN) : U(~u);
    else if (std::is_signed<K>::value) u ^= SIGN;
    return cook(u);
  }
};

__device__ __forceinline__ int pass_of_shift(int shift) { return shift >> 3; }

// Status word: 2 flag bits on top, running count below.
template <class ST>
struct Status {
  static constexpr int SHIFT = sizeof(ST) * 8 - 2;
  static constexpr ST AGG = ST(1) << SHIFT;
  static constexpr ST INCL = ST(2) << SHIFT;
  static constexpr ST MASK = (ST(1) << SHIFT) - 1;
};

// Byte-aligned digit of an order-preserving key: one byte permute of the
// key's 32-bit half that holds it (sel = 0x4440 | byte within the half; the
// upper result bytes come from the zero operand).
__device__ __forceinline__ uint32_t digit_of(uint32_t u, bool, uint32_t sel) {
  return __byte_perm(u, 0u, sel);
}
__device__ __forceinline__ uint32_t digit_of(uint64_t u, bool hi, uint32_t sel) {
  return __byte_perm(hi ? uint32_t(u >> 32) : uint32_t(u), 0u, sel);
}

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
// Every digit position's histogram from one read of the keys.  Each warp
// counts into its own shared histograms with plain shared atomics (a warp's
// lanes rarely collide on uniform digits, and a skewed digit costs a few
// replays, not a serialised warp vote).  The kernel also zeroes the first
// pass's look-back status words, so no separate memset pass is needed.
template <class K, int P>
__global__ void __launch_bounds__(RB)
hist_kernel(const K* __restrict__ keys, size_t n, int desc, uint32_t* __restrict__ hist,
            uint4* __restrict__ status0, size_t status_vec4) {
  using KB = KeyBits<K>;
  using U = typename KB::U;
  extern __shared__ uint32_t shh[];  // [WARPS][P][RADIX]
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < WARPS * P * RADIX; i += RB) shh[i] = 0;
  const size_t gt = size_t(blockIdx.x) * RB + tid;
  const size_t nt = size_t(gridDim.x) * RB;
  for (size_t i = gt; i < status_vec4; i += nt) status0[i] = make_uint4(0, 0, 0, 0);
  __syncthreads();
  uint32_t* my = shh + warp * P * RADIX;
  constexpr int VN = 16 / sizeof(K);
  size_t done = 0;
  if (reinterpret_cast<uintptr_t>(keys) % 16 == 0) {
    const size_t nvec = n / VN;
    constexpr int UN = 4;
    size_t v = gt;
    for (; v + (UN - 1) * nt < nvec; v += UN * nt) {
      Vec16<K> q[UN];
#pragma unroll
      for (int u = 0; u < UN; ++u) q[u] = ld_vec_stream(keys + (v + u * nt) * VN);
#pragma unroll
      for (int u = 0; u < UN; ++u)
#pragma unroll
        for (int e = 0; e < VN; ++e) {
          const U x = KB::to_ord(q[u].v[e], desc != 0);
#pragma unroll
          for (int p = 0; p < P; ++p) atomicAdd(my + p * RADIX + uint32_t((x >> (8 * p)) & 0xff), 1u);
        }
    }
    for (; v < nvec; v += nt) {
      const Vec16<K> q = ld_vec_stream(keys + v * VN);
#pragma unroll
      for (int e = 0; e < VN; ++e) {
        const U x = KB::to_ord(q.v[e], desc != 0);
#pragma unroll
        for (int p = 0; p < P; ++p) atomicAdd(my + p * RADIX + uint32_t((x >> (8 * p)) & 0xff), 1u);
      }
    }
    done = nvec * VN;
  }
  for (size_t i = done + gt; i < n; i += nt) {
    const U x = KB::to_ord(keys[i], desc != 0);
#pragma unroll
    for (int p = 0; p < P; ++p) atomicAdd(my + p * RADIX + uint32_t((x >> (8 * p)) & 0xff), 1u);
  }
  __syncthreads();
  for (int i = tid; i < P * RADIX; i += RB) {
    uint32_t c = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) c += shh[w * P * RADIX + i];
    if (c) atomicAdd(hist + i, c);
  }
}

// Exclusive scan of each pass's histogram -> digit bases.
// A pass whose digit is the same for every key (one bin holds all n) keeps
// the order: it is flagged in `same`, and runs as a plain copy.
template <int P>
__global__ void __launch_bounds__(RADIX) bins_kernel(const uint32_t* __restrict__ hist,
                                                     uint32_t* __restrict__ bins, uint32_t n,
                                                     int* __restrict__ same) {
  __shared__ uint32_t wsum[RADIX / 32];
  const int d = threadIdx.x, lane = d & 31, w = d >> 5;
  for (int p = 0; p < P; ++p) {
    const uint32_t c = hist[p * RADIX + d];
    const int one_bin = __syncthreads_or(c == n);
    if (d == 0) same[p] = one_bin;
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

// Decoupled look-back for digit d of tile `tile`: the global start of the
// tile's run of digit d.  LBW predecessors per poll: the loads of one window
// are independent, then consumed in order until an inclusive count is
// found.  A not-yet-published tile stops the consumption; the wait is
// bounded (the status word records a give-up).  Publishes the tile's
// inclusive count (start + cnt) before returning.
template <class ST>
__device__ __forceinline__ ST digit_lookback(const ST* __restrict__ status,
                                             const uint32_t* __restrict__ bins, size_t tile, int d,
                                             uint32_t cnt, ST* my_status, uint32_t* err,
                                             uint32_t spin_limit) {
  using S = Status<ST>;
  if (tile == 0) return ST(bins[d]);
  constexpr int LBW = 8;
  ST acc = 0;
  long long t = (long long)tile - 1;
  uint32_t spins = 0;
  bool done = false;
  while (!done) {
    ST w[LBW];
#pragma unroll
    for (int j = 0; j < LBW; ++j)
      w[j] = (t - j >= 0) ? ld_relaxed(status + size_t(t - j) * RADIX + d) : ST(S::INCL);
    int used = LBW;
#pragma unroll
    for (int j = 0; j < LBW; ++j) {
      if (j >= used) break;
      const ST flag = w[j] & ~S::MASK;
      if (flag == 0) { used = j; break; }
      acc += w[j] & S::MASK;
      if (flag == S::INCL) { done = true; break; }
    }
    if (done) break;
    t -= used;
    if (used < LBW) {
      if (++spins > spin_limit) {
        atomicOr_system(err, kStatusSortTimeout);
        break;
      }
      __nanosleep(100);
    }
  }
  st_relaxed(my_status, ST(S::INCL | (acc + cnt)));
  return acc;
}

// ------------------------------------------------------------- onesweep
// One tile per block.  Tiles take their id from an atomic counter in launch
// order, so every predecessor of a tile has started and publishes its
// counts without waiting: the look-back terminates (and is bounded anyway).
// The tile arrives by one TMA bulk copy into shared memory and stays there:
// the ranking reads the digits from it (packed four per register) and
// scatters only each key's 16-bit tile position into digit order; the
// write-out fetches key and value through that index.  One copy of the tile
// in shared memory and few registers, so four to six blocks fit per SM and
// their loads, rankings and look-backs overlap.  The pass type (first /
// last) is a template parameter and bounds are tile-local 32-bit compares,
// to keep the instruction count down.
template <class K, class V, bool HAS_V, class ST>
struct SweepSmem {
  static constexpr int TILE = SweepShape<K, HAS_V>::TILE;
  alignas(128) K kin[TILE];                       // the tile as loaded (TMA)
  alignas(128) V vin[HAS_V ? TILE : 1];
  uint16_t idx[TILE];                             // tile position of the i-th key in digit order
  uint32_t wcnt[SweepShape<K, HAS_V>::WARPS][RADIX];  // per-warp digit counts, then running starts
  ST gdst[RADIX];                                 // global dst = gdst[d] + local position
  uint32_t wtot[RADIX / 32];
  uint64_t bar;
  uint32_t tile;
  int same;                                       // this pass's digit is one value
};

// Blocks per SM the shared memory allows (228 KB per SM, 1 KB reserved per
// block), at most five and at most 2048 threads (48 registers, no spills);
// the register budget is cut to match.
template <class K, class V, bool HAS_V, class ST>
constexpr int sweep_min_blocks() {
  constexpr int b = 233472 / int(sizeof(SweepSmem<K, V, HAS_V, ST>) + 1024);
  constexpr int cap = 2048 / SweepShape<K, HAS_V>::RB < 5 ? 2048 / SweepShape<K, HAS_V>::RB : 5;
  return b < 1 ? 1 : (b > cap ? cap : b);
}

// The tile of a pass whose digit is the same for every key keeps its
// order: its keys (mapped to / from order-preserving form on the first /
// last pass) and values go straight to the same positions of the
// destination.  A full tile that TMA brought into shared memory (st, sv)
// is written from there in 16-byte vectors; otherwise element by element
// from global memory.  Out of line, so that the ranking path keeps its
// register allocation.
template <class K, bool FIRST, bool LAST>
__device__ __forceinline__ K same_digit_key(K k, int desc) {
  using KB = KeyBits<K>;
  using U = typename KB::U;
  if (FIRST) {
    const U x = KB::to_ord(k, false);
    return KB::cook(desc ? U(~x) : x);
  }
  if (LAST) {
    const U uk = KB::raw(k);
    return KB::from_ord(desc ? U(~uk) : uk, false);
  }
  return k;
}
template <class K, class V, bool HAS_V, class ST, bool FIRST, bool LAST, int SRB, int TILE>
__device__ __noinline__ void same_digit_copy(const K* __restrict__ kin, K* __restrict__ kout,
                                             const V* __restrict__ vin, V* __restrict__ vout,
                                             const K* st, const V* sv, bool staged, size_t tbase, int lim,
                                             int desc, ST* status_row, bool downer) {
  const int tid = threadIdx.x;
  if (status_row && downer) status_row[tid] = ST(0);
  const bool vec = staged && (reinterpret_cast<uintptr_t>(kout + tbase) % 16 == 0) &&
                   (!HAS_V || reinterpret_cast<uintptr_t>(vout + tbase) % 16 == 0);
  if (vec) {
    constexpr int KN = Vec16<K>::N, KV = TILE / KN / SRB;
    static_assert(TILE % (KN * SRB) == 0, "whole key vectors per thread");
#pragma unroll
    for (int j = 0; j < KV; ++j) {
      const int g = j * SRB + tid;
      Vec16<K> q = *reinterpret_cast<const Vec16<K>*>(st + size_t(g) * KN);
#pragma unroll
      for (int e = 0; e < KN; ++e) q.v[e] = same_digit_key<K, FIRST, LAST>(q.v[e], desc);
      st_vec_stream(kout + tbase + size_t(g) * KN, q);
    }
    if (HAS_V) {
      constexpr int VN = Vec16<V>::N, VV = TILE / VN / SRB;
      static_assert(TILE % (VN * SRB) == 0, "whole value vectors per thread");
#pragma unroll
      for (int j = 0; j < VV; ++j) {
        const int g = j * SRB + tid;
        st_vec_stream(vout + tbase + size_t(g) * VN, *reinterpret_cast<const Vec16<V>*>(sv + size_t(g) * VN));
      }
    }
    return;
  }
  for (int e = tid; e < lim; e += SRB) {
    kout[tbase + e] = same_digit_key<K, FIRST, LAST>(kin[tbase + e], desc);
    if (HAS_V) vout[tbase + e] = vin[tbase + e];
  }
}

// HI: which 32-bit half of a 64-bit key holds this pass's digit (0 or 1,
// known at compile time so the half is selected without a branch; 0 for
// 32-bit keys).
template <class K, class V, bool HAS_V, class ST, bool FIRST, bool LAST, int HI>
__global__ void __launch_bounds__(SweepShape<K, HAS_V>::RB, (sweep_min_blocks<K, V, HAS_V, ST>()))
onesweep_kernel(const K* __restrict__ kin, K* __restrict__ kout, const V* __restrict__ vin,
                V* __restrict__ vout, size_t n, int shift, int desc,
                const uint32_t* __restrict__ bins, ST* __restrict__ status,
                ST* __restrict__ status_next, uint32_t* __restrict__ tile_counter,
                uint32_t* __restrict__ err, uint32_t spin_limit, int tma_ok,
                const int* __restrict__ same_digit, uint32_t pf_tiles) {
  using KB = KeyBits<K>;
  using U = typename KB::U;
  using S = Status<ST>;
  constexpr int KPT = SweepShape<K, HAS_V>::KPT, TILE = SweepShape<K, HAS_V>::TILE;
  constexpr int SRB = SweepShape<K, HAS_V>::RB, SW = SweepShape<K, HAS_V>::WARPS;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SweepSmem<K, V, HAS_V, ST>& sm = *reinterpret_cast<SweepSmem<K, V, HAS_V, ST>*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool downer = SRB == RADIX || tid < RADIX;  // owns digit tid in the per-digit phase
#pragma unroll
  for (int i = tid; i < SW * RADIX; i += SRB) (&sm.wcnt[0][0])[i] = 0;
  if (tid == 0) {
    const uint32_t t = atomicAdd(tile_counter, 1u);
    sm.tile = t;
    mbar_init(&sm.bar, 1);
    fence_mbar_init();
    const size_t b0 = size_t(t) * TILE;
    if (tma_ok && b0 + TILE <= n) {
      constexpr uint32_t kb = TILE * sizeof(K), vb = HAS_V ? TILE * sizeof(V) : 0;
      mbar_arrive_expect_tx(&sm.bar, kb + vb);
      tma_load_1d(sm.kin, kin + b0, kb, &sm.bar);
      if (HAS_V) tma_load_1d(sm.vin, vin + b0, vb, &sm.bar);
    }
    // the tile a block claims about one SM's worth of tiles later: into L2
    // now, so that its TMA load is an L2 read
    const size_t pb = b0 + size_t(pf_tiles) * TILE;
    if (pf_tiles && tma_ok && pb + TILE <= n) {
      prefetch_l2_bulk(kin + pb, TILE * sizeof(K));
      if (HAS_V) prefetch_l2_bulk(vin + pb, TILE * sizeof(V));
    }
    // read after the copy is under way: it lands while the flag arrives
    sm.same = same_digit[pass_of_shift(shift)];
  }
  __syncthreads();
  const size_t tile = sm.tile;
  const size_t tbase = tile * TILE;
  const int lim = (tbase + TILE <= n) ? TILE : int(n - tbase);  // valid keys in this tile
  if (__builtin_expect(sm.same, 0)) {
    // every key has this pass's digit: the order is unchanged, so the tile
    // is copied to the same positions; no ranking, no look-back
    const bool staged = tma_ok && lim == TILE;
    if (staged && !mbar_wait(&sm.bar, 0, spin_limit)) {
      if (tid == 0) atomicOr_system(err, kStatusTmaTimeout);
      mbar_drain(&sm.bar, 0);  // let the copy land before the block goes on
    }
    same_digit_copy<K, V, HAS_V, ST, FIRST, LAST, SRB, TILE>(kin, kout, vin, vout, sm.kin, sm.vin, staged,
                                                             tbase, lim, desc,
                                                             LAST ? nullptr : status_next + tile * RADIX,
                                                             downer);
    return;
  }
  if (tma_ok && lim == TILE) {
    if (!mbar_wait(&sm.bar, 0, spin_limit)) {
      if (tid == 0) atomicOr_system(err, kStatusTmaTimeout);
      mbar_drain(&sm.bar, 0);  // let the copy land before the block goes on
    }
  } else {
    // partial (last) tile: padding keys sort after every real key
    const K padk = FIRST ? KB::pad(desc != 0) : KB::cook(~U(0));
    for (int e = tid; e < TILE; e += SRB) {
      sm.kin[e] = (e < lim) ? kin[tbase + e] : padk;
      if (HAS_V && e < lim) sm.vin[e] = vin[tbase + e];
    }
    __syncthreads();
  }
  // this tile's row of the next pass's status words starts at zero
  if (!LAST && downer) status_next[tile * RADIX + tid] = ST(0);

  // key e of the tile in order-preserving form (padding is all ones)
  auto ukey = [&](int e) -> U {
    if (FIRST) {
      const U x = KB::to_ord(sm.kin[e], false);
      return desc ? U(~x) : x;
    }
    return KB::raw(sm.kin[e]);
  };
  const int wofs = warp * (32 * KPT) + lane;  // warp-striped positions
  constexpr bool dhi = HI == 1;
  const uint32_t dsel = 0x4440u | uint32_t((shift >> 3) & 3);

  // ---- early counts: per-warp digit histograms with shared atomics, so
  // the tile's counts are published before the expensive ranking and the
  // look-backs of later tiles rarely wait for this one
  uint32_t digs[KPT / 4];  // four 8-bit digits per register
#pragma unroll
  for (int q = 0; q < KPT / 4; ++q) digs[q] = 0;
#pragma unroll
  for (int k = 0; k < KPT; ++k) {
    uint32_t d;
    if constexpr (sizeof(K) == 8 && !FIRST) {
      // only the half that holds the digit is read (keys are already in
      // order-preserving form after the first pass)
      d = __byte_perm(reinterpret_cast<const uint32_t*>(&sm.kin[wofs + k * 32])[HI], 0u, dsel);
    } else {
      d = digit_of(ukey(wofs + k * 32), dhi, dsel);
    }
    digs[k / 4] += d << (8 * (k % 4));
    atomicAdd(&sm.wcnt[warp][d], 1u);
  }
  __syncthreads();

  // ---- per-digit counts: thread d < RADIX owns digit d (whole warps, so
  // the shuffles below see full warps)
  const int d = downer ? tid : 0;
  uint32_t cnt = 0, inc = 0;
  ST* my_status = status + tile * RADIX + d;
  if (downer) {
#pragma unroll
    for (int w = 0; w < SW; ++w) {
      const uint32_t c = sm.wcnt[w][d];
      sm.wcnt[w][d] = cnt;  // exclusive offset of warp w inside digit d
      cnt += c;
    }
    if (tile == 0) st_relaxed(my_status, ST(S::INCL | (ST(bins[d]) + cnt)));
    else st_relaxed(my_status, ST(S::AGG | ST(cnt)));

    // block exclusive scan of the counts -> local digit starts
    inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) sm.wtot[warp] = inc;
  }
  __syncthreads();
  uint32_t lstart = inc - cnt;
  if (downer) {
#pragma unroll
    for (int w = 0; w < RADIX / 32 - 1; ++w)
      if (w < warp) lstart += sm.wtot[w];
#pragma unroll
    for (int w = 0; w < SW; ++w) sm.wcnt[w][d] += lstart;  // tile-local start of (warp, digit)
  }
  __syncthreads();

  // ---- warp-level multisplit ranking, scattered straight into digit order
  // in shared memory: the lanes holding the same digit are found with eight
  // ballots (one per digit bit); the lowest such lane bumps the warp's
  // running start for that digit and shares the old one, which with the
  // lane's rank among its peers is the key's tile-local position.
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int k = 0; k < KPT; ++k) {
    const int e = wofs + k * 32;
    const uint32_t dk = __byte_perm(digs[k / 4], 0u, 0x4440u + (k % 4));
    uint32_t peers = 0xffffffffu;
#pragma unroll
    for (int bit = 0; bit < 8; ++bit) {
      const uint32_t bal = __ballot_sync(0xffffffffu, (dk >> bit) & 1u);
      // keep lanes whose bit equals mine: ~(bal ^ mine), mine = 0 or ~0
      peers &= ~(bal ^ (0u - ((dk >> bit) & 1u)));
    }
    const int leader = __ffs(peers) - 1;
    uint32_t old = 0;
    if (lane == leader) old = atomicAdd(&sm.wcnt[warp][dk], uint32_t(__popc(peers)));
    const uint32_t p = __shfl_sync(0xffffffffu, old, leader) + __popc(peers & lt);
    sm.idx[p] = uint16_t(e);
  }

  // ---- decoupled look-back for digit d (global start of this tile's run)
  ST gstart = 0;
  if (downer) gstart = digit_lookback<ST>(status, bins, tile, d, cnt, my_status, err, spin_limit);
  if (downer) sm.gdst[d] = gstart - ST(lstart);
  __syncthreads();

  // ---- write out in runs (one digit's run is contiguous in global): the
  // i-th key in digit order is fetched from the loaded tile through idx.
  // Padding positions (e >= lim, last tile only) are skipped; every real
  // key's destination lies in [0, n).
#pragma unroll
  for (int j = 0; j < KPT; ++j) {
    const int i = j * SRB + tid;
    const int e = sm.idx[i];
    if (e < lim) {
      const U uk = ukey(e);
      const ST dst = sm.gdst[digit_of(uk, dhi, dsel)] + ST(i);
      if (LAST) {
        const U x = desc ? U(~uk) : uk;
        kout[dst] = KB::from_ord(x, false);
      } else {
        kout[dst] = KB::cook(uk);
      }
      if (HAS_V) vout[dst] = sm.vin[e];
    }
  }
}

// Launch one pass (one block per tile).
template <class K, class V, bool HAS_V, class ST, bool FIRST, bool LAST, int HI>
int launch_sweep_t(const char* name, size_t tiles, cudaStream_t s, const K* src, K* dst,
                   const V* vsrc, V* vdst, size_t n, int shift, int desc, const uint32_t* bins,
                   ST* status, ST* status_next, uint32_t* counter, uint32_t* err, uint32_t lim,
                   const int* same) {
  const int tma_ok = (reinterpret_cast<uintptr_t>(src) % 16 == 0) &&
                     (!HAS_V || reinterpret_cast<uintptr_t>(vsrc) % 16 == 0);
  using SM = SweepSmem<K, V, HAS_V, ST>;
  auto kern = onesweep_kernel<K, V, HAS_V, ST, FIRST, LAST, HI>;
  constexpr int threads = SweepShape<K, HAS_V>::RB;
  static KernelSetup ks;
  DeviceProps props;
  B200_TRY(device_props(&props));
  int bps = 0;
  B200_TRY(kernel_setup(ks, props, kern, threads, sizeof(SM), &bps));
  // L2 prefetch distance: one tile per SM.  Measured on GB300 at 2^28 keys
  // (sort u32 / u64 / f32-i32 pairs): none 4.142 / 9.795 / 4.972 ms; 152
  // tiles 4.093 / 9.462 / 4.836; 304 and 456 within 0.2% of 152.
  const uint32_t pf = uint32_t(props.sms);
  B200_LAUNCH(name, kern, (unsigned)tiles, threads, sizeof(SM), s, src, dst, vsrc, vdst, n, shift, desc,
              bins, status, status_next, counter, err, lim, tma_ok, same, pf);
  return B200_OK;
}

template <class K, class V, bool HAS_V, class ST>
int launch_sweep(const char* name, size_t tiles, cudaStream_t s, const K* src, K* dst,
                 const V* vsrc, V* vdst, size_t n, int shift, int first, int last, int desc,
                 const uint32_t* bins, ST* status, ST* status_next, uint32_t* counter,
                 uint32_t* err, uint32_t lim, const int* same) {
  // the first pass takes digit 0 (low half), the last the top digit
  constexpr int TOP = sizeof(K) == 8 ? 1 : 0;
  if (first)
    return launch_sweep_t<K, V, HAS_V, ST, true, false, 0>(name, tiles, s, src, dst, vsrc, vdst, n,
                                                           shift, desc, bins, status, status_next,
                                                           counter, err, lim, same);
  if (last)
    return launch_sweep_t<K, V, HAS_V, ST, false, true, TOP>(name, tiles, s, src, dst, vsrc, vdst, n,
                                                             shift, desc, bins, status, status_next,
                                                             counter, err, lim, same);
  if constexpr (sizeof(K) == 8) {
    if (shift >= 32)
      return launch_sweep_t<K, V, HAS_V, ST, false, false, 1>(name, tiles, s, src, dst, vsrc, vdst, n,
                                                              shift, desc, bins, status, status_next,
                                                              counter, err, lim, same);
  }
  return launch_sweep_t<K, V, HAS_V, ST, false, false, 0>(name, tiles, s, src, dst, vsrc, vdst, n,
                                                          shift, desc, bins, status, status_next,
                                                          counter, err, lim, same);
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
  constexpr int TILE = SweepShape<K, HAS_V>::TILE;
  const size_t tiles = (n + TILE - 1) / TILE;
  const bool wide = n >= (size_t(1) << 30);
  const size_t st_bytes = wide ? sizeof(uint64_t) : sizeof(uint32_t);
  const size_t st_buf = round_up(tiles * RADIX * st_bytes, 256);  // one pass's status words
  Sizer z;
  z.take<K>(n);                                    // alternate keys
  if (HAS_V) z.take<V>(n);                         // alternate values
  z.take<uint32_t>(P * RADIX);                     // bins
  z.take<int>(P);                                  // passes whose digit is one value
  z.take<uint32_t>(P * RADIX + 64);                // hist + tile counters (memset)
  z.take<unsigned char>(2 * st_buf);               // ping-pong status words
  void* scr = nullptr;
  B200_TRY(scratch(s, z.bytes(), &scr, nullptr));
  Carver cv(scr);
  K* kalt = cv.take<K>(n);
  V* valt = HAS_V ? cv.take<V>(n) : nullptr;
  uint32_t* bins = cv.take<uint32_t>(P * RADIX);
  int* same = cv.take<int>(P);
  uint32_t* hist = cv.take<uint32_t>(P * RADIX + 64);
  uint32_t* counters = hist + P * RADIX;
  unsigned char* stat = cv.take<unsigned char>(2 * st_buf);
  B200_CUDA(cudaMemsetAsync(hist, 0, (P * RADIX + 64) * sizeof(uint32_t), s));
  uint32_t* err = nullptr;
  B200_TRY(status_word(&err));

  DeviceProps props;
  B200_TRY(device_props(&props));
  {
    const size_t smem = size_t(WARPS) * P * RADIX * sizeof(uint32_t);
    static KernelSetup ks;
    int bps = 0;
    B200_TRY(kernel_setup(ks, props, hist_kernel<K, P>, RB, smem, &bps));
    size_t g = size_t(props.sms) * bps;
    const size_t need = (n + RB - 1) / RB;
    if (g > need) g = need;
    B200_LAUNCH("b200_sort_hist", (hist_kernel<K, P>), (unsigned)g, RB, smem, s, kin, n, desc, hist,
                reinterpret_cast<uint4*>(stat), st_buf / 16);
  }
  B200_LAUNCH("b200_sort_bins", bins_kernel<P>, 1, RADIX, 0, s, hist, bins, uint32_t(n), same);

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
    void* cur = stat + size_t(p & 1) * st_buf;
    void* nxt = last ? nullptr : stat + size_t((p + 1) & 1) * st_buf;
    if (wide) {
      B200_TRY((launch_sweep<K, VV, HAS_V, uint64_t>(sweep_name, tiles, s, src, dstk, vsrc, vdst, n,
                                                     8 * p, first, last, desc, bins + p * RADIX,
                                                     static_cast<uint64_t*>(cur),
                                                     static_cast<uint64_t*>(nxt), counters + p,
                                                     err, lim, same)));
    } else {
      B200_TRY((launch_sweep<K, VV, HAS_V, uint32_t>(sweep_name, tiles, s, src, dstk, vsrc, vdst, n,
                                                     8 * p, first, last, desc, bins + p * RADIX,
                                                     static_cast<uint32_t*>(cur),
                                                     static_cast<uint32_t*>(nxt), counters + p,
                                                     err, lim, same)));
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
B200_SORT_PAIRS(i64_i32, int64_t, int32_t)
B200_SORT_PAIRS(u32_i64, uint32_t, int64_t)
B200_SORT_PAIRS(i32_i64, int32_t, int64_t)
B200_SORT_PAIRS(f32_i64, float, int64_t)
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
