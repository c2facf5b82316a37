// ORACLE -- test infrastructure only.
//
// CPU restatement of RAJA's seq_exec / omp_parallel_for_exec semantics for
// the data-parallel primitive path (forall, reducers, scans, sorts,
// MultiReduce histogram), plus an exact long accumulator for floating-point
// sums.  It is the checker for libb200prims: tests/, __graft_entry__.smoke()
// and the CPU-baseline legs of bench.py load it; nothing in the product
// links or calls it.
//
// Pinned against RAJA itself: oracle/refbuild/ compiles RAJA's own host
// policies from the unmodified reference headers (with a hand-written
// config.hpp and a clean-room subset of the camp library, whose submodule
// is empty in the reference tree), and tests/golden/make_ref_fixtures.py
// records their outputs.  tests/test_ref_fixtures.py requires this file to
// reproduce them bit for bit: reducers (MinLoc/MaxLoc ties included), every
// scan kind and op under seq and OpenMP (four threads), stable sorts under
// both policies, histograms and the daxpy body; unstable sorts follow
// RAJA's own rule (same keys, same values per key).  The known answers of
// RAJA's test suite (tests/test_oracle_pins.py) are checked as well.
//
// Build: oracle/build_oracle.py (g++ -O2 -fopenmp -ffp-contract=off).
// -ffp-contract=off keeps a*b+c as two rounded operations, as written in
// the reference's loop bodies, on every host (x86 and Arm alike).
#include <omp.h>

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <type_traits>
#include <vector>

namespace {

// ---------------------------------------------------------------- limits
// RAJA::operators::limits (util/Operators.hpp:248-333): min() is the most
// negative finite value for floating point, max() the largest finite.
template <class T>
T lim_max() {
  return std::numeric_limits<T>::max();
}
template <class T>
T lim_min() {
  return std::is_floating_point<T>::value ? -std::numeric_limits<T>::max()
                                          : std::numeric_limits<T>::min();
}

// operators::minimum / maximum (util/Operators.hpp:555-591): the candidate
// (rhs) replaces the current value only if strictly better, so the first
// extreme is kept.
template <class T>
T op_min(T lhs, T rhs) { return (rhs < lhs) ? rhs : lhs; }
template <class T>
T op_max(T lhs, T rhs) { return (lhs < rhs) ? rhs : lhs; }

template <class T>
struct ValLoc {
  T val;
  int64_t loc;
};

// ------------------------------------------------------------ seq reducers
// ReduceSeq = BaseCombinable (pattern/detail/reduce.hpp:287-358,
// policy/sequential/reduce.hpp:36-50): the lambda's copy starts at the
// identity, accumulates in loop order, and its destructor folds it into the
// parent (which holds init): result = init OP (identity OP x0 OP x1 ...).
template <class T>
T seq_sum(const T* x, int64_t n, T init) {
  T child = T(0);
  for (int64_t i = 0; i < n; ++i) child = child + x[i];
  return init + child;
}
template <class T>
T seq_dot(const T* x, const T* y, int64_t n, T init) {
  T child = T(0);
  for (int64_t i = 0; i < n; ++i) child = child + x[i] * y[i];
  return init + child;
}
// Integer sums wrap around modulo 2^bits (computed unsigned to stay defined).
template <class T>
T seq_sum_int(const T* x, int64_t n, T init) {
  using U = typename std::make_unsigned<T>::type;
  U child = 0;
  for (int64_t i = 0; i < n; ++i) child = U(child + U(x[i]));
  return T(U(U(init) + child));
}

// MinLoc/MaxLoc: ValueLoc compares values only (pattern/detail/reduce.hpp:
// 127-179); identity = (limits max|min, -1) (DefaultLoc, :111-125).
template <class T, bool MIN>
ValLoc<T> seq_loc(const T* x, int64_t n, ValLoc<T> init) {
  ValLoc<T> child{MIN ? lim_max<T>() : lim_min<T>(), -1};
  for (int64_t i = 0; i < n; ++i) {
    const bool take = MIN ? (x[i] < child.val) : (child.val < x[i]);
    if (take) child = ValLoc<T>{x[i], i};
  }
  const bool take = MIN ? (child.val < init.val) : (init.val < child.val);
  return take ? child : init;
}

// ------------------------------------------------------------ omp reducers
// ReduceOMP (policy/openmp/reduce.hpp:40-60): each thread accumulates a
// private copy over its static block of iterations (omp for schedule(static),
// policy/openmp/forall.hpp), then folds it into the parent in a critical
// section.
template <class T>
T omp_sum(const T* x, int64_t n, T init) {
  T parent = init;
#pragma omp parallel
  {
    T mine = T(0);
#pragma omp for schedule(static)
    for (int64_t i = 0; i < n; ++i) mine = mine + x[i];
#pragma omp critical(oracle_reduce)
    parent = parent + mine;
  }
  return parent;
}
template <class T>
T omp_dot(const T* x, const T* y, int64_t n, T init) {
  T parent = init;
#pragma omp parallel
  {
    T mine = T(0);
#pragma omp for schedule(static)
    for (int64_t i = 0; i < n; ++i) mine = mine + x[i] * y[i];
#pragma omp critical(oracle_reduce)
    parent = parent + mine;
  }
  return parent;
}
template <class T, bool MIN>
ValLoc<T> omp_loc(const T* x, int64_t n) {
  ValLoc<T> parent{MIN ? lim_max<T>() : lim_min<T>(), -1};
#pragma omp parallel
  {
    ValLoc<T> mine{MIN ? lim_max<T>() : lim_min<T>(), -1};
#pragma omp for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
      const bool take = MIN ? (x[i] < mine.val) : (mine.val < x[i]);
      if (take) mine = ValLoc<T>{x[i], i};
    }
#pragma omp critical(oracle_reduce)
    {
      const bool take = MIN ? (mine.val < parent.val) : (parent.val < mine.val);
      if (take) parent = mine;
    }
  }
  return parent;
}

// ------------------------------------------------------------------ scans
// policy/sequential/scan.hpp:43-153.
template <class T, class F>
void seq_inclusive(const T* in, T* out, int64_t n, F f) {
  if (n <= 0) return;
  T agg = in[0];
  out[0] = agg;
  for (int64_t i = 1; i < n; ++i) {
    agg = f(agg, in[i]);
    out[i] = agg;
  }
}
template <class T, class F>
void seq_exclusive(const T* in, T* out, int64_t n, F f, T v) {
  if (n <= 0) return;
  // the copy form (:127-153) reads in[i] before writing out[i]; in-place is
  // the same sequence of values
  T agg = v;
  for (int64_t i = 0; i < n; ++i) {
    const T t = in[i];
    out[i] = agg;
    agg = f(agg, t);
  }
}

// RAJA::detail::firstIndex (util/macros.hpp / policy/openmp): block split
// of n over p threads.
inline int64_t first_index(int64_t n, int64_t p, int64_t pid) {
  return (n * pid) / p;
}

// policy/openmp/scan.hpp:44-135: each thread scans its block, the block
// totals are exclusive-scanned, and each block adds its offset.
template <class T, class F>
void omp_inclusive(const T* in, T* out, int64_t n, F f, T ident) {
  if (n <= 0) return;
  if (in != out) std::copy(in, in + n, out);
  const int p0 = int(std::min<int64_t>(n, omp_get_max_threads()));
  std::vector<T> sums(p0, T());
#pragma omp parallel num_threads(p0)
  {
    const int p = omp_get_num_threads();
    const int pid = omp_get_thread_num();
    const int64_t b = first_index(n, p, pid), e = first_index(n, p, pid + 1);
    if (b != e) {
      seq_inclusive(out + b, out + b, e - b, f);
      sums[pid] = out[e - 1];
    }
#pragma omp barrier
#pragma omp single
    seq_exclusive(sums.data(), sums.data(), p, f, ident);
    for (int64_t i = b; i < e; ++i) out[i] = f(out[i], sums[pid]);
  }
}
template <class T, class F>
void omp_exclusive(const T* in, T* out, int64_t n, F f, T v, T ident) {
  if (n <= 0) return;
  if (in != out) std::copy(in, in + n, out);
  const int p0 = int(std::min<int64_t>(n, omp_get_max_threads()));
  std::vector<T> sums(p0, v);
#pragma omp parallel num_threads(p0)
  {
    const int p = omp_get_num_threads();
    const int pid = omp_get_thread_num();
    const int64_t b = first_index(n, p, pid), e = first_index(n, p, pid + 1);
    const T init = (pid == 0) ? v : out[b - 1];
#pragma omp barrier
    if (b != e) {
      seq_exclusive(out + b, out + b, e - b, f, init);
      sums[pid] = out[e - 1];
    }
#pragma omp barrier
#pragma omp single
    seq_exclusive(sums.data(), sums.data(), p, f, ident);
    for (int64_t i = b; i < e; ++i) out[i] = f(out[i], sums[pid]);
  }
}

template <class T>
struct Plus {
  T operator()(T a, T b) const {
    if (std::is_integral<T>::value) {
      using U = typename std::make_unsigned<typename std::conditional<std::is_integral<T>::value, T, int>::type>::type;
      return T(U(U(a) + U(b)));
    }
    return a + b;
  }
};
template <class T>
struct Min {
  T operator()(T a, T b) const { return op_min(a, b); }
};
template <class T>
struct Max {
  T operator()(T a, T b) const { return op_max(a, b); }
};

template <class T>
T ident_for(int op) {
  if (op == 0) return T(0);
  if (op == 1) return lim_max<T>();
  return lim_min<T>();
}

template <class T>
int scan(const T* in, T* out, int64_t n, int op, int exclusive, T init, int parallel) {
  if (op < 0 || op > 2) return 1;
  const T id = ident_for<T>(op);
  if (!parallel) {
    if (exclusive) {
      if (op == 0) seq_exclusive(in, out, n, Plus<T>(), init);
      else if (op == 1) seq_exclusive(in, out, n, Min<T>(), init);
      else seq_exclusive(in, out, n, Max<T>(), init);
    } else {
      if (op == 0) seq_inclusive(in, out, n, Plus<T>());
      else if (op == 1) seq_inclusive(in, out, n, Min<T>());
      else seq_inclusive(in, out, n, Max<T>());
    }
  } else {
    if (exclusive) {
      if (op == 0) omp_exclusive(in, out, n, Plus<T>(), init, id);
      else if (op == 1) omp_exclusive(in, out, n, Min<T>(), init, id);
      else omp_exclusive(in, out, n, Max<T>(), init, id);
    } else {
      if (op == 0) omp_inclusive(in, out, n, Plus<T>(), id);
      else if (op == 1) omp_inclusive(in, out, n, Min<T>(), id);
      else omp_inclusive(in, out, n, Max<T>(), id);
    }
  }
  return 0;
}

// ------------------------------------------------------------------ sorts
// seq: stable_sort -> RAJA merge_sort (util/sort.hpp:577), sort ->
// intro_sort (:415); pairs sort a zip of (key, value) by key
// (policy/sequential/sort.hpp:51-156).  A stable sort's output is unique,
// and every correct unstable sort yields the same keys, so the oracle uses
// the standard library's stable merge sort for both.
// omp (policy/openmp/sort.hpp:96-196): each thread sorts its block, then
// blocks are merged pairwise in a tree (inplace_merge).
template <class K>
struct Less {
  bool operator()(const K& a, const K& b) const { return a < b; }
};
template <class K>
struct Greater {
  bool operator()(const K& a, const K& b) const { return b < a; }
};

template <class It, class C>
void omp_tree_sort(It begin, int64_t n, C comp, bool stable) {
  const int p0 = int(std::max<int64_t>(1, std::min<int64_t>(omp_get_max_threads(), n / 1024)));
#pragma omp parallel num_threads(p0)
  {
    const int p = omp_get_num_threads();
    const int tid = omp_get_thread_num();
    const int64_t b = first_index(n, p, tid);
    {
      const int64_t e = first_index(n, p, tid + 1);
      if (stable) std::stable_sort(begin + b, begin + e, comp);
      else std::sort(begin + b, begin + e, comp);
    }
    for (int mid = 1; mid < p; mid *= 2) {
      const int end_off = 2 * mid;
      const int64_t m = first_index(n, p, std::min(tid + mid, p));
      const int64_t e = first_index(n, p, std::min(tid + end_off, p));
#pragma omp barrier
      if (tid % end_off == 0) std::inplace_merge(begin + b, begin + m, begin + e, comp);
    }
  }
}

template <class K>
void sort_keys(K* keys, int64_t n, int desc, int parallel, int stable) {
  if (n <= 1) return;
  if (!parallel) {
    if (desc) std::stable_sort(keys, keys + n, Greater<K>());
    else std::stable_sort(keys, keys + n, Less<K>());
  } else {
    if (desc) omp_tree_sort(keys, n, Greater<K>(), stable != 0);
    else omp_tree_sort(keys, n, Less<K>(), stable != 0);
  }
}

template <class K, class V>
struct KV {
  K k;
  V v;
};
template <class K, class V>
void sort_pairs(K* keys, V* vals, int64_t n, int desc, int parallel, int stable) {
  if (n <= 1) return;
  std::vector<KV<K, V>> z(n);
  for (int64_t i = 0; i < n; ++i) z[i] = KV<K, V>{keys[i], vals[i]};
  auto lt = [](const KV<K, V>& a, const KV<K, V>& b) { return a.k < b.k; };
  auto gt = [](const KV<K, V>& a, const KV<K, V>& b) { return b.k < a.k; };
  if (!parallel) {
    if (desc) std::stable_sort(z.begin(), z.end(), gt);
    else std::stable_sort(z.begin(), z.end(), lt);
  } else {
    if (desc) omp_tree_sort(z.begin(), n, gt, stable != 0);
    else omp_tree_sort(z.begin(), n, lt, stable != 0);
  }
  for (int64_t i = 0; i < n; ++i) {
    keys[i] = z[i].k;
    vals[i] = z[i].v;
  }
}

// ------------------------------------------------------ exact accumulator
// Fixed-point sum of doubles over the whole exponent range: bit b of a
// value's significand lands in limb (b + BIAS) / 32.  Limbs are int64 so
// up to 2^31 additions of 32-bit chunks need no carry propagation.
struct LongAcc {
  static constexpr int BIAS = 1074 + 64;        // 2^-1074 -> bit 64
  static constexpr int LIMBS = (2100 + 128) / 32 + 4;
  int64_t limb[LIMBS];
  int64_t count = 0;
  LongAcc() { std::memset(limb, 0, sizeof(limb)); }
  void normalize() {
    int64_t carry = 0;
    for (int i = 0; i < LIMBS; ++i) {
      int64_t v = limb[i] + carry;
      // floor division by 2^32
      carry = v >> 32;
      limb[i] = v - (carry << 32);
    }
    limb[LIMBS - 1] += carry << 32;
    count = 0;
  }
  void add(double x) {
    if (x == 0.0 || !std::isfinite(x)) return;
    int e;
    const double m = std::frexp(std::fabs(x), &e);  // x = m * 2^e, m in [0.5,1)
    uint64_t mant = uint64_t(std::ldexp(m, 53));    // 53-bit integer
    int lsb = e - 53;                               // value = mant * 2^lsb
    const int pos = lsb + BIAS;                     // >= 11 for subnormals
    const int li = pos / 32, sh = pos % 32;
    // mant << sh spans up to 85 bits: split into 32-bit limbs
    unsigned __int128 w = (unsigned __int128)mant << sh;
    const int64_t sgn = x < 0 ? -1 : 1;
    for (int k = 0; k < 3; ++k) {
      limb[li + k] += sgn * int64_t(uint64_t(w) & 0xffffffffull);
      w >>= 32;
    }
    if (++count >= (int64_t(1) << 30)) normalize();
  }
  // Round the exact value to double, and the remainder to a second double.
  void result(double* hi, double* lo) {
    normalize();
    // Two's complement across limbs: a negative total leaves every upper
    // limb at 2^32-1 and a negative top limb.  Convert |total| instead.
    const bool neg = limb[LIMBS - 1] < 0;
    if (neg) {
      for (int i = 0; i < LIMBS; ++i) limb[i] = -limb[i];
      normalize();
    }
    // value = sum limb[i] * 2^(32 i - BIAS); the top limb carries the
    // sign.  Convert by accumulating from the top with a double-double.
    double h = 0, l = 0;
    for (int i = LIMBS - 1; i >= 0; --i) {
      if (limb[i] == 0) continue;
      const double v = std::ldexp(double(limb[i]), 32 * i - BIAS);  // exact: |limb| < 2^33
      // two-sum (h, v)
      const double s = h + v;
      const double bb = s - h;
      const double err = (h - (s - bb)) + (v - bb);
      h = s;
      l += err;
    }
    const double s = h + l;
    const double e2 = l - (s - h);
    *hi = neg ? -s : s;
    *lo = neg ? -e2 : e2;
  }
};

}  // namespace

extern "C" {

int orc_abi_version(void) { return 1; }
int orc_max_threads(void) { return omp_get_max_threads(); }
void orc_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }

// ---- forall daxpy (policy/sequential/forall.hpp:58-102 loop body)
void orc_seq_axpy_f64(double a, const double* x, double* y, int64_t n) {
  for (int64_t i = 0; i < n; ++i) y[i] += a * x[i];
}
void orc_seq_axpy_f32(float a, const float* x, float* y, int64_t n) {
  for (int64_t i = 0; i < n; ++i) y[i] += a * x[i];
}
void orc_omp_axpy_f64(double a, const double* x, double* y, int64_t n) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) y[i] += a * x[i];
}
void orc_omp_axpy_f32(float a, const float* x, float* y, int64_t n) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) y[i] += a * x[i];
}

// ---- reducers
double orc_seq_sum_f64(const double* x, int64_t n, double init) { return seq_sum(x, n, init); }
float orc_seq_sum_f32(const float* x, int64_t n, float init) { return seq_sum(x, n, init); }
int32_t orc_seq_sum_i32(const int32_t* x, int64_t n, int32_t init) { return seq_sum_int(x, n, init); }
int64_t orc_seq_sum_i64(const int64_t* x, int64_t n, int64_t init) { return seq_sum_int(x, n, init); }
uint32_t orc_seq_sum_u32(const uint32_t* x, int64_t n, uint32_t init) { return seq_sum_int(x, n, init); }
uint64_t orc_seq_sum_u64(const uint64_t* x, int64_t n, uint64_t init) { return seq_sum_int(x, n, init); }
double orc_seq_dot_f64(const double* x, const double* y, int64_t n, double init) { return seq_dot(x, y, n, init); }
float orc_seq_dot_f32(const float* x, const float* y, int64_t n, float init) { return seq_dot(x, y, n, init); }
double orc_omp_sum_f64(const double* x, int64_t n, double init) { return omp_sum(x, n, init); }
float orc_omp_sum_f32(const float* x, int64_t n, float init) { return omp_sum(x, n, init); }
double orc_omp_dot_f64(const double* x, const double* y, int64_t n, double init) { return omp_dot(x, y, n, init); }
float orc_omp_dot_f32(const float* x, const float* y, int64_t n, float init) { return omp_dot(x, y, n, init); }

#define ORC_LOC(SUF, T)                                                                   \
  void orc_seq_minloc_##SUF(const T* x, int64_t n, T init_val, int64_t init_loc, T* val,  \
                            int64_t* loc) {                                               \
    ValLoc<T> r = seq_loc<T, true>(x, n, ValLoc<T>{init_val, init_loc});                  \
    *val = r.val;                                                                         \
    *loc = r.loc;                                                                         \
  }                                                                                       \
  void orc_seq_maxloc_##SUF(const T* x, int64_t n, T init_val, int64_t init_loc, T* val,  \
                            int64_t* loc) {                                               \
    ValLoc<T> r = seq_loc<T, false>(x, n, ValLoc<T>{init_val, init_loc});                 \
    *val = r.val;                                                                         \
    *loc = r.loc;                                                                         \
  }                                                                                       \
  void orc_omp_minloc_##SUF(const T* x, int64_t n, T* val, int64_t* loc) {                \
    ValLoc<T> r = omp_loc<T, true>(x, n);                                                 \
    *val = r.val;                                                                         \
    *loc = r.loc;                                                                         \
  }                                                                                       \
  void orc_omp_maxloc_##SUF(const T* x, int64_t n, T* val, int64_t* loc) {                \
    ValLoc<T> r = omp_loc<T, false>(x, n);                                                \
    *val = r.val;                                                                         \
    *loc = r.loc;                                                                         \
  }                                                                                       \
  T orc_seq_min_##SUF(const T* x, int64_t n, T init) {                                    \
    T c = lim_max<T>();                                                                   \
    for (int64_t i = 0; i < n; ++i) c = op_min(c, x[i]);                                  \
    return op_min(init, c);                                                               \
  }                                                                                       \
  T orc_seq_max_##SUF(const T* x, int64_t n, T init) {                                    \
    T c = lim_min<T>();                                                                   \
    for (int64_t i = 0; i < n; ++i) c = op_max(c, x[i]);                                  \
    return op_max(init, c);                                                               \
  }
ORC_LOC(f32, float)
ORC_LOC(f64, double)
ORC_LOC(i32, int32_t)
ORC_LOC(i64, int64_t)
ORC_LOC(u32, uint32_t)
ORC_LOC(u64, uint64_t)
#undef ORC_LOC

#define ORC_BIT(SUF, T)                                                  \
  T orc_seq_bitor_##SUF(const T* x, int64_t n, T init) {                 \
    T c = 0;                                                             \
    for (int64_t i = 0; i < n; ++i) c = T(c | x[i]);                     \
    return T(init | c);                                                  \
  }                                                                      \
  T orc_seq_bitand_##SUF(const T* x, int64_t n, T init) {                \
    T c = T(~T(0));                                                      \
    for (int64_t i = 0; i < n; ++i) c = T(c & x[i]);                     \
    return T(init & c);                                                  \
  }
ORC_BIT(i32, int32_t)
ORC_BIT(i64, int64_t)
ORC_BIT(u32, uint32_t)
ORC_BIT(u64, uint64_t)
#undef ORC_BIT

// ---- scans: op 0=plus 1=minimum 2=maximum; parallel 0=seq 1=omp
#define ORC_SCAN(SUF, T)                                                                     \
  int orc_scan_##SUF(const T* in, T* out, int64_t n, int op, int exclusive, T init,          \
                     int parallel) {                                                         \
    return scan<T>(in, out, n, op, exclusive, init, parallel);                               \
  }
ORC_SCAN(i32, int32_t)
ORC_SCAN(i64, int64_t)
ORC_SCAN(u32, uint32_t)
ORC_SCAN(u64, uint64_t)
ORC_SCAN(f32, float)
ORC_SCAN(f64, double)
#undef ORC_SCAN

// ---- sorts
#define ORC_SORT(SUF, K)                                                            \
  void orc_sort_##SUF(K* keys, int64_t n, int desc, int parallel, int stable) {     \
    sort_keys<K>(keys, n, desc, parallel, stable);                                  \
  }
ORC_SORT(u32, uint32_t)
ORC_SORT(u64, uint64_t)
ORC_SORT(i32, int32_t)
ORC_SORT(i64, int64_t)
ORC_SORT(f32, float)
ORC_SORT(f64, double)
#undef ORC_SORT

#define ORC_PAIRS(SUF, K, V)                                                                  \
  void orc_sort_pairs_##SUF(K* keys, V* vals, int64_t n, int desc, int parallel, int stable) { \
    sort_pairs<K, V>(keys, vals, n, desc, parallel, stable);                                  \
  }
ORC_PAIRS(u32_i32, uint32_t, int32_t)
ORC_PAIRS(u32_u32, uint32_t, uint32_t)
ORC_PAIRS(i32_i32, int32_t, int32_t)
ORC_PAIRS(f32_i32, float, int32_t)
ORC_PAIRS(u64_i32, uint64_t, int32_t)
ORC_PAIRS(i64_i32, int64_t, int32_t)
ORC_PAIRS(u64_i64, uint64_t, int64_t)
ORC_PAIRS(i64_i64, int64_t, int64_t)
ORC_PAIRS(f64_i64, double, int64_t)
ORC_PAIRS(f64_i32, double, int32_t)
ORC_PAIRS(u32_i64, uint32_t, int64_t)
ORC_PAIRS(i32_i64, int32_t, int64_t)
ORC_PAIRS(f32_i64, float, int64_t)
#undef ORC_PAIRS

// ---- MultiReduceSum histogram (+1 per element); bins outside [0,nbins)
// are skipped.  omp: per-thread private bins folded in a critical section
// (policy/openmp/multi_reduce.hpp:71-140).
void orc_seq_histogram_i32(const int32_t* x, int64_t n, int32_t nbins, uint64_t* counts) {
  for (int64_t i = 0; i < n; ++i)
    if (x[i] >= 0 && x[i] < nbins) counts[x[i]] += 1;
}
void orc_omp_histogram_i32(const int32_t* x, int64_t n, int32_t nbins, uint64_t* counts) {
#pragma omp parallel
  {
    std::vector<uint64_t> mine(size_t(nbins), 0);
#pragma omp for schedule(static)
    for (int64_t i = 0; i < n; ++i)
      if (x[i] >= 0 && x[i] < nbins) mine[x[i]] += 1;
#pragma omp critical(oracle_multi_reduce)
    for (int32_t b = 0; b < nbins; ++b) counts[b] += mine[b];
  }
}

// ---- MultiReduce{Sum,Min,Max,BitOr,BitAnd}: out[b] starts as given and
// every element with bins[i] == b is combined in index order with the
// reduce op's rule (policy/sequential/multi_reduce.hpp:135 combine ->
// MultiReduceOp{}(m_data[bin], val)): sum val += v, min `if (v < val) val =
// v`, max `if (val < v) val = v` (equal values keep the first, NaN never
// enters), bit ops |= and &=.  Bins outside [0, nbins) are skipped.
extern "C++" {
template <class T, class F>
static void multi_reduce(const int32_t* bins, const T* vals, int64_t n, int32_t nbins, T* out,
                         F op) {
  for (int64_t i = 0; i < n; ++i)
    if (bins[i] >= 0 && bins[i] < nbins) op(out[bins[i]], vals[i]);
}
}
#define ORC_MR(OP, SUF, T, BODY)                                                                 \
  void orc_multi_reduce_##OP##_##SUF(const int32_t* bins, const T* vals, int64_t n,             \
                                     int32_t nbins, T* out) {                                   \
    multi_reduce<T>(bins, vals, n, nbins, out, [](T& val, T v) { BODY; });                      \
  }
#define ORC_MR_ALL(SUF, T)                                                                       \
  ORC_MR(sum, SUF, T, val = T(val + v))                                                          \
  ORC_MR(min, SUF, T, if (v < val) val = v)                                                      \
  ORC_MR(max, SUF, T, if (val < v) val = v)
ORC_MR_ALL(i32, int32_t)
ORC_MR_ALL(i64, int64_t)
ORC_MR_ALL(u32, uint32_t)
ORC_MR_ALL(u64, uint64_t)
ORC_MR_ALL(f32, float)
ORC_MR_ALL(f64, double)
ORC_MR(bitor, i32, int32_t, val |= v)
ORC_MR(bitor, i64, int64_t, val |= v)
ORC_MR(bitor, u32, uint32_t, val |= v)
ORC_MR(bitor, u64, uint64_t, val |= v)
ORC_MR(bitand, i32, int32_t, val &= v)
ORC_MR(bitand, i64, int64_t, val &= v)
ORC_MR(bitand, u32, uint32_t, val &= v)
ORC_MR(bitand, u64, uint64_t, val &= v)
#undef ORC_MR_ALL
#undef ORC_MR

// ---- exact sums: (hi, lo) with hi = round(sum), lo = round(sum - hi)
void orc_exact_sum_f64(const double* x, int64_t n, double* hi, double* lo) {
  LongAcc a;
  for (int64_t i = 0; i < n; ++i) a.add(x[i]);
  a.result(hi, lo);
}
void orc_exact_sum_f32(const float* x, int64_t n, double* hi, double* lo) {
  LongAcc a;
  for (int64_t i = 0; i < n; ++i) a.add(double(x[i]));
  a.result(hi, lo);
}
// float*float is exact in double; double*double splits with fma.
void orc_exact_dot_f32(const float* x, const float* y, int64_t n, double* hi, double* lo) {
  LongAcc a;
  for (int64_t i = 0; i < n; ++i) a.add(double(x[i]) * double(y[i]));
  a.result(hi, lo);
}
void orc_exact_dot_f64(const double* x, const double* y, int64_t n, double* hi, double* lo) {
  LongAcc a;
  for (int64_t i = 0; i < n; ++i) {
    const double p = x[i] * y[i];
    const double e = std::fma(x[i], y[i], -p);
    a.add(p);
    a.add(e);
  }
  a.result(hi, lo);
}
// Sum of |x| (for condition numbers), exact to double rounding.
double orc_exact_abs_sum_f32(const float* x, int64_t n) {
  LongAcc a;
  for (int64_t i = 0; i < n; ++i) a.add(std::fabs(double(x[i])));
  double h, l;
  a.result(&h, &l);
  return h;
}
// Prefix sums of float input carried in double-double: out[i] is the
// inclusive prefix rounded to double (error ~1e-32 relative per step).
void orc_dd_scan_f32(const float* x, int64_t n, double* out) {
  double h = 0, l = 0;
  for (int64_t i = 0; i < n; ++i) {
    const double v = double(x[i]);
    const double s = h + v;
    const double bb = s - h;
    const double err = (h - (s - bb)) + (v - bb);
    l += err;
    h = s;
    const double t = h + l;
    l = l - (t - h);
    h = t;
    out[i] = h;
  }
}

// ---- one 7-point Jacobi sweep of one 3-D mesh (x fastest) with the max
// residual; the iteration / residual structure follows the reference's
// examples/jacobi.cpp:223-489 (there 2-D), extended to 3-D as the batched
// mesh configuration specifies.  Operation order matches the documented
// definition: ((u[i-1]+u[i+1]) + (u[j-1]+u[j+1])) + (u[k-1]+u[k+1]) (+ f),
// then * (1/6).
double orc_jacobi_sweep_f64(int nx, int ny, int nz, const double* u, double* unew,
                            const double* f) {
  const int64_t sx = nx, sy = int64_t(nx) * ny;
  double rmax = 0.0;
  for (int k = 1; k < nz - 1; ++k)
    for (int j = 1; j < ny - 1; ++j)
      for (int i = 1; i < nx - 1; ++i) {
        const int64_t c = k * sy + j * sx + i;
        double acc = u[c - 1] + u[c + 1];
        acc += u[c - sx] + u[c + sx];
        acc += u[c - sy] + u[c + sy];
        if (f) acc += f[c];
        const double v = acc * (1.0 / 6.0);
        unew[c] = v;
        const double r = std::fabs(v - u[c]);
        if (r > rmax) rmax = r;
      }
  return rmax;
}

}  // extern "C"
