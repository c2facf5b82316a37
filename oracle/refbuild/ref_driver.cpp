// Reference runner -- test infrastructure only.
//
// Runs RAJA's own host policies (seq_exec, omp_parallel_for_exec and the
// matching reducers, scans, sorts, MultiReduce and WorkGroup), compiled
// from the unmodified reference headers against the clean-room camp subset
// beside this file, on inputs read from raw binary files, and writes the
// results as raw binary files.  tests/golden/make_ref_fixtures.py drives it
// to produce the committed reference fixtures that pin oracle/oracle.cpp
// and the GPU path to RAJA's actual outputs.
//
//   ref_driver reduce <T> <seq|omp> <n> <in> <out>
//       T in i32 i64 f32 f64; out = sum, min, max (T), minloc value (T) and
//       index (int64), maxloc value (T) and index (int64), then for integer
//       T bitor and bitand (T); ReduceSum/Min/Max/MinLoc/MaxLoc/BitOr/BitAnd
//       with their default identities.
//   ref_driver params <T> <n> <in> <out>
//       the same sum/min/max/minloc/maxloc through expt::Reduce and
//       expt::ReduceLoc params on seq_exec.
//   ref_driver scan <T> <seq|omp> <inclusive|exclusive|inclusive_inplace|exclusive_inplace>
//                   <plus|minimum|maximum> <n> <in> <out> [init]
//   ref_driver sort <T> <seq|omp> <sort|stable_sort> <asc|desc> <n> <keys_in> <keys_out>
//                   [<vals_in> <vals_out>]            (T in u32 i32 u64 i64 f32 f64; values int32)
//   ref_driver hist <seq|omp> <n> <nbins> <bins_in> <counts_out>
//       MultiReduceSum<int64> counting: counts[bins[i]] += 1
//   ref_driver daxpy <seq|omp> <n> <a> <x_in> <y_in> <y_out>
//   ref_driver workgroup <nloops> <total> <begins_in> <ends_in> <out>
//       WorkPool/WorkGroup (seq_work, ordered): loop l adds i + 5 to a[i]
//       for i in [begins[l], ends[l]), then the group runs a second time.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "RAJA/RAJA.hpp"

namespace
{
[[noreturn]] void die(const char* msg)
{
  std::fprintf(stderr, "ref_driver: %s\n", msg);
  std::exit(2);
}

template <class T>
std::vector<T> read_vec(const char* path, size_t n)
{
  std::vector<T> v(n);
  FILE* f = std::fopen(path, "rb");
  if (!f) die("cannot open input");
  if (n && std::fread(v.data(), sizeof(T), n, f) != n) die("short input");
  std::fclose(f);
  return v;
}

struct Out {
  FILE* f;
  explicit Out(const char* path) : f(std::fopen(path, "wb"))
  {
    if (!f) die("cannot open output");
  }
  ~Out() { std::fclose(f); }
  template <class T>
  void put(const T& x)
  {
    std::fwrite(&x, sizeof(T), 1, f);
  }
  template <class T>
  void put(const std::vector<T>& v)
  {
    if (!v.empty()) std::fwrite(v.data(), sizeof(T), v.size(), f);
  }
};

using seq_pol = RAJA::seq_exec;
#if defined(RAJA_ENABLE_OPENMP)
using omp_pol = RAJA::omp_parallel_for_exec;
using omp_red = RAJA::omp_reduce;
using omp_mred = RAJA::omp_multi_reduce;
#else
using omp_pol = RAJA::seq_exec;
using omp_red = RAJA::seq_reduce;
using omp_mred = RAJA::seq_multi_reduce;
#endif

// ------------------------------------------------------------------ reduce
template <class T, class POL, class RED>
void run_reduce(size_t n, const char* in, const char* out)
{
  std::vector<T> x = read_vec<T>(in, n);
  const T* xp = x.data();
  RAJA::ReduceSum<RED, T> sum(T(0));
  RAJA::ReduceMin<RED, T> mn(std::numeric_limits<T>::max());
  RAJA::ReduceMax<RED, T> mx(std::numeric_limits<T>::lowest());
  RAJA::ReduceMinLoc<RED, T, RAJA::Index_type> mnl(std::numeric_limits<T>::max(), -1);
  RAJA::ReduceMaxLoc<RED, T, RAJA::Index_type> mxl(std::numeric_limits<T>::lowest(), -1);
  RAJA::forall<POL>(RAJA::TypedRangeSegment<RAJA::Index_type>(0, RAJA::Index_type(n)),
                    [=](RAJA::Index_type i) {
                      sum += xp[i];
                      mn.min(xp[i]);
                      mx.max(xp[i]);
                      mnl.minloc(xp[i], i);
                      mxl.maxloc(xp[i], i);
                    });
  Out o(out);
  o.put(T(sum.get()));
  o.put(T(mn.get()));
  o.put(T(mx.get()));
  o.put(T(mnl.get()));
  o.put(int64_t(mnl.getLoc()));
  o.put(T(mxl.get()));
  o.put(int64_t(mxl.getLoc()));
  if constexpr (std::is_integral<T>::value) {
    RAJA::ReduceBitOr<RED, T> bor(T(0));
    RAJA::ReduceBitAnd<RED, T> band(T(~T(0)));
    RAJA::forall<POL>(RAJA::TypedRangeSegment<RAJA::Index_type>(0, RAJA::Index_type(n)),
                      [=](RAJA::Index_type i) {
                        bor |= xp[i];
                        band &= xp[i];
                      });
    o.put(T(bor.get()));
    o.put(T(band.get()));
  }
}

template <class T>
void run_params(size_t n, const char* in, const char* out)
{
  std::vector<T> x = read_vec<T>(in, n);
  const T* xp = x.data();
  T s = T(0), mn = std::numeric_limits<T>::max(), mx = std::numeric_limits<T>::lowest();
  T mnv = std::numeric_limits<T>::max(), mxv = std::numeric_limits<T>::lowest();
  RAJA::Index_type mnl = -1, mxl = -1;
  using SUM = RAJA::expt::ValOp<T, RAJA::operators::plus>;
  using MIN = RAJA::expt::ValOp<T, RAJA::operators::minimum>;
  using MAX = RAJA::expt::ValOp<T, RAJA::operators::maximum>;
  using MINL = RAJA::expt::ValLocOp<T, RAJA::Index_type, RAJA::operators::minimum>;
  using MAXL = RAJA::expt::ValLocOp<T, RAJA::Index_type, RAJA::operators::maximum>;
  RAJA::forall<seq_pol>(RAJA::TypedRangeSegment<RAJA::Index_type>(0, RAJA::Index_type(n)),
                        RAJA::expt::Reduce<RAJA::operators::plus>(&s),
                        RAJA::expt::Reduce<RAJA::operators::minimum>(&mn),
                        RAJA::expt::Reduce<RAJA::operators::maximum>(&mx),
                        RAJA::expt::ReduceLoc<RAJA::operators::minimum>(&mnv, &mnl),
                        RAJA::expt::ReduceLoc<RAJA::operators::maximum>(&mxv, &mxl),
                        RAJA::Name("ref_params"),
                        [=](RAJA::Index_type i, SUM& ps, MIN& pmn, MAX& pmx, MINL& pml, MAXL& pxl) {
                          ps += xp[i];
                          pmn.min(xp[i]);
                          pmx.max(xp[i]);
                          pml.minloc(xp[i], i);
                          pxl.maxloc(xp[i], i);
                        });
  Out o(out);
  o.put(s);
  o.put(mn);
  o.put(mx);
  o.put(mnv);
  o.put(int64_t(mnl));
  o.put(mxv);
  o.put(int64_t(mxl));
}

// -------------------------------------------------------------------- scan
template <class T, class POL, class OP>
void run_scan_op(const std::string& kind, size_t n, const char* in, const char* out, bool has_init,
                 T init)
{
  std::vector<T> x = read_vec<T>(in, n);
  std::vector<T> y(n);
  auto xs = RAJA::make_span(x.data(), RAJA::Index_type(n));
  auto ys = RAJA::make_span(y.data(), RAJA::Index_type(n));
  if (kind == "inclusive") {
    RAJA::inclusive_scan<POL>(xs, ys, OP{});
  } else if (kind == "exclusive") {
    if (has_init) RAJA::exclusive_scan<POL>(xs, ys, OP{}, init);
    else RAJA::exclusive_scan<POL>(xs, ys, OP{});
  } else if (kind == "inclusive_inplace") {
    y = x;
    RAJA::inclusive_scan_inplace<POL>(ys, OP{});
  } else if (kind == "exclusive_inplace") {
    y = x;
    if (has_init) RAJA::exclusive_scan_inplace<POL>(ys, OP{}, init);
    else RAJA::exclusive_scan_inplace<POL>(ys, OP{});
  } else {
    die("unknown scan kind");
  }
  Out o(out);
  o.put(y);
}

template <class T, class POL>
void run_scan(const std::string& kind, const std::string& op, size_t n, const char* in,
              const char* out, int argc, char** argv, int iarg)
{
  const bool has_init = argc > iarg;
  T init = T(0);
  if (has_init) {
    if (std::is_floating_point<T>::value) init = T(std::strtod(argv[iarg], nullptr));
    else init = T(std::strtoll(argv[iarg], nullptr, 10));
  }
  if (op == "plus") run_scan_op<T, POL, RAJA::operators::plus<T>>(kind, n, in, out, has_init, init);
  else if (op == "minimum")
    run_scan_op<T, POL, RAJA::operators::minimum<T>>(kind, n, in, out, has_init, init);
  else if (op == "maximum")
    run_scan_op<T, POL, RAJA::operators::maximum<T>>(kind, n, in, out, has_init, init);
  else die("unknown scan op");
}

// -------------------------------------------------------------------- sort
template <class K, class POL, class CMP>
void run_sort_cmp(bool stable, size_t n, int argc, char** argv, int iarg)
{
  std::vector<K> k = read_vec<K>(argv[iarg], n);
  auto ks = RAJA::make_span(k.data(), RAJA::Index_type(n));
  if (argc > iarg + 3) {
    std::vector<int32_t> v = read_vec<int32_t>(argv[iarg + 2], n);
    auto vs = RAJA::make_span(v.data(), RAJA::Index_type(n));
    if (stable) RAJA::stable_sort_pairs<POL>(ks, vs, CMP{});
    else RAJA::sort_pairs<POL>(ks, vs, CMP{});
    Out ov(argv[iarg + 3]);
    ov.put(v);
  } else {
    if (stable) RAJA::stable_sort<POL>(ks, CMP{});
    else RAJA::sort<POL>(ks, CMP{});
  }
  Out o(argv[iarg + 1]);
  o.put(k);
}

template <class K, class POL>
void run_sort(const std::string& kind, const std::string& dir, size_t n, int argc, char** argv,
              int iarg)
{
  const bool stable = kind == "stable_sort";
  if (!stable && kind != "sort") die("unknown sort kind");
  if (dir == "asc") run_sort_cmp<K, POL, RAJA::operators::less<K>>(stable, n, argc, argv, iarg);
  else if (dir == "desc") run_sort_cmp<K, POL, RAJA::operators::greater<K>>(stable, n, argc, argv, iarg);
  else die("unknown sort direction");
}

// --------------------------------------------------------------- histogram
template <class POL, class MRED>
void run_hist(size_t n, int nbins, const char* in, const char* out)
{
  std::vector<int32_t> b = read_vec<int32_t>(in, n);
  const int32_t* bp = b.data();
  RAJA::MultiReduceSum<MRED, long long> counts(size_t(nbins), 0LL);
  RAJA::forall<POL>(RAJA::TypedRangeSegment<RAJA::Index_type>(0, RAJA::Index_type(n)),
                    [=](RAJA::Index_type i) { counts[bp[i]] += 1LL; });
  std::vector<long long> totals(static_cast<size_t>(nbins));
  for (int i = 0; i < nbins; ++i) totals[size_t(i)] = counts.get(size_t(i));
  Out o(out);
  o.put(totals);
}

// ------------------------------------------------------------------- daxpy
template <class POL>
void run_daxpy(size_t n, double a, const char* xin, const char* yin, const char* out)
{
  std::vector<double> x = read_vec<double>(xin, n), y = read_vec<double>(yin, n);
  const double* xp = x.data();
  double* yp = y.data();
  RAJA::forall<POL>(RAJA::TypedRangeSegment<RAJA::Index_type>(0, RAJA::Index_type(n)),
                    [=](RAJA::Index_type i) { yp[i] += a * xp[i]; });
  Out o(out);
  o.put(y);
}

// --------------------------------------------------------------- workgroup
void run_workgroup(size_t nloops, size_t total, const char* bin, const char* ein, const char* out)
{
  std::vector<int64_t> b = read_vec<int64_t>(bin, nloops), e = read_vec<int64_t>(ein, nloops);
  std::vector<int64_t> a(total, 0);
  int64_t* ap = a.data();
  using policy = RAJA::WorkGroupPolicy<RAJA::seq_work, RAJA::ordered,
                                       RAJA::ragged_array_of_objects>;
  using pool_t = RAJA::WorkPool<policy, RAJA::Index_type, RAJA::xargs<>, std::allocator<char>>;
  using group_t = RAJA::WorkGroup<policy, RAJA::Index_type, RAJA::xargs<>, std::allocator<char>>;
  pool_t pool(std::allocator<char>{});
  for (size_t l = 0; l < nloops; ++l) {
    pool.enqueue(RAJA::TypedRangeSegment<RAJA::Index_type>(b[l], e[l]),
                 [=](RAJA::Index_type i) { ap[i] += i + 5; });
  }
  group_t group = pool.instantiate();
  group.run();
  group.run();
  Out o(out);
  o.put(a);
}

template <class F>
void by_key_type(const std::string& t, F&& f)
{
  if (t == "u32") f(uint32_t{});
  else if (t == "i32") f(int32_t{});
  else if (t == "u64") f(uint64_t{});
  else if (t == "i64") f(int64_t{});
  else if (t == "f32") f(float{});
  else if (t == "f64") f(double{});
  else die("unknown type");
}
}  // namespace

int main(int argc, char** argv)
{
  if (argc < 2) die("usage: see the file header");
  const std::string job = argv[1];
  if (job == "reduce" && argc == 7) {
    const std::string pol = argv[3];
    const size_t n = std::strtoull(argv[4], nullptr, 10);
    const std::string t = argv[2];
    auto go = [&](auto tag) {
      using T = decltype(tag);
      if constexpr (std::is_same<T, uint32_t>::value || std::is_same<T, uint64_t>::value) {
        die("reduce types are i32 i64 f32 f64");
      } else {
        if (pol == "seq") run_reduce<T, seq_pol, RAJA::seq_reduce>(n, argv[5], argv[6]);
        else run_reduce<T, omp_pol, omp_red>(n, argv[5], argv[6]);
      }
    };
    by_key_type(t, go);
  } else if (job == "params" && argc == 6) {
    const size_t n = std::strtoull(argv[3], nullptr, 10);
    auto go = [&](auto tag) {
      using T = decltype(tag);
      if constexpr (std::is_same<T, uint32_t>::value || std::is_same<T, uint64_t>::value) die("types");
      else run_params<T>(n, argv[4], argv[5]);
    };
    by_key_type(argv[2], go);
  } else if (job == "scan" && argc >= 9) {
    const std::string pol = argv[3], kind = argv[4], op = argv[5];
    const size_t n = std::strtoull(argv[6], nullptr, 10);
    auto go = [&](auto tag) {
      using T = decltype(tag);
      if (pol == "seq") run_scan<T, seq_pol>(kind, op, n, argv[7], argv[8], argc, argv, 9);
      else run_scan<T, omp_pol>(kind, op, n, argv[7], argv[8], argc, argv, 9);
    };
    by_key_type(argv[2], go);
  } else if (job == "sort" && (argc == 9 || argc == 11)) {
    const std::string pol = argv[3], kind = argv[4], dir = argv[5];
    const size_t n = std::strtoull(argv[6], nullptr, 10);
    auto go = [&](auto tag) {
      using K = decltype(tag);
      if (pol == "seq") run_sort<K, seq_pol>(kind, dir, n, argc, argv, 7);
      else run_sort<K, omp_pol>(kind, dir, n, argc, argv, 7);
    };
    by_key_type(argv[2], go);
  } else if (job == "hist" && argc == 7) {
    const std::string pol = argv[2];
    const size_t n = std::strtoull(argv[3], nullptr, 10);
    const int nbins = std::atoi(argv[4]);
    if (pol == "seq") run_hist<seq_pol, RAJA::seq_multi_reduce>(n, nbins, argv[5], argv[6]);
    else run_hist<omp_pol, omp_mred>(n, nbins, argv[5], argv[6]);
  } else if (job == "daxpy" && argc == 8) {
    const std::string pol = argv[2];
    const size_t n = std::strtoull(argv[3], nullptr, 10);
    const double a = std::strtod(argv[4], nullptr);
    if (pol == "seq") run_daxpy<seq_pol>(n, a, argv[5], argv[6], argv[7]);
    else run_daxpy<omp_pol>(n, a, argv[5], argv[6], argv[7]);
  } else if (job == "workgroup" && argc == 7) {
    run_workgroup(std::strtoull(argv[2], nullptr, 10), std::strtoull(argv[3], nullptr, 10), argv[4],
                  argv[5], argv[6]);
  } else {
    die("bad arguments (see the file header)");
  }
  return 0;
}
