// RAJA-API programs on the b200 policies, checked against seq_exec on the
// same inputs.  Mirrors the reference's functional tests:
//   test/functional/forall/reduce-basic (segments, init values, planted
//   MinLoc/MaxLoc extremes, reset, two-loop accumulation), the expt param
//   reducers, forall over IndexSets, test/functional/scan (iota inputs,
//   N in {357, 32000}, plus/min/max, non-identity offsets), sort /
//   stable_sort / sort_pairs, and test/functional/workgroup (a[i] += i + 5).
// Prints one PASS/FAIL line per case; the exit status is the failure count.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cmath>
#include <cstdlib>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "RAJA/RAJA.hpp"
#include "raja_b200/RAJA_b200.hpp"

using RAJA::Index_type;
using exec = RAJA::b200_exec<256>;
using red = RAJA::b200_reduce;

static int g_fail = 0;
#define CHECK(name, cond)                              \
  do {                                                 \
    if (cond) {                                        \
      printf("PASS %s\n", name);                       \
    } else {                                           \
      printf("FAIL %s (%s:%d)\n", name, __FILE__, __LINE__); \
      ++g_fail;                                        \
    }                                                  \
  } while (0)

template <class T>
T* managed(size_t n) {
  T* p = nullptr;
  if (cudaMallocManaged(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) {
    printf("FAIL cudaMallocManaged\n");
    exit(1);
  }
  return p;
}

// ------------------------------------------------------------ reducers
template <class Seg>
void reduce_case(const char* tag, const Seg& seg, const std::vector<Index_type>& idx, std::mt19937& rng) {
  const Index_type data_len = idx.back() + 1;
  double* a = managed<double>(data_len);
  int* b = managed<int>(data_len);
  for (Index_type i = 0; i < data_len; ++i) {
    a[i] = double(rng() % 100);
    b[i] = int(rng() % 100);
  }
  const Index_type loc_idx = idx[idx.size() * 2 / 3];
  a[loc_idx] = -100.0;  // planted unique minimum
  char nm[128];

  // device reducers (init 0 and 2, as the reference tests)
  RAJA::ReduceSum<red, double> sum(0.0), sum2(2.0);
  RAJA::ReduceMin<red, double> mn(1e9);
  RAJA::ReduceMax<red, double> mx(-1e9);
  RAJA::ReduceMinLoc<red, double, Index_type> mnl(101.0, -1), mninit(-100.0, -1);
  RAJA::ReduceMaxLoc<red, double, Index_type> mxl(-100.0, -1);
  RAJA::ReduceBitOr<red, int> bor(0);
  RAJA::ReduceBitAnd<red, int> band(~0);
  RAJA::forall<exec>(seg, [=] RAJA_DEVICE(Index_type i) {
    sum += a[i];
    sum2 += a[i];
    mn.min(a[i]);
    mx.max(a[i]);
    mnl.minloc(a[i], i);
    mninit.minloc(a[i], i);
    mxl.maxloc(a[i], i);
    bor |= b[i];
    band &= b[i];
  });
  // host references (seq semantics)
  RAJA::ReduceSum<RAJA::seq_reduce, double> hs(0.0);
  RAJA::ReduceMinLoc<RAJA::seq_reduce, double, Index_type> hml(101.0, -1), hminit(-100.0, -1);
  RAJA::ReduceMaxLoc<RAJA::seq_reduce, double, Index_type> hxl(-100.0, -1);
  RAJA::ReduceMin<RAJA::seq_reduce, double> hmn(1e9);
  RAJA::ReduceMax<RAJA::seq_reduce, double> hmx(-1e9);
  RAJA::ReduceBitOr<RAJA::seq_reduce, int> hbor(0);
  RAJA::ReduceBitAnd<RAJA::seq_reduce, int> hband(~0);
  RAJA::forall<RAJA::seq_exec>(seg, [=](Index_type i) {
    hs += a[i];
    hml.minloc(a[i], i);
    hminit.minloc(a[i], i);
    hxl.maxloc(a[i], i);
    hmn.min(a[i]);
    hmx.max(a[i]);
    hbor |= b[i];
    hband &= b[i];
  });
  snprintf(nm, sizeof nm, "reduce_sum_%s", tag);
  CHECK(nm, sum.get() == hs.get() && sum2.get() == hs.get() + 2.0);
  snprintf(nm, sizeof nm, "reduce_minmax_%s", tag);
  CHECK(nm, mn.get() == hmn.get() && mx.get() == hmx.get());
  snprintf(nm, sizeof nm, "reduce_minloc_%s", tag);
  CHECK(nm, mnl.get() == hml.get() && mnl.getLoc() == hml.getLoc() && mnl.get() == -100.0 &&
                mnl.getLoc() == loc_idx);
  snprintf(nm, sizeof nm, "reduce_minloc_init_wins_%s", tag);
  CHECK(nm, mninit.get() == -100.0 && mninit.getLoc() == -1 && hminit.getLoc() == -1);
  snprintf(nm, sizeof nm, "reduce_maxloc_%s", tag);
  CHECK(nm, mxl.get() == hxl.get() && mxl.getLoc() == hxl.getLoc());
  snprintf(nm, sizeof nm, "reduce_bit_%s", tag);
  CHECK(nm, bor.get() == hbor.get() && band.get() == hband.get());

  // reset, then two loops accumulate twice (test-forall-basic-ReduceSum.hpp)
  sum.reset(0.0);
  for (int k = 0; k < 2; ++k) RAJA::forall<exec>(seg, [=] RAJA_DEVICE(Index_type i) { sum += a[i]; });
  snprintf(nm, sizeof nm, "reduce_sum_two_loops_%s", tag);
  CHECK(nm, sum.get() == 2.0 * hs.get());
  cudaFree(a);
  cudaFree(b);
}

void test_reducers() {
  std::mt19937 rng(12345);
  std::vector<Index_type> idx;
  auto range = [&](Index_type b, Index_type e) {
    idx.clear();
    for (Index_type i = b; i < e; ++i) idx.push_back(i);
  };
  range(0, 28);
  reduce_case("r0_28", RAJA::RangeSegment(0, 28), idx, rng);
  range(3, 642);
  reduce_case("r3_642", RAJA::RangeSegment(3, 642), idx, rng);
  range(0, 2057);
  reduce_case("r0_2057", RAJA::RangeSegment(0, 2057), idx, rng);
  idx.clear();
  for (Index_type i = 0; i < 188; i += 2) idx.push_back(i);
  reduce_case("s0_188_2", RAJA::RangeStrideSegment(0, 188, 2), idx, rng);
  idx.clear();
  for (Index_type i = 3; i < 1029; i += 3) idx.push_back(i);
  reduce_case("s3_1029_3", RAJA::RangeStrideSegment(3, 1029, 3), idx, rng);
  // random list segment (test-forall-basic-ReduceSum list case)
  idx.clear();
  for (Index_type i = 0; i < 10567; ++i)
    if (Index_type(rng() % 10567) > i) idx.push_back(i);
  Index_type* lst = managed<Index_type>(idx.size());
  for (size_t i = 0; i < idx.size(); ++i) lst[i] = idx[i];
  reduce_case("list", RAJA::ListSegment(lst, Index_type(idx.size())), idx, rng);
  cudaFree(lst);

  // large: fp64 ties everywhere, MinLoc picks the first index like seq
  const Index_type n = (1 << 22) + 3;
  double* x = managed<double>(n);
  for (Index_type i = 0; i < n; ++i) x[i] = double(rng() % 5);
  RAJA::ReduceMinLoc<red, double, Index_type> m(1e9, -1);
  RAJA::ReduceMaxLoc<red, double, Index_type> M(-1e9, -1);
  RAJA::forall<exec>(RAJA::RangeSegment(0, n), [=] RAJA_DEVICE(Index_type i) {
    m.minloc(x[i], i);
    M.maxloc(x[i], i);
  });
  Index_type first0 = -1, first4 = -1;
  for (Index_type i = 0; i < n && (first0 < 0 || first4 < 0); ++i) {
    if (x[i] == 0.0 && first0 < 0) first0 = i;
    if (x[i] == 4.0 && first4 < 0) first4 = i;
  }
  CHECK("minloc_ties_lowest_index", m.get() == 0.0 && m.getLoc() == first0);
  CHECK("maxloc_ties_lowest_index", M.get() == 4.0 && M.getLoc() == first4);
  cudaFree(x);
}

// -------------------------------------------------------- forall + params
void test_forall_and_params() {
  const Index_type n = (1 << 20) + 7;
  double* x = managed<double>(n);
  double* y = managed<double>(n);
  double* yh = managed<double>(n);
  std::mt19937 rng(7);
  for (Index_type i = 0; i < n; ++i) {
    x[i] = double(rng() % 1000) / 8.0;
    y[i] = yh[i] = double(rng() % 1000) / 16.0;
  }
  const double alpha = 2.5;
  RAJA::forall<exec>(RAJA::RangeSegment(0, n), [=] RAJA_DEVICE(Index_type i) { y[i] += alpha * x[i]; });
  RAJA::forall<RAJA::seq_exec>(RAJA::RangeSegment(0, n), [=](Index_type i) { yh[i] += alpha * x[i]; });
  bool ok = true;
  for (Index_type i = 0; i < n; ++i) ok = ok && (y[i] == yh[i]);  // exact: multiples of 1/16
  CHECK("forall_daxpy", ok);

  // expt::Reduce / ReduceLoc params: target = op(target, result)
  double s = 10.0, lo = 1e300, hi = -1e300, vmin = 1e300;
  Index_type imin = -1;
  RAJA::forall<exec>(RAJA::RangeSegment(0, n), RAJA::Name("expt_reduce"),
                     RAJA::expt::Reduce<RAJA::operators::plus>(&s),
                     RAJA::expt::Reduce<RAJA::operators::minimum>(&lo),
                     RAJA::expt::Reduce<RAJA::operators::maximum>(&hi),
                     RAJA::expt::ReduceLoc<RAJA::operators::minimum>(&vmin, &imin),
                     [=] RAJA_DEVICE(Index_type i, RAJA::expt::ValOp<double, RAJA::operators::plus>& vs,
                                     RAJA::expt::ValOp<double, RAJA::operators::minimum>& vlo,
                                     RAJA::expt::ValOp<double, RAJA::operators::maximum>& vhi,
                                     RAJA::expt::ValOp<RAJA::expt::ValLoc<double, Index_type>,
                                                       RAJA::operators::minimum>& vml) {
                       vs += x[i];
                       vlo.min(x[i]);
                       vhi.max(x[i]);
                       vml.minloc(x[i], i);
                     });
  double hs = 10.0, hlo = 1e300, hhi = -1e300;
  Index_type himin = -1;
  double hvmin = 1e300;
  for (Index_type i = 0; i < n; ++i) {
    hs += x[i];
    hlo = x[i] < hlo ? x[i] : hlo;
    hhi = hhi < x[i] ? x[i] : hhi;
    if (x[i] < hvmin) {
      hvmin = x[i];
      himin = i;
    }
  }
  CHECK("expt_reduce_sum", s == hs);
  CHECK("expt_reduce_min_max", lo == hlo && hi == hhi);
  CHECK("expt_reduceloc_min", vmin == hvmin && imin == himin);

  // IndexSet: all segments in one launch
  RAJA::TypedIndexSet<RAJA::RangeSegment> is;
  is.push_back(RAJA::RangeSegment(0, 100));
  is.push_back(RAJA::RangeSegment(1000, 5000));
  is.push_back(RAJA::RangeSegment(7, 7));
  is.push_back(RAJA::RangeSegment(200000, 200333));
  for (Index_type i = 0; i < n; ++i) y[i] = yh[i] = 0.0;
  RAJA::ReduceSum<red, double> cnt(0.0);
  RAJA::forall<exec>(is, [=] RAJA_DEVICE(Index_type i) {
    y[i] += double(i);
    cnt += 1.0;
  });
  RAJA::forall<RAJA::seq_exec>(is, [=](Index_type i) { yh[i] += double(i); });
  ok = cnt.get() == 100 + 4000 + 333;
  for (Index_type i = 0; i < n; ++i) ok = ok && (y[i] == yh[i]);
  CHECK("forall_indexset_one_launch", ok);
  cudaFree(x);
  cudaFree(y);
  cudaFree(yh);
}

// ------------------------------------------------------------------ scans
template <class T, class Op>
void scan_case(const char* tag, Index_type n, T offset) {
  T* in = managed<T>(n);
  T* out = managed<T>(n);
  T* ref = managed<T>(n);
  for (Index_type i = 0; i < n; ++i) in[i] = T(i + 1);  // std::iota(.., 1)
  char nm[128];
  RAJA::inclusive_scan<exec>(RAJA::make_span((const T*)in, n), RAJA::make_span(out, n), Op{});
  RAJA::inclusive_scan<RAJA::seq_exec>(RAJA::make_span((const T*)in, n), RAJA::make_span(ref, n), Op{});
  bool ok = true;
  for (Index_type i = 0; i < n; ++i) ok = ok && out[i] == ref[i];
  snprintf(nm, sizeof nm, "inclusive_scan_%s_%ld", tag, (long)n);
  CHECK(nm, ok);
  RAJA::exclusive_scan<exec>(RAJA::make_span((const T*)in, n), RAJA::make_span(out, n), Op{}, offset);
  RAJA::exclusive_scan<RAJA::seq_exec>(RAJA::make_span((const T*)in, n), RAJA::make_span(ref, n), Op{}, offset);
  ok = true;
  for (Index_type i = 0; i < n; ++i) ok = ok && out[i] == ref[i];
  snprintf(nm, sizeof nm, "exclusive_scan_%s_%ld", tag, (long)n);
  CHECK(nm, ok);
  for (Index_type i = 0; i < n; ++i) out[i] = in[i];
  RAJA::inclusive_scan_inplace<exec>(RAJA::make_span(out, n), Op{});
  RAJA::inclusive_scan<RAJA::seq_exec>(RAJA::make_span((const T*)in, n), RAJA::make_span(ref, n), Op{});
  ok = true;
  for (Index_type i = 0; i < n; ++i) ok = ok && out[i] == ref[i];
  snprintf(nm, sizeof nm, "inclusive_scan_inplace_%s_%ld", tag, (long)n);
  CHECK(nm, ok);
  cudaFree(in);
  cudaFree(out);
  cudaFree(ref);
}

void test_scans() {
  for (Index_type n : {Index_type(357), Index_type(32000), Index_type((1 << 20) + 1)}) {
    const int off = n == 357 ? 15 : 2;
    scan_case<int, RAJA::operators::plus<int>>("plus_int", n, off);
    scan_case<int, RAJA::operators::minimum<int>>("min_int", n, off);
    scan_case<int, RAJA::operators::maximum<int>>("max_int", n, off);
    scan_case<double, RAJA::operators::plus<double>>("plus_double", n, double(off));
    scan_case<double, RAJA::operators::minimum<double>>("min_double", n, double(off));
    scan_case<long, RAJA::operators::plus<long>>("plus_long", n, long(off));
  }
}

// ------------------------------------------------------------------ sorts
void test_sorts() {
  std::mt19937 rng(99);
  for (Index_type n : {Index_type(0), Index_type(1), Index_type(10), Index_type(10000), Index_type(1 << 20)}) {
    int* k = managed<int>(n);
    int* kr = managed<int>(n);
    int* v = managed<int>(n);
    int* vr = managed<int>(n);
    auto fill = [&] {
      for (Index_type i = 0; i < n; ++i) {
        k[i] = kr[i] = int(rng() % (2 * n + 1)) - int(n);  // U[-N, N]: duplicates
        v[i] = vr[i] = int(i);
      }
    };
    char nm[96];
    fill();
    RAJA::sort<exec>(RAJA::make_span(k, n));
    RAJA::sort<RAJA::seq_exec>(RAJA::make_span(kr, n));
    bool ok = true;
    for (Index_type i = 0; i < n; ++i) ok = ok && k[i] == kr[i];
    snprintf(nm, sizeof nm, "sort_%ld", (long)n);
    CHECK(nm, ok);
    fill();
    RAJA::stable_sort<exec>(RAJA::make_span(k, n), RAJA::operators::greater<int>{});
    RAJA::stable_sort<RAJA::seq_exec>(RAJA::make_span(kr, n), RAJA::operators::greater<int>{});
    ok = true;
    for (Index_type i = 0; i < n; ++i) ok = ok && k[i] == kr[i];
    snprintf(nm, sizeof nm, "stable_sort_greater_%ld", (long)n);
    CHECK(nm, ok);
    fill();
    RAJA::stable_sort_pairs<exec>(RAJA::make_span(k, n), RAJA::make_span(v, n));
    RAJA::stable_sort_pairs<RAJA::seq_exec>(RAJA::make_span(kr, n), RAJA::make_span(vr, n));
    ok = true;
    for (Index_type i = 0; i < n; ++i) ok = ok && k[i] == kr[i] && v[i] == vr[i];
    snprintf(nm, sizeof nm, "stable_sort_pairs_%ld", (long)n);
    CHECK(nm, ok);
    fill();
    RAJA::sort_pairs<exec>(RAJA::make_span(k, n), RAJA::make_span(v, n), RAJA::operators::greater<int>{});
    RAJA::stable_sort_pairs<RAJA::seq_exec>(RAJA::make_span(kr, n), RAJA::make_span(vr, n),
                                            RAJA::operators::greater<int>{});
    ok = true;
    for (Index_type i = 0; i < n; ++i) ok = ok && k[i] == kr[i] && v[i] == vr[i];
    snprintf(nm, sizeof nm, "sort_pairs_greater_%ld", (long)n);
    CHECK(nm, ok);
    // any 4- or 8-byte value type: double and Index_type values, float keys
    {
      double* dv = managed<double>(n);
      double* dvr = managed<double>(n);
      Index_type* iv = managed<Index_type>(n);
      Index_type* ivr = managed<Index_type>(n);
      float* fk = managed<float>(n);
      float* fkr = managed<float>(n);
      fill();
      for (Index_type i = 0; i < n; ++i) {
        dv[i] = dvr[i] = 0.5 * double(i);
        iv[i] = ivr[i] = n - i;
        fk[i] = fkr[i] = float(k[i]) * 0.25f;
      }
      RAJA::stable_sort_pairs<exec>(RAJA::make_span(k, n), RAJA::make_span(dv, n));
      RAJA::stable_sort_pairs<RAJA::seq_exec>(RAJA::make_span(kr, n), RAJA::make_span(dvr, n));
      RAJA::stable_sort_pairs<exec>(RAJA::make_span(fk, n), RAJA::make_span(iv, n),
                                    RAJA::operators::greater<float>{});
      RAJA::stable_sort_pairs<RAJA::seq_exec>(RAJA::make_span(fkr, n), RAJA::make_span(ivr, n),
                                              RAJA::operators::greater<float>{});
      ok = true;
      for (Index_type i = 0; i < n; ++i)
        ok = ok && k[i] == kr[i] && dv[i] == dvr[i] && fk[i] == fkr[i] && iv[i] == ivr[i];
      snprintf(nm, sizeof nm, "stable_sort_pairs_double_and_index_values_%ld", (long)n);
      CHECK(nm, ok);
      cudaFree(dv);
      cudaFree(dvr);
      cudaFree(iv);
      cudaFree(ivr);
      cudaFree(fk);
      cudaFree(fkr);
    }
    cudaFree(k);
    cudaFree(kr);
    cudaFree(v);
    cudaFree(vr);
  }
}

// -------------------------------------------------------------- WorkGroup
template <class ORDER>
void workgroup_case(const char* tag) {
  const Index_type n = 1 << 20;
  int* a = managed<int>(n);
  int* r = managed<int>(n);
  for (Index_type i = 0; i < n; ++i) a[i] = r[i] = 0;
  using pool_t = RAJA::WorkPool<RAJA::WorkGroupPolicy<RAJA::b200_work<256>, ORDER>, Index_type>;
  using hpool_t = RAJA::WorkPool<RAJA::WorkGroupPolicy<RAJA::seq_exec, RAJA::ordered>, Index_type>;
  pool_t pool;
  hpool_t hpool;
  std::mt19937 rng(5);
  Index_type b = 0;
  int loops = 0;
  while (b < n) {
    const Index_type len = Index_type(rng() % 5000);  // uneven lengths, some empty
    const Index_type e = b + len < n ? b + len : n;
    pool.enqueue(RAJA::RangeSegment(b, e), [=] RAJA_DEVICE(Index_type i) { a[i] += int(i) + 5; });
    hpool.enqueue(RAJA::RangeSegment(b, e), [=](Index_type i) { r[i] += int(i) + 5; });
    b = e + Index_type(rng() % 7);  // gaps stay untouched
    ++loops;
  }
  auto g = pool.instantiate();
  auto hg = hpool.instantiate();
  g.run();
  g.run();  // a group runs again with the same loops
  hg.run();
  hg.run();
  bool ok = true;
  for (Index_type i = 0; i < n; ++i) ok = ok && a[i] == r[i];
  char nm[96];
  snprintf(nm, sizeof nm, "workgroup_%s_%d_loops", tag, loops);
  CHECK(nm, ok);
  cudaFree(a);
  cudaFree(r);
}

// MultiReduce on b200 against seq, and b200 atomics in device code
// WorkGroup with a dispatch policy and an allocator; pool reuse after
// instantiate and a group run twice (test-workgroup-*-MultipleReuse.hpp)
void test_workgroup_reuse() {
  const int n = 5000;
  int* a = managed<int>(2 * n);
  for (int i = 0; i < 2 * n; ++i) a[i] = 0;
  using wpol = RAJA::WorkGroupPolicy<RAJA::b200_work<256>, RAJA::unordered, RAJA::ragged_array_of_objects,
                                     RAJA::indirect_function_call_dispatch>;
  RAJA::WorkPool<wpol, Index_type, RAJA::xargs<>, std::allocator<char>> pool(std::allocator<char>{});
  bool ok = true;
  for (int reuse = 0; reuse < 2; ++reuse) {
    pool.enqueue(RAJA::RangeSegment(0, n), [=] __device__(Index_type i) { a[i] += 1; });
    pool.enqueue(RAJA::RangeSegment(n, 2 * n), [=] __device__(Index_type i) { a[i] += 10; });
    auto group = pool.instantiate();
    ok = ok && pool.num_loops() == 0;
    group.run();
    group.run();
  }
  for (int i = 0; i < 2 * n; ++i) ok = ok && a[i] == (i < n ? 4 : 40);
  CHECK("workgroup_b200_dispatch_allocator_reuse", ok);
  cudaFree(a);
}

// Loops whose bodies capture ReduceSum / ReduceMinLoc on b200_reduce: the
// batched-loops configuration (4096 loops, lognormal lengths with median
// 2000 and sigma 1.5 clipped to [32, 2^20]), fp64 axpy plus one sum and one
// MinLoc per loop, run twice.  The unordered runner combines each loop's
// reducers inside its single launch (the reference's unordered CUDA runner
// leaves reducers unsupported, policy/cuda/WorkGroup/WorkRunner.hpp:323-329);
// the ordered runner launches the loops one by one.  Values are multiples of
// 1/8 so sums are exact in any order: both must equal seq_exec loop by loop.
template <class ORDER>
void workgroup_reducers_case(const char* tag) {
  std::mt19937 rng(41);
  std::lognormal_distribution<double> ln(std::log(2000.0), 1.5);
  const int nloops = 4096;
  std::vector<Index_type> lens(nloops), offs(nloops + 1, 0);
  for (int l = 0; l < nloops; ++l) {
    double v = std::round(ln(rng));
    v = v < 32 ? 32 : (v > double(1 << 20) ? double(1 << 20) : v);
    lens[l] = Index_type(v);
    offs[l + 1] = offs[l] + lens[l];
  }
  lens[7] = 0;  // an empty loop keeps its reducers' values
  for (int l = 7; l < nloops; ++l) offs[l + 1] = offs[l] + lens[l];
  const Index_type total = offs[nloops];
  double* x = managed<double>(total);
  double* y = managed<double>(total);
  double* hy = managed<double>(total);
  for (Index_type i = 0; i < total; ++i) {
    x[i] = double(int(rng() % 257) - 128) / 8.0;
    y[i] = hy[i] = double(int(rng() % 257) - 128) / 8.0;
  }
  using pool_t = RAJA::WorkPool<RAJA::WorkGroupPolicy<RAJA::b200_work<256>, ORDER>, Index_type>;
  using hpool_t = RAJA::WorkPool<RAJA::WorkGroupPolicy<RAJA::seq_exec, RAJA::ordered>, Index_type>;
  using dsum_t = RAJA::ReduceSum<RAJA::b200_reduce, double>;
  using dloc_t = RAJA::ReduceMinLoc<RAJA::b200_reduce, double, Index_type>;
  using hsum_t = RAJA::ReduceSum<RAJA::seq_reduce, double>;
  using hloc_t = RAJA::ReduceMinLoc<RAJA::seq_reduce, double, Index_type>;
  std::vector<std::unique_ptr<dsum_t>> ds;
  std::vector<std::unique_ptr<dloc_t>> dl;
  std::vector<std::unique_ptr<hsum_t>> hs;
  std::vector<std::unique_ptr<hloc_t>> hl;
  pool_t pool;
  hpool_t hpool;
  const double a = 0.5;
  for (int l = 0; l < nloops; ++l) {
    ds.emplace_back(new dsum_t(1.0));
    dl.emplace_back(new dloc_t(1e300, -1));
    hs.emplace_back(new hsum_t(1.0));
    hl.emplace_back(new hloc_t(1e300, -1));
    const dsum_t& s = *ds.back();
    const dloc_t& m = *dl.back();
    const hsum_t& hsr = *hs.back();
    const hloc_t& hm = *hl.back();
    pool.enqueue(RAJA::RangeSegment(offs[l], offs[l + 1]), [=] RAJA_DEVICE(Index_type i) {
      y[i] += a * x[i];
      s += y[i];
      m.minloc(y[i], i);
    });
    hpool.enqueue(RAJA::RangeSegment(offs[l], offs[l + 1]), [=](Index_type i) {
      hy[i] += a * x[i];
      hsr += hy[i];
      hm.minloc(hy[i], i);
    });
  }
  auto g = pool.instantiate();
  auto hg = hpool.instantiate();
  g.run();
  g.run();  // the reducers accumulate over both runs
  hg.run();
  hg.run();
  bool ok = true;
  int bad = -1;
  for (int l = 0; l < nloops && ok; ++l) {
    ok = ds[l]->get() == hs[l]->get() && dl[l]->get() == hl[l]->get() && dl[l]->getLoc() == hl[l]->getLoc();
    if (!ok) bad = l;
  }
  for (Index_type i = 0; i < total && ok; ++i) ok = y[i] == hy[i];
  char nm[128];
  snprintf(nm, sizeof nm, "workgroup_%s_fused_reducers_%d_loops_%lld_elems%s", tag, nloops, (long long)total,
           ok ? "" : " (first mismatch logged)");
  if (bad >= 0)
    printf("  loop %d: sum %.17g vs %.17g, minloc %.17g@%lld vs %.17g@%lld\n", bad, ds[bad]->get(),
           hs[bad]->get(), dl[bad]->get(), (long long)dl[bad]->getLoc(), hl[bad]->get(),
           (long long)hl[bad]->getLoc());
  CHECK(nm, ok);
  cudaFree(x);
  cudaFree(y);
  cudaFree(hy);
}

// b200_exec<0> / b200_work<0>: the launch shape is tuned on line.  Every
// call must be right whatever shape it runs with, and the tuners settle
// once each candidate has been timed.
void test_autotune() {
  const Index_type n = (Index_type(1) << 20) + 3;
  double* x = managed<double>(n);
  double* y = managed<double>(n);
  long long hx = 0;
  for (Index_type i = 0; i < n; ++i) {
    x[i] = double(i % 17);
    y[i] = 0.0;
    hx += (long long)(i % 17);
  }
  using tuned = RAJA::b200_exec<0>;
  const int calls = 40;
  bool sums_ok = true, params_ok = true;
  for (int c = 0; c < calls; ++c) {
    RAJA::forall<tuned>(RAJA::RangeSegment(0, n), [=] RAJA_DEVICE(Index_type i) { y[i] += x[i]; });
    RAJA::ReduceSum<red, long long> s(5);
    RAJA::forall<tuned>(RAJA::RangeSegment(0, n), [=] RAJA_DEVICE(Index_type i) { s += (long long)x[i]; });
    sums_ok = sums_ok && s.get() == hx + 5;
    double ps = 1.0;
    RAJA::forall<tuned>(RAJA::RangeSegment(0, n), RAJA::expt::Reduce<RAJA::operators::plus>(&ps),
                        [=] RAJA_DEVICE(Index_type i, RAJA::expt::ValOp<double, RAJA::operators::plus>& v) {
                          v += x[i];
                        });
    params_ok = params_ok && ps == double(hx) + 1.0;
  }
  bool y_ok = true;
  for (Index_type i = 0; i < n && y_ok; ++i) y_ok = y[i] == double(calls) * x[i];
  CHECK("autotuned_forall_every_call_exact", y_ok);
  CHECK("autotuned_forall_reducer_every_call_exact", sums_ok);
  CHECK("autotuned_forall_params_every_call_exact", params_ok);
  int settled = 0, seen = 0;
  for (const auto& r : RAJA::b200::tune::reports()) {
    if (r.size_class != 20) continue;
    ++seen;
    printf("  tuner %s class 2^%d: %s, %d candidates, %d timed, shape %d x %d\n", r.name.c_str(), r.size_class,
           r.settled ? "settled" : "tuning", r.candidates, r.timed_calls, r.best.block, r.best.items);
    settled += r.settled ? 1 : 0;
  }
  CHECK("autotuned_forall_tuners_settle", seen >= 3 && settled == seen);

  // WorkGroup: 600 uneven loops with fused reducers, the tile shape tuned
  // over the runs; integer-valued data keeps every sum exact
  std::mt19937 rng(5);
  std::lognormal_distribution<double> ln(std::log(2000.0), 1.5);
  const int nloops = 600;
  std::vector<Index_type> offs(nloops + 1, 0);
  for (int l = 0; l < nloops; ++l) {
    double v = std::round(ln(rng));
    v = v < 32 ? 32 : (v > double(1 << 18) ? double(1 << 18) : v);
    offs[l + 1] = offs[l] + Index_type(v);
  }
  const Index_type total = offs[nloops];
  double* w = managed<double>(total);
  for (Index_type i = 0; i < total; ++i) w[i] = double(int(rng() % 33) - 16);
  using pool_t = RAJA::WorkPool<RAJA::WorkGroupPolicy<RAJA::b200_work<0>, RAJA::unordered>, Index_type>;
  std::vector<std::unique_ptr<RAJA::ReduceSum<red, double>>> ds;
  std::vector<double> expect(nloops, 0.0);
  pool_t pool;
  for (int l = 0; l < nloops; ++l) {
    ds.emplace_back(new RAJA::ReduceSum<red, double>(0.0));
    const RAJA::ReduceSum<red, double>& s = *ds.back();
    for (Index_type i = offs[l]; i < offs[l + 1]; ++i) expect[l] += w[i];
    pool.enqueue(RAJA::RangeSegment(offs[l], offs[l + 1]), [=] RAJA_DEVICE(Index_type i) { s += w[i]; });
  }
  auto g = pool.instantiate();
  const int runs = 12 * 3 + 4;
  bool wg_ok = true;
  for (int r = 0; r < runs; ++r) {
    g.run();
    for (int l = 0; l < nloops && wg_ok; ++l) wg_ok = ds[l]->get() == double(r + 1) * expect[l];
  }
  const RAJA::b200::tune::Report rep = g.tuning();
  printf("  WorkGroup tuner: %s, %d candidates, %d timed, tile %d x %d\n", rep.settled ? "settled" : "tuning",
         rep.candidates, rep.timed_calls, rep.best.block, rep.best.items);
  CHECK("autotuned_workgroup_reducers_every_run_exact", wg_ok);
  CHECK("autotuned_workgroup_settles", rep.settled && rep.candidates == 12);
  cudaFree(x);
  cudaFree(y);
  cudaFree(w);
}

// Stream capture of RAJA-API loops into a CUDA graph, then replays: a
// repeated sweep of forall loops and a WorkGroup run costs one graph launch.
void test_graph_capture() {
  namespace res = RAJA::resources;
  const Index_type n = (Index_type(1) << 20) + 5;
  double* x = managed<double>(n);
  double* y = managed<double>(n);
  int* a = managed<int>(n);
  for (Index_type i = 0; i < n; ++i) {
    x[i] = double(i % 7);
    y[i] = 0.0;
    a[i] = 0;
  }
  cudaStream_t cs = nullptr;
  cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  res::Cuda r = res::Cuda::CudaFromStream(cs);
  using aexec = RAJA::b200_exec_async<256>;
  // first calls outside the capture: per-kernel launch setup, WorkGroup upload
  RAJA::forall<aexec>(r, RAJA::RangeSegment(0, n), [=] __device__(Index_type i) { y[i] += x[i]; });
  using wpol = RAJA::WorkGroupPolicy<RAJA::b200_work<256, true>, RAJA::unordered>;
  RAJA::WorkPool<wpol, Index_type> pool;
  pool.enqueue(RAJA::RangeSegment(0, n / 2), [=] __device__(Index_type i) { a[i] += 1; });
  pool.enqueue(RAJA::RangeSegment(n / 2, n), [=] __device__(Index_type i) { a[i] += 2; });
  auto group = pool.instantiate();
  group.run(r);
  cudaStreamSynchronize(cs);
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  bool ok = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  for (int k = 0; k < 4; ++k)
    RAJA::forall<aexec>(r, RAJA::RangeSegment(0, n), [=] __device__(Index_type i) { y[i] += x[i]; });
  group.run(r);
  ok = ok && cudaStreamEndCapture(cs, &g) == cudaSuccess;
  ok = ok && cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
  for (int rep = 0; ok && rep < 10; ++rep) ok = cudaGraphLaunch(ge, cs) == cudaSuccess;
  ok = ok && cudaStreamSynchronize(cs) == cudaSuccess;
  for (Index_type i = 0; i < n && ok; ++i) ok = y[i] == 41.0 * x[i] && a[i] == (i < n / 2 ? 11 : 22);
  CHECK("graph_capture_forall_and_workgroup_replayed", ok);
  if (ge) cudaGraphExecDestroy(ge);
  if (g) cudaGraphDestroy(g);
  cudaStreamDestroy(cs);
  cudaFree(x);
  cudaFree(y);
  cudaFree(a);
}

void test_multi_reduce_and_atomics() {
  const Index_type n = 200003;
  const int nb = 37;
  int* bins = nullptr;
  double* vals = nullptr;
  cudaMallocManaged(&bins, n * sizeof(int));
  cudaMallocManaged(&vals, n * sizeof(double));
  std::mt19937 rng(17);
  for (Index_type i = 0; i < n; ++i) {
    bins[i] = int(rng() % nb);
    vals[i] = double(int(rng() % 2001) - 1000) / 8.0;  // exact sums
  }
  using exec = RAJA::b200_exec<256>;
  RAJA::MultiReduceSum<RAJA::b200_multi_reduce, double> dsum(nb, 1.5);
  RAJA::MultiReduceMin<RAJA::b200_multi_reduce, double> dmin(nb);
  RAJA::MultiReduceMax<RAJA::b200_multi_reduce, double> dmax(nb);
  RAJA::MultiReduceBitOr<RAJA::b200_multi_reduce, long long> dor(nb);
  RAJA::MultiReduceBitAnd<RAJA::b200_multi_reduce, unsigned> dand(nb);
  RAJA::forall<exec>(RAJA::RangeSegment(0, n), [=] RAJA_DEVICE(Index_type i) {
    const int b = bins[i];
    dsum[b] += vals[i];
    dmin[b].min(vals[i]);
    dmax[b].max(vals[i]);
    dor[b] |= (long long)(i & 0xff) << (b % 8);
    dand[b] &= ~(1u << (i % 13));
  });
  RAJA::MultiReduceSum<RAJA::seq_multi_reduce, double> hsum(nb, 1.5);
  RAJA::MultiReduceMin<RAJA::seq_multi_reduce, double> hmin(nb);
  RAJA::MultiReduceMax<RAJA::seq_multi_reduce, double> hmax(nb);
  RAJA::MultiReduceBitOr<RAJA::seq_multi_reduce, long long> hor(nb);
  RAJA::MultiReduceBitAnd<RAJA::seq_multi_reduce, unsigned> hand(nb);
  RAJA::forall<RAJA::seq_exec>(RAJA::RangeSegment(0, n), [=](Index_type i) {
    const int b = bins[i];
    hsum[b] += vals[i];
    hmin[b].min(vals[i]);
    hmax[b].max(vals[i]);
    hor[b] |= (long long)(i & 0xff) << (b % 8);
    hand[b] &= ~(1u << (i % 13));
  });
  bool ok = true;
  for (int b = 0; b < nb; ++b)
    ok = ok && dsum.get(b) == hsum.get(b) && dmin.get(b) == hmin.get(b) &&
         dmax[b].get() == hmax[b].get() && dor.get(b) == hor.get(b) && dand.get(b) == hand.get(b);
  CHECK("multi_reduce_b200_vs_seq", ok);

  // device atomics: a counter, a bounded wrap-around counter, a max by
  // compare-and-swap (doubles), and an AtomicRef
  unsigned long long* cnt = nullptr;
  unsigned* wrap = nullptr;
  double* dmx = nullptr;
  int* ref = nullptr;
  cudaMallocManaged(&cnt, sizeof(*cnt));
  cudaMallocManaged(&wrap, sizeof(*wrap));
  cudaMallocManaged(&dmx, sizeof(*dmx));
  cudaMallocManaged(&ref, sizeof(*ref));
  *cnt = 0;
  *wrap = 0;
  *dmx = -1e300;
  *ref = 0;
  RAJA::forall<exec>(RAJA::RangeSegment(0, n), [=] RAJA_DEVICE(Index_type i) {
    RAJA::atomicAdd<RAJA::b200_atomic>(cnt, 1ull);
    RAJA::atomicInc<RAJA::b200_atomic>(wrap, 999u);
    RAJA::atomicMax<RAJA::b200_atomic>(dmx, vals[i]);
    RAJA::AtomicRef<int, RAJA::b200_atomic> r(ref);
    r += int(i % 3);
  });
  RAJA::b200::wait();
  double hmx = -1e300;
  long long hr = 0;
  for (Index_type i = 0; i < n; ++i) {
    hmx = hmx < vals[i] ? vals[i] : hmx;
    hr += i % 3;
  }
  CHECK("atomics_b200", *cnt == (unsigned long long)n && *wrap == unsigned(n % 1000) &&
                            *dmx == hmx && *ref == int(hr));
  cudaFree(cnt);
  cudaFree(wrap);
  cudaFree(dmx);
  cudaFree(ref);
  cudaFree(bins);
  cudaFree(vals);
}

// Resources and events (test/unit/resource/tests/*.hpp): stream-ordered
// copies, cross-stream dependencies through events, joins, several
// streams writing one array, sync vs async policies, and scans, sorts,
// reducers and WorkGroup runs on a resource.
__device__ inline void spin_cycles(long long c) {
  const long long t0 = clock64();
  while (clock64() - t0 < c) {
  }
}

template <class Pol>
void resource_semantics(const char* tag) {
  namespace res = RAJA::resources;
  char nm[96];
  res::Host host;
  {  // BasicAsyncSemantics
    const int n = 10000000;
    res::Cuda dev;
    int* d = res::Resource{dev}.allocate<int>(n);
    int* h = host.allocate<int>(n);
    RAJA::forall<RAJA::seq_exec>(host, RAJA::RangeSegment(0, n), [=](Index_type i) { h[i] = int(i); });
    dev.memcpy(d, h, sizeof(int) * n);
    RAJA::forall<Pol>(dev, RAJA::RangeSegment(0, n), [=] __device__(Index_type i) { d[i] = int(i) + 2; });
    dev.memcpy(h, d, sizeof(int) * n);
    dev.wait();
    bool ok = true;
    for (int i = 0; i < n; ++i) ok = ok && h[i] == i + 2;
    snprintf(nm, sizeof nm, "resource_basic_async_%s", tag);
    CHECK(nm, ok);
    dev.deallocate(d);
    host.deallocate(h);
  }
  {  // Depends
    const int n = 10000;
    res::Cuda dev1, dev2;
    int* d1 = res::Resource{dev1}.allocate<int>(n);
    int* d2 = res::Resource{dev2}.allocate<int>(n);
    int* h = host.allocate<int>(n);
    RAJA::forall<Pol>(dev1, RAJA::RangeSegment(0, n), [=] __device__(Index_type i) { d1[i] = int(i); });
    res::Event e = RAJA::forall<Pol>(dev2, RAJA::RangeSegment(0, n), [=] __device__(Index_type i) {
      spin_cycles(20000);
      d2[i] = -1;
    });
    dev1.wait_for(&e);
    RAJA::forall<Pol>(dev1, RAJA::RangeSegment(0, n), [=] __device__(Index_type i) { d1[i] *= d2[i]; });
    dev1.memcpy(h, d1, sizeof(int) * n);
    dev1.wait();
    bool ok = dev1 != dev2;
    for (int i = 0; i < n; ++i) ok = ok && h[i] == -i;
    snprintf(nm, sizeof nm, "resource_depends_%s", tag);
    CHECK(nm, ok);
    dev1.deallocate(d1);
    dev2.deallocate(d2);
    host.deallocate(h);
  }
  {  // JoinAsyncSemantics
    const int n = 1000000;
    res::Cuda dev1, dev2;
    int* d = res::Resource{dev1}.allocate<int>(n);
    int* h = host.allocate<int>(n);
    RAJA::forall<RAJA::seq_exec>(host, RAJA::RangeSegment(0, n), [=](Index_type i) { h[i] = int(i); });
    dev2.memcpy(d, h, sizeof(int) * n);
    auto e1 = dev2.get_event_erased();
    dev1.wait_for(&e1);
    res::Event e2 = RAJA::forall<Pol>(dev1, RAJA::RangeSegment(0, n), [=] __device__(Index_type i) { d[i] = int(i) + 2; });
    dev2.wait_for(&e2);
    dev2.memcpy(h, d, sizeof(int) * n);
    dev2.wait();
    bool ok = true;
    for (int i = 0; i < n; ++i) ok = ok && h[i] == i + 2;
    snprintf(nm, sizeof nm, "resource_join_%s", tag);
    CHECK(nm, ok);
    dev1.deallocate(d);
    host.deallocate(h);
  }
  {  // MultiStream
    const int n = 10000;
    res::Cuda dev1, dev2;
    int* d = res::Resource{dev1}.allocate<int>(n);
    int* h = host.allocate<int>(n);
    res::Event e1 = RAJA::forall<Pol>(dev1, RAJA::RangeSegment(0, n), [=] __device__(Index_type i) {
      if (i % 3 == 0) d[i] = int(i);
    });
    res::Event e2 = RAJA::forall<Pol>(dev2, RAJA::RangeSegment(0, n), [=] __device__(Index_type i) {
      if (i % 3 == 1) d[i] = int(i);
    });
    res::Event e3 = RAJA::forall<Pol>(dev2, RAJA::RangeSegment(0, n), [=] __device__(Index_type i) {
      if (i % 3 == 2) d[i] = int(i);
    });
    dev1.wait_for(&e2);
    dev1.wait_for(&e3);
    dev1.memcpy(h, d, sizeof(int) * n);
    dev1.wait();
    bool ok = e1.try_get<res::CudaEvent>() != nullptr;
    for (int i = 0; i < n; ++i) ok = ok && h[i] == i;
    snprintf(nm, sizeof nm, "resource_multistream_%s", tag);
    CHECK(nm, ok);
    dev1.deallocate(d);
    host.deallocate(h);
  }
}

// One spinning forall per resource, then a wait on each; seconds.
template <class Pol>
double timed_spins(RAJA::resources::Cuda* dev, int ns, long long cycles) {
  const auto t0 = std::chrono::steady_clock::now();
  for (int s = 0; s < ns; ++s)
    RAJA::forall<Pol>(dev[s], RAJA::RangeSegment(0, 10000), [=] __device__(Index_type) { spin_cycles(cycles); });
  for (int s = 0; s < ns; ++s) dev[s].wait();
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void test_resources() {
  namespace res = RAJA::resources;
  using async = RAJA::b200_exec_async<256>;
  static_assert(std::is_same<res::get_resource<exec>::type, res::Cuda>::value, "b200 resource");
  resource_semantics<async>("async");
  resource_semantics<exec>("sync");

  // a synchronous policy has finished when forall returns
  {
    const int n = 1 << 20;
    res::Cuda dev;
    int* m = dev.allocate<int>(n, res::MemoryAccess::Managed);
    RAJA::forall<exec>(dev, RAJA::RangeSegment(0, n), [=] __device__(Index_type i) {
      spin_cycles(2000);
      m[i] = 7 * int(i);
    });
    bool ok = true;
    for (int i = 0; i < n; ++i) ok = ok && m[i] == 7 * i;
    CHECK("resource_sync_policy_done_on_return", ok);
    dev.deallocate(m);
  }
  // AsyncTime: eight resources, one ~2 ms kernel each.  Asynchronous
  // launches overlap; synchronous ones run one after another.
  {
    constexpr int NS = 8;
    res::Cuda dev[NS];
    int clk_khz = 0;
    cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, 0);
    const long long cycles = (long long)(clk_khz > 0 ? clk_khz : 2000000) * 2;  // about 2 ms
    timed_spins<async>(dev, NS, cycles);  // warm-up
    const double t_sync = timed_spins<exec>(dev, NS, cycles);
    const double t_async = timed_spins<async>(dev, NS, cycles);
    printf("async_time: sync %.2f ms, async %.2f ms\n", t_sync * 1e3, t_async * 1e3);
    CHECK("resource_async_time", t_async < 0.5 * t_sync);
  }
  // scans, sorts and reducers on a resource; EventProxy to CudaEvent
  {
    const int n = 32000;
    res::Cuda dev;
    int* in = dev.allocate<int>(n, res::MemoryAccess::Managed);
    int* out = dev.allocate<int>(n, res::MemoryAccess::Managed);
    for (int i = 0; i < n; ++i) in[i] = (i * 7919) % 1000 - 500;
    res::CudaEvent ce = RAJA::exclusive_scan<async>(dev, RAJA::make_span((const int*)in, n), RAJA::make_span(out, n),
                                                    RAJA::operators::plus<int>{}, 5);
    ce.wait();
    bool ok = true;
    long acc = 5;
    for (int i = 0; i < n; ++i) {
      ok = ok && out[i] == int(acc);
      acc += in[i];
    }
    CHECK("resource_exclusive_scan_event", ok);
    int* vals = dev.allocate<int>(n, res::MemoryAccess::Managed);
    for (int i = 0; i < n; ++i) vals[i] = i;
    res::Event se = RAJA::stable_sort_pairs<async>(res::Resource{dev}, RAJA::make_span(in, n), RAJA::make_span(vals, n));
    se.wait();
    ok = true;
    for (int i = 1; i < n; ++i) ok = ok && (in[i - 1] < in[i] || (in[i - 1] == in[i] && vals[i - 1] < vals[i]));
    CHECK("resource_stable_sort_pairs", ok);
    RAJA::ReduceSum<red, long long> s(0);
    RAJA::ReduceMin<red, int> mn(1 << 30);
    RAJA::forall<exec>(dev, RAJA::RangeSegment(0, n), [=] __device__(Index_type i) {
      s += vals[i];
      mn.min(in[i]);
    });
    CHECK("resource_reducers", s.get() == (long long)n * (n - 1) / 2 && mn.get() == in[0]);
    dev.deallocate(in);
    dev.deallocate(out);
    dev.deallocate(vals);
  }
  // WorkGroup::run(resource)
  {
    const int n = 4096;
    res::Cuda dev;
    int* a = dev.allocate<int>(n, res::MemoryAccess::Managed);
    for (int i = 0; i < n; ++i) a[i] = 0;
    using wpol = RAJA::WorkGroupPolicy<RAJA::b200_work<256, true>, RAJA::unordered>;
    RAJA::WorkPool<wpol, Index_type> pool;
    pool.enqueue(RAJA::RangeSegment(0, n / 2), [=] __device__(Index_type i) { a[i] += int(i) + 5; });
    pool.enqueue(RAJA::RangeSegment(n / 2, n), [=] __device__(Index_type i) { a[i] -= int(i); });
    auto group = pool.instantiate();
    auto site = group.run(dev);
    site.get_resource().wait();
    bool ok = site.get_resource() == dev;
    for (int i = 0; i < n; ++i) ok = ok && a[i] == (i < n / 2 ? i + 5 : -i);
    CHECK("resource_workgroup_run", ok);
    dev.deallocate(a);
  }
  // WorkGroup reducers across runs on two streams, read after the group and
  // one of the resources are gone: get() waits for both streams' runs
  {
    const int n = 3000;
    int* a = nullptr;
    cudaMallocManaged(&a, n * sizeof(int));
    for (int i = 0; i < n; ++i) a[i] = i % 11;
    long long expect = 0;
    for (int i = 0; i < n; ++i) expect += a[i];
    RAJA::ReduceSum<red, long long> s(3);
    RAJA::ReduceMax<red, int> mx(-1);
    {
      using wpol = RAJA::WorkGroupPolicy<RAJA::b200_work<256, true>, RAJA::unordered>;
      RAJA::WorkPool<wpol, Index_type> pool;
      pool.enqueue(RAJA::RangeSegment(0, n / 3), [=] __device__(Index_type i) { s += a[i]; });
      pool.enqueue(RAJA::RangeSegment(n / 3, n), [=] __device__(Index_type i) {
        s += a[i];
        mx.max(a[i]);
      });
      auto group = pool.instantiate();
      res::Cuda keep;
      {
        res::Cuda gone;
        group.run(keep);
        group.run(gone);
        group.run(keep);
      }
    }
    CHECK("workgroup_reducers_two_streams_after_group_destroyed", s.get() == 3 + 3 * expect && mx.get() == 10);
    cudaFree(a);
  }
}

// RAJA::launch on the b200 policies (test/functional/launch): nested
// direct / loop policies over a 6-D View, tile_tcount + loop_icount,
// dynamic (including > 48 KB) and static team shared memory, reducer
// params against the host launch, run-time place switch, resources,
// flattened thread policies and the three segment kinds.
using dlaunch = RAJA::LaunchPolicy<RAJA::b200_launch_t<false>>;
using hdlaunch = RAJA::LaunchPolicy<RAJA::seq_launch_t, RAJA::b200_launch_t<false>>;
template <class P>
using lp = RAJA::LoopPolicy<RAJA::seq_exec, P>;

template <class TX, class TY, class TZ, class BX, class BY, class BZ>
void launch_nested_case(const char* tag, int M) {
  const RAJA::RangeSegment r1(0, 2 * M), r2(0, 3 * M), r3(0, 4 * M), r4(0, 4 * M), r5(0, 5 * M), r6(0, 6 * M);
  const Index_type N1 = 2 * M, N2 = 3 * M, N3 = 4 * M, N4 = 4 * M, N5 = 5 * M, N6 = 6 * M;
  const Index_type N = N1 * N2 * N3 * N4 * N5 * N6;
  Index_type* a = managed<Index_type>(N);
  for (Index_type i = 0; i < N; ++i) a[i] = 0;
  RAJA::View<Index_type, RAJA::Layout<6>> Av(a, N6, N5, N4, N3, N2, N1);
  RAJA::launch<dlaunch>(RAJA::LaunchParams(RAJA::Teams(4, 5, 6), RAJA::Threads(2, 3, 4)),
                        [=] RAJA_HOST_DEVICE(RAJA::LaunchContext ctx) {
    RAJA::loop<BZ>(ctx, r6, [&](Index_type bz) {
      RAJA::loop<BY>(ctx, r5, [&](Index_type by) {
        RAJA::loop<BX>(ctx, r4, [&](Index_type bx) {
          RAJA::loop<TZ>(ctx, r3, [&](Index_type tz) {
            RAJA::loop<TY>(ctx, r2, [&](Index_type ty) {
              RAJA::loop<TX>(ctx, r1, [&](Index_type tx) {
                const Index_type idx = tx + N1 * (ty + N2 * (tz + N3 * (bx + N4 * (by + N5 * bz))));
                Av(bz, by, bx, tz, ty, tx) += idx;
              });
            });
          });
        });
      });
    });
  });
  bool ok = true;
  for (Index_type i = 0; i < N; ++i) ok = ok && a[i] == i;
  char nm[96];
  snprintf(nm, sizeof nm, "launch_nested_%s", tag);
  CHECK(nm, ok);
  cudaFree(a);
}

template <class TEAM, class THREAD>
void launch_tile_case(const char* tag, int M, int teams, int threads) {
  constexpr int ts = 4;
  const int NT = M * ts + 1;
  int* tt = managed<int>(NT);
  int* ii = managed<int>(NT);
  for (int i = 0; i < NT; ++i) tt[i] = ii[i] = -1;
  const RAJA::RangeSegment r(0, NT);
  RAJA::launch<dlaunch>(RAJA::LaunchParams(RAJA::Teams(teams), RAJA::Threads(threads)),
                        [=] RAJA_HOST_DEVICE(RAJA::LaunchContext ctx) {
    RAJA::tile_tcount<TEAM>(ctx, ts, r, [&](const RAJA::RangeSegment& tile, Index_type bx) {
      RAJA::loop_icount<THREAD>(ctx, tile, [&](Index_type tx, Index_type ix) {
        tt[tx] = int(bx);
        ii[tx] = int(ix);
      });
    });
  });
  bool ok = true;
  for (int i = 0; i < NT; ++i) ok = ok && tt[i] == i / ts && ii[i] == i % ts;
  char nm[96];
  snprintf(nm, sizeof nm, "launch_tile_tcount_icount_%s", tag);
  CHECK(nm, ok);
  cudaFree(tt);
  cudaFree(ii);
}

void launch_shared_case(const char* tag, int teams, int th, int per_thread) {
  // each team stages `len` longs and ints in dynamic shared memory, then
  // reads them back reversed after a team barrier
  const int len = th * per_thread;
  long* out = managed<long>(size_t(teams) * len);
  const size_t shm = size_t(len) * (sizeof(long) + sizeof(int));
  RAJA::launch<dlaunch>(RAJA::LaunchParams(RAJA::Teams(teams), RAJA::Threads(th), shm),
                        [=] RAJA_HOST_DEVICE(RAJA::LaunchContext ctx) {
    RAJA::loop<lp<RAJA::b200_block_x_direct>>(ctx, RAJA::RangeSegment(0, teams), [&](Index_type b) {
      long* tile = ctx.getSharedMemory<long>(len);
      int* itile = ctx.getSharedMemory<int>(len);
      RAJA::loop<lp<RAJA::b200_thread_x_loop>>(ctx, RAJA::RangeSegment(0, len), [&](Index_type t) {
        itile[t] = int(t);
        tile[len - t - 1] = len - t - 1 + long(len) * b;
      });
      ctx.teamSync();
      RAJA::loop<lp<RAJA::b200_thread_x_loop>>(ctx, RAJA::RangeSegment(0, len), [&](Index_type t) {
        out[t + long(len) * b] = tile[t] + itile[t];
      });
      ctx.releaseSharedMemory();
    });
  });
  bool ok = true;
  for (int b = 0; b < teams; ++b)
    for (int t = 0; t < len; ++t) ok = ok && out[t + long(len) * b] == long(t) + long(len) * b + t;
  char nm[96];
  snprintf(nm, sizeof nm, "launch_dynamic_shared_%s", tag);
  CHECK(nm, ok);
  cudaFree(out);
}

void test_launch() {
  namespace res = RAJA::resources;
  static_assert(std::is_same<res::get_resource<RAJA::b200_launch_t<true>>::type, res::Cuda>::value, "launch res");
  launch_nested_case<lp<RAJA::b200_thread_x_direct>, lp<RAJA::b200_thread_y_direct>, lp<RAJA::b200_thread_z_direct>,
                     lp<RAJA::b200_block_x_direct>, lp<RAJA::b200_block_y_direct>, lp<RAJA::b200_block_z_direct>>(
      "direct", 1);
  launch_nested_case<lp<RAJA::b200_thread_x_loop>, lp<RAJA::b200_thread_y_loop>, lp<RAJA::b200_thread_z_loop>,
                     lp<RAJA::b200_block_x_loop>, lp<RAJA::b200_block_y_loop>, lp<RAJA::b200_block_z_loop>>("loop", 2);
  launch_tile_case<lp<RAJA::b200_block_x_loop>, lp<RAJA::b200_thread_x_loop>>("loop", 5, 1, 3);
  launch_tile_case<lp<RAJA::b200_block_x_direct>, lp<RAJA::b200_thread_x_direct>>("direct", 5, 6, 4);
  launch_shared_case("5x32", 5, 32, 1);
  launch_shared_case("3x256_96KB", 3, 256, 32);  // 8192 longs + ints: 96 KB of dynamic shared memory

  // static team shared memory (test-launch-StaticMem.hpp)
  {
    constexpr int TH = 64;
    const int teams = 7;
    int* out = managed<int>(teams * TH);
    RAJA::launch<dlaunch>(RAJA::LaunchParams(RAJA::Teams(teams), RAJA::Threads(TH)),
                          [=] RAJA_HOST_DEVICE(RAJA::LaunchContext ctx) {
      RAJA::loop<lp<RAJA::b200_block_x_direct>>(ctx, RAJA::RangeSegment(0, teams), [&](Index_type b) {
        RAJA_TEAM_SHARED int tile[TH];
        RAJA::loop<lp<RAJA::b200_thread_x_direct>>(ctx, RAJA::RangeSegment(0, TH), [&](Index_type t) {
          tile[t] = int(t + TH * b);
        });
        ctx.teamSync();
        RAJA::loop<lp<RAJA::b200_thread_x_direct>>(ctx, RAJA::RangeSegment(0, TH), [&](Index_type t) {
          out[t + TH * b] = tile[TH - 1 - t];
        });
      });
    });
    bool ok = true;
    for (int b = 0; b < teams; ++b)
      for (int t = 0; t < TH; ++t) ok = ok && out[t + TH * b] == TH - 1 - t + TH * b;
    CHECK("launch_static_shared", ok);
    cudaFree(out);
  }

  // reducer params (test-launch-basic-param-expt-Reduce*.hpp): device
  // against host through the run-time place switch
  {
    const int n = 1000003;
    double* x = managed<double>(n);
    int* bits = managed<int>(n);
    std::mt19937 rng(11);
    for (int i = 0; i < n; ++i) {
      x[i] = double(int(rng() % 100));
      bits[i] = int(rng()) | 0x11;
    }
    x[777777] = -5.0;
    x[999999] = -5.0;
    const int threads = 256, blocks = (n - 1) / threads + 1;
    using VS = RAJA::expt::ValOp<double, RAJA::operators::plus>;
    using VM = RAJA::expt::ValOp<double, RAJA::operators::minimum>;
    using VX = RAJA::expt::ValOp<double, RAJA::operators::maximum>;
    using VA = RAJA::expt::ValOp<int, RAJA::operators::bit_and>;
    using VL = RAJA::expt::ValOp<RAJA::expt::ValLoc<double, Index_type>, RAJA::operators::minimum>;
    struct R {
      double sum, sum2, mn, mx;
      int band;
      double lv;
      Index_type li;
    } got[2];
    const RAJA::ExecPlace places[2] = {RAJA::ExecPlace::DEVICE, RAJA::ExecPlace::HOST};
    for (int k = 0; k < 2; ++k) {
      R& r = got[k];
      r = R{0.0, 2.0, 1e300, -1e300, -1, 1e300, -1};
      RAJA::launch<hdlaunch>(
          places[k], RAJA::LaunchParams(RAJA::Teams(blocks), RAJA::Threads(threads)),
          RAJA::expt::Reduce<RAJA::operators::plus>(&r.sum), RAJA::expt::Reduce<RAJA::operators::plus>(&r.sum2),
          RAJA::Name("LaunchReduceParams"), RAJA::expt::Reduce<RAJA::operators::minimum>(&r.mn),
          RAJA::expt::Reduce<RAJA::operators::maximum>(&r.mx), RAJA::expt::Reduce<RAJA::operators::bit_and>(&r.band),
          RAJA::expt::ReduceLoc<RAJA::operators::minimum>(&r.lv, &r.li),
          [=] RAJA_HOST_DEVICE(RAJA::LaunchContext ctx, VS & s, VS & s2, VM & m, VX & M, VA & a, VL & l) {
            RAJA::loop<lp<RAJA::b200_global_thread_x>>(ctx, RAJA::RangeSegment(0, n), [&](Index_type i) {
              s += x[i];
              s2 += x[i];
              m.min(x[i]);
              M.max(x[i]);
              a &= bits[i];
              l.minloc(x[i], i);
            });
          });
    }
    const R& d = got[0];
    const R& h = got[1];
    CHECK("launch_reduce_params_vs_host", d.sum == h.sum && d.sum2 == h.sum + 2.0 && d.mn == h.mn && d.mx == h.mx &&
                                              d.band == h.band && d.lv == -5.0 && d.li == 777777 && h.li == 777777);
    // two launches accumulate into one target; fewer teams than needed with a loop policy
    double s = 0.0;
    for (int j = 0; j < 2; ++j)
      RAJA::launch<dlaunch>(RAJA::LaunchParams(RAJA::Teams(37), RAJA::Threads(128)),
                            RAJA::expt::Reduce<RAJA::operators::plus>(&s),
                            [=] RAJA_HOST_DEVICE(RAJA::LaunchContext ctx, VS & v) {
                              RAJA::loop<lp<RAJA::b200_global_x_loop>>(ctx, RAJA::RangeSegment(0, n),
                                                                       [&](Index_type i) { v += x[i]; });
                            });
    CHECK("launch_reduce_two_loops", s == 2.0 * h.sum);
    // a captured ReduceSum<b200_reduce> and a MultiReduce in a 2-D launch
    RAJA::ReduceSum<red, double> rs(0.0);
    RAJA::MultiReduceSum<RAJA::b200_multi_reduce, int> hist(4);
    RAJA::launch<dlaunch>(RAJA::LaunchParams(RAJA::Teams(19), RAJA::Threads(16, 8)),
                          [=] RAJA_HOST_DEVICE(RAJA::LaunchContext ctx) {
      RAJA::tile<lp<RAJA::b200_block_x_loop>>(ctx, 4096, RAJA::RangeSegment(0, n), [&](const RAJA::RangeSegment& t) {
        RAJA::loop<lp<RAJA::b200_flatten_block_threads_xy_loop>>(ctx, t, [&](Index_type i) {
          rs += x[i];
          hist[int(i & 3)] += 1;
        });
      });
    });
    int hb[4];
    for (int b = 0; b < 4; ++b) hb[b] = hist.get(b);
    const double rsv = rs.get();
    printf("captured 2d: rs %.1f (host %.1f) hist %d %d %d %d\n", rsv, h.sum, hb[0], hb[1], hb[2], hb[3]);
    CHECK("launch_captured_reducesum_2d_flatten", rsv == h.sum);
    CHECK("launch_captured_multireduce_2d_flatten", hb[0] + hb[1] + hb[2] + hb[3] == n && hb[3] == n / 4);
    // the same captured reducer with 1-D teams of threads
    RAJA::ReduceSum<red, double> rs1(0.0);
    RAJA::launch<dlaunch>(RAJA::LaunchParams(RAJA::Teams(23), RAJA::Threads(128)),
                          [=] RAJA_HOST_DEVICE(RAJA::LaunchContext ctx) {
      RAJA::loop<lp<RAJA::b200_global_x_loop>>(ctx, RAJA::RangeSegment(0, n), [&](Index_type i) { rs1 += x[i]; });
    });
    const double rs1v = rs1.get();
    printf("captured 1d: rs %.1f (host %.1f)\n", rs1v, h.sum);
    CHECK("launch_captured_reducesum_1d", rs1v == h.sum);
    // forall with a __host__ __device__ body: its closure copies the
    // captured reducer more than once on the host, still one result per launch
    RAJA::ReduceSum<red, double> rs2(1.0);
    RAJA::ReduceMinLoc<red, double, Index_type> ml2(1e300, -1);
    for (int j = 0; j < 2; ++j)
      RAJA::forall<exec>(RAJA::RangeSegment(0, n), [=] RAJA_HOST_DEVICE(Index_type i) {
        rs2 += x[i];
        ml2.minloc(x[i], i);
      });
    CHECK("forall_hd_lambda_reducers", rs2.get() == 1.0 + 2.0 * h.sum && ml2.get() == -5.0 && ml2.getLoc() == 777777);
    cudaFree(x);
    cudaFree(bits);
  }

  // resources: launch on a Resource returns an event; strided and list segments
  {
    const int n = 4099;
    res::Cuda dev;
    int* a = dev.allocate<int>(n, res::MemoryAccess::Managed);
    Index_type* lst = dev.allocate<Index_type>(3, res::MemoryAccess::Managed);
    lst[0] = 4098;  // even indices: the strided loop writes the odd ones
    lst[1] = 8;
    lst[2] = 0;
    for (int i = 0; i < n; ++i) a[i] = 0;
    res::Event e = RAJA::launch<RAJA::LaunchPolicy<RAJA::seq_launch_t, RAJA::b200_launch_t<true, 256>>>(
        res::Resource{dev}, RAJA::LaunchParams(RAJA::Teams(8), RAJA::Threads(256)),
        [=] RAJA_HOST_DEVICE(RAJA::LaunchContext ctx) {
          RAJA::loop<lp<RAJA::b200_global_x_loop>>(ctx, RAJA::RangeStrideSegment(1, n, 2),
                                                   [&](Index_type i) { a[i] = int(i); });
          RAJA::loop<lp<RAJA::b200_global_x_direct>>(ctx, RAJA::ListSegment(lst, 3),
                                                     [&](Index_type i) { a[i] = -1; });
        });
    e.wait();
    bool ok = e.try_get<res::CudaEvent>() != nullptr;
    for (int i = 0; i < n; ++i) ok = ok && a[i] == ((i == 4098 || i == 8 || i == 0) ? -1 : (i & 1 ? i : 0));
    CHECK("launch_resource_stride_list_segments", ok);
    dev.deallocate(a);
    dev.deallocate(lst);
  }
}

// 7-point Jacobi through RAJA::launch over Views with an OffsetLayout
// (interior [0, N), halo at -1 and N), max residual by an expt::Reduce
// param: the device launch against the same body run by the host launch,
// bit-exact, over several sweeps.  The operation order follows the oracle's
// sweep: ((x pair) + (y pair)) + (z pair), then * (1/6); the product and
// the residual's difference are rounded separately on both sides.
RAJA_HOST_DEVICE inline double mul_rn(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
RAJA_HOST_DEVICE inline double sub_rn(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}

double jacobi_launch(RAJA::ExecPlace place, int Nx, int Ny, int Nz, double* u, double* unew) {
  using pol = RAJA::LaunchPolicy<RAJA::seq_launch_t, RAJA::b200_launch_t<false>>;
  using kpol = RAJA::LoopPolicy<RAJA::seq_exec, RAJA::b200_block_x_direct>;
  using jtile = RAJA::LoopPolicy<RAJA::seq_exec, RAJA::b200_block_y_direct>;
  using jpol = RAJA::LoopPolicy<RAJA::seq_exec, RAJA::b200_thread_y_direct>;
  using ipol = RAJA::LoopPolicy<RAJA::seq_exec, RAJA::b200_thread_x_loop>;
  const auto lay = RAJA::make_offset_layout<3>({{-1, -1, -1}}, {{Nz + 1, Ny + 1, Nx + 1}});
  RAJA::View<double, RAJA::OffsetLayout<3>> U(u, lay), Un(unew, lay);
  constexpr int JT = 4;
  double rmax = 0.0;
  RAJA::launch<pol>(place, RAJA::LaunchParams(RAJA::Teams(Nz, (Ny + JT - 1) / JT), RAJA::Threads(32, JT)),
                    RAJA::expt::Reduce<RAJA::operators::maximum>(&rmax),
                    [=] RAJA_HOST_DEVICE(RAJA::LaunchContext ctx,
                                         RAJA::expt::ValOp<double, RAJA::operators::maximum>& r) {
    RAJA::loop<kpol>(ctx, RAJA::RangeSegment(0, Nz), [&](Index_type k) {
      RAJA::tile<jtile>(ctx, JT, RAJA::RangeSegment(0, Ny), [&](const RAJA::RangeSegment& jt) {
        RAJA::loop<jpol>(ctx, jt, [&](Index_type j) {
          RAJA::loop<ipol>(ctx, RAJA::RangeSegment(0, Nx), [&](Index_type i) {
            double acc = U(k, j, i - 1) + U(k, j, i + 1);
            acc += U(k, j - 1, i) + U(k, j + 1, i);
            acc += U(k - 1, j, i) + U(k + 1, j, i);
            const double v = mul_rn(acc, 1.0 / 6.0);
            Un(k, j, i) = v;
            r.max(fabs(sub_rn(v, U(k, j, i))));
          });
        });
      });
    });
  });
  return rmax;
}

void test_launch_jacobi() {
  const int dims[2][3] = {{64, 64, 64}, {130, 37, 21}};
  for (const auto& d : dims) {
    const int Nx = d[0], Ny = d[1], Nz = d[2];
    const size_t tot = size_t(Nx + 2) * (Ny + 2) * (Nz + 2);
    double* ud = managed<double>(tot);
    double* vd = managed<double>(tot);
    std::vector<double> uh(tot), vh(tot);
    std::mt19937_64 rng(5);
    std::uniform_real_distribution<double> dist(-1.0, 1.0);
    for (size_t q = 0; q < tot; ++q) ud[q] = vd[q] = uh[q] = vh[q] = dist(rng);
    double rd = 0.0, rh = 0.0;
    for (int sweep = 0; sweep < 6; ++sweep) {
      double* a = (sweep & 1) ? vd : ud;
      double* b = (sweep & 1) ? ud : vd;
      double* ah = (sweep & 1) ? vh.data() : uh.data();
      double* bh = (sweep & 1) ? uh.data() : vh.data();
      rd = jacobi_launch(RAJA::ExecPlace::DEVICE, Nx, Ny, Nz, a, b);
      rh = jacobi_launch(RAJA::ExecPlace::HOST, Nx, Ny, Nz, ah, bh);
    }
    bool ok = rd == rh && rd > 0.0;
    for (size_t q = 0; q < tot; ++q) ok = ok && ud[q] == uh[q] && vd[q] == vh[q];
    char nm[96];
    snprintf(nm, sizeof nm, "launch_jacobi_offset_view_%dx%dx%d", Nx, Ny, Nz);
    printf("%s: residual device %.17g host %.17g\n", nm, rd, rh);
    CHECK(nm, ok);
    cudaFree(ud);
    cudaFree(vd);
  }
}

// expt::Reduce params over strided and list segments, device vs seq
void test_params_segments() {
  const int n = 200003;
  double* x = managed<double>(n);
  for (int i = 0; i < n; ++i) x[i] = double((i * 7919) % 1000) - 500.0;
  x[123457] = -777.0;
  Index_type* lst = managed<Index_type>(5000);
  for (int i = 0; i < 5000; ++i) lst[i] = Index_type((i * 40009) % n);
  using VS = RAJA::expt::ValOp<double, RAJA::operators::plus>;
  using VL = RAJA::expt::ValOp<RAJA::expt::ValLoc<double, Index_type>, RAJA::operators::minimum>;
  double res[2][4];
  Index_type loc[2][2];
  for (int dev = 0; dev < 2; ++dev) {
    double s1 = 0.0, v1 = 1e300, s2 = 0.0, v2 = 1e300;
    Index_type i1 = -1, i2 = -1;
    auto body = [=] RAJA_HOST_DEVICE(Index_type i, VS& s, VL& m) {
      s += x[i];
      m.minloc(x[i], i);
    };
    if (dev) {
      RAJA::forall<exec>(RAJA::RangeStrideSegment(1, n, 2), RAJA::expt::Reduce<RAJA::operators::plus>(&s1),
                         RAJA::expt::ReduceLoc<RAJA::operators::minimum>(&v1, &i1), body);
      RAJA::forall<exec>(RAJA::ListSegment(lst, 5000), RAJA::expt::Reduce<RAJA::operators::plus>(&s2),
                         RAJA::expt::ReduceLoc<RAJA::operators::minimum>(&v2, &i2), body);
    } else {
      RAJA::forall<RAJA::seq_exec>(RAJA::RangeStrideSegment(1, n, 2), RAJA::expt::Reduce<RAJA::operators::plus>(&s1),
                                   RAJA::expt::ReduceLoc<RAJA::operators::minimum>(&v1, &i1), body);
      RAJA::forall<RAJA::seq_exec>(RAJA::ListSegment(lst, 5000), RAJA::expt::Reduce<RAJA::operators::plus>(&s2),
                                   RAJA::expt::ReduceLoc<RAJA::operators::minimum>(&v2, &i2), body);
    }
    res[dev][0] = s1; res[dev][1] = v1; res[dev][2] = s2; res[dev][3] = v2;
    loc[dev][0] = i1; loc[dev][1] = i2;
  }
  // integer-valued doubles: the sums are exact in any order; MinLoc keeps
  // the lowest index of the stride segment, the first list position's
  // index on the device only up to ties, so values are compared there
  // a kernel name reaches the b200 launch (NVTX range under RAJA_ENABLE_NVTX)
  RAJA::b200::last_kernel_name() = nullptr;
  double sn = 0.0;
  RAJA::forall<exec>(RAJA::RangeSegment(0, 1000), RAJA::Name("b200_named_loop"),
                     RAJA::expt::Reduce<RAJA::operators::plus>(&sn),
                     [=] RAJA_HOST_DEVICE(Index_type i, VS& s) { s += double(i); });
  const char* seen = RAJA::b200::last_kernel_name();
  RAJA::launch<dlaunch>(RAJA::LaunchParams(RAJA::Teams(1), RAJA::Threads(32)), RAJA::Name("b200_named_launch"),
                        [=] RAJA_HOST_DEVICE(RAJA::LaunchContext) {});
  const char* seen2 = RAJA::b200::last_kernel_name();
  CHECK("kernel_name_reaches_b200", sn == 499500.0 && seen && std::string(seen) == "b200_named_loop" && seen2 &&
                                        std::string(seen2) == "b200_named_launch");
  CHECK("expt_reduce_stride_list_b200",
        res[1][0] == res[0][0] && res[1][1] == res[0][1] && loc[1][0] == loc[0][0] && loc[0][0] == 123457 &&
        res[1][2] == res[0][2] && res[1][3] == res[0][3]);
  cudaFree(x);
  cudaFree(lst);
}

// Empty and tiny inputs through the RAJA API on the b200 policies: empty
// segments leave reducers at their init values and params targets
// unchanged; launches with zero teams do nothing; scans and sorts of
// length 0, 1 and 2; an empty WorkGroup; waiting on an unused resource.
void test_edge_cases() {
  bool ok = true;
  int* a = managed<int>(4);
  a[0] = 5; a[1] = -3; a[2] = 7; a[3] = 1;
  {
    RAJA::ReduceSum<red, int> s(11);
    RAJA::ReduceMinLoc<red, int, Index_type> m(100, -1);
    RAJA::forall<exec>(RAJA::RangeSegment(4, 4), [=] RAJA_HOST_DEVICE(Index_type i) {
      s += a[i];
      m.minloc(a[i], i);
    });
    RAJA::forall<exec>(RAJA::RangeStrideSegment(0, 0, 2), [=] RAJA_HOST_DEVICE(Index_type i) { s += a[i]; });
    RAJA::forall<exec>(RAJA::ListSegment(nullptr, 0), [=] RAJA_HOST_DEVICE(Index_type i) { s += a[i]; });
    ok = ok && s.get() == 11 && m.get() == 100 && m.getLoc() == -1;
    double t = 2.5;
    RAJA::forall<exec>(RAJA::RangeSegment(0, 0), RAJA::expt::Reduce<RAJA::operators::plus>(&t),
                       [=] RAJA_HOST_DEVICE(Index_type i, RAJA::expt::ValOp<double, RAJA::operators::plus>& v) {
                         v += double(a[i]);
                       });
    ok = ok && t == 2.5;
  }
  CHECK("edge_empty_segments_b200", ok);
  ok = true;
  {
    double t = 1.0;
    RAJA::launch<dlaunch>(RAJA::LaunchParams(RAJA::Teams(0), RAJA::Threads(32)),
                          RAJA::expt::Reduce<RAJA::operators::plus>(&t),
                          [=] RAJA_HOST_DEVICE(RAJA::LaunchContext ctx,
                                               RAJA::expt::ValOp<double, RAJA::operators::plus>& v) {
                            RAJA::loop<lp<RAJA::b200_global_thread_x>>(ctx, RAJA::RangeSegment(0, 4),
                                                                       [&](Index_type i) { v += 1.0; });
                          });
    RAJA::launch<dlaunch>(RAJA::LaunchParams(RAJA::Teams(4), RAJA::Threads(0)),
                          [=] RAJA_HOST_DEVICE(RAJA::LaunchContext) { a[0] = 99; });
    ok = ok && t == 1.0 && a[0] == 5;
    bool threw = false;
    try {
      RAJA::launch<dlaunch>(RAJA::LaunchParams(RAJA::Teams(1), RAJA::Threads(64, 32)),
                            [=] RAJA_HOST_DEVICE(RAJA::LaunchContext) {});
    } catch (const std::runtime_error&) {
      threw = true;  // 2048 threads per team
    }
    ok = ok && threw;
  }
  CHECK("edge_launch_empty_and_oversized", ok);
  ok = true;
  {
    int* o = managed<int>(4);
    o[0] = o[1] = o[2] = o[3] = -9;
    RAJA::inclusive_scan<exec>(RAJA::make_span((const int*)a, 0), RAJA::make_span(o, 0));
    ok = ok && o[0] == -9;
    RAJA::exclusive_scan<exec>(RAJA::make_span((const int*)a, 1), RAJA::make_span(o, 1),
                               RAJA::operators::plus<int>{}, 4);
    ok = ok && o[0] == 4 && o[1] == -9;
    RAJA::inclusive_scan<exec>(RAJA::make_span((const int*)a, 2), RAJA::make_span(o, 2),
                               RAJA::operators::minimum<int>{});
    ok = ok && o[0] == 5 && o[1] == -3;
    RAJA::stable_sort<exec>(RAJA::make_span(a, 0));
    RAJA::stable_sort<exec>(RAJA::make_span(a, 1));
    ok = ok && a[0] == 5;
    int* v = managed<int>(2);
    v[0] = 10; v[1] = 20;
    RAJA::stable_sort_pairs<exec>(RAJA::make_span(a, 2), RAJA::make_span(v, 2));
    ok = ok && a[0] == -3 && a[1] == 5 && v[0] == 20 && v[1] == 10;
    cudaFree(o);
    cudaFree(v);
  }
  CHECK("edge_scan_sort_lengths_0_1_2", ok);
  {
    // forall_Icount on b200 over an IndexSet and a list segment, with a
    // captured reducer
    RAJA::TypedIndexSet<RAJA::RangeSegment> is;
    is.push_back(RAJA::RangeSegment(0, 5000));
    is.push_back(RAJA::RangeSegment(7000, 7003));
    is.push_back(RAJA::RangeSegment(9000, 12000));
    Index_type* w = managed<Index_type>(8003);
    for (int i = 0; i < 8003; ++i) w[i] = -1;
    RAJA::ReduceSum<red, long long> cnt(0);
    RAJA::forall_Icount<exec>(is, [=] RAJA_HOST_DEVICE(Index_type ic, Index_type idx) {
      w[ic] = idx;
      cnt += 1;
    });
    bool okc = cnt.get() == 8003;
    for (int i = 0; i < 8003; ++i)
      okc = okc && w[i] == (i < 5000 ? i : (i < 5003 ? 7000 + (i - 5000) : 9000 + (i - 5003)));
    Index_type* lst = managed<Index_type>(4);
    lst[0] = 40; lst[1] = 3; lst[2] = 17; lst[3] = 8;
    RAJA::forall_Icount<exec>(RAJA::ListSegment(lst, 4), Index_type(100),
                              [=] RAJA_HOST_DEVICE(Index_type ic, Index_type idx) { w[ic - 100] = idx * 2; });
    okc = okc && w[0] == 80 && w[1] == 6 && w[2] == 34 && w[3] == 16;
    CHECK("forall_icount_b200", okc);
    // a mixed IndexSet on b200: per-segment launches, reducer across them
    Index_type* ml = managed<Index_type>(3);
    ml[0] = 6000; ml[1] = 5; ml[2] = 6500;
    RAJA::IndexSet mis;
    mis.push_back(RAJA::RangeSegment(0, 3000));
    mis.push_back(RAJA::ListSegment(ml, 3));
    mis.push_back(RAJA::RangeStrideSegment(7000, 8000, 7));
    for (int i = 0; i < 8003; ++i) w[i] = -1;
    RAJA::ReduceSum<red, long long> msum(0);
    RAJA::forall<exec>(mis, [=] RAJA_HOST_DEVICE(Index_type i) { msum += i; });
    RAJA::forall_Icount<exec>(mis, [=] RAJA_HOST_DEVICE(Index_type ic, Index_type i) { w[ic] = i; });
    long long want = 0;
    std::vector<Index_type> order;
    for (Index_type i = 0; i < 3000; ++i) order.push_back(i);
    order.push_back(6000); order.push_back(5); order.push_back(6500);
    for (Index_type i = 7000; i < 8000; i += 7) order.push_back(i);
    for (Index_type i : order) want += i;
    bool okm = msum.get() == want && mis.getLength() == order.size();
    for (size_t k = 0; k < order.size(); ++k) okm = okm && w[k] == order[k];
    CHECK("indexset_mixed_b200", okm);
    cudaFree(ml);
    cudaFree(w);
    cudaFree(lst);
  }
  {
    // One-launch IndexSets of 12,000 segments whose lengths mix long
    // segments with runs of hundreds of empty and one-element segments, so
    // that a thread's forward walk over segments outgrows its bound and
    // falls back to a search; range-only and mixed (range, strided, list)
    // tables, against seq_exec on disjoint indices.  The GPU writes device
    // memory and the comparison reads a bulk copy of it.
    std::mt19937 g(5);
    const Index_type lens_pick[] = {0, 0, 1, 1, 2, 3, 40, 300, 2000};
    std::vector<Index_type> lens;
    for (int i = 0; i < 12000; ++i) {
      const bool tiny_run = (i / 400) % 3 == 1;  // 400 segments of length 0 or 1
      lens.push_back(tiny_run ? Index_type(g() % 2) : lens_pick[g() % 9]);
    }
    Index_type span = 0, nlist = 0;
    for (size_t i = 0; i < lens.size(); ++i) {
      span += 3 * lens[i] + 1;
      if (i % 3 == 2) nlist += lens[i];
    }
    double* yd = nullptr;
    cudaMalloc(&yd, span * sizeof(double));
    std::vector<double> yg(span), yh2(span);
    Index_type* lists = managed<Index_type>(nlist + 1);  // written here before any launch reads it
    RAJA::TypedIndexSet<RAJA::RangeSegment> rset;
    RAJA::IndexSet mset;
    Index_type base = 0, lpos = 0;
    for (size_t i = 0; i < lens.size(); ++i) {
      const Index_type n = lens[i];
      rset.push_back(RAJA::RangeSegment(base, base + n));
      if (i % 3 == 0) {
        mset.push_back(RAJA::RangeSegment(base, base + n));
      } else if (i % 3 == 1) {
        mset.push_back(RAJA::RangeStrideSegment(base, base + 3 * n, 3));
      } else {
        for (Index_type k = 0; k < n; ++k) lists[lpos + k] = base + 2 * n - 1 - k;
        mset.push_back(RAJA::ListSegment(lists + lpos, n));
        lpos += n;
      }
      base += 3 * n + 1;
    }
    long long want = 0;
    for (Index_type n : lens) want += n;
    bool oki = true;
    double* yh = yh2.data();
    for (int which = 0; which < 2; ++which) {
      std::fill(yh2.begin(), yh2.end(), -1.0);
      cudaMemcpy(yd, yh2.data(), span * sizeof(double), cudaMemcpyHostToDevice);
      RAJA::ReduceSum<red, long long> icnt(0);
      auto body = [=] RAJA_DEVICE(Index_type i) {
        yd[i] += 2.0 * double(i) + 1.0;
        icnt += 1;
      };
      if (which == 0) RAJA::forall<exec>(rset, body);
      else RAJA::forall<exec>(mset, body);
      auto hbody = [=](Index_type i) { yh[i] += 2.0 * double(i) + 1.0; };
      if (which == 0) RAJA::forall<RAJA::seq_exec>(rset, hbody);
      else RAJA::forall<RAJA::seq_exec>(mset, hbody);
      oki = oki && icnt.get() == want;
      cudaMemcpy(yg.data(), yd, span * sizeof(double), cudaMemcpyDeviceToHost);
      oki = oki && yg == yh2;
    }
    CHECK("indexset_one_launch_tiny_segment_runs", oki);
    cudaFree(yd);
    cudaFree(lists);
  }
  {
    using wpol = RAJA::WorkGroupPolicy<RAJA::b200_work<256, false>, RAJA::unordered>;
    RAJA::WorkPool<wpol, Index_type> pool;
    auto group = pool.instantiate();
    auto site = group.run();
    RAJA::resources::Cuda fresh;
    fresh.wait();
    CHECK("edge_empty_workgroup_and_idle_resource", pool.num_loops() == 0);
  }
  cudaFree(a);
}

// Bandwidth of the lambda-body paths (printed, not asserted): daxpy through
// forall<b200_exec_async>, a ReduceSum<b200_reduce> dot, an expt::Reduce
// dot, and daxpy through RAJA::launch, at 2^27 doubles (above the L2).
// dynamic_forall with a b200 entry, CombiningAdapter (plain and permuted)
// and an atomic view on b200 policies, checked against the host loops.
void test_forall_adapters() {
  using pols = camp::list<RAJA::seq_exec, exec>;
  bool ok = true;
  Index_type* w = managed<Index_type>(1000);
  for (int pol = 0; pol < 2; ++pol) {
    for (int i = 0; i < 1000; ++i) w[i] = -1;
    RAJA::dynamic_forall<pols>(pol, RAJA::TypedRangeSegment<Index_type>(5, 1005),
                               [=] RAJA_HOST_DEVICE(Index_type i) { w[i - 5] = i; });
    cudaDeviceSynchronize();
    for (int i = 0; i < 1000; ++i) ok = ok && w[i] == i + 5;
  }
  CHECK("dynamic_forall_seq_and_b200", ok);

  const int f0 = -7, l0 = 120, f1 = 3, l1 = 260, f2 = 1, l2 = 9;
  const int N0 = l0 - f0, N1 = l1 - f1, N2 = l2 - f2;
  int* c = managed<int>(size_t(N0) * N1 * N2 + 1);
  for (int k = 0; k <= N0 * N1 * N2; ++k) c[k] = 0;
  auto a3 = RAJA::make_CombiningAdapter(
      [=] RAJA_HOST_DEVICE(int i0, int i1, int i2) {
        if (i0 >= f0 && i0 < l0 && i1 >= f1 && i1 < l1 && i2 >= f2 && i2 < l2)
          c[((i0 - f0) * N1 + (i1 - f1)) * N2 + (i2 - f2)] += ((i0 - f0) * N1 + (i1 - f1)) * N2 + (i2 - f2);
        else
          RAJA::atomicAdd<RAJA::b200_atomic>(c + N0 * N1 * N2, 1);
      },
      RAJA::TypedRangeSegment<int>(f0, l0), RAJA::TypedRangeSegment<int>(f1, l1), RAJA::TypedRangeSegment<int>(f2, l2));
  RAJA::forall<exec>(a3.getRange(), a3);
  cudaDeviceSynchronize();
  ok = a3.size() == N0 * N1 * N2 && c[N0 * N1 * N2] == 0;
  for (int k = 0; k < N0 * N1 * N2; ++k) ok = ok && c[k] == k;
  CHECK("combining_adapter_3d_b200", ok);

  // permuted (PERM_JI: the first range fastest): each linear index writes its (i, j)
  int* pi = managed<int>(size_t(N0) * N1);
  auto ap = RAJA::make_PermutedCombiningAdapter<RAJA::PERM_JI>(
      [=] RAJA_HOST_DEVICE(int i0, int i1) { pi[(i1 - f1) * N0 + (i0 - f0)] = i0 * 1000 + i1; },
      RAJA::TypedRangeSegment<int>(f0, l0), RAJA::TypedRangeSegment<int>(f1, l1));
  RAJA::forall<exec>(ap.getRange(), ap);
  cudaDeviceSynchronize();
  ok = true;
  for (int lin = 0; lin < N0 * N1; ++lin) {
    const int i0 = f0 + lin % N0, i1 = f1 + lin / N0;
    ok = ok && pi[lin] == i0 * 1000 + i1;
  }
  CHECK("permuted_combining_adapter_b200", ok);

  // atomic view: a 2-D histogram with b200_atomic against the host count
  int* h = managed<int>(8 * 16);
  for (int k = 0; k < 128; ++k) h[k] = 0;
  RAJA::View<int, RAJA::Layout<2>> hv(h, 8, 16);
  auto av = RAJA::make_atomic_view<RAJA::b200_atomic>(hv);
  RAJA::forall<exec>(RAJA::RangeSegment(0, 1 << 20), [=] RAJA_HOST_DEVICE(Index_type k) {
    const Index_type x = (k * 2654435761ll) & 0xffff;
    av(x % 8, (x / 8) % 16) += 1;
  });
  cudaDeviceSynchronize();
  std::vector<int> ref(128, 0);
  for (Index_type k = 0; k < (1 << 20); ++k) {
    const Index_type x = (k * 2654435761ll) & 0xffff;
    ref[(x % 8) * 16 + (x / 8) % 16] += 1;
  }
  ok = true;
  for (int k = 0; k < 128; ++k) ok = ok && h[k] == ref[k];
  CHECK("atomic_view_b200", ok);
  cudaFree(w);
  cudaFree(c);
  cudaFree(pi);
  cudaFree(h);
}

void perf_lambda_paths() {
  const Index_type n = Index_type(1) << 27;
  double *x = nullptr, *y = nullptr;
  if (cudaMalloc(&x, n * sizeof(double)) != cudaSuccess || cudaMalloc(&y, n * sizeof(double)) != cudaSuccess) {
    printf("perf: allocation failed\n");
    return;
  }
  cudaMemset(x, 0, n * sizeof(double));
  cudaMemset(y, 0, n * sizeof(double));
  using async = RAJA::b200_exec_async<256>;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  auto timed = [&](const char* what, double bytes, int reps, auto&& f) {
    f();
    cudaDeviceSynchronize();
    cudaEventRecord(a, 0);
    for (int r = 0; r < reps; ++r) f();
    cudaEventRecord(b, 0);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    ms /= reps;
    printf("perf: %-34s %8.4f ms  %7.1f GB/s\n", what, ms, bytes / (ms * 1e6));
  };
  timed("forall daxpy (lambda, async)", 24.0 * n, 10, [&] {
    RAJA::forall<async>(RAJA::RangeSegment(0, n), [=] __device__(Index_type i) { y[i] += 2.5 * x[i]; });
  });
  timed("ReduceSum dot (lambda)", 16.0 * n, 5, [&] {
    RAJA::ReduceSum<red, double> d(0.0);
    RAJA::forall<async>(RAJA::RangeSegment(0, n), [=] __device__(Index_type i) { d += x[i] * y[i]; });
    (void)d.get();
  });
  timed("expt::Reduce dot (lambda)", 16.0 * n, 5, [&] {
    double d = 0.0;
    RAJA::forall<async>(RAJA::RangeSegment(0, n), RAJA::expt::Reduce<RAJA::operators::plus>(&d),
                        [=] __device__(Index_type i, RAJA::expt::ValOp<double, RAJA::operators::plus>& v) {
                          v += x[i] * y[i];
                        });
  });
  using alaunch = RAJA::LaunchPolicy<RAJA::b200_launch_t<true>>;
  timed("launch daxpy (global thread loop)", 24.0 * n, 10, [&] {
    RAJA::launch<alaunch>(RAJA::LaunchParams(RAJA::Teams(152 * 8), RAJA::Threads(256)),
                          [=] __device__(RAJA::LaunchContext ctx) {
      RAJA::loop<RAJA::LoopPolicy<RAJA::b200_global_x_loop>>(ctx, RAJA::RangeSegment(0, n),
                                                              [&](Index_type i) { y[i] += 2.5 * x[i]; });
    });
  });
  cudaDeviceSynchronize();

  // Per-call cost at a size where launch and combine latency dominate
  // (4096 elements): host time to submit an async forall, and the full
  // round trip of the synchronous forms.
  const Index_type m = 4096;
  auto per_call = [&](const char* what, int reps, auto&& f) {
    f();
    cudaDeviceSynchronize();
    const auto t0 = std::chrono::steady_clock::now();
    for (int r = 0; r < reps; ++r) f();
    const auto t1 = std::chrono::steady_clock::now();
    cudaDeviceSynchronize();
    const auto t2 = std::chrono::steady_clock::now();
    const double host = std::chrono::duration<double, std::micro>(t1 - t0).count() / reps;
    const double all = std::chrono::duration<double, std::micro>(t2 - t0).count() / reps;
    printf("perf: %-34s %8.2f us host  %8.2f us per call\n", what, host, all);
  };
  per_call("forall 4096 (async)", 2000, [&] {
    RAJA::forall<async>(RAJA::RangeSegment(0, m), [=] __device__(Index_type i) { y[i] += 2.5 * x[i]; });
  });
  per_call("forall 4096 (sync)", 2000, [&] {
    RAJA::forall<RAJA::b200_exec<256>>(RAJA::RangeSegment(0, m), [=] __device__(Index_type i) { y[i] += 2.5 * x[i]; });
  });
  per_call("ReduceSum 4096 + get()", 2000, [&] {
    RAJA::ReduceSum<red, double> d(0.0);
    RAJA::forall<async>(RAJA::RangeSegment(0, m), [=] __device__(Index_type i) { d += x[i] * y[i]; });
    (void)d.get();
  });
  per_call("expt::Reduce 4096 (sync)", 2000, [&] {
    double d = 0.0;
    RAJA::forall<RAJA::b200_exec<256>>(RAJA::RangeSegment(0, m), RAJA::expt::Reduce<RAJA::operators::plus>(&d),
                                       [=] __device__(Index_type i, RAJA::expt::ValOp<double, RAJA::operators::plus>& v) {
                                         v += x[i] * y[i];
                                       });
  });
  cudaDeviceSynchronize();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(x);
  cudaFree(y);
}

int main() {
  setvbuf(stdout, nullptr, _IONBF, 0);  // every PASS line reaches the log even if the run aborts
  test_workgroup_reuse();
  workgroup_reducers_case<RAJA::unordered>("unordered");
  workgroup_reducers_case<RAJA::ordered>("ordered");
  test_autotune();
  test_graph_capture();
  test_multi_reduce_and_atomics();
  test_reducers();
  test_forall_and_params();
  test_scans();
  test_sorts();
  workgroup_case<RAJA::unordered>("unordered");
  workgroup_case<RAJA::ordered>("ordered");
  test_resources();
  test_launch();
  test_launch_jacobi();
  test_params_segments();
  test_edge_cases();
  test_forall_adapters();
  perf_lambda_paths();
  printf("%d failures\n", g_fail);
  return g_fail;
}
