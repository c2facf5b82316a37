// Host-only checks of the raja_compat front-end (seq_exec / omp policies)
// against the known answers of the reference's functional tests.
#include <algorithm>
#include <cstdio>
#include <sstream>
#include <stdexcept>
#include <string>
#include <memory>
#include <mutex>
#include <numeric>
#include <vector>

#include "RAJA/RAJA.hpp"

using RAJA::Index_type;
static int g_fail = 0;
#define CHECK(name, cond)                                  \
  do {                                                     \
    if (cond) printf("PASS %s\n", name);                   \
    else { printf("FAIL %s (line %d)\n", name, __LINE__); ++g_fail; } \
  } while (0)

// A counting plugin (test/integration/plugin/plugin_to_test.cpp): hooks
// must pair up, with the loop's platform, around every forall.  Registered
// statically, so every forall below runs through the hooks.
struct PluginCounts {
  int pre_capture = 0, post_capture = 0, pre_launch = 0, post_launch = 0;
  RAJA::Platform capture_active = RAJA::Platform::undefined, launch_active = RAJA::Platform::undefined;
  bool paired = true;
  std::string last_name;
};
static PluginCounts g_plugin;
static std::mutex g_plugin_mu;  // foralls inside an OpenMP region call the hooks from every thread
class CounterPlugin : public RAJA::util::PluginStrategy {
 public:
  void preCapture(const RAJA::util::PluginContext& p) override {
    std::lock_guard<std::mutex> lk(g_plugin_mu);
    g_plugin.paired = g_plugin.paired && g_plugin.capture_active == RAJA::Platform::undefined;
    ++g_plugin.pre_capture;
    g_plugin.capture_active = p.platform;
    g_plugin.last_name = p.kernel_name;
  }
  void postCapture(const RAJA::util::PluginContext& p) override {
    std::lock_guard<std::mutex> lk(g_plugin_mu);
    g_plugin.paired = g_plugin.paired && g_plugin.capture_active == p.platform;
    ++g_plugin.post_capture;
    g_plugin.capture_active = RAJA::Platform::undefined;
  }
  void preLaunch(const RAJA::util::PluginContext& p) override {
    std::lock_guard<std::mutex> lk(g_plugin_mu);
    g_plugin.paired = g_plugin.paired && g_plugin.launch_active == RAJA::Platform::undefined;
    ++g_plugin.pre_launch;
    g_plugin.launch_active = p.platform;
  }
  void postLaunch(const RAJA::util::PluginContext& p) override {
    std::lock_guard<std::mutex> lk(g_plugin_mu);
    g_plugin.paired = g_plugin.paired && g_plugin.launch_active == p.platform;
    ++g_plugin.post_launch;
    g_plugin.launch_active = RAJA::Platform::undefined;
  }
};
static RAJA::util::PluginRegistry::add<CounterPlugin> g_counter_plugin("counter-plugin", "Counter");

// test-plugin-forall.hpp: ten one-iteration loops, each seeing the capture
// and launch hooks active with the host platform while it runs.
static void plugin_hooks() {
  // earlier loops include foralls issued from every thread of an OpenMP
  // region, whose hooks interleave; pairing is checked from here on
  g_plugin.paired = true;
  g_plugin.capture_active = g_plugin.launch_active = RAJA::Platform::undefined;
  const PluginCounts before = g_plugin;
  std::vector<int> seen(10, 0);
  int* sp = seen.data();
  for (int i = 0; i < 10; ++i) {
    RAJA::forall<RAJA::seq_exec>(RAJA::RangeSegment(i, i + 1), [=](Index_type k) {
      sp[k] = (g_plugin.launch_active == RAJA::Platform::host) ? g_plugin.pre_launch - before.pre_launch : -1;
    });
  }
  bool ok = true;
  for (int i = 0; i < 10; ++i) ok = ok && seen[i] == i + 1;
  CHECK("plugin_launch_active_during_loop", ok);
  CHECK("plugin_counts_pair_up", g_plugin.pre_capture - before.pre_capture == 10 &&
                                     g_plugin.post_capture - before.post_capture == 10 &&
                                     g_plugin.pre_launch - before.pre_launch == 10 &&
                                     g_plugin.post_launch - before.post_launch == 10 && g_plugin.paired &&
                                     g_plugin.capture_active == RAJA::Platform::undefined &&
                                     g_plugin.launch_active == RAJA::Platform::undefined);
  double t = 0.0;
  RAJA::forall<RAJA::seq_exec>(RAJA::RangeSegment(0, 4), RAJA::Name("named_loop"),
                               RAJA::expt::Reduce<RAJA::operators::plus>(&t),
                               [=](Index_type k, RAJA::expt::ValOp<double, RAJA::operators::plus>& v) { v += double(k); });
  CHECK("plugin_sees_kernel_name", g_plugin.last_name == "named_loop" && t == 6.0);

  // launch (test-plugin-launch.hpp): one capture and one launch per call
  PluginCounts b = g_plugin;
  int launch_seen = 0;
  int* ls = &launch_seen;
  RAJA::launch<RAJA::LaunchPolicy<RAJA::seq_launch_t>>(RAJA::LaunchParams(RAJA::Teams(1), RAJA::Threads(1)),
                                                        [=](RAJA::LaunchContext) {
                                                          *ls = g_plugin.launch_active == RAJA::Platform::host;
                                                        });
  CHECK("plugin_launch_hooks", launch_seen == 1 && g_plugin.pre_capture - b.pre_capture == 1 &&
                                   g_plugin.pre_launch - b.pre_launch == 1 &&
                                   g_plugin.post_launch - b.post_launch == 1 && g_plugin.paired);

  // WorkGroup (test-plugin-workgroup.hpp): a capture per enqueue, one launch per run
  b = g_plugin;
  std::vector<int> wseen(10, 0);
  int* wsp = wseen.data();
  RAJA::WorkPool<RAJA::WorkGroupPolicy<RAJA::seq_exec, RAJA::ordered>, Index_type> pool;
  for (int i = 0; i < 10; ++i)
    pool.enqueue(RAJA::TypedRangeSegment<Index_type>(i, i + 1),
                 [=](Index_type k) { wsp[k] = g_plugin.launch_active == RAJA::Platform::host ? 1 : -1; });
  const bool after_enqueue = g_plugin.pre_capture - b.pre_capture == 10 &&
                             g_plugin.post_capture - b.post_capture == 10 && g_plugin.pre_launch == b.pre_launch;
  auto group = pool.instantiate();
  group.run();
  ok = after_enqueue && g_plugin.pre_launch - b.pre_launch == 1 && g_plugin.post_launch - b.post_launch == 1 &&
            g_plugin.pre_capture - b.pre_capture == 10 && g_plugin.paired;
  for (int v : wseen) ok = ok && v == 1;
  CHECK("plugin_workgroup_hooks", ok);
}

// Strongly typed indices (test/include/RAJA_test-index-types.hpp)
RAJA_INDEX_VALUE(StrongIndexType, "StrongIndexType");
RAJA_INDEX_VALUE_T(StrongInt, int, "StrongIntType");
RAJA_INDEX_VALUE_T(RowIdx, int, "RowIdx");
RAJA_INDEX_VALUE_T(ColIdx, int, "ColIdx");

// forall over segments of strongly typed indices (the StrongIdxTypeList
// cases of test/functional/forall/segment)
template <typename IDX>
static bool strong_forall_case() {
  const Index_type first = 3, last = 1030;
  std::vector<Index_type> w(last - first, 0), w2(last - first, 0);
  Index_type* wp = w.data();
  Index_type* wp2 = w2.data();
  RAJA::TypedRangeSegment<IDX> r{IDX(first), IDX(last)};
  RAJA::forall<RAJA::seq_exec>(r, [=](IDX i) { wp[RAJA::stripIndexType(i) - first] += RAJA::stripIndexType(i); });
  RAJA::forall<RAJA::omp_parallel_for_exec>(r, [=](IDX i) { wp2[RAJA::stripIndexType(i - IDX(first))] += 1; });
  std::vector<IDX> lst;
  for (Index_type i = first; i < last; i += 7) lst.push_back(IDX(i));
  RAJA::TypedListSegment<IDX> ls(lst.data(), Index_type(lst.size()));
  RAJA::forall<RAJA::seq_exec>(ls, [=](IDX i) { wp2[RAJA::stripIndexType(i) - first] += 10; });
  RAJA::TypedIndexSet<RAJA::TypedRangeSegment<IDX>> is;
  is.push_back(RAJA::TypedRangeSegment<IDX>(IDX(first), IDX(first + 5)));
  is.push_back(RAJA::TypedRangeSegment<IDX>(IDX(first + 5), IDX(last)));
  Index_type count = 0;
  Index_type* cp = &count;
  RAJA::forall<RAJA::seq_exec>(is, [=](IDX) { ++*cp; });
  bool ok = Index_type(RAJA::stripIndexType(r.size())) == last - first && count == last - first &&
            is.getLength() == size_t(last - first);
  for (Index_type i = first; i < last; ++i) {
    ok = ok && w[i - first] == i && w2[i - first] == 1 + ((i - first) % 7 == 0 ? 10 : 0);
  }
  return ok;
}

// Several reducers in one loop body, with staggered initial values and
// two accumulating loops (forall/reduce-multiple-segment).
template <typename EXEC, typename RED>
static bool multiple_reducers_case() {
  const Index_type first = 5, last = 1357;
  std::vector<double> a(last, 2.0);
  double* p = a.data();
  RAJA::ReduceSum<RED, double> s0(0.0), s1(2.0), s2(0.0), s3(6.0);
  RAJA::ReduceMin<RED, double> mn0(1e9), mn1(-5.0);
  RAJA::ReduceMax<RED, double> mx0(-1e9), mx1(50.0);
  RAJA::ReduceMinLoc<RED, double, Index_type> ml(1e9, -1);
  RAJA::ReduceMaxLoc<RED, double, Index_type> xl(-1e9, -1);
  bool ok = true;
  const double len = double(last - first);
  for (int j = 0; j < 2; ++j) {
    a[700] = -3.0 - j;       // the minimum moves on the second loop
    a[900] = 40.0 + j;       // and so does the maximum
    RAJA::forall<EXEC>(RAJA::TypedRangeSegment<Index_type>(first, last), [=](Index_type i) {
      s0 += p[i];
      s1 += p[i] * 2;
      s2 += p[i] * 3;
      s3 += p[i] * 4;
      mn0.min(p[i]);
      mn1.min(p[i]);
      mx0.max(p[i]);
      mx1.max(p[i]);
      ml.minloc(p[i], i);
      xl.maxloc(p[i], i);
    });
    double acc = 0.0;
    for (int k = 0; k <= j; ++k) acc += 2.0 * (len - 2) + (-3.0 - k) + (40.0 + k);
    ok = ok && s0.get() == acc && s1.get() == 2 * acc + 2.0 && s2.get() == 3 * acc && s3.get() == 4 * acc + 6.0;
    ok = ok && mn0.get() == -3.0 - j && mn1.get() == -5.0 && mx0.get() == 40.0 + j && mx1.get() == 50.0;
    ok = ok && ml.get() == -3.0 - j && ml.getLoc() == 700 && xl.get() == 40.0 + j && xl.getLoc() == 900;
  }
  return ok;
}

// IndexSets under ExecPolicy<seq_segit | omp_parallel_segit, ...>
// (forall/indexset) and getIndices[Conditional] (index/IndexSetUtils.hpp)
static void indexset_exec_policies() {
  std::vector<Index_type> lst{40, 41, 45, 47, 60};
  RAJA::TypedIndexSet<RAJA::RangeSegment, RAJA::ListSegment, RAJA::RangeStrideSegment> is;
  is.push_back(RAJA::RangeSegment(0, 10));
  is.push_back(RAJA::ListSegment(lst.data(), Index_type(lst.size())));
  is.push_back(RAJA::RangeStrideSegment(100, 130, 3));
  is.push_back(RAJA::RangeSegment(200, 1200));
  std::vector<Index_type> expect;
  for (Index_type i = 0; i < 10; ++i) expect.push_back(i);
  for (Index_type v : lst) expect.push_back(v);
  for (Index_type i = 100; i < 130; i += 3) expect.push_back(i);
  for (Index_type i = 200; i < 1200; ++i) expect.push_back(i);
  std::vector<Index_type> got;
  RAJA::getIndices(got, is);
  CHECK("get_indices_indexset", got == expect);
  std::vector<Index_type> even;
  RAJA::getIndicesConditional(even, is, [](Index_type i) { return i % 2 == 0; });
  bool ok = true;
  size_t k = 0;
  for (Index_type v : expect)
    if (v % 2 == 0) ok = ok && k < even.size() && even[k++] == v;
  std::vector<Index_type> rseg;
  RAJA::getIndices(rseg, RAJA::RangeSegment(3, 7));
  CHECK("get_indices_conditional_and_segment", ok && k == even.size() && (rseg == std::vector<Index_type>{3, 4, 5, 6}));

  std::vector<int> hit(1200, 0);
  int* hp = hit.data();
  RAJA::forall<RAJA::ExecPolicy<RAJA::seq_segit, RAJA::seq_exec>>(is, [=](Index_type i) { hp[i] += 1; });
  RAJA::forall<RAJA::ExecPolicy<RAJA::seq_segit, RAJA::omp_parallel_for_exec>>(is, [=](Index_type i) { hp[i] += 2; });
  RAJA::forall<RAJA::ExecPolicy<RAJA::omp_parallel_segit, RAJA::seq_exec>>(is, [=](Index_type i) { hp[i] += 4; });
  ok = true;
  std::vector<int> ref(1200, 0);
  for (Index_type v : expect) ref[v] = 7;
  for (int i = 0; i < 1200; ++i) ok = ok && hit[i] == ref[i];
  std::vector<Index_type> ic(1200, -1);
  Index_type* icp = ic.data();
  RAJA::forall_Icount<RAJA::ExecPolicy<RAJA::seq_segit, RAJA::seq_exec>>(
      is, [=](Index_type icount, Index_type i) { icp[i] = icount; });
  for (size_t j = 0; j < expect.size(); ++j) ok = ok && ic[expect[j]] == Index_type(j);
  CHECK("indexset_exec_policies", ok);
  double total = 1.0, vmin = 1e9;
  Index_type imin = -1;
  RAJA::forall<RAJA::ExecPolicy<RAJA::seq_segit, RAJA::seq_exec>>(
      is, RAJA::expt::Reduce<RAJA::operators::plus>(&total), RAJA::expt::ReduceLoc<RAJA::operators::minimum>(&vmin, &imin),
      [=](Index_type i, RAJA::expt::ValOp<double, RAJA::operators::plus>& s,
          RAJA::expt::ValOp<RAJA::expt::ValLoc<double, Index_type>, RAJA::operators::minimum>& m) {
        s += double(i);
        m.minloc(double((i * 37) % 101), i);
      });
  double ref_total = 1.0, ref_min = 1e9;
  Index_type ref_loc = -1;
  for (Index_type v : expect) {
    ref_total += double(v);
    const double x = double((v * 37) % 101);
    if (x < ref_min) { ref_min = x; ref_loc = v; }
  }
  CHECK("indexset_exec_policy_params", total == ref_total && vmin == ref_min && imin == ref_loc);
}

// index views (util/IndexLayout.hpp) and the for_each utilities
static void index_views_and_for_each() {
  std::vector<double> a(4 * 5);
  for (int k = 0; k < 20; ++k) a[k] = k;
  std::vector<Index_type> rows{3, 0, 2};
  auto lay = RAJA::make_index_layout(
      RAJA::make_index_tuple(RAJA::IndexList<>{rows.data()}, RAJA::DirectIndex<>()), 4, 5);
  auto v = RAJA::make_index_view(a.data(), lay);
  RAJA::View<double, RAJA::IndexLayout<1, Index_type, RAJA::ConditionalIndexList<>>> c0(
      a.data(), RAJA::make_index_layout(RAJA::make_index_tuple(RAJA::ConditionalIndexList<>{nullptr}), 20));
  std::vector<Index_type> pick{19, 4};
  RAJA::View<double, RAJA::IndexLayout<1, Index_type, RAJA::ConditionalIndexList<>>> c1(
      a.data(), RAJA::make_index_layout(RAJA::make_index_tuple(RAJA::ConditionalIndexList<>{pick.data()}), 20));
  CHECK("index_view", v(0, 1) == 16 && v(1, 4) == 4 && v(2, 0) == 10 && c0(7) == 7 && c1(0) == 19 && c1(1) == 4);
  int sum = 0;
  std::vector<int> xs{1, 2, 3, 4};
  RAJA::for_each(xs, [&](int x) { sum += x; });
  int types = 0;
  RAJA::for_each_type(camp::list<int, double, char>{}, [&](auto t) { types += int(sizeof(t)); });
  std::string cat;
  RAJA::for_each_tuple(std::make_tuple(1, std::string("b"), 'c'), [&](const auto& x) {
    std::ostringstream o;
    o << x;
    cat += o.str();
  });
  std::vector<int> g(2 * 3 * 4);
  for (int k = 0; k < 24; ++k) g[k] = k;
  auto vr = RAJA::make_permuted_view<RAJA::layout_right>(g.data(), 2, 3, 4);
  auto vl = RAJA::make_permuted_view<RAJA::layout_left>(g.data(), 2, 3, 4);
  auto vp = RAJA::make_permuted_view<RAJA::PERM_JIK>(g.data(), 2, 3, 4);   // k fastest, then i, then j
  CHECK("permuted_views", vr(1, 0, 2) == 14 && vl(1, 0, 2) == 13 && vp(1, 0, 2) == 6 && vr(1, 2, 3) == 23);
  CHECK("math_helpers", RAJA::log2(1) == 0 && RAJA::log2(1023) == 9 && RAJA::log2(1024) == 10 && RAJA::log2(-5) == 0 &&
                            RAJA::next_pow2(0) == 0 && RAJA::next_pow2(5) == 8 && RAJA::next_pow2(64) == 64 &&
                            RAJA::next_pow2(-3) == 0 && RAJA::prev_pow2(5) == 4 && RAJA::prev_pow2(64) == 64 &&
                            RAJA::prev_pow2(-1) == 0 && RAJA::power_of_2_mod(37, 16) == 5 &&
                            RAJA::next_pow2(uint8_t(200)) == 0 && RAJA::prev_pow2(uint8_t(200)) == 128);
  CHECK("for_each_utilities", sum == 10 && types == int(sizeof(int) + sizeof(double) + sizeof(char)) && cat == "1bc");
}

// buildIndexSetAligned (test/functional/indexset-build/test-aligned-indexset.cpp)
static void indexset_builders() {
  std::vector<Index_type> idx(16);
  std::iota(idx.begin(), idx.end(), 0);
  idx.push_back(17);
  idx.push_back(18);
  for (Index_type i = 20; i < 28; ++i) idx.push_back(i);
  idx.push_back(29);
  idx.push_back(30);
  idx.push_back(31);
  RAJA::resources::Resource res{RAJA::resources::Host::get_default()};
  RAJA::TypedIndexSet<RAJA::RangeSegment, RAJA::ListSegment> iset;
  RAJA::buildIndexSetAligned(iset, res, idx.data(), Index_type(idx.size()), 8, 2);
  using RS = RAJA::RangeSegment;
  using LS = RAJA::ListSegment;
  bool ok = iset.getLength() == idx.size() && iset.getNumSegments() == 5;
  ok = ok && iset.getSegment<RS>(0).size() == 16 && *iset.getSegment<RS>(0).begin() == 0;
  ok = ok && iset.getSegment<LS>(1).size() == 2 && *iset.getSegment<LS>(1).begin() == 17;
  ok = ok && iset.getSegment<RS>(2).size() == 8 && *iset.getSegment<RS>(2).begin() == 20;
  ok = ok && iset.getSegment<LS>(3).size() == 1 && *iset.getSegment<LS>(3).begin() == 29;
  ok = ok && iset.getSegment<RS>(4).size() == 2 && *iset.getSegment<RS>(4).begin() == 30;
  CHECK("index_set_aligned_reference_case", ok);
  // the segments visit exactly the input indices, in order
  std::vector<Index_type> seen;
  RAJA::forall<RAJA::seq_exec>(iset, [&](Index_type i) { seen.push_back(i); });
  CHECK("index_set_aligned_order", seen == idx);
  // short input, or a split that saves too little: one list segment
  RAJA::TypedIndexSet<RAJA::RangeSegment, RAJA::ListSegment> s1, s2, s3;
  RAJA::buildIndexSetAligned(s1, res, idx.data(), 8, 8, 2);
  std::vector<Index_type> scattered;
  for (Index_type i = 0; i < 40; ++i) scattered.push_back(3 * i + 1);
  RAJA::buildIndexSetAligned(s2, res, scattered.data(), 40, 8, 2);
  std::vector<Index_type> dense(1000);
  std::iota(dense.begin(), dense.end(), 64);
  RAJA::buildIndexSetAligned(s3, res, dense.data(), 1000, 8, 32);
  CHECK("index_set_aligned_short_and_scattered", s1.getNumSegments() == 1 && s1.getLength() == 8 &&
                                                      s2.getNumSegments() == 1 && s2.getLength() == 40);
  CHECK("index_set_aligned_dense_is_one_range",
        s3.getNumSegments() == 1 && s3.getSegment<RS>(0).size() == 1000 && *s3.getSegment<RS>(0).begin() == 64);
}

// dynamic_forall, CombiningAdapter, permuted layouts, atomic views,
// omp_atomic and regions (test/functional/dynamic_forall,
// forall/CombiningAdapter, forall/atomic-view, forall/region,
// unit/view-layout).
static void forall_adapters_and_regions() {
  using pols = camp::list<RAJA::seq_exec, RAJA::omp_parallel_for_exec, RAJA::simd_exec>;
  for (int pol = 0; pol < 3; ++pol) {
    std::vector<Index_type> w(100, -1);
    Index_type* wp = w.data();
    RAJA::dynamic_forall<pols>(pol, RAJA::TypedRangeSegment<Index_type>(7, 107),
                               [=](Index_type i) { wp[i - 7] = i; });
    bool ok = true;
    for (Index_type i = 0; i < 100; ++i) ok = ok && w[i] == i + 7;
    CHECK("dynamic_forall_range", ok);
  }
  {
    int zero = 0;
    int* zp = &zero;
    RAJA::dynamic_forall<pols>(1, RAJA::TypedRangeSegment<int>(5, 5), [=](int) { ++*zp; });
    bool threw = false;
    try {
      RAJA::dynamic_forall<pols>(3, RAJA::RangeSegment(0, 4), [=](Index_type) {});
    } catch (const std::runtime_error&) {
      threw = true;
    }
    std::vector<int> w(10, 0);
    int* wp = w.data();
    RAJA::resources::Resource host{RAJA::resources::Host::get_default()};
    auto ev = RAJA::dynamic_forall<pols>(host, 0, RAJA::RangeSegment(0, 10), [=](Index_type i) { wp[i] = 3; });
    ev.get().wait();
    CHECK("dynamic_forall_empty_range_and_bad_policy", zero == 0 && threw);
    CHECK("dynamic_forall_resource", std::accumulate(w.begin(), w.end(), 0) == 30);
  }
  // CombiningAdapter 1-D, 2-D, 3-D with non-zero begins (and an empty range)
  {
    const int f0 = -3, l0 = 5, f1 = 2, l1 = 9, f2 = 1, l2 = 4;
    const int N0 = l0 - f0, N1 = l1 - f1, N2 = l2 - f2;
    std::vector<int> w(N0 * N1 * N2 + 1, 0);
    int* wp = w.data();
    auto a2 = RAJA::make_CombiningAdapter(
        [=](int i0, int i1) {
          if (i0 >= f0 && i0 < l0 && i1 >= f1 && i1 < l1) wp[(i0 - f0) * N1 + (i1 - f1)] += (i0 - f0) * N1 + (i1 - f1);
          else wp[N0 * N1 * N2]++;
        },
        RAJA::TypedRangeSegment<int>(f0, l0), RAJA::TypedRangeSegment<int>(f1, l1));
    RAJA::forall<RAJA::omp_parallel_for_exec>(a2.getRange(), a2);
    bool ok = a2.size() == N0 * N1 && w[N0 * N1 * N2] == 0;
    for (int k = 0; k < N0 * N1; ++k) ok = ok && w[k] == k;
    CHECK("combining_adapter_2d", ok);
    std::fill(w.begin(), w.end(), 0);
    auto a3 = RAJA::make_CombiningAdapter([=](int i0, int i1, int i2) { wp[((i0 - f0) * N1 + (i1 - f1)) * N2 + (i2 - f2)] += 1; },
                                          RAJA::TypedRangeSegment<int>(f0, l0), RAJA::TypedRangeSegment<int>(f1, l1),
                                          RAJA::TypedRangeSegment<int>(f2, l2));
    RAJA::forall<RAJA::seq_exec>(a3.getRange(), a3);
    ok = a3.size() == N0 * N1 * N2;
    for (int k = 0; k < N0 * N1 * N2; ++k) ok = ok && w[k] == 1;
    CHECK("combining_adapter_3d", ok);
    int calls = 0;
    int* cp = &calls;
    auto a1 = RAJA::make_CombiningAdapter([=](int i) { *cp += i; }, RAJA::TypedRangeSegment<int>(10, 13));
    RAJA::forall<RAJA::seq_exec>(a1.getRange(), a1);
    auto ae = RAJA::make_CombiningAdapter([=](int, int) { *cp += 1000; }, RAJA::TypedRangeSegment<int>(0, 4),
                                          RAJA::TypedRangeSegment<int>(3, 3));
    RAJA::forall<RAJA::seq_exec>(ae.getRange(), ae);
    CHECK("combining_adapter_1d_and_empty", calls == 33 && ae.size() == 0);
    // permuted: PERM_JI makes the first range the fastest
    std::vector<int> order;
    auto ap = RAJA::make_PermutedCombiningAdapter<RAJA::PERM_JI>([&](int i, int j) { order.push_back(10 * i + j); },
                                                                 RAJA::TypedRangeSegment<int>(0, 3),
                                                                 RAJA::TypedRangeSegment<int>(0, 2));
    RAJA::forall<RAJA::seq_exec>(ap.getRange(), ap);
    CHECK("permuted_combining_adapter_order", (order == std::vector<int>{0, 10, 20, 1, 11, 21}));
  }
  // permuted layouts: strides and toIndices round trip
  {
    auto L = RAJA::make_permuted_layout<3>({{4, 5, 6}}, RAJA::as_array<RAJA::PERM_KIJ>::get());
    // PERM_KIJ: j has stride 1, then i, then k
    bool ok = L.strides[1] == 1 && L.strides[0] == 5 && L.strides[2] == 20 && L.size() == 120;
    for (Index_type lin = 0; lin < 120; ++lin) {
      int i = -1, j = -1, k = -1;
      L.toIndices(lin, i, j, k);
      ok = ok && L(i, j, k) == lin && i < 4 && j < 5 && k < 6;
    }
    RAJA::Layout<2> rm(3, 7);
    Index_type i = 0, j = 0;
    rm.toIndices(17, i, j);
    CHECK("permuted_layout_strides_and_to_indices", ok && i == 2 && j == 3 && rm(i, j) == 17);
  }
  // atomic views: a histogram through make_atomic_view under an omp loop
  {
    std::vector<int> bins(7, 0);
    RAJA::View<int, RAJA::Layout<1>> v(bins.data(), 7);
    auto av = RAJA::make_atomic_view<RAJA::omp_atomic>(v);
    RAJA::forall<RAJA::omp_parallel_for_exec>(RAJA::RangeSegment(0, 7000), [=](Index_type k) { av(k % 7) += 1; });
    std::vector<double> fb(3, 0.0);
    RAJA::View<double, RAJA::Layout<1>> fv(fb.data(), 3);
    auto sv = RAJA::make_atomic_view<RAJA::seq_atomic>(fv);
    RAJA::forall<RAJA::seq_exec>(RAJA::RangeSegment(0, 30), [=](Index_type k) { sv(k % 3) += 0.5; });
    bool ok = fb[0] == 5.0 && fb[1] == 5.0 && fb[2] == 5.0;
    for (int b : bins) ok = ok && b == 1000;
    CHECK("atomic_view_omp_and_seq", ok);
  }
  // omp_atomic under an omp loop: min / max / bounded inc / CAS on floats
  {
    double mn = 1e9, mx = -1e9, fsum = 0.0;
    unsigned wrap = 0;
    int cas_hits = 0;
    int flag = 0;
    double* pmn = &mn; double* pmx = &mx; double* pfs = &fsum;
    unsigned* pw = &wrap; int* ph = &cas_hits; int* pf = &flag;
    RAJA::forall<RAJA::omp_parallel_for_exec>(RAJA::RangeSegment(0, 10000), [=](Index_type k) {
      const double x = double((k * 7919) % 10007) - 5000.0;
      RAJA::atomicMin<RAJA::omp_atomic>(pmn, x);
      RAJA::atomicMax<RAJA::omp_atomic>(pmx, x);
      RAJA::atomicAdd<RAJA::omp_atomic>(pfs, 0.25);
      RAJA::atomicInc<RAJA::omp_atomic>(pw, 9u);
      if (RAJA::atomicCAS<RAJA::omp_atomic>(pf, 0, 1) == 0) RAJA::atomicAdd<RAJA::omp_atomic>(ph, 1);
    });
    double rmn = 1e9, rmx = -1e9;
    for (Index_type k = 0; k < 10000; ++k) {
      const double x = double((k * 7919) % 10007) - 5000.0;
      rmn = std::min(rmn, x);
      rmx = std::max(rmx, x);
    }
    CHECK("omp_atomic_min_max_add_inc_cas", mn == rmn && mx == rmx && fsum == 2500.0 && wrap == 10000u % 10u &&
                                                cas_hits == 1 && flag == 1);
  }
  // regions: two loops inside one region (test-forall-region.hpp)
  {
    std::vector<int> idx(1000);
    std::iota(idx.begin(), idx.end(), 0);
    RAJA::TypedListSegment<int> lseg(idx.data(), 1000);
    std::vector<int> w(1000, 0), w2(1000, 0);
    int* wp = w.data();
    int* wp2 = w2.data();
    RAJA::region<RAJA::seq_region>([=]() {
      RAJA::forall<RAJA::seq_exec>(RAJA::TypedRangeSegment<int>(0, 1000), [=](int i) { wp[i] += 1; });
      RAJA::forall<RAJA::seq_exec>(lseg, [=](int i) { wp[i] += 2; });
    });
    RAJA::region<RAJA::omp_parallel_region>([=]() {
      RAJA::forall<RAJA::omp_for_nowait_static_exec<>>(RAJA::TypedRangeSegment<int>(0, 1000), [=](int i) { wp2[i] += 1; });
      RAJA::forall<RAJA::omp_for_nowait_static_exec<>>(lseg, [=](int i) { wp2[i] += 2; });
    });
    bool ok = true;
    for (int i = 0; i < 1000; ++i) ok = ok && w[i] == 3 && w2[i] == 3;
    CHECK("region_seq_and_omp", ok);
  }
}

int main() {
  // ReduceSum with init 0 and 2; reset and two loops (test-forall-basic-ReduceSum.hpp)
  std::vector<double> a(2057);
  for (size_t i = 0; i < a.size(); ++i) a[i] = double((i * 7919) % 100);
  double* p = a.data();
  RAJA::ReduceSum<RAJA::seq_reduce, double> s0(0.0), s2(2.0);
  RAJA::forall<RAJA::seq_exec>(RAJA::RangeSegment(3, 642), [=](Index_type i) { s0 += p[i]; s2 += p[i]; });
  double ref = 0;
  for (int i = 3; i < 642; ++i) ref += a[i];
  CHECK("sum_init0_init2", s0.get() == ref && s2.get() == ref + 2);
  s0.reset(0.0);
  for (int k = 0; k < 2; ++k) RAJA::forall<RAJA::seq_exec>(RAJA::RangeSegment(3, 642), [=](Index_type i) { s0 += p[i]; });
  CHECK("sum_reset_two_loops", s0.get() == 2 * ref);
  // MinLoc: init tie wins (mininit(-100, -1) with planted -100)
  a[400] = -100.0;
  RAJA::ReduceMinLoc<RAJA::seq_reduce, double, Index_type> mi(-100.0, -1), m(101.0, -1);
  RAJA::forall<RAJA::seq_exec>(RAJA::RangeSegment(0, 2057), [=](Index_type i) { mi.minloc(p[i], i); m.minloc(p[i], i); });
  CHECK("minloc_init_wins", mi.get() == -100.0 && mi.getLoc() == -1);
  CHECK("minloc_planted", m.get() == -100.0 && m.getLoc() == 400);
  // omp reducer agrees with seq
  RAJA::ReduceSum<RAJA::omp_reduce, double> so(0.0);
  RAJA::forall<RAJA::omp_parallel_for_exec>(RAJA::RangeSegment(0, 2057), [=](Index_type i) { so += p[i]; });
  double all = 0;
  for (double v : a) all += v;
  CHECK("omp_sum", so.get() == all);
  // BitOr: 9 | 5 == 13
  std::vector<int> nines(100, 9);
  int* q = nines.data();
  RAJA::ReduceBitOr<RAJA::seq_reduce, int> bo(5);
  RAJA::forall<RAJA::seq_exec>(RAJA::RangeSegment(0, 100), [=](Index_type i) { bo |= q[i]; });
  CHECK("bitor_9_5", bo.get() == 13);
  // scans: iota, plus / min / max, offsets 13, 15, 2
  for (int n : {0, 357, 32000}) {
    std::vector<int> in(n), out(n);
    std::iota(in.begin(), in.end(), 1);
    RAJA::inclusive_scan<RAJA::seq_exec>(RAJA::make_span((const int*)in.data(), n), RAJA::make_span(out.data(), n));
    bool ok = true;
    long acc = 0;
    for (int i = 0; i < n; ++i) { acc += i + 1; ok = ok && out[i] == int(acc); }
    CHECK("inclusive_plus_iota", ok);
    const int off = n == 0 ? 13 : (n == 357 ? 15 : 2);
    RAJA::exclusive_scan<RAJA::seq_exec>(RAJA::make_span((const int*)in.data(), n), RAJA::make_span(out.data(), n),
                                         RAJA::operators::plus<int>{}, off);
    ok = true;
    acc = off;
    for (int i = 0; i < n; ++i) { ok = ok && out[i] == int(acc); acc += i + 1; }
    CHECK("exclusive_plus_offset", ok);
    RAJA::inclusive_scan<RAJA::seq_exec>(RAJA::make_span((const int*)in.data(), n), RAJA::make_span(out.data(), n),
                                         RAJA::operators::maximum<int>{});
    ok = true;
    for (int i = 0; i < n; ++i) ok = ok && out[i] == i + 1;
    CHECK("inclusive_max_iota", ok);
  }
  // sorts: stable pairs keep input order among equal keys
  std::vector<int> k{3, 1, 3, 2, 1}, v{0, 1, 2, 3, 4};
  RAJA::stable_sort_pairs<RAJA::seq_exec>(RAJA::make_span(k.data(), 5), RAJA::make_span(v.data(), 5));
  CHECK("stable_sort_pairs", k == std::vector<int>({1, 1, 2, 3, 3}) && v == std::vector<int>({1, 4, 3, 0, 2}));
  RAJA::stable_sort<RAJA::seq_exec>(RAJA::make_span(k.data(), 5), RAJA::operators::greater<int>{});
  CHECK("stable_sort_greater", k == std::vector<int>({3, 3, 2, 1, 1}));
  // expt::Reduce on host: target = op(target, result)
  double t = 1.0;
  RAJA::forall<RAJA::seq_exec>(RAJA::RangeSegment(0, 10), RAJA::expt::Reduce<RAJA::operators::plus>(&t),
                               [=](Index_type i, RAJA::expt::ValOp<double, RAJA::operators::plus>& s) { s += double(i); });
  CHECK("expt_reduce_host", t == 46.0);
  // kernel names may sit before, between or after the reducer params
  double t1 = 0.0, t2 = 100.0;
  RAJA::forall<RAJA::seq_exec>(RAJA::RangeSegment(0, 10), RAJA::Name("a"),
                               RAJA::expt::Reduce<RAJA::operators::plus>(&t1), RAJA::Name("b"),
                               RAJA::expt::Reduce<RAJA::operators::minimum>(&t2), RAJA::Name("c"),
                               [=](Index_type i, RAJA::expt::ValOp<double, RAJA::operators::plus>& s,
                                   RAJA::expt::ValOp<double, RAJA::operators::minimum>& m) {
                                 s += double(i);
                                 m.min(double(i) + 3.0);
                               });
  CHECK("expt_reduce_names_anywhere", t1 == 45.0 && t2 == 3.0);
  // params over strided and list segments (test-forall-basic-param-expt-ReduceSum.hpp segments)
  {
    double ts = 0.0, tm = 1e9;
    RAJA::forall<RAJA::seq_exec>(RAJA::RangeStrideSegment(3, 1029, 3), RAJA::expt::Reduce<RAJA::operators::plus>(&ts),
                                 RAJA::expt::Reduce<RAJA::operators::minimum>(&tm),
                                 [=](Index_type i, RAJA::expt::ValOp<double, RAJA::operators::plus>& s,
                                     RAJA::expt::ValOp<double, RAJA::operators::minimum>& m) {
                                   s += double(i);
                                   m.min(double(1000 - i));
                                 });
    double want = 0.0;
    for (int i = 3; i < 1029; i += 3) want += i;
    const Index_type lst[4] = {7, 2, 11, 5};
    double tl = 0.0;
    RAJA::forall<RAJA::seq_exec>(RAJA::ListSegment(lst, 4), RAJA::expt::Reduce<RAJA::operators::plus>(&tl),
                                 [=](Index_type i, RAJA::expt::ValOp<double, RAJA::operators::plus>& s) {
                                   s += double(i * i);
                                 });
    CHECK("expt_reduce_stride_list_segments", ts == want && tm == double(1000 - 1026) && tl == 49.0 + 4 + 121 + 25);
  }
  // forall_Icount over a segment and over an IndexSet (test-forall-IcountIndexSet.hpp)
  {
    RAJA::TypedIndexSet<RAJA::RangeSegment> is;
    is.push_back(RAJA::RangeSegment(0, 5));
    is.push_back(RAJA::RangeSegment(10, 13));
    is.push_back(RAJA::RangeSegment(20, 24));
    std::vector<Index_type> got(12, -1);
    Index_type* gp = got.data();
    RAJA::forall_Icount<RAJA::seq_exec>(is, [=](Index_type ic, Index_type idx) { gp[ic] = idx; });
    const std::vector<Index_type> want{0, 1, 2, 3, 4, 10, 11, 12, 20, 21, 22, 23};
    std::vector<Index_type> g2(3, -1);
    Index_type* g2p = g2.data();
    RAJA::forall_Icount<RAJA::seq_exec>(RAJA::RangeStrideSegment(5, 11, 2), Index_type(0),
                                        [=](Index_type ic, Index_type idx) { g2p[ic] = idx; });
    CHECK("forall_icount_indexset_and_stride", got == want && g2 == std::vector<Index_type>({5, 7, 9}));
  }
  // a mixed IndexSet: range, list and strided segments (buildIndexSet in the
  // reference's IndexSet tests); traversal order and counts
  {
    const Index_type lst[3] = {50, 41, 47};
    RAJA::IndexSet is;
    is.push_back(RAJA::RangeSegment(0, 4));
    is.push_back(RAJA::ListSegment(lst, 3));
    is.push_back(RAJA::RangeStrideSegment(60, 69, 3));
    is.push_front(RAJA::RangeSegment(100, 102));
    std::vector<Index_type> seen, ics;
    RAJA::forall<RAJA::seq_exec>(is, [&](Index_type i) { seen.push_back(i); });
    RAJA::forall_Icount<RAJA::seq_exec>(is, [&](Index_type ic, Index_type i) { ics.push_back(ic * 1000 + i); });
    const std::vector<Index_type> want{100, 101, 0, 1, 2, 3, 50, 41, 47, 60, 63, 66};
    bool oki = seen == want && is.getNumSegments() == 4 && is.getLength() == 12 && is.getStartingIcount(2) == 6;
    for (size_t k = 0; k < ics.size(); ++k) oki = oki && ics[k] == Index_type(k) * 1000 + want[k];
    oki = oki && is.getSegment<RAJA::ListSegment>(2).size() == 3;
    CHECK("indexset_mixed_segments", oki && ics.size() == 12);
  }
  // segment iterators and slices (index/RangeSegment.hpp)
  {
    RAJA::RangeSegment r(3, 10);
    RAJA::RangeStrideSegment rs(2, 11, 3);
    const std::vector<Index_type> vr(r.begin(), r.end()), vs(rs.begin(), rs.end());
    const RAJA::RangeSegment sl = r.slice(2, 10);
    CHECK("segment_iterators_slice",
          r.end() - r.begin() == 7 && *r.begin() == 3 && r.begin()[2] == 5 &&
              vr == std::vector<Index_type>({3, 4, 5, 6, 7, 8, 9}) && vs == std::vector<Index_type>({2, 5, 8}) &&
              rs.end() - rs.begin() == 3 && sl == RAJA::RangeSegment(5, 10));
  }
  // simd and scheduled OpenMP policies agree with seq (resource-forall example policies)
  {
    std::vector<long> r0(1000, 0), r1(1000, 0), r2(1000, 0), r3(1000, 0);
    long *p0 = r0.data(), *p1 = r1.data(), *p2 = r2.data(), *p3 = r3.data();
    RAJA::forall<RAJA::simd_exec>(RAJA::RangeSegment(0, 1000), [=](Index_type i) { p0[i] = 3 * i; });
    RAJA::forall<RAJA::omp_parallel_for_static_exec<>>(RAJA::RangeSegment(0, 1000), [=](Index_type i) { p1[i] = 3 * i; });
    RAJA::forall<RAJA::omp_parallel_for_dynamic_exec<16>>(RAJA::RangeStrideSegment(0, 1000, 1),
                                                          [=](Index_type i) { p2[i] = 3 * i; });
    RAJA::forall<RAJA::omp_parallel_for_guided_exec<8>>(RAJA::RangeSegment(0, 1000), [=](Index_type i) { p3[i] = 3 * i; });
    CHECK("simd_and_scheduled_omp_policies", r0 == r1 && r1 == r2 && r2 == r3 && r3[999] == 2997);
  }
  // WorkGroup with a dispatch policy and an allocator, pool and group reuse
  // (test-workgroup-*-MultipleReuse.hpp)
  {
    using wpol = RAJA::WorkGroupPolicy<RAJA::seq_exec, RAJA::reverse_ordered, RAJA::array_of_pointers,
                                       RAJA::indirect_function_call_dispatch>;
    RAJA::WorkPool<wpol, Index_type, RAJA::xargs<>, std::allocator<char>> pool(std::allocator<char>{});
    std::vector<int> w2(40, 0);
    int* w2p = w2.data();
    bool okw = true;
    for (int reuse = 0; reuse < 2; ++reuse) {
      pool.enqueue(RAJA::RangeSegment(0, 20), [=](Index_type i) { w2p[i] += 1; });
      pool.enqueue(RAJA::RangeSegment(20, 40), [=](Index_type i) { w2p[i] += 10; });
      auto grp = pool.instantiate();
      okw = okw && pool.num_loops() == 0;
      grp.run();
      grp.run();  // a group runs again
    }
    for (int i = 0; i < 40; ++i) okw = okw && w2[i] == (i < 20 ? 4 : 40);
    CHECK("workgroup_dispatch_allocator_reuse", okw);
  }
  int named = 0;
  RAJA::forall<RAJA::seq_exec>(RAJA::RangeSegment(0, 4), RAJA::Name("only"),
                               [&](Index_type) { ++named; });
  CHECK("forall_name_only", named == 4);
  // WorkGroup (ordered): a[i] += i + 5 (test-workgroup-Unordered-Single.hpp)
  std::vector<int> w(100, 0);
  int* wp = w.data();
  RAJA::WorkPool<RAJA::WorkGroupPolicy<RAJA::seq_exec, RAJA::ordered>, Index_type> pool;
  pool.enqueue(RAJA::RangeSegment(10, 60), [=](Index_type i) { wp[i] += int(i) + 5; });
  auto g = pool.instantiate();
  g.run();
  bool ok = true;
  for (int i = 0; i < 100; ++i) ok = ok && w[i] == ((i >= 10 && i < 60) ? i + 5 : 0);
  CHECK("workgroup_seq", ok);

  // MultiReduce (seq): bins combined in index order with each op's rule
  {
    const int nb = 5;
    RAJA::MultiReduceSum<RAJA::seq_multi_reduce, int> msum(nb);
    RAJA::MultiReduceMin<RAJA::seq_multi_reduce, int> mmin(nb, 100);
    RAJA::MultiReduceMax<RAJA::seq_multi_reduce, int> mmax(nb);
    RAJA::MultiReduceBitOr<RAJA::seq_multi_reduce, int> mor(nb);
    RAJA::MultiReduceBitAnd<RAJA::seq_multi_reduce, int> mand(nb);
    std::vector<int> sum(nb, 0), mn(nb, 100), mx(nb, std::numeric_limits<int>::lowest()),
        bo(nb, 0), ba(nb, -1);
    RAJA::forall<RAJA::seq_exec>(RAJA::RangeSegment(0, 50), [=](Index_type i) {
      const int b = int(i % nb), v = int((i * 37) % 23) - 7;
      msum[b] += v;
      mmin[b].min(v);
      mmax[b].max(v);
      mor[b] |= v;
      mand[b] &= v;
    });
    for (int i = 0; i < 50; ++i) {
      const int b = i % nb, v = (i * 37) % 23 - 7;
      sum[b] += v;
      mn[b] = v < mn[b] ? v : mn[b];
      mx[b] = mx[b] < v ? v : mx[b];
      bo[b] |= v;
      ba[b] &= v;
    }
    bool okm = msum.size() == size_t(nb);
    std::vector<int> all(nb);
    msum.get_all(all);
    for (int b = 0; b < nb; ++b)
      okm = okm && all[b] == sum[b] && mmin.get(b) == mn[b] && mmax[b].get() == mx[b] &&
            mor.get(b) == bo[b] && mand.get(b) == ba[b];
    CHECK("multi_reduce_seq", okm);
    msum.reset();
    CHECK("multi_reduce_reset", msum.get(0) == 0 && msum.get(4) == 0);
  }

  // atomics (seq) and AtomicRef, including the bounded inc / dec rules
  {
    unsigned u = 3;
    bool oka = RAJA::atomicInc<RAJA::seq_atomic>(&u, 3u) == 3u && u == 0u;
    oka = oka && RAJA::atomicDec<RAJA::seq_atomic>(&u, 5u) == 0u && u == 5u;
    oka = oka && RAJA::atomicCAS<RAJA::seq_atomic>(&u, 5u, 9u) == 5u && u == 9u;
    oka = oka && RAJA::atomicCAS<RAJA::seq_atomic>(&u, 5u, 1u) == 9u && u == 9u;
    int x = 10;
    RAJA::AtomicRef<int, RAJA::seq_atomic> r(&x);
    oka = oka && (r += 5) == 15 && r.fetch_sub(3) == 15 && r.load() == 12;
    oka = oka && r.min(4) == 4 && r.max(20) == 20 && (r++) == 20 && x == 21;
    oka = oka && RAJA::atomicExchange<RAJA::seq_atomic>(&x, 7) == 21 && x == 7;
    oka = oka && RAJA::atomicXor<RAJA::seq_atomic>(&x, 5) == 7 && x == 2;
    CHECK("atomics_seq", oka);
  }
  // resources on the host: Host, type-erased Resource and Event, EventProxy
  // returned by forall / scan / sort (test/unit/resource/tests/*.hpp)
  {
    namespace res = RAJA::resources;
    static_assert(std::is_same<res::get_resource<RAJA::seq_exec>::type, res::Host>::value, "host policy");
    res::Host host;
    const int n = 1000;
    int* h = host.allocate<int>(n);
    int* g = res::Resource{host}.allocate<int>(n);
    host.memset(g, 0, sizeof(int) * n);
    RAJA::forall<RAJA::seq_exec>(host, RAJA::RangeSegment(0, n), [=](Index_type i) { h[i] = int(i) + 2; });
    res::Resource er{host};
    er.memcpy(g, h, sizeof(int) * n);
    res::Event e = RAJA::forall<RAJA::seq_exec>(er, RAJA::RangeSegment(0, n), [=](Index_type i) { g[i] *= 3; });
    er.wait_for(&e);
    er.wait();
    bool okr = e.check() && er.get_platform() == res::Platform::host && er.try_get<res::Host>() != nullptr;
    for (int i = 0; i < n; ++i) okr = okr && g[i] == 3 * (i + 2);
    res::HostEvent he = RAJA::forall<RAJA::seq_exec>(RAJA::RangeSegment(0, 1), [](Index_type) {});
    okr = okr && he.check();
    res::Event pe = host.get_event_erased();
    okr = okr && pe.try_get<res::HostEvent>() != nullptr && pe.try_get<int>() == nullptr;
    bool threw = false;
    try {
      (void)pe.get<int>();
    } catch (const std::runtime_error&) {
      threw = true;
    }
    okr = okr && threw;
    // scans and sorts on a resource
    res::Event se = RAJA::inclusive_scan<RAJA::seq_exec>(host, RAJA::make_span((const int*)h, n),
                                                         RAJA::make_span(g, n));
    se.wait();
    long acc = 0;
    for (int i = 0; i < n; ++i) {
      acc += i + 2;
      okr = okr && g[i] == int(acc);
    }
    RAJA::stable_sort<RAJA::seq_exec>(er, RAJA::make_span(g, n), RAJA::operators::greater<int>{});
    for (int i = 1; i < n; ++i) okr = okr && g[i - 1] >= g[i];
    // WorkGroup::run(resource) hands the resource to the WorkSite
    RAJA::WorkPool<RAJA::WorkGroupPolicy<RAJA::seq_exec, RAJA::ordered>, Index_type> pool2;
    pool2.enqueue(RAJA::RangeSegment(0, n), [=](Index_type i) { h[i] = -int(i); });
    auto g2 = pool2.instantiate();
    auto site = g2.run(host);
    okr = okr && site.get_resource().get_platform() == res::Platform::host && h[n - 1] == -(n - 1);
    host.deallocate(h);
    er.deallocate(g);
    CHECK("resources_host", okr);
  }
  // RAJA::launch on the host (test/functional/launch): nested loops over a
  // View, dynamic shared memory with teamSync, tile_tcount + loop_icount,
  // reducer params, run-time place and a resource
  {
    using lpol = RAJA::LaunchPolicy<RAJA::seq_launch_t>;
    using loop = RAJA::LoopPolicy<RAJA::seq_exec>;
    const int N1 = 2, N2 = 3, N3 = 4;
    std::vector<int> a3(N1 * N2 * N3, 0);
    RAJA::View<int, RAJA::Layout<3>> A(a3.data(), N3, N2, N1);
    RAJA::launch<lpol>(RAJA::LaunchParams(RAJA::Teams(N3), RAJA::Threads(N2, N1)), [=](RAJA::LaunchContext ctx) {
      RAJA::loop<loop>(ctx, RAJA::RangeSegment(0, N3), [&](Index_type z) {
        RAJA::loop<loop>(ctx, RAJA::RangeSegment(0, N2), [&](Index_type y) {
          RAJA::loop<loop>(ctx, RAJA::RangeSegment(0, N1), [&](Index_type x) {
            A(z, y, x) += int(x + N1 * (y + N2 * z));
          });
        });
      });
    });
    bool okl = true;
    for (int i = 0; i < N1 * N2 * N3; ++i) okl = okl && a3[i] == i;
    CHECK("launch_seq_nested_view", okl);

    // dynamic shared memory: a reversed tile plus an int tile per team
    const int teams = 5, th = 32;
    std::vector<long> out(teams * th, 0);
    long* op = out.data();
    RAJA::launch<lpol>(RAJA::LaunchParams(RAJA::Teams(teams), RAJA::Threads(th), th * (sizeof(long) + sizeof(int))),
                       [=](RAJA::LaunchContext ctx) {
                         RAJA::loop<loop>(ctx, RAJA::RangeSegment(0, teams), [&](Index_type b) {
                           long* tile = ctx.getSharedMemory<long>(th);
                           int* itile = ctx.getSharedMemory<int>(th);
                           RAJA::loop<loop>(ctx, RAJA::RangeSegment(0, th), [&](Index_type t) {
                             itile[t] = int(t);
                             tile[th - t - 1] = th - t - 1 + th * b;
                           });
                           ctx.teamSync();
                           RAJA::loop<loop>(ctx, RAJA::RangeSegment(0, th), [&](Index_type t) {
                             op[t + th * b] = tile[t] + itile[t];
                           });
                           ctx.releaseSharedMemory();
                         });
                       });
    okl = true;
    for (int b = 0; b < teams; ++b)
      for (int t = 0; t < th; ++t) okl = okl && out[t + th * b] == long(t + th * b) + t;
    CHECK("launch_seq_shared_mem", okl);

    // tile_tcount + loop_icount: tile size 4 over 0..4M (test-launch-nested-Tile-iCount-tCount-Loop.hpp)
    const int M = 5, ts = 4, NT = M * ts + 1;
    std::vector<int> tt(NT, -1), ii(NT, -1);
    int* ttp = tt.data();
    int* iip = ii.data();
    RAJA::launch<lpol>(RAJA::LaunchParams(RAJA::Teams(1), RAJA::Threads(3)), [=](RAJA::LaunchContext ctx) {
      RAJA::tile_tcount<loop>(ctx, ts, RAJA::RangeSegment(0, NT), [&](const RAJA::RangeSegment& tile, Index_type bx) {
        RAJA::loop_icount<loop>(ctx, tile, [&](Index_type tx, Index_type ix) {
          ttp[tx] = int(bx);
          iip[tx] = int(ix);
        });
      });
    });
    okl = true;
    for (int i = 0; i < NT; ++i) okl = okl && tt[i] == i / ts && ii[i] == i % ts;
    CHECK("launch_seq_tile_tcount_icount", okl);

    // reducer params and a kernel name, run-time place, resource
    double s = 2.0;
    int mn = 1000;
    RAJA::launch<RAJA::LaunchPolicy<RAJA::seq_launch_t, RAJA::seq_launch_t>>(
        RAJA::ExecPlace::HOST, RAJA::LaunchParams(RAJA::Teams(4), RAJA::Threads(64)),
        RAJA::expt::Reduce<RAJA::operators::plus>(&s), RAJA::Name("launch_reduce"),
        RAJA::expt::Reduce<RAJA::operators::minimum>(&mn),
        [=](RAJA::LaunchContext ctx, RAJA::expt::ValOp<double, RAJA::operators::plus>& vs,
            RAJA::expt::ValOp<int, RAJA::operators::minimum>& vm) {
          RAJA::loop<loop>(ctx, RAJA::RangeStrideSegment(0, 100, 3), [&](Index_type i) {
            vs += double(i);
            vm.min(int(i) + 7);
          });
        });
    CHECK("launch_seq_reduce_params", s == 2.0 + 1683.0 && mn == 7);
    RAJA::resources::Host host;
    RAJA::resources::Event le = RAJA::launch<lpol>(
        RAJA::resources::Resource{host}, RAJA::LaunchParams(RAJA::Teams(1), RAJA::Threads(1)),
        [=](RAJA::LaunchContext ctx) {
          const Index_type idx[3] = {5, 1, 3};
          RAJA::loop<loop>(ctx, RAJA::ListSegment(idx, 3), [&](Index_type i) { op[i] = -1; });
        });
    le.wait();
    CHECK("launch_seq_resource_list_segment", out[5] == -1 && out[1] == -1 && out[3] == -1 && out[2] != -1);
  }
  forall_adapters_and_regions();
  plugin_hooks();
  indexset_builders();
  indexset_exec_policies();
  index_views_and_for_each();
  CHECK("multiple_reducers_seq", (multiple_reducers_case<RAJA::seq_exec, RAJA::seq_reduce>()));
  CHECK("multiple_reducers_omp", (multiple_reducers_case<RAJA::omp_parallel_for_exec, RAJA::omp_reduce>()));
  CHECK("strong_index_forall", strong_forall_case<StrongIndexType>() && strong_forall_case<StrongInt>());
  {
    StrongIndexType a(5), b(7);
    std::vector<double> m(6 * 9, 0.0);
    RAJA::TypedView<double, RAJA::Layout<2>, RowIdx, ColIdx> tv(m.data(), 6, 9);
    RAJA::forall<RAJA::seq_exec>(RAJA::TypedRangeSegment<RowIdx>{RowIdx(0), RowIdx(6)}, [=](RowIdx r) {
      for (ColIdx c(0); c < 9; ++c) tv(r, c) = 10.0 * *r + *c;
    });
    bool tv_ok = true;
    for (int r = 0; r < 6; ++r)
      for (int c = 0; c < 9; ++c) tv_ok = tv_ok && m[r * 9 + c] == 10.0 * r + c;
    CHECK("typed_view_strong_indices", tv_ok);
    CHECK("strong_index_ops", *(a + b) == 12 && (b - a) == 2 && a < b && RAJA::convertIndex<StrongInt>(b) == 7 &&
                                  StrongIndexType::getName() == "StrongIndexType");
  }
  printf("%d failures\n", g_fail);
  return g_fail;
}
