// Host-only checks of the raja_compat front-end (seq_exec / omp policies)
// against the known answers of the reference's functional tests.
#include <cstdio>
#include <memory>
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
  printf("%d failures\n", g_fail);
  return g_fail;
}
