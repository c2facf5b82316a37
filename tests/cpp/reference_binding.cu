// A RAJA application that switches one policy alias from seq_exec to
// b200_exec, built against an installed RAJA (the reference's own headers)
// plus raja_b200/RAJA_b200.hpp.  Every b200 result is checked against the
// seq_exec result of the same code.  Without a CUDA device only the
// sequential half runs (the program still proves that each RAJA front-end
// binds to a b200 overload: forall over ranges and IndexSets, ReduceSum /
// ReduceMinLoc on b200_reduce, expt::Reduce params, scans, sorts,
// MultiReduceSum on b200_multi_reduce, atomicAdd on b200_atomic, and
// WorkPool / WorkGroup through the b200_work WorkRunner).
#include "raja_b200/RAJA_b200.hpp"  // before RAJA/RAJA.hpp, which it includes

// Loop bodies run on the host (seq_exec) and the device (b200_exec).  RAJA
// spells this RAJA_HOST_DEVICE, which is empty in a RAJA configured without
// its own CUDA back-end (as here), so the bodies say it directly.
#define APP_HOST_DEVICE __host__ __device__

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <vector>

namespace {
int failures = 0;
void check(bool ok, const char* what)
{
  std::printf("%s %s\n", ok ? "PASS" : "FAIL", what);
  if (!ok) ++failures;
}

template <typename ExecPol, typename RedPol>
struct Results {
  std::vector<double> y;
  double sum = 0, psum = 0;
  double minv = 0;
  RAJA::Index_type minloc = -1;
  RAJA::expt::ValLoc<double> pmin;
  std::vector<long long> incl, excl;
  std::vector<int> keys, vals;
  std::vector<double> iset;
};

// The application code: one alias decides where it runs.
template <typename ExecPol, typename RedPol>
Results<ExecPol, RedPol> run(const std::vector<double>& x0, const std::vector<int>& k0, double* x,
                             double* y, long long* a, long long* b, int* k, int* v, double* z)
{
  const RAJA::Index_type n = RAJA::Index_type(x0.size());
  for (RAJA::Index_type i = 0; i < n; ++i) {
    x[i] = x0[i];
    y[i] = 1.0;
    a[i] = (long long)(i % 7);
    k[i] = k0[i];
    v[i] = int(i);
    z[i] = 0.0;
  }
  Results<ExecPol, RedPol> r;
  // forall: daxpy
  RAJA::forall<ExecPol>(RAJA::TypedRangeSegment<RAJA::Index_type>(0, n),
                        [=] APP_HOST_DEVICE(RAJA::Index_type i) { y[i] += 2.5 * x[i]; });
  // classic reducers captured by the body
  RAJA::ReduceSum<RedPol, double> sum(0.0);
  RAJA::ReduceMinLoc<RedPol, double, RAJA::Index_type> mnl(1e300, -1);
  RAJA::forall<ExecPol>(RAJA::TypedRangeSegment<RAJA::Index_type>(0, n),
                        [=] APP_HOST_DEVICE(RAJA::Index_type i) {
                          sum += y[i];
                          mnl.minloc(x[i], i);
                        });
  r.sum = sum.get();
  r.minv = mnl.get();
  r.minloc = mnl.getLoc();
  // expt params
  double ps = 0.0;
  RAJA::expt::ValLoc<double> pm(1e300, -1);
  using SUM = RAJA::expt::ValOp<double, RAJA::operators::plus>;
  using MINL = RAJA::expt::ValLocOp<double, RAJA::Index_type, RAJA::operators::minimum>;
  RAJA::forall<ExecPol>(RAJA::TypedRangeSegment<RAJA::Index_type>(0, n),
                        RAJA::expt::Reduce<RAJA::operators::plus>(&ps),
                        RAJA::expt::Reduce<RAJA::operators::minimum>(&pm), RAJA::Name("binding params"),
                        [=] APP_HOST_DEVICE(RAJA::Index_type i, SUM & s, MINL & m) {
                          s += y[i];
                          m.minloc(x[i], i);
                        });
  r.psum = ps;
  r.pmin = pm;
  // scans
  RAJA::inclusive_scan<ExecPol>(RAJA::make_span(a, n), RAJA::make_span(b, n));
  r.incl.assign(b, b + n);
  RAJA::exclusive_scan_inplace<ExecPol>(RAJA::make_span(a, n), RAJA::operators::maximum<long long>{});
  r.excl.assign(a, a + n);
  // sorts
  RAJA::stable_sort_pairs<ExecPol>(RAJA::make_span(k, n), RAJA::make_span(v, n),
                                   RAJA::operators::greater<int>{});
  r.keys.assign(k, k + n);
  r.vals.assign(v, v + n);
  // IndexSet: a range, a list and a strided segment
  RAJA::TypedIndexSet<RAJA::TypedRangeSegment<RAJA::Index_type>, RAJA::TypedListSegment<RAJA::Index_type>,
                      RAJA::TypedRangeStrideSegment<RAJA::Index_type>>
      is;
  is.push_back(RAJA::TypedRangeSegment<RAJA::Index_type>(0, n / 4));
  std::vector<RAJA::Index_type> odd;
  for (RAJA::Index_type i = n / 2 + 1; i < n; i += 2) odd.push_back(i);
  camp::resources::Resource res = RAJA::resources::get_resource<ExecPol>::type::get_default();
  is.push_back(RAJA::TypedListSegment<RAJA::Index_type>(odd.data(), odd.size(), res));
  is.push_back(RAJA::TypedRangeStrideSegment<RAJA::Index_type>(n / 4, n / 2, 3));
  RAJA::forall<RAJA::ExecPolicy<RAJA::seq_segit, ExecPol>>(
      is, [=] APP_HOST_DEVICE(RAJA::Index_type i) { z[i] = y[i] * 2.0; });
  r.iset.assign(z, z + n);
  return r;
}
// A WorkGroup of uneven loops, each w[i] += i + 5 and a per-loop ReduceSum
// of w[i], run `runs` times; the sums are read after the group is gone (RAJA's
// host reducers fold their loop copies into the parent when the group's
// storage is destroyed).
struct WgResults {
  std::vector<long long> w, sums;
};
template <typename WorkPol, typename OrderPol, typename RedPol>
WgResults run_workgroup(long long* w, const std::vector<RAJA::Index_type>& offs, int runs)
{
  const int nloops = int(offs.size()) - 1;
  const RAJA::Index_type total = offs.back();
  for (RAJA::Index_type i = 0; i < total; ++i) w[i] = i % 13;
  using policy = RAJA::WorkGroupPolicy<WorkPol, OrderPol, RAJA::ragged_array_of_objects>;
  using pool_t = RAJA::WorkPool<policy, RAJA::Index_type, RAJA::xargs<>, std::allocator<char>>;
  std::vector<std::unique_ptr<RAJA::ReduceSum<RedPol, long long>>> sums;
  {
    pool_t pool(std::allocator<char>{});
    for (int l = 0; l < nloops; ++l) {
      sums.emplace_back(new RAJA::ReduceSum<RedPol, long long>(l));
      const RAJA::ReduceSum<RedPol, long long>& s = *sums.back();
      pool.enqueue(RAJA::TypedRangeSegment<RAJA::Index_type>(offs[l], offs[l + 1]),
                   [=] APP_HOST_DEVICE(RAJA::Index_type i) {
                     w[i] += i + 5;
                     s += w[i];
                   });
    }
    auto group = pool.instantiate();
    for (int r = 0; r < runs; ++r) group.run();
  }
  WgResults out;
  out.w.assign(w, w + total);
  for (auto& s : sums) out.sums.push_back(s->get());
  return out;
}
// MultiReduceSum over bins and per-bin counts by atomicAdd (integer-valued
// data: every order gives the same sums).
struct MultiResults {
  std::vector<double> sums;
  std::vector<int> counts;
};
template <typename ExecPol, typename MRPol, typename AtomPol>
MultiResults run_multi(const int* bins, const double* vals, int* cnt, RAJA::Index_type n, int nb)
{
  for (int b = 0; b < nb; ++b) cnt[b] = 0;
  RAJA::MultiReduceSum<MRPol, double> mr(nb, 0.5);
  RAJA::forall<ExecPol>(RAJA::TypedRangeSegment<RAJA::Index_type>(0, n),
                        [=] APP_HOST_DEVICE(RAJA::Index_type i) {
                          mr[bins[i]] += vals[i];
                          RAJA::atomicAdd<AtomPol>(cnt + bins[i], 1);
                        });
  MultiResults r;
  for (int b = 0; b < nb; ++b) r.sums.push_back(mr.get(b));
  r.counts.assign(cnt, cnt + nb);
  return r;
}
}  // namespace

int main()
{
  const RAJA::Index_type n = 100003;
  std::vector<double> x0(n);
  std::vector<int> k0(n);
  unsigned s = 12345u;
  for (RAJA::Index_type i = 0; i < n; ++i) {
    s = s * 1664525u + 1013904223u;
    x0[i] = double(s >> 8) / double(1u << 24) - 0.5;
    k0[i] = int(s % 1000u);
  }
  std::vector<double> hx(n), hy(n), hz(n);
  std::vector<long long> ha(n), hb(n);
  std::vector<int> hk(n), hv(n);
  auto seq = run<RAJA::seq_exec, RAJA::seq_reduce>(x0, k0, hx.data(), hy.data(), ha.data(), hb.data(),
                                                    hk.data(), hv.data(), hz.data());
  std::printf("seq_exec: sum %.17g, minloc %.17g at %ld\n", seq.sum, seq.minv, (long)seq.minloc);
  std::vector<RAJA::Index_type> offs(1, 0);
  for (int l = 0; l < 37; ++l) offs.push_back(offs.back() + 17 + (l * 7919) % 4000);
  std::vector<long long> hw(offs.back());
  auto wseq = run_workgroup<RAJA::seq_work, RAJA::ordered, RAJA::seq_reduce>(hw.data(), offs, 3);
  const int nb = 37;
  std::vector<int> hbins(n), hcnt(nb);
  std::vector<double> hvals(n);
  for (RAJA::Index_type i = 0; i < n; ++i) {
    hbins[i] = int((i * 2654435761u) % nb);
    hvals[i] = double(int(i % 9) - 4);
  }
  auto mseq = run_multi<RAJA::seq_exec, RAJA::seq_multi_reduce, RAJA::seq_atomic>(hbins.data(), hvals.data(),
                                                                                  hcnt.data(), n, nb);

  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    std::printf("no CUDA device: b200 half not run (the program compiled and linked)\n");
    return failures ? 1 : 0;
  }
  double *x, *y, *z;
  long long *a, *b;
  int *k, *v;
  cudaMallocManaged(&x, n * sizeof(double));
  cudaMallocManaged(&y, n * sizeof(double));
  cudaMallocManaged(&z, n * sizeof(double));
  cudaMallocManaged(&a, n * sizeof(long long));
  cudaMallocManaged(&b, n * sizeof(long long));
  cudaMallocManaged(&k, n * sizeof(int));
  cudaMallocManaged(&v, n * sizeof(int));
  auto dev = run<RAJA::b200_exec<256>, RAJA::b200_reduce>(x0, k0, x, y, a, b, k, v, z);
  cudaDeviceSynchronize();
  // the same application with its launch shape tuned on line (BLOCK 0),
  // run enough times for the tuners to cycle through their shapes
  int *mbins = nullptr, *mcnt = nullptr;
  double* mvals = nullptr;
  cudaMallocManaged(&mbins, n * sizeof(int));
  cudaMallocManaged(&mvals, n * sizeof(double));
  cudaMallocManaged(&mcnt, nb * sizeof(int));
  std::copy(hbins.begin(), hbins.end(), mbins);
  std::copy(hvals.begin(), hvals.end(), mvals);
  auto mdev = run_multi<RAJA::b200_exec<256>, RAJA::b200_multi_reduce, RAJA::b200_atomic>(mbins, mvals, mcnt, n, nb);
  check(mdev.sums == mseq.sums && mdev.counts == mseq.counts,
        "MultiReduceSum<b200_multi_reduce> and atomicAdd<b200_atomic>");
  cudaFree(mbins);
  cudaFree(mvals);
  cudaFree(mcnt);
  long long* w = nullptr;
  cudaMallocManaged(&w, offs.back() * sizeof(long long));
  auto wdev = run_workgroup<RAJA::b200_work<256>, RAJA::b200_unordered, RAJA::b200_reduce>(w, offs, 3);
  auto word = run_workgroup<RAJA::b200_work<256>, RAJA::ordered, RAJA::b200_reduce>(w, offs, 3);
  auto wtun = run_workgroup<RAJA::b200_work<0>, RAJA::b200_unordered, RAJA::b200_reduce>(w, offs, 3);
  check(wdev.w == wseq.w && wdev.sums == wseq.sums,
        "WorkGroup<b200_work<256>, b200_unordered> with ReduceSum<b200_reduce> per loop");
  check(word.w == wseq.w && word.sums == wseq.sums, "WorkGroup<b200_work<256>, ordered>");
  check(wtun.w == wseq.w && wtun.sums == wseq.sums, "WorkGroup<b200_work<0>, b200_unordered> (tuned tiles)");
  cudaFree(w);
  bool tuned_ok = true;
  for (int rep = 0; rep < 30; ++rep) {
    auto t = run<RAJA::b200_exec<0>, RAJA::b200_reduce>(x0, k0, x, y, a, b, k, v, z);
    cudaDeviceSynchronize();
    tuned_ok = tuned_ok && t.incl == dev.incl && t.excl == dev.excl && t.keys == dev.keys && t.vals == dev.vals &&
               t.iset == dev.iset && t.minv == dev.minv && t.minloc == dev.minloc;
  }
  double tol = 4.0 * n * 1.1102230246251565e-16 * 4.0 * n;
  bool y_ok = true;
  for (RAJA::Index_type i = 0; i < n; ++i)
    y_ok = y_ok && std::fabs(dev.iset[i] - seq.iset[i]) <= 4e-16 * std::fabs(seq.iset[i]) + 1e-300;
  check(std::fabs(dev.sum - seq.sum) <= tol, "ReduceSum<b200_reduce>");
  check(dev.minv == seq.minv && dev.minloc == seq.minloc, "ReduceMinLoc<b200_reduce> (value, first index)");
  check(std::fabs(dev.psum - seq.psum) <= tol, "expt::Reduce<plus> on b200_exec");
  check(dev.pmin.getVal() == seq.pmin.getVal() && dev.pmin.getLoc() == seq.pmin.getLoc(),
        "expt::Reduce<minimum> over ValLoc on b200_exec");
  check(dev.incl == seq.incl, "inclusive_scan<b200_exec>");
  check(dev.excl == seq.excl, "exclusive_scan_inplace<b200_exec>(maximum)");
  check(dev.keys == seq.keys && dev.vals == seq.vals, "stable_sort_pairs<b200_exec>(greater)");
  check(y_ok, "forall over an IndexSet (range + list + strided) on ExecPolicy<seq_segit, b200_exec>");
  check(tuned_ok, "the same application on b200_exec<0> (launch shape tuned on line)");
  return failures ? 1 : 0;
}
