// Timing of the batched forms through the RAJA API on the b200 policies.
//
// IndexSet: forall over 10,000 segments with Pareto(alpha 1.5) lengths (32
// and up, at most 2^20), body y[i] += a x[i] on doubles; one launch for the
// whole IndexSet (ExecPolicy<seq_segit, b200_exec>) against one launch per
// segment, the reference's CUDA schedule (policy/cuda/forall.hpp:675-706);
// all-range sets and sets mixing range, strided and list segments.
//
// WorkGroup: 4096 loops with lognormal lengths (median 2000, sigma 1.5,
// clipped to [32, 2^20]), each y[i] += a x[i] on floats plus a per-loop
// ReduceSum<b200_reduce, float>; one run() of an unordered group (one
// launch, reducers combined inside it) with the fixed shape b200_work<256>
// and with the tuned shape b200_work<0>, against an ordered group (one
// launch per loop, the reference's ordered CUDA runner,
// policy/cuda/WorkGroup/WorkRunner.hpp:38-162).  Each run() returns after
// its work is done (synchronous policy); the tuned shape is also timed with
// the asynchronous policy b200_work<0, true>, whose runs queue behind one
// another, which gives the device time of a run.
//
// Prints one JSON object; bench.py builds and runs it.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <functional>
#include <memory>
#include <random>
#include <vector>

#include "RAJA/RAJA.hpp"
#include "raja_b200/RAJA_b200.hpp"

using Index_type = RAJA::Index_type;

namespace {
float time_ms(int reps, const std::function<void()>& f) {
  f();
  cudaDeviceSynchronize();
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, RAJA::b200::stream());
  for (int r = 0; r < reps; ++r) f();
  cudaEventRecord(b, RAJA::b200::stream());
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / reps;
}
}  // namespace

// One WorkGroup variant: build the pool (4096 reducers), run `warm` times,
// then time `reps` runs.  Returns ms per run; the per-loop sums of all runs
// and the final y go to the caller.
template <class WPOL, class ORDER>
float workgroup_ms(const std::vector<Index_type>& offs, const float* x, float* y, int warm, int reps,
                   std::vector<double>* sums, RAJA::b200::tune::Report* tuning) {
  using pool_t = RAJA::WorkPool<RAJA::WorkGroupPolicy<WPOL, ORDER>, Index_type>;
  using red_t = RAJA::ReduceSum<RAJA::b200_reduce, float>;
  const int nloops = int(offs.size()) - 1;
  std::vector<std::unique_ptr<red_t>> red;
  pool_t pool;
  const float a = 1e-3f;
  for (int l = 0; l < nloops; ++l) {
    red.emplace_back(new red_t(0.0f));
    const red_t& s = *red.back();
    pool.enqueue(RAJA::RangeSegment(offs[l], offs[l + 1]), [=] RAJA_DEVICE(Index_type i) {
      y[i] += a * x[i];
      s += y[i];
    });
  }
  auto g = pool.instantiate();
  for (int w = 0; w < warm; ++w) g.run();
  const float ms = time_ms(reps, [&] { g.run(); });
  sums->assign(nloops, 0.0);
  for (int l = 0; l < nloops; ++l) (*sums)[l] = red[l]->get();
  *tuning = g.tuning();
  return ms;
}

int main() {
  const int nseg = 10000;
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  std::vector<Index_type> lens(nseg);
  Index_type total = 0;
  for (int i = 0; i < nseg; ++i) {
    double l = std::floor(32.0 * std::pow(1.0 - u(rng), -1.0 / 1.5));
    lens[i] = Index_type(l > double(1 << 20) ? double(1 << 20) : l);
    total += lens[i];
  }
  // every segment covers its own block of 2 * len elements; range segments
  // take the first half, strided ones every other element, lists the
  // second half in reverse
  double *x = nullptr, *y = nullptr, *y2 = nullptr;
  Index_type* lists = nullptr;
  cudaMallocManaged(&x, 2 * total * sizeof(double));
  cudaMallocManaged(&y, 2 * total * sizeof(double));
  cudaMallocManaged(&y2, 2 * total * sizeof(double));
  cudaMallocManaged(&lists, total * sizeof(Index_type));
  for (Index_type i = 0; i < 2 * total; ++i) {
    x[i] = double(i % 97) / 8.0;
    y[i] = y2[i] = 1.0;
  }
  using R = RAJA::TypedRangeSegment<Index_type>;
  using S = RAJA::TypedRangeStrideSegment<Index_type>;
  using L = RAJA::TypedListSegment<Index_type>;
  RAJA::TypedIndexSet<R> ranges;
  RAJA::TypedIndexSet<R, S, L> mixed;
  Index_type base = 0, lpos = 0;
  std::vector<int> kind(nseg);
  for (int i = 0; i < nseg; ++i) {
    const Index_type n = lens[i];
    ranges.push_back(R(base, base + n));
    kind[i] = i % 3;
    if (kind[i] == 0) {
      mixed.push_back(R(base, base + n));
    } else if (kind[i] == 1) {
      mixed.push_back(S(base, base + 2 * n, 2));
    } else {
      for (Index_type k = 0; k < n; ++k) lists[lpos + k] = base + 2 * n - 1 - k;
      mixed.push_back(L(lists + lpos, n));
      lpos += n;
    }
    base += 2 * n;
  }
  cudaMemPrefetchAsync(x, 2 * total * sizeof(double), cudaMemLocation{cudaMemLocationTypeDevice, 0}, 0);
  cudaMemPrefetchAsync(y, 2 * total * sizeof(double), cudaMemLocation{cudaMemLocationTypeDevice, 0}, 0);
  cudaMemPrefetchAsync(y2, 2 * total * sizeof(double), cudaMemLocation{cudaMemLocationTypeDevice, 0}, 0);
  cudaMemPrefetchAsync(lists, total * sizeof(Index_type), cudaMemLocation{cudaMemLocationTypeDevice, 0}, 0);
  cudaDeviceSynchronize();
  const double a = 0.25;
  using one_launch = RAJA::ExecPolicy<RAJA::seq_segit, RAJA::b200_exec_async<256>>;
  using per_seg = RAJA::b200_exec_async<256>;
  auto body = [=] __device__(Index_type i) { y[i] += a * x[i]; };
  auto body2 = [=] __device__(Index_type i) { y2[i] += a * x[i]; };
  const int reps = 5;
  // all-range IndexSet
  const float r_one = time_ms(reps, [&] { RAJA::forall<one_launch>(ranges, body); });
  const float r_per = time_ms(reps, [&] {
    for (const auto& v : ranges.segments()) std::visit([&](const auto& g) { RAJA::forall<per_seg>(g, body2); }, v);
  });
  // mixed IndexSet
  const float m_one = time_ms(reps, [&] { RAJA::forall<one_launch>(mixed, body); });
  const float m_per = time_ms(reps, [&] {
    for (const auto& v : mixed.segments()) std::visit([&](const auto& g) { RAJA::forall<per_seg>(g, body2); }, v);
  });
  cudaDeviceSynchronize();
  bool same = true;
  for (Index_type i = 0; i < 2 * total; ++i) same = same && (y[i] == y2[i]);
  const double bytes = 24.0 * double(total);  // read x, read + write y per element

  // ---- WorkGroup
  const int nloops = 4096;
  std::mt19937_64 wrng(11);
  std::lognormal_distribution<double> ln(std::log(2000.0), 1.5);
  std::vector<Index_type> offs(nloops + 1, 0);
  for (int l = 0; l < nloops; ++l) {
    double v = std::round(ln(wrng));
    v = v < 32 ? 32 : (v > double(1 << 20) ? double(1 << 20) : v);
    offs[l + 1] = offs[l] + Index_type(v);
  }
  const Index_type wtotal = offs[nloops];
  float *wx = nullptr, *wy[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaMalloc(&wx, wtotal * sizeof(float));
  std::vector<float> hx(wtotal), hy(wtotal);
  for (Index_type i = 0; i < wtotal; ++i) {
    hx[i] = float(u(wrng) * 2.0 - 1.0);
    hy[i] = float(u(wrng) * 2.0 - 1.0);
  }
  cudaMemcpy(wx, hx.data(), wtotal * sizeof(float), cudaMemcpyHostToDevice);
  for (auto& p : wy) {
    cudaMalloc(&p, wtotal * sizeof(float));
    cudaMemcpy(p, hy.data(), wtotal * sizeof(float), cudaMemcpyHostToDevice);
  }
  const int warm = 40, wreps = 20;
  std::vector<double> s_ord, s_fix, s_tun, s_asy;
  RAJA::b200::tune::Report t_ord, t_fix, t_tun, t_asy;
  const float w_ord = workgroup_ms<RAJA::b200_work<256>, RAJA::ordered>(offs, wx, wy[0], 3, 5, &s_ord, &t_ord);
  const float w_fix =
      workgroup_ms<RAJA::b200_work<256>, RAJA::unordered>(offs, wx, wy[1], warm, wreps, &s_fix, &t_fix);
  const float w_tun =
      workgroup_ms<RAJA::b200_work<0>, RAJA::unordered>(offs, wx, wy[2], warm, wreps, &s_tun, &t_tun);
  const float w_asy =
      workgroup_ms<RAJA::b200_work<0, true>, RAJA::unordered>(offs, wx, wy[3], warm, wreps, &s_asy, &t_asy);
  // the three groups ran different numbers of times: compare y and the sums
  // only between the two unordered groups (same runs), and check y of the
  // ordered group against a host restatement of its runs (3 warm-up, one
  // untimed and 5 timed)
  std::vector<float> wy0(wtotal), wy1(wtotal), wy2(wtotal), wy3(wtotal);
  cudaMemcpy(wy0.data(), wy[0], wtotal * sizeof(float), cudaMemcpyDeviceToHost);
  cudaMemcpy(wy1.data(), wy[1], wtotal * sizeof(float), cudaMemcpyDeviceToHost);
  cudaMemcpy(wy2.data(), wy[2], wtotal * sizeof(float), cudaMemcpyDeviceToHost);
  cudaMemcpy(wy3.data(), wy[3], wtotal * sizeof(float), cudaMemcpyDeviceToHost);
  bool wy_equal = wy1 == wy2 && wy1 == wy3;
  bool wy0_ok = true;
  for (Index_type i = 0; i < wtotal && wy0_ok; ++i) {
    float v = hy[i];
    for (int r = 0; r < 3 + 1 + 5; ++r) v = std::fma(1e-3f, hx[i], v);
    wy0_ok = v == wy0[i];
  }
  double sum_rel = 0.0;
  for (int l = 0; l < nloops; ++l) {
    for (const std::vector<double>* o : {&s_tun, &s_asy}) {
      const double d = std::fabs(s_fix[l] - (*o)[l]) / (std::fabs(s_fix[l]) + 1e-30);
      sum_rel = d > sum_rel ? d : sum_rel;
    }
  }
  const double wbytes = 12.0 * double(wtotal);  // read x, read + write y per element
  std::printf("{\"segments\": %d, \"elements\": %lld, \"reps\": %d, "
              "\"ranges_one_launch_ms\": %.4f, \"ranges_per_segment_ms\": %.4f, \"ranges_speedup\": %.2f, "
              "\"ranges_one_launch_gbs\": %.1f, "
              "\"mixed_one_launch_ms\": %.4f, \"mixed_per_segment_ms\": %.4f, \"mixed_speedup\": %.2f, "
              "\"mixed_one_launch_gbs\": %.1f, \"results_equal\": %s, "
              "\"workgroup_loops\": %d, \"workgroup_elements\": %lld, "
              "\"workgroup_ordered_per_loop_ms\": %.4f, \"workgroup_unordered_b200_work_256_ms\": %.4f, "
              "\"workgroup_unordered_tuned_ms\": %.4f, \"workgroup_tuned_shape\": [%d, %d], "
              "\"workgroup_tuner_settled\": %s, \"workgroup_tuned_gbs\": %.1f, "
              "\"workgroup_unordered_tuned_async_ms\": %.4f, \"workgroup_async_shape\": [%d, %d], "
              "\"workgroup_async_gbs\": %.1f, "
              "\"workgroup_speedup_tuned_vs_ordered\": %.1f, \"workgroup_y_equal\": %s, "
              "\"workgroup_ordered_y_exact\": %s, \"workgroup_sums_max_rel_diff_fixed_vs_tuned\": %.3g}\n",
              nseg, (long long)total, reps, r_one, r_per, r_per / r_one, bytes / r_one / 1e6, m_one, m_per,
              m_per / m_one, bytes / m_one / 1e6, same ? "true" : "false", nloops, (long long)wtotal, w_ord, w_fix,
              w_tun, t_tun.best.block, t_tun.best.items, t_tun.settled ? "true" : "false",
              wbytes / w_tun / 1e6, w_asy, t_asy.best.block, t_asy.best.items, wbytes / w_asy / 1e6, w_ord / w_tun, wy_equal ? "true" : "false", wy0_ok ? "true" : "false", sum_rel);
  return (same && wy_equal && wy0_ok) ? 0 : 1;
}
