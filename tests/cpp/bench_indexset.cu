// Timing of forall over an IndexSet of many uneven segments on the b200
// policies: one launch for the whole IndexSet (ExecPolicy<seq_segit,
// b200_exec>) against one launch per segment, the reference's CUDA
// schedule (policy/cuda/forall.hpp:675-706).  10,000 segments with
// Pareto(alpha 1.5) lengths (32 and up, at most 2^20), body y[i] += a x[i]
// on doubles; all-range sets and sets mixing range, strided and list
// segments.  Prints one JSON object; bench.py builds and runs it.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <functional>
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
  std::printf("{\"segments\": %d, \"elements\": %lld, \"reps\": %d, "
              "\"ranges_one_launch_ms\": %.4f, \"ranges_per_segment_ms\": %.4f, \"ranges_speedup\": %.2f, "
              "\"ranges_one_launch_gbs\": %.1f, "
              "\"mixed_one_launch_ms\": %.4f, \"mixed_per_segment_ms\": %.4f, \"mixed_speedup\": %.2f, "
              "\"mixed_one_launch_gbs\": %.1f, \"results_equal\": %s}\n",
              nseg, (long long)total, reps, r_one, r_per, r_per / r_one, bytes / r_one / 1e6, m_one, m_per,
              m_per / m_one, bytes / m_one / 1e6, same ? "true" : "false");
  return same ? 0 : 1;
}
