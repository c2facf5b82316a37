// Fixed-type forall bodies: y[i] += a * x[i].
//
// Reference: forallp_cuda_kernel (policy/cuda/forall.hpp:371-542) launched
// by forall_impl (:554-655) with grid = ceil(N / BLOCK) and one element per
// thread.  Here a persistent grid (SM count x resident blocks) walks the
// range in 16-byte vectors, four independent vectors per thread per step,
// so each SM keeps enough loads in flight to saturate HBM3e.  Arbitrary
// lambda bodies use the templated b200_exec policy (include/raja_b200).
#include "b200_internal.cuh"

namespace b200 {
namespace {

constexpr int FBLOCK = 256;
constexpr int FUNROLL = 4;

template <class T>
__global__ void __launch_bounds__(FBLOCK)
axpy_kernel(T a, const T* __restrict__ x, T* __restrict__ y, size_t n, int vec_ok) {
  constexpr int VN = 16 / sizeof(T);
  const size_t tid = size_t(blockIdx.x) * FBLOCK + threadIdx.x;
  const size_t nthreads = size_t(gridDim.x) * FBLOCK;
  size_t done = 0;
  if (vec_ok) {
    const size_t nvec = n / VN;
    const size_t step = nthreads * FUNROLL;
    size_t v = tid;
    for (; v + (FUNROLL - 1) * nthreads < nvec; v += step) {
      Vec16<T> vx[FUNROLL], vy[FUNROLL];
#pragma unroll
      for (int u = 0; u < FUNROLL; ++u) {
        vx[u] = ld_vec_stream(x + (v + u * nthreads) * VN);
        vy[u] = ld_vec_stream(y + (v + u * nthreads) * VN);
      }
#pragma unroll
      for (int u = 0; u < FUNROLL; ++u) {
#pragma unroll
        for (int k = 0; k < VN; ++k) vy[u].v[k] += a * vx[u].v[k];
        st_vec_stream(y + (v + u * nthreads) * VN, vy[u]);
      }
    }
    for (; v < nvec; v += nthreads) {
      Vec16<T> vx = ld_vec_stream(x + v * VN), vy = ld_vec_stream(y + v * VN);
#pragma unroll
      for (int k = 0; k < VN; ++k) vy.v[k] += a * vx.v[k];
      st_vec_stream(y + v * VN, vy);
    }
    done = nvec * VN;
  }
  for (size_t i = done + tid; i < n; i += nthreads) y[i] += a * x[i];
}

template <class T>
int run_axpy(const char* name, T a, const T* x, T* y, size_t n, b200_stream_t stream) {
  if (n == 0) return B200_OK;
  if (!x || !y) return fail(B200_ERR_ARG, "%s: null pointer", name);
  static KernelSetup ks;
  DeviceProps p;
  B200_TRY(device_props(&p));
  int bps = 0;
  B200_TRY(kernel_setup(ks, p, axpy_kernel<T>, FBLOCK, 0, &bps));
  const bool vec_ok = reinterpret_cast<uintptr_t>(x) % 16 == 0 &&
                      reinterpret_cast<uintptr_t>(y) % 16 == 0;
  const size_t work = vec_ok ? (n * sizeof(T) + 15) / 16 : n;
  size_t grid = size_t(p.sms) * bps;
  const size_t need = (work + FBLOCK - 1) / FBLOCK;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  B200_LAUNCH(name, axpy_kernel<T>, int(grid), FBLOCK, 0, s, a, x, y, n, int(vec_ok));
  clear_error();
  return B200_OK;
}

}  // namespace
}  // namespace b200

extern "C" {
int b200_forall_axpy_f64(double a, const double* x, double* y, size_t n, b200_stream_t s) {
  return b200::run_axpy<double>("b200_forall_axpy_f64", a, x, y, n, s);
}
int b200_forall_axpy_f32(float a, const float* x, float* y, size_t n, b200_stream_t s) {
  return b200::run_axpy<float>("b200_forall_axpy_f32", a, x, y, n, s);
}
}
