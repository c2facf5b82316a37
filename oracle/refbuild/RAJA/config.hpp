// Hand-written RAJA configuration for building the reference's host
// policies (sequential and OpenMP) with g++ -- test infrastructure only.
//
// RAJA's CMake normally generates RAJA/config.hpp from a template.  This
// file stands in for it: it sits first on the include path and gives the
// macro values of a GCC host build with OpenMP enabled and every device
// back-end (CUDA, HIP, SYCL, OpenMP target) disabled.  It defines only the
// configuration switches and helper macros the included RAJA headers test
// for; nothing here changes RAJA's algorithms.
#ifndef RAJA_config_HPP
#define RAJA_config_HPP

#include <cstddef>
#include <type_traits>
#include <utility>

#define RAJA_CXX_VER __cplusplus
#define RAJA_HAS_SOME_CXX14 1
#if defined(__cpp_lib_is_invocable) && (__cpp_lib_is_invocable >= 201703L)
#define RAJA_HAS_CXX17_IS_INVOCABLE 1
#else
#define RAJA_HAS_CXX17_IS_INVOCABLE 0
#endif

// floating-point and pointer flavours of the default build
#define RAJA_USE_DOUBLE
#define RAJA_USE_RESTRICT_PTR

// back-ends: host sequential and OpenMP only
#if defined(_OPENMP)
#define RAJA_ENABLE_OPENMP
#endif
#define RAJA_CUDA_WARPSIZE 32
#define RAJA_USE_CHRONO

#if defined(__clang__)
#define RAJA_COMPILER_CLANG
#elif defined(__GNUC__)
#define RAJA_COMPILER_GNU
#endif

#define RAJA_STRINGIFY_HELPER(...) #__VA_ARGS__
#define RAJA_STRINGIFY(...) RAJA_STRINGIFY_HELPER(__VA_ARGS__)
#define RAJA_PRAGMA(x) _Pragma(RAJA_STRINGIFY(x))

#define RAJA_VERSION_MAJOR 2025
#define RAJA_VERSION_MINOR 9
#define RAJA_VERSION_PATCHLEVEL 1

namespace RAJA
{
const int DATA_ALIGN = 64;
}

#define RAJA_RESTRICT __restrict__
#define RAJA_COLLAPSE(X) collapse(X)
#define RAJA_BOUNDS_CHECK_constexpr constexpr
#define RAJASHAREDDLL_API
#define RAJA_ALIGNED_ATTR(N) __attribute__((aligned(N)))
#define RAJA_MAX_ALIGN 16
#define RAJA_FORCEINLINE_RECURSIVE
#define RAJA_INLINE inline __attribute__((always_inline))
#if defined(__clang__)
#define RAJA_UNROLL RAJA_PRAGMA(clang loop unroll(enable))
#define RAJA_UNROLL_COUNT(N) RAJA_PRAGMA(clang loop unroll_count(N))
#else
#define RAJA_UNROLL RAJA_PRAGMA(GCC unroll 10000)
#define RAJA_UNROLL_COUNT(N) RAJA_PRAGMA(GCC unroll N)
#endif
#define RAJA_ALIGN_DATA(d) __builtin_assume_aligned(d, RAJA::DATA_ALIGN)
#if defined(_OPENMP)
#define RAJA_SIMD RAJA_PRAGMA(omp simd)
#else
#define RAJA_SIMD RAJA_PRAGMA(GCC ivdep)
#endif
#define RAJA_HAVE_POSIX_MEMALIGN

namespace RAJA
{
template <typename T>
RAJA_INLINE T* align_hint(T* x)
{
  return static_cast<T*>(RAJA_ALIGN_DATA(x));
}
}  // namespace RAJA

#endif
