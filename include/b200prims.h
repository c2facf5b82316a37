/*
 * b200prims.h -- C ABI of the GB300 (sm_103a) data-parallel primitive library
 * (libb200prims.so).
 *
 * This is the drop-in boundary that replaces RAJA's CUDA back-end for the
 * fixed-type primitives of its data-parallel path.  Every entry point below
 * names the reference interface it stands in for (paths are relative to the
 * RAJA v2025.09.1 source tree).  The templated C++ layer in
 * include/raja_b200/ (the b200_exec / b200_reduce / b200_work policies) and
 * the Python host mirror (raja_gb300) both call these functions.
 *
 * Conventions
 *   - Plain pointers and sizes only.  All data pointers are device-accessible
 *     (cudaMalloc'd, managed, or mapped pinned memory).  Results of reductions
 *     are written by the device into `out*` pointers, which must also be
 *     device-accessible.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *     Every call is stream-ordered and returns once the work is enqueued; call
 *     b200_stream_synchronize() to wait and to collect device-side errors.
 *   - Every function returns an int status (B200_OK == 0).  Nothing aborts or
 *     throws across this boundary; b200_last_error_string() explains the last
 *     failure on the calling host thread.
 *   - Element counts are size_t.  The reference scans and sorts use an `int`
 *     length (policy/cuda/scan.hpp:163, policy/cuda/sort.hpp:115); this
 *     library accepts any n < 2^40 for scans and reductions and n < 2^32 for
 *     sorts.
 */
#ifndef B200PRIMS_H
#define B200PRIMS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define B200_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------
 * Replace the reference's error paths: CUDA API failures raised as
 * std::runtime_error by CAMP_CUDA_API_INVOKE_AND_CHECK
 * (policy/cuda/raja_cudaerrchk.hpp:116-137) and RAJA_ABORT_OR_THROW for bad
 * launch geometry (util/macros.hpp:143-152).                              */
#define B200_OK 0
#define B200_ERR_ARG 1         /* invalid argument (size, op, alignment)   */
#define B200_ERR_CUDA 2        /* a CUDA runtime call failed                */
#define B200_ERR_TIMEOUT 3     /* a bounded device wait gave up             */
#define B200_ERR_NOMEM 4       /* scratch allocation failed                 */
#define B200_ERR_UNSUPPORTED 5 /* type/op combination not provided          */

/* ---- reduction modes (bit flags) ---------------------------------------
 * NAIVE: accumulate in the element type, like cuda_reduce
 *        (policy/cuda/reduce.hpp:133-214).
 * COMPENSATED: per-thread two-sum (Neumaier) accumulation in the element
 *        type, cross-block combine in FP64 (FP32 inputs) or double-double
 *        (FP64 inputs).  Affects floating-point sums, dots and scans only.
 * DETERMINISTIC: fixed-size chunks and a fixed combine tree, so the result
 *        depends only on (n, data) and not on the grid or the GPU.        */
#define B200_MODE_NAIVE 0
#define B200_MODE_COMPENSATED 1
#define B200_MODE_DETERMINISTIC 2

/* ---- scan operators (RAJA::operators::plus/minimum/maximum,
 *      util/Operators.hpp:363-372, 555-591)                              */
#define B200_OP_SUM 0
#define B200_OP_MIN 1
#define B200_OP_MAX 2

typedef void* b200_stream_t;

/* ======================================================================
 * Runtime (replaces MemUtils_CUDA.hpp:69-284 pools/launch/sync glue and
 * src/MemUtils_CUDA.cpp:44-53 globals)
 * ====================================================================== */

/* ABI version of the loaded library (== B200_ABI_VERSION). */
int b200_abi_version(void);

/* Message for the last failing call on this host thread ("" if none). */
const char* b200_last_error_string(void);

/* Wait for `stream`, then read and clear the status word of the current
 * device.  Returns B200_ERR_TIMEOUT if a bounded device wait (scan or sort
 * look-back) gave up since the last check.  Work queued on other streams is
 * not waited for; the word itself is shared by all streams of the device.
 * It lives in mapped pinned host memory, so the check costs no copy.
 * Replaces cuda::synchronize / res.wait() (MemUtils_CUDA.hpp:205-247). */
int b200_stream_synchronize(b200_stream_t stream);

/* Host address of the current device's status word (a uint32_t in mapped
 * pinned memory that is 0 while no bounded device wait has given up).  A
 * caller that synchronises a stream itself reads it afterwards instead of
 * calling b200_stream_synchronize(); on a non-zero value,
 * b200_stream_synchronize() reports and clears it. */
int b200_status_word_address(const uint32_t** out);

/* Test hook: upper bound on polling iterations of every device-side wait
 * (0 restores the default).  Used to exercise the timeout path without a
 * GPU fault (the reference spins without a bound, reduce.hpp:425-426). */
int b200_set_spin_limit(uint64_t limit);

/* Test hook: launch one scan tile whose predecessor never publishes, so its
 * bounded look-back must give up; the next b200_stream_synchronize() on
 * `stream` returns B200_ERR_TIMEOUT.  Exercises the failure path without a
 * GPU fault, trap or hang. */
int b200_selftest_scan_timeout(b200_stream_t stream);

/* Device properties the launch heuristics use (current device). */
int b200_device_info(int* sm_count, int* cc_major, int* cc_minor);

/* Release the scratch arenas held for every stream of the current device. */
int b200_release_scratch(void);

/* Kernel timing instrumentation: when enabled, every library kernel launch
 * is bracketed by CUDA events on its stream; b200_prof_read() accumulates
 * per-kernel launch counts and total milliseconds (read after a sync).
 * Returns the number of kernel names written (at most `cap`). */
int b200_prof_enable(int enable);
int b200_prof_reset(void);
int b200_prof_read(char* names, size_t name_stride, uint64_t* launches,
                   double* total_ms, int cap);

/* ======================================================================
 * forall -- fixed-type bodies of the RAJA::forall hot loop
 * (policy/cuda/forall.hpp:371-655, kernel forallp_cuda_kernel).  Arbitrary
 * lambda bodies go through the templated b200_exec policy in
 * include/raja_b200/RAJA_b200.hpp; these entry points cover the fixed
 * daxpy / fp32 axpy loop bodies.
 * ====================================================================== */

/* y[i] += a * x[i]  for i in [0, n) */
int b200_forall_axpy_f64(double a, const double* x, double* y, size_t n,
                         b200_stream_t stream);
int b200_forall_axpy_f32(float a, const float* x, float* y, size_t n,
                         b200_stream_t stream);

/* ======================================================================
 * Reducers -- ReduceSum / ReduceMin / ReduceMax / ReduceMinLoc /
 * ReduceMaxLoc / ReduceBitOr / ReduceBitAnd over a contiguous array
 * (policy/cuda/reduce.hpp:968-1378; last-block combine :133-214;
 * expt::Reduce params policy/cuda/params/reduce.hpp:21-62).
 *
 * Results are the reduction of x[0..n) alone (the identity when n == 0):
 * the reducer's init value is folded in by the caller, as RAJA's host-side
 * final combine does (reduce.hpp:1128-1149).
 * Sum output type is the accumulator type: double for f32/f64 inputs,
 * the element type (two's-complement wrap-around) for integers.
 * MinLoc/MaxLoc break ties by the lowest index, which reproduces seq_exec's
 * first-wins rule (util/Operators.hpp:555-591); plain Min/Max do the same
 * internally so that +0.0/-0.0 ties are bit-identical to seq_exec.
 * ====================================================================== */

int b200_reduce_sum_f32(const float* x, size_t n, int mode, double* out,
                        b200_stream_t stream);
int b200_reduce_sum_f64(const double* x, size_t n, int mode, double* out,
                        b200_stream_t stream);
int b200_reduce_sum_i32(const int32_t* x, size_t n, int mode, int32_t* out,
                        b200_stream_t stream);
int b200_reduce_sum_i64(const int64_t* x, size_t n, int mode, int64_t* out,
                        b200_stream_t stream);
int b200_reduce_sum_u32(const uint32_t* x, size_t n, int mode, uint32_t* out,
                        b200_stream_t stream);
int b200_reduce_sum_u64(const uint64_t* x, size_t n, int mode, uint64_t* out,
                        b200_stream_t stream);

/* dot = sum_i x[i]*y[i]  (ReduceSum of products; the daxpy/dot and the
 * ill-conditioned fp32 accuracy workloads) */
int b200_dot_f32(const float* x, const float* y, size_t n, int mode,
                 double* out, b200_stream_t stream);
int b200_dot_f64(const double* x, const double* y, size_t n, int mode,
                 double* out, b200_stream_t stream);

int b200_reduce_min_f32(const float* x, size_t n, float* out, b200_stream_t stream);
int b200_reduce_min_f64(const double* x, size_t n, double* out, b200_stream_t stream);
int b200_reduce_min_i32(const int32_t* x, size_t n, int32_t* out, b200_stream_t stream);
int b200_reduce_min_i64(const int64_t* x, size_t n, int64_t* out, b200_stream_t stream);
int b200_reduce_min_u32(const uint32_t* x, size_t n, uint32_t* out, b200_stream_t stream);
int b200_reduce_min_u64(const uint64_t* x, size_t n, uint64_t* out, b200_stream_t stream);
int b200_reduce_max_f32(const float* x, size_t n, float* out, b200_stream_t stream);
int b200_reduce_max_f64(const double* x, size_t n, double* out, b200_stream_t stream);
int b200_reduce_max_i32(const int32_t* x, size_t n, int32_t* out, b200_stream_t stream);
int b200_reduce_max_i64(const int64_t* x, size_t n, int64_t* out, b200_stream_t stream);
int b200_reduce_max_u32(const uint32_t* x, size_t n, uint32_t* out, b200_stream_t stream);
int b200_reduce_max_u64(const uint64_t* x, size_t n, uint64_t* out, b200_stream_t stream);

/* Allocation-free variant of b200_reduce_sum_f64 for callers that cannot
 * let a library allocate device memory (a host whose own memory manager
 * owns all of the GPU's memory; a latency-critical loop that cannot afford
 * allocator calls).  It has no counterpart in the reference.  Its scratch
 * is one static 128 KB device array per GPU, resident until the process
 * exits: it calls no cudaMalloc or cudaFree.  The first call on a device
 * looks up that array's device address (make that first call before any
 * stream capture).  Deterministic mode accepts n <= 16,777,216 and returns
 * B200_ERR_ARG beyond; the other modes take any n.  All calls on a device
 * share the array, so calls that overlap on the GPU race. */
int b200_reduce_sum_f64_noalloc(const double* x, size_t n, int mode, double* out,
                                b200_stream_t stream);

/* (value, index) of the minimum / maximum; identity (n == 0) is
 * (+max / lowest, -1) like ValueLoc (pattern/detail/reduce.hpp:127-179). */
int b200_reduce_minloc_f32(const float* x, size_t n, float* val, int64_t* idx,
                           b200_stream_t stream);
int b200_reduce_minloc_f64(const double* x, size_t n, double* val, int64_t* idx,
                           b200_stream_t stream);
int b200_reduce_minloc_i32(const int32_t* x, size_t n, int32_t* val, int64_t* idx,
                           b200_stream_t stream);
int b200_reduce_minloc_i64(const int64_t* x, size_t n, int64_t* val, int64_t* idx,
                           b200_stream_t stream);
int b200_reduce_maxloc_f32(const float* x, size_t n, float* val, int64_t* idx,
                           b200_stream_t stream);
int b200_reduce_maxloc_f64(const double* x, size_t n, double* val, int64_t* idx,
                           b200_stream_t stream);
int b200_reduce_maxloc_i32(const int32_t* x, size_t n, int32_t* val, int64_t* idx,
                           b200_stream_t stream);
int b200_reduce_maxloc_i64(const int64_t* x, size_t n, int64_t* val, int64_t* idx,
                           b200_stream_t stream);

/* ReduceBitOr / ReduceBitAnd (pattern/detail/reduce.hpp:505-560) */
int b200_reduce_bitor_i32(const int32_t* x, size_t n, int32_t* out, b200_stream_t stream);
int b200_reduce_bitor_i64(const int64_t* x, size_t n, int64_t* out, b200_stream_t stream);
int b200_reduce_bitor_u32(const uint32_t* x, size_t n, uint32_t* out, b200_stream_t stream);
int b200_reduce_bitor_u64(const uint64_t* x, size_t n, uint64_t* out, b200_stream_t stream);
int b200_reduce_bitand_i32(const int32_t* x, size_t n, int32_t* out, b200_stream_t stream);
int b200_reduce_bitand_i64(const int64_t* x, size_t n, int64_t* out, b200_stream_t stream);
int b200_reduce_bitand_u32(const uint32_t* x, size_t n, uint32_t* out, b200_stream_t stream);
int b200_reduce_bitand_u64(const uint64_t* x, size_t n, uint64_t* out, b200_stream_t stream);

/* ======================================================================
 * Scans -- impl::scan::{inclusive, exclusive, inclusive_inplace,
 * exclusive_inplace} (policy/cuda/scan.hpp:45-235, which forwards to
 * cub::DeviceScan).  Single-pass decoupled look-back; `in == out` gives the
 * in-place forms.  `op` is B200_OP_*.  Exclusive scans write `init` first
 * (policy/sequential/scan.hpp:127-153).  Integer sums wrap around; `mode`
 * (B200_MODE_COMPENSATED) only affects f32/f64 sums.
 * ====================================================================== */

int b200_scan_inclusive_i32(const int32_t* in, int32_t* out, size_t n, int op,
                            b200_stream_t stream);
int b200_scan_inclusive_i64(const int64_t* in, int64_t* out, size_t n, int op,
                            b200_stream_t stream);
int b200_scan_inclusive_u32(const uint32_t* in, uint32_t* out, size_t n, int op,
                            b200_stream_t stream);
int b200_scan_inclusive_u64(const uint64_t* in, uint64_t* out, size_t n, int op,
                            b200_stream_t stream);
int b200_scan_inclusive_f32(const float* in, float* out, size_t n, int op,
                            int mode, b200_stream_t stream);
int b200_scan_inclusive_f64(const double* in, double* out, size_t n, int op,
                            int mode, b200_stream_t stream);
int b200_scan_exclusive_i32(const int32_t* in, int32_t* out, size_t n, int op,
                            int32_t init, b200_stream_t stream);
int b200_scan_exclusive_i64(const int64_t* in, int64_t* out, size_t n, int op,
                            int64_t init, b200_stream_t stream);
int b200_scan_exclusive_u32(const uint32_t* in, uint32_t* out, size_t n, int op,
                            uint32_t init, b200_stream_t stream);
int b200_scan_exclusive_u64(const uint64_t* in, uint64_t* out, size_t n, int op,
                            uint64_t init, b200_stream_t stream);
int b200_scan_exclusive_f32(const float* in, float* out, size_t n, int op,
                            float init, int mode, b200_stream_t stream);
int b200_scan_exclusive_f64(const double* in, double* out, size_t n, int op,
                            double init, int mode, b200_stream_t stream);

/* ======================================================================
 * Sorts -- impl::sort::{stable, unstable, stable_pairs, unstable_pairs}
 * (policy/cuda/sort.hpp:92-653, which forwards to cub::DeviceRadixSort).
 * LSD radix sort, 8-bit digits, onesweep passes.  Always stable, so it
 * serves both sort and stable_sort.  `descending` != 0 gives
 * operators::greater order (stable: equal keys keep input order).
 * Floating-point keys are ordered by their IEEE bit pattern (-0.0 before
 * +0.0; NaNs at the ends), which matches operators::less on every non-NaN,
 * non-signed-zero input.
 * In-place forms sort `keys` (and permute `vals`) in place.  The _copy forms
 * read keys_in/vals_in and write keys_out/vals_out, leaving the inputs
 * untouched.  Scratch memory comes from the library's per-stream arena.
 * ====================================================================== */

int b200_sort_keys_u32(uint32_t* keys, size_t n, int descending, b200_stream_t stream);
int b200_sort_keys_u64(uint64_t* keys, size_t n, int descending, b200_stream_t stream);
int b200_sort_keys_i32(int32_t* keys, size_t n, int descending, b200_stream_t stream);
int b200_sort_keys_i64(int64_t* keys, size_t n, int descending, b200_stream_t stream);
int b200_sort_keys_f32(float* keys, size_t n, int descending, b200_stream_t stream);
int b200_sort_keys_f64(double* keys, size_t n, int descending, b200_stream_t stream);

int b200_sort_keys_copy_u32(const uint32_t* keys_in, uint32_t* keys_out, size_t n,
                            int descending, b200_stream_t stream);
int b200_sort_keys_copy_u64(const uint64_t* keys_in, uint64_t* keys_out, size_t n,
                            int descending, b200_stream_t stream);
int b200_sort_keys_copy_f32(const float* keys_in, float* keys_out, size_t n,
                            int descending, b200_stream_t stream);

/* sort_pairs / stable_sort_pairs (pattern/sort.hpp:196-230) */
int b200_sort_pairs_u32_i32(uint32_t* keys, int32_t* vals, size_t n, int descending,
                            b200_stream_t stream);
int b200_sort_pairs_u32_u32(uint32_t* keys, uint32_t* vals, size_t n, int descending,
                            b200_stream_t stream);
int b200_sort_pairs_i32_i32(int32_t* keys, int32_t* vals, size_t n, int descending,
                            b200_stream_t stream);
int b200_sort_pairs_f32_i32(float* keys, int32_t* vals, size_t n, int descending,
                            b200_stream_t stream);
int b200_sort_pairs_u64_i32(uint64_t* keys, int32_t* vals, size_t n, int descending,
                            b200_stream_t stream);
int b200_sort_pairs_u64_i64(uint64_t* keys, int64_t* vals, size_t n, int descending,
                            b200_stream_t stream);
int b200_sort_pairs_i64_i64(int64_t* keys, int64_t* vals, size_t n, int descending,
                            b200_stream_t stream);
int b200_sort_pairs_f64_i64(double* keys, int64_t* vals, size_t n, int descending,
                            b200_stream_t stream);
int b200_sort_pairs_f64_i32(double* keys, int32_t* vals, size_t n, int descending,
                            b200_stream_t stream);
/* with the four above, every key type pairs with 32- and 64-bit values
 * (the C++ layer sorts any 4- or 8-byte value type through these as bit
 * patterns) */
int b200_sort_pairs_i64_i32(int64_t* keys, int32_t* vals, size_t n, int descending,
                            b200_stream_t stream);
int b200_sort_pairs_u32_i64(uint32_t* keys, int64_t* vals, size_t n, int descending,
                            b200_stream_t stream);
int b200_sort_pairs_i32_i64(int32_t* keys, int64_t* vals, size_t n, int descending,
                            b200_stream_t stream);
int b200_sort_pairs_f32_i64(float* keys, int64_t* vals, size_t n, int descending,
                            b200_stream_t stream);
int b200_sort_pairs_copy_f32_i32(const float* keys_in, const int32_t* vals_in,
                                 float* keys_out, int32_t* vals_out, size_t n,
                                 int descending, b200_stream_t stream);
int b200_sort_pairs_copy_u32_i32(const uint32_t* keys_in, const int32_t* vals_in,
                                 uint32_t* keys_out, int32_t* vals_out, size_t n,
                                 int descending, b200_stream_t stream);

/* ======================================================================
 * Histogram -- MultiReduceSum<cuda_multi_reduce_atomic, T> with a +1 body,
 * i.e. the binned atomic reduction of policy/cuda/multi_reduce.hpp:80-690.
 * counts[b] += #{ i : x[i] == b } for b in [0, nbins); values outside
 * [0, nbins) are not counted.  `counts` is accumulated into (zero it first
 * for a fresh histogram, as MultiReduceSum(num_bins, 0) does).
 * ====================================================================== */

int b200_histogram_i32(const int32_t* x, size_t n, int32_t nbins, uint64_t* counts,
                       b200_stream_t stream);

/* ======================================================================
 * Binned reductions -- MultiReduce{Sum,Min,Max,BitOr,BitAnd}<policy, T>
 * (pattern/multi_reduce.hpp:68-190; combine rule per bin in
 * pattern/detail/multi_reduce.hpp:172-402 and
 * policy/sequential/multi_reduce.hpp:135; CUDA atomics in
 * policy/cuda/multi_reduce.hpp:80-690).
 * out[b] = op(out[b], vals[i]) for every i with bins[i] == b; bins outside
 * [0, nbins) are skipped.  `out` holds the initial values (the MultiReduce
 * constructor's init) and is combined into.  min keeps `if (v < val) val =
 * v`, max `if (val < v) val = v`: NaN values never enter.  Integer and bit
 * results are exact; floating-point sums depend on the atomic order.
 * ====================================================================== */
int b200_multi_reduce_sum_i32(const int32_t* bins, const int32_t* vals, size_t n, int32_t nbins,
                              int32_t* out, b200_stream_t stream);
int b200_multi_reduce_sum_i64(const int32_t* bins, const int64_t* vals, size_t n, int32_t nbins,
                              int64_t* out, b200_stream_t stream);
int b200_multi_reduce_sum_u32(const int32_t* bins, const uint32_t* vals, size_t n, int32_t nbins,
                              uint32_t* out, b200_stream_t stream);
int b200_multi_reduce_sum_u64(const int32_t* bins, const uint64_t* vals, size_t n, int32_t nbins,
                              uint64_t* out, b200_stream_t stream);
int b200_multi_reduce_sum_f32(const int32_t* bins, const float* vals, size_t n, int32_t nbins,
                              float* out, b200_stream_t stream);
int b200_multi_reduce_sum_f64(const int32_t* bins, const double* vals, size_t n, int32_t nbins,
                              double* out, b200_stream_t stream);
int b200_multi_reduce_min_i32(const int32_t* bins, const int32_t* vals, size_t n, int32_t nbins,
                              int32_t* out, b200_stream_t stream);
int b200_multi_reduce_min_i64(const int32_t* bins, const int64_t* vals, size_t n, int32_t nbins,
                              int64_t* out, b200_stream_t stream);
int b200_multi_reduce_min_u32(const int32_t* bins, const uint32_t* vals, size_t n, int32_t nbins,
                              uint32_t* out, b200_stream_t stream);
int b200_multi_reduce_min_u64(const int32_t* bins, const uint64_t* vals, size_t n, int32_t nbins,
                              uint64_t* out, b200_stream_t stream);
int b200_multi_reduce_min_f32(const int32_t* bins, const float* vals, size_t n, int32_t nbins,
                              float* out, b200_stream_t stream);
int b200_multi_reduce_min_f64(const int32_t* bins, const double* vals, size_t n, int32_t nbins,
                              double* out, b200_stream_t stream);
int b200_multi_reduce_max_i32(const int32_t* bins, const int32_t* vals, size_t n, int32_t nbins,
                              int32_t* out, b200_stream_t stream);
int b200_multi_reduce_max_i64(const int32_t* bins, const int64_t* vals, size_t n, int32_t nbins,
                              int64_t* out, b200_stream_t stream);
int b200_multi_reduce_max_u32(const int32_t* bins, const uint32_t* vals, size_t n, int32_t nbins,
                              uint32_t* out, b200_stream_t stream);
int b200_multi_reduce_max_u64(const int32_t* bins, const uint64_t* vals, size_t n, int32_t nbins,
                              uint64_t* out, b200_stream_t stream);
int b200_multi_reduce_max_f32(const int32_t* bins, const float* vals, size_t n, int32_t nbins,
                              float* out, b200_stream_t stream);
int b200_multi_reduce_max_f64(const int32_t* bins, const double* vals, size_t n, int32_t nbins,
                              double* out, b200_stream_t stream);
int b200_multi_reduce_bitor_i32(const int32_t* bins, const int32_t* vals, size_t n, int32_t nbins,
                                int32_t* out, b200_stream_t stream);
int b200_multi_reduce_bitor_i64(const int32_t* bins, const int64_t* vals, size_t n, int32_t nbins,
                                int64_t* out, b200_stream_t stream);
int b200_multi_reduce_bitor_u32(const int32_t* bins, const uint32_t* vals, size_t n, int32_t nbins,
                                uint32_t* out, b200_stream_t stream);
int b200_multi_reduce_bitor_u64(const int32_t* bins, const uint64_t* vals, size_t n, int32_t nbins,
                                uint64_t* out, b200_stream_t stream);
int b200_multi_reduce_bitand_i32(const int32_t* bins, const int32_t* vals, size_t n, int32_t nbins,
                                 int32_t* out, b200_stream_t stream);
int b200_multi_reduce_bitand_i64(const int32_t* bins, const int64_t* vals, size_t n, int32_t nbins,
                                 int64_t* out, b200_stream_t stream);
int b200_multi_reduce_bitand_u32(const int32_t* bins, const uint32_t* vals, size_t n, int32_t nbins,
                                 uint32_t* out, b200_stream_t stream);
int b200_multi_reduce_bitand_u64(const int32_t* bins, const uint64_t* vals, size_t n, int32_t nbins,
                                 uint64_t* out, b200_stream_t stream);

/* ======================================================================
 * Batched loops -- WorkPool/WorkGroup with many uneven loops
 * (pattern/WorkGroup.hpp:207-530; CUDA runners
 * policy/cuda/WorkGroup/WorkRunner.hpp:38-407, which launch once per loop
 * (ordered) or once with an average-length grid and no reducer support
 * (unordered, :323-329)), IndexSet segments (policy/cuda/forall.hpp:675-706)
 * and segmented scan / sort (no RAJA counterpart: the reference composition
 * is one scan or sort call per segment).
 *
 * A plan is built once from the host array of loop lengths, like
 * WorkPool::instantiate (pattern/WorkGroup.hpp:459-487).  Loop i covers
 * indices [0, lens[i]); for the segmented primitives, segment i covers
 * [offsets[i], offsets[i+1]) of one flattened array, offsets being the
 * prefix sums of lens.  A plan belongs to the device current at creation.
 * A plan holds the warp partials of its runs, so calls with one plan must
 * not overlap on the GPU: issue them on one stream, or order the streams.
 * ====================================================================== */
typedef struct b200_batch_plan_s* b200_batch_plan;

int b200_batch_plan_create(const int64_t* lens_host, int nloops, b200_batch_plan* out);
int b200_batch_plan_destroy(b200_batch_plan plan);
int b200_batch_plan_info(b200_batch_plan plan, int64_t* total, int64_t* ntiles, int* tile,
                         int* block);
/* device array of the nloops+1 segment offsets */
const int64_t* b200_batch_plan_offsets(b200_batch_plan plan);
/* Pin the launch shape of the plan's batched loops: `block` threads with
 * `items` elements per thread per tile, one of the shapes the autotuner
 * times (256x8, 256x16, 512x8, 128x16, 256x4); B200_ERR_ARG for any other
 * pair.  Like the fixed BLOCK of a b200_work<BLOCK> group. */
int b200_batch_plan_set_shape(b200_batch_plan plan, int block, int items);

/* Every loop i: y_i[j] += a * x_i[j]; sums[i] = sum_j y_i[j] (after the
 * update), for all loops in one persistent launch.  xs, ys: device arrays
 * of nloops device pointers; sums: device array of nloops doubles.
 * mode: B200_MODE_COMPENSATED for TwoSum partials (else naive FP32
 * partials); each loop's partials are added in a fixed order (the sums are
 * deterministic for a given plan shape). */
int b200_batched_axpy_sum_f32(b200_batch_plan plan, float a, const float* const* xs,
                              float* const* ys, double* sums, int mode, b200_stream_t stream);
/* Time the kernel variants (block size x items per thread) on this plan and
 * keep the fastest for later calls.  Runs the loops several times: y is
 * updated by every run. */
int b200_batch_autotune_axpy_sum_f32(b200_batch_plan plan, float a, const float* const* xs,
                                     float* const* ys, double* sums, int mode,
                                     b200_stream_t stream);
/* One loop: the fused axpy + sum of a single loop (one launch per loop is
 * what the ordered WorkGroup runner does). */
int b200_loop_axpy_sum_f32(float a, const float* x, float* y, size_t n, double* sum, int mode,
                           b200_stream_t stream);
/* The ordered WorkGroup runner's schedule for the same work: loop i runs
 * as its own launch (b200_loop_axpy_sum_f32), in order, all issued from
 * this call (policy/cuda/WorkGroup/WorkRunner.hpp:38-162 launches one forall
 * per enqueued loop).  lens_host, xs_host, ys_host: host arrays of nloops
 * lengths and device pointers; sums: device array of nloops doubles. */
int b200_loops_axpy_sum_f32(int nloops, const int64_t* lens_host, float a, const float* const* xs_host,
                            float* const* ys_host, double* sums, int mode, b200_stream_t stream);

/* Segmented sum scans of int32 over the plan's segments (restart at each
 * segment; exclusive writes 0 at each head). */
int b200_segmented_scan_inclusive_i32(b200_batch_plan plan, const int32_t* in, int32_t* out,
                                      b200_stream_t stream);
int b200_segmented_scan_exclusive_i32(b200_batch_plan plan, const int32_t* in, int32_t* out,
                                      b200_stream_t stream);
/* Sort the keys of every segment independently, in place.  When the plan
 * has several segments longer than 4096 keys, averaging at most 2^18, they
 * are sorted together in one 64-bit sort, and the plan holds a buffer of
 * 8 bytes per key of those segments for it. */
int b200_segmented_sort_keys_u32(b200_batch_plan plan, uint32_t* keys, int descending,
                                 b200_stream_t stream);

/* ======================================================================
 * Batched 3-D Jacobi sweeps over many meshes of different sizes, which the reference
 * writes with RAJA::launch + View/OffsetLayout and a ReduceMax residual
 * (pattern/launch/launch_core.hpp:150-460, util/OffsetLayout.hpp:166-244,
 * examples/jacobi.cpp:223-489), one launch per mesh per sweep.
 * Meshes are stored back to back, x fastest (mesh m starts at point
 * offsets[m]).  One sweep updates the interior of every mesh:
 *   unew = (f + sum of the six neighbours of u) / 6,
 *   resid[m] = max |unew - u| over mesh m's interior;
 * f may be NULL (f = 0).  Boundary points are never written, so u and
 * unew must carry the same boundary values.
 * ====================================================================== */
typedef struct b200_jacobi_plan_s* b200_jacobi_plan;

int b200_jacobi_plan_create(const int* nx, const int* ny, const int* nz, int nmeshes,
                            b200_jacobi_plan* out);
int b200_jacobi_plan_destroy(b200_jacobi_plan plan);
int b200_jacobi_plan_info(b200_jacobi_plan plan, int64_t* total_points, int64_t* interior_points,
                          int64_t* ntiles);
/* host array of the nmeshes+1 point offsets */
const int64_t* b200_jacobi_plan_offsets(b200_jacobi_plan plan);
/* one sweep over every mesh of the plan in one launch */
int b200_jacobi_sweep_f64(b200_jacobi_plan plan, const double* u, double* unew, const double* f,
                          double* resid, b200_stream_t stream);
/* one sweep of one mesh (the per-mesh launch of the reference formulation) */
int b200_jacobi_mesh_sweep_f64(int nx, int ny, int nz, const double* u, double* unew,
                               const double* f, double* resid, b200_stream_t stream);

/* ---- CUDA graph capture of repeated sweeps (replaces per-call launches) */
typedef struct b200_graph_s* b200_graph;
int b200_graph_capture_begin(b200_stream_t stream);
int b200_graph_capture_end(b200_stream_t stream, b200_graph* out);
int b200_graph_launch(b200_graph graph, b200_stream_t stream);
int b200_graph_destroy(b200_graph graph);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* B200PRIMS_H */
