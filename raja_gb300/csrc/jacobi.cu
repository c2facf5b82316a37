// Batched 3-D Jacobi sweeps with a per-mesh max residual.
//
// Reference: the RAJA::launch + View/OffsetLayout formulation of a Jacobi
// sweep (pattern/launch/launch_core.hpp:150-460, policy/cuda/launch.hpp:
// 32-400, util/OffsetLayout.hpp:166-244; examples/jacobi.cpp:223-489 for
// the iteration with a residual reducer), where each mesh is one launch per
// sweep with a ReduceMax.
//
// One sweep of mesh m (interior points 1..n-2 in each axis):
//   unew[i,j,k] = (f[i,j,k] + u[i-1,j,k] + u[i+1,j,k] + u[i,j-1,k]
//                  + u[i,j+1,k] + u[i,j,k-1] + u[i,j,k+1]) / 6
//   resid[m]    = max |unew - u| over the interior
// with f == nullptr meaning f = 0 (Laplace).  Boundary points are never
// written: both buffers must hold the same boundary values.
//
// GB300 design: a plan lays all meshes out back to back (x fastest) and
// cuts every interior into tiles of whole x-rows (a few rows of one z
// plane); one launch sweeps every tile of every mesh, each block taking a
// contiguous run of the tile table, so thousands of small meshes cost one
// launch instead of one each.  Each thread computes points along x
// (coalesced); the y and z neighbours of a tile's rows are re-read from
// L1/L2.  The sweep is bound by the FP64 pipe (7 FP64 operations per point
// for the Laplace case), so the residual maximum is kept as integer bits:
// per-mesh residuals are block maxima folded with a 64-bit atomicMax on the
// bit pattern (valid for non-negative doubles).  Sweeps can be captured in
// a CUDA graph (b200_graph_*), so a 20-sweep solve is one graph launch.
#include <algorithm>
#include <vector>

#include "b200_internal.cuh"

struct b200_jacobi_plan_s {
  int device = -1;
  int nmeshes = 0;
  std::vector<int> nx, ny, nz;
  std::vector<int64_t> off;     // first point of each mesh
  int64_t total = 0;            // points over all meshes
  int64_t ntiles = 0;
  int4* d_tiles = nullptr;      // (mesh, z, y0, y1)
  int4* d_dims = nullptr;       // (nx, ny, nz, 0) per mesh
  int64_t* d_off = nullptr;
};

namespace b200 {
namespace {

constexpr int JBLOCK = 256;
// Interior points per thread in a tile.  Larger tiles spread the tile
// descriptor and mesh loads over more stencil points (2 -> 4 took a 512^3
// sweep from 2.05 to 1.87 ms); beyond 4 the blocks' runs of small meshes
// balance worse (16: 18% slower on 256 meshes of edge 16..128).
constexpr int JPTS = 4;

// The stencil in the oracle's operation order, with explicitly rounded
// operations so that no multiply-add is contracted.  HAS_F is a template
// parameter: a run-time test on f inside the loop is if-converted, and the
// predicated add then still occupies the FP64 pipe.
template <bool HAS_F>
__device__ __forceinline__ double jac_point(const double* __restrict__ u, const double* __restrict__ f,
                                            int64_t c, int64_t sx, int64_t sy) {
  double acc = __dadd_rn(u[c - 1], u[c + 1]);
  acc = __dadd_rn(acc, __dadd_rn(u[c - sx], u[c + sx]));
  acc = __dadd_rn(acc, __dadd_rn(u[c - sy], u[c + sy]));
  if (HAS_F) acc = __dadd_rn(acc, f[c]);
  return __dmul_rn(acc, 1.0 / 6.0);
}

// Running maximum of |v - u| over the non-NaN differences (NaN never wins
// "r > rmax"), kept as the two 32-bit words of the double's bits.  For
// non-negative doubles the unsigned order of the bits is the numeric order,
// so the maximum and its block and mesh reductions are integer operations
// on 32-bit words: on GB300 the FP64 pipe issues about 2 lanes per clock
// per SM and is kept for the stencil itself.
struct RunMax {
  unsigned hi = 0, lo = 0;
  __device__ __forceinline__ void take(double v, double uc) {
    const double d = __dsub_rn(v, uc);
    const unsigned h = static_cast<unsigned>(__double2hiint(d)) & 0x7fffffffu;
    const unsigned l = static_cast<unsigned>(__double2loint(d));
    const bool nan = h > 0x7ff00000u || (h == 0x7ff00000u && l != 0u);
    const bool gt = h > hi || (h == hi && l > lo);
    if (gt && !nan) {
      hi = h;
      lo = l;
    }
  }
  __device__ __forceinline__ unsigned long long bits() const {
    return (static_cast<unsigned long long>(hi) << 32) | lo;
  }
};

__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}

// Block maximum of `rb`, folded into *dst with a 64-bit atomicMax.  Called
// by every thread of the block.
__device__ __forceinline__ void flush_resid(unsigned long long rb, unsigned long long* dst,
                                            unsigned long long* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) rb = umax64(rb, __shfl_xor_sync(0xffffffffu, rb, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = rb;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long bm = sh[0];
    for (int q = 1; q < JBLOCK / 32; ++q) bm = umax64(bm, sh[q]);
    if (bm != 0) atomicMax(dst, bm);
  }
  __syncthreads();
}

// One sweep over all tiles of the plan.  Each block takes a contiguous run
// of the tile table, so consecutive tiles mostly belong to one mesh: the
// residual stays in registers across them and is reduced once per mesh
// change instead of once per tile.
template <bool HAS_F>
__global__ void __launch_bounds__(JBLOCK)
jacobi_kernel(const int4* __restrict__ tiles, int64_t ntiles, const int4* __restrict__ dims,
              const int64_t* __restrict__ offs, const double* __restrict__ u,
              double* __restrict__ unew, const double* __restrict__ f,
              unsigned long long* __restrict__ resid) {
  __shared__ unsigned long long sh[JBLOCK / 32];
  const int64_t per = (ntiles + gridDim.x - 1) / gridDim.x;
  const int64_t t0 = int64_t(blockIdx.x) * per;
  const int64_t t1 = t0 + per < ntiles ? t0 + per : ntiles;
  if (t0 >= t1) return;                           // block-uniform
  int cur = -1;                                   // mesh of the running residual
  RunMax rb;
  int64_t sx = 0, sy = 0, moff = 0;
  int w = 0;
  int4 tl = tiles[t0];
  for (int64_t t = t0; t < t1; ++t) {
    const int4 nxt = t + 1 < t1 ? tiles[t + 1] : tl;   // next descriptor, loaded one tile ahead
    const int m = tl.x, k = tl.y, y0 = tl.z, y1 = tl.w;
    if (m != cur) {                               // block-uniform: all threads read the same tile
      if (cur >= 0) flush_resid(rb.bits(), resid + cur, sh);
      cur = m;
      rb = RunMax();
      const int4 d = dims[m];
      sx = d.x;
      sy = int64_t(d.x) * d.y;
      moff = offs[m];
      w = d.x - 2;                                // interior points per row
    }
    const int64_t base = moff + int64_t(k) * sy;
    const int cnt = w * (y1 - y0);
#pragma unroll 1
    for (int p = threadIdx.x; p < cnt; p += JBLOCK) {
      const int j = y0 + p / w;
      const int i = 1 + p % w;
      const int64_t c = base + int64_t(j) * sx + i;
      const double v = jac_point<HAS_F>(u, f, c, sx, sy);
      unew[c] = v;
      rb.take(v, u[c]);
    }
    tl = nxt;
  }
  flush_resid(rb.bits(), resid + cur, sh);
}

// Plain per-mesh sweep (one launch per mesh per sweep).
template <bool HAS_F>
__global__ void __launch_bounds__(JBLOCK)
jacobi_mesh_kernel(int nx, int ny, int nz, const double* __restrict__ u, double* __restrict__ unew,
                   const double* __restrict__ f, unsigned long long* __restrict__ resid) {
  __shared__ unsigned long long sh[JBLOCK / 32];
  const int64_t sx = nx, sy = int64_t(nx) * ny;
  const int w = nx - 2, h = ny - 2, dz = nz - 2;
  const int64_t cnt = int64_t(w) * h * dz;
  RunMax rb;
  for (int64_t p = int64_t(blockIdx.x) * JBLOCK + threadIdx.x; p < cnt; p += int64_t(gridDim.x) * JBLOCK) {
    const int i = 1 + int(p % w);
    const int64_t q = p / w;
    const int j = 1 + int(q % h);
    const int k = 1 + int(q / h);
    const int64_t c = int64_t(k) * sy + int64_t(j) * sx + i;
    const double v = jac_point<HAS_F>(u, f, c, sx, sy);
    unew[c] = v;
    rb.take(v, u[c]);
  }
  flush_resid(rb.bits(), resid, sh);
}

int check_jplan(b200_jacobi_plan_s* p, const char* name) {
  if (!p) return fail(B200_ERR_ARG, "%s: null plan", name);
  int dev = 0;
  B200_CUDA(cudaGetDevice(&dev));
  if (dev != p->device) return fail(B200_ERR_ARG, "%s: plan belongs to device %d", name, p->device);
  return B200_OK;
}

}  // namespace
}  // namespace b200

using namespace b200;

extern "C" {

int b200_jacobi_plan_create(const int* nx, const int* ny, const int* nz, int nmeshes,
                            b200_jacobi_plan* out) {
  const char* name = "b200_jacobi_plan_create";
  if (!out) return fail(B200_ERR_ARG, "%s: null out", name);
  *out = nullptr;
  if (nmeshes <= 0 || !nx || !ny || !nz) return fail(B200_ERR_ARG, "%s: bad meshes", name);
  auto* p = new b200_jacobi_plan_s();
  B200_CUDA(cudaGetDevice(&p->device));
  p->nmeshes = nmeshes;
  p->nx.assign(nx, nx + nmeshes);
  p->ny.assign(ny, ny + nmeshes);
  p->nz.assign(nz, nz + nmeshes);
  p->off.assign(size_t(nmeshes) + 1, 0);
  std::vector<int4> tiles, dims(nmeshes);
  for (int m = 0; m < nmeshes; ++m) {
    if (nx[m] < 3 || ny[m] < 3 || nz[m] < 3 || nx[m] > (1 << 20) || ny[m] > (1 << 20) || nz[m] > (1 << 20)) {
      delete p;
      return fail(B200_ERR_ARG, "%s: mesh %d has an edge outside [3, 2^20]", name, m);
    }
    p->off[m + 1] = p->off[m] + int64_t(nx[m]) * ny[m] * nz[m];
    dims[m] = make_int4(nx[m], ny[m], nz[m], 0);
    // rows of one z plane per tile, about JPTS interior points per thread
    const int w = nx[m] - 2;
    int rows = std::max(1, (JPTS * JBLOCK) / std::max(w, 1));
    for (int k = 1; k < nz[m] - 1; ++k)
      for (int y = 1; y < ny[m] - 1; y += rows)
        tiles.push_back(make_int4(m, k, y, std::min(y + rows, ny[m] - 1)));
  }
  p->total = p->off[nmeshes];
  p->ntiles = int64_t(tiles.size());
  int rc = B200_OK;
  auto ck = [&](cudaError_t e, const char* w) { if (rc == B200_OK && e != cudaSuccess) rc = cuda_check(e, w); };
  ck(cudaMalloc(&p->d_tiles, std::max<size_t>(tiles.size(), 1) * sizeof(int4)), "jacobi tiles");
  ck(cudaMalloc(&p->d_dims, dims.size() * sizeof(int4)), "jacobi dims");
  ck(cudaMalloc(&p->d_off, p->off.size() * sizeof(int64_t)), "jacobi offsets");
  if (rc == B200_OK && !tiles.empty())
    ck(cudaMemcpy(p->d_tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice), "jacobi tiles");
  if (rc == B200_OK)
    ck(cudaMemcpy(p->d_dims, dims.data(), dims.size() * sizeof(int4), cudaMemcpyHostToDevice), "jacobi dims");
  if (rc == B200_OK)
    ck(cudaMemcpy(p->d_off, p->off.data(), p->off.size() * sizeof(int64_t), cudaMemcpyHostToDevice), "jacobi offs");
  if (rc != B200_OK) {
    b200_jacobi_plan_destroy(p);
    return rc;
  }
  *out = p;
  clear_error();
  return B200_OK;
}

int b200_jacobi_plan_destroy(b200_jacobi_plan p) {
  if (!p) return B200_OK;
  cudaFree(p->d_tiles);
  cudaFree(p->d_dims);
  cudaFree(p->d_off);
  delete p;
  return B200_OK;
}

int b200_jacobi_plan_info(b200_jacobi_plan p, int64_t* total_points, int64_t* interior_points,
                          int64_t* ntiles) {
  if (!p) return fail(B200_ERR_ARG, "b200_jacobi_plan_info: null plan");
  int64_t interior = 0;
  for (int m = 0; m < p->nmeshes; ++m) interior += int64_t(p->nx[m] - 2) * (p->ny[m] - 2) * (p->nz[m] - 2);
  if (total_points) *total_points = p->total;
  if (interior_points) *interior_points = interior;
  if (ntiles) *ntiles = p->ntiles;
  return B200_OK;
}

const int64_t* b200_jacobi_plan_offsets(b200_jacobi_plan p) { return p ? p->off.data() : nullptr; }

int b200_jacobi_sweep_f64(b200_jacobi_plan p, const double* u, double* unew, const double* f,
                          double* resid, b200_stream_t stream) {
  const char* name = "b200_jacobi_sweep_f64";
  B200_TRY(check_jplan(p, name));
  if (!u || !unew || !resid) return fail(B200_ERR_ARG, "%s: null pointer", name);
  if (u == unew) return fail(B200_ERR_ARG, "%s: u and unew must differ", name);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  B200_CUDA(cudaMemsetAsync(resid, 0, p->nmeshes * sizeof(double), s));
  if (p->ntiles == 0) return B200_OK;
  static KernelSetup ks[2];
  DeviceProps props;
  B200_TRY(device_props(&props));
  const auto kern = f ? jacobi_kernel<true> : jacobi_kernel<false>;
  int bps = 0;
  B200_TRY(kernel_setup(ks[f ? 1 : 0], props, kern, JBLOCK, 0, &bps));
  int64_t grid = int64_t(props.sms) * bps;
  if (grid > p->ntiles) grid = p->ntiles;
  B200_LAUNCH(name, kern, unsigned(grid), JBLOCK, 0, s, p->d_tiles, p->ntiles, p->d_dims,
              p->d_off, u, unew, f, reinterpret_cast<unsigned long long*>(resid));
  clear_error();
  return B200_OK;
}

int b200_jacobi_mesh_sweep_f64(int nx, int ny, int nz, const double* u, double* unew, const double* f,
                               double* resid, b200_stream_t stream) {
  const char* name = "b200_jacobi_mesh_sweep_f64";
  if (nx < 3 || ny < 3 || nz < 3) return fail(B200_ERR_ARG, "%s: edges must be >= 3", name);
  if (!u || !unew || !resid || u == unew) return fail(B200_ERR_ARG, "%s: bad pointers", name);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  B200_CUDA(cudaMemsetAsync(resid, 0, sizeof(double), s));
  static KernelSetup ks[2];
  DeviceProps props;
  B200_TRY(device_props(&props));
  const auto kern = f ? jacobi_mesh_kernel<true> : jacobi_mesh_kernel<false>;
  int bps = 0;
  B200_TRY(kernel_setup(ks[f ? 1 : 0], props, kern, JBLOCK, 0, &bps));
  const int64_t cnt = int64_t(nx - 2) * (ny - 2) * (nz - 2);
  int64_t grid = (cnt + JBLOCK - 1) / JBLOCK;
  if (grid > int64_t(props.sms) * bps) grid = int64_t(props.sms) * bps;
  B200_LAUNCH(name, kern, unsigned(grid), JBLOCK, 0, s, nx, ny, nz, u, unew, f,
              reinterpret_cast<unsigned long long*>(resid));
  clear_error();
  return B200_OK;
}

}  // extern "C"
