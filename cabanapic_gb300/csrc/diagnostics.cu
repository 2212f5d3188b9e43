// diagnostics.cu -- FP64 diagnostics of the step: node charge density, the
// discrete Gauss-law residual div E - rho/eps0, and particle kinetic energy.
//
// None of these exist in the reference (its only diagnostic is the field
// energy, src/fields.h:556-615).  They measure what its scheme conserves:
// with rho deposited trilinearly to the nodes (node (i,j,k) is the low corner
// of voxel (i,j,k); a particle at offsets (x,y,z) in [-1,1] gives node weights
// (1 -/+ x)/2 (1 -/+ y)/2 (1 -/+ z)/2) and div E taken with backward
// differences of the edge fields (ex(i) - ex(i-1)) / dx + ..., the push's
// charge-conserving deposit (src/push.h:218-254, src/move_p.h:154-190) and the
// Yee update (src/fields.h:618-665) keep div E - rho/eps0 constant in time to
// round-off.  All sums are double, with fixed reduction trees.
#include <cuda_runtime.h>

#include "common.cuh"

namespace cpic {

constexpr int kDiagThreads = 256;
constexpr int kDiagBlocks = 592;

struct DiagScratch {
  double part[4 * kDiagBlocks];
  unsigned int done;
};

// ------------------------------------------------------------ charge density
// Sum of v[0..7] over the 32 lanes, scattered: lanes 4k..4k+3 hold the total
// of value index k (k = lane >> 2).
__device__ __forceinline__ double reduce_scatter8(const double v[8], int lane) {
  const bool h16 = lane & 16, h8 = lane & 8, h4 = lane & 4;
  double a[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    double send = h16 ? v[k] : v[k + 4];
    double keep = h16 ? v[k + 4] : v[k];
    a[k] = keep + __shfl_xor_sync(kFull, send, 16);
  }
  double b[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    double send = h8 ? a[k] : a[k + 2];
    double keep = h8 ? a[k + 2] : a[k];
    b[k] = keep + __shfl_xor_sync(kFull, send, 8);
  }
  double c = (h4 ? b[1] : b[0]) + __shfl_xor_sync(kFull, h4 ? b[0] : b[1], 4);
  c += __shfl_xor_sync(kFull, c, 2);
  return c + __shfl_xor_sync(kFull, c, 1);
}

template <class R, int VL>
__global__ void __launch_bounds__(kDiagThreads)
rho_deposit_kernel(const unsigned char* __restrict__ part, int n, double* __restrict__ rho,
                   const GridDev g, double q_over_vol, int* __restrict__ bad) {
  using L = PLayout<R, VL>;
  const int lane = lane_id();
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool valid = p < n;
  double x = 0, y = 0, z = 0, w = 0;
  int cell = 0;
  if (valid) {
    x = (double)*reinterpret_cast<const R*>(part + L::off(p, 0));
    y = (double)*reinterpret_cast<const R*>(part + L::off(p, 1));
    z = (double)*reinterpret_cast<const R*>(part + L::off(p, 2));
    w = (double)*reinterpret_cast<const R*>(part + L::off(p, 6));
    cell = *reinterpret_cast<const int*>(part + L::cell_off(p));
    // nodes up to cell + 1 + sx + sx*sy must exist
    if ((unsigned)cell >= (unsigned)(g.num_cells - 1 - g.sx - g.sx * g.sy)) {
      atomicOr(bad, 1);
      valid = false;
      cell = 0;
    }
  }
  const double q = valid ? w * q_over_vol : 0.0;
  const double wx[2] = {0.5 * (1.0 - x), 0.5 * (1.0 + x)};
  const double wy[2] = {0.5 * (1.0 - y), 0.5 * (1.0 + y)};
  const double wz[2] = {0.5 * (1.0 - z), 0.5 * (1.0 + z)};
  double v[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = q * wx[k & 1] * wy[(k >> 1) & 1] * wz[k >> 2];
  const int off_of[8] = {0, 1, g.sx, g.sx + 1, g.sx * g.sy, g.sx * g.sy + 1,
                         g.sx * g.sy + g.sx, g.sx * g.sy + g.sx + 1};
  const int cell0 = __shfl_sync(kFull, cell, 0);
  if (__all_sync(kFull, valid && cell == cell0)) {
    const double t = reduce_scatter8(v, lane);
    if ((lane & 3) == 0) atomicAdd(rho + cell0 + off_of[lane >> 2], t);
  } else if (valid) {
#pragma unroll
    for (int k = 0; k < 8; ++k) atomicAdd(rho + cell + off_of[k], v[k]);
  }
}

// Periodic fold of the node ghosts at index n+1 into index 1, one axis per
// launch (x, then y, then z), over whole planes so corners fold correctly.
__global__ void __launch_bounds__(kDiagThreads)
rho_fold_kernel(double* __restrict__ rho, const GridDev g, int axis) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  int a, b, from, to;
  if (axis == 0) {
    if (t >= g.sy * g.sz) return;
    a = t % g.sy; b = t / g.sy;
    from = g.vox(g.nx + 1, a, b); to = g.vox(1, a, b);
  } else if (axis == 1) {
    if (t >= g.sx * g.sz) return;
    a = t % g.sx; b = t / g.sx;
    from = g.vox(a, g.ny + 1, b); to = g.vox(a, 1, b);
  } else {
    if (t >= g.sx * g.sy) return;
    a = t % g.sx; b = t / g.sx;
    from = g.vox(a, b, g.nz + 1); to = g.vox(a, b, 1);
  }
  rho[to] += rho[from];
  rho[from] = 0.0;
}

// ------------------------------------------------------------ reductions
template <int NV>
__device__ void block_store_partials(double (&v)[NV], DiagScratch* sc, double* out, bool want_max0,
                                     double scale) {
  __shared__ double sh[kDiagThreads / 32][NV];
  __shared__ bool last;
  for (int k = 0; k < NV; ++k) {
    for (int o = 16; o > 0; o >>= 1) {
      const double t = __shfl_xor_sync(kFull, v[k], o);
      v[k] = (want_max0 && k == 0) ? fmax(v[k], t) : v[k] + t;
    }
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < NV; ++k) sh[w][k] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < NV; ++k) {
      double t = sh[0][k];
      for (int j = 1; j < kDiagThreads / 32; ++j) t = (want_max0 && k == 0) ? fmax(t, sh[j][k]) : t + sh[j][k];
      sc->part[NV * blockIdx.x + k] = t;
    }
    __threadfence();
    last = (atomicAdd(&sc->done, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {  // block-uniform
    __threadfence();
    double r[NV];
    reduce_partials<NV, kDiagThreads>(sc->part, gridDim.x, want_max0 ? 1u : 0u, r);
    if (threadIdx.x == 0) {
      for (int k = 0; k < NV; ++k) out[k] = (want_max0 && k == 0) ? r[k] : r[k] * scale;
      sc->done = 0;
    }
  }
}

__device__ __forceinline__ int wrap_low(int i, int n) { return i == 0 ? n : i; }

// Gauss residual r = div E - rho/eps0 (- ref) at every interior node.
// out = {max |r|, sum r^2, sum (rho/eps0)^2}; resid (optional) gets r.
template <class R>
__global__ void __launch_bounds__(kDiagThreads)
gauss_kernel(const R* __restrict__ F, const double* __restrict__ rho, const double* __restrict__ ref,
             double* __restrict__ resid, const GridDev g, double idx, double idy, double idz,
             double ieps0, double* __restrict__ out, DiagScratch* __restrict__ sc) {
  const unsigned rows = (unsigned)g.ny * (unsigned)g.nz;
  const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  double v[3] = {0.0, 0.0, 0.0};
  for (unsigned r = warp; r < rows; r += nwarps) {
    const int y = (int)(r % (unsigned)g.ny) + 1, z = (int)(r / (unsigned)g.ny) + 1;
    const int ym = wrap_low(y - 1, g.ny), zm = wrap_low(z - 1, g.nz);
    for (int x = 1 + lane; x <= g.nx; x += 32) {
      const int i = g.vox(x, y, z);
      const int ixm = g.vox(wrap_low(x - 1, g.nx), y, z);
      const int iym = g.vox(x, ym, z), izm = g.vox(x, y, zm);
      const double div = ((double)F[cell_at<9>(i, CPIC_F_EX)] - (double)F[cell_at<9>(ixm, CPIC_F_EX)]) * idx +
                         ((double)F[cell_at<9>(i, CPIC_F_EY)] - (double)F[cell_at<9>(iym, CPIC_F_EY)]) * idy +
                         ((double)F[cell_at<9>(i, CPIC_F_EZ)] - (double)F[cell_at<9>(izm, CPIC_F_EZ)]) * idz;
      const double rq = rho[i] * ieps0;
      double res = div - rq;
      if (ref) res -= ref[i];
      if (resid) resid[i] = res;
      v[0] = fmax(v[0], fabs(res));
      v[1] += res * res;
      v[2] += rq * rq;
    }
  }
  block_store_partials<3>(v, sc, out, true, 1.0);
}

// Kinetic energy sum w m c^2 (gamma - 1), gamma - 1 = u^2 / (1 + gamma).
template <class R, int VL>
__global__ void __launch_bounds__(kDiagThreads)
kinetic_kernel(const unsigned char* __restrict__ part, int n, double mc2, double* __restrict__ out,
               DiagScratch* __restrict__ sc) {
  using L = PLayout<R, VL>;
  double v[1] = {0.0};
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x) {
    const double ux = *reinterpret_cast<const R*>(part + L::off(p, 3));
    const double uy = *reinterpret_cast<const R*>(part + L::off(p, 4));
    const double uz = *reinterpret_cast<const R*>(part + L::off(p, 5));
    const double w = *reinterpret_cast<const R*>(part + L::off(p, 6));
    const double u2 = ux * ux + uy * uy + uz * uz;
    v[0] += w * (u2 / (1.0 + sqrt(1.0 + u2)));
  }
  block_store_partials<1>(v, sc, out, false, mc2);
}

template <class R, int VL>
static int rho_typed(const void* particles, int n, const GridDev& g, double q_over_vol, double* rho,
                     int* bad, cudaStream_t s) {
  if (n > 0) {
    const unsigned blocks = (unsigned)(((int64_t)n + kDiagThreads - 1) / kDiagThreads);
    rho_deposit_kernel<R, VL><<<blocks, kDiagThreads, 0, s>>>(
        static_cast<const unsigned char*>(particles), n, rho, g, q_over_vol, bad);
  }
  const int planes[3] = {g.sy * g.sz, g.sx * g.sz, g.sx * g.sy};
  for (int axis = 0; axis < 3; ++axis)
    rho_fold_kernel<<<(planes[axis] + kDiagThreads - 1) / kDiagThreads, kDiagThreads, 0, s>>>(rho, g, axis);
  return launch_status();
}

static bool bad_scratch(void* sc, size_t bytes) {
  return !sc || bytes < sizeof(DiagScratch) || ((uintptr_t)sc & 7);
}

}  // namespace cpic

using namespace cpic;

// Self-test of the bounded device waits: one warp waits on phase 0 of a
// shared-memory mbarrier that expects one arrival and gets none.  The wait
// (the tiled push's warp_wait) gives up after `limit` cycles and the kernel
// sets CPIC_STATUS_PIPELINE, as the push does when one of its waits gives up.
// Nothing else is pending on the barrier, so the block then simply exits.
__global__ void __launch_bounds__(32) bounded_wait_selftest_kernel(long long limit, int* __restrict__ status) {
  __shared__ unsigned long long bar;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (!warp_wait(&bar, 0u, limit) && threadIdx.x == 0) atomicOr(status, CPIC_STATUS_PIPELINE);
}

extern "C" size_t cpic_diag_scratch_bytes(void) { return sizeof(DiagScratch); }

extern "C" int cpic_selftest_bounded_wait(int64_t limit_cycles, int32_t* d_status, cpic_stream_t stream) {
  // at most 2^31 cycles, the push's own limit
  if (!d_status || ((uintptr_t)d_status & 3) || limit_cycles < 0 || limit_cycles > (1LL << 31))
    return CPIC_EINVAL;
  bounded_wait_selftest_kernel<<<1, 32, 0, reinterpret_cast<cudaStream_t>(stream)>>>((long long)limit_cycles,
                                                                                   d_status);
  return launch_status();
}

extern "C" int cpic_charge_density(const void* particles, int64_t num_particles, const cpic_grid* grid,
                                   int32_t precision, int32_t particle_vl, double qsp, double dx,
                                   double dy, double dz, double* d_rho, int32_t* d_status,
                                   cpic_stream_t stream) {
  int rc = check_grid(grid);
  if (rc) return rc;
  if (precision != CPIC_FLOAT && precision != CPIC_DOUBLE) return CPIC_EINVAL;
  if (particle_vl != 16 && particle_vl != 32) return CPIC_EINVAL;
  if (num_particles < 0 || num_particles > 0x7fffffffLL - 64) return CPIC_EINVAL;
  if (!d_rho || !d_status || (num_particles > 0 && !particles)) return CPIC_EINVAL;
  if (!(dx > 0 && dy > 0 && dz > 0)) return CPIC_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const GridDev g = make_grid(grid);
  if (cudaMemsetAsync(d_rho, 0, sizeof(double) * (size_t)g.num_cells, s) != cudaSuccess) return CPIC_ECUDA;
  const double qv = qsp / (dx * dy * dz);
  const int n = (int)num_particles;
  if (precision == CPIC_FLOAT)
    return particle_vl == 32 ? rho_typed<float, 32>(particles, n, g, qv, d_rho, d_status, s)
                             : rho_typed<float, 16>(particles, n, g, qv, d_rho, d_status, s);
  return particle_vl == 32 ? rho_typed<double, 32>(particles, n, g, qv, d_rho, d_status, s)
                           : rho_typed<double, 16>(particles, n, g, qv, d_rho, d_status, s);
}

extern "C" int cpic_gauss_residual(const void* fields, const double* d_rho, const double* d_ref,
                                   double eps0, double dx, double dy, double dz, const cpic_grid* grid,
                                   int32_t precision, double* d_resid, double* d_out, void* d_scratch,
                                   size_t scratch_bytes, cpic_stream_t stream) {
  int rc = check_grid(grid);
  if (rc) return rc;
  if (precision != CPIC_FLOAT && precision != CPIC_DOUBLE) return CPIC_EINVAL;
  if (!fields || !d_rho || !d_out) return CPIC_EINVAL;
  if (!(dx > 0 && dy > 0 && dz > 0 && eps0 > 0)) return CPIC_EINVAL;
  if (bad_scratch(d_scratch, scratch_bytes)) return bad_scratch(d_scratch, 1 << 30) ? CPIC_EINVAL : CPIC_ESCRATCH;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  DiagScratch* sc = static_cast<DiagScratch*>(d_scratch);
  if (cudaMemsetAsync(&sc->done, 0, sizeof(unsigned), s) != cudaSuccess) return CPIC_ECUDA;
  const GridDev g = make_grid(grid);
  if (precision == CPIC_FLOAT)
    gauss_kernel<float><<<kDiagBlocks, kDiagThreads, 0, s>>>(static_cast<const float*>(fields), d_rho, d_ref,
                                                             d_resid, g, 1.0 / dx, 1.0 / dy, 1.0 / dz,
                                                             1.0 / eps0, d_out, sc);
  else
    gauss_kernel<double><<<kDiagBlocks, kDiagThreads, 0, s>>>(static_cast<const double*>(fields), d_rho, d_ref,
                                                              d_resid, g, 1.0 / dx, 1.0 / dy, 1.0 / dz,
                                                              1.0 / eps0, d_out, sc);
  return launch_status();
}

extern "C" int cpic_kinetic_energy(const void* particles, int64_t num_particles, int32_t precision,
                                   int32_t particle_vl, double mc2, double* d_out, void* d_scratch,
                                   size_t scratch_bytes, cpic_stream_t stream) {
  if (precision != CPIC_FLOAT && precision != CPIC_DOUBLE) return CPIC_EINVAL;
  if (particle_vl != 16 && particle_vl != 32) return CPIC_EINVAL;
  if (num_particles < 0 || num_particles > 0x7fffffffLL - 64) return CPIC_EINVAL;
  if (!d_out || (num_particles > 0 && !particles)) return CPIC_EINVAL;
  if (bad_scratch(d_scratch, scratch_bytes)) return bad_scratch(d_scratch, 1 << 30) ? CPIC_EINVAL : CPIC_ESCRATCH;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  DiagScratch* sc = static_cast<DiagScratch*>(d_scratch);
  if (cudaMemsetAsync(&sc->done, 0, sizeof(unsigned), s) != cudaSuccess) return CPIC_ECUDA;
  const int n = (int)num_particles;
  const unsigned char* p = static_cast<const unsigned char*>(particles);
  if (precision == CPIC_FLOAT) {
    if (particle_vl == 32) kinetic_kernel<float, 32><<<kDiagBlocks, kDiagThreads, 0, s>>>(p, n, mc2, d_out, sc);
    else kinetic_kernel<float, 16><<<kDiagBlocks, kDiagThreads, 0, s>>>(p, n, mc2, d_out, sc);
  } else {
    if (particle_vl == 32) kinetic_kernel<double, 32><<<kDiagBlocks, kDiagThreads, 0, s>>>(p, n, mc2, d_out, sc);
    else kinetic_kernel<double, 16><<<kDiagBlocks, kDiagThreads, 0, s>>>(p, n, mc2, d_out, sc);
  }
  return launch_status();
}
