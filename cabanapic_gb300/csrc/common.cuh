// common.cuh -- device-side layout access and launch helpers shared by the
// hot-path kernels.  Layouts are the reference's (include/cpic/layout.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cpic/capi.h"

namespace cpic {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kCellBlock = CPIC_CELL_BLOCK;

// Division by a fixed d >= 1 for 0 <= n < 2^31: q = (n * m) >> (31 + l) with
// l = ceil(log2 d) and m = ceil(2^(31 + l) / d) < 2^32.  Exact: the product is
// n / d plus less than n / 2^(31 + l) < 1 / d, which never reaches the next
// integer.
struct DivMagic {
  unsigned m;
  int shift;  // 31 + l
};

inline DivMagic make_div_magic(unsigned d) {
  int l = 0;
  while ((1ull << l) < d) ++l;
  DivMagic r;
  r.m = (unsigned)(((1ull << (31 + l)) + d - 1) / d);
  r.shift = 31 + l;
  return r;
}

__device__ __forceinline__ int div_magic(int n, DivMagic q) {
  return (int)(((unsigned long long)(unsigned)n * q.m) >> q.shift);
}

// Ghosted grid extents and VOXEL (src/types.h:195).
struct GridDev {
  int nx, ny, nz;   // interior cells
  int sx, sy, sz;   // ghosted extents (n + 2)
  int num_cells;    // sx * sy * sz
  DivMagic dsx, dsy;  // division by sx and sy (RANK_TO_INDEX)
  __host__ __device__ int vox(int x, int y, int z) const { return x + sx * (y + sy * z); }
};

inline GridDev make_grid(const cpic_grid* g) {
  GridDev d;
  d.nx = (int)g->nx; d.ny = (int)g->ny; d.nz = (int)g->nz;
  d.sx = d.nx + 2; d.sy = d.ny + 2; d.sz = d.nz + 2;
  d.num_cells = d.sx * d.sy * d.sz;
  d.dsx = make_div_magic((unsigned)d.sx);
  d.dsy = make_div_magic((unsigned)d.sy);
  return d;
}

// Launch shape of the per-cell stencil kernels: each warp takes K
// consecutive 32-cell AoSoA blocks of the linear cell index, so a warp's
// access to one member is one aligned 128-byte line, and a lane skips a cell
// outside the kernel's box [1, hx] x [1, hy] x [1, hz].
struct CellRange {
  int begin, end;   // linear cells [begin, end); begin is a multiple of 32
  unsigned blocks;  // launch grid of THREADS-thread blocks
};

template <int K, int THREADS>
inline CellRange cell_range(const GridDev& g, int hx, int hy, int hz) {
  CellRange r;
  r.begin = g.vox(1, 1, 1) & ~31;
  r.end = g.vox(hx, hy, hz) + 1;
  const int64_t warps = ((int64_t)(r.end - r.begin) + 32 * K - 1) / (32 * K);
  const int64_t blocks = (warps * 32 + THREADS - 1) / THREADS;
  r.blocks = (unsigned)(blocks < 1 ? 1 : blocks);
  return r;
}

// This lane's cell in the first of its warp's K blocks (the k-th is 32 k on).
template <int K, int THREADS>
__device__ __forceinline__ int lane_cell0(int begin) {
  const int64_t warp = (int64_t)blockIdx.x * (THREADS / 32) + (threadIdx.x >> 5);
  return (int)(begin + warp * (32 * K) + (threadIdx.x & 31));
}

// Whether cell c (< end) lies in the box, with its coordinates.
__device__ __forceinline__ bool cell_in_box(int c, int end, const GridDev& g, int hx, int hy, int hz,
                                            int& x, int& y, int& z) {
  if (c >= end) return false;
  y = div_magic(c, g.dsx);
  x = c - y * g.sx;
  z = div_magic(y, g.dsy);
  y -= z * g.sy;
  return x >= 1 && x <= hx && y >= 1 && y <= hy && z >= 1 && z <= hz;
}

__device__ __forceinline__ bool cell_in_box(int c, int end, const GridDev& g, int hx, int hy, int hz) {
  int x, y, z;
  return cell_in_box(c, end, g, hx, hy, hz, x, y, z);
}

// Member m of cell c in a cell AoSoA with NM members (interpolator 18, field 9).
template <int NM>
__host__ __device__ __forceinline__ size_t cell_at(int c, int m) {
  return (size_t)(c >> 5) * (NM * kCellBlock) + (size_t)m * kCellBlock + (c & 31);
}

// Particle AoSoA of vector length VL: byte offset of member m (0..6 real, 7 cell) of particle p.
template <class R, int VL>
struct PLayout {
  static constexpr size_t kBlock = (size_t)VL * (7 * sizeof(R) + sizeof(int));
  __device__ __forceinline__ static size_t off(int64_t p, int m) {
    return (size_t)(p / VL) * kBlock + (size_t)m * VL * sizeof(R) + (size_t)(p % VL) * sizeof(R);
  }
  __device__ __forceinline__ static size_t cell_off(int64_t p) {
    return (size_t)(p / VL) * kBlock + (size_t)7 * VL * sizeof(R) + (size_t)(p % VL) * sizeof(int);
  }
};

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31; }

__device__ __forceinline__ void red_add(float* a, float v) { atomicAdd(a, v); }
__device__ __forceinline__ void red_add(double* a, double v) { atomicAdd(a, v); }

// Four consecutive accumulator values (16-byte aligned) in one vector reduction.
__device__ __forceinline__ void red_add4(float* a, float v0, float v1, float v2, float v3) {
  asm volatile("red.global.add.v4.f32 [%0], {%1,%2,%3,%4};" ::"l"(a), "f"(v0), "f"(v1), "f"(v2),
               "f"(v3)
               : "memory");
}
__device__ __forceinline__ void red_add4(double* a, double v0, double v1, double v2, double v3) {
  atomicAdd(a + 0, v0); atomicAdd(a + 1, v1); atomicAdd(a + 2, v2); atomicAdd(a + 3, v3);
}

// ---- shared-memory mbarriers (CTA scope)
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
// Arrive (release): the caller's earlier shared-memory writes are visible to
// threads that then observe the phase completion.
__device__ __forceinline__ void mbar_arrive(unsigned long long* b) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}" ::"r"(smem_u32(b)) : "memory");
}
// Arrive once every cp.async copy issued so far by this thread has landed.
__device__ __forceinline__ void cp_async_mbar_arrive(unsigned long long* b) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(b)) : "memory");
}
// Arrive and add `bytes` to the phase's expected transaction count (the
// bulk copies that complete on this mbarrier count down by their sizes).
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
               : "memory");
}
// Bulk copy (the TMA engine, not the load/store pipe) of `bytes` from global
// to shared memory, completing on mbarrier b.  Both addresses 16-byte aligned,
// bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void* dst_smem, const void* src, unsigned bytes,
                                              unsigned long long* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_u32(dst_smem)), "l"(src), "r"(bytes), "r"(smem_u32(b))
               : "memory");
}
// Orders this thread's (and, after a __syncwarp, its warp's) earlier generic
// shared-memory accesses before later bulk-copy writes to the same memory.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Warp-uniform wait for the completion of phase `parity` of mbarrier b.
// Returns false, for the whole warp, after `limit` cycles (by default 2^31,
// about a second).
__device__ __forceinline__ bool warp_wait(unsigned long long* b, unsigned parity,
                                          long long limit = 1LL << 31) {
  bool done = mbar_try_wait(b, parity);
  if (__all_sync(kFull, done)) return true;
  const long long t0 = clock64();
  for (;;) {
    done = done || mbar_try_wait(b, parity);
    if (__all_sync(kFull, done)) return true;
    const int late = (clock64() - t0) > limit ? 1 : 0;
    if (__shfl_sync(kFull, late, 0)) return false;
  }
}

// Final step of a two-pass reduction, run by every thread of the last block:
// partial b of value k is part[NV * b + k], b < nparts.  Thread t combines
// partials t, t + THREADS, ... in that order, then a fixed shuffle tree and
// thread 0 over the warps: the same order on every run (deterministic), and
// the L2 loads of the partials are spread over the block instead of one
// thread's dependent chain.  Bit k of max_mask selects max instead of sum.
// res is valid in thread 0.
template <int NV, int THREADS>
__device__ __forceinline__ void reduce_partials(const double* __restrict__ part, unsigned nparts,
                                                unsigned max_mask, double (&res)[NV]) {
  __shared__ double sh[THREADS / 32][NV];
  double v[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = ((max_mask >> k) & 1u) ? -1.0e308 : 0.0;
  for (unsigned b = threadIdx.x; b < nparts; b += THREADS) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const double u = __ldcg(part + (size_t)NV * b + k);
      v[k] = ((max_mask >> k) & 1u) ? fmax(v[k], u) : v[k] + u;
    }
  }
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    for (int o = 16; o > 0; o >>= 1) {
      const double t = __shfl_xor_sync(kFull, v[k], o);
      v[k] = ((max_mask >> k) & 1u) ? fmax(v[k], t) : v[k] + t;
    }
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[threadIdx.x >> 5][k] = v[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = sh[0][k];
      for (int w = 1; w < THREADS / 32; ++w) t = ((max_mask >> k) & 1u) ? fmax(t, sh[w][k]) : t + sh[w][k];
      res[k] = t;
    }
  }
}

inline int launch_status() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? CPIC_OK : CPIC_ECUDA;
}

// Number of SMs of the current device (cached per device).
int sm_count();

// Common grid validation: periodic, one ghost layer, cell count in int range.
int check_grid(const cpic_grid* g);

}  // namespace cpic
