// fields.cu -- per-cell kernels of the step: interpolator load, accumulator
// clear/unload, periodic ghost fold and copy, the EM Yee updates and the
// field-energy reduction.
//
// Reference: src/interpolator.cpp:4-172, src/accumulator.cpp:5-122,
// src/fields.h:11-271 (ghosts), 556-719 (EM solver), 722-763 (dump_energies).
//
// The cell arrays keep the reference's AoSoA layout (32-cell blocks), so one
// warp handling 32 consecutive x cells reads and writes each member as one
// 128-byte line.  Arithmetic follows the reference operation by operation and
// this file is compiled with --fmad=false, so every field value is
// bit-identical to a CPU build of the reference without FMA contraction.  The
// energy reduction accumulates in double (the reference sums in real_t) with a
// fixed reduction tree, so it is deterministic.
#include <cuda_runtime.h>

#include <atomic>

#include "common.cuh"

namespace cpic {

constexpr int kThreads = 256;

inline unsigned blocks_for(int64_t n, int threads = kThreads) {
  int64_t b = (n + threads - 1) / threads;
  return (unsigned)(b < 1 ? 1 : b);
}

// ------------------------------------------------------------ interpolator
// load_interpolator_array (interpolator.cpp:48-136): interior cells.
template <class R>
__global__ void __launch_bounds__(kThreads)
load_interpolator_kernel(const R* __restrict__ F, R* __restrict__ I, const GridDev g, int begin, int end) {
  const int i = lane_cell0<1, kThreads>(begin);
  if (!cell_in_box(i, end, g, g.nx, g.ny, g.nz)) return;
  const int ox = 1, oy = g.sx, oz = g.sx * g.sy;
  const R fourth = 1.0 / 4.0, half = 1.0 / 2.0;
  auto f = [&](int c, int m) { return __ldg(F + cell_at<9>(c, m)); };
  const R ex0 = f(i, CPIC_F_EX), ex1 = f(i + oy, CPIC_F_EX), ex2 = f(i + oz, CPIC_F_EX),
          ex3 = f(i + oy + oz, CPIC_F_EX);
  const R ey0 = f(i, CPIC_F_EY), ey1 = f(i + oz, CPIC_F_EY), ey2 = f(i + ox, CPIC_F_EY),
          ey3 = f(i + ox + oz, CPIC_F_EY);
  const R ez0 = f(i, CPIC_F_EZ), ez1 = f(i + ox, CPIC_F_EZ), ez2 = f(i + oy, CPIC_F_EZ),
          ez3 = f(i + ox + oy, CPIC_F_EZ);
  const R bx0 = f(i, CPIC_F_CBX), bx1 = f(i + ox, CPIC_F_CBX);
  const R by0 = f(i, CPIC_F_CBY), by1 = f(i + oy, CPIC_F_CBY);
  const R bz0 = f(i, CPIC_F_CBZ), bz1 = f(i + oz, CPIC_F_CBZ);
  auto four = [&](int m0, R w0, R w1, R w2, R w3) {
    I[cell_at<18>(i, m0 + 0)] = fourth * ((w3 + w0) + (w1 + w2));
    I[cell_at<18>(i, m0 + 1)] = fourth * ((w3 - w0) + (w1 - w2));
    I[cell_at<18>(i, m0 + 2)] = fourth * ((w3 - w0) - (w1 - w2));
    I[cell_at<18>(i, m0 + 3)] = fourth * ((w3 + w0) - (w1 + w2));
  };
  four(CPIC_I_EX, ex0, ex1, ex2, ex3);
  four(CPIC_I_EY, ey0, ey1, ey2, ey3);
  four(CPIC_I_EZ, ez0, ez1, ez2, ez3);
  I[cell_at<18>(i, CPIC_I_CBX)] = half * (bx1 + bx0);
  I[cell_at<18>(i, CPIC_I_DCBXDX)] = half * (bx1 - bx0);
  I[cell_at<18>(i, CPIC_I_CBY)] = half * (by1 + by0);
  I[cell_at<18>(i, CPIC_I_DCBYDY)] = half * (by1 - by0);
  I[cell_at<18>(i, CPIC_I_CBZ)] = half * (bz1 + bz0);
  I[cell_at<18>(i, CPIC_I_DCBZDZ)] = half * (bz1 - bz0);
}

// ------------------------------------------------------------ accumulator
// unload_accumulator_array (accumulator.cpp:71-110): cells [1, n+1] per axis.
// LEFT: the accumulator in Kokkos' LayoutLeft (value k = 4 comp + q of cell c
// at c + num_cells (comp + 3 q)); the sums are the same, in the same order.
template <class R, class Acc = R, bool LEFT = false>
__global__ void __launch_bounds__(kThreads)
unload_kernel(R* __restrict__ F, const Acc* __restrict__ A, const GridDev g, Acc cx, Acc cy, Acc cz,
              int begin, int end) {
  constexpr int K = 2;
  const int c0 = lane_cell0<K, kThreads>(begin);
  const int oy = g.sx, oz = g.sx * g.sy;
  auto a = [&](int c, int k) {
    if constexpr (LEFT) return __ldg(A + (size_t)c + (size_t)g.num_cells * ((k >> 2) + 3 * (k & 3)));
    else return __ldg(A + (size_t)c * 12 + k);
  };
  Acc v[K][12];
  bool ok[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int i = c0 + 32 * k;
    ok[k] = cell_in_box(i, end, g, g.nx + 1, g.ny + 1, g.nz + 1);
    if (ok[k]) {
      // neighbours x-1, y-1, z-1 and the diagonals (accumulator.cpp:82-107)
      v[k][0] = a(i, 0); v[k][1] = a(i - oy, 1); v[k][2] = a(i - oz, 2); v[k][3] = a(i - oy - oz, 3);
      v[k][4] = a(i, 4); v[k][5] = a(i - oz, 5); v[k][6] = a(i - 1, 6); v[k][7] = a(i - 1 - oz, 7);
      v[k][8] = a(i, 8); v[k][9] = a(i - 1, 9); v[k][10] = a(i - oy, 10); v[k][11] = a(i - 1 - oy, 11);
    }
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
    if (!ok[k]) continue;
    const int i = c0 + 32 * k;
    F[cell_at<9>(i, CPIC_F_JFX)] = (R)(cx * (v[k][0] + v[k][1] + v[k][2] + v[k][3]));
    F[cell_at<9>(i, CPIC_F_JFY)] = (R)(cy * (v[k][4] + v[k][5] + v[k][6] + v[k][7]));
    F[cell_at<9>(i, CPIC_F_JFZ)] = (R)(cz * (v[k][8] + v[k][9] + v[k][10] + v[k][11]));
  }
}

// ------------------------------------------------------------ ghosts
// Periodic fold (+=) of the jf ghosts, serial_update_ghosts (fields.h:102-271).
// One block per outer index and component; the two passes of a component run
// in the reference's order, separated by a block barrier.
template <class R>
__global__ void __launch_bounds__(kThreads)
current_fold_kernel(R* __restrict__ F, const GridDev g) {
  const int comp = blockIdx.y;
  const int o = blockIdx.x + 1;
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  if (comp == 0 && o <= nx) {  // jfx, x = o: fold y then z
    for (int z = 1 + threadIdx.x; z <= nz + 1; z += blockDim.x)
      F[cell_at<9>(g.vox(o, 1, z), CPIC_F_JFX)] += F[cell_at<9>(g.vox(o, ny + 1, z), CPIC_F_JFX)];
    __syncthreads();
    for (int y = 1 + threadIdx.x; y <= ny + 1; y += blockDim.x)
      F[cell_at<9>(g.vox(o, y, 1), CPIC_F_JFX)] += F[cell_at<9>(g.vox(o, y, nz + 1), CPIC_F_JFX)];
  } else if (comp == 1 && o <= ny) {  // jfy, y = o: fold z then x
    for (int x = 1 + threadIdx.x; x <= nx + 1; x += blockDim.x)
      F[cell_at<9>(g.vox(x, o, 1), CPIC_F_JFY)] += F[cell_at<9>(g.vox(x, o, nz + 1), CPIC_F_JFY)];
    __syncthreads();
    for (int z = 1 + threadIdx.x; z <= nz + 1; z += blockDim.x)
      F[cell_at<9>(g.vox(1, o, z), CPIC_F_JFY)] += F[cell_at<9>(g.vox(nx + 1, o, z), CPIC_F_JFY)];
  } else if (comp == 2 && o <= nz) {  // jfz, z = o: fold x then y
    for (int y = 1 + threadIdx.x; y <= ny + 1; y += blockDim.x)
      F[cell_at<9>(g.vox(1, y, o), CPIC_F_JFZ)] += F[cell_at<9>(g.vox(nx + 1, y, o), CPIC_F_JFZ)];
    __syncthreads();
    for (int x = 1 + threadIdx.x; x <= nx + 1; x += blockDim.x)
      F[cell_at<9>(g.vox(x, 1, o), CPIC_F_JFZ)] += F[cell_at<9>(g.vox(x, ny + 1, o), CPIC_F_JFZ)];
  }
}

// Periodic ghost copy of three members, serial_update_ghosts_B
// (fields.h:11-100).  The reference's three face passes copy interior values
// only, so each ghost cell ends up holding the interior cell at its periodic
// image; one pass over the ghost shell does the same copies.
__device__ __forceinline__ int wrap(int c, int n) { return c == 0 ? n : (c == n + 1 ? 1 : c); }

template <class R>
__global__ void __launch_bounds__(kThreads)
ghost_copy_kernel(R* __restrict__ F, const GridDev g, int m0) {
  const int sx = g.sx, sy = g.sy, nx = g.nx, ny = g.ny, nz = g.nz;
  const int64_t zfaces = 2LL * sx * sy;        // z = 0 and z = nz+1, all x, y
  const int64_t yfaces = 2LL * sx * nz;        // y = 0 and y = ny+1, all x, z in [1, nz]
  const int64_t xfaces = 2LL * ny * nz;        // x = 0 and x = nx+1, y in [1, ny], z in [1, nz]
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int x, y, z;
  if (t < zfaces) {
    const int64_t plane = t / ((int64_t)sx * sy), r = t % ((int64_t)sx * sy);
    z = plane ? nz + 1 : 0; y = (int)(r / sx); x = (int)(r % sx);
  } else if ((t -= zfaces) < yfaces) {
    const int64_t plane = t / ((int64_t)sx * nz), r = t % ((int64_t)sx * nz);
    y = plane ? ny + 1 : 0; z = (int)(r / sx) + 1; x = (int)(r % sx);
  } else if ((t -= yfaces) < xfaces) {
    const int64_t plane = t / ((int64_t)ny * nz), r = t % ((int64_t)ny * nz);
    x = plane ? nx + 1 : 0; z = (int)(r / ny) + 1; y = (int)(r % ny) + 1;
  } else {
    return;
  }
  const int to = g.vox(x, y, z);
  const int from = g.vox(wrap(x, nx), wrap(y, ny), wrap(z, nz));
  F[cell_at<9>(to, m0 + 0)] = F[cell_at<9>(from, m0 + 0)];
  F[cell_at<9>(to, m0 + 1)] = F[cell_at<9>(from, m0 + 1)];
  F[cell_at<9>(to, m0 + 2)] = F[cell_at<9>(from, m0 + 2)];
}

template <class R>
static int ghost_copy(R* F, const GridDev& g, int m0, cudaStream_t s) {
  const int64_t n = 2LL * g.sx * g.sy + 2LL * g.sx * g.nz + 2LL * g.ny * g.nz;
  ghost_copy_kernel<R><<<blocks_for(n), kThreads, 0, s>>>(F, g, m0);
  return launch_status();
}

// ------------------------------------------------------------ EM solver
// EM_Field_Solver::advance_b (fields.h:692-717): interior cells.
template <class R>
__global__ void __launch_bounds__(kThreads)
advance_b_kernel(R* __restrict__ F, const GridDev g, R px, R py, R pz, int begin, int end) {
  constexpr int K = 2;
  const int c0 = lane_cell0<K, kThreads>(begin);
  const int oy = g.sx, oz = g.sx * g.sy;
  auto e = [&](int c, int m) { return __ldg(F + cell_at<9>(c, m)); };  // E is not written here
  R ex0[K], ey0[K], ez0[K], ezy[K], eyz[K], exz[K], ezx[K], eyx[K], exy[K], bx[K], by[K], bz[K];
  bool ok[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int f0 = c0 + 32 * k;
    ok[k] = cell_in_box(f0, end, g, g.nx, g.ny, g.nz);
    if (ok[k]) {
      ex0[k] = e(f0, CPIC_F_EX); ey0[k] = e(f0, CPIC_F_EY); ez0[k] = e(f0, CPIC_F_EZ);
      ezy[k] = e(f0 + oy, CPIC_F_EZ); eyz[k] = e(f0 + oz, CPIC_F_EY);
      exz[k] = e(f0 + oz, CPIC_F_EX); ezx[k] = e(f0 + 1, CPIC_F_EZ);
      eyx[k] = e(f0 + 1, CPIC_F_EY); exy[k] = e(f0 + oy, CPIC_F_EX);
      bx[k] = F[cell_at<9>(f0, CPIC_F_CBX)]; by[k] = F[cell_at<9>(f0, CPIC_F_CBY)];
      bz[k] = F[cell_at<9>(f0, CPIC_F_CBZ)];
    }
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
    if (!ok[k]) continue;
    const int f0 = c0 + 32 * k;
    F[cell_at<9>(f0, CPIC_F_CBX)] = bx[k] - (py * (ezy[k] - ez0[k]) - pz * (eyz[k] - ey0[k]));
    F[cell_at<9>(f0, CPIC_F_CBY)] = by[k] - (pz * (exz[k] - ex0[k]) - px * (ezx[k] - ez0[k]));
    F[cell_at<9>(f0, CPIC_F_CBZ)] = bz[k] - (px * (eyx[k] - ey0[k]) - py * (exy[k] - ex0[k]));
  }
}

// EM_Field_Solver::advance_e (fields.h:646-664): cells [1, n+1] per axis.
template <class R>
__global__ void __launch_bounds__(kThreads)
advance_e_kernel(R* __restrict__ F, const GridDev g, R px, R py, R pz, R cj, int begin, int end) {
  constexpr int K = 2;
  const int c0 = lane_cell0<K, kThreads>(begin);
  const int oy = g.sx, oz = g.sx * g.sy;
  auto b = [&](int c, int m) { return __ldg(F + cell_at<9>(c, m)); };  // B and J are not written here
  R bx0[K], by0[K], bz0[K], bzy[K], byz[K], bxz[K], bzx[K], byx[K], bxy[K], jx[K], jy[K], jz[K];
  R ex[K], ey[K], ez[K];
  bool ok[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int f0 = c0 + 32 * k;
    ok[k] = cell_in_box(f0, end, g, g.nx + 1, g.ny + 1, g.nz + 1);
    if (ok[k]) {
      bx0[k] = b(f0, CPIC_F_CBX); by0[k] = b(f0, CPIC_F_CBY); bz0[k] = b(f0, CPIC_F_CBZ);
      bzy[k] = b(f0 - oy, CPIC_F_CBZ); byz[k] = b(f0 - oz, CPIC_F_CBY);
      bxz[k] = b(f0 - oz, CPIC_F_CBX); bzx[k] = b(f0 - 1, CPIC_F_CBZ);
      byx[k] = b(f0 - 1, CPIC_F_CBY); bxy[k] = b(f0 - oy, CPIC_F_CBX);
      jx[k] = b(f0, CPIC_F_JFX); jy[k] = b(f0, CPIC_F_JFY); jz[k] = b(f0, CPIC_F_JFZ);
      ex[k] = F[cell_at<9>(f0, CPIC_F_EX)]; ey[k] = F[cell_at<9>(f0, CPIC_F_EY)];
      ez[k] = F[cell_at<9>(f0, CPIC_F_EZ)];
    }
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
    if (!ok[k]) continue;
    const int f0 = c0 + 32 * k;
    F[cell_at<9>(f0, CPIC_F_EX)] = ex[k] + (-cj * jx[k]) + (py * (bz0[k] - bzy[k]) - pz * (by0[k] - byz[k]));
    F[cell_at<9>(f0, CPIC_F_EY)] = ey[k] + (-cj * jy[k]) + (pz * (bx0[k] - bxz[k]) - px * (bz0[k] - bzx[k]));
    F[cell_at<9>(f0, CPIC_F_EZ)] = ez[k] + (-cj * jz[k]) + (px * (by0[k] - byx[k]) - py * (bx0[k] - bxy[k]));
  }
}

// ------------------------------------------------------------ energies
// e_energy / b_energy (fields.h:556-615) accumulated in double.  A fixed grid
// of kEnergyBlocks blocks writes per-block partial sums to scratch; the last
// block to finish (counter in scratch) adds them in block order.
constexpr int kEnergyBlocks = 592;  // fixed, so the sum order is device-independent

struct EnergyScratch {
  double part[2 * kEnergyBlocks];
  unsigned int done;
};

// Sum of squares per thread.  FP32: each square is split exactly into
// p + q (p = a*a rounded, q = fma(a, a, -p)), the p are summed in float-float
// (two-sum: the rounding error of every addition is kept in `lo`) and the q in
// `lo`; the thread's total hi + lo goes to the FP64 reduction.  Relative
// accuracy ~1e-14, without FP64 arithmetic per cell (slow on GB300's FP64
// pipe).  FP64: plain double sums.
template <class R>
struct SqAcc {
  double s = 0.0;
  __device__ __forceinline__ void add(R a) { s += (double)a * (double)a; }
  __device__ __forceinline__ double value() const { return s; }
};

template <>
struct SqAcc<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float a) {
    const float p = __fmul_rn(a, a);
    const float q = __fmaf_rn(a, a, -p);
    const float t = __fadd_rn(hi, p);
    const float bp = __fsub_rn(t, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    hi = t;
    lo = __fadd_rn(lo, __fadd_rn(err, q));
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

template <class R>
__global__ void __launch_bounds__(kThreads)
energy_kernel(const R* __restrict__ F, const GridDev g, double* __restrict__ out,
              EnergyScratch* __restrict__ sc) {
  __shared__ double se[kThreads / 32], sb[kThreads / 32];
  __shared__ bool last;
  // one warp per x row (y, z), lanes along x: coalesced AoSoA reads
  const unsigned rows = (unsigned)g.ny * (unsigned)g.nz;
  const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
  const int lane = threadIdx.x & 31;
  SqAcc<R> ea, ba;
  for (unsigned r = warp; r < rows; r += nwarps) {
    const int y = (int)(r % (unsigned)g.ny) + 1, z = (int)(r / (unsigned)g.ny) + 1;
    const int row = g.vox(0, y, z);
    int x = 1 + lane;
    // four x steps with their 24 loads in flight together; the sums take the
    // values in the same order as the one-step loop below
    for (; x + 96 <= g.nx; x += 128) {
      R v[4][6];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int i = row + x + 32 * j;
        v[j][0] = F[cell_at<9>(i, CPIC_F_EX)]; v[j][1] = F[cell_at<9>(i, CPIC_F_EY)];
        v[j][2] = F[cell_at<9>(i, CPIC_F_EZ)]; v[j][3] = F[cell_at<9>(i, CPIC_F_CBX)];
        v[j][4] = F[cell_at<9>(i, CPIC_F_CBY)]; v[j][5] = F[cell_at<9>(i, CPIC_F_CBZ)];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        ea.add(v[j][0]); ea.add(v[j][1]); ea.add(v[j][2]);
        ba.add(v[j][3]); ba.add(v[j][4]); ba.add(v[j][5]);
      }
    }
    for (; x <= g.nx; x += 32) {
      const int i = row + x;
      ea.add(F[cell_at<9>(i, CPIC_F_EX)]); ea.add(F[cell_at<9>(i, CPIC_F_EY)]); ea.add(F[cell_at<9>(i, CPIC_F_EZ)]);
      ba.add(F[cell_at<9>(i, CPIC_F_CBX)]); ba.add(F[cell_at<9>(i, CPIC_F_CBY)]); ba.add(F[cell_at<9>(i, CPIC_F_CBZ)]);
    }
  }
  double e = ea.value(), bb = ba.value();
  for (int o = 16; o > 0; o >>= 1) {
    e += __shfl_xor_sync(kFull, e, o);
    bb += __shfl_xor_sync(kFull, bb, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { se[w] = e; sb[w] = bb; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double te = 0.0, tb = 0.0;
    for (int k = 0; k < kThreads / 32; ++k) { te += se[k]; tb += sb[k]; }
    sc->part[2 * blockIdx.x] = te;
    sc->part[2 * blockIdx.x + 1] = tb;
    __threadfence();
    const unsigned prev = atomicAdd(&sc->done, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {  // block-uniform
    __threadfence();
    double r[2];
    reduce_partials<2, kThreads>(sc->part, gridDim.x, 0u, r);
    if (threadIdx.x == 0) {
      out[0] = r[0] * 0.5;
      out[1] = r[1] * 0.5;
      sc->done = 0;  // ready for the next call
    }
  }
}

// ------------------------------------------------------------ ES solver
// ES_Field_Solver(_1D)::advance_e (fields.h:400-436, 511-544): E -= cj J over
// every cell of the array (ghosts included, as the reference does); the 1-D
// variant folds the jf ghosts first (same fold as the EM path).
template <class R>
__global__ void __launch_bounds__(kThreads)
es_advance_e_kernel(R* __restrict__ F, int num_cells, R cj) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= num_cells) return;
  F[cell_at<9>(i, CPIC_F_EX)] = F[cell_at<9>(i, CPIC_F_EX)] + (-cj * F[cell_at<9>(i, CPIC_F_JFX)]);
  F[cell_at<9>(i, CPIC_F_EY)] = F[cell_at<9>(i, CPIC_F_EY)] + (-cj * F[cell_at<9>(i, CPIC_F_JFY)]);
  F[cell_at<9>(i, CPIC_F_EZ)] = F[cell_at<9>(i, CPIC_F_EZ)] + (-cj * F[cell_at<9>(i, CPIC_F_JFZ)]);
}

// ES e_energy (fields.h:438-463, 484-509): 0.5 sum over every cell of E^2, in
// double with the fixed-tree reduction of the EM energies (out[1] = 0).
template <class R>
__global__ void __launch_bounds__(kThreads)
es_energy_kernel(const R* __restrict__ F, int num_cells, double* __restrict__ out,
                 EnergyScratch* __restrict__ sc) {
  __shared__ double se[kThreads / 32];
  __shared__ bool last;
  double e = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < num_cells; i += gridDim.x * blockDim.x) {
    const double a0 = F[cell_at<9>(i, CPIC_F_EX)], a1 = F[cell_at<9>(i, CPIC_F_EY)], a2 = F[cell_at<9>(i, CPIC_F_EZ)];
    e += a0 * a0 + a1 * a1 + a2 * a2;
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(kFull, e, o);
  if ((threadIdx.x & 31) == 0) se[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < kThreads / 32; ++k) t += se[k];
    sc->part[2 * blockIdx.x] = t;
    sc->part[2 * blockIdx.x + 1] = 0.0;
    __threadfence();
    last = (atomicAdd(&sc->done, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {  // block-uniform
    __threadfence();
    double r[2];
    reduce_partials<2, kThreads>(sc->part, gridDim.x, 0u, r);
    if (threadIdx.x == 0) {
      out[0] = r[0] * 0.5;
      out[1] = 0.0;
      sc->done = 0;
    }
  }
}

// ------------------------------------------------------------ host side
template <class R>
static int typed_load_interp(const void* f, void* i, const GridDev& g, cudaStream_t s) {
  const CellRange r = cell_range<1, kThreads>(g, g.nx, g.ny, g.nz);
  load_interpolator_kernel<R><<<r.blocks, kThreads, 0, s>>>(static_cast<const R*>(f), static_cast<R*>(i), g,
                                                            r.begin, r.end);
  return launch_status();
}

template <class R, class Acc = R, bool LEFT = false>
static int typed_unload(void* f, const void* a, const GridDev& g, double dx, double dy, double dz,
                        double dt, cudaStream_t s) {
  const R rdx = (R)dx, rdy = (R)dy, rdz = (R)dz, rdt = (R)dt;
  // cx = 0.25 / (dy*dz*dt) with the double literal (accumulator.cpp:66-68)
  const R cx = (R)(0.25 / (double)(R)(rdy * rdz * rdt));
  const R cy = (R)(0.25 / (double)(R)(rdz * rdx * rdt));
  const R cz = (R)(0.25 / (double)(R)(rdx * rdy * rdt));
  const CellRange r = cell_range<2, kThreads>(g, g.nx + 1, g.ny + 1, g.nz + 1);
  unload_kernel<R, Acc, LEFT><<<r.blocks, kThreads, 0, s>>>(static_cast<R*>(f), static_cast<const Acc*>(a), g,
                                                      (Acc)cx, (Acc)cy, (Acc)cz, r.begin, r.end);
  return launch_status();
}

template <class R>
static int typed_advance_b(void* f, double px, double py, double pz, const GridDev& g, cudaStream_t s) {
  const CellRange r = cell_range<2, kThreads>(g, g.nx, g.ny, g.nz);
  advance_b_kernel<R><<<r.blocks, kThreads, 0, s>>>(static_cast<R*>(f), g, (R)px, (R)py, (R)pz, r.begin,
                                                    r.end);
  int rc = launch_status();
  if (rc) return rc;
  return ghost_copy<R>(static_cast<R*>(f), g, CPIC_F_CBX, s);
}

template <class R>
static int typed_advance_e(void* f, double px, double py, double pz, double dt_eps0,
                           const GridDev& g, cudaStream_t s) {
  R* F = static_cast<R*>(f);
  int outer = g.nx > g.ny ? g.nx : g.ny;
  outer = outer > g.nz ? outer : g.nz;
  current_fold_kernel<R><<<dim3((unsigned)outer, 3), 128, 0, s>>>(F, g);
  int rc = launch_status();
  if (rc) return rc;
  rc = ghost_copy<R>(F, g, CPIC_F_JFX, s);
  if (rc) return rc;
  const CellRange r = cell_range<2, kThreads>(g, g.nx + 1, g.ny + 1, g.nz + 1);
  advance_e_kernel<R><<<r.blocks, kThreads, 0, s>>>(F, g, (R)px, (R)py, (R)pz, (R)dt_eps0, r.begin, r.end);
  return launch_status();
}

template <class R>
static int typed_energies(const void* f, const GridDev& g, double* out, void* scratch, cudaStream_t s) {
  energy_kernel<R><<<kEnergyBlocks, kThreads, 0, s>>>(static_cast<const R*>(f), g, out,
                                                      static_cast<EnergyScratch*>(scratch));
  return launch_status();
}

int sm_count() {
  static std::atomic<int> cached[64];  // per device, 0: not yet queried
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  int n = cached[dev].load(std::memory_order_relaxed);
  if (n == 0) {
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 1;
    cached[dev].store(n, std::memory_order_relaxed);
  }
  return n;
}

int check_grid(const cpic_grid* g) {
  if (!g) return CPIC_EINVAL;
  if (g->nx < 1 || g->ny < 1 || g->nz < 1) return CPIC_EINVAL;
  if (g->boundary != CPIC_PERIODIC && g->boundary != CPIC_REFLECT) return CPIC_EINVAL;
  if (g->boundary == CPIC_REFLECT) return CPIC_EUNSUPPORTED;  // the reference exit(1)s
  if (g->num_ghosts != 1) return CPIC_EUNSUPPORTED;           // the reference assumes one layer
  const int64_t cells = (g->nx + 2) * (g->ny + 2) * (g->nz + 2);
  if (g->nx > (1 << 20) || g->ny > (1 << 20) || g->nz > (1 << 20) || cells > 0x7fffffffLL - 64)
    return CPIC_EINVAL;
  return CPIC_OK;
}

}  // namespace cpic

using namespace cpic;

#define CPIC_CHECK_PREC(p) \
  if ((p) != CPIC_FLOAT && (p) != CPIC_DOUBLE) return CPIC_EINVAL

extern "C" int cpic_load_interpolator(const void* fields, void* interpolators, const cpic_grid* grid,
                                      int32_t precision, cpic_stream_t stream) {
  int rc = check_grid(grid);
  if (rc) return rc;
  CPIC_CHECK_PREC(precision);
  if (!fields || !interpolators) return CPIC_EINVAL;
  const GridDev g = make_grid(grid);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  return precision == CPIC_FLOAT ? typed_load_interp<float>(fields, interpolators, g, s)
                                 : typed_load_interp<double>(fields, interpolators, g, s);
}

extern "C" int cpic_initialize_interpolator(void* interpolators, int64_t num_cells, int32_t precision,
                                            cpic_stream_t stream) {
  CPIC_CHECK_PREC(precision);
  if (!interpolators || num_cells < 0) return CPIC_EINVAL;
  const size_t bytes = cpic_cell_array_bytes(num_cells, CPIC_INTERP_MEMBERS, precision);
  return cudaMemsetAsync(interpolators, 0, bytes, reinterpret_cast<cudaStream_t>(stream)) == cudaSuccess
             ? CPIC_OK : CPIC_ECUDA;
}

extern "C" int cpic_clear_accumulator(void* accumulators, int64_t num_cells, int32_t precision,
                                      cpic_stream_t stream) {
  CPIC_CHECK_PREC(precision);
  if (!accumulators || num_cells < 0) return CPIC_EINVAL;
  const size_t bytes = (size_t)num_cells * CPIC_ACC_VALUES * (size_t)precision;
  return cudaMemsetAsync(accumulators, 0, bytes, reinterpret_cast<cudaStream_t>(stream)) == cudaSuccess
             ? CPIC_OK : CPIC_ECUDA;
}

extern "C" int cpic_unload_accumulator(void* fields, const void* accumulators, const cpic_grid* grid,
                                       double dx, double dy, double dz, double dt, int32_t precision,
                                       cpic_stream_t stream) {
  int rc = check_grid(grid);
  if (rc) return rc;
  CPIC_CHECK_PREC(precision);
  if (!fields || !accumulators) return CPIC_EINVAL;
  const GridDev g = make_grid(grid);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  return precision == CPIC_FLOAT ? typed_unload<float>(fields, accumulators, g, dx, dy, dz, dt, s)
                                 : typed_unload<double>(fields, accumulators, g, dx, dy, dz, dt, s);
}

extern "C" int cpic_unload_accumulator_left(void* fields, const void* accumulators, const cpic_grid* grid,
                                            double dx, double dy, double dz, double dt, int32_t precision,
                                            cpic_stream_t stream) {
  int rc = check_grid(grid);
  if (rc) return rc;
  CPIC_CHECK_PREC(precision);
  if (!fields || !accumulators) return CPIC_EINVAL;
  const GridDev g = make_grid(grid);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  return precision == CPIC_FLOAT ? typed_unload<float, float, true>(fields, accumulators, g, dx, dy, dz, dt, s)
                                 : typed_unload<double, double, true>(fields, accumulators, g, dx, dy, dz, dt, s);
}

extern "C" int cpic_unload_accumulator_f64(void* fields, const double* accumulators, const cpic_grid* grid,
                                           double dx, double dy, double dz, double dt, int32_t precision,
                                           cpic_stream_t stream) {
  int rc = check_grid(grid);
  if (rc) return rc;
  CPIC_CHECK_PREC(precision);
  if (!fields || !accumulators) return CPIC_EINVAL;
  const GridDev g = make_grid(grid);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  return precision == CPIC_FLOAT ? typed_unload<float, double>(fields, accumulators, g, dx, dy, dz, dt, s)
                                 : typed_unload<double>(fields, accumulators, g, dx, dy, dz, dt, s);
}

extern "C" int cpic_advance_b(void* fields, double px, double py, double pz, const cpic_grid* grid,
                              int32_t precision, cpic_stream_t stream) {
  int rc = check_grid(grid);
  if (rc) return rc;
  CPIC_CHECK_PREC(precision);
  if (!fields) return CPIC_EINVAL;
  const GridDev g = make_grid(grid);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  return precision == CPIC_FLOAT ? typed_advance_b<float>(fields, px, py, pz, g, s)
                                 : typed_advance_b<double>(fields, px, py, pz, g, s);
}

extern "C" int cpic_advance_e(void* fields, double px, double py, double pz, const cpic_grid* grid,
                              double dt_eps0, int32_t precision, cpic_stream_t stream) {
  int rc = check_grid(grid);
  if (rc) return rc;
  CPIC_CHECK_PREC(precision);
  if (!fields) return CPIC_EINVAL;
  const GridDev g = make_grid(grid);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  return precision == CPIC_FLOAT ? typed_advance_e<float>(fields, px, py, pz, dt_eps0, g, s)
                                 : typed_advance_e<double>(fields, px, py, pz, dt_eps0, g, s);
}

extern "C" size_t cpic_energy_scratch_bytes(void) { return sizeof(EnergyScratch); }

extern "C" int cpic_field_energies(const void* fields, const cpic_grid* grid, int32_t precision,
                                   double* d_out, void* d_scratch, size_t scratch_bytes,
                                   cpic_stream_t stream) {
  int rc = check_grid(grid);
  if (rc) return rc;
  CPIC_CHECK_PREC(precision);
  if (!fields || !d_out || !d_scratch) return CPIC_EINVAL;
  if (scratch_bytes < sizeof(EnergyScratch)) return CPIC_ESCRATCH;
  if (((uintptr_t)d_scratch & 7) || ((uintptr_t)d_out & 7)) return CPIC_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  // the completion counter must start at zero: clear it (the kernel leaves it zero)
  if (cudaMemsetAsync(&static_cast<EnergyScratch*>(d_scratch)->done, 0, sizeof(unsigned), s) != cudaSuccess)
    return CPIC_ECUDA;
  const GridDev g = make_grid(grid);
  return precision == CPIC_FLOAT ? typed_energies<float>(fields, g, d_out, d_scratch, s)
                                 : typed_energies<double>(fields, g, d_out, d_scratch, s);
}

// ------------------------------------------------------------ energies without allocation
// Some callers cannot allocate device memory: a host code whose device memory
// is all owned by its own pool or arena, a language binding that has no CUDA
// runtime allocator to call, or a per-step diagnostic that must not allocate
// in the middle of a time loop.  cpic_field_energies_noalloc serves them: the
// energy reduction's scratch (one partial sum pair per block of the fixed
// 592-block launch, plus the completion counter: 9,480 bytes) lives in the
// static device array below.  Every GPU that loads this library holds the
// array until the process exits.
static_assert(sizeof(EnergyScratch) == 9480, "static energy scratch size is documented as 9,480 bytes");
static __device__ __align__(256) EnergyScratch g_energy_noalloc_scratch;

// Device address of g_energy_noalloc_scratch in the current device's context.
// The array's name in host code is only a host-side stand-in, so the address
// is looked up with that device current, on every call: a cached address
// would go stale if the context were destroyed and recreated (for example by
// cudaDeviceReset), which reloads the module, possibly elsewhere.  Once the
// module is loaded the lookup is a host-side table read.  The first call on a
// device may load the module (lazy loading), which is why that first call
// should come before any stream capture.
static EnergyScratch* energy_noalloc_scratch() {
  void* addr = nullptr;
  if (cudaGetSymbolAddress(&addr, g_energy_noalloc_scratch) != cudaSuccess || addr == nullptr)
    return nullptr;
  return static_cast<EnergyScratch*>(addr);
}

extern "C" int cpic_field_energies_noalloc(const void* fields, const cpic_grid* grid,
                                           int32_t precision, double* d_out,
                                           cpic_stream_t stream) {
  // The scratch need is fixed (592 block partials), so every grid the library
  // accepts fits; check_grid rejects the rest (n > 2^20 per axis, >= 2^31 cells).
  int rc = check_grid(grid);
  if (rc) return rc;
  CPIC_CHECK_PREC(precision);
  if (!fields || !d_out) return CPIC_EINVAL;
  if ((uintptr_t)d_out & 7) return CPIC_EINVAL;
  EnergyScratch* sc = energy_noalloc_scratch();
  if (sc == nullptr) return CPIC_ECUDA;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  // the array keeps the previous call's contents: the counter must start at zero
  if (cudaMemsetAsync(&sc->done, 0, sizeof(unsigned), s) != cudaSuccess) return CPIC_ECUDA;
  const GridDev g = make_grid(grid);
  return precision == CPIC_FLOAT ? typed_energies<float>(fields, g, d_out, sc, s)
                                 : typed_energies<double>(fields, g, d_out, sc, s);
}

extern "C" int cpic_es_advance_e(void* fields, const cpic_grid* grid, double dt_eps0, int32_t fold_ghosts,
                                 int32_t precision, cpic_stream_t stream) {
  int rc = check_grid(grid);
  if (rc) return rc;
  CPIC_CHECK_PREC(precision);
  if (!fields) return CPIC_EINVAL;
  const GridDev g = make_grid(grid);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int outer = g.nx > g.ny ? g.nx : g.ny;
  outer = outer > g.nz ? outer : g.nz;
  if (precision == CPIC_FLOAT) {
    if (fold_ghosts) current_fold_kernel<float><<<dim3((unsigned)outer, 3), 128, 0, s>>>(static_cast<float*>(fields), g);
    es_advance_e_kernel<float><<<blocks_for(g.num_cells), kThreads, 0, s>>>(static_cast<float*>(fields), g.num_cells,
                                                                           (float)dt_eps0);
  } else {
    if (fold_ghosts) current_fold_kernel<double><<<dim3((unsigned)outer, 3), 128, 0, s>>>(static_cast<double*>(fields), g);
    es_advance_e_kernel<double><<<blocks_for(g.num_cells), kThreads, 0, s>>>(static_cast<double*>(fields), g.num_cells,
                                                                            dt_eps0);
  }
  return launch_status();
}

extern "C" int cpic_es_e_energy(const void* fields, const cpic_grid* grid, int32_t precision, double* d_out,
                                void* d_scratch, size_t scratch_bytes, cpic_stream_t stream) {
  int rc = check_grid(grid);
  if (rc) return rc;
  CPIC_CHECK_PREC(precision);
  if (!fields || !d_out || !d_scratch) return CPIC_EINVAL;
  if (scratch_bytes < sizeof(EnergyScratch)) return CPIC_ESCRATCH;
  if (((uintptr_t)d_scratch & 7) || ((uintptr_t)d_out & 7)) return CPIC_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  EnergyScratch* sc = static_cast<EnergyScratch*>(d_scratch);
  if (cudaMemsetAsync(&sc->done, 0, sizeof(unsigned), s) != cudaSuccess) return CPIC_ECUDA;
  const GridDev g = make_grid(grid);
  if (precision == CPIC_FLOAT)
    es_energy_kernel<float><<<kEnergyBlocks, kThreads, 0, s>>>(static_cast<const float*>(fields), g.num_cells, d_out, sc);
  else
    es_energy_kernel<double><<<kEnergyBlocks, kThreads, 0, s>>>(static_cast<const double*>(fields), g.num_cells, d_out, sc);
  return launch_status();
}

extern "C" int cpic_status_clear(int32_t* d_status, cpic_stream_t stream) {
  if (!d_status) return CPIC_EINVAL;
  return cudaMemsetAsync(d_status, 0, sizeof(int32_t), reinterpret_cast<cudaStream_t>(stream)) == cudaSuccess
             ? CPIC_OK : CPIC_ECUDA;
}

extern "C" int cpic_status_read(const int32_t* d_status, cpic_stream_t stream, int32_t* h_status) {
  if (!d_status || !h_status) return CPIC_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (cudaMemcpyAsync(h_status, d_status, sizeof(int32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return CPIC_ECUDA;
  return cudaStreamSynchronize(s) == cudaSuccess ? CPIC_OK : CPIC_ECUDA;
}

extern "C" int cpic_version(void) { return 1; }

extern "C" const char* cpic_strerror(int code) {
  switch (code) {
    case CPIC_OK: return "ok";
    case CPIC_EINVAL: return "invalid argument";
    case CPIC_EUNSUPPORTED: return "unsupported (Reflect boundary or num_ghosts != 1)";
    case CPIC_ECUDA: return "CUDA error";
    case CPIC_ESCRATCH: return "scratch buffer too small";
    default: return "unknown cpic error";
  }
}
