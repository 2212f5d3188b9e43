// push_impl.cuh -- particle push with charge-conserving current deposit.
//
// GB300 implementation of push() (reference src/push.h:7-300) and of the
// move_p it calls for cell-crossing particles (src/move_p.h:9-374).  This
// header is compiled twice, into different namespaces (CPIC_PUSH_NS):
//   push.cu       exact variant: --fmad=false, IEEE division and sqrtf.  A
//                 particle's new offset and momentum are bit-identical to a CPU
//                 build of the reference compiled without FMA contraction.
//   push_fast.cu  production variant: fused multiply-adds and the hardware
//                 reciprocal / reciprocal square root for the three gamma and
//                 Boris divisions (FP32).  Per-particle results agree with the
//                 exact arithmetic to ~1e-6 relative (tested at the 1e-5
//                 tolerance stated for FP32).
//
// Two kernels share the per-particle arithmetic (one CUDA thread per particle,
// one warp per 32-particle AoSoA chunk, the next chunk's eight members held in
// registers while the current one is processed):
//
//   push_kernel (CPIC_PUSH_STREAMING).  Warps stream 32-particle chunks: 18 read-only
//   gathers per particle; in-cell deposits are reduced by shuffles over the
//   largest group of lanes sharing a cell (all of them once particles are in
//   cell order: a 13-shuffle reduce-scatter leaves 12 totals for 12 lanes,
//   one atomic each), the other lanes use 16-byte vector reductions
//   (red.global.add.v4.f32).
//   push_tiled_kernel (default).  A 512-thread CTA takes tiles of
//   32 * 15 * chunks_per_warp consecutive particles.  Once particles are in
//   cell order a tile covers a short run of voxels; its cell window is a
//   segment of wx voxels [c0, c0 + wx) around that run together with the
//   segments offset by -1 and +1 in y (stride sx) and in z (stride sx*sy): 5
//   segments, a cross, holding the cells the tile's particles reach within a
//   sort interval except those displaced in both y and z (the diagonal rows;
//   the 9-segment block is a build option, CPIC_TILE_WINDOW).  Warp 0 is a producer:
//   it anchors each tile's window on the median of 32 sampled cells and stages
//   the 18 interpolator coefficients of the window's cells in shared memory
//   (rows of 20 values, 16-byte aligned) with cp.async, into two buffers
//   handed over through mbarriers.  Warps 1..15 push the particles: a gather
//   is five vector shared loads instead of 18 dependent global loads; a
//   particle whose cell has no slot gathers from global memory, so results do
//   not depend on the order or the tile shape, only the speed does.  Deposits
//   as in push_kernel.  (Measured and dropped: a shared accumulator window, since
//   shared float atomics are compare-and-swap loops and the global reductions
//   of reduced groups are cheap; and a CTA-wide barrier per tile in place of
//   the producer warp, which cost a fifth of the warps' time in barrier stalls.)
//
// In both, cell-crossing particles are compacted into a per-warp shared-memory
// queue (ballot + prefix popcount) holding the particle's offsets, remaining
// displacement, charge, cell and index; whenever 32 are queued the warp moves
// them together, so the common path stays branch-free and the streak loop
// runs on full warps.  The streak loop is capped; hitting the cap sets
// CPIC_STATUS_MOVER_CAP.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "common.cuh"

#ifndef CPIC_PUSH_NS
#error "define CPIC_PUSH_NS before including push_impl.cuh"
#endif

namespace cpic {

// Where value vi = 4 comp + q of a cell's accumulator lives: LayoutRight rows
// [cell][3][4] (12 contiguous values, the reference's host build), or the
// Kokkos-Cuda default LayoutLeft [q][comp][cell] (value (comp, q) of cell c
// at c + n (comp + 3 q), n = num_cells: src/types.h:120 under a Cuda build).
struct AccMap {
  int left;  // 0: LayoutRight
  int n;     // the accumulator's first extent (num_cells)
  __device__ __forceinline__ size_t at(int cell, int vi) const {
    return left ? (size_t)cell + (size_t)n * (size_t)((vi >> 2) + 3 * (vi & 3)) : (size_t)cell * 12 + vi;
  }
};

template <class R>
struct PushArgs {
  R qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp;
  GridDev g;
  AccMap acc;
};

// Cell window of one tile: segments [c0 + off_s, c0 + off_s + wx) with
// off_s = (kz - 1) * sx * sy + (ky - 1) * sx for the rows (ky, kz) of the
// window's shape (segment_start).
struct TileWin {
  int c0, wx;
};

namespace CPIC_PUSH_NS {

constexpr int kPushThreads = 256;
constexpr int kWarps = kPushThreads / 32;
constexpr int kQueueCap = 64;    // per warp: drained whenever it holds >= 32
constexpr int kMaxStreaks = 16;  // a Courant-limited move needs at most 4
constexpr int kRow = 20;         // window row: 18 coefficients + 2 pad

template <class R>
struct MoverQueue {
  R px[kQueueCap], py[kQueueCap], pz[kQueueCap];  // offsets before the move
  R dx[kQueueCap], dy[kQueueCap], dz[kQueueCap];  // normalised half displacement
  R q[kQueueCap];
  int cell[kQueueCap];
  int idx[kQueueCap];
};

// 1 / sqrt(1 + u^2) factors of push.h:148,169.  The reference calls sqrtf even
// for real_t = double (LITERAL keeps that).  FAST (FP32 only) uses the
// hardware reciprocal square root.
template <class R, bool LITERAL, bool FAST>
__device__ __forceinline__ R scaled_rgamma(R num, R arg) {
  if constexpr (sizeof(R) == 4 && FAST) {
    return num * rsqrtf(arg);
  } else if constexpr (sizeof(R) == 8 && LITERAL) {
    return num / (R)sqrtf((float)arg);
  } else if constexpr (sizeof(R) == 8) {
    return num / sqrt(arg);
  } else {
    return num / sqrtf(arg);
  }
}

template <class R, bool FAST>
__device__ __forceinline__ R quotient(R a, R b) {
  if constexpr (sizeof(R) == 4 && FAST) return __fdividef(a, b);
  else return a / b;
}

// Four quadrant currents of one axis (src/push.h:218-232, src/move_p.h:156-170).
template <class R>
__device__ __forceinline__ void quad(R qu, R da, R db, R corr, R& a0, R& a1, R& a2, R& a3) {
  const R one = 1;
  R t = qu;
  a1 = t * da;
  a0 = t - a1;
  a1 += t;
  R s = one + db;
  a2 = a0 * s;
  a3 = a1 * s;
  s = one - db;
  a0 *= s;
  a1 *= s;
  a0 += corr;
  a1 -= corr;
  a2 -= corr;
  a3 += corr;
}

template <class R>
__device__ __forceinline__ void currents12(R q, R ux, R uy, R uz, R mx, R my, R mz, R corr,
                                           R v[12]) {
  quad<R>(q * ux, my, mz, corr, v[0], v[1], v[2], v[3]);    // jx: CALC_J(x,y,z)
  quad<R>(q * uy, mz, mx, corr, v[4], v[5], v[6], v[7]);    // jy: CALC_J(y,z,x)
  quad<R>(q * uz, mx, my, corr, v[8], v[9], v[10], v[11]);  // jz: CALC_J(z,x,y)
}

// Sum of v[0..11] over the 32 lanes, scattered: afterwards lane l holds the
// total of value index value_of_lane(l) (12 lanes hold distinct values).
template <class R>
__device__ __forceinline__ R reduce_scatter12(const R v[12], int lane) {
  const bool h16 = lane & 16, h8 = lane & 8, h4 = lane & 4, h2 = lane & 2;
  R a[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    R send = h16 ? v[k] : v[k + 6];
    R keep = h16 ? v[k + 6] : v[k];
    a[k] = keep + __shfl_xor_sync(kFull, send, 16);
  }
  R b[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    R send = h8 ? a[k] : a[k + 3];
    R keep = h8 ? a[k + 3] : a[k];
    b[k] = keep + __shfl_xor_sync(kFull, send, 8);
  }
  // third level over (b0, b1, b2, 0)
  R c0 = (h4 ? b[2] : b[0]) + __shfl_xor_sync(kFull, h4 ? b[0] : b[2], 4);
  R c1 = (h4 ? R(0) : b[1]) + __shfl_xor_sync(kFull, h4 ? b[1] : R(0), 4);
  R d = (h2 ? c1 : c0) + __shfl_xor_sync(kFull, h2 ? c0 : c1, 2);
  return d + __shfl_xor_sync(kFull, d, 1);
}

// Value index held by `lane` after reduce_scatter12, or -1.
__device__ __forceinline__ int value_of_lane(int lane) {
  if (lane & 1) return -1;
  int j = ((lane & 4) ? 2 : 0) + ((lane & 2) ? 1 : 0);
  if (j == 3) return -1;
  return ((lane & 16) ? 6 : 0) + ((lane & 8) ? 3 : 0) + j;
}

// Adds 12 deposits to one accumulator row (16-byte vector reductions for
// FP32 rows; FP64 rows, the compensated accumulation, take scalar atomics).
template <class R, class Acc>
__device__ __forceinline__ void red_add12(Acc* __restrict__ a, const R v[12]) {
  red_add4(a + 0, (Acc)v[0], (Acc)v[1], (Acc)v[2], (Acc)v[3]);
  red_add4(a + 4, (Acc)v[4], (Acc)v[5], (Acc)v[6], (Acc)v[7]);
  red_add4(a + 8, (Acc)v[8], (Acc)v[9], (Acc)v[10], (Acc)v[11]);
}

// Adds 12 deposits to `cell`'s accumulator values in either layout (LayoutLeft:
// 12 scalar reductions, n apart).
template <class R, class Acc>
__device__ __forceinline__ void red_add12(Acc* __restrict__ acc, const AccMap& m, int cell, const R v[12]) {
  if (m.left) {
#pragma unroll
    for (int k = 0; k < 12; ++k) red_add(acc + m.at(cell, k), (Acc)v[k]);
  } else {
    red_add12(acc + (size_t)cell * 12, v);
  }
}

// Deposit of the in-cell particles of one warp into accumulator_array.  `dep`
// lanes add v[0..11] to accumulator row `cell`; `vi` is value_of_lane(lane).
template <class R, class Acc>
__device__ __forceinline__ void warp_deposit(Acc* __restrict__ acc, const AccMap& am, int cell, bool dep,
                                             const R v[12], int lane, int vi) {
  const unsigned dm = __ballot_sync(kFull, dep);
  if (dm == 0u) return;
  const int cell0 = __shfl_sync(kFull, cell, __ffs(dm) - 1);
  if (__all_sync(kFull, !dep || cell == cell0)) {  // every depositing lane in one cell
    R w[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) w[k] = dep ? v[k] : R(0);
    const R tot = reduce_scatter12<R>(w, lane);
    if (vi >= 0) red_add(acc + am.at(cell0, vi), (Acc)tot);
    return;
  }
  const int key = dep ? cell : -1 - lane;
  const unsigned peers = __match_any_sync(kFull, key);
  const unsigned score = dep ? ((unsigned)__popc(peers) << 5) | (unsigned)(31 - (__ffs(peers) - 1)) : 0u;
  const unsigned best = __reduce_max_sync(kFull, score);
  const int bsize = (int)(best >> 5);
  const int leader = 31 - (int)(best & 31);
  bool in_major = false;
  if (bsize >= 2) {  // warp-uniform
    in_major = dep && ((peers >> leader) & 1u);
    R w[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) w[k] = in_major ? v[k] : R(0);
    const R tot = reduce_scatter12<R>(w, lane);
    const int major_cell = __shfl_sync(kFull, cell, leader);
    if (vi >= 0) red_add(acc + am.at(major_cell, vi), (Acc)tot);
  }
  if (dep && !in_major) red_add12(acc, am, cell, v);
}

// Twice the fractional distance to a face, (dir - p) / s (move_p.h:115-117).
// FAST (FP32): the hardware division, within 2 ulp; two faces closer than
// that may then be crossed in the other order, with a streak of ~1e-7 of the
// displacement between them.  Displacements below 1e-30 count as none.
template <class R, bool FAST>
__device__ __forceinline__ R face_fraction(R dir, R p, R s) {
  if constexpr (sizeof(R) == 4 && FAST) {
    return (fabsf(s) < 1e-30f) ? R(3.4e38) : __fdividef(dir - p, s);
  } else {
    return (s == 0) ? R(3.4e38) : (dir - p) / s;
  }
}

// move_p for one particle (src/move_p.h:93-371), positions and displacement in
// registers; writes the final offsets and cell of particle `pidx`.
template <class R, int VL, bool FAST, class Acc>
__device__ __forceinline__ void move_one(unsigned char* __restrict__ part, R px, R py, R pz, R dx,
                                      R dy, R dz, R q, int cell, int pidx, Acc* __restrict__ acc,
                                      const GridDev g, const AccMap& am, int* __restrict__ status) {
  using L = PLayout<R, VL>;
  if (!(isfinite(dx) && isfinite(dy) && isfinite(dz))) atomicOr(status, CPIC_STATUS_NONFINITE);
  bool done = false;
  for (int it = 0; it < kMaxStreaks; ++it) {
    if ((unsigned)cell >= (unsigned)g.num_cells) {
      atomicOr(status, CPIC_STATUS_CELL_RANGE);
      done = true;
      break;
    }
    R sx = dx, sy = dy, sz = dz;
    const R dirx = (sx > 0) ? R(1) : R(-1);
    const R diry = (sy > 0) ? R(1) : R(-1);
    const R dirz = (sz > 0) ? R(1) : R(-1);
    // twice the fractional distance to each face (move_p.h:115-117)
    const R fx = face_fraction<R, FAST>(dirx, px, sx);
    const R fy = face_fraction<R, FAST>(diry, py, sy);
    const R fz = face_fraction<R, FAST>(dirz, pz, sz);
    R len = 2;
    int axis = 3;
    if (fx < len) { len = fx; axis = 0; }
    if (fy < len) { len = fy; axis = 1; }
    if (fz < len) { len = fz; axis = 2; }
    len *= R(0.5);
    sx *= len; sy *= len; sz *= len;
    const R mx = px + sx, my = py + sy, mz = pz + sz;
    // correction with the double 1/3 literal of move_p.h:154
    const R corr = (R)((double)(q * sx * sy * sz) * (1. / 3.));
    R v[12];
    currents12<R>(q, sx, sy, sz, mx, my, mz, corr, v);
    red_add12(acc, am, cell, v);
    dx -= sx; dy -= sy; dz -= sz;
    px += sx + sx; py += sy + sy; pz += sz + sz;
    if (axis == 3) { done = true; break; }

    const R fs = (axis == 0) ? dirx : (axis == 1) ? diry : dirz;
    // RANK_TO_INDEX (src/types.h:184-193); cell is in [0, num_cells) here
    int ix = cell, iy, iz;
    iy = div_magic(ix, g.dsx); ix -= iy * g.sx;
    iz = div_magic(iy, g.dsy); iy -= iz * g.sy;
    const int step = fs > 0 ? 1 : -1;
    if (axis == 0) ix += step; else if (axis == 1) iy += step; else iz += step;
    // detect_leaving_domain (move_p.h:9-54): the last matching test wins
    int leaving = -1;
    if (ix == 0) leaving = 0;
    if (iy == 0) leaving = 1;
    if (iz == 0) leaving = 2;
    if (ix == g.nx + 1) leaving = 3;
    if (iy == g.ny + 1) leaving = 4;
    if (iz == g.nz + 1) leaving = 5;
    // periodic wrap (move_p.h:271-288), one ghost layer
    if (leaving == 0) ix = g.nx;
    else if (leaving == 1) iy = g.ny;
    else if (leaving == 2) iz = g.nz;
    else if (leaving == 3) ix = 1;
    else if (leaving == 4) iy = 1;
    else if (leaving == 5) iz = 1;
    cell = g.vox(ix, iy, iz);
    // land on the face of the new cell (move_p.h:225-227, 368-370)
    if (axis == 0) px = -fs; else if (axis == 1) py = -fs; else pz = -fs;
  }
  if (!done) atomicOr(status, CPIC_STATUS_MOVER_CAP);
  *reinterpret_cast<R*>(part + L::off(pidx, 0)) = px;
  *reinterpret_cast<R*>(part + L::off(pidx, 1)) = py;
  *reinterpret_cast<R*>(part + L::off(pidx, 2)) = pz;
  *reinterpret_cast<int*>(part + L::cell_off(pidx)) = cell;
}

// The eight members of one particle.
template <class R>
struct PState {
  R x, y, z, ux, uy, uz, w;
  int cell;
};

template <class R, int VL>
__device__ __forceinline__ void load_state(const unsigned char* __restrict__ chunk_base, int lane_off,
                                           int lane_cell_off, bool valid, PState<R>& s) {
  constexpr int kMem = VL * (int)sizeof(R);
  if (valid) {
    const unsigned char* b = chunk_base + lane_off;
    s.x = __ldcs(reinterpret_cast<const R*>(b + 0 * kMem));
    s.y = __ldcs(reinterpret_cast<const R*>(b + 1 * kMem));
    s.z = __ldcs(reinterpret_cast<const R*>(b + 2 * kMem));
    s.ux = __ldcs(reinterpret_cast<const R*>(b + 3 * kMem));
    s.uy = __ldcs(reinterpret_cast<const R*>(b + 4 * kMem));
    s.uz = __ldcs(reinterpret_cast<const R*>(b + 5 * kMem));
    s.w = __ldcs(reinterpret_cast<const R*>(b + 6 * kMem));
    s.cell = __ldcs(reinterpret_cast<const int*>(chunk_base + lane_cell_off));
  } else {
    s.x = s.y = s.z = s.ux = s.uy = s.uz = s.w = R(0);
    s.cell = 0;
  }
}

// The 18 interpolator coefficients of one cell, in interpolator_array member
// order (src/types.h interpolator members, src/push.h:74-93).
template <class R>
struct Coeffs {
  R ex, dexdy, dexdz, d2exdydz;
  R ey, deydz, deydx, d2eydzdx;
  R ez, dezdx, dezdy, d2ezdxdy;
  R cbx, dcbxdx, cby, dcbydy;
  R cbz, dcbzdz;
};

template <class R>
__device__ __forceinline__ void gather_global(const R* __restrict__ interp, int cell, Coeffs<R>& c) {
  const R* f = interp + ((size_t)(cell >> 5) * (18 * kCellBlock) + (cell & 31));
  c.ex = __ldg(f + 0 * 32); c.dexdy = __ldg(f + 1 * 32);
  c.dexdz = __ldg(f + 2 * 32); c.d2exdydz = __ldg(f + 3 * 32);
  c.ey = __ldg(f + 4 * 32); c.deydz = __ldg(f + 5 * 32);
  c.deydx = __ldg(f + 6 * 32); c.d2eydzdx = __ldg(f + 7 * 32);
  c.ez = __ldg(f + 8 * 32); c.dezdx = __ldg(f + 9 * 32);
  c.dezdy = __ldg(f + 10 * 32); c.d2ezdxdy = __ldg(f + 11 * 32);
  c.cbx = __ldg(f + 12 * 32); c.dcbxdx = __ldg(f + 13 * 32);
  c.cby = __ldg(f + 14 * 32); c.dcbydy = __ldg(f + 15 * 32);
  c.cbz = __ldg(f + 16 * 32); c.dcbzdz = __ldg(f + 17 * 32);
}

__device__ __forceinline__ void gather_row(const float* row, Coeffs<float>& c) {
  const float4 a = *reinterpret_cast<const float4*>(row + 0);
  const float4 b = *reinterpret_cast<const float4*>(row + 4);
  const float4 d = *reinterpret_cast<const float4*>(row + 8);
  const float4 e = *reinterpret_cast<const float4*>(row + 12);
  const float2 f = *reinterpret_cast<const float2*>(row + 16);
  c.ex = a.x; c.dexdy = a.y; c.dexdz = a.z; c.d2exdydz = a.w;
  c.ey = b.x; c.deydz = b.y; c.deydx = b.z; c.d2eydzdx = b.w;
  c.ez = d.x; c.dezdx = d.y; c.dezdy = d.z; c.d2ezdxdy = d.w;
  c.cbx = e.x; c.dcbxdx = e.y; c.cby = e.z; c.dcbydy = e.w;
  c.cbz = f.x; c.dcbzdz = f.y;
}

__device__ __forceinline__ void gather_row(const double* row, Coeffs<double>& c) {
  const double2* r = reinterpret_cast<const double2*>(row);
  double2 t;
  t = r[0]; c.ex = t.x; c.dexdy = t.y;
  t = r[1]; c.dexdz = t.x; c.d2exdydz = t.y;
  t = r[2]; c.ey = t.x; c.deydz = t.y;
  t = r[3]; c.deydx = t.x; c.d2eydzdx = t.y;
  t = r[4]; c.ez = t.x; c.dezdx = t.y;
  t = r[5]; c.dezdy = t.x; c.d2ezdxdy = t.y;
  t = r[6]; c.cbx = t.x; c.dcbxdx = t.y;
  t = r[7]; c.cby = t.x; c.dcbydy = t.y;
  t = r[8]; c.cbz = t.x; c.dcbzdz = t.y;
}

// Field at the particle, relativistic Boris rotation with half E kicks
// (push.h:124-163).  Updates (ux, uy, uz) in place.
template <class R, bool LITERAL, bool FAST>
__device__ __forceinline__ void boris(const Coeffs<R>& c, R x, R y, R z, R& ux, R& uy, R& uz,
                                      const R qdt_2mc) {
  const R one = 1., one_third = 1. / 3., two_fifteenths = 2. / 15.;
  const R hax = qdt_2mc * ((c.ex + y * c.dexdy) + z * (c.dexdz + y * c.d2exdydz));
  const R hay = qdt_2mc * ((c.ey + z * c.deydz) + x * (c.deydx + z * c.d2eydzdx));
  const R haz = qdt_2mc * ((c.ez + x * c.dezdx) + y * (c.dezdy + x * c.d2ezdxdy));
  const R cbx = c.cbx + x * c.dcbxdx;
  const R cby = c.cby + y * c.dcbydy;
  const R cbz = c.cbz + z * c.dcbzdz;
  ux += hax; uy += hay; uz += haz;
  const R b0 = scaled_rgamma<R, LITERAL, FAST>(qdt_2mc, one + (ux * ux + (uy * uy + uz * uz)));
  const R b1 = cbx * cbx + (cby * cby + cbz * cbz);
  const R b2 = (b0 * b0) * b1;
  const R b3 = b0 * (one + b2 * (one_third + b2 * two_fifteenths));
  R b4 = quotient<R, FAST>(b3, one + b1 * (b3 * b3));
  b4 += b4;
  const R tx = ux + b3 * (uy * cbz - uz * cby);
  const R ty = uy + b3 * (uz * cbx - ux * cbz);
  const R tz = uz + b3 * (ux * cby - uy * cbx);
  ux += b4 * (ty * cbz - tz * cby);
  uy += b4 * (tz * cbx - tx * cbz);
  uz += b4 * (tx * cby - ty * cbx);
  ux += hax; uy += hay; uz += haz;
}

// Per-warp constants of the chunk loop.
struct LaneCtx {
  int lane, vi, lane_off, lane_cell_off;
  unsigned lt_mask;
};

__host__ __device__ __forceinline__ int window_slot(int cell, const TileWin& w, int ys, int zs);

// One 32-particle chunk: gather, Boris, in-cell move and deposit, queueing of
// the crossers.  TILED gathers from the shared-memory window `wbuf` when the
// particle's cell has a slot in window `w`.
template <class R, int VL, bool LITERAL, bool FAST, bool TILED, class Acc, bool OUT = false>
__device__ __forceinline__ void push_chunk(unsigned char* __restrict__ part, int n, int chunk,
                                           const PState<R>& cur, const R* __restrict__ interp,
                                           Acc* __restrict__ acc, const PushArgs<R>& a,
                                           int* __restrict__ status, MoverQueue<R>& Q, int& qn,
                                           const LaneCtx& lc, const R* __restrict__ wbuf,
                                           const TileWin& w, int ys, int zs) {
  constexpr int kMem = VL * (int)sizeof(R);
  constexpr size_t kChunk = (size_t)32 * (7 * sizeof(R) + sizeof(int));
  const R one = 1., one_third = 1. / 3.;
  unsigned char* base = part + (size_t)chunk * kChunk;
  const int p = chunk * 32 + lc.lane;
  bool valid = p < n;
  const bool inrange = valid;
  const R x = cur.x, y = cur.y, z = cur.z;
  R ux = cur.ux, uy = cur.uy, uz = cur.uz;
  int cell = cur.cell;
  if (valid && (unsigned)cell >= (unsigned)a.g.num_cells) {
    atomicOr(status, CPIC_STATUS_CELL_RANGE);
    valid = false;
    cell = 0;
  }
  Coeffs<R> c;
  int li = -1;
  if constexpr (TILED) {
    li = valid ? window_slot(cell, w, ys, zs) : -1;
    if (li >= 0) gather_row(wbuf + li * kRow, c);
    else gather_global<R>(interp, cell, c);
  } else {
    gather_global<R>(interp, cell, c);
  }
  boris<R, LITERAL, FAST>(c, x, y, z, ux, uy, uz, a.qdt_2mc);
  if (valid) {
    __stcs(reinterpret_cast<R*>(base + lc.lane_off + 3 * kMem), ux);
    __stcs(reinterpret_cast<R*>(base + lc.lane_off + 4 * kMem), uy);
    __stcs(reinterpret_cast<R*>(base + lc.lane_off + 5 * kMem), uz);
    if constexpr (OUT) __stcs(reinterpret_cast<R*>(base + lc.lane_off + 6 * kMem), cur.w);
  } else if (OUT && inrange) {  // a skipped particle is copied unchanged to the output list
    __stcs(reinterpret_cast<R*>(base + lc.lane_off + 0 * kMem), x);
    __stcs(reinterpret_cast<R*>(base + lc.lane_off + 1 * kMem), y);
    __stcs(reinterpret_cast<R*>(base + lc.lane_off + 2 * kMem), z);
    __stcs(reinterpret_cast<R*>(base + lc.lane_off + 3 * kMem), cur.ux);
    __stcs(reinterpret_cast<R*>(base + lc.lane_off + 4 * kMem), cur.uy);
    __stcs(reinterpret_cast<R*>(base + lc.lane_off + 5 * kMem), cur.uz);
    __stcs(reinterpret_cast<R*>(base + lc.lane_off + 6 * kMem), cur.w);
    __stcs(reinterpret_cast<int*>(base + lc.lane_cell_off), cur.cell);
  }

  // normalised half displacement and the in-cell test (push.h:169-187)
  const R rg = scaled_rgamma<R, LITERAL, FAST>(one, one + (ux * ux + (uy * uy + uz * uz)));
  ux *= a.cdt_dx; uy *= a.cdt_dy; uz *= a.cdt_dz;
  ux *= rg; uy *= rg; uz *= rg;
  const R mx = x + ux, my = y + uy, mz = z + uz;
  const R nx = mx + ux, ny = my + uy, nz = mz + uz;
  const R q = cur.w * a.qsp;
  const bool inb = valid && (nx <= one && ny <= one && nz <= one && -nx <= one && -ny <= one &&
                             -nz <= one);
  if (inb) {
    __stcs(reinterpret_cast<R*>(base + lc.lane_off + 0 * kMem), nx);
    __stcs(reinterpret_cast<R*>(base + lc.lane_off + 1 * kMem), ny);
    __stcs(reinterpret_cast<R*>(base + lc.lane_off + 2 * kMem), nz);
    if constexpr (OUT) __stcs(reinterpret_cast<int*>(base + lc.lane_cell_off), cell);
  }
  R v[12];
  const R corr = q * ux * uy * uz * one_third;
  currents12<R>(q, ux, uy, uz, mx, my, mz, corr, v);
  warp_deposit<R, Acc>(acc, a.acc, cell, inb, v, lc.lane, lc.vi);

  // compact the cell-crossing particles into the warp queue
  const bool cross = valid && !inb;
  const unsigned cm = __ballot_sync(kFull, cross);
  if (cm) {
    if (cross) {
      const int s = qn + __popc(cm & lc.lt_mask);
      Q.px[s] = x; Q.py[s] = y; Q.pz[s] = z;
      Q.dx[s] = ux; Q.dy[s] = uy; Q.dz[s] = uz;
      Q.q[s] = q; Q.cell[s] = cell; Q.idx[s] = p;
    }
    qn += __popc(cm);
    if (qn >= 32) {
      __syncwarp();
      const int s = qn - 32 + lc.lane;
      const R ex0 = Q.px[s], ey0 = Q.py[s], ez0 = Q.pz[s];
      const R ddx = Q.dx[s], ddy = Q.dy[s], ddz = Q.dz[s], qq = Q.q[s];
      const int cc = Q.cell[s], ii = Q.idx[s];
      __syncwarp();
      qn -= 32;
      move_one<R, VL, FAST, Acc>(part, ex0, ey0, ez0, ddx, ddy, ddz, qq, cc, ii, acc, a.g, a.acc, status);
    }
  }
}

template <class R, int VL>
__device__ __forceinline__ LaneCtx make_lane_ctx() {
  constexpr int kBlk = VL * (7 * (int)sizeof(R) + (int)sizeof(int));
  constexpr int kMem = VL * (int)sizeof(R);
  LaneCtx lc;
  lc.lane = (int)lane_id();
  lc.lt_mask = (1u << lc.lane) - 1u;
  lc.vi = value_of_lane(lc.lane);
  lc.lane_off = (lc.lane / VL) * kBlk + (lc.lane % VL) * (int)sizeof(R);
  lc.lane_cell_off = (lc.lane / VL) * kBlk + 7 * kMem + (lc.lane % VL) * (int)sizeof(int);
  return lc;
}

template <class R, int VL, bool FAST, class Acc>
__device__ __forceinline__ void drain_queue(unsigned char* __restrict__ part, MoverQueue<R>& Q, int qn,
                                            int lane, const PushArgs<R>& a, Acc* __restrict__ acc,
                                            int* __restrict__ status) {
  __syncwarp();
  if (lane < qn)
    move_one<R, VL, FAST, Acc>(part, Q.px[lane], Q.py[lane], Q.pz[lane], Q.dx[lane], Q.dy[lane], Q.dz[lane],
                    Q.q[lane], Q.cell[lane], Q.idx[lane], acc, a.g, a.acc, status);
}

// ------------------------------------------------------------ streaming kernel
template <class R, int VL, bool LITERAL, bool FAST, class Acc>
__global__ void __launch_bounds__(kPushThreads, sizeof(R) == 4 ? 4 : 2)  // FP32: 64 registers
push_kernel(unsigned char* __restrict__ part, int n, const R* __restrict__ interp,
            Acc* __restrict__ acc, const PushArgs<R> a, int* __restrict__ status) {
  constexpr size_t kChunk = (size_t)32 * (7 * sizeof(R) + sizeof(int));
  __shared__ MoverQueue<R> queues[kWarps];
  MoverQueue<R>& Q = queues[threadIdx.x >> 5];
  const LaneCtx lc = make_lane_ctx<R, VL>();
  const int nchunks = (n + 31) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const TileWin nowin{0, 0};
  int qn = 0;

  int chunk = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  PState<R> cur;
  load_state<R, VL>(part + (size_t)chunk * kChunk, lc.lane_off, lc.lane_cell_off,
                    chunk < nchunks && chunk * 32 + lc.lane < n, cur);
  for (; chunk < nchunks; chunk += nwarps) {
    const int next = chunk + nwarps;
    PState<R> nxt;
    load_state<R, VL>(part + (size_t)next * kChunk, lc.lane_off, lc.lane_cell_off,
                      next < nchunks && next * 32 + lc.lane < n, nxt);
    push_chunk<R, VL, LITERAL, FAST, false, Acc>(part, n, chunk, cur, interp, acc, a, status, Q, qn, lc,
                                            nullptr, nowin, 0, 0);
    cur = nxt;
  }
  drain_queue<R, VL, FAST, Acc>(part, Q, qn, lc.lane, a, acc, status);
}

// ------------------------------------------------------------ tiled kernel
// Shape of a tile's window, as segments of rows (y offset ky, z offset kz,
// each 0..2 for -1, 0, +1): 9 = the 3 x 3 rows around the tile's row; 3 = the
// tile's plane only (ky = 0..2, kz = 1); 5 = a cross, the tile's plane and the
// tile's row in the planes above and below (the diagonal rows left out).
// Measured at 128^3 x 64 ppc, look-ahead sort keys (mean push ms): 9 rows,
// 7 chunks, 44 voxels 2.301-2.302; 5 rows, 7 chunks, 56 or 64 voxels
// 2.271-2.273 (8 chunks 2.276, 6 chunks 2.298, 48 voxels 2.308); 3 rows, 7
// chunks, 64 voxels 2.311 (fastest where the list is in cell order, slowest
// 10 steps away from it, when a sixth of the particles sit in another plane).
#ifndef CPIC_TILE_WINDOW
#define CPIC_TILE_WINDOW 5
#endif
static_assert(CPIC_TILE_WINDOW == 9 || CPIC_TILE_WINDOW == 5 || CPIC_TILE_WINDOW == 3, "window: 9, 5 or 3 rows");
constexpr int kWinSeg = CPIC_TILE_WINDOW;  // window segments

// Segment of rows (ky, kz), or -1 if the window leaves them out.
__host__ __device__ __forceinline__ int row_segment(int ky, int kz) {
  if constexpr (kWinSeg == 9) return ky + 3 * kz;
  if (kz == 1) return ky;
  if constexpr (kWinSeg == 5) return ky == 1 ? (kz == 0 ? 3 : 4) : -1;
  return -1;
}

// Slot of `cell` in the window, or -1.  With r = cell - c0 + sx*sy + sx the
// rows around the tile's are r = dx + ky * ys + kz * zs, dx < wx <= ys.
__host__ __device__ __forceinline__ int window_slot(int cell, const TileWin& w, int ys, int zs) {
  int r = cell - w.c0 + ys + zs;
  if ((unsigned)r >= (unsigned)(3 * zs)) return -1;
  const int kz = (r >= zs) + (r >= 2 * zs);
  r -= kz * zs;
  const int ky = (r >= ys) + (r >= 2 * ys);
  r -= ky * ys;
  const int sg = row_segment(ky, kz);
  return (r < w.wx && sg >= 0) ? r + w.wx * sg : -1;
}

// First voxel of window segment s.
__host__ __device__ __forceinline__ int segment_start(const TileWin& w, int s, int ys, int zs) {
  int ky, kz;
  if (kWinSeg == 9) { kz = s / 3; ky = s - 3 * kz; }
  else if (s < 3) { ky = s; kz = 1; }
  else { ky = 1; kz = s == 3 ? 0 : 2; }
  return w.c0 + (kz - 1) * zs + (ky - 1) * ys;
}

// Window of a tile from the cells of 32 of its particles, one per lane (the
// first particle of every 32nd part of the tile).  Some steps after a sort a
// sampled particle may sit one cell away in y or z (a voxel index off by sx
// or sx*sy), so the anchor is the median sample, and the run [lo, hi] is
// taken over the samples within wxmax voxels of it.  Warp-uniform result.
__device__ __forceinline__ TileWin window_from_samples(int c, int lane, int wxmax, int num_cells) {
  if ((unsigned)c >= (unsigned)num_cells) c = 0;
  int sorted = c;  // bitonic sort of the 32 samples, ascending over the lanes
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      const int o = __shfl_xor_sync(kFull, sorted, j);
      const bool up = (lane & k) == 0;
      const bool low = (lane & j) == 0;
      sorted = (low == up) ? min(sorted, o) : max(sorted, o);
    }
  }
  const int m = __shfl_sync(kFull, sorted, 16);
  const bool near = c >= m - wxmax && c <= m + wxmax;
  const int lo = __reduce_min_sync(kFull, near ? c : 0x7fffffff);
  const int hi = __reduce_max_sync(kFull, near ? c : -1);
  TileWin w;
  if (hi - lo <= wxmax - 3) {
    w.c0 = lo - 1;
    w.wx = hi - lo + 3;
  } else {
    w.wx = wxmax;
    w.c0 = m - (wxmax >> 1);
  }
  return w;
}

template <class R>
__device__ __forceinline__ void cp_async_elem(R* dst_smem, const R* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
  if constexpr (sizeof(R) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Window segment of slot i: s = floor(i / wx), exact in float for i < 9 * 64.
__device__ __forceinline__ int slot_segment(int i, float inv_wx) {
  return min((int)(((float)i + 0.5f) * inv_wx), kWinSeg - 1);
}

// Issues the copies of the window's interpolator rows; cells outside the
// array read as 0.  One copy instruction covers 8 cells x 4 members: lane l
// takes slot 8g + l / 4 and members l % 4, l % 4 + 4, ...  Rows are 20 words,
// so the 8 slots start in 8 distinct banks (20 * slot mod 32) and the 4
// members fill the banks between: each copy writes 32 distinct banks.
template <class R>
__device__ __forceinline__ void stage_window(R* __restrict__ buf, const R* __restrict__ interp,
                                             const TileWin w, int ys, int zs, int num_cells, int lane) {
  const int ncell = kWinSeg * w.wx;
  const float inv_wx = 1.0f / (float)w.wx;
  const int q = lane & 3;
  for (int i = lane >> 2; i < ncell; i += 8) {
    const int s = slot_segment(i, inv_wx);
    const int gc = segment_start(w, s, ys, zs) + (i - s * w.wx);
    R* row = buf + i * kRow;
    if ((unsigned)gc < (unsigned)num_cells) {
      const R* src = interp + ((size_t)(gc >> 5) * (18 * kCellBlock) + (gc & 31));
#pragma unroll
      for (int m = q; m < 18; m += 4) cp_async_elem<R>(row + m, src + m * kCellBlock);
    } else {
#pragma unroll
      for (int m = q; m < 18; m += 4) row[m] = R(0);
    }
  }
}

#ifndef CPIC_TILE_BULK
#define CPIC_TILE_BULK 0  // stage windows with per-element cp.async (0, faster) or bulk copies (1)
#endif

// Window staging through the bulk-copy (TMA) engine.  Each of the segments
// of wx <= 64 voxels lies in at most 3 consecutive 32-cell AoSoA blocks of
// the interpolator array (cell arrays hold whole blocks: cpic_cell_array_bytes);
// lane 0 copies those blocks whole (18 x 32 values each) into one of two
// landing buffers, completing on the buffer's mbarrier, while the warp
// transposes the previous segment from its landing buffer into window rows
// (18 conflict-free 4-byte shared loads per 32 cells, 16-byte row stores).
// The global reads take no load/store-pipe instructions, which the
// consumers' gathers, deposits and particle stream need.  Measured at 128^3 x
// 64 ppc it is not faster: the landing buffers' 14 KB per CTA take the
// shared-memory carveout to its maximum, L1 shrinks from ~60 KB to ~28 KB,
// and the global gathers of drifted particles, which hit L1, slow down (mean
// push 2.51 -> 2.77 ms; with 5-chunk tiles, whose windows cover the tile,
// 2.56 -> 2.54 ms).  Kept as a build option (CPIC_TILE_BULK=1).
constexpr int kLandBlocks = 3;  // blocks per landing buffer

// values per landing buffer
constexpr size_t kLandElems = (size_t)kLandBlocks * 18 * kCellBlock;

// Copy state of the producer's two landing buffers.
struct LandState {
  unsigned parity;  // bit k: parity of buffer k's next phase
  unsigned pending;  // bit k: a phase of buffer k issued and not yet waited for
};

// Issues segment s of window w into landing buffer k (lane 0; the warp first
// finishes its reads of that buffer).  Valid cells of the segment: [lo, hi).
template <class R>
__device__ __forceinline__ void land_issue(R* __restrict__ land, unsigned long long* lbar, LandState& ls,
                                           const R* __restrict__ interp, const TileWin& w, int s, int ys,
                                           int zs, int nc, int lane) {
  const int k = s & 1;
  const int a = segment_start(w, s, ys, zs);
  const int lo = max(a, 0), hi = min(a + w.wx, nc);
  const int blo = lo >> 5;
  const int nb = lo < hi ? ((hi - 1) >> 5) - blo + 1 : 0;
  __syncwarp();
  if (lane == 0) {
    fence_proxy_async_smem();
    constexpr unsigned kBlk = 18 * kCellBlock * sizeof(R);
    if (nb > 0) {
      mbar_arrive_expect_tx(&lbar[k], (unsigned)nb * kBlk);
      for (int j = 0; j < nb; ++j)
        bulk_copy_g2s(land + k * kLandElems + (size_t)j * 18 * kCellBlock,
                      interp + (size_t)(blo + j) * (18 * kCellBlock), kBlk, &lbar[k]);
    } else {
      mbar_arrive(&lbar[k]);
    }
  }
  ls.pending |= 1u << k;
}

// Waits for segment s's landing buffer and writes the segment's window rows
// (cells outside the array read as 0).  False if the wait gave up.
template <class R>
__device__ __forceinline__ bool land_transpose(R* __restrict__ buf, const R* __restrict__ land,
                                               unsigned long long* lbar, LandState& ls, const TileWin& w,
                                               int s, int ys, int zs, int nc, int lane) {
  const int k = s & 1;
  if (!warp_wait(&lbar[k], (ls.parity >> k) & 1u)) return false;
  ls.parity ^= 1u << k;
  ls.pending &= ~(1u << k);
  const int a = segment_start(w, s, ys, zs);
  const int lo = max(a, 0), hi = min(a + w.wx, nc);
  const int base = (lo >> 5) << 5;
  const R* lk = land + k * kLandElems;
  for (int x = lane; x < w.wx; x += 32) {
    const int gc = a + x;
    R v[18];
    if (gc >= lo && gc < hi) {
      const int li = gc - base;
      const R* src = lk + (li >> 5) * (18 * kCellBlock) + (li & 31);
#pragma unroll
      for (int m = 0; m < 18; ++m) v[m] = src[m * kCellBlock];
    } else {
#pragma unroll
      for (int m = 0; m < 18; ++m) v[m] = R(0);
    }
    R* row = buf + (size_t)(s * w.wx + x) * kRow;
    if constexpr (sizeof(R) == 4) {
      float4* r4 = reinterpret_cast<float4*>(row);
      r4[0] = make_float4(v[0], v[1], v[2], v[3]);
      r4[1] = make_float4(v[4], v[5], v[6], v[7]);
      r4[2] = make_float4(v[8], v[9], v[10], v[11]);
      r4[3] = make_float4(v[12], v[13], v[14], v[15]);
      *reinterpret_cast<float2*>(row + 16) = make_float2(v[16], v[17]);
    } else {
      double2* r2 = reinterpret_cast<double2*>(row);
#pragma unroll
      for (int q = 0; q < 9; ++q) r2[q] = make_double2(v[2 * q], v[2 * q + 1]);
    }
  }
  return true;
}

// Stages all segments of window w into buf: segment s + 1's copy is in
// flight while segment s is transposed.  False if a wait gave up.
template <class R>
__device__ __forceinline__ bool stage_window_bulk(R* __restrict__ buf, R* __restrict__ land,
                                                  unsigned long long* lbar, LandState& ls,
                                                  const R* __restrict__ interp, const TileWin& w, int ys,
                                                  int zs, int nc, int lane) {
  land_issue<R>(land, lbar, ls, interp, w, 0, ys, zs, nc, lane);
  for (int s = 0; s < kWinSeg; ++s) {
    if (s + 1 < kWinSeg) land_issue<R>(land, lbar, ls, interp, w, s + 1, ys, zs, nc, lane);
    if (!land_transpose<R>(buf, land, lbar, ls, w, s, ys, zs, nc, lane)) return false;
  }
  return true;
}

constexpr int kTiledThreads = 512;                // tiled kernel: 16 warps per CTA
constexpr int kConsumers = kTiledThreads / 32 - 1;  // warps 1..15 push; warp 0 stages windows

template <class R>
constexpr size_t tiled_dyn_smem(int wxmax) {
  return (size_t)kWinSeg * wxmax * 2 * kRow * sizeof(R) + (CPIC_TILE_BULK ? 2 * kLandElems * sizeof(R) : 0);
}

// Cell of the lane-th sample particle of tile t (tiles of T particles).
template <class R, int VL>
__device__ __forceinline__ int tile_sample(const unsigned char* __restrict__ part, int n, int T, int t,
                                           int lane) {
  using L = PLayout<R, VL>;
  int64_t p = (int64_t)t * T + (int64_t)lane * (T >> 5);
  if (p > n - 1) p = n - 1;
  return __ldcg(reinterpret_cast<const int*>(part + L::cell_off(p)));
}

// Warp 0 produces: for tile j it waits until the consumers have released
// buffer j % 2 (used by tile j - 2), computes the window from the samples,
// publishes it and stages the rows with cp.async; each lane arrives on
// full[j % 2] twice, once when its copies land and once (release) after its
// plain shared stores.  Warps 1..7 consume: they wait for full[j % 2], push
// their chunks of tile j gathering from the window, and arrive on
// empty[j % 2].  No CTA-wide barrier: a warp delayed by a queue drain holds up
// nobody until the producer needs its buffer again.
// OUT: particles are read from `src` and written, all members, to the
// same slots of `part` (a distinct list); otherwise `part` is pushed in place.
template <class R, int VL, bool LITERAL, bool FAST, class Acc, bool OUT = false>
__global__ void __launch_bounds__(kTiledThreads, sizeof(R) == 4 ? 2 : 1)  // FP32: 64 registers
push_tiled_kernel(unsigned char* __restrict__ part, int n, const R* __restrict__ interp,
                  Acc* __restrict__ acc, const PushArgs<R> a, int* __restrict__ status,
                  int chunks_per_warp, int wxmax, const unsigned char* __restrict__ src) {
  const unsigned char* in = OUT ? src : part;
  constexpr size_t kChunk = (size_t)32 * (7 * sizeof(R) + sizeof(int));
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* const wbuf = reinterpret_cast<R*>(smem_raw);  // two windows of 9 * wxmax rows
  __shared__ MoverQueue<R> queues[kConsumers];
  __shared__ TileWin wins[2];
  __shared__ __align__(8) unsigned long long full[2], empty[2], lbar[2];
  const int warp = threadIdx.x >> 5;
  const LaneCtx lc = make_lane_ctx<R, VL>();
  const int cpt = kConsumers * chunks_per_warp;  // chunks per tile
  const int T = 32 * cpt;                        // particles per tile
  const int ntiles = (int)(((int64_t)n + T - 1) / T);
  const int nchunks = (n + 31) >> 5;
  const int ys = a.g.sx, zs = a.g.sx * a.g.sy, nc = a.g.num_cells;
  const int G = gridDim.x;
  const size_t wrows = (size_t)kWinSeg * wxmax * kRow;
  if ((int)blockIdx.x >= ntiles) return;
  R* const land = wbuf + 2 * wrows;  // bulk staging: two landing buffers after the windows
  if (threadIdx.x == 0) {
    // producer lanes arrive on full twice (cp.async staging) or once (bulk staging)
    mbar_init(&full[0], CPIC_TILE_BULK ? 32 : 64);
    mbar_init(&full[1], CPIC_TILE_BULK ? 32 : 64);
    mbar_init(&empty[0], kConsumers);
    mbar_init(&empty[1], kConsumers);
    mbar_init(&lbar[0], 1);
    mbar_init(&lbar[1], 1);
  }
  __syncthreads();

  if (warp == 0 && CPIC_TILE_BULK) {  // ------------------------ producer, bulk staging
    int s_cur = tile_sample<R, VL>(in, n, T, blockIdx.x, lc.lane);
    int s_nxt = (int)blockIdx.x + G < ntiles ? tile_sample<R, VL>(in, n, T, blockIdx.x + G, lc.lane) : 0;
    LandState ls{0u, 0u};
    bool ok = true;
    int j = 0;
    for (int t = blockIdx.x; t < ntiles; t += G, ++j) {
      const int b = j & 1;
      if (j >= 2 && !warp_wait(&empty[b], (unsigned)((j >> 1) - 1) & 1u)) {
        ok = false;
        break;
      }
      const TileWin w = window_from_samples(s_cur, lc.lane, wxmax, nc);
      s_cur = s_nxt;
      if (t + 2 * G < ntiles) s_nxt = tile_sample<R, VL>(in, n, T, t + 2 * G, lc.lane);
      if (lc.lane == 0) wins[b] = w;
      if (!stage_window_bulk<R>(wbuf + b * wrows, land, lbar, ls, interp, w, ys, zs, nc, lc.lane)) {
        ok = false;
        break;
      }
      mbar_arrive(&full[b]);
    }
    if (!ok) {
      // copies still in flight land before the block exits (bounded waits)
      for (int k = 0; k < 2; ++k)
        if ((ls.pending >> k) & 1u) warp_wait(&lbar[k], (ls.parity >> k) & 1u);
      if (lc.lane == 0) atomicOr(status, CPIC_STATUS_PIPELINE);
    }
    return;
  }

  if (warp == 0) {  // ---------------------------------------- producer, cp.async staging
    int s_cur = tile_sample<R, VL>(in, n, T, blockIdx.x, lc.lane);
    int s_nxt = (int)blockIdx.x + G < ntiles ? tile_sample<R, VL>(in, n, T, blockIdx.x + G, lc.lane) : 0;
    bool ok = true;
    int j = 0;
    for (int t = blockIdx.x; t < ntiles; t += G, ++j) {
      const int b = j & 1;
      if (j >= 2 && !warp_wait(&empty[b], (unsigned)((j >> 1) - 1) & 1u)) {
        ok = false;
        break;
      }
      const TileWin w = window_from_samples(s_cur, lc.lane, wxmax, nc);
      s_cur = s_nxt;
      if (t + 2 * G < ntiles) s_nxt = tile_sample<R, VL>(in, n, T, t + 2 * G, lc.lane);
      if (lc.lane == 0) wins[b] = w;
      stage_window<R>(wbuf + b * wrows, interp, w, ys, zs, nc, lc.lane);
      cp_async_mbar_arrive(&full[b]);
      mbar_arrive(&full[b]);
    }
    cp_async_wait_all();
    if (!ok && lc.lane == 0) atomicOr(status, CPIC_STATUS_PIPELINE);
    return;
  }

  // ---------------------------------------------------------- consumers
  const int cw = warp - 1;
  MoverQueue<R>& Q = queues[cw];
  int qn = 0;
  int t = blockIdx.x;
  int chunk = t * cpt + cw;
  PState<R> cur;
  load_state<R, VL>(in + (size_t)chunk * kChunk, lc.lane_off, lc.lane_cell_off,
                    chunk < nchunks && chunk * 32 + lc.lane < n, cur);
  bool ok = true;
  for (int j = 0; t < ntiles; ++j, t += G) {
    const int b = j & 1;
    if (!warp_wait(&full[b], (unsigned)(j >> 1) & 1u)) {
      ok = false;
      break;
    }
    const TileWin w = wins[b];
    const R* const wb = wbuf + b * wrows;
    const int t1 = t + G;
    for (int i = 0; i < chunks_per_warp; ++i) {
      chunk = t * cpt + cw + kConsumers * i;
      const bool last = i + 1 == chunks_per_warp;
      const int next = last ? t1 * cpt + cw : chunk + kConsumers;
      PState<R> nxt;
      load_state<R, VL>(in + (size_t)next * kChunk, lc.lane_off, lc.lane_cell_off,
                        (!last || t1 < ntiles) && next < nchunks && next * 32 + lc.lane < n, nxt);
      if (chunk < nchunks)
        push_chunk<R, VL, LITERAL, FAST, true, Acc, OUT>(part, n, chunk, cur, interp, acc, a, status, Q, qn,
                                               lc, wb, w, ys, zs);
      cur = nxt;
    }
    __syncwarp();
    if (lc.lane == 0) mbar_arrive(&empty[b]);
  }
  if (!ok && lc.lane == 0) atomicOr(status, CPIC_STATUS_PIPELINE);
  drain_queue<R, VL, FAST, Acc>(part, Q, qn, lc.lane, a, acc, status);
}

// ------------------------------------------------------------ host side
template <class R, int VL, bool LITERAL, bool FAST, class Acc>
int launch_push(void* particles, int n, const void* interp, void* acc, const PushArgs<R>& a,
                int* status, cudaStream_t s) {
  auto kern = push_kernel<R, VL, LITERAL, FAST, Acc>;
  static std::atomic<int> per_sm[64];  // blocks per SM, per device (0: not yet queried)
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return CPIC_ECUDA;
  int b = per_sm[dev].load(std::memory_order_relaxed);
  if (b == 0) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, kPushThreads, 0) != cudaSuccess || b < 1) b = 1;
    per_sm[dev].store(b, std::memory_order_relaxed);
  }
  const int64_t chunks = ((int64_t)n + 31) / 32;
  int64_t blocks = (int64_t)sm_count() * b;
  const int64_t need = (chunks + kWarps - 1) / kWarps;
  if (blocks > need) blocks = need;
  if (blocks < 1) blocks = 1;
  kern<<<(unsigned)blocks, kPushThreads, 0, s>>>(static_cast<unsigned char*>(particles), n,
                                                static_cast<const R*>(interp), static_cast<Acc*>(acc), a,
                                                status);
  return launch_status();
}

// Tile shape: chunks per consumer warp and the largest window segment.  Each
// tile sizes its own window from its sampled cells (a run of tile / ppc
// voxels plus margins), so the shape does not depend on the mean particle
// density, which says little when particles fill part of the box; wxmax only
// bounds the shared memory.  Runs longer than wxmax - 3 voxels get a window
// centred on the median sample and the rest of the tile gathers from global
// memory.
struct TileShape {
  int chunks_per_warp, wxmax;
};

// 7 chunks per consumer warp (3,360 particles a tile) and cross windows of 56
// voxels per segment: 2 x (44 KB window buffers + 35 KB static) per SM, which
// leaves ~90 KB of L1 for the global gathers of the cells outside the window.
// At 64 particles per cell a tile spans ~52 voxels, so the window covers it
// once the particles are in cell order.  With 9-row windows the shared memory
// allowed only 44 voxels (larger windows crossed the 196 KB carveout and cost
// 5%), so a tile's edge cells gathered from global memory; larger tiles still
// measured faster than windows covering the whole tile (4 chunks and 36
// voxels: 2.55 ms, 7 and 44: 2.47 ms at 128^3 x 64 ppc on cell keys).
#ifndef CPIC_TILE_CHUNKS
#define CPIC_TILE_CHUNKS 7  // chunks per consumer warp and tile
#endif
#ifndef CPIC_TILE_WXMAX
#define CPIC_TILE_WXMAX 56  // longest window segment (voxels)
#endif
static_assert(CPIC_TILE_WXMAX <= 64, "a window segment must fit the 3-block landing buffers");
inline TileShape tile_shape(const GridDev& g) {
  TileShape ts{CPIC_TILE_CHUNKS, CPIC_TILE_WXMAX};
  if (ts.wxmax > g.sx) ts.wxmax = g.sx;  // segments of one window must not overlap
  if (ts.wxmax < 3) ts.wxmax = 3;
  return ts;
}

template <class R, int VL, bool LITERAL, bool FAST, class Acc, bool OUT = false>
int launch_push_tiled(void* particles, int n, const void* interp, void* acc, const PushArgs<R>& a,
                      int* status, cudaStream_t s, const void* src = nullptr) {
  auto kern = push_tiled_kernel<R, VL, LITERAL, FAST, Acc, OUT>;
  const TileShape ts = tile_shape(a.g);
  const size_t dyn = tiled_dyn_smem<R>(ts.wxmax);
  // Per device: the largest dynamic shared memory opted in so far (the
  // attribute only ever grows, under the mutex, so a concurrent launch that
  // needs less never lowers it under another), and the occupancy for the
  // last size queried, packed as dyn << 16 | blocks per SM.
  static std::atomic<size_t> opted[64];
  static std::atomic<uint64_t> occ[64];
  static std::mutex opt_in;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return CPIC_ECUDA;
  // the 48 KB default covers static + dynamic shared memory: opt in for any size
  if (opted[dev].load(std::memory_order_acquire) < dyn) {
    std::lock_guard<std::mutex> lock(opt_in);
    if (opted[dev].load(std::memory_order_relaxed) < dyn) {
      if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn) != cudaSuccess)
        return CPIC_ECUDA;
      opted[dev].store(dyn, std::memory_order_release);
    }
  }
  uint64_t o = occ[dev].load(std::memory_order_relaxed);
  if ((o >> 16) != (uint64_t)dyn) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, kTiledThreads, dyn) != cudaSuccess || b < 1) b = 1;
    o = ((uint64_t)dyn << 16) | (uint64_t)(b & 0xffff);
    occ[dev].store(o, std::memory_order_relaxed);
  }
  const int64_t T = 32LL * kConsumers * ts.chunks_per_warp;
  const int64_t ntiles = ((int64_t)n + T - 1) / T;
  int64_t blocks = (int64_t)sm_count() * (int64_t)(o & 0xffff);
  if (blocks > ntiles) blocks = ntiles;
  if (blocks < 1) blocks = 1;
  kern<<<(unsigned)blocks, kTiledThreads, dyn, s>>>(static_cast<unsigned char*>(particles), n,
                                                  static_cast<const R*>(interp), static_cast<Acc*>(acc), a,
                                                  status, ts.chunks_per_warp, ts.wxmax,
                                                  static_cast<const unsigned char*>(src));
  return launch_status();
}

template <class R, int VL, bool LITERAL, bool FAST, class Acc = R>
int launch_any(bool tiled, void* particles, int n, const void* interp, void* acc, const PushArgs<R>& a,
               int* status, cudaStream_t s) {
  return tiled ? launch_push_tiled<R, VL, LITERAL, FAST, Acc>(particles, n, interp, acc, a, status, s)
               : launch_push<R, VL, LITERAL, FAST, Acc>(particles, n, interp, acc, a, status, s);
}

// Dispatch over real_t, vector length, the sqrt variant and the kernel.
template <bool FAST>
int push_dispatch(void* particles, int n, const void* interp, void* acc, const cpic_grid* g,
                  const cpic_push_params* prm, int* status, cudaStream_t s) {
  const bool literal = !(prm->flags & CPIC_PUSH_TRUE_SQRT);
  const GridDev gd = make_grid(g);
  // the window arithmetic keeps 3 * sx * sy and cell + sx * sy + sx in int range
  const bool tiled = !(prm->flags & CPIC_PUSH_STREAMING) && gd.num_cells <= (1 << 30);
  const AccMap am{(prm->flags & CPIC_PUSH_ACC_LAYOUT_LEFT) ? 1 : 0, gd.num_cells};
  if (prm->precision == CPIC_FLOAT) {
    PushArgs<float> a{(float)prm->qdt_2mc, (float)prm->cdt_dx, (float)prm->cdt_dy,
                      (float)prm->cdt_dz, (float)prm->qsp, gd, am};
    if (prm->flags & CPIC_PUSH_ACC_F64)  // FP32 particles, FP64 accumulator rows
      return prm->particle_vl == 32
                 ? launch_any<float, 32, true, FAST, double>(tiled, particles, n, interp, acc, a, status, s)
                 : launch_any<float, 16, true, FAST, double>(tiled, particles, n, interp, acc, a, status, s);
    return prm->particle_vl == 32 ? launch_any<float, 32, true, FAST>(tiled, particles, n, interp, acc, a, status, s)
                                  : launch_any<float, 16, true, FAST>(tiled, particles, n, interp, acc, a, status, s);
  }
  PushArgs<double> a{prm->qdt_2mc, prm->cdt_dx, prm->cdt_dy, prm->cdt_dz, prm->qsp, gd, am};
  if (prm->particle_vl == 32)
    return literal ? launch_any<double, 32, true, FAST>(tiled, particles, n, interp, acc, a, status, s)
                   : launch_any<double, 32, false, FAST>(tiled, particles, n, interp, acc, a, status, s);
  return literal ? launch_any<double, 16, true, FAST>(tiled, particles, n, interp, acc, a, status, s)
                 : launch_any<double, 16, false, FAST>(tiled, particles, n, interp, acc, a, status, s);
}

// The out-of-place push (tiled kernel): particle p of `src` is pushed into
// slot p of `dst`.
template <bool FAST>
int push_into_dispatch(const void* src, void* dst, int n, const void* interp, void* acc,
                       const cpic_grid* g, const cpic_push_params* prm, int* status, cudaStream_t s) {
  const bool literal = !(prm->flags & CPIC_PUSH_TRUE_SQRT);
  const GridDev gd = make_grid(g);
  if (gd.num_cells > (1 << 30)) return CPIC_EUNSUPPORTED;
  const AccMap am{(prm->flags & CPIC_PUSH_ACC_LAYOUT_LEFT) ? 1 : 0, gd.num_cells};
  if (prm->precision == CPIC_FLOAT) {
    PushArgs<float> a{(float)prm->qdt_2mc, (float)prm->cdt_dx, (float)prm->cdt_dy,
                      (float)prm->cdt_dz, (float)prm->qsp, gd, am};
    if (prm->flags & CPIC_PUSH_ACC_F64)
      return prm->particle_vl == 32
                 ? launch_push_tiled<float, 32, true, FAST, double, true>(dst, n, interp, acc, a, status, s, src)
                 : launch_push_tiled<float, 16, true, FAST, double, true>(dst, n, interp, acc, a, status, s, src);
    return prm->particle_vl == 32
               ? launch_push_tiled<float, 32, true, FAST, float, true>(dst, n, interp, acc, a, status, s, src)
               : launch_push_tiled<float, 16, true, FAST, float, true>(dst, n, interp, acc, a, status, s, src);
  }
  PushArgs<double> a{prm->qdt_2mc, prm->cdt_dx, prm->cdt_dy, prm->cdt_dz, prm->qsp, gd, am};
  if (prm->particle_vl == 32)
    return literal ? launch_push_tiled<double, 32, true, FAST, double, true>(dst, n, interp, acc, a, status, s, src)
                   : launch_push_tiled<double, 32, false, FAST, double, true>(dst, n, interp, acc, a, status, s, src);
  return literal ? launch_push_tiled<double, 16, true, FAST, double, true>(dst, n, interp, acc, a, status, s, src)
                 : launch_push_tiled<double, 16, false, FAST, double, true>(dst, n, interp, acc, a, status, s, src);
}

}  // namespace CPIC_PUSH_NS
}  // namespace cpic
