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
// Design (one CUDA thread per particle, one warp per 32-particle AoSoA chunk):
//   * a warp streams 32-particle chunks: with VL = 32 a chunk is one
//     contiguous 1 KiB AoSoA block (128 B per member), with VL = 16 two; each
//     lane's byte offsets inside a chunk are loop-invariant, and the next
//     chunk's eight members are loaded before the current chunk is processed
//     (one chunk of register prefetch per warp).  A ring of bulk asynchronous
//     copies (cp.async.bulk into shared memory, four chunks ahead) was
//     measured slower: it cut the latency stalls but added instructions and,
//     with 200 KB of shared memory per SM, left too little L1 for the
//     interpolator gathers;
//   * the 18 interpolator coefficients of the particle's cell are gathered
//     through the read-only cache; after a cell sort a warp mostly shares one
//     cell, so the gather is a broadcast;
//   * in-cell particles deposit their 12 currents through a warp reduction:
//     when every depositing lane of the warp is in one cell, a 13-shuffle
//     reduce-scatter leaves one total per lane and 12 lanes write it with one
//     atomic each;
//     otherwise the largest group of lanes sharing a cell is reduced that way
//     and the other lanes use 16-byte vector reductions (red.global.add.v4);
//   * cell-crossing particles are compacted into a per-warp shared-memory
//     queue (ballot + prefix popcount) and moved 32 at a time, so the common
//     path stays branch-free and the streak loop runs on full warps.  The
//     streak loop is capped; hitting the cap sets CPIC_STATUS_MOVER_CAP.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

#ifndef CPIC_PUSH_NS
#error "define CPIC_PUSH_NS before including push_impl.cuh"
#endif

namespace cpic {

template <class R>
struct PushArgs {
  R qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp;
  GridDev g;
};

namespace CPIC_PUSH_NS {

constexpr int kPushThreads = 256;
constexpr int kQueueCap = 64;    // per warp: drained whenever it holds >= 32
constexpr int kMaxStreaks = 16;  // a Courant-limited move needs at most 4

template <class R>
struct MoverQueue {
  R px[kQueueCap], py[kQueueCap], pz[kQueueCap];  // offsets before the move
  R dx[kQueueCap], dy[kQueueCap], dz[kQueueCap];  // normalised displacement
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

// Deposit of the in-cell particles of one warp.  `dep` lanes add v[0..11] to
// accumulator row `cell`; `vi` is value_of_lane(lane).
template <class R>
__device__ __forceinline__ void warp_deposit(R* __restrict__ acc, int cell, bool dep,
                                             const R v[12], int lane, int vi) {
  const unsigned dm = __ballot_sync(kFull, dep);
  if (dm == 0u) return;
  const int cell0 = __shfl_sync(kFull, cell, __ffs(dm) - 1);
  if (__all_sync(kFull, !dep || cell == cell0)) {  // every depositing lane in one cell
    R w[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) w[k] = dep ? v[k] : R(0);
    const R tot = reduce_scatter12<R>(w, lane);
    if (vi >= 0) red_add(acc + (size_t)cell0 * 12 + vi, tot);
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
    if (vi >= 0) red_add(acc + (size_t)major_cell * 12 + vi, tot);
  }
  if (dep && !in_major) {
    R* a = acc + (size_t)cell * 12;
    red_add4(a + 0, v[0], v[1], v[2], v[3]);
    red_add4(a + 4, v[4], v[5], v[6], v[7]);
    red_add4(a + 8, v[8], v[9], v[10], v[11]);
  }
}

// move_p for one particle (src/move_p.h:93-371), positions and displacement in
// registers; writes the final offsets and cell of particle `pidx`.
template <class R, int VL>
__device__ __noinline__ void move_one(unsigned char* __restrict__ part, R px, R py, R pz, R dx,
                                      R dy, R dz, R q, int cell, int pidx, R* __restrict__ acc,
                                      const GridDev g, int* __restrict__ status) {
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
    const R fx = (sx == 0) ? R(3.4e38) : (dirx - px) / sx;
    const R fy = (sy == 0) ? R(3.4e38) : (diry - py) / sy;
    const R fz = (sz == 0) ? R(3.4e38) : (dirz - pz) / sz;
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
    R* a = acc + (size_t)cell * 12;
    red_add4(a + 0, v[0], v[1], v[2], v[3]);
    red_add4(a + 4, v[4], v[5], v[6], v[7]);
    red_add4(a + 8, v[8], v[9], v[10], v[11]);
    dx -= sx; dy -= sy; dz -= sz;
    px += sx + sx; py += sy + sy; pz += sz + sz;
    if (axis == 3) { done = true; break; }

    const R fs = (axis == 0) ? dirx : (axis == 1) ? diry : dirz;
    // RANK_TO_INDEX (src/types.h:184-193)
    int ix = cell, iy, iz;
    iy = ix / g.sx; ix -= iy * g.sx;
    iz = iy / g.sy; iy -= iz * g.sy;
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

template <class R, int VL, bool LITERAL, bool FAST>
__global__ void __launch_bounds__(kPushThreads)
push_kernel(unsigned char* __restrict__ part, int n, const R* __restrict__ interp,
            R* __restrict__ acc, const PushArgs<R> a, int* __restrict__ status) {
  constexpr size_t kBlk = (size_t)VL * (7 * sizeof(R) + sizeof(int));  // SoA block bytes
  constexpr size_t kChunk = (size_t)32 * (7 * sizeof(R) + sizeof(int));  // 32 particles
  constexpr int kMem = VL * (int)sizeof(R);
  __shared__ MoverQueue<R> queues[kPushThreads / 32];
  MoverQueue<R>& Q = queues[threadIdx.x >> 5];
  const int lane = lane_id();
  const unsigned lt_mask = (1u << lane) - 1u;
  const int vi = value_of_lane(lane);
  // this lane's byte offsets inside a 32-particle chunk (loop-invariant)
  const int lane_off = (lane / VL) * (int)kBlk + (lane % VL) * (int)sizeof(R);
  const int lane_cell_off = (lane / VL) * (int)kBlk + 7 * kMem + (lane % VL) * (int)sizeof(int);
  const int nchunks = (n + 31) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const R one = 1., one_third = 1. / 3., two_fifteenths = 2. / 15.;
  int qn = 0;

  int chunk = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  PState<R> cur;
  load_state<R, VL>(part + (size_t)chunk * kChunk, lane_off, lane_cell_off,
                    chunk < nchunks && chunk * 32 + lane < n, cur);
  for (; chunk < nchunks; chunk += nwarps) {
    // prefetch the next chunk of this warp
    const int next = chunk + nwarps;
    PState<R> nxt;
    load_state<R, VL>(part + (size_t)next * kChunk, lane_off, lane_cell_off,
                      next < nchunks && next * 32 + lane < n, nxt);

    unsigned char* base = part + (size_t)chunk * kChunk;
    const int p = chunk * 32 + lane;
    bool valid = p < n;
    const R x = cur.x, y = cur.y, z = cur.z;
    R ux = cur.ux, uy = cur.uy, uz = cur.uz;
    int cell = cur.cell;
    if (valid && (unsigned)cell >= (unsigned)a.g.num_cells) {
      atomicOr(status, CPIC_STATUS_CELL_RANGE);
      valid = false;
      cell = 0;
    }
    // gather (push.h:74-93)
    const R* f = interp + ((size_t)(cell >> 5) * (18 * kCellBlock) + (cell & 31));
    const R ex = __ldg(f + 0 * 32), dexdy = __ldg(f + 1 * 32);
    const R dexdz = __ldg(f + 2 * 32), d2exdydz = __ldg(f + 3 * 32);
    const R ey = __ldg(f + 4 * 32), deydz = __ldg(f + 5 * 32);
    const R deydx = __ldg(f + 6 * 32), d2eydzdx = __ldg(f + 7 * 32);
    const R ez = __ldg(f + 8 * 32), dezdx = __ldg(f + 9 * 32);
    const R dezdy = __ldg(f + 10 * 32), d2ezdxdy = __ldg(f + 11 * 32);
    R cbx = __ldg(f + 12 * 32);
    const R dcbxdx = __ldg(f + 13 * 32);
    R cby = __ldg(f + 14 * 32);
    const R dcbydy = __ldg(f + 15 * 32);
    R cbz = __ldg(f + 16 * 32);
    const R dcbzdz = __ldg(f + 17 * 32);

    // field at the particle (push.h:124-138)
    const R hax = a.qdt_2mc * ((ex + y * dexdy) + z * (dexdz + y * d2exdydz));
    const R hay = a.qdt_2mc * ((ey + z * deydz) + x * (deydx + z * d2eydzdx));
    const R haz = a.qdt_2mc * ((ez + x * dezdx) + y * (dezdy + x * d2ezdxdy));
    cbx = cbx + x * dcbxdx;
    cby = cby + y * dcbydy;
    cbz = cbz + z * dcbzdz;

    // relativistic Boris rotation with half E kicks (push.h:144-163)
    ux += hax; uy += hay; uz += haz;
    const R b0 = scaled_rgamma<R, LITERAL, FAST>(a.qdt_2mc, one + (ux * ux + (uy * uy + uz * uz)));
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
    if (valid) {
      __stcs(reinterpret_cast<R*>(base + lane_off + 3 * kMem), ux);
      __stcs(reinterpret_cast<R*>(base + lane_off + 4 * kMem), uy);
      __stcs(reinterpret_cast<R*>(base + lane_off + 5 * kMem), uz);
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
      __stcs(reinterpret_cast<R*>(base + lane_off + 0 * kMem), nx);
      __stcs(reinterpret_cast<R*>(base + lane_off + 1 * kMem), ny);
      __stcs(reinterpret_cast<R*>(base + lane_off + 2 * kMem), nz);
    }
    R v[12];
    const R corr = q * ux * uy * uz * one_third;
    currents12<R>(q, ux, uy, uz, mx, my, mz, corr, v);
    warp_deposit<R>(acc, cell, inb, v, lane, vi);

    // compact the cell-crossing particles into the warp queue
    const bool cross = valid && !inb;
    const unsigned cm = __ballot_sync(kFull, cross);
    if (cm) {
      if (cross) {
        const int s = qn + __popc(cm & lt_mask);
        Q.px[s] = x; Q.py[s] = y; Q.pz[s] = z;
        Q.dx[s] = ux; Q.dy[s] = uy; Q.dz[s] = uz;
        Q.q[s] = q; Q.cell[s] = cell; Q.idx[s] = p;
      }
      qn += __popc(cm);
      if (qn >= 32) {
        __syncwarp();
        const int s = qn - 32 + lane;
        const R ex0 = Q.px[s], ey0 = Q.py[s], ez0 = Q.pz[s];
        const R ddx = Q.dx[s], ddy = Q.dy[s], ddz = Q.dz[s], qq = Q.q[s];
        const int cc = Q.cell[s], ii = Q.idx[s];
        __syncwarp();
        qn -= 32;
        move_one<R, VL>(part, ex0, ey0, ez0, ddx, ddy, ddz, qq, cc, ii, acc, a.g, status);
      }
    }
    cur = nxt;
  }
  __syncwarp();
  if (lane < qn) {
    move_one<R, VL>(part, Q.px[lane], Q.py[lane], Q.pz[lane], Q.dx[lane], Q.dy[lane], Q.dz[lane],
                    Q.q[lane], Q.cell[lane], Q.idx[lane], acc, a.g, status);
  }
}

template <class R, int VL, bool LITERAL, bool FAST>
int launch_push(void* particles, int n, const void* interp, void* acc, const PushArgs<R>& a,
                int* status, cudaStream_t s) {
  auto kern = push_kernel<R, VL, LITERAL, FAST>;
  static int per_sm[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return CPIC_ECUDA;
  if (per_sm[dev] == 0) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, kPushThreads, 0) != cudaSuccess || b < 1) b = 1;
    per_sm[dev] = b;
  }
  const int64_t chunks = ((int64_t)n + 31) / 32;
  int64_t blocks = (int64_t)sm_count() * per_sm[dev];
  const int64_t need = (chunks + kPushThreads / 32 - 1) / (kPushThreads / 32);
  if (blocks > need) blocks = need;
  if (blocks < 1) blocks = 1;
  kern<<<(unsigned)blocks, kPushThreads, 0, s>>>(static_cast<unsigned char*>(particles), n,
                                                static_cast<const R*>(interp), static_cast<R*>(acc), a,
                                                status);
  return launch_status();
}

// Dispatch over real_t, vector length and the sqrt variant.
template <bool FAST>
int push_dispatch(void* particles, int n, const void* interp, void* acc, const cpic_grid* g,
                  const cpic_push_params* prm, int* status, cudaStream_t s) {
  const bool literal = !(prm->flags & CPIC_PUSH_TRUE_SQRT);
  const GridDev gd = make_grid(g);
  if (prm->precision == CPIC_FLOAT) {
    PushArgs<float> a{(float)prm->qdt_2mc, (float)prm->cdt_dx, (float)prm->cdt_dy,
                      (float)prm->cdt_dz, (float)prm->qsp, gd};
    return prm->particle_vl == 32 ? launch_push<float, 32, true, FAST>(particles, n, interp, acc, a, status, s)
                                  : launch_push<float, 16, true, FAST>(particles, n, interp, acc, a, status, s);
  }
  PushArgs<double> a{prm->qdt_2mc, prm->cdt_dx, prm->cdt_dy, prm->cdt_dz, prm->qsp, gd};
  if (prm->particle_vl == 32)
    return literal ? launch_push<double, 32, true, FAST>(particles, n, interp, acc, a, status, s)
                   : launch_push<double, 32, false, FAST>(particles, n, interp, acc, a, status, s);
  return literal ? launch_push<double, 16, true, FAST>(particles, n, interp, acc, a, status, s)
                 : launch_push<double, 16, false, FAST>(particles, n, interp, acc, a, status, s);
}

}  // namespace CPIC_PUSH_NS
}  // namespace cpic
